#!/usr/bin/env python3
"""Generate golden vectors by running the reference astrea hot path in-process.

Usage:  python tests/golden/make_golden.py --reference <path of a mervyzr/astrea checkout>
        (or set ASTREA_REFERENCE)

The reference (mervyzr/astrea) is pure Python + NumPy; its CLI needs h5py,
PyYAML and tinydb, so this script builds the ``sim_variables`` namedtuple
directly, mirroring functions/generic.py:handle_variables (lines 240-264):
``solver_category``, ``magnetic_2d``, the convert functions, ``permutations``
and ``ortho_axis``.  Each case runs the reference's own
``evolvers.evolve_space`` / ``evolvers.evolve_time`` and the dt rule of
astrea.core_run (astrea.py:66-85) for a few steps and stores the inputs and
outputs as compressed ``.npz`` files next to this script.  Unit cases call
the reference's limiter / solver / conversion functions directly.

The fixtures are what the CPU test suite pins the oracle against; the GPU
box never reads the reference.
"""

import argparse
import itertools
import json
import os
import sys
from collections import namedtuple

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SEED = 20261203

HLL = ["hllc", "c", "hlld", "d"]
COMPLETE = ["os", "osher", "solomon", "osher-solomon", "osher solomon", "es", "entropy", "entropy-stable"]


def reference_path():
    """The reference checkout: ``--reference <path>`` on the command line, or $ASTREA_REFERENCE."""
    if "--reference" in sys.argv[1:-1]:
        return sys.argv[sys.argv.index("--reference") + 1]
    path = os.environ.get("ASTREA_REFERENCE")
    if not path:
        sys.exit("the reference checkout is needed: pass --reference <path> or set ASTREA_REFERENCE")
    return path


def load_reference(path):
    sys.dont_write_bytecode = True
    sys.path.insert(0, path)
    from functions import fv, constructor  # noqa: E402
    from num_methods import evolvers, limiters, solvers, mag_field  # noqa: E402
    from schemes import ppm, weno, plm  # noqa: E402
    from static import tests as rtests  # noqa: E402
    return dict(fv=fv, constructor=constructor, evolvers=evolvers, limiters=limiters, solvers=solvers,
                mag_field=mag_field, ppm=ppm, weno=weno, plm=plm, tests=rtests)


def make_sv(R, config, cells, dim, subgrid, solver, timestep, cfl=0.8, gamma=1.4, magnetic_2d=False, **over):
    fv = R["fv"]
    d = dict(config=config, cells=cells, cfl=cfl, gamma=gamma, dimension=dim, precision="float64",
             subgrid=subgrid, timestep=timestep, solver=solver, run_type="single", checkpoints=1)
    d.update(R["tests"].generate_test_conditions(config, cells, gamma))
    d["solver_category"] = "hll" if solver in HLL else ("complete" if solver in COMPLETE else "lax")
    d["magnetic_2d"] = magnetic_2d
    if subgrid.startswith("w") or subgrid in ["ppm", "parabolic", "p"]:
        d["convert_primitive"] = fv.high_order_convert_primitive
        d["convert_conservative"] = fv.high_order_convert_conservative
    else:
        d["convert_primitive"] = fv.point_convert_primitive
        d["convert_conservative"] = fv.point_convert_conservative
    perms = [a for a in itertools.permutations(range(dim + 1)) if a[-1] == dim]
    d["permutations"] = {i: a for i, a in enumerate(perms)}
    d["ortho_axis"] = perms[-1]
    d.update(over)
    return namedtuple("simulation_variables", d)(**d)


def quadrant_ic(rng, n, mhd=False):
    """Four-quadrant Riemann data (point primitives) on an n x n grid."""
    w = np.zeros((n, n, 8))
    h = n // 2
    for (i0, i1), (j0, j1) in itertools.product([(0, h), (h, n)], [(0, h), (h, n)]):
        s = np.zeros(8)
        s[0], s[4] = rng.uniform(.1, 2), rng.uniform(.1, 2)
        s[1], s[2] = rng.uniform(-1, 1), rng.uniform(-1, 1)
        if mhd:
            s[5:8] = rng.uniform(-1, 1, 3)
        w[i0:i1, j0:j1] = s
    return w


ONLY = None  # case-name prefixes to generate (None: all)


def wanted(name):
    return ONLY is None or any(name.startswith(p) for p in ONLY)


def run_case(R, name, sv, steps, grid0=None, store_space=True, space_steps=2):
    """Run ``steps`` steps of the reference loop and save inputs/outputs (the fluxes of the
    first ``space_steps`` steps)."""
    if not wanted(name):
        return
    evolvers, constructor = R["evolvers"], R["constructor"]
    grid = constructor.initialise(sv, convert=True) if grid0 is None else sv.convert_primitive(grid0, sv)
    if grid0 is not None:
        grid = R["fv"].high_order_convert("cntr", grid, sv)
    out = {"q0": np.copy(grid)}
    chkpt = sv.t_end / sv.checkpoints
    t, idx = 0.0, 1
    for s in range(steps):
        fluxes = evolvers.evolve_space(grid, sv)
        if store_space and s < space_steps:
            for pos, (axes, val) in enumerate(fluxes.items()):
                out[f"flux_s{s}_p{pos}"] = np.copy(val["flux"])
                out[f"eigmax_s{s}_p{pos}"] = np.float64(val["eigmax"])
                if "mag_corner" in val:
                    out[f"corner_s{s}_p{pos}"] = np.copy(val["mag_corner"])
        dt = sv.cfl * min([sv.dx / r["eigmax"] for r in fluxes.values()])
        if t + dt >= chkpt * idx:
            dt = chkpt * idx - t
            idx += 1
        grid = evolvers.evolve_time(np.copy(grid), fluxes, dt, sv)
        if not np.all(np.isfinite(grid)):
            raise np.linalg.LinAlgError("non-finite state")
        t += dt
        out[f"q_{s + 1}"] = np.copy(grid)
        out[f"dt_{s + 1}"] = np.float64(dt)
        sv = sv._replace(permutations=dict(reversed(list(sv.permutations.items()))))
    meta = dict(name=name, steps=steps, dim=sv.dimension, subgrid=sv.subgrid, solver=sv.solver,
                timestep=sv.timestep, gamma=sv.gamma, boundary=sv.boundary, dx=sv.dx, cfl=sv.cfl,
                magnetic_2d=sv.magnetic_2d, t_end=sv.t_end, cells=sv.cells)
    out["meta"] = np.array(json.dumps(meta))
    np.savez_compressed(os.path.join(HERE, f"case_{name}.npz"), **out)
    print(f"{name}: steps={steps} dt1={out['dt_1']:.6e}")


def run_full(R, name, sv):
    """Run to t_end (final grid only)."""
    if not wanted(name):
        return
    evolvers, constructor = R["evolvers"], R["constructor"]
    grid = constructor.initialise(sv, convert=True)
    q0 = np.copy(grid)
    chkpt = sv.t_end / sv.checkpoints
    t, idx, n = 0.0, 1, 0
    while t <= sv.t_end:
        if t == sv.t_end:
            break
        fluxes = evolvers.evolve_space(grid, sv)
        dt = sv.cfl * min([sv.dx / r["eigmax"] for r in fluxes.values()])
        if t + dt >= chkpt * idx:
            dt = chkpt * idx - t
            idx += 1
        grid = evolvers.evolve_time(grid, fluxes, dt, sv)
        t += dt
        n += 1
        sv = sv._replace(permutations=dict(reversed(list(sv.permutations.items()))))
    meta = dict(name=name, steps=n, dim=sv.dimension, subgrid=sv.subgrid, solver=sv.solver, timestep=sv.timestep,
                gamma=sv.gamma, boundary=sv.boundary, dx=sv.dx, cfl=sv.cfl, magnetic_2d=sv.magnetic_2d,
                t_end=sv.t_end, cells=sv.cells)
    np.savez_compressed(os.path.join(HERE, f"full_{name}.npz"), q0=q0, qT=grid, t=np.float64(t),
                        meta=np.array(json.dumps(meta)))
    print(f"full {name}: steps={n} t={t}")


def unit_cases(R):
    """Direct calls of the reference's limiter / solver / conversion functions."""
    rng = np.random.default_rng(SEED)
    fv, limiters, solvers, constructor, weno_mod = R["fv"], R["limiters"], R["solvers"], R["constructor"], R["weno"]
    out = {}
    n = 40
    w = np.abs(rng.standard_normal((n, 8))) + .2
    w[:, 1:4] = rng.standard_normal((n, 3))
    w[:, 5:8] = rng.standard_normal((n, 3))
    out["w"] = w
    for bc in ("edge", "wrap"):
        wp = fv.add_boundary(w, bc)
        out[f"minmod_{bc}"] = limiters.minmod_limiter(wp)
        out[f"superbee_{bc}"] = limiters.superbee_limiter(wp)
        # the face interpolation and limiter call exactly as ppm.run does them (ppm.py:30-72)
        w2 = fv.add_boundary(w, bc, 2)
        wv = np.copy(w2[1:-1])
        wF = 7 / 12 * (w + wv[2:]) - 1 / 12 * (wv[:-2] + w2[4:])
        wF_pad2 = fv.add_boundary(wF, bc, 2)
        wL, wR = limiters.extrapolant_limiter(w, wv, w2, wF_pad2, "mc", bc, np.copy(wF_pad2[1:-3]), np.copy(wF_pad2[2:-2]))
        out[f"ppm_wL_{bc}"], out[f"ppm_wR_{bc}"] = wL, wR
        for order in (3, 5, 7):
            svw = make_sv(R, "sod", n, 1, f"weno{order}", "lf", "ssprk(3,3)", boundary=bc)
            data = weno_mod.run(R["fv"].point_convert_primitive(w, svw), svw)
            out[f"weno{order}_wS_{bc}"] = data[(0, 1)]["wS"]
            out[f"weno{order}_wp_{bc}"], out[f"weno{order}_wm_{bc}"] = data[(0, 1)]["wFs"]
    for axis in (0, 1, 2):
        out[f"flux_axis{axis}"] = constructor.make_flux(w, 1.4, axis)
    wpl, wmi = w[1:], w[:-1]
    out["roe"] = constructor.make_Roe_average(wpl, wmi)
    out["p2c"] = fv.point_convert_primitive(w, make_sv(R, "sod", n, 1, "plm", "lf", "ssprk(3,3)"))
    out["c2p"] = fv.point_convert_conservative(out["p2c"], make_sv(R, "sod", n, 1, "plm", "lf", "ssprk(3,3)"))
    svh = make_sv(R, "sod", n, 1, "plm", "hllc", "ssprk(3,3)")
    qpl, qmi = fv.point_convert_primitive(wpl, svh), fv.point_convert_primitive(wmi, svh)
    fpl, fmi = constructor.make_flux(wpl, 1.4, 0), constructor.make_flux(wmi, 1.4, 0)
    for label in (0, 1):
        out[f"hllc_label{label}"] = solvers.calculate_HLLC_flux(label, svh, wFs=(wpl, wmi), qFs=(qpl, qmi), fluxFs=(fpl, fmi))
        out[f"hlld_label{label}"] = solvers.calculate_HLLD_flux(label, svh, wS=w[:-2], wFs=(wpl, wmi), qFs=(qpl, qmi), fluxFs=(fpl, fmi))
    np.savez_compressed(os.path.join(HERE, "unit_functions.npz"), **out)
    print("unit cases:", len(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("ASTREA_REFERENCE"),
                    help="path of a mervyzr/astrea checkout (default: $ASTREA_REFERENCE)")
    ap.add_argument("--only", default=None, help="comma-separated case-name prefixes to (re)generate")
    args = ap.parse_args()
    if not args.reference:
        ap.error("--reference (or ASTREA_REFERENCE) is required")
    global ONLY
    ONLY = args.only.split(",") if args.only else None
    np.seterr(all="ignore")
    R = load_reference(args.reference)
    rng = np.random.default_rng(SEED)

    # 1D hydro (Sod, outflow) -- the plain-method config and its scheme/solver/integrator variants
    for sub, sol in [("plm", "lf"), ("ppm", "lf"), ("ppm", "hllc"), ("weno5", "hllc"), ("weno3", "lf"),
                     ("weno7", "lf"), ("pcm", "lf"), ("plm", "hllc")]:
        run_case(R, f"sod1d_{sub}_{sol}", make_sv(R, "sod", 64, 1, sub, sol, "ssprk(3,3)"), 4)
    for ts in ["euler", "rk4", "ssprk(2,2)", "ssprk(4,3)", "ssprk(5,3)", "ssprk(5,4)", "ssprk(10,4)"]:
        tag = ts.replace("(", "").replace(")", "").replace(",", "")
        run_case(R, f"sod1d_plm_lf_{tag}", make_sv(R, "sod", 48, 1, "plm", "lf", ts), 2, store_space=False)
    run_case(R, "shu1d_ppm_hllc", make_sv(R, "shu-osher", 64, 1, "ppm", "hllc", "ssprk(3,3)"), 3)
    # 1D MHD (Brio-Wu): HLLD and LLF
    run_case(R, "bw1d_plm_hlld", make_sv(R, "brio-wu", 64, 1, "plm", "hlld", "ssprk(3,3)", gamma=2.0), 3)
    run_case(R, "bw1d_weno5_hlld", make_sv(R, "brio-wu", 64, 1, "weno5", "hlld", "ssprk(3,3)", gamma=2.0), 3)
    run_case(R, "bw1d_ppm_lf", make_sv(R, "brio-wu", 64, 1, "ppm", "lf", "ssprk(3,3)", gamma=2.0), 3)
    # full run of the plain config at reduced N
    run_full(R, "sod1d_plm_lf_n128", make_sv(R, "sod", 128, 1, "plm", "lf", "ssprk(3,3)"))

    # 2D hydro, periodic (built-in KHI and Lax-Liu 3)
    run_case(R, "khi2d_ppm_hllc", make_sv(R, "khi", 24, 2, "ppm", "hllc", "ssprk(3,3)"), 3)
    run_case(R, "khi2d_plm_lf", make_sv(R, "khi", 24, 2, "plm", "lf", "ssprk(3,3)"), 3)
    run_case(R, "khi2d_weno5_hllc", make_sv(R, "khi", 24, 2, "weno5", "hllc", "ssprk(3,3)"), 3)
    run_case(R, "ll6_2d_weno5_hllc", make_sv(R, "ll6", 20, 2, "weno5", "hllc", "ssprk(3,3)"), 3)
    run_case(R, "ll3_2d_ppm_lf", make_sv(R, "ll3", 20, 2, "ppm", "lf", "ssprk(3,3)"), 2)
    # 2D hydro, outflow, seeded four-quadrant data (per-intermediate outflow padding)
    # (the reference's 2D HLLC can produce NaN on some draws; the first draw that stays finite is kept)
    for sub, sol in [("plm", "lf"), ("ppm", "hllc"), ("weno5", "lf"), ("ppm", "lf")]:
        sv = make_sv(R, "ll1", 24, 2, sub, sol, "ssprk(3,3)", boundary="edge", t_end=0.25)
        for draw in range(50):
            try:
                run_case(R, f"quad2d_edge_{sub}_{sol}", sv, 3, grid0=quadrant_ic(np.random.default_rng(SEED + draw), 24))
                break
            except np.linalg.LinAlgError:
                continue
    # 2D MHD with constrained transport (Orszag-Tang)
    for sub, sol in [("weno5", "hlld"), ("plm", "hlld"), ("ppm", "hlld")]:
        sv = make_sv(R, "orszag-tang", 24, 2, sub, sol, "ssprk(3,3)", gamma=5 / 3, magnetic_2d=True, cfl=0.4)
        run_case(R, f"ot2d_{sub}_{sol}", sv, 3)
    multitile_cases(R)
    # Lax-Wendroff (solvers.py:79-88): its coefficient column and runs (lw_columns.npz)
    if wanted("lw_columns"):
        lw_columns(R)
    if wanted("unit"):
        unit_cases(R)


def lw_columns(R):
    """The reference's Lax-Wendroff 'sound speed' next to the entropy-wave eigenvalue.

    solvers.py:84 takes ``np.unique(characteristics, axis=-1)[..., 1]``: the second of the
    eigenvalue *columns* of the whole interface array, sorted lexicographically, so which wave
    it is depends on the first interface where the candidate columns differ (and on LAPACK's
    order within each row).  Stored per step of three 1D runs: that column, v_n (the Jacobian's
    diagonal) and the reference's grid after the step."""
    fv, constructor, evolvers = R["fv"], R["constructor"], R["evolvers"]
    out = {}
    for tag, config, sub, steps in [("sod_plm", "sod", "plm", 4), ("sod_ppm", "sod", "ppm", 4),
                                    ("sin_plm", "sin", "plm", 2)]:
        sv = make_sv(R, config, 64, 1, sub, "lw", "ssprk(3,3)")
        grid = constructor.initialise(sv, convert=True)
        out[f"{tag}_q0"] = np.copy(grid)
        for s in range(steps):
            data = R["plm"].run(grid, sv) if sub == "plm" else R["ppm"].run(grid, sv, author="mc")
            jac = data[(0, 1)]["Jacobian"]
            ch, _ = fv.compute_eigen(jac)
            out[f"{tag}_col_s{s}"] = np.real(np.unique(ch, axis=-1)[..., 1])
            out[f"{tag}_vn_s{s}"] = np.copy(jac[..., 1, 1])
            fluxes = evolvers.evolve_space(grid, sv)
            dt = sv.cfl * min([sv.dx / r["eigmax"] for r in fluxes.values()])
            grid = evolvers.evolve_time(np.copy(grid), fluxes, dt, sv)
            out[f"{tag}_q_{s + 1}"] = np.copy(grid)
        out[f"{tag}_meta"] = np.array(json.dumps(dict(config=config, subgrid=sub, steps=steps, cells=64, dx=sv.dx,
                                                      gamma=sv.gamma, cfl=sv.cfl, boundary=sv.boundary,
                                                      t_end=sv.t_end)))
    np.savez_compressed(os.path.join(HERE, "lw_columns.npz"), **out)
    print("lw columns:", len(out))


def multitile_cases(R):
    """Grids of several sweep tiles per axis (tiles are 32 cells along the sweep and 8 or 15 rows
    across it), so that interior tiles, tile seams, shared-stencil strips and bulk-copied boxes are
    compared with the reference, not only tiles clamped at the grid's edges: 96^2 hydro in edge
    and wrap, 64^2 constrained-transport MHD.  Three steps each (both axis orders); the fluxes of
    the first step."""
    kw = dict(space_steps=1)
    run_case(R, "mt96_khi_ppm_hllc", make_sv(R, "khi", 96, 2, "ppm", "hllc", "ssprk(3,3)"), 3, **kw)
    run_case(R, "mt96_khi_weno5_hllc", make_sv(R, "khi", 96, 2, "weno5", "hllc", "ssprk(3,3)"), 3, **kw)
    run_case(R, "mt96_khi_plm_lf", make_sv(R, "khi", 96, 2, "plm", "lf", "ssprk(3,3)"), 3, **kw)
    for sub, sol in [("ppm", "hllc"), ("plm", "lf"), ("weno5", "lf")]:
        name = f"mt96_quad_edge_{sub}_{sol}"
        sv = make_sv(R, "ll1", 96, 2, sub, sol, "ssprk(3,3)", boundary="edge", t_end=0.25)
        for draw in range(50):
            try:
                run_case(R, name, sv, 3, grid0=quadrant_ic(np.random.default_rng(SEED + draw), 96), **kw)
                break
            except np.linalg.LinAlgError:
                continue
    sv = make_sv(R, "orszag-tang", 64, 2, "weno5", "hlld", "ssprk(3,3)", gamma=5 / 3, magnetic_2d=True, cfl=0.4)
    run_case(R, "mt64_ot_weno5_hlld", sv, 3, **kw)
    sv = make_sv(R, "orszag-tang", 64, 2, "ppm", "hlld", "ssprk(3,3)", gamma=5 / 3, magnetic_2d=True, cfl=0.4)
    run_case(R, "mt64_ot_ppm_hlld", sv, 3, **kw)


if __name__ == "__main__":
    main()
