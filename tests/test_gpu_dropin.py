"""The drop-in Python API (astrea_gb300.evolvers) driven the way the reference drives its own.

Each case builds a ``sim_variables`` namedtuple from the golden case's
settings with the fields functions/generic.py:240-264 derives
(``solver_category``, ``magnetic_2d``, ``permutations``, ``ortho_axis``) and
runs the body of core_run (astrea.py:66-85) on NumPy grids:

    fluxes = evolve_space(grid, sim_variables)
    dt = cfl * min(dx / eigmax)            (clipped at the checkpoint)
    grid = evolve_time(grid, fluxes, dt, sim_variables)
    sim_variables = sim_variables._replace(permutations=reversed(...))

and compares with what the reference's own evolve_space / evolve_time gave on
the same case (tests/golden): the per-axis fluxes and eigmax of the first
steps (keyed and ordered like ``permutations``), the corner field of the
constrained-transport cases, and the grid after every step.  Bars: 1e-12
relative to the array's largest magnitude (WENO-7: 1e-11, because dt differs
from LAPACK's in the last bit and WENO-7's weights amplify it); eigmax 1e-13.
"""

import numpy as np
import pytest

from astrea_gb300 import config as C
from astrea_gb300 import evolvers
from oracle import stepper
from tests import golden_io

pytestmark = pytest.mark.gpu

RUNNABLE = {"euler", "ssprk22", "ssprk33", "ssprk43", "ssprk53", "ssprk54", "ssprk104", "rk4"}
CASES = [n for n in golden_io.case_names()
         if C.integrator_of(golden_io.load(n)["meta"]["timestep"]) in RUNNABLE]


def rel_err(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def sim_variables(meta):
    perms, ortho = C.permutations_for(meta["dim"])
    return C.make_sim_variables(
        dimension=meta["dim"], cells=meta["cells"], subgrid=meta["subgrid"], solver=meta["solver"],
        solver_category=C.solver_category(meta["solver"]), timestep=meta["timestep"], gamma=meta["gamma"],
        boundary=meta["boundary"], dx=meta["dx"], cfl=meta["cfl"], t_end=meta["t_end"], checkpoints=1,
        precision="float64", magnetic_2d=meta["magnetic_2d"], permutations=perms, ortho_axis=ortho)


@pytest.mark.parametrize("name", CASES)
def test_core_run_body_through_the_evolvers(name):
    g = golden_io.load(name)
    meta = g["meta"]
    sv = sim_variables(meta)
    tol = 1e-11 if C.scheme_of(meta["subgrid"]) == "weno7" else 1e-12
    grid = np.copy(g["q0"])
    chkpt = sv.t_end / sv.checkpoints
    t, idx = 0.0, 1
    with np.errstate(all="ignore"):
        for s in range(meta["steps"]):
            fluxes = evolvers.evolve_space(grid, sv)
            assert list(fluxes.keys()) == list(sv.permutations.values())
            for pos, (axes, val) in enumerate(fluxes.items()):
                assert isinstance(val["eigmax"], float)
                if f"flux_s{s}_p{pos}" in g:
                    assert val["flux"].shape == g[f"flux_s{s}_p{pos}"].shape
                    assert rel_err(val["flux"], g[f"flux_s{s}_p{pos}"]) <= tol, (name, s, pos)
                    assert val["eigmax"] == pytest.approx(float(g[f"eigmax_s{s}_p{pos}"]), rel=1e-13)
                if f"corner_s{s}_p{pos}" in g:
                    assert rel_err(val["mag_corner"], g[f"corner_s{s}_p{pos}"]) <= tol, (name, s, pos)
            dt = sv.cfl * min(sv.dx / r["eigmax"] for r in fluxes.values())
            if t + dt >= chkpt * idx:
                dt = chkpt * idx - t
                idx += 1
            assert dt == pytest.approx(float(g[f"dt_{s + 1}"]), rel=1e-13)
            grid = evolvers.evolve_time(grid, fluxes, dt, sv)
            assert isinstance(grid, np.ndarray) and grid.shape == g["q0"].shape
            assert rel_err(grid, g[f"q_{s + 1}"]) <= tol, (name, s, rel_err(grid, g[f"q_{s + 1}"]))
            t += dt
            sv = sv._replace(permutations=dict(reversed(list(sv.permutations.items()))))


@pytest.mark.parametrize("name", [n for n in CASES if golden_io.load(n)["meta"]["magnetic_2d"]])
def test_evolve_time_overwrites_the_input_B_with_face_averages(name):
    """evolvers.py:73-76: the caller's grid leaves evolve_time with B_x, B_y at their face averages."""
    g = golden_io.load(name)
    sv = sim_variables(g["meta"])
    grid = np.copy(g["q0"])
    fluxes = evolvers.evolve_space(grid, sv)
    dt = .5 * sv.cfl * min(sv.dx / r["eigmax"] for r in fluxes.values())
    evolvers.evolve_time(grid, fluxes, dt, sv)
    with np.errstate(all="ignore"):
        ofl = stepper.evolve_space(g["q0"], _oracle_cfg(g["meta"]), [0, 1])
    for axis in (0, 1):
        face = ofl[axis]["wF"].transpose(stepper.PERM[axis])[..., 5 + axis]
        assert rel_err(grid[..., 5 + axis], face) <= 1e-14
    untouched = [v for v in range(8) if v not in (5, 6)]
    assert np.array_equal(grid[..., untouched], g["q0"][..., untouched])


def _oracle_cfg(meta):
    return stepper.OracleConfig(
        dim=meta["dim"], scheme=C.scheme_of(meta["subgrid"]), solver=C.solver_of(meta["solver"]),
        integrator=C.integrator_of(meta["timestep"]), gamma=meta["gamma"], bc=meta["boundary"], dx=meta["dx"],
        cfl=meta["cfl"], magnetic_2d=meta["magnetic_2d"], eig="analytic", t_end=meta["t_end"])


@pytest.mark.parametrize("name", ["sod1d_ppm_hllc", "khi2d_weno5_hllc", "quad2d_edge_ppm_lf", "ot2d_plm_hlld"])
@pytest.mark.parametrize("scale", [.37, 1.0])
def test_evolve_time_with_a_caller_dt(name, scale):
    """astrea_time with a dt of the caller's choosing (not the CFL step) against the oracle's evolve_time."""
    g = golden_io.load(name)
    meta = g["meta"]
    sv = sim_variables(meta)
    oc = _oracle_cfg(meta)
    order = stepper.initial_order(meta["dim"])
    with np.errstate(all="ignore"):
        ofl = stepper.evolve_space(g["q0"], oc, order)
        dt = scale * stepper.timestep(ofl, oc, order)
        want = stepper.evolve_time(g["q0"], ofl, dt, oc, order)
    grid = np.copy(g["q0"])
    fluxes = evolvers.evolve_space(grid, sv)
    got = evolvers.evolve_time(grid, fluxes, dt, sv)
    assert rel_err(got, want) <= 1e-14, rel_err(got, want)


def test_simulate_runs_core_run_to_t_end():
    """evolvers.simulate: the core_run loop on the device to t_end, equal to the reference's full run."""
    g = golden_io.load("sod1d_plm_lf_n128", prefix="full_")
    meta = g["meta"]
    sv = sim_variables(meta)
    q, clock = evolvers.simulate(sv, np.copy(g["q0"]))
    assert clock["done"] and clock["t"] == g["t"] and clock["steps"] == meta["steps"]
    assert rel_err(q, g["qT"]) <= 1e-12
