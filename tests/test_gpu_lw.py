"""Lax-Wendroff (num_methods/solvers.py:79-88) on the GPU: ASTREA_LW against the oracle.

The kernels run LW as LLF's flux with the per-interface coefficient
v_n^2 / max|lambda| (v_n: the entropy-wave eigenvalue of the interface
average).  The reference's own coefficient column changes wave between steps
and stages (tests/test_lw_host.py), so the bar here is the oracle in its
'analytic' mode, which evaluates the same closed form: 1e-14 relative in FP64,
on 1D and 2D grids with outflow and periodic boundaries.  The drop-in
evolvers accept the reference's 'lw' string.
"""

import numpy as np
import pytest

from astrea_gb300 import config as C
from astrea_gb300 import evolvers
from astrea_gb300.solver import Solver, RunConfig
from oracle import stepper
from tests import golden_io

pytestmark = pytest.mark.gpu


def rel_err(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("name,scheme", [("sod1d_plm_lf", "plm"), ("sod1d_ppm_lf", "ppm"), ("shu1d_ppm_hllc", "weno5"),
                                         ("khi2d_plm_lf", "plm"), ("quad2d_edge_ppm_lf", "ppm"),
                                         ("mt96_quad_edge_plm_lf", "plm")])
def test_lw_steps_match_oracle(name, scheme):
    g = golden_io.load(name)
    meta = g["meta"]
    dim, n = meta["dim"], meta["cells"]
    q0 = g["q0"]
    model = 3 if dim == 1 else 4
    cfg = RunConfig(dim=dim, n0=n, n1=n if dim == 2 else 1, model=model, precision=64, scheme=scheme, solver="lw",
                    integrator="ssprk33", boundary=meta["boundary"], gamma=meta["gamma"], dx=meta["dx"],
                    cfl=meta["cfl"], t_end=meta["t_end"])
    s = Solver(cfg)
    s.load_conservative(q0)
    s.reset_clock(0.0, 1, 0)
    oc = stepper.OracleConfig(dim=dim, scheme=scheme, solver="lw", integrator="ssprk33", gamma=meta["gamma"],
                              bc=meta["boundary"], dx=meta["dx"], cfl=meta["cfl"], eig="analytic", t_end=meta["t_end"])
    q, t, idx, order = q0, 0.0, 1, stepper.initial_order(dim)
    with np.errstate(all="ignore"):
        for k in range(3):
            s.step(1, graph=False)
            q, t, idx, order, dt = stepper.step(q, oc, t, idx, order)
            assert s.clock()["dt"] == pytest.approx(dt, rel=1e-14, abs=0)
            got = s.conservative().cpu().numpy()
            assert rel_err(got, q) <= 1e-14, (name, k, rel_err(got, q))


def test_dropin_accepts_the_lw_string():
    perms, ortho = C.permutations_for(1)
    sv = C.make_sim_variables(dimension=1, cells=64, subgrid="plm", solver="lw", solver_category="lax",
                              timestep="ssprk(3,3)", gamma=1.4, boundary="edge", dx=1 / 64, cfl=.8, t_end=.2,
                              checkpoints=1, precision="float64", magnetic_2d=False, permutations=perms,
                              ortho_axis=ortho)
    g = golden_io.load("sod1d_plm_lf")
    fl = evolvers.evolve_space(np.copy(g["q0"]), sv)
    dt = sv.cfl * min(sv.dx / r["eigmax"] for r in fl.values())
    got = evolvers.evolve_time(np.copy(g["q0"]), fl, dt, sv)
    oc = stepper.OracleConfig(dim=1, scheme="plm", solver="lw", integrator="ssprk33", gamma=1.4, bc="edge",
                              dx=1 / 64, cfl=.8, eig="analytic", t_end=.2)
    with np.errstate(all="ignore"):
        ofl = stepper.evolve_space(g["q0"], oc, [0])
        want = stepper.evolve_time(g["q0"], ofl, dt, oc, [0])
    assert rel_err(got, want) <= 1e-14
