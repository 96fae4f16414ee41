"""PLM with the superbee slope limiter (num_methods/limiters.py:47-49) on the GPU.

The reference defines superbee but its PLM always calls minmod (plm.py:27), so
there is no reference run to compare with; the oracle's superbee is pinned to
the reference's own ``superbee_limiter`` on edge and wrap inputs
(tests/golden/unit_functions.npz, tests/test_oracle_golden.py).  Here the
kernels' PLM-superbee steps (limiter = 1) are compared with the oracle's on 1D
and 2D grids, outflow and periodic, at the FP64 bar of 1e-14 relative, and
checked to differ from the minmod steps (the limiter really switched).
"""

import numpy as np
import pytest

from astrea_gb300.solver import Solver, RunConfig
from oracle import stepper
from tests import golden_io

pytestmark = pytest.mark.gpu


def rel_err(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


# (golden case supplying the initial grid, solver, boundary)
CASES = [("sod1d_plm_lf", "llf", "edge"), ("sod1d_plm_hllc", "hllc", "edge"), ("shu1d_ppm_hllc", "llf", "edge"),
         ("quad2d_edge_plm_lf", "llf", "edge"), ("khi2d_plm_lf", "hllc", "wrap"), ("khi2d_ppm_hllc", "llf", "wrap")]


def run(name, solver, bc, limiter, steps=3):
    g = golden_io.load(name)
    meta = g["meta"]
    q0 = g["q0"]
    dim = meta["dim"]
    n = meta["cells"]
    model = 8 if np.any(q0[..., [3, 5, 6, 7] if dim == 2 else [2, 3, 5, 6, 7]] != 0) else (3 if dim == 1 else 4)
    cfg = RunConfig(dim=dim, n0=n, n1=n if dim == 2 else 1, model=model, precision=64, scheme="plm", solver=solver,
                    integrator="ssprk33", boundary=bc, limiter=limiter, gamma=meta["gamma"], dx=meta["dx"],
                    cfl=meta["cfl"], t_end=meta["t_end"])
    s = Solver(cfg)
    s.load_conservative(q0)
    s.reset_clock(0.0, 1, 0)
    oc = stepper.OracleConfig(dim=dim, scheme="plm", solver=solver, integrator="ssprk33", gamma=meta["gamma"], bc=bc,
                              dx=meta["dx"], cfl=meta["cfl"], limiter=limiter, eig="analytic", t_end=meta["t_end"])
    q, t, idx, order = q0, 0.0, 1, stepper.initial_order(dim)
    out = []
    with np.errstate(all="ignore"):
        for _ in range(steps):
            s.step(1, graph=False)
            q, t, idx, order, dt = stepper.step(q, oc, t, idx, order)
            gpu = s.conservative().cpu().numpy()
            assert s.clock()["dt"] == pytest.approx(dt, rel=1e-14, abs=0)
            out.append((gpu, q))
    return out


@pytest.mark.parametrize("name,solver,bc", CASES)
def test_superbee_steps_match_oracle(name, solver, bc):
    sb = run(name, solver, bc, "superbee")
    for k, (gpu, ora) in enumerate(sb):
        assert rel_err(gpu, ora) <= 1e-14, (name, k, rel_err(gpu, ora))
    mm = run(name, solver, bc, "minmod", steps=2)
    assert rel_err(sb[1][0], mm[1][0]) > 1e-10  # superbee and minmod give different steps
