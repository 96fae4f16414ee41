"""TMA staging of the sweep tiles: same results as plain loads, and as the oracle.

Interior tiles of 2D grids whose rows are whole 16-byte units are staged by one
bulk tensor copy (cp.async.bulk.tensor) instead of per-thread loads; tiles near
the edges keep the mapped loads.  ASTREA_TMA=0 turns the copies off for a grid,
so both paths can be compared: they must agree bit for bit (same arithmetic),
and the FP64 result must match the oracle to 1e-14.
"""

import os

import numpy as np
import pytest
import torch

from astrea_gb300.solver import RunConfig, Solver
from oracle import stepper

pytestmark = pytest.mark.gpu


def quadrants(n, seed=21):
    rng = np.random.default_rng(seed)
    w = np.zeros((n, n, 8))
    h = n // 2
    for sl in ((slice(0, h), slice(0, h)), (slice(0, h), slice(h, n)), (slice(h, n), slice(0, h)),
               (slice(h, n), slice(h, n))):
        w[sl + (0,)], w[sl + (4,)] = rng.uniform(.5, 2), rng.uniform(.5, 2)
        w[sl + (1,)], w[sl + (2,)] = rng.uniform(-.5, .5), rng.uniform(-.5, .5)
    return w


def run(cfg, w, steps, tma):
    old = os.environ.get("ASTREA_TMA")
    os.environ["ASTREA_TMA"] = "1" if tma else "0"
    try:
        s = Solver(cfg)
        s.initialise(w)
        s.reset_clock()
        s.step(steps, graph=True)
        torch.cuda.synchronize()
        assert s.clock()["status"] == 0
        return s.conservative().cpu().numpy()
    finally:
        if old is None:
            os.environ.pop("ASTREA_TMA", None)
        else:
            os.environ["ASTREA_TMA"] = old


def cfg_of(n, precision, scheme, solver, bc, dissipation=False):
    return RunConfig(dim=2, n0=n, n1=n, model=4, precision=precision, scheme=scheme, solver=solver,
                     integrator="ssprk33", boundary=bc, gamma=1.4, dx=1.0 / n, cfl=0.4, t_end=1.0, compat=False,
                     flatten=dissipation, viscosity=dissipation)


# PPM with flattening and viscosity also copies the viscous faces' state strip in bulk
@pytest.mark.parametrize("precision", [64, 32])
@pytest.mark.parametrize("scheme,solver,bc,dissipation", [("ppm", "hllc", "edge", False), ("plm", "llf", "wrap", False),
                                                          ("weno5", "hllc", "wrap", False),
                                                          ("ppm", "hllc", "wrap", True), ("ppm", "llf", "edge", True)])
def test_tma_equals_plain_loads(precision, scheme, solver, bc, dissipation):
    n = 128
    w = quadrants(n)
    a = run(cfg_of(n, precision, scheme, solver, bc, dissipation), w, 3, True)
    b = run(cfg_of(n, precision, scheme, solver, bc, dissipation), w, 3, False)
    assert np.array_equal(a, b)


def test_tma_fp64_matches_oracle():
    n = 128
    w = quadrants(n)
    got = run(cfg_of(n, 64, "ppm", "hllc", "edge"), w, 2, True)
    oc = stepper.OracleConfig(dim=2, scheme="ppm", solver="hllc", integrator="ssprk33", gamma=1.4, bc="edge",
                              dx=1.0 / n, cfl=0.4, eig="analytic", t_end=1.0, compat=False)
    q = stepper.initialise(w, oc)
    t, idx, order = 0.0, 1, [0, 1]
    with np.errstate(all="ignore"):
        for _ in range(2):
            q, t, idx, order, dt = stepper.step(q, oc, t, idx, order)
    assert float(np.max(np.abs(got - q)) / np.max(np.abs(q))) <= 1e-14
