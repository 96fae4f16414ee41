"""Properties of the oracle's 2D update that hold without reference vectors:
mirror symmetry (the published solvers label axes physically) and exact
conservation on a periodic grid (flux-difference form)."""

import numpy as np
import pytest

from oracle import stepper


def symmetric_state(n):
    x = (np.arange(n) + .5) / n
    X, Y = np.meshgrid(x, x, indexing="ij")
    r2 = (X - .5) ** 2 + (Y - .5) ** 2
    q = np.zeros((n, n, 8))
    rho = 1 + .5 * np.exp(-r2 / .01)
    vx, vy = .2 * (X - .5) * np.exp(-r2 / .02), .2 * (Y - .5) * np.exp(-r2 / .02)
    p = 1 + 4 * np.exp(-r2 / .005)
    q[..., 0], q[..., 1], q[..., 2] = rho, rho * vx, rho * vy
    q[..., 4] = p / .4 + .5 * rho * (vx ** 2 + vy ** 2)
    return q


@pytest.mark.parametrize("scheme,solver,dissipation", [("ppm", "hllc", True), ("weno5", "llf", False),
                                                       ("plm", "hllc", False)])
def test_update_keeps_mirror_symmetry(scheme, solver, dissipation):
    n = 32
    q = symmetric_state(n)
    assert np.array_equal(q[..., 0], q[..., 0].T) and np.array_equal(q[..., 1], q[..., 2].T)
    cfg = stepper.OracleConfig(dim=2, scheme=scheme, solver=solver, integrator="ssprk33", gamma=1.4, bc="wrap",
                               dx=1.0 / n, cfl=.8, eig="analytic", t_end=1.0, compat=False, flatten=dissipation,
                               viscosity=dissipation)
    t, idx, order = 0.0, 1, [0, 1]
    with np.errstate(all="ignore"):
        for _ in range(3):
            q, t, idx, order, dt = stepper.step(q, cfg, t, idx, order)
    assert np.isfinite(q).all()
    assert np.array_equal(q[..., 0], q[..., 0].T)
    assert np.array_equal(q[..., 1], q[..., 2].T)
    assert np.array_equal(q[..., 4], q[..., 4].T)


def test_periodic_update_conserves():
    n = 32
    q = symmetric_state(n)
    cfg = stepper.OracleConfig(dim=2, scheme="ppm", solver="hllc", integrator="ssprk33", gamma=1.4, bc="wrap",
                               dx=1.0 / n, cfl=.8, eig="analytic", t_end=1.0, compat=False, flatten=True,
                               viscosity=True)
    before = q.sum(axis=(0, 1))
    t, idx, order = 0.0, 1, [0, 1]
    with np.errstate(all="ignore"):
        for _ in range(3):
            q, t, idx, order, dt = stepper.step(q, cfg, t, idx, order)
    after = q.sum(axis=(0, 1))
    for k in (0, 1, 2, 4):
        assert abs(after[k] - before[k]) <= 1e-12 * max(1.0, abs(before[k])), k
