"""Size-independent properties at the benchmark's full size (2048^2), where the
oracle would take hours: mirror symmetry of the FP64 update, and conservation
of the FP32 headline update on a periodic grid."""

import numpy as np
import pytest
import torch

from astrea_gb300.solver import RunConfig, Solver

pytestmark = pytest.mark.gpu

N = 2048


def blast(n):
    """A transpose-symmetric state: a pressure bump and a radial flow about the centre."""
    x = (np.arange(n) + .5) / n
    X, Y = np.meshgrid(x, x, indexing="ij")
    r2 = (X - .5) ** 2 + (Y - .5) ** 2
    w = np.zeros((n, n, 8))
    w[..., 0] = 1 + .5 * np.exp(-r2 / .01)
    w[..., 1] = .2 * (X - .5) * np.exp(-r2 / .02)
    w[..., 2] = .2 * (Y - .5) * np.exp(-r2 / .02)
    w[..., 4] = 1 + 4 * np.exp(-r2 / .005)
    return w


@pytest.mark.parametrize("scheme,solver,dissipation", [("ppm", "hllc", True), ("weno5", "llf", False)])
def test_fp64_update_keeps_mirror_symmetry_at_full_size(scheme, solver, dissipation):
    # the published solvers label the axes physically, so the update of a state symmetric under
    # x <-> y (with v_x <-> v_y) is symmetric bit for bit: both sweeps compute the same expressions
    # in mirror image and their divergences are added commutatively
    cfg = RunConfig(dim=2, n0=N, n1=N, model=4, precision=64, scheme=scheme, solver=solver, integrator="ssprk33",
                    boundary="wrap", gamma=1.4, dx=1.0 / N, cfl=0.8, t_end=1.0, compat=False, flatten=dissipation,
                    viscosity=dissipation)
    w = blast(N)
    # conservative state loaded as is (the centre -> average conversion of ``initialise`` adds
    # the two axes' corrections in a fixed order, which is not mirror-symmetric in the last bit)
    q0 = np.zeros_like(w)
    q0[..., 0] = w[..., 0]
    q0[..., 1] = w[..., 0] * w[..., 1]
    q0[..., 2] = w[..., 0] * w[..., 2]
    q0[..., 4] = w[..., 4] / .4 + .5 * w[..., 0] * (w[..., 1] ** 2 + w[..., 2] ** 2)
    assert np.array_equal(q0[..., 0], q0[..., 0].T) and np.array_equal(q0[..., 1], q0[..., 2].T)
    assert np.array_equal(q0[..., 4], q0[..., 4].T)
    s = Solver(cfg)
    s.load_conservative(q0)
    s.reset_clock()
    q = s.state
    assert torch.equal(q[0], q[0].T) and torch.equal(q[1], q[2].T)
    s.step(3)
    assert s.clock()["status"] == 0
    q = s.state  # planes rho, m_x, m_y, E
    assert torch.equal(q[0], q[0].T)
    assert torch.equal(q[1], q[2].T)
    assert torch.equal(q[3], q[3].T)
    del s
    torch.cuda.empty_cache()


def test_fp32_headline_conserves_at_full_size():
    cfg = RunConfig(dim=2, n0=N, n1=N, model=4, precision=32, scheme="ppm", solver="hllc", integrator="ssprk33",
                    boundary="wrap", gamma=1.4, dx=1.0 / N, cfl=0.8, t_end=1.0, compat=False, flatten=True,
                    viscosity=True)
    rng = np.random.default_rng(20261203)
    x = (np.arange(N) + .5) / N
    X, Y = np.meshgrid(x, x, indexing="ij")
    w = np.zeros((N, N, 8))
    inner = np.abs(Y - .5) < .25
    w[..., 0] = np.where(inner, 2.0, 1.0)
    w[..., 1] = np.where(inner, .5, -.5)
    w[..., 2] = .01 * np.sin(4 * np.pi * X) + rng.uniform(-1e-3, 1e-3, size=(N, N))
    w[..., 4] = 2.5
    s = Solver(cfg)
    s.initialise(w)
    s.reset_clock()
    before = s.conserved_sums()
    s.step(10)
    after = s.conserved_sums()
    assert s.clock()["status"] == 0
    # mass and energy telescope up to FP32 rounding of the per-cell updates
    for k in (0, 3):
        assert abs(after[k] - before[k]) <= 1e-6 * abs(before[k]), (k, before[k], after[k])
    del s
    torch.cuda.empty_cache()


def test_fp64_headline_workload_matches_oracle_at_full_size():
    """The bench's own workload (shear layer 2048^2, PPM + flattening + viscosity, textbook HLLC,
    SSPRK3, CFL 0.8) in FP64 against the oracle's first two steps (tests/golden/fullsize_shear2048.npz,
    made by make_fullsize_golden.py): dt bit for bit in value to 1e-15, the full rows and columns at
    the tile seams and shear interfaces to 1e-14 of each variable's largest magnitude, and the
    compensated plane sums against the correctly rounded sums."""
    import bench
    from tests.golden_io import GOLDEN
    import json
    import os
    with np.load(os.path.join(GOLDEN, "fullsize_shear2048.npz")) as z:
        g = {k: z[k] for k in z.files}
    meta = json.loads(str(g["meta"]))
    s = Solver(bench.run_config(N, 64))
    s.initialise(bench.shear_layer(N))
    s.reset_clock()
    for k in range(1, meta["steps"] + 1):
        s.step(1, graph=False)
        clk = s.clock()
        assert clk["status"] == 0
        assert clk["dt"] == pytest.approx(float(g[f"dt_{k}"]), rel=1e-15, abs=0)
        q = s.state  # planes rho, m_x, m_y, E == reference variables 0, 1, 2, 4
        scale = g[f"absmax_{k}"]
        rows = q[:, meta["rows"], :].permute(1, 2, 0).cpu().numpy()
        cols = q[:, :, meta["cols"]].permute(1, 2, 0).cpu().numpy()
        assert np.max(np.abs(rows - g[f"rows_{k}"]) / scale) <= 1e-14
        assert np.max(np.abs(cols - g[f"cols_{k}"]) / scale) <= 1e-14
        sums = s.conserved_sums()
        assert np.all(np.abs(sums - g[f"sums_{k}"]) <= 1e-13 * scale * N * N)
    del s
    torch.cuda.empty_cache()

