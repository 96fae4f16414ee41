"""Batched engine: every grid of a batch evolves exactly as it does alone.

The batched persistent kernel runs the same tile code as the single-grid
kernel, so in FP64 the per-grid states must be identical bit for bit, and the
per-grid clocks (dt, t, step count) equal.
"""

import numpy as np
import pytest
import torch

from astrea_gb300.batch import Batch
from astrea_gb300.solver import Solver, RunConfig

pytestmark = pytest.mark.gpu


def quadrant(n, rng):
    w = np.zeros((n, n, 8))
    h = n // 2
    for (i0, i1) in [(0, h), (h, n)]:
        for (j0, j1) in [(0, h), (h, n)]:
            w[i0:i1, j0:j1, 0] = rng.uniform(.1, 2)
            w[i0:i1, j0:j1, 4] = rng.uniform(.1, 2)
            w[i0:i1, j0:j1, 1] = rng.uniform(-1, 1)
            w[i0:i1, j0:j1, 2] = rng.uniform(-1, 1)
    return w


def make_cfgs(precision, compat=False):
    combos = [(40, "plm", "llf"), (24, "ppm", "hllc"), (56, "weno5", "hllc"), (32, "ppm", "llf"), (20, "plm", "hllc")]
    return [RunConfig(dim=2, n0=n, n1=n, model=4, precision=precision, scheme=s, solver=v, integrator="ssprk33",
                      boundary="edge", gamma=1.4, dx=1.0 / n, cfl=0.8, t_end=0.25, compat=compat)
            for n, s, v in combos]


@pytest.mark.parametrize("graph", [False, True])
def test_batch_equals_alone_fp64(graph):
    rng = np.random.default_rng(3)
    cfgs = make_cfgs(64)
    ws = [quadrant(c.n0, rng) for c in cfgs]
    b = Batch(cfgs)
    b.initialise(ws)
    b.step(5, graph=graph)
    clk = b.clocks()
    for g, (c, w) in enumerate(zip(cfgs, ws)):
        s = Solver(c)
        s.initialise(w)
        s.reset_clock()
        s.step(5)
        assert torch.equal(b.planes(g), s.state), g
        sc = s.clock()
        assert sc["t"] == clk["t"][g] and sc["steps"] == clk["steps"][g]


def test_batch_1d_mixed_sizes_equals_alone():
    rng = np.random.default_rng(4)
    cfgs = []
    ws = []
    for n, sch, sol in [(64, "plm", "llf"), (200, "ppm", "hllc"), (33, "weno5", "llf")]:
        cfgs.append(RunConfig(dim=1, n0=n, model=3, precision=64, scheme=sch, solver=sol, integrator="ssprk33",
                              boundary="edge", gamma=1.4, dx=1.0 / n, cfl=0.8, t_end=0.2))
        w = np.zeros((n, 8))
        w[: n // 2] = [rng.uniform(.1, 2), rng.uniform(-1, 1), 0, 0, rng.uniform(.1, 2), 0, 0, 0]
        w[n // 2:] = [rng.uniform(.1, 2), rng.uniform(-1, 1), 0, 0, rng.uniform(.1, 2), 0, 0, 0]
        ws.append(w)
    b = Batch(cfgs)
    b.initialise(ws)
    b.step(6)
    for g, (c, w) in enumerate(zip(cfgs, ws)):
        s = Solver(c)
        s.initialise(w)
        s.reset_clock()
        s.step(6)
        assert torch.equal(b.planes(g), s.state), g


def test_batch_runs_each_grid_to_its_own_end_time():
    # CFL 0.4: at 0.8 the unsplit 2D update loses positivity on some of these random
    # quadrant problems (the FP64 oracle goes non-finite on the PPM+LLF grid as well)
    rng = np.random.default_rng(5)
    cfgs = make_cfgs(32)
    for i, c in enumerate(cfgs):
        c.t_end = 0.01 * (i + 1)
        c.cfl = 0.4
    b = Batch(cfgs)
    b.initialise([quadrant(c.n0, rng) for c in cfgs])
    clk = b.run()
    assert clk["done"].all()
    for g, c in enumerate(cfgs):
        assert clk["t"][g] == pytest.approx(c.t_end, rel=1e-6)


def test_slots_can_be_released_and_refilled_between_steps():
    from astrea_gb300.batch import SlotBatch
    rng = np.random.default_rng(6)
    cfgs = make_cfgs(64)[:3]
    sizes = [4 * c.n0 * c.n1 for c in cfgs]
    sb = SlotBatch(2, 4, 64, "ssprk33", max_slots=4, capacity_elems=sum(sizes) + 4 * 64 * 64)
    ws = [quadrant(c.n0, rng) for c in cfgs]
    sb.occupy(0, cfgs[0], 0, ws[0])
    sb.occupy(1, cfgs[1], sizes[0], ws[1])
    sb.step(2)
    sb.release(0)
    sb.occupy(2, cfgs[2], sizes[0] + sizes[1], ws[2])
    sb.step(3)
    clk = sb.clocks()
    assert clk["steps"][1] == 5 and clk["steps"][2] == 3
    for slot, w, c, k in [(1, ws[1], cfgs[1], 5), (2, ws[2], cfgs[2], 3)]:
        s = Solver(c)
        s.initialise(w)
        s.reset_clock()
        s.step(k)
        assert torch.equal(sb.planes(slot), s.state)


def test_batch_non_square_periodic_and_outflow_fp64_equals_alone():
    # non-square grids of every method class, periodic and outflow, through the batched
    # cell-average pre-pass (one warp per strip) and the single-grid one (bulk copies where
    # the rows are whole 16-byte units, mapped loads elsewhere): bit for bit
    rng = np.random.default_rng(9)
    shapes = [((40, 56), "ppm", "hllc", "wrap"), ((72, 24), "weno5", "llf", "wrap"), ((30, 50), "plm", "hllc", "edge"),
              ((50, 34), "ppm", "llf", "edge"), ((33, 45), "weno5", "hllc", "edge")]
    cfgs, ws = [], []
    for (n0, n1), sch, sol, bc in shapes:
        cfgs.append(RunConfig(dim=2, n0=n0, n1=n1, model=4, precision=64, scheme=sch, solver=sol,
                              integrator="ssprk33", boundary=bc, gamma=1.4, dx=1.0 / n1, cfl=0.4, t_end=0.25,
                              compat=False))
        x, y = (np.arange(n0) + .5) / n0, (np.arange(n1) + .5) / n1
        X, Y = np.meshgrid(x, y, indexing="ij")
        w = np.zeros((n0, n1, 8))
        w[..., 0] = 1 + .3 * np.sin(2 * np.pi * X) * np.cos(2 * np.pi * Y) + rng.uniform(0, .05)
        w[..., 1] = .4 * np.sin(2 * np.pi * Y)
        w[..., 2] = -.3 * np.cos(2 * np.pi * X)
        w[..., 4] = 1 + .2 * np.cos(2 * np.pi * (X + Y))
        ws.append(w)
    b = Batch(cfgs)
    b.initialise(ws)
    b.step(5)
    clk = b.clocks()
    for g, (c, w) in enumerate(zip(cfgs, ws)):
        s = Solver(c)
        s.initialise(w)
        s.reset_clock()
        s.step(5)
        assert torch.equal(b.planes(g), s.state), g
        assert s.clock()["t"] == clk["t"][g]
