"""Sweep-tile autotuner: every candidate tile gives the same update, and the tuner picks a built one.

2D FP32 Euler grids have two tile candidates (32 x 8 cells with 256 threads,
32 x 15 with 512); the engine times both on the grid at its first step.  The
tile only changes which CTA computes a cell, not the cell's formulas.  In FP32
the two instantiations may contract multiply-adds differently, and a rounding
difference can flip a limiter branch near a discontinuity, so the bar is
statistical: mean difference <= 1e-6 and largest difference <= 1e-4 of the
largest magnitude.
"""

import os

import numpy as np
import pytest
import torch

from astrea_gb300.solver import RunConfig, Solver

pytestmark = pytest.mark.gpu


def close(x, y):
    scale = np.max(np.abs(x))
    d = np.abs(x - y)
    return float(np.mean(d)) <= 1e-6 * scale and float(np.max(d)) <= 1e-4 * scale


def shear(n, seed=4):
    rng = np.random.default_rng(seed)
    x = (np.arange(n) + .5) / n
    X, Y = np.meshgrid(x, x, indexing="ij")
    w = np.zeros((n, n, 8))
    inner = np.abs(Y - .5) < .25
    w[..., 0] = np.where(inner, 2.0, 1.0)
    w[..., 1] = np.where(inner, .5, -.5)
    w[..., 2] = .01 * np.sin(4 * np.pi * X) + rng.uniform(-1e-3, 1e-3, size=(n, n))
    w[..., 4] = 2.5
    return w


def run(n, precision, tile, boundary="wrap", steps=6):
    old = os.environ.get("ASTREA_SWEEP_TILE")
    if tile is None:
        os.environ.pop("ASTREA_SWEEP_TILE", None)
    else:
        os.environ["ASTREA_SWEEP_TILE"] = str(tile)
    try:
        s = Solver(RunConfig(dim=2, n0=n, n1=n, model=4, precision=precision, scheme="ppm", solver="hllc",
                             integrator="ssprk33", boundary=boundary, gamma=1.4, dx=1.0 / n, cfl=0.8, t_end=1.0,
                             compat=False, flatten=True, viscosity=True))
        s.initialise(shear(n))
        s.reset_clock()
        s.step(steps, graph=True)
        torch.cuda.synchronize()
        return s.state.double().cpu().numpy(), s.sweep_tiles()
    finally:
        if old is None:
            os.environ.pop("ASTREA_SWEEP_TILE", None)
        else:
            os.environ["ASTREA_SWEEP_TILE"] = old


@pytest.mark.parametrize("boundary", ["wrap", "edge"])
def test_both_tiles_give_the_same_update(boundary):
    a, ta = run(96, 32, 0, boundary)
    b, tb = run(96, 32, 1, boundary)
    assert ta == [(32, 8), (32, 8)] and tb == [(32, 15), (32, 15)]
    assert close(a, b)


def test_tile_forced_per_axis():
    # ASTREA_SWEEP_TILE=<axis 0>,<axis 1>: the mix the tuner may pick gives the same update
    a, ta = run(96, 32, 0)
    b, tb = run(96, 32, "1,0")
    assert tb == [(32, 15), (32, 8)]
    assert close(a, b)


def test_tuner_picks_a_built_tile():
    _, t32 = run(256, 32, None)
    assert all(t in [(32, 8), (32, 15)] for t in t32)
    _, t64 = run(64, 64, None)
    assert t64 == [(32, 8), (32, 8)]  # FP64 builds one 2D tile


def run_batch(tile, steps=5):
    from astrea_gb300.batch import Batch
    old = os.environ.get("ASTREA_BATCH_TILE")
    if tile is None:
        os.environ.pop("ASTREA_BATCH_TILE", None)
    else:
        os.environ["ASTREA_BATCH_TILE"] = str(tile)
    try:
        sizes = [64, 96, 40, 128]
        cfgs = [RunConfig(dim=2, n0=n, n1=n, model=4, precision=32, scheme=s, solver=v, integrator="ssprk33",
                          boundary="edge", gamma=1.4, dx=1.0 / n, cfl=0.4, t_end=1.0, compat=False)
                for n, (s, v) in zip(sizes, [("ppm", "hllc"), ("plm", "llf"), ("weno5", "hllc"), ("ppm", "llf")])]
        b = Batch(cfgs)
        b.initialise([shear(c.n0) for c in cfgs])
        b.step(steps, graph=True)
        torch.cuda.synchronize()
        return [b.planes(g).double().cpu().numpy() for g in range(len(cfgs))], b.tiles()
    finally:
        if old is None:
            os.environ.pop("ASTREA_BATCH_TILE", None)
        else:
            os.environ["ASTREA_BATCH_TILE"] = old


def test_batch_tiles_give_the_same_update():
    a, ta = run_batch(0)
    b, tb = run_batch(1)
    assert ta == [(32, 8), (32, 8)] and tb == [(32, 15), (32, 15)]
    for x, y in zip(a, b):
        assert close(x, y)
    _, tauto = run_batch(None)
    assert all(t in [(32, 8), (32, 15)] for t in tauto)
