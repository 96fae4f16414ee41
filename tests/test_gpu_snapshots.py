"""Snapshots written while the GPU keeps stepping equal the step-by-step
snapshots of the same run (the reference's loop, astrea.py:44-84: the
primitive grid before every step and at t_end, named str(float(t)))."""

import numpy as np
import pytest
import torch

from astrea_gb300 import snapshots
from astrea_gb300.solver import RunConfig, Solver

pytestmark = pytest.mark.gpu


def sod(n):
    x = (np.arange(n) + .5) / n
    w = np.zeros((n, 8))
    w[:, 0] = np.where(x <= .5, 1.0, .125)
    w[:, 4] = np.where(x <= .5, 1.0, .1)
    return w


def quadrants(n, seed=3):
    rng = np.random.default_rng(seed)
    w = np.zeros((n, n, 8))
    h = n // 2
    for sl in ((slice(0, h), slice(0, h)), (slice(0, h), slice(h, n)), (slice(h, n), slice(0, h)),
               (slice(h, n), slice(h, n))):
        w[sl + (0,)], w[sl + (4,)] = rng.uniform(.5, 2), rng.uniform(.5, 2)
        w[sl + (1,)], w[sl + (2,)] = rng.uniform(-.5, .5), rng.uniform(-.5, .5)
    return w


def stepwise(cfg, w, every):
    """The reference loop: snapshot, then step, until t reaches t_end (every ``every`` steps)."""
    s = Solver(cfg)
    s.initialise(w)
    s.reset_clock()
    out = []
    while True:
        c = s.clock()
        out.append((c["t"], s.primitive().cpu().numpy()))
        if c["t"] >= cfg.t_end or c["done"]:
            return out
        s.step(every, graph=False)


@pytest.mark.parametrize("case", ["sod_fp64_every1", "quadrants_fp32_every3"])
def test_overlapped_snapshots_equal_stepwise(case, tmp_path):
    if case == "sod_fp64_every1":
        n, every = 256, 1
        cfg = RunConfig(dim=1, n0=n, model=3, precision=64, scheme="plm", solver="llf", integrator="ssprk33",
                        boundary="edge", gamma=1.4, dx=1.0 / n, cfl=.8, t_end=.02)
        w = sod(n)
    else:
        n, every = 48, 3
        cfg = RunConfig(dim=2, n0=n, n1=n, model=4, precision=32, scheme="ppm", solver="hllc", integrator="ssprk33",
                        boundary="edge", gamma=1.4, dx=1.0 / n, cfl=.4, t_end=.03, compat=False)
        w = quadrants(n)
    ref = stepwise(cfg, w, every)
    s = Solver(cfg)
    s.initialise(w)
    s.reset_clock()
    store = snapshots.DirectoryStore(str(tmp_path / "run.d"), snapshots.new_file_attrs(seed=1))
    written = snapshots.run_with_snapshots(s, store, "run0", every=every, graph=True)
    run = snapshots.read_directory_run(str(tmp_path / "run.d"), "run0")
    assert len(run) == len(ref) == len(written) >= 3
    assert run[-1][1]["t"] == cfg.t_end
    for (name, attrs, arr), (t, snap) in zip(run, ref):
        assert name == str(float(t)) and attrs["t"] == t
        assert np.array_equal(arr, snap)
    torch.cuda.synchronize()
