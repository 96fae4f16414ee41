"""Device-built initial conditions against the reference's constructor.initialise.

The golden file holds, for 20 (config, dimension, cells) cases, the grid the
reference's initialise returns (point primitives from its own test table, then
its centre -> average step), together with the table values it used.  The
device builder (astrea_point_state) must reproduce the point primitives from
those values; the oracle's centre -> average step then gives the reference's
grid.  The expressions are the same, so the only differences are last-bit ones
of sin/exp/pow (bar: 1e-14 of the grid's largest magnitude).
"""

import os
from types import SimpleNamespace

import numpy as np
import pytest
import torch

from astrea_gb300 import initial
from astrea_gb300.solver import RunConfig, Solver
from oracle import fvcore

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "initial_conditions.npz")


def cases():
    g = np.load(GOLDEN)
    n = len([k for k in g.files if k.endswith("_config")])
    out = []
    for i in range(n):
        k = f"c{i}_"
        misc = {f[len(k) + 5:]: (g[f] if g[f].ndim else float(g[f])) for f in g.files if f.startswith(k + "misc_")}
        sv = SimpleNamespace(config=str(g[k + "config"]), dimension=int(g[k + "dim"]), cells=int(g[k + "cells"]),
                             gamma=float(g[k + "gamma"]), start_pos=float(g[k + "start_pos"]),
                             end_pos=float(g[k + "end_pos"]), shock_pos=float(g[k + "shock_pos"]),
                             initial_left=g[k + "initial_left"], initial_right=g[k + "initial_right"],
                             misc=misc or None, boundary=str(g[k + "boundary"]))
        out.append((sv, g[k + "w"]))
    return out


CASES = cases()


@pytest.mark.parametrize("idx", range(len(CASES)), ids=[f"{c[0].config}-{c[0].dimension}d" for c in CASES])
def test_point_primitives_match_reference(idx):
    sv, ref = CASES[idx]
    point = initial.point_primitives(sv, model=8, precision=64).cpu().numpy()
    got = fvcore.centre_to_avg(point, sv.boundary, list(range(sv.dimension)))
    assert got.shape == ref.shape
    scale = max(np.max(np.abs(ref)), 1e-300)
    assert np.max(np.abs(got - ref)) <= 1e-14 * scale, (sv.config, np.max(np.abs(got - ref)))


def test_device_initialise_equals_host_upload():
    sv, ref = next(c for c in CASES if c[0].config == "orszag-tang")
    n = sv.cells
    cfg = RunConfig(dim=2, n0=n, n1=n, model=8, precision=64, scheme="weno5", solver="hlld", boundary="wrap",
                    gamma=sv.gamma, dx=1.0 / n, cfl=0.4, t_end=0.5, compat=False)
    a, b = Solver(cfg), Solver(cfg)
    initial.initialise(a, sv)
    b.initialise(initial.point_primitives(sv, model=8, precision=64).cpu().numpy())
    torch.cuda.synchronize()
    x, y = a.state.cpu().numpy(), b.state.cpu().numpy()
    assert np.max(np.abs(x - y)) <= 1e-14 * np.max(np.abs(y))
