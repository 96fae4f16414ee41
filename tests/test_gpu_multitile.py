"""The default (reference-compatible) method on grids of several sweep tiles, against the reference.

The golden cases ``mt*`` (tests/golden/make_golden.py:multitile_cases) are
96^2 hydro grids (edge and wrap: PPM+HLLC, WENO5+HLLC, PLM+LLF, WENO5+LLF)
and 64^2 constrained-transport MHD grids (PPM, WENO5 + HLLD) run by the
reference's own evolve_space / evolve_time.  With sweep tiles of 32 cells
along the sweep and 8 or 15 rows across, these grids have interior tiles
(unclamped, shared-stencil PPM strips, bulk-copied staging boxes), tile
seams along and across the sweep, and ragged last tiles, besides the clamped
edge tiles.  Each case runs with every tile candidate, with the bulk copies on
and off, and must match the reference's grid after every step to 1e-12 and
the oracle's to 1e-14 (reference-compatible HLLC/HLLD: the reference's axis
label, star momentum component and upwind choice).
"""

import os

import numpy as np
import pytest

from astrea_gb300 import config as C
from astrea_gb300.solver import Solver, RunConfig, pick_model
from oracle import stepper
from tests import golden_io

pytestmark = pytest.mark.gpu

MT = [n for n in golden_io.case_names() if n.startswith("mt")]


def rel_err(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def configs(meta, q0):
    oc = stepper.OracleConfig(
        dim=2, scheme=C.scheme_of(meta["subgrid"]), solver=C.solver_of(meta["solver"]),
        integrator=C.integrator_of(meta["timestep"]), gamma=meta["gamma"], bc=meta["boundary"], dx=meta["dx"],
        cfl=meta["cfl"], magnetic_2d=meta["magnetic_2d"], eig="analytic", t_end=meta["t_end"])
    n = meta["cells"]
    model = 8 if meta["magnetic_2d"] else pick_model(2, oc.solver, q0)
    gc = RunConfig(dim=2, n0=n, n1=n, model=model, precision=64, scheme=oc.scheme, solver=oc.solver,
                   integrator=oc.integrator, boundary=oc.bc, gamma=oc.gamma, dx=oc.dx, cfl=oc.cfl, t_end=oc.t_end,
                   magnetic_2d=meta["magnetic_2d"])
    return gc, oc


@pytest.fixture(scope="module")
def oracle_runs():
    """The oracle's grid after every step of each case (computed once per case)."""
    cache = {}

    def get(name):
        if name not in cache:
            g = golden_io.load(name)
            _, oc = configs(g["meta"], g["q0"])
            q, t, idx, order, out = g["q0"], 0.0, 1, [0, 1], []
            with np.errstate(all="ignore"):
                for _ in range(g["meta"]["steps"]):
                    q, t, idx, order, _dt = stepper.step(q, oc, t, idx, order)
                    out.append(q)
            cache[name] = out
        return cache[name]
    return get


@pytest.mark.parametrize("tma", [1, 0])
@pytest.mark.parametrize("tile", [0, 1])
@pytest.mark.parametrize("name", MT)
def test_multitile_steps_match_reference(name, tile, tma, oracle_runs, monkeypatch):
    monkeypatch.setenv("ASTREA_SWEEP_TILE", str(tile))
    monkeypatch.setenv("ASTREA_TMA", str(tma))
    g = golden_io.load(name)
    meta = g["meta"]
    gc, _ = configs(meta, g["q0"])
    s = Solver(gc)
    s.load_conservative(g["q0"])
    s.reset_clock(0.0, 1, 0)
    want = oracle_runs(name)
    for k in range(meta["steps"]):
        s.step(1, graph=False)
        q = s.conservative().cpu().numpy()
        assert s.clock()["status"] == 0
        assert rel_err(q, want[k]) <= 1e-14, (name, k, rel_err(q, want[k]))
        assert rel_err(q, g[f"q_{k + 1}"]) <= 1e-12, (name, k, rel_err(q, g[f"q_{k + 1}"]))
    ts = s.sweep_tiles()
    assert ts[0] == ts[1] and ts[0][1] in (8, 15)  # the forced candidate ran on both axes
