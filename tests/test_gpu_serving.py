"""Serving: continuous batching gives every request the result it gets alone.

A small mixed stream (1D/2D, Euler/MHD, PLM/PPM/WENO5 x LLF/HLLC/HLLD) is
served with arrivals spread over time so that requests join and leave the
batches while others are running; each finished state is compared with the
same request solved alone by the single-grid solver.  Both paths run the same
tile code and take the 2D high-order cell averages from a pre-pass (the
single-grid one per grid, the batched one over the strips of every grid of a
batch), but they are separate FP32 builds that contract multiply-adds
differently and stage through different paths, so the bar is FP32 rounding,
not bit equality: mean difference <= 1e-6 and largest <= 1e-4 of the state's
scale (in FP64 the two paths agree bit for bit, test_gpu_batch.py).
"""

import numpy as np
import pytest
import torch

from astrea_gb300.serving import Server, arena_copies, make_requests
from astrea_gb300.solver import Solver

pytestmark = pytest.mark.gpu


def test_mix_equals_alone():
    reqs = make_requests(14, rate=400.0, seed=11, n1d=(64, 512), n2d=(16, 64), t_end=(0.02, 0.06))
    for r in reqs:
        r.cfl = 0.4
    srv = Server(hbm_budget_bytes=2e8, precision=32, max_slots=8, keep_results=True, steps_per_poll=2)
    stats = srv.serve(reqs)
    assert len(stats.latencies_ms) == len(reqs)
    assert stats.max_active > 1
    for r in reqs:
        s = Solver(r.config(32))
        s.initialise(r.initial_state())
        s.reset_clock()
        clk = s.run()
        assert clk["steps"] == r.steps, r
        assert bool(clk["status"]) == bool(r.status), r
        a, b = r.result.double(), s.state.double()
        # some random MHD Riemann problems lose positivity (the FP64 oracle goes
        # non-finite on them too): the non-finite pattern must match as well
        fa, fb = torch.isfinite(a), torch.isfinite(b)
        assert torch.equal(fa, fb), r
        if fb.any():
            scale = float(torch.max(torch.abs(b[fb])))
            d = torch.abs(a[fb] - b[fb])
            assert float(torch.mean(d)) <= 1e-6 * scale and float(torch.max(d)) <= 1e-4 * scale, \
                (r, float(torch.max(d)) / scale)


def test_admission_respects_the_memory_budget():
    reqs = make_requests(6, rate=1e6, seed=12, n1d=(64, 128), n2d=(128, 128), frac_1d=0.0, frac_mhd=0.0,
                         t_end=(0.01, 0.02))
    # room for exactly two 128^2 Euler grids in the (2, 4) class
    srv = Server(hbm_budget_bytes=arena_copies(2, 32) * 4 * 4 * 128 * 128 * 2 / 0.5, precision=32, max_slots=8,
                 shares={(1, 3): 0, (1, 8): 0, (2, 4): .5, (2, 8): .5}, steps_per_poll=1)
    stats = srv.serve(reqs, realtime=False)
    assert len(stats.latencies_ms) == len(reqs)
    assert stats.max_active <= 2
