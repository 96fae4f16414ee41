"""The server's loop on the host with a stand-in batch (no GPU): admission under
the memory budget, completion and latency accounting, retirement of stalled
requests, and polls sized to land on completions."""

import contextlib
import math

import numpy as np
import pytest
import torch

from astrea_gb300 import serving
from astrea_gb300.serving import Server, make_requests


class FakeSlotBatch:
    """A slot batch whose grids advance by a fixed dt per step (t_end / 10, or a collapsed dt)."""

    instances = []

    def __init__(self, dim, model, precision, integrator, max_slots, capacity, device):
        self.max_slots = max_slots
        self.capacity = capacity
        self.slot = {}
        self.polls = []
        FakeSlotBatch.instances.append(self)

    def occupy_ic(self, slot, cfg, offset, ic):
        assert slot not in self.slot and 0 <= offset and offset + cfg.model * cfg.n0 * cfg.n1 <= self.capacity
        collapsed = cfg.cfl < 0.01  # the test marks stalling requests by a tiny CFL number
        self.slot[slot] = {"t": 0.0, "dt": (1e-9 if collapsed else cfg.t_end / 10), "steps": 0, "t_end": cfg.t_end,
                           "off": offset, "size": cfg.model * cfg.n0 * cfg.n1}

    def step(self, n=1, graph=False):
        self.polls.append(n)
        for s in self.slot.values():
            for _ in range(n):
                if s["t"] >= s["t_end"]:
                    break
                # the device clock clips the last step onto t_end (astrea.py:74-78)
                s["t"] = s["t_end"] if s["t"] + s["dt"] >= s["t_end"] * (1 - 1e-12) else s["t"] + s["dt"]
                s["steps"] += 1

    def clocks(self):
        g = self.max_slots
        out = {"t": np.zeros(g), "dt": np.zeros(g), "steps": np.zeros(g, dtype=np.int64),
               "done": np.zeros(g, dtype=bool), "status": np.zeros(g, dtype=np.int64)}
        for k, s in self.slot.items():
            out["t"][k], out["dt"][k], out["steps"][k] = s["t"], s["dt"], s["steps"]
            out["done"][k] = s["t"] >= s["t_end"]
        return out

    def release(self, slot):
        self.slot.pop(slot)

    def planes(self, slot):
        return torch.zeros(1)


@pytest.fixture
def fake_device(monkeypatch):
    FakeSlotBatch.instances = []
    monkeypatch.setattr(serving, "SlotBatch", FakeSlotBatch)
    monkeypatch.setattr(torch.cuda, "Stream", lambda *a, **k: None)
    monkeypatch.setattr(torch.cuda, "stream", lambda s: contextlib.nullcontext())
    monkeypatch.setattr(torch.cuda, "synchronize", lambda *a, **k: None)
    yield


def test_every_request_completes_within_the_budget(fake_device):
    reqs = make_requests(40, rate=1e9, seed=3, n1d=(64, 256), n2d=(16, 64), t_end=(.05, .1))
    budget = 4e6
    srv = Server(hbm_budget_bytes=budget, precision=32, max_slots=4, steps_per_poll=2)
    caps = {cls: srv.arenas[cls].capacity for cls in srv.classes}
    stats = srv.serve(reqs, realtime=False)
    assert len(stats.latencies_ms) == len(reqs) and stats.failed == 0 and not stats.unfinished
    assert stats.max_active <= 4 * len(srv.classes)
    for r in reqs:
        assert r.steps == 10 and r.finished >= r.admitted >= 0 and r.status == 0
    # arena budgets: a class holds at most its capacity at any time (checked at occupation) and
    # its arena is whole again at the end
    for cls in srv.classes:
        assert srv.arenas[cls].free == [(0, caps[cls])]


def test_stalled_requests_are_retired(fake_device):
    reqs = make_requests(6, rate=1e9, seed=4, n1d=(64, 64), n2d=(16, 16), t_end=(.05, .06))
    for r in reqs[::2]:
        r.cfl = 1e-3  # the stand-in batch gives these a collapsed time step
    srv = Server(hbm_budget_bytes=4e6, precision=32, max_slots=8, steps_per_poll=4, max_steps=2000)
    stats = srv.serve(reqs, realtime=False)
    assert stats.stalled == 3 and stats.failed == 3
    for k, r in enumerate(reqs):
        if k % 2 == 0:
            assert r.status & 4 and 1000 <= r.steps <= 1000 + 32  # judged once past the check point
        else:
            assert r.status == 0 and r.steps == 10


def test_polls_land_on_completions(fake_device):
    reqs = make_requests(3, rate=1e9, seed=5, n1d=(64, 64), n2d=(16, 16), frac_1d=1.0, frac_mhd=0.0,
                         t_end=(.05, .1))
    srv = Server(hbm_budget_bytes=4e6, precision=32, max_slots=8, steps_per_poll=3)
    srv.serve(reqs, realtime=False)
    fb = [b for b in FakeSlotBatch.instances if b.polls]
    assert len(fb) == 1
    polls = fb[0].polls
    # the first poll of new requests takes steps_per_poll; then each poll covers the steps the
    # nearest request still needs (10 per request here), so the polls add up to 10 exactly
    assert polls[0] == 3 and sum(polls) == 10 and max(polls) <= 32
