"""Snapshot stores on the host: the directory form of the reference's HDF5 layout."""

import json
import os

import numpy as np
import pytest

from astrea_gb300 import snapshots
from astrea_gb300.solver import RunConfig


def test_directory_store_round_trip(tmp_path):
    st = snapshots.DirectoryStore(str(tmp_path / "run.d"), {"datetime": "2026-01-01 00:00:00", "seed": 7})
    cfg = RunConfig(dim=1, n0=64, model=3, precision=64, scheme="plm", solver="llf", integrator="ssprk33",
                    boundary="edge", gamma=1.4, dx=1 / 64, cfl=.8, t_end=.2)
    attrs = snapshots.group_attrs(cfg, config="sod")
    st.create_group("20260101000000123", attrs)
    arrays = [np.random.default_rng(k).normal(size=(64, 8)) for k in range(3)]
    for t, a in zip((0.0, 0.01, 0.02), arrays):
        st.write("20260101000000123", str(float(t)), a, {"t": float(t)})
    st.close()
    with open(tmp_path / "run.d" / "attrs.json") as f:
        assert json.load(f) == {"datetime": "2026-01-01 00:00:00", "seed": 7}
    with open(tmp_path / "run.d" / "20260101000000123" / "attrs.json") as f:
        g = json.load(f)
    # the run group's attributes of astrea.py:166-173
    assert set(g) == {"config", "cells", "cfl", "gamma", "dimension", "subgrid", "timestep", "solver"}
    assert g["cells"] == 64 and g["dimension"] == 1 and g["config"] == "sod"
    run = snapshots.read_directory_run(str(tmp_path / "run.d"), "20260101000000123")
    assert [r[0] for r in run] == ["0.0", "0.01", "0.02"]
    assert [r[1]["t"] for r in run] == [0.0, 0.01, 0.02]
    for (_, _, a), b in zip(run, arrays):
        assert np.array_equal(a, b)


def test_reference_layout_fills_the_model_variables():
    planes = np.arange(4 * 3 * 5, dtype=np.float32).reshape(4, 3, 5)  # model 4: rho, vx, vy, p
    out = snapshots._reference_layout(planes, 4, 2)
    assert out.shape == (3, 5, 8)
    assert np.array_equal(out[..., 0], planes[0]) and np.array_equal(out[..., 4], planes[3])
    assert not out[..., 3].any() and not out[..., 5:].any()
    one = snapshots._reference_layout(planes[:3, :, :1], 3, 1)
    assert one.shape == (3, 8) and np.array_equal(one[:, 4], planes[2, :, 0])


def test_open_store_falls_back_to_a_directory(tmp_path):
    st = snapshots.open_store(str(tmp_path / "out.h5"), {"seed": 1})
    try:
        import h5py  # noqa: F401
        assert isinstance(st, snapshots.HDF5Store)
    except ImportError:
        assert isinstance(st, snapshots.DirectoryStore) and os.path.isdir(tmp_path / "out.h5.d")


class _FakeEvent:
    def record(self, stream=None):
        pass

    def synchronize(self):
        pass


class _FakeStream:
    def wait_event(self, ev):
        pass


class _FakeSolver:
    """A 'grid' on the host whose clock advances by a fixed dt per step (clipped onto t_end); the
    stand-in library writes its primitives and clock through the same pointers the device path uses."""

    def __init__(self, cfg, dt):
        import ctypes
        import torch
        self.cfg, self.dt = cfg, dt
        self.state = torch.arange(cfg.model * cfg.n0 * cfg.n1, dtype=torch.float64).reshape(cfg.model, cfg.n0, cfg.n1)
        self.t, self.steps, self.handle = 0.0, 0, None
        solver = self

        class Lib:
            def astrea_to_primitive(self, h, state, out, stream):
                src = (solver.state + solver.t).contiguous()  # held until the copy is done
                ctypes.memmove(out.value, src.data_ptr(), src.numel() * 8)
                return 0

            def astrea_clock_async(self, h, t, steps, done, stream):
                ctypes.memmove(t.value, ctypes.byref(ctypes.c_double(solver.t)), 8)
                ctypes.memmove(steps.value, ctypes.byref(ctypes.c_int(solver.steps)), 4)
                ctypes.memmove(done.value, ctypes.byref(ctypes.c_int(int(solver.t >= solver.cfg.t_end))), 4)
                return 0

        self.lib = Lib()

    def step(self, n=1, graph=True):
        for _ in range(n):
            if self.t >= self.cfg.t_end:
                return
            self.t = self.cfg.t_end if self.t + self.dt >= self.cfg.t_end * (1 - 1e-12) else self.t + self.dt
            self.steps += 1


def test_snapshot_loop_sequence_on_the_host(tmp_path, monkeypatch):
    import torch
    monkeypatch.setattr(torch.Tensor, "pin_memory", lambda self: self)
    monkeypatch.setattr(torch.cuda, "Stream", lambda *a, **k: _FakeStream())
    monkeypatch.setattr(torch.cuda, "Event", lambda *a, **k: _FakeEvent())
    monkeypatch.setattr(torch.cuda, "current_stream", lambda *a, **k: None)
    monkeypatch.setattr(torch.cuda, "stream", lambda s: __import__("contextlib").nullcontext())
    monkeypatch.setattr(torch.cuda, "synchronize", lambda *a, **k: None)
    monkeypatch.setattr(snapshots, "_stream", lambda: None)
    cfg = RunConfig(dim=2, n0=6, n1=5, model=4, precision=64, scheme="ppm", solver="hllc", integrator="ssprk33",
                    boundary="wrap", gamma=1.4, dx=.2, cfl=.8, t_end=.25)
    for every, expect_t in ((1, [0, .1, .2, .25]), (2, [0, .2, .25])):
        s = _FakeSolver(cfg, dt=.1)
        st = snapshots.DirectoryStore(str(tmp_path / f"e{every}"))
        written = snapshots.run_with_snapshots(s, st, "run", every=every)
        run = snapshots.read_directory_run(str(tmp_path / f"e{every}"), "run")
        assert [w[0] for w in written] == pytest.approx(expect_t)
        assert [r[0] for r in run] == [str(float(t)) for t, _ in written]
        for (name, attrs, arr), (t, _) in zip(run, written):
            # the snapshot of time t is the state at t, in the reference layout
            assert arr.shape == (6, 5, 8) and arr[0, 0, 0] == pytest.approx(t)
