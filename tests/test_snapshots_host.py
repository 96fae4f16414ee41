"""Snapshot stores on the host: the directory form of the reference's HDF5 layout."""

import json
import os

import numpy as np

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
