"""astrea_reduce_conserved_static: conserved sums with no device allocation.

The entry point keeps its partial sums in a fixed device array instead of
engine buffers.  It must give the same sums as astrea_reduce_conserved on the
same state, on consecutive calls (the scratch is reused, never cleared), and
reject variable counts beyond what the fixed array holds.  This file is
collected last so that it also runs after every other GPU test in one process.
"""

import ctypes

import numpy as np
import pytest
import torch

from astrea_gb300 import _lib
from astrea_gb300.solver import RunConfig, Solver

pytestmark = pytest.mark.gpu

ERR_ARG = -6


def _static_fn():
    lib = _lib.load()
    fn = lib.astrea_reduce_conserved_static
    fn.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong, ctypes.c_int,
                   ctypes.POINTER(ctypes.c_double), ctypes.c_void_p]
    fn.restype = ctypes.c_int
    return lib, fn


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _sums_static(fn, state, precision, nv):
    out = (ctypes.c_double * nv)()
    rc = fn(ctypes.c_void_p(state.data_ptr()), precision, state.numel() // nv, nv, out, _stream())
    assert rc == 0, _lib.load().astrea_last_error()
    return np.array(out[:])


def _sums_handle(lib, s):
    out = (ctypes.c_double * s.nv)()
    rc = lib.astrea_reduce_conserved(s.handle, ctypes.c_void_p(s.state.data_ptr()), out, _stream())
    assert rc == 0, lib.astrea_last_error()
    return np.array(out[:])


def _seeded(cfg, seed):
    rng = np.random.default_rng(seed)
    shape = (cfg.n0, 8) if cfg.dim == 1 else (cfg.n0, cfg.n1, 8)
    w = np.zeros(shape)
    w[..., 0] = rng.uniform(0.5, 2.0, shape[:-1])
    w[..., 4] = rng.uniform(0.5, 2.0, shape[:-1])
    w[..., 1:4] = rng.uniform(-1.0, 1.0, shape[:-1] + (3,))
    if cfg.model == 8:
        w[..., 5:8] = rng.uniform(-1.0, 1.0, shape[:-1] + (3,))
    if cfg.dim == 1 and cfg.model == 3:
        w[..., 2:4] = 0.0
    if cfg.model == 4:
        w[..., 3] = 0.0
    return w


@pytest.mark.parametrize("cfg", [
    RunConfig(dim=2, n0=256, n1=192, model=4, precision=64, scheme="ppm", solver="hllc", integrator="ssprk33",
              boundary="wrap", gamma=1.4, dx=1.0 / 256, cfl=0.4, t_end=1.0, compat=False),
    RunConfig(dim=1, n0=4099, n1=1, model=8, precision=32, scheme="plm", solver="llf", integrator="ssprk22",
              boundary="edge", gamma=5.0 / 3.0, dx=1.0 / 4099, cfl=0.4, t_end=1.0),
], ids=["2d_euler_fp64", "1d_mhd_fp32"])
def test_static_sums_match_the_handle_sums(cfg):
    lib, fn = _static_fn()
    s = Solver(cfg)
    s.initialise(_seeded(cfg, 7))
    s.reset_clock()
    ref0 = _sums_handle(lib, s)
    a = _sums_static(fn, s.state, cfg.precision, s.nv)
    b = _sums_static(fn, s.state, cfg.precision, s.nv)
    scale = np.maximum(np.abs(ref0), 1.0)
    assert np.all(np.abs(a - ref0) <= 1e-12 * scale), (a, ref0)
    assert np.all(np.abs(b - ref0) <= 1e-12 * scale), (b, ref0)
    # after the state changes, the reused scratch gives the new sums
    s.step(3)
    torch.cuda.synchronize()
    ref1 = _sums_handle(lib, s)
    c = _sums_static(fn, s.state, cfg.precision, s.nv)
    assert np.all(np.abs(c - ref1) <= 1e-12 * np.maximum(np.abs(ref1), 1.0)), (c, ref1)


def test_static_sums_take_no_device_memory_after_the_first_call():
    """Once the first call has loaded the module, further calls leave the device's free memory unchanged."""
    lib, fn = _static_fn()
    x = torch.rand(8, 1 << 16, dtype=torch.float64, device="cuda")
    first = _sums_static(fn, x, 64, 8)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(5):
        again = _sums_static(fn, x, 64, 8)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert np.array_equal(first, again)


def test_static_sums_reject_what_the_scratch_cannot_hold():
    lib, fn = _static_fn()
    x = torch.ones(9 * 16, dtype=torch.float64, device="cuda")
    out = (ctypes.c_double * 9)()
    assert fn(ctypes.c_void_p(x.data_ptr()), 64, 16, 9, out, _stream()) == ERR_ARG
    assert b"at most 8" in lib.astrea_last_error()
    assert fn(ctypes.c_void_p(x.data_ptr()), 64, 16, 0, out, _stream()) == ERR_ARG
    assert fn(ctypes.c_void_p(x.data_ptr()), 16, 16, 8, out, _stream()) == ERR_ARG
    assert fn(ctypes.c_void_p(x.data_ptr()), 64, 0, 8, out, _stream()) == ERR_ARG
    # a plain call still works after the rejections
    got = _sums_static(fn, x[:8 * 16], 64, 8)
    assert np.array_equal(got, np.full(8, 16.0))
