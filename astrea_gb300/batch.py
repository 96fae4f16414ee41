"""Batched solver: many independent grids of uneven sizes in one device arena.

All grids of a ``Batch`` share dimension, variable model, precision and
integrator; each has its own size, scheme x solver (PLM/PPM/WENO5 x
LLF/HLLC, or LLF/HLLD for the MHD model), boundary, gamma, dx, CFL and end
time, and its own device clock.  One ``step`` advances every unfinished grid
by one of *its* time steps; finished grids are skipped on the device.
"""

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from . import config as C
from .solver import MODEL_VARS, RunConfig, _stream


class GridSpec(ctypes.Structure):
    _fields_ = [("n0", ctypes.c_int), ("n1", ctypes.c_int), ("scheme", ctypes.c_int), ("solver", ctypes.c_int),
                ("boundary", ctypes.c_int), ("limiter", ctypes.c_int), ("flags", ctypes.c_int),
                ("gamma", ctypes.c_double), ("dx", ctypes.c_double), ("cfl", ctypes.c_double),
                ("t_end", ctypes.c_double), ("checkpoints", ctypes.c_int)]


_SIGS = {
    "astrea_batch_create": ([ctypes.c_int] * 4 + [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)], ctypes.c_int),
    "astrea_batch_destroy": ([ctypes.c_void_p], None),
    "astrea_batch_layout": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int),
                             ctypes.POINTER(ctypes.c_longlong)], ctypes.c_int),
    "astrea_batch_initialise": ([ctypes.c_void_p] * 4, ctypes.c_int),
    "astrea_batch_step": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p], ctypes.c_int),
    "astrea_batch_graph_step": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p], ctypes.c_int),
    "astrea_batch_clocks": ([ctypes.c_void_p] * 7, ctypes.c_int),
}


def _lib_batch():
    lib = _lib.load()
    for name, (args, res) in _SIGS.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    return lib


def spec_of(cfg: RunConfig):
    if cfg.scheme not in ("plm", "ppm", "weno5"):
        raise C.ConfigError("batched grids use PLM, PPM or WENO5")
    return GridSpec(n0=cfg.n0, n1=cfg.n1 if cfg.dim == 2 else 1, scheme=C.SCHEME[cfg.scheme],
                    solver=C.SOLVER[cfg.solver], boundary=C.BOUNDARY[cfg.boundary], limiter=C.LIMITER[cfg.limiter],
                    flags=0 if cfg.compat else 1, gamma=cfg.gamma, dx=cfg.dx, cfl=cfg.cfl, t_end=cfg.t_end,
                    checkpoints=cfg.checkpoints)


class Batch:
    def __init__(self, cfgs, device=None):
        if not torch.cuda.is_available():
            raise _lib.AstreaError(-2, "no CUDA device: the astrea_gb300 update runs only on the GPU")
        c0 = cfgs[0]
        for c in cfgs:
            if (c.dim, c.model, c.precision, c.integrator) != (c0.dim, c0.model, c0.precision, c0.integrator):
                raise C.ConfigError("a batch shares dim, model, precision and integrator")
        self.cfgs = list(cfgs)
        self.dim, self.model, self.precision = c0.dim, c0.model, c0.precision
        self.lib = _lib_batch()
        self.device = torch.device(device or "cuda")
        specs = (GridSpec * len(cfgs))(*[spec_of(c) for c in cfgs])
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(self.lib.astrea_batch_create(c0.dim, c0.model, c0.precision, C.INTEGRATOR[c0.integrator],
                                                    ctypes.cast(specs, ctypes.c_void_p), len(cfgs), ctypes.byref(h)))
        self.handle = h
        offs = (ctypes.c_longlong * (len(cfgs) + 1))()
        nv, total = ctypes.c_int(), ctypes.c_longlong()
        _lib.check(self.lib.astrea_batch_layout(self.handle, ctypes.cast(offs, ctypes.c_void_p), ctypes.byref(nv),
                                                ctypes.byref(total)))
        self.offsets = list(offs)
        self.nv = nv.value
        dtype = torch.float64 if c0.precision == 64 else torch.float32
        self.arena = torch.zeros(total.value, dtype=dtype, device=self.device)

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                torch.cuda.synchronize(self.device)
            except Exception:
                pass
            self.lib.astrea_batch_destroy(h)
            self.handle = None

    def __len__(self):
        return len(self.cfgs)

    def planes(self, g):
        """View (nv, n0, n1) of grid g's state in the arena."""
        c = self.cfgs[g]
        n1 = c.n1 if c.dim == 2 else 1
        return self.arena[self.offsets[g]:self.offsets[g + 1]].view(self.nv, c.n0, n1)

    def initialise(self, prims):
        """Point primitives (one (n0[, n1], 8) array per grid) -> cell-averaged conservatives."""
        prim_arena = torch.zeros_like(self.arena)
        idx = MODEL_VARS[self.model]
        for g, w in enumerate(prims):
            t = torch.as_tensor(w)
            if t.dim() == 2:
                t = t[:, None, :]
            prim_arena[self.offsets[g]:self.offsets[g + 1]].view(self.nv, *t.shape[:2]).copy_(
                t[..., idx].permute(2, 0, 1).to(self.arena.dtype))
        _lib.check(self.lib.astrea_batch_initialise(self.handle, ctypes.c_void_p(prim_arena.data_ptr()),
                                                    ctypes.c_void_p(self.arena.data_ptr()), _stream()))
        torch.cuda.current_stream().synchronize()

    def step(self, n=1, graph=True):
        fn = self.lib.astrea_batch_graph_step if graph else self.lib.astrea_batch_step
        _lib.check(fn(self.handle, ctypes.c_void_p(self.arena.data_ptr()), int(n), _stream()))

    def clocks(self):
        g = len(self.cfgs)
        t, dt = (ctypes.c_double * g)(), (ctypes.c_double * g)()
        steps, done, status = (ctypes.c_int * g)(), (ctypes.c_int * g)(), (ctypes.c_int * g)()
        _lib.check(self.lib.astrea_batch_clocks(self.handle, *[ctypes.cast(x, ctypes.c_void_p) for x in
                                                               (t, dt, steps, done, status)], _stream()))
        return {"t": np.array(t[:]), "dt": np.array(dt[:]), "steps": np.array(steps[:]),
                "done": np.array(done[:], dtype=bool), "status": np.array(status[:])}

    def run(self, max_steps=None, check_every=16, graph=True):
        n = 0
        while True:
            k = check_every if max_steps is None else min(check_every, max_steps - n)
            if k <= 0:
                break
            self.step(k, graph=graph)
            n += k
            c = self.clocks()
            if c["done"].all():
                break
        return self.clocks()
