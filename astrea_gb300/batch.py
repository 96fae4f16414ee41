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
    "astrea_batch_create": ([ctypes.c_int] * 5 + [ctypes.c_longlong, ctypes.POINTER(ctypes.c_void_p)], ctypes.c_int),
    "astrea_batch_destroy": ([ctypes.c_void_p], None),
    "astrea_batch_set": ([ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_longlong], ctypes.c_int),
    "astrea_batch_clear": ([ctypes.c_void_p, ctypes.c_int], ctypes.c_int),
    "astrea_batch_initialise": ([ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p],
                                ctypes.c_int),
    "astrea_batch_step": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p], ctypes.c_int),
    "astrea_batch_graph_step": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p], ctypes.c_int),
    "astrea_batch_clocks": ([ctypes.c_void_p] * 7, ctypes.c_int),
    "astrea_batch_tile": ([ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)],
                          ctypes.c_int),
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


class SlotBatch:
    """A fixed-capacity batch whose slots are filled and released between steps."""

    def __init__(self, dim, model, precision, integrator, max_slots, capacity_elems, device=None):
        if not torch.cuda.is_available():
            raise _lib.AstreaError(-2, "no CUDA device: the astrea_gb300 update runs only on the GPU")
        self.dim, self.model, self.precision = dim, model, precision
        self.max_slots = max_slots
        self.lib = _lib_batch()
        self.device = torch.device(device or "cuda")
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(self.lib.astrea_batch_create(dim, model, precision, C.INTEGRATOR[integrator], max_slots,
                                                    int(capacity_elems), ctypes.byref(h)))
        self.handle = h
        self.nv = model
        dtype = torch.float64 if precision == 64 else torch.float32
        self.arena = torch.zeros(int(capacity_elems), dtype=dtype, device=self.device)
        self.prim_arena = torch.zeros_like(self.arena)
        self.slots = {}  # slot -> (cfg, offset)

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                torch.cuda.synchronize(self.device)
            except Exception:
                pass
            self.lib.astrea_batch_destroy(h)
            self.handle = None

    def occupy(self, slot, cfg, offset, w_point):
        """Put grid ``cfg`` at element ``offset`` into ``slot`` and initialise it from point primitives."""
        spec = spec_of(cfg)
        _lib.check(self.lib.astrea_batch_set(self.handle, int(slot), ctypes.byref(spec), int(offset)))
        self.slots[slot] = (cfg, int(offset))
        t = torch.as_tensor(w_point)
        if t.dim() == 2:
            t = t[:, None, :]
        n = self.nv * t.shape[0] * t.shape[1]
        self.prim_arena[offset:offset + n].view(self.nv, t.shape[0], t.shape[1]).copy_(
            t[..., MODEL_VARS[self.model]].permute(2, 0, 1).to(self.arena.dtype))
        _lib.check(self.lib.astrea_batch_initialise(self.handle, int(slot), ctypes.c_void_p(self.prim_arena.data_ptr()),
                                                    ctypes.c_void_p(self.arena.data_ptr()), _stream()))

    def occupy_ic(self, slot, cfg, offset, ic):
        """Like ``occupy``, with the point primitives built on the device from an ``initial.IC``."""
        from . import initial
        spec = spec_of(cfg)
        _lib.check(self.lib.astrea_batch_set(self.handle, int(slot), ctypes.byref(spec), int(offset)))
        self.slots[slot] = (cfg, int(offset))
        lib = initial._lib_ic()
        esize = self.prim_arena.element_size()
        ptr = self.prim_arena.data_ptr() + int(offset) * esize
        _lib.check(lib.astrea_point_state(ctypes.byref(ic), self.precision, self.model, ctypes.c_void_p(ptr), _stream()))
        _lib.check(self.lib.astrea_batch_initialise(self.handle, int(slot), ctypes.c_void_p(self.prim_arena.data_ptr()),
                                                    ctypes.c_void_p(self.arena.data_ptr()), _stream()))

    def release(self, slot):
        _lib.check(self.lib.astrea_batch_clear(self.handle, int(slot)))
        self.slots.pop(slot, None)

    def planes(self, slot):
        cfg, off = self.slots[slot]
        n1 = cfg.n1 if cfg.dim == 2 else 1
        return self.arena[off:off + self.nv * cfg.n0 * n1].view(self.nv, cfg.n0, n1)

    def step(self, n=1, graph=False):
        fn = self.lib.astrea_batch_graph_step if graph else self.lib.astrea_batch_step
        _lib.check(fn(self.handle, ctypes.c_void_p(self.arena.data_ptr()), int(n), _stream()))

    def tiles(self):
        """The (cells along, rows across) tile of each axis's batched sweep (tuned at the first step)."""
        out = []
        for ax in range(self.dim):
            ts, tt = ctypes.c_int(), ctypes.c_int()
            _lib.check(self.lib.astrea_batch_tile(self.handle, ax, ctypes.byref(ts), ctypes.byref(tt)))
            out.append((ts.value, tt.value))
        return out

    def clocks(self):
        g = self.max_slots
        t, dt = (ctypes.c_double * g)(), (ctypes.c_double * g)()
        steps, done, status = (ctypes.c_int * g)(), (ctypes.c_int * g)(), (ctypes.c_int * g)()
        _lib.check(self.lib.astrea_batch_clocks(self.handle, *[ctypes.cast(x, ctypes.c_void_p) for x in
                                                               (t, dt, steps, done, status)], _stream()))
        return {"t": np.array(t[:]), "dt": np.array(dt[:]), "steps": np.array(steps[:]),
                "done": np.array(done[:], dtype=bool), "status": np.array(status[:])}


class Batch:
    """A static batch: every grid occupies one slot of a packed arena."""

    def __init__(self, cfgs, device=None):
        c0 = cfgs[0]
        for c in cfgs:
            if (c.dim, c.model, c.precision, c.integrator) != (c0.dim, c0.model, c0.precision, c0.integrator):
                raise C.ConfigError("a batch shares dim, model, precision and integrator")
        self.cfgs = list(cfgs)
        self.dim, self.model, self.precision = c0.dim, c0.model, c0.precision
        self.nv = c0.model
        sizes = [self.nv * c.n0 * (c.n1 if c.dim == 2 else 1) for c in cfgs]
        self.offsets = [0] + list(np.cumsum(sizes))
        self.sb = SlotBatch(c0.dim, c0.model, c0.precision, c0.integrator, len(cfgs), self.offsets[-1], device)
        self.arena = self.sb.arena
        for g, c in enumerate(cfgs):
            _lib.check(self.sb.lib.astrea_batch_set(self.sb.handle, g, ctypes.byref(spec_of(c)),
                                                    int(self.offsets[g])))
            self.sb.slots[g] = (c, int(self.offsets[g]))

    def __len__(self):
        return len(self.cfgs)

    def planes(self, g):
        return self.sb.planes(g)

    def initialise_one(self, g, w):
        """Point primitives (n0[, n1], 8) of grid g (NumPy or torch, host or device) -> its averages."""
        cfg, off = self.sb.slots[g]
        t = torch.as_tensor(w)
        if t.dim() == 2:
            t = t[:, None, :]
        n = self.nv * t.shape[0] * t.shape[1]
        self.sb.prim_arena[off:off + n].view(self.nv, t.shape[0], t.shape[1]).copy_(
            t[..., MODEL_VARS[self.model]].permute(2, 0, 1).to(self.arena.dtype))
        _lib.check(self.sb.lib.astrea_batch_initialise(self.sb.handle, g,
                                                       ctypes.c_void_p(self.sb.prim_arena.data_ptr()),
                                                       ctypes.c_void_p(self.arena.data_ptr()), _stream()))

    def initialise(self, prims):
        for g, w in enumerate(prims):
            self.initialise_one(g, w)
        torch.cuda.current_stream().synchronize()

    def step(self, n=1, graph=True):
        self.sb.step(n, graph=graph)

    def clocks(self):
        return self.sb.clocks()

    def tiles(self):
        return self.sb.tiles()

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
