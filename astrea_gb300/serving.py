"""Continuous-batching server for solve requests.

A request is one independent simulation: an initial state (point
primitives), a method (scheme x solver), and an end time.  The server keeps
one slot batch per (dimension, variable model) class on the GPU.  Requests
are admitted as soon as they have arrived *and* their class has a free slot
and room in its arena; the device memory of all classes together is bounded
by an HBM budget fixed at start-up.  Every iteration advances all admitted,
unfinished requests of every class by a few of their own time steps (the
classes run on separate CUDA streams, so their kernels overlap), then
retires finished requests, frees their memory, and admits waiting ones.
Latency = completion time - arrival time.

The reference has no serving layer (one simulation per process,
astrea.py:90-226); this is built on the batched engine.
"""

import bisect
import math
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np
import torch

from .batch import SlotBatch
from .solver import RunConfig

# arenas of the state's size a class holds: the caller-side state and primitive arenas
# plus the engine's two stage, two divergence and one scratch arena, and in 2D the cell
# averages of the high-order schemes (one arena in FP32, one per sweep order in FP64)
ARENA_COPIES = 7


def arena_copies(dim, precision):
    return ARENA_COPIES + (0 if dim == 1 else (1 if precision == 32 else 2))


@dataclass
class Request:
    rid: int
    arrival: float
    dim: int
    n: int
    mhd: bool
    scheme: str
    solver: str
    t_end: float
    seed: int
    boundary: str = "edge"
    gamma: float = 1.4
    cfl: float = 0.8  # make_requests: 0.8 in 1D, 0.4 in 2D
    compat: bool = False
    # filled in by the server
    admitted: float = math.nan
    finished: float = math.nan
    steps: int = 0
    status: int = 0
    result: object = None

    @property
    def model(self):
        return 8 if self.mhd else (3 if self.dim == 1 else 4)

    @property
    def cells(self):
        return self.n * (self.n if self.dim == 2 else 1)

    def config(self, precision):
        return RunConfig(dim=self.dim, n0=self.n, n1=self.n if self.dim == 2 else 1, model=self.model,
                         precision=precision, scheme=self.scheme, solver=self.solver, integrator="ssprk33",
                         boundary=self.boundary, gamma=self.gamma, dx=1.0 / self.n, cfl=self.cfl, t_end=self.t_end,
                         compat=self.compat)

    def states(self):
        """The seeded Riemann states: two in 1D (left, right), four in 2D (quadrants in row-major order)."""
        rng = np.random.default_rng(self.seed)

        def state():
            s = np.zeros(8)
            s[0], s[4] = rng.uniform(.1, 2), rng.uniform(.1, 2)
            s[1:4] = rng.uniform(-1, 1, 3) if self.mhd else [rng.uniform(-1, 1), 0 if self.dim == 1 else
                                                              rng.uniform(-1, 1), 0]
            if self.mhd:
                s[5:8] = rng.uniform(-1, 1, 3)
            return s

        return [state() for _ in range(2 if self.dim == 1 else 4)]

    def initial_state(self):
        """Point primitives on the host: seeded Riemann data (two states in 1D, four quadrants in 2D)."""
        st = self.states()
        n = self.n
        if self.dim == 1:
            w = np.zeros((n, 8))
            w[: n // 2], w[n // 2:] = st
        else:
            w = np.zeros((n, n, 8))
            h = n // 2
            w[:h, :h], w[:h, h:], w[h:, :h], w[h:, h:] = st
        return w

    def ic(self):
        """The same data as an ``initial.IC`` for the device builder: a jump at x = 1/2 on [0, 1] (even n)."""
        from . import initial
        st = self.states()
        c = initial.IC(kind=initial.SPLIT if self.dim == 1 else initial.QUADRANT, abs_mask=0, dim=self.dim, n=self.n,
                       start=0.0, end=1.0, shock=0.5, gamma=self.gamma)
        slots = ("left", "right") if self.dim == 1 else ("left", "bottom_left", "right", "bottom_right")
        for name, s in zip(slots, st):
            arr = getattr(c, name)
            for k in range(8):
                arr[k] = float(s[k])
        return c


def make_requests(count, rate, seed=20261203, n1d=(256, 65536), n2d=(128, 2048), frac_1d=0.4, frac_mhd=0.5,
                  t_end=(0.05, 0.3)):
    """Seeded request stream: Poisson arrivals at ``rate``/s, the mixed sizes and methods of the serving workload."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(count):
        t += rng.exponential(1.0 / rate)
        dim = 1 if rng.uniform() < frac_1d else 2
        lo, hi = n1d if dim == 1 else n2d
        n = int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))
        n = max(8, n - n % 2)
        mhd = bool(rng.uniform() < frac_mhd)
        scheme = ["plm", "ppm", "weno5"][rng.integers(3)]
        solver = ["llf", "hlld" if mhd else "hllc"][rng.integers(2)]
        # the reference's dt rule takes the CFL number per axis (astrea.py:70-71), which the
        # unsplit 2D update adds over both axes: 0.4 keeps that sum at 0.8, as 0.8 does in 1D
        out.append(Request(rid=i, arrival=t, dim=dim, n=n, mhd=mhd, scheme=scheme, solver=solver,
                           t_end=float(rng.uniform(*t_end)), seed=int(rng.integers(1 << 31)),
                           cfl=0.8 if dim == 1 else 0.4))
    return out


class Arena:
    """First-fit allocator of element ranges."""

    def __init__(self, capacity):
        self.capacity = capacity
        self.free = [(0, capacity)]  # sorted (start, size)

    def alloc(self, size):
        for i, (s, n) in enumerate(self.free):
            if n >= size:
                if n == size:
                    self.free.pop(i)
                else:
                    self.free[i] = (s + size, n - size)
                return s
        return None

    def release(self, start, size):
        i = bisect.bisect(self.free, (start, size))
        self.free.insert(i, (start, size))
        merged = []
        for s, n in self.free:
            if merged and merged[-1][0] + merged[-1][1] == s:
                merged[-1] = (merged[-1][0], merged[-1][1] + n)
            else:
                merged.append((s, n))
        self.free = merged


def stalled(steps, t, dt, t_end, max_steps, check_after=1000):
    """Whether a running request is retired for its time step: past ``max_steps`` steps, or, once it has
    taken ``check_after`` steps, when its current dt would need more than ``max_steps`` steps in all to
    reach ``t_end`` (a step that collapsed on near-vacuum states does not recover in time)."""
    if max_steps is None:
        return False
    if steps > max_steps:
        return True
    if steps < check_after:
        return False
    return not (dt > 0) or (t_end - t) / dt > max_steps - steps


@dataclass
class ServeStats:
    latencies_ms: list = field(default_factory=list)
    cell_updates: float = 0.0         # of requests that finished with status 0
    failed_cell_updates: float = 0.0  # spent on requests retired with a non-zero status
    wall_s: float = 0.0
    failed: int = 0   # requests retired with a non-zero status (non-finite state, or stalled)
    stalled: int = 0  # of those, retired for exceeding the step limit
    max_active: int = 0
    unfinished: list = field(default_factory=list)  # requests cut off by the wall-clock cap (diagnostics)

    def summary(self):
        lat = np.array(self.latencies_ms) if self.latencies_ms else np.array([math.nan])
        return {"requests": len(self.latencies_ms), "p50_ms": float(np.percentile(lat, 50)),
                "p99_ms": float(np.percentile(lat, 99)), "cell_updates_per_s": self.cell_updates / max(self.wall_s, 1e-9),
                "failed_cell_updates_per_s": self.failed_cell_updates / max(self.wall_s, 1e-9),
                "wall_s": self.wall_s, "failed": self.failed, "stalled": self.stalled, "max_active": self.max_active}


class Server:
    """Continuous batching of solve requests under an HBM budget."""

    CLASSES = ((1, 3), (1, 8), (2, 4), (2, 8))

    def __init__(self, hbm_budget_bytes=150e9, precision=32, max_slots=256, shares=None, keep_results=False,
                 steps_per_poll=4, device=None, max_steps=None, max_steps_per_poll=32, graph=True):
        self.precision = precision
        # a request whose time step collapsed (near-vacuum states with finite speeds) would never reach its
        # end time; once it is past, or projected past, ``max_steps`` steps it is retired with status bit 2
        # (value 4; see ``stalled``)
        self.max_steps = max_steps
        esize = 4 if precision == 32 else 8
        shares = shares or {(1, 3): .1, (1, 8): .1, (2, 4): .5, (2, 8): .3}
        self.device = torch.device(device or "cuda")
        self.batches, self.arenas, self.streams, self.free_slots = {}, {}, {}, {}
        self.classes = []
        for cls in self.CLASSES:
            cap = int(hbm_budget_bytes * shares.get(cls, 0) / (arena_copies(cls[0], precision) * esize))
            cap -= cap % 8
            if cap <= 0:
                continue
            self.classes.append(cls)
            self.batches[cls] = SlotBatch(cls[0], cls[1], precision, "ssprk33", max_slots, cap, self.device)
            self.arenas[cls] = Arena(cap)
            self.streams[cls] = torch.cuda.Stream(self.device)
            self.free_slots[cls] = list(range(max_slots))[::-1]
        self.keep_results = keep_results
        # steps per poll of a class: ``steps_per_poll`` while it has requests without a clock reading yet,
        # else the fewest steps any of its requests still needs (at least 1, at most ``max_steps_per_poll``),
        # so that polls land on completions; every poll's steps replay one captured CUDA graph
        self.steps_per_poll = steps_per_poll
        self.max_steps_per_poll = max_steps_per_poll
        self.graph = graph
        self.last_clk = {}

    def _admit(self, r, now):
        cls = (r.dim, r.model)
        size = r.model * r.cells
        if not self.free_slots[cls]:
            return False
        off = self.arenas[cls].alloc(size)
        if off is None:
            return False
        slot = self.free_slots[cls].pop()
        with torch.cuda.stream(self.streams[cls]):
            # the initial state is built on the device from the request's few Riemann states
            self.batches[cls].occupy_ic(slot, r.config(self.precision), off, r.ic())
        r.admitted = now
        self.active[cls][slot] = (r, off, size)
        return True

    def _poll_steps(self, cls):
        last = self.last_clk.get(cls)
        if last is None or any(last[1].get(slot) != e[0].rid for slot, e in self.active[cls].items()):
            return self.steps_per_poll
        clk = last[0]
        need = self.max_steps_per_poll
        for slot, (r, _, _) in self.active[cls].items():
            dt = float(clk["dt"][slot])
            if dt > 0 and math.isfinite(dt):
                need = min(need, math.ceil((r.t_end - float(clk["t"][slot])) / dt))
            else:
                need = 1
        return max(1, min(need, self.max_steps_per_poll))

    def serve(self, requests, realtime=True, max_wall_s=None):
        """Run the request stream; returns ServeStats (requests are updated in place)."""
        stats = ServeStats()
        pending = {cls: deque() for cls in self.classes}
        for r in sorted(requests, key=lambda x: x.arrival):
            cls = (r.dim, r.model)
            if cls not in pending:
                raise ValueError(f"request {r.rid}: no device memory was budgeted for class {cls}")
            size = r.model * r.cells
            if size > self.arenas[cls].capacity:
                raise ValueError(f"request {r.rid} ({size} elements) exceeds its class arena")
            pending[cls].append(r)
        self.active = {cls: {} for cls in self.classes}
        self.last_clk = {}
        t0 = time.perf_counter()
        while any(pending.values()) or any(self.active.values()):
            now = time.perf_counter() - t0
            if max_wall_s is not None and now > max_wall_s:
                break
            for cls in self.classes:
                q = pending[cls]
                while q and (q[0].arrival <= now or not realtime):
                    if not self._admit(q[0], now):
                        break
                    q.popleft()
            n_active = sum(len(a) for a in self.active.values())
            stats.max_active = max(stats.max_active, n_active)
            if n_active == 0:
                nxt = min((q[0].arrival for q in pending.values() if q), default=None)
                if nxt is not None and realtime:
                    time.sleep(max(0.0, min(nxt - now, 0.05)))
                continue
            for cls in self.classes:
                if self.active[cls]:
                    with torch.cuda.stream(self.streams[cls]):
                        self.batches[cls].step(self._poll_steps(cls), graph=self.graph)
            for cls in self.classes:
                if not self.active[cls]:
                    continue
                with torch.cuda.stream(self.streams[cls]):
                    clk = self.batches[cls].clocks()
                self.last_clk[cls] = (clk, {slot: e[0].rid for slot, e in self.active[cls].items()})
                now = time.perf_counter() - t0
                for slot in list(self.active[cls].keys()):
                    r = self.active[cls][slot][0]
                    over = not clk["done"][slot] and stalled(int(clk["steps"][slot]), float(clk["t"][slot]),
                                                             float(clk["dt"][slot]), r.t_end, self.max_steps)
                    if not clk["done"][slot] and not over:
                        continue
                    r, off, size = self.active[cls].pop(slot)
                    r.finished = now
                    r.steps = int(clk["steps"][slot])
                    r.status = int(clk["status"][slot]) | (4 if over and not clk["done"][slot] else 0)
                    if r.status:
                        stats.failed += 1
                    if r.status & 4:
                        stats.stalled += 1
                    if r.status:
                        stats.failed_cell_updates += r.cells * r.steps
                    else:
                        stats.cell_updates += r.cells * r.steps
                    stats.latencies_ms.append(1e3 * (r.finished - r.arrival))
                    if self.keep_results:
                        with torch.cuda.stream(self.streams[cls]):
                            r.result = self.batches[cls].planes(slot).clone()
                    self.batches[cls].release(slot)
                    self.arenas[cls].release(off, size)
                    self.free_slots[cls].append(slot)
        torch.cuda.synchronize(self.device)
        stats.wall_s = time.perf_counter() - t0
        # requests still running when the wall-clock cap ends the loop give their slots and memory back
        for cls in self.classes:
            clk = self.batches[cls].clocks() if self.active[cls] else None
            for slot, (r, off, size) in list(self.active[cls].items()):
                stats.unfinished.append({"rid": r.rid, "class": cls, "n": r.n, "scheme": r.scheme, "solver": r.solver,
                                         "t_end": r.t_end, "t": float(clk["t"][slot]), "dt": float(clk["dt"][slot]),
                                         "steps": int(clk["steps"][slot]), "status": int(clk["status"][slot])})
                self.batches[cls].release(slot)
                self.arenas[cls].release(off, size)
                self.free_slots[cls].append(slot)
            self.active[cls] = {}
            for r in pending[cls]:
                stats.unfinished.append({"rid": r.rid, "class": cls, "n": r.n, "pending": True})
        return stats
