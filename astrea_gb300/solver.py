"""Device-resident solver for one grid: the host side of the C ABI.

A ``Solver`` owns a handle of ``libastrea_gb300.so`` and the grid's
conservative state as a torch tensor on the GPU, laid out as the library
expects: ``nv`` component planes (structure of arrays) of shape (n0, n1).  The
reference's (n0[, n1], 8) arrays convert to and from that layout with
``to_planes`` / ``from_planes``.

PyTorch is used for device memory and streams only; all arithmetic of the
update runs in the library's CUDA kernels.
"""

import ctypes
from dataclasses import dataclass, asdict

import numpy as np
import torch

from . import _lib
from . import config as C

MODEL_VARS = {3: [0, 1, 4], 4: [0, 1, 2, 4], 8: list(range(8))}


@dataclass
class RunConfig:
    dim: int
    n0: int
    n1: int = 1
    model: int = 3
    precision: int = 64
    scheme: str = "plm"
    solver: str = "llf"
    integrator: str = "ssprk33"
    boundary: str = "edge"
    limiter: str = "minmod"
    gamma: float = 1.4
    dx: float = 1.0
    cfl: float = 0.8
    t_end: float = 0.2
    checkpoints: int = 1
    compat: bool = True  # False: textbook HLLC/HLLD (not a reference option)
    magnetic_2d: bool = False  # constrained-transport 2D MHD (sim_variables.magnetic_2d)
    flatten: bool = False  # PPM flattening (schemes/ppm.py:111-134; not run by the reference)
    viscosity: bool = False  # PPM artificial viscosity (schemes/ppm.py:138-170; not run by the reference)

    def to_c(self):
        if self.solver not in C.SOLVER:
            raise C.ConfigError(f"solver {self.solver!r} is not provided by the CUDA library")
        if self.magnetic_2d and self.integrator not in ("euler", "ssprk22", "ssprk33", "ssprk43"):
            raise C.ConfigError("constrained transport runs with Euler and SSP-RK (2,2), (3,3), (4,3)")
        return _lib.Cfg(dim=self.dim, n0=self.n0, n1=self.n1 if self.dim == 2 else 1, model=self.model,
                        precision=self.precision, scheme=C.SCHEME[self.scheme], solver=C.SOLVER[self.solver],
                        integrator=C.INTEGRATOR[self.integrator], boundary=C.BOUNDARY[self.boundary],
                        limiter=C.LIMITER[self.limiter], gamma=float(self.gamma), dx=float(self.dx),
                        cfl=float(self.cfl), t_end=float(self.t_end), checkpoints=int(self.checkpoints),
                        flags=(0 if self.compat else 1) | (2 if self.magnetic_2d else 0)
                        | (4 if self.flatten else 0) | (8 if self.viscosity else 0))

    @property
    def shape(self):
        return (self.n0,) if self.dim == 1 else (self.n0, self.n1)

    @property
    def dtype(self):
        return torch.float64 if self.precision == 64 else torch.float32


def pick_model(dim, solver, grid=None):
    """Smallest variable model that carries every non-zero variable of ``grid``."""
    if solver == "hlld":
        return 8
    if grid is not None:
        g = grid if isinstance(grid, np.ndarray) else grid.detach().cpu().numpy()
        nonzero = [bool(np.any(g[..., v] != 0)) for v in range(8)]
        extra = [2, 3, 5, 6, 7] if dim == 1 else [3, 5, 6, 7]
        if any(nonzero[v] for v in extra):
            return 8
    return 3 if dim == 1 else 4


def config_from_sim_variables(sv, precision=64, model=None, grid=None):
    """RunConfig from a reference ``sim_variables`` namedtuple (generic.py:159-286 fields)."""
    dim = int(sv.dimension)
    scheme = C.scheme_of(sv.subgrid)
    solver = C.solver_of(sv.solver, getattr(sv, "solver_category", None))
    integrator = C.integrator_of(sv.timestep)
    magnetic_2d = bool(getattr(sv, "magnetic_2d", False))
    n = int(sv.cells)
    if model is None:
        model = 8 if magnetic_2d else pick_model(dim, solver, grid)
    return RunConfig(dim=dim, n0=n, n1=n if dim == 2 else 1, model=model, precision=precision, scheme=scheme,
                     solver=solver, integrator=integrator, boundary=sv.boundary, gamma=float(sv.gamma),
                     dx=float(sv.dx), cfl=float(sv.cfl), t_end=float(sv.t_end),
                     checkpoints=int(getattr(sv, "checkpoints", 1)), magnetic_2d=magnetic_2d)


def to_planes(grid, model, dtype, device):
    """(n0[, n1], 8) array -> (nv, n0, n1) device tensor of the model's variables."""
    g = torch.as_tensor(grid)
    if g.dim() == 2:
        g = g[:, None, :]
    idx = torch.tensor(MODEL_VARS[model], device=g.device)
    return g.index_select(-1, idx).permute(2, 0, 1).contiguous().to(device=device, dtype=dtype)


def from_planes(planes, model, dim):
    """(nv, n0, n1) tensor -> (n0[, n1], 8) tensor with the model's zero variables filled in."""
    nv, n0, n1 = planes.shape
    out = torch.zeros((n0, n1, 8), dtype=planes.dtype, device=planes.device)
    out[..., MODEL_VARS[model]] = planes.permute(1, 2, 0)
    return out[:, 0, :] if dim == 1 else out


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class Solver:
    """One grid on the GPU, advanced by the CUDA library."""

    def __init__(self, cfg: RunConfig, device=None):
        if not torch.cuda.is_available():
            raise _lib.AstreaError(-2, "no CUDA device: the astrea_gb300 update runs only on the GPU")
        self.cfg = cfg
        self.lib = _lib.load()
        self.device = torch.device(device or "cuda")
        with torch.cuda.device(self.device):
            h = ctypes.c_void_p()
            c = cfg.to_c()
            _lib.check(self.lib.astrea_create(ctypes.byref(c), ctypes.byref(h)))
            self.handle = h
            nv = ctypes.c_int()
            cells = ctypes.c_longlong()
            _lib.check(self.lib.astrea_layout(self.handle, ctypes.byref(nv), ctypes.byref(cells)))
            self.nv = nv.value
            n1 = cfg.n1 if cfg.dim == 2 else 1
            self.state = torch.zeros((self.nv, cfg.n0, n1), dtype=cfg.dtype, device=self.device)

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                torch.cuda.synchronize(self.device)
            except Exception:
                pass
            self.lib.astrea_destroy(h)
            self.handle = None

    # -- state in/out ---------------------------------------------------------
    def load_conservative(self, grid):
        """Set the state from a reference-layout conservative grid (n0[, n1], 8)."""
        self.state.copy_(to_planes(grid, self.cfg.model, self.cfg.dtype, self.device))

    def load_planes(self, planes):
        self.state.copy_(planes)

    def initialise(self, w_point):
        """Point primitives (n0[, n1], 8) -> cell-averaged conservatives (constructor.initialise :105-109)."""
        prim = to_planes(w_point, self.cfg.model, self.cfg.dtype, self.device)
        _lib.check(self.lib.astrea_initialise(self.handle, ctypes.c_void_p(prim.data_ptr()),
                                              ctypes.c_void_p(self.state.data_ptr()), _stream()))
        torch.cuda.current_stream().synchronize()

    def initialise_planes(self, prim):
        """Point primitives already in the state layout (nv, n0, n1) on the device -> cell-averaged conservatives."""
        prim = prim.to(dtype=self.cfg.dtype).contiguous()
        _lib.check(self.lib.astrea_initialise(self.handle, ctypes.c_void_p(prim.data_ptr()),
                                              ctypes.c_void_p(self.state.data_ptr()), _stream()))
        torch.cuda.current_stream().synchronize()

    def conservative(self):
        """The state as a reference-layout (n0[, n1], 8) tensor."""
        return from_planes(self.state, self.cfg.model, self.cfg.dim)

    def primitive(self):
        """sim_variables.convert_conservative of the state (the per-step snapshot of astrea.py:47)."""
        out = torch.empty_like(self.state)
        _lib.check(self.lib.astrea_to_primitive(self.handle, ctypes.c_void_p(self.state.data_ptr()),
                                                ctypes.c_void_p(out.data_ptr()), _stream()))
        return from_planes(out, self.cfg.model, self.cfg.dim)

    def primitive_planes(self):
        """The primitive snapshot as the model's planes on the device (for astrea_gb300.diagnostics)."""
        out = torch.empty_like(self.state)
        _lib.check(self.lib.astrea_to_primitive(self.handle, ctypes.c_void_p(self.state.data_ptr()),
                                                ctypes.c_void_p(out.data_ptr()), _stream()))
        return out

    # -- time stepping ----------------------------------------------------------
    def reset_clock(self, t=0.0, idx=1, order=0):
        _lib.check(self.lib.astrea_reset_clock(self.handle, float(t), int(idx), int(order), _stream()))

    def step(self, n=1, graph=True):
        """Enqueue ``n`` steps of the core_run loop body (asynchronous)."""
        fn = self.lib.astrea_graph_step if graph else self.lib.astrea_step
        _lib.check(fn(self.handle, ctypes.c_void_p(self.state.data_ptr()), int(n), _stream()))

    def step_host(self, host_in, host_out):
        """One step with the state taken from ``host_in`` and the result left in ``host_out`` (host
        tensors in the state layout; page-locked ones let the last sweep write the result directly)."""
        vp = ctypes.c_void_p
        _lib.check(self.lib.astrea_step_host(self.handle, vp(self.state.data_ptr()),
                                             vp(host_in.data_ptr() if host_in is not None else 0),
                                             vp(host_out.data_ptr() if host_out is not None else 0), _stream()))

    def clock(self):
        t, dt = ctypes.c_double(), ctypes.c_double()
        steps, done, status = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _lib.check(self.lib.astrea_get_clock(self.handle, ctypes.byref(t), ctypes.byref(dt), ctypes.byref(steps),
                                             ctypes.byref(done), ctypes.byref(status), _stream()))
        return {"t": t.value, "dt": dt.value, "steps": steps.value, "done": bool(done.value), "status": status.value}

    def run(self, max_steps=None, check_every=32, graph=True):
        """Advance until t reaches t_end (or ``max_steps``); returns the clock."""
        done_steps = 0
        while True:
            n = check_every if max_steps is None else min(check_every, max_steps - done_steps)
            if n <= 0:
                break
            self.step(n, graph=graph)
            done_steps += n
            c = self.clock()
            if c["status"]:
                raise _lib.AstreaError(-4, f"non-finite wave speed or dt at t={c['t']}")
            if c["done"]:
                break
        return self.clock()

    # -- reference evolver interface ----------------------------------------------
    def space(self, order=0):
        """evolve_space: per-axis interface fluxes (planes, sweep-index major) and eigmax."""
        cfg = self.cfg
        n1 = cfg.n1 if cfg.dim == 2 else 1
        f0 = torch.empty((self.nv, cfg.n0 + 1, n1), dtype=cfg.dtype, device=self.device)
        f1 = torch.empty((self.nv, n1 + 1, cfg.n0), dtype=cfg.dtype, device=self.device) if cfg.dim == 2 else None
        eig = (ctypes.c_double * 2)()
        _lib.check(self.lib.astrea_space(self.handle, ctypes.c_void_p(self.state.data_ptr()), int(order),
                                         ctypes.c_void_p(f0.data_ptr()),
                                         ctypes.c_void_p(f1.data_ptr() if f1 is not None else 0), eig, _stream()))
        return (f0, f1), (eig[0], eig[1])

    def space_ct(self, order=0):
        """evolve_space of a constrained-transport grid: fluxes, eigmax, each sweep's face
        values (2, 8, n0, n1) and the corner field E_z (n0, n1), physical layout."""
        cfg = self.cfg
        f0 = torch.empty((self.nv, cfg.n0 + 1, cfg.n1), dtype=cfg.dtype, device=self.device)
        f1 = torch.empty((self.nv, cfg.n1 + 1, cfg.n0), dtype=cfg.dtype, device=self.device)
        faces = torch.empty((2, 8, cfg.n0, cfg.n1), dtype=cfg.dtype, device=self.device)
        corner = torch.empty((cfg.n0, cfg.n1), dtype=cfg.dtype, device=self.device)
        eig = (ctypes.c_double * 2)()
        vp = ctypes.c_void_p
        _lib.check(self.lib.astrea_space_ct(self.handle, vp(self.state.data_ptr()), int(order), vp(f0.data_ptr()),
                                            vp(f1.data_ptr()), eig, vp(faces[0].data_ptr()), vp(faces[1].data_ptr()),
                                            vp(corner.data_ptr()), _stream()))
        return (f0, f1), (eig[0], eig[1]), faces, corner

    def time(self, dt, order=0):
        """evolve_time with the given dt, in place on the state."""
        _lib.check(self.lib.astrea_time(self.handle, ctypes.c_void_p(self.state.data_ptr()), float(dt), int(order),
                                        _stream()))

    def sweep_tiles(self):
        """The (cells along, rows across) tile of each axis's sweep kernel (tuned at the first step)."""
        out = []
        for ax in range(self.cfg.dim):
            ts, tt = ctypes.c_int(), ctypes.c_int()
            _lib.check(self.lib.astrea_sweep_tile(self.handle, ax, ctypes.byref(ts), ctypes.byref(tt)))
            out.append((ts.value, tt.value))
        return out

    def conserved_sums(self):
        """Neumaier-compensated FP64 sums of the stored variables."""
        out = (ctypes.c_double * self.nv)()
        _lib.check(self.lib.astrea_reduce_conserved(self.handle, ctypes.c_void_p(self.state.data_ptr()), out,
                                                    _stream()))
        return np.array(out[:], dtype=np.float64)

    def describe(self):
        return asdict(self.cfg)
