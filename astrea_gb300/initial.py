"""Initial conditions built on the device (functions/constructor.py:11-109).

``constructor.initialise`` fills the point primitives of a test problem from
the values the test table puts into ``sim_variables`` (``initial_left``,
``initial_right``, ``start_pos``, ``end_pos``, ``shock_pos``, ``misc``) and a
dispatch on the config name, then converts them to cell averages.  Here the
same dispatch picks an ``astrea_ic`` kind, a kernel evaluates the point
primitives per cell on the GPU, and ``astrea_initialise`` forms the averages:
nothing grid-sized crosses the bus.
"""

import ctypes

import numpy as np
import torch

from . import _lib
from .solver import MODEL_VARS, _stream

SPLIT, RADIAL, GAUSS, KHI, VORTEX, QUADRANT, OT, SHU, SINE, LINEAR, LINEAR_MHD = range(11)


class IC(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("abs_mask", ctypes.c_int), ("dim", ctypes.c_int), ("n", ctypes.c_int),
                ("start", ctypes.c_double), ("end", ctypes.c_double), ("shock", ctypes.c_double),
                ("left", ctypes.c_double * 8), ("right", ctypes.c_double * 8),
                ("bottom_left", ctypes.c_double * 8), ("bottom_right", ctypes.c_double * 8),
                ("ampl", ctypes.c_double), ("freq", ctypes.c_double), ("y_offset", ctypes.c_double),
                ("fwhm", ctypes.c_double), ("peak_pos", ctypes.c_double), ("perturb_ampl", ctypes.c_double),
                ("vortex_str", ctypes.c_double), ("omega", ctypes.c_double), ("gamma", ctypes.c_double)]


def kind_of(config, dim):
    """(kind, abs_mask) of a config name, following constructor.initialise's tests (constructor.py:28-99)."""
    config = config.lower()
    if dim == 2:
        if config == "sedov" or "blast" in config:
            return RADIAL, 0
        if config.startswith("gauss"):
            return GAUSS, 0
        if config in ["khi", "kelvin-helmholtz"] or ("kelvin" in config or "helmholtz" in config):
            return KHI, 0
        if config in ["ivc", "vortex", "isentropic vortex"]:
            return VORTEX, 0
        if "ll" in config or "lax-liu" in config:
            return QUADRANT, 0
        if config in ["orszag-tang", "orszag", "tang", "ot"]:
            return OT, 0
        if "rotor" in config:
            return RADIAL, 0  # the reference's rotor velocity assignment writes into a copy (constructor.py:71-72)
        return SPLIT, 0
    abs_mask = 1 if (config == "sedov" or config.startswith("sq")) else 0
    if "shu" in config or "osher" in config:
        return SHU, abs_mask
    if config.startswith("sin"):
        return SINE, abs_mask
    if config.startswith("gauss"):
        return GAUSS, abs_mask
    if config.startswith("lin"):
        return (LINEAR_MHD if "mhd" in config else LINEAR), abs_mask
    return SPLIT, abs_mask


def ic_of(sim_variables):
    """The ``astrea_ic`` of a reference ``sim_variables`` namedtuple (or any object with the same fields)."""
    sv = sim_variables
    dim = int(sv.dimension)
    kind, abs_mask = kind_of(str(sv.config), dim)
    c = IC(kind=kind, abs_mask=abs_mask, dim=dim, n=int(sv.cells), start=float(sv.start_pos), end=float(sv.end_pos),
           shock=float(sv.shock_pos), gamma=float(sv.gamma))
    for name, src in (("left", sv.initial_left), ("right", sv.initial_right)):
        arr = getattr(c, name)
        for k, v in enumerate(np.asarray(src, dtype=np.float64).ravel()[:8]):
            arr[k] = v
    misc = getattr(sv, "misc", None) or {}
    for key in ("ampl", "freq", "y_offset", "fwhm", "peak_pos", "perturb_ampl", "vortex_str", "omega"):
        if key in misc:
            setattr(c, key, float(misc[key]))
    for key in ("bottom_left", "bottom_right"):
        if key in misc:
            arr = getattr(c, key)
            for k, v in enumerate(np.asarray(misc[key], dtype=np.float64).ravel()[:8]):
                arr[k] = v
    return c


def _lib_ic():
    lib = _lib.load()
    fn = lib.astrea_point_state
    fn.argtypes = [ctypes.POINTER(IC), ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    return lib


def point_planes(ic, model, precision=64, device="cuda"):
    """Point primitives of ``ic`` as the model's planes (nv, n0, n1) on the device."""
    if not torch.cuda.is_available():
        raise _lib.AstreaError(-2, "no CUDA device: the astrea_gb300 initial conditions are built on the GPU")
    lib = _lib_ic()
    n1 = ic.n if ic.dim == 2 else 1
    dtype = torch.float64 if precision == 64 else torch.float32
    out = torch.empty((model, ic.n, n1), dtype=dtype, device=device)
    _lib.check(lib.astrea_point_state(ctypes.byref(ic), precision, model, ctypes.c_void_p(out.data_ptr()), _stream()))
    return out


def point_primitives(sim_variables, model=8, precision=64, device="cuda"):
    """The reference's point primitive grid (n[, n], 8) of ``sim_variables``, built on the device."""
    ic = ic_of(sim_variables)
    planes = point_planes(ic, model, precision, device)
    shape = (ic.n, ic.n if ic.dim == 2 else 1, 8)
    out = torch.zeros(shape, dtype=planes.dtype, device=planes.device)
    out[..., MODEL_VARS[model]] = planes.permute(1, 2, 0)
    return out[:, 0, :] if ic.dim == 1 else out


def initialise(solver, sim_variables):
    """Fill ``solver``'s state with the cell-averaged conservatives of the test problem (constructor.initialise
    with convert=True, constructor.py:105-109), without a host round trip."""
    ic = ic_of(sim_variables)
    cfg = solver.cfg
    if ic.dim != cfg.dim or ic.n != cfg.n0:
        raise ValueError("the solver's grid does not match sim_variables")
    planes = point_planes(ic, cfg.model, cfg.precision, solver.state.device)
    solver.initialise_planes(planes)
    return solver
