"""ctypes binding of the C ABI declared in include/astrea_gb300.h.

The library is built in-tree (``astrea_gb300/_lib/libastrea_gb300.so``, see
``astrea_gb300.build``).  There is no CPU fallback: if the library is missing
or fails to load, every entry point raises.
"""

import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libastrea_gb300.so")

EXPORTS = [
    "astrea_version", "astrea_last_error", "astrea_create", "astrea_destroy", "astrea_layout", "astrea_initialise",
    "astrea_reset_clock", "astrea_step", "astrea_graph_step", "astrea_get_clock", "astrea_space", "astrea_time",
    "astrea_to_primitive", "astrea_reduce_conserved", "astrea_step_timed", "astrea_reduce_conserved_static",
    "astrea_sweep_tile", "astrea_point_state", "astrea_total_variation", "astrea_solution_error",
    "astrea_clock_async", "astrea_space_ct", "astrea_step_host",
]


class AstreaError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"astrea error {code}: {msg}")
        self.code = code


class Cfg(ctypes.Structure):
    _fields_ = [
        ("dim", ctypes.c_int), ("n0", ctypes.c_int), ("n1", ctypes.c_int), ("model", ctypes.c_int),
        ("precision", ctypes.c_int), ("scheme", ctypes.c_int), ("solver", ctypes.c_int),
        ("integrator", ctypes.c_int), ("boundary", ctypes.c_int), ("limiter", ctypes.c_int),
        ("gamma", ctypes.c_double), ("dx", ctypes.c_double), ("cfl", ctypes.c_double), ("t_end", ctypes.c_double),
        ("checkpoints", ctypes.c_int), ("flags", ctypes.c_int),
    ]


_lock = threading.Lock()
_lib = None


def load(path=LIB_PATH):
    """Load (once) and return the shared library; raise if it is not built."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(path):
            raise AstreaError(-2, f"CUDA library not built: {path} (run `python -m astrea_gb300.build`)")
        lib = ctypes.CDLL(path)
        vp, i, d = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
        ip, dp, llp = ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_longlong)
        sig = {
            "astrea_version": ([], i),
            "astrea_last_error": ([], ctypes.c_char_p),
            "astrea_create": ([ctypes.POINTER(Cfg), ctypes.POINTER(vp)], i),
            "astrea_destroy": ([vp], None),
            "astrea_layout": ([vp, ip, llp], i),
            "astrea_initialise": ([vp, vp, vp, vp], i),
            "astrea_reset_clock": ([vp, d, i, i, vp], i),
            "astrea_step": ([vp, vp, i, vp], i),
            "astrea_graph_step": ([vp, vp, i, vp], i),
            "astrea_step_host": ([vp, vp, vp, vp, vp], i),
            "astrea_get_clock": ([vp, dp, dp, ip, ip, ip, vp], i),
            "astrea_clock_async": ([vp, vp, vp, vp, vp], i),
            "astrea_space": ([vp, vp, i, vp, vp, dp, vp], i),
            "astrea_space_ct": ([vp, vp, i, vp, vp, dp, vp, vp, vp, vp], i),
            "astrea_time": ([vp, vp, d, i, vp], i),
            "astrea_to_primitive": ([vp, vp, vp, vp], i),
            "astrea_reduce_conserved": ([vp, vp, dp, vp], i),
            "astrea_reduce_conserved_static": ([vp, i, ctypes.c_longlong, i, dp, vp], i),
            "astrea_sweep_tile": ([vp, i, ip, ip], i),
            "astrea_step_timed": ([vp, vp, i, dp, ip, vp], i),
        }
        for name, (args, res) in sig.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = res
        _lib = lib
        return lib


def check(rc):
    if rc != 0:
        msg = load().astrea_last_error().decode(errors="replace")
        raise AstreaError(rc, msg)
    return rc
