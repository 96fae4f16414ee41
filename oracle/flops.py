"""Floating-point operation count of one oracle step (test infrastructure).

The algorithmic operation count per cell-update of a workload: one SSPRK3
step of the oracle, with every NumPy ufunc call on the state's arrays
counted.  add, subtract, multiply, divide, square root, square and power
count one operation per output element; comparisons, minimum/maximum,
absolute value, sign and selections count none (the GPU counters the kernels
are measured with count the same way: FP adds, multiplies and two per fused
multiply-add).  The oracle's arrays are wrapped in an ndarray subclass that
counts through ``__array_ufunc__``; the oracle modules' ``numpy`` is swapped
for a view of NumPy whose constructors keep the subclass while counting.

Run:  python -m oracle.flops        (prints the counts of the workloads)
"""

import contextlib
import sys

import numpy as np

from . import ct, fvcore, recon, riemann, stepper

_OPS = {np.add: 1, np.subtract: 1, np.multiply: 1, np.true_divide: 1, np.sqrt: 1, np.square: 1, np.power: 1,
        np.reciprocal: 1}


class _Tally:
    ops = 0


def _base(x):
    if isinstance(x, Counted):
        return x.view(np.ndarray)
    if isinstance(x, tuple):
        return tuple(_base(v) for v in x)
    if isinstance(x, list):
        return [_base(v) for v in x]
    if isinstance(x, dict):
        return {k: _base(v) for k, v in x.items()}
    return x


def _wrap(x):
    if isinstance(x, np.ndarray) and not isinstance(x, Counted) and x.dtype.kind == "f":
        return x.view(Counted)
    if isinstance(x, tuple):
        return tuple(_wrap(v) for v in x)
    if isinstance(x, list):
        return [_wrap(v) for v in x]
    return x


class Counted(np.ndarray):
    """A float array whose arithmetic is tallied in ``_Tally.ops``."""

    def __array_ufunc__(self, ufunc, method, *inputs, **kwargs):
        args = [_base(x) for x in inputs]
        if "out" in kwargs:
            kwargs["out"] = tuple(_base(o) for o in kwargs["out"])
        res = getattr(ufunc, method)(*args, **kwargs)
        w = _OPS.get(ufunc, 0)
        if w:
            if method == "__call__":
                first = res[0] if isinstance(res, tuple) else res
                n = np.size(first)
                where = kwargs.get("where", True)
                if where is not True:
                    n = int(np.count_nonzero(np.broadcast_to(_base(where), np.shape(first))))
                _Tally.ops += w * n
            elif method == "reduce":
                _Tally.ops += w * max(0, np.size(args[0]) - np.size(res))
        return _wrap(res)

    def __array_function__(self, func, types, args, kwargs):
        res = func(*_base(args), **_base(kwargs))
        if func in (np.sum, np.prod, np.mean, np.cumsum):
            # reductions through the function interface: one operation per element folded in
            _Tally.ops += max(0, np.size(_base(args[0])) - (np.size(res) if func is not np.cumsum else 0))
        return _wrap(res)


class _CountingNumpy:
    """NumPy as the oracle modules see it while counting: asarray keeps the subclass, and
    zeros / empty / ones / full make counted arrays."""

    def __getattr__(self, name):
        if name == "asarray":
            return np.asanyarray
        if name in ("zeros", "empty", "ones", "full"):
            make = getattr(np, name)
            return lambda *a, **k: _wrap(make(*a, **k))
        return getattr(np, name)


@contextlib.contextmanager
def counting():
    mods = [ct, fvcore, recon, riemann, stepper]
    saved = [m.np for m in mods]
    proxy = _CountingNumpy()
    try:
        for m in mods:
            m.np = proxy
        _Tally.ops = 0
        yield _Tally
    finally:
        for m, s in zip(mods, saved):
            m.np = s


def ops_per_cell_update(w_point, cfg):
    """Operations of one oracle step per cell, for point primitives ``w_point`` under ``cfg``."""
    q = stepper.initialise(w_point, cfg)
    cells = int(np.prod(q.shape[:-1]))
    with counting() as tally, np.errstate(all="ignore"):
        stepper.step(q.view(Counted), cfg, 0.0, 1, list(range(cfg.dim)))
        ops = tally.ops
    return ops / cells


def shear_point(n, seed=20261203):
    rng = np.random.default_rng(seed)
    x = (np.arange(n) + .5) / n
    X, Y = np.meshgrid(x, x, indexing="ij")
    w = np.zeros((n, n, 8))
    inner = np.abs(Y - .5) < .25
    w[..., 0] = np.where(inner, 2.0, 1.0)
    w[..., 1] = np.where(inner, .5, -.5)
    w[..., 2] = .01 * np.sin(4 * np.pi * X) + rng.uniform(-1e-3, 1e-3, size=(n, n))
    w[..., 4] = 2.5
    return w


def headline_cfg(n):
    return stepper.OracleConfig(dim=2, scheme="ppm", solver="hllc", integrator="ssprk33", gamma=1.4, bc="wrap",
                                dx=1.0 / n, cfl=0.8, eig="analytic", t_end=1.0, compat=False, flatten=True,
                                viscosity=True)


def main(argv=None):
    n = 32
    print(f"2D shear layer {n}^2, PPM(mc) + flattening + viscosity, textbook HLLC, SSPRK3: "
          f"{ops_per_cell_update(shear_point(n), headline_cfg(n)):.1f} operations per cell-update")
    return 0


if __name__ == "__main__":
    sys.exit(main())
