"""Diagnostics of the solution (functions/analytic.py), the reductions on the device.

``total_variation`` and ``solution_error`` take primitive snapshots as the
model's planes on the device (``Solver.primitive`` gives the reference layout;
``Solver.primitive_planes`` the planes) and return the ten quantities of the
reference: the eight primitives, the specific total energy and the specific
internal energy.  ``sod_exact`` is the reference's Sod solution (a scalar
root-find and a fill on the host; it is not a reduction).
"""

import ctypes

import numpy as np
import scipy.optimize

from . import _lib
from .solver import _stream


def _lib_diag():
    lib = _lib.load()
    d, i, vp = ctypes.c_double, ctypes.c_int, ctypes.c_void_p
    lib.astrea_total_variation.argtypes = [vp, i, i, i, i, i, d, ctypes.POINTER(d), vp]
    lib.astrea_total_variation.restype = i
    lib.astrea_solution_error.argtypes = [vp, vp, i, i, i, i, i, d, d, ctypes.POINTER(d), vp]
    lib.astrea_solution_error.restype = i
    return lib


def _shape(planes, dim):
    nv, n0, n1 = planes.shape
    return nv, n0, (n1 if dim == 2 else 1), (64 if planes.element_size() == 8 else 32)


def total_variation(planes, dim, gamma):
    """calculate_TV (analytic.py:48-63) of one snapshot: 10 sums of |differences|."""
    nv, n0, n1, prec = _shape(planes, dim)
    out = (ctypes.c_double * 10)()
    _lib.check(_lib_diag().astrea_total_variation(ctypes.c_void_p(planes.contiguous().data_ptr()), prec, nv, dim, n0, n1,
                                                  float(gamma), out, _stream()))
    return np.array(out[:])


def solution_error(planes, ref_planes, dim, gamma, norm=1):
    """calculate_solution_error (analytic.py:24-45): L1 (norm <= 0), max (norm > 10) or L_norm, per quantity."""
    nv, n0, n1, prec = _shape(planes, dim)
    out = (ctypes.c_double * 10)()
    _lib.check(_lib_diag().astrea_solution_error(ctypes.c_void_p(planes.contiguous().data_ptr()),
                                                 ctypes.c_void_p(ref_planes.contiguous().data_ptr()), prec, nv, dim, n0,
                                                 n1, float(gamma), float(norm), out, _stream()))
    return np.array(out[:])


def _round_off(value):
    # analytic.round_off: rounds half up by the fractional part of value % int(value)
    if value % int(value) >= .5:
        return int(value) + 1
    return int(value)


def sod_exact(grid, t, gamma, start_pos, end_pos, shock_pos):
    """calculate_Sod_analytical (analytic.py:98-155): the exact Sod solution on ``grid``'s cells at time t.

    ``grid`` is a 1D primitive grid (N, 8) whose first and last cells hold the
    left and right initial states.  Same construction as the reference: fsolve
    for the post-shock pressure from (P5 - P1)/2, region boundaries by its
    rounding, the rarefaction sampled by a linspace.
    """
    grid = np.asarray(grid, dtype=np.float64)
    arr = np.zeros_like(grid)
    rho5, vx5, vy5, vz5, P5, Bx5, By5, Bz5 = grid[0]
    rho1, vx1, vy1, vz1, P1, Bx1, By1, Bz1 = grid[-1]
    cs5, cs1 = np.sqrt(gamma * P5 / rho5), np.sqrt(gamma * P1 / rho1)
    mu, beta = (gamma - 1) / (gamma + 1), 2 / (gamma - 1)

    def f(x):
        return (((x / P1) - 1) * np.sqrt((1 - mu) / (gamma * (mu + (x / P1))))) - (
            beta * (cs5 / cs1) * (1 - ((x / P5) ** (1 / (gamma * beta)))))

    P2 = scipy.optimize.fsolve(f, (P5 - P1) / 2)[0]
    rho2, rho3 = rho1 * ((P2 + (mu * P1)) / (P1 + (mu * P2))), rho5 * (P2 / P5) ** (1 / gamma)
    vx2 = (beta * cs5) * (1 - (P2 / P5) ** (1 / (gamma * beta)))
    v_t = cs5 - (vx2 / (1 - mu))
    v_s = vx2 / (1 - (rho1 / rho2))
    n, width = len(grid), end_pos - start_pos
    b54 = _round_off(((shock_pos - (cs5 * t) - start_pos) / width) * n)
    b43 = _round_off(((shock_pos - (v_t * t) - start_pos) / width) * n)
    b32 = _round_off(((shock_pos + (vx2 * t) - start_pos) / width) * n)
    b21 = _round_off(((shock_pos + (v_s * t) - start_pos) / width) * n)
    rare = _round_off(((cs5 * t - v_t * t) / width) * n)
    if rare - (b43 - b54) < 0:
        rare += 1
    elif rare - (b43 - b54) > 0:
        rare -= 1
    rarefaction = np.linspace(shock_pos - (cs5 * t), shock_pos - (v_t * t), rare) - shock_pos
    arr[:b54] = grid[0]
    arr[b21:] = grid[-1]
    arr[b43:b21, 1] = vx2
    arr[b43:b21, 4] = P2
    arr[b43:b32, 0] = rho3
    arr[b32:b21, 0] = rho2
    arr[b54:b43, 0] = rho5 * ((1 - mu) - mu * rarefaction / (cs5 * t)) ** beta
    arr[b54:b43, 4] = P5 * ((1 - mu) - mu * rarefaction / (cs5 * t)) ** (gamma * beta)
    arr[b54:b43, 1] = (1 - mu) * (cs5 + (rarefaction / t))
    return arr
