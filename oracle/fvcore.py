"""Finite-volume primitives of the oracle (test infrastructure only).

Arrays are in a *sweep frame*: axis 0 is the sweep axis, axis 1 (2D only) the
transverse axis, the last axis holds the eight variables
``[rho, v_x|m_x, v_y|m_y, v_z|m_z, p|E, B_x, B_y, B_z]``.

Every function states the reference lines whose arithmetic it restates; the
operation order (left-to-right, no re-association, no fused multiply-add) is
kept so that FP64 results match the reference bit for bit.
"""

import numpy as np

C24 = 1 / 24  # Laplacian weight of the average<->centre conversions (fv.py:287-289)


# --------------------------------------------------------------------------
# boundary-mapped gathers (fv.add_boundary, fv.py:57-61, applied per intermediate)
# --------------------------------------------------------------------------

def bc_index(n, idx, bc):
    """Map virtual indices onto [0, n): clamp for 'edge', modulo for 'wrap'."""
    idx = np.asarray(idx)
    if bc == "edge":
        return np.clip(idx, 0, n - 1)
    if bc == "wrap":
        return np.mod(idx, n)
    raise ValueError(f"unknown boundary {bc!r}")


def gather(X, offset, bc, axis=0):
    """``X[bc(i + offset)]`` for every i along ``axis`` (same length as X)."""
    n = X.shape[axis]
    return np.take(X, bc_index(n, np.arange(n) + offset, bc), axis=axis)


def gather_range(X, start, count, bc, axis=0):
    """``X[bc(start + j)]`` for j in [0, count)."""
    n = X.shape[axis]
    return np.take(X, bc_index(n, np.arange(count) + start, bc), axis=axis)


def d2(X, axis, bc):
    """Undivided second difference with one boundary-mapped neighbour each side.

    fv.derivative of a once-padded array (fv.py:41-44):
    ``(X[i+1] - X[i]) - (X[i] - X[i-1])``.
    """
    return (gather(X, 1, bc, axis) - X) - (X - gather(X, -1, bc, axis))


# --------------------------------------------------------------------------
# masked arithmetic (fv.py:17-33)
# --------------------------------------------------------------------------

def divide(a, b):
    """a/b where b != 0, else 0 (fv.divide, fv.py:19-20)."""
    a = np.asarray(a)
    b = np.asarray(b)
    out = np.zeros(np.broadcast_shapes(a.shape, b.shape), dtype=a.dtype)
    np.divide(a, b, out=out, where=(b != 0))
    return out


def nsq(v):
    """Squared Euclidean norm as the reference forms it: ``norm(v)**2``.

    ``np.linalg.norm(axis=-1)`` is ``sqrt((v0*v0 + v1*v1) + v2*v2)``; the
    reference then squares it again, so the result is ``r*r`` and not the sum.
    """
    r = np.sqrt((v[..., 0] * v[..., 0] + v[..., 1] * v[..., 1]) + v[..., 2] * v[..., 2])
    return r * r


def norm3(v):
    """``np.linalg.norm(v, axis=-1)`` over three components: ``sqrt((v0*v0 + v1*v1) + v2*v2)``."""
    return np.sqrt((v[..., 0] * v[..., 0] + v[..., 1] * v[..., 1]) + v[..., 2] * v[..., 2])


def vdot(a, b):
    """``np.sum(a*b, axis=-1)`` over three components, sequential order."""
    p = a * b
    return (p[..., 0] + p[..., 1]) + p[..., 2]


# --------------------------------------------------------------------------
# primitive <-> conservative (fv.py:49-53, 89-101)
# --------------------------------------------------------------------------

def p2c(w, gamma):
    """Pointwise primitive -> conservative (fv.point_convert_primitive, fv.py:89-93)."""
    q = np.copy(w)
    q[..., 4] = w[..., 4] / (gamma - 1) + .5 * (w[..., 0] * nsq(w[..., 1:4]) + nsq(w[..., 5:8]))
    q[..., 1:4] = w[..., 1:4] * w[..., 0][..., None]
    return q


def c2p(q, gamma):
    """Pointwise conservative -> primitive (fv.point_convert_conservative, fv.py:97-101)."""
    w = np.copy(q)
    v = divide(q[..., 1:4], q[..., 0][..., None])
    w[..., 4] = (gamma - 1) * (q[..., 4] - .5 * (q[..., 0] * nsq(v) + nsq(q[..., 5:8])))
    w[..., 1:4] = v
    return w


def ho_c2p(q, gamma, bc, axes):
    """4th-order average conservative -> average primitive.

    fv.high_order_convert_conservative (fv.py:126-143).  ``axes`` lists the
    frame axes in the order the reference visits them: the sweep axis first,
    then the transverse axis (2D cell arrays), or only the transverse axis
    (2D face arrays), or none (1D face arrays).
    """
    w = np.zeros_like(q)
    qq = np.copy(q)
    for ax in axes:
        qq = qq - C24 * d2(q, ax, bc)
        w = w + C24 * d2(c2p(q, gamma), ax, bc)
    return c2p(qq, gamma) + w


def ho_p2c(w, gamma, bc, axes):
    """4th-order average primitive -> average conservative.

    fv.high_order_convert_primitive (fv.py:105-122).
    """
    q = np.zeros_like(w)
    ww = np.copy(w)
    for ax in axes:
        ww = ww - C24 * d2(w, ax, bc)
        q = q + C24 * d2(p2c(w, gamma), ax, bc)
    return p2c(ww, gamma) + q


def avg_to_centre(X, bc, axes):
    """``X - 1/24 d2 X`` over ``axes`` (fv.high_order_convert('avg'), fv.py:67-85)."""
    Y = np.copy(X)
    for ax in axes:
        Y = Y - C24 * d2(X, ax, bc)
    return Y


def centre_to_avg(X, bc, axes):
    """``X + 1/24 d2 X`` over ``axes`` (fv.high_order_convert('cntr'), fv.py:67-85)."""
    Y = np.copy(X)
    for ax in axes:
        Y = Y + C24 * d2(X, ax, bc)
    return Y


def flux_centre(F_centre, F_avg, bc, dim):
    """``F_c - 1/24 d2_perp F_avg`` (fv.high_order_compute_flux, fv.py:147-153)."""
    F = np.copy(F_centre)
    for ax in range(1, dim):
        F = F - C24 * d2(F_avg, ax, bc)
    return F


# --------------------------------------------------------------------------
# physical flux, interface averages (constructor.py:113-176)
# --------------------------------------------------------------------------

def make_flux(w, gamma, axis):
    """Ideal-MHD physical flux along ``axis`` from primitives (constructor.make_flux, :113-125)."""
    a, o, p = axis % 3, (axis + 1) % 3, (axis + 2) % 3
    rho, v, P, B = w[..., 0], w[..., 1:4], w[..., 4], w[..., 5:8]
    F = np.zeros_like(w)
    F[..., 0] = rho * v[..., axis]
    F[..., a + 1] = rho * v[..., axis] ** 2 + P + .5 * nsq(B) - B[..., axis] ** 2
    F[..., o + 1] = rho * v[..., axis] * v[..., o] - B[..., axis] * B[..., o]
    F[..., p + 1] = rho * v[..., axis] * v[..., p] - B[..., axis] * B[..., p]
    F[..., 4] = v[..., axis] * (.5 * rho * nsq(v) + (gamma * P) / (gamma - 1) + nsq(B)) - B[..., axis] * vdot(v, B)
    F[..., o + 5] = B[..., o] * v[..., axis] - B[..., axis] * v[..., o]
    F[..., p + 5] = B[..., p] * v[..., axis] - B[..., axis] * v[..., p]
    return F


def arith_average(w_plus, w_minus):
    """PLM interface state ``.5*(w+ + w-)`` (plm.py:45)."""
    return .5 * (w_plus + w_minus)


def roe_average(w_plus, w_minus):
    """sqrt(rho)-weighted interface state (constructor.make_Roe_average, :167-176).

    Note the reference weights B with the *opposite* square roots to v and p.
    """
    with np.errstate(invalid="ignore"):
        r_m = np.sqrt(w_minus[..., 0])
        r_p = np.sqrt(w_plus[..., 0])
    avg = np.zeros_like(w_plus)
    den = r_m + r_p
    avg[..., 0] = r_m * r_p
    avg[..., 1:4] = divide(w_plus[..., 1:4] * r_p[..., None] + w_minus[..., 1:4] * r_m[..., None], den[..., None])
    avg[..., 4] = divide(r_p * w_plus[..., 4] + r_m * w_minus[..., 4], den)
    avg[..., 5:8] = divide(w_plus[..., 5:8] * r_m[..., None] + w_minus[..., 5:8] * r_p[..., None], den[..., None])
    return avg


# --------------------------------------------------------------------------
# wave speeds (fv.compute_eigen + constructor.make_Jacobian, fv.py:157-168, :129-163)
# --------------------------------------------------------------------------

def primitive_jacobian(w, gamma, axis):
    """8x8 primitive-variable Jacobian along ``axis`` (constructor.make_Jacobian, :129-163)."""
    a, o, p = axis % 3, (axis + 1) % 3, (axis + 2) % 3
    rho, v, P, B = w[..., 0], w[..., 1:4], w[..., 4], w[..., 5:8]
    J = np.zeros(w.shape + (8,), dtype=w.dtype)
    for k in range(8):
        J[..., k, k] = v[..., a]
    J[..., 0, a + 1] = rho
    with np.errstate(divide="ignore"):
        J[..., a + 1, 4] = 1 / rho
    J[..., 4, a + 1] = gamma * P
    J[..., a + 5, a + 5] = 0
    J[..., a + 1, a + 5] = -divide(B[..., a], rho)
    J[..., a + 1, o + 5] = divide(B[..., o], rho)
    J[..., a + 1, p + 5] = divide(B[..., p], rho)
    J[..., o + 1, o + 5] = -divide(B[..., a], rho)
    J[..., p + 1, p + 5] = -divide(B[..., a], rho)
    J[..., o + 1, a + 5] = -divide(B[..., o], rho)
    J[..., p + 1, a + 5] = -divide(B[..., p], rho)
    J[..., o + 5, a + 1] = B[..., o]
    J[..., p + 5, a + 1] = B[..., p]
    J[..., 4, a + 5] = (gamma - 1) * vdot(v, B)
    J[..., o + 5, o + 1] = -B[..., a]
    J[..., p + 5, p + 1] = -B[..., a]
    J[..., o + 5, a + 5] = -v[..., o]
    J[..., p + 5, a + 5] = -v[..., p]
    return J


def max_speed_lapack(w, gamma, axis):
    """Largest |eigenvalue| of the primitive Jacobian by LAPACK, as the reference does."""
    J = primitive_jacobian(w, gamma, axis)
    with np.errstate(all="ignore"):
        return np.max(np.abs(np.linalg.eigvals(J)), axis=-1)


def max_speed_analytic(w, gamma, axis):
    """Largest |eigenvalue| of the same Jacobian in closed form: ``|v_n| + c_f``.

    The Jacobian's B_n row is zero (one eigenvalue 0); the remaining 7x7 block
    is the standard primitive MHD matrix with eigenvalues v_n, v_n +- c_a,
    v_n +- c_s, v_n +- c_f.  A negative ``gamma p / rho`` (unphysical state)
    makes the sound pair complex, ``v_n +- i sqrt(-a2)``, whose modulus is
    returned instead, like the modulus LAPACK's eigenvalues would give.
    This is the formula the CUDA kernels evaluate (same operation order).
    """
    rho, v, P, B = w[..., 0], w[..., 1:4], w[..., 4], w[..., 5:8]
    vn = v[..., axis % 3]
    with np.errstate(all="ignore"):
        a2 = (gamma * P) / rho
        b2 = nsq(B) / rho
        bn2 = (B[..., axis % 3] * B[..., axis % 3]) / rho
        s = a2 + b2
        cf2 = .5 * (s + np.sqrt(s * s - 4 * a2 * bn2))
        fast = np.abs(vn) + np.sqrt(cf2)
        cplx = np.sqrt(vn * vn - a2)
    out = np.where(a2 < 0, np.maximum(cplx, np.abs(vn)), fast)
    return out


def max_speed(w, gamma, axis, mode):
    if mode == "lapack":
        return max_speed_lapack(w, gamma, axis)
    if mode == "analytic":
        return max_speed_analytic(w, gamma, axis)
    raise ValueError(mode)
