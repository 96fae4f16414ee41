"""Reconstruction schemes of the oracle (test infrastructure only).

All functions work along axis 0 of a sweep-frame array of cell-averaged
primitives ``wS`` and return the left/right face values of every cell:
``wL[i]`` at face i-1/2 and ``wR[i]`` at face i+1/2.
"""

import numpy as np

from .fvcore import gather, divide


# --------------------------------------------------------------------------
# slope limiters (num_methods/limiters.py)
# --------------------------------------------------------------------------

def minmod(wS, bc):
    """minmod of the backward and forward differences (limiters.minmod_limiter, :10-19)."""
    a = wS - gather(wS, -1, bc)
    b = gather(wS, 1, bc) - wS
    same = a * b > 0
    return np.where(same & (np.abs(a) < np.abs(b)), a, np.where(same & (np.abs(a) >= np.abs(b)), b, np.zeros_like(a)))


def superbee(wS, bc):
    """Superbee-limited slope phi(r)*forward difference (limiters.superbee_limiter, :47-49)."""
    a = wS - gather(wS, -1, bc)
    b = gather(wS, 1, bc) - wS
    r = divide(a, b)
    phi = np.maximum(np.zeros_like(r), np.maximum(np.minimum(2 * r, np.ones_like(r)), np.minimum(r, np.full_like(r, 2))))
    return phi * b


def plm(wS, bc, limiter="minmod"):
    """Piecewise-linear faces ``wS -+ 0.5*slope`` (plm.py:26-36)."""
    slope = minmod(wS, bc) if limiter == "minmod" else superbee(wS, bc)
    g = .5 * slope
    return wS - g, wS + g


# --------------------------------------------------------------------------
# PPM with the McCorquodale & Colella extremum-preserving limiter
# --------------------------------------------------------------------------

def ppm_face(wS, bc):
    """4th-order face value at i+1/2 (ppm.py:38): 7/12(w_i + w_i+1) - 1/12(w_i-1 + w_i+2)."""
    return 7 / 12 * (wS + gather(wS, 1, bc)) - 1 / 12 * (gather(wS, -1, bc) + gather(wS, 2, bc))


def flatten_coefficient(wS, axis, bc, delta=.33, z0=.75, z1=.85):
    """Flattening coefficient chi per cell (1: keep the PPM faces, 0: flat).

    The reference's ``apply_flattener`` (ppm.py:111-134) cannot run (it
    returns an (N,8) array that the caller broadcasts against (N,8) again).
    This follows its formulas -- chi_bar = 1 - (z - z0)/(z1 - z0) clipped by
    z0/z1, z = |p_{i+1}-p_{i-1}| / |p_{i+2}-p_{i-2}|, then the minimum with the
    upstream neighbour by the sign of the pressure difference -- with one
    correction taken from Colella & Woodward (1984), eq. A.1-A.2, the method it
    cites: flattening applies only where the pressure jump is strong
    (|dp|/min(p) > delta) *and* the flow is compressive (u_{i-1} > u_{i+1});
    elsewhere chi_bar = 1.  (As written, ppm.py:124 sets chi_bar = 0 -- full
    flattening -- exactly where the flow is neither, which would drop smooth
    flow to first order.)  Parity unpinned.
    """
    P = wS[..., 4]
    dp1 = gather(P, 1, bc) - gather(P, -1, bc)
    dp2 = gather(P, 2, bc) - gather(P, -2, bc)
    z = divide(np.abs(dp1), np.abs(dp2))
    chi_bar = np.copy(1 - divide(z - z0, np.full_like(z, z1 - z0)))
    chi_bar[z > z1] = 0
    chi_bar[z < z0] = 1
    vn = wS[..., axis + 1]
    not_compressive = (gather(vn, -1, bc) - gather(vn, 1, bc)) <= 0
    weak = divide(np.abs(dp1), np.minimum(gather(P, 1, bc), gather(P, -1, bc))) <= delta
    chi_bar[not_compressive | weak] = 1
    sgn = np.sign(dp1)
    chi = np.copy(chi_bar)
    lo = sgn < 0
    hi = sgn > 0
    chi[lo] = np.minimum(chi_bar, gather(chi_bar, 1, bc))[lo]
    chi[hi] = np.minimum(chi_bar, gather(chi_bar, -1, bc))[hi]
    return chi


def ppm_mc(wS, bc, flatten_axis=None):
    """PPM faces limited by the McCorquodale-Colella extrapolant limiter.

    ppm.run(author='mc') (ppm.py:30-72) and limiters.extrapolant_limiter
    'mc' branch (limiters.py:82-143).  Returns (wL, wR, wF) where wF is the
    unlimited 4th-order face value at i+1/2 (the reference's data['wF']).

    The reference evaluates a second formula set when *no* cell of the whole
    array is a local extremum (limiters.py:141-143); for finite inputs that
    set gives the same numbers as the main one, so only the main one is kept.
    ``flatten_axis`` (not None) applies the flattening blend before limiting
    (the reference's ``dissipate=True`` path; parity unpinned).
    """
    C = 5 / 4
    wF = ppm_face(wS, bc)
    if flatten_axis is not None:
        eta = flatten_coefficient(wS, flatten_axis, bc)
        wF = wF * eta[..., None] + wS * (1 - eta)[..., None]
    wF_L = gather(wF, -1, bc)
    wF_R = np.copy(wF)
    w_m1, w_p1 = gather(wS, -1, bc), gather(wS, 1, bc)
    w_m2, w_p2 = gather(wS, -2, bc), gather(wS, 2, bc)

    dw_minus = wS - wF_L
    dw_plus = wF_R - wS
    wL, wR = np.copy(wF_L), np.copy(wF_R)

    d2w = 6 * (wF_L - 2 * wS + wF_R)
    d2w_C = w_m1 - 2 * wS + w_p1
    d3w = gather(d2w_C, 1, bc) - d2w_C
    extremum = (dw_minus * dw_plus <= 0) | ((wS - w_m2) * (w_p2 - wS) <= 0)

    d2C_m, d2C_p = gather(d2w_C, -1, bc), gather(d2w_C, 1, bc)
    curv = np.sign(d2w_C) * np.minimum(np.minimum(np.abs(d2w), C * np.abs(d2w_C)),
                                       np.minimum(C * np.abs(d2C_p), C * np.abs(d2C_m)))
    d2w_lim = np.zeros_like(wS)
    d2w_lim[extremum] = curv[extremum]

    scale = np.maximum(np.abs(wS), np.maximum(np.maximum(np.abs(w_m1), np.abs(w_p1)),
                                              np.maximum(np.abs(w_m2), np.abs(w_p2))))
    sensitive = np.abs(d2w) > 1e-12 * scale
    rho_lim = np.zeros_like(wS)
    phi = divide(d2w_lim, d2w)
    rho_lim[sensitive] = phi[sensitive]

    # third-derivative spread over cells i-2, i-1, i, i+2 (limiters.py:126-129)
    d3_m2, d3_m1, d3_p2 = gather(d3w, -2, bc), gather(d3w, -1, bc), gather(d3w, 2, bc)
    d3_min = np.minimum(np.minimum(d3_m1, d3w), np.minimum(d3_m2, d3_p2))
    d3_max = np.maximum(np.maximum(d3_m1, d3w), np.maximum(d3_m2, d3_p2))
    limit = (rho_lim < (1 - 1e-12)) | (.1 * np.maximum(np.abs(d3_max), np.abs(d3_min)) <= (d3_max - d3_min))

    m = (dw_minus * dw_plus < 0) & limit
    wL[m] = (wS - rho_lim * dw_minus)[m]
    wR[m] = (wS + rho_lim * dw_plus)[m]
    m = limit & (np.abs(dw_minus) >= 2 * np.abs(dw_plus))
    wL[m] = (wS - 2 * (1 - rho_lim) * dw_plus - rho_lim * dw_minus)[m]
    m = limit & (np.abs(dw_plus) >= 2 * np.abs(dw_minus))
    wR[m] = (wS + 2 * (1 - rho_lim) * dw_minus + rho_lim * dw_plus)[m]
    return wL, wR, wF


# --------------------------------------------------------------------------
# WENO-JS (schemes/weno.py:22-149)
# --------------------------------------------------------------------------

def weno(wS, bc, order=5):
    """WENO-JS faces of order 3, 5 or 7; eps = 1e-6 (weno.reconstruct, weno.py:22-149)."""
    eps = 1e-6
    z = wS
    m1, p1 = gather(wS, -1, bc), gather(wS, 1, bc)
    if order == 3:
        g0, g1 = 1 / 3, 2 / 3
        b0 = (z - m1) ** 2
        b1 = (p1 - z) ** 2
        a0 = lambda d: d / (b0 + eps) ** 2
        a1 = lambda d: d / (b1 + eps) ** 2
        wR = (a0(g0) / (a0(g0) + a1(g1))) * (1.5 * z - .5 * m1) + (a1(g1) / (a0(g0) + a1(g1))) * (.5 * z + .5 * p1)
        wL = (a1(g0) / (a0(g1) + a1(g0))) * (1.5 * z - .5 * p1) + (a0(g1) / (a0(g1) + a1(g0))) * (.5 * z + .5 * m1)
        return wL, wR
    m2, p2 = gather(wS, -2, bc), gather(wS, 2, bc)
    if order == 7:
        m3, p3 = gather(wS, -3, bc), gather(wS, 3, bc)
        g0, g1, g2, g3 = 1 / 35, 12 / 35, 18 / 35, 4 / 35
        b0 = (m3 * (547 * m3 - 3882 * m2 + 4642 * m1 - 1854 * z)
              + m2 * (7043 * m2 - 17246 * m1 + 7042 * z)
              + m1 * (11003 * m1 - 9402 * z)
              + z * (2107 * z))
        b1 = (m2 * (267 * m2 - 1642 * m1 + 1602 * z - 494 * p1)
              + m1 * (2843 * m1 - 5966 * z + 1922 * p1)
              + z * (3443 * z - 2522 * p1)
              + p1 * (547 * p1))
        b2 = (m1 * (547 * m1 - 2522 * z + 1922 * p1 - 494 * p2)
              + z * (3443 * z - 5966 * p1 + 1602 * p2)
              + p1 * (2843 * p1 - 1642 * p2)
              + p2 * (267 * p2))
        b3 = (z * (2107 * z - 9402 * p1 + 7042 * p2 - 1854 * p3)
              + p1 * (11003 * p1 - 17246 * p2 + 4642 * p3)
              + p2 * (7043 * p2 - 3882 * p3)
              + p3 * (547 * p3))
        a0 = lambda d: d / (b0 + eps) ** 2
        a1 = lambda d: d / (b1 + eps) ** 2
        a2 = lambda d: d / (b2 + eps) ** 2
        a3 = lambda d: d / (b3 + eps) ** 2
        sR = a0(g0) + a1(g1) + a2(g2) + a3(g3)
        wR = ((a0(g0) / sR) * (-1 / 4 * m3 + 13 / 12 * m2 - 23 / 12 * m1 + 25 / 12 * z)
              + (a1(g1) / sR) * (1 / 12 * m2 - 5 / 12 * m1 + 13 / 12 * z + 1 / 4 * p1)
              + (a2(g2) / sR) * (-1 / 12 * m1 + 7 / 12 * z + 7 / 12 * p1 - 1 / 12 * p2)
              + (a3(g3) / sR) * (1 / 4 * z + 13 / 12 * p1 - 5 / 12 * p2 + 1 / 12 * p3))
        sL = a0(g3) + a1(g2) + a2(g1) + a3(g0)
        wL = ((a0(g3) / sL) * (1 / 4 * z + 13 / 12 * m1 - 5 / 12 * m2 + 1 / 12 * m3)
              + (a1(g2) / sL) * (-1 / 12 * p1 + 7 / 12 * z + 7 / 12 * m1 - 1 / 12 * m2)
              + (a2(g1) / sL) * (1 / 12 * p2 - 5 / 12 * p1 + 13 / 12 * z + 1 / 4 * m1)
              + (a3(g0) / sL) * (-1 / 4 * p3 + 13 / 12 * p2 - 23 / 12 * p1 + 25 / 12 * z))
        return wL, wR
    # order 5
    g0, g1, g2 = 1 / 10, 3 / 5, 3 / 10
    b0 = 13 / 12 * (m2 - 2 * m1 + z) ** 2 + 1 / 4 * (m2 - 4 * m1 + 3 * z) ** 2
    b1 = 13 / 12 * (m1 - 2 * z + p1) ** 2 + 1 / 4 * (m1 - p1) ** 2
    b2 = 13 / 12 * (z - 2 * p1 + p2) ** 2 + 1 / 4 * (3 * z - 4 * p1 + p2) ** 2
    a0 = lambda d: d / (b0 + eps) ** 2
    a1 = lambda d: d / (b1 + eps) ** 2
    a2 = lambda d: d / (b2 + eps) ** 2
    wR = ((a0(g0) / (a0(g0) + a1(g1) + a2(g2))) * (1 / 3 * m2 - 7 / 6 * m1 + 11 / 6 * z)
          + (a1(g1) / (a0(g0) + a1(g1) + a2(g2))) * (-1 / 6 * m1 + 5 / 6 * z + 1 / 3 * p1)
          + (a2(g2) / (a0(g0) + a1(g1) + a2(g2))) * (1 / 3 * z + 5 / 6 * p1 - 1 / 6 * p2))
    wL = ((a0(g2) / (a0(g2) + a1(g1) + a2(g0))) * (1 / 3 * z + 5 / 6 * m1 - 1 / 6 * m2)
          + (a1(g1) / (a0(g2) + a1(g1) + a2(g0))) * (-1 / 6 * p1 + 5 / 6 * z + 1 / 3 * m1)
          + (a2(g0) / (a0(g2) + a1(g1) + a2(g0))) * (1 / 3 * p2 - 7 / 6 * p1 + 11 / 6 * z))
    return wL, wR
