"""The FP32 kernels' own forms of the reference's formulas, checked on the host.

The FP32 sweep (astrea_gb300/csrc/{physics,recon,sweep}.cuh) rewrites several of the
reference's expressions into forms with fewer instructions.  Each rewrite is an identity of
exact arithmetic; these tests check it in float64 on seeded random states (to round-off), and
the one rewrite the FP64 kernels share, C * min(|a|, |b|, |c|), for bit equality in both
precisions.
"""
import numpy as np

RNG = np.random.default_rng(20240611)
C24 = 1.0 / 24.0
GAMMA = 1.4


def p2c(w):
    """fv.point_convert_primitive of a 2D Euler state w = (rho, u, v, p) (last axis)."""
    rho, u, v, p = w[..., 0], w[..., 1], w[..., 2], w[..., 3]
    return np.stack([rho, rho * u, rho * v, p / (GAMMA - 1) + 0.5 * rho * (u * u + v * v)], axis=-1)


def states(n):
    w = np.empty((n, 4))
    w[:, 0] = RNG.uniform(0.1, 3.0, n)
    w[:, 1] = RNG.uniform(-2.0, 2.0, n)
    w[:, 2] = RNG.uniform(-2.0, 2.0, n)
    w[:, 3] = RNG.uniform(0.1, 3.0, n)
    return w


def test_face_conversion_linear_parts_are_the_identity():
    # fv.high_order_convert_primitive on a face array across the sweep:
    # q = p2c(w - d2w/24) + d2(p2c w)/24, d2 over the rows above and below
    w0, wm, wp = states(1000), states(1000), states(1000)
    d2 = lambda a0, am, ap: (ap - a0) - (a0 - am)
    ref = p2c(w0 - C24 * d2(w0, wm, wp)) + C24 * d2(p2c(w0), p2c(wm), p2c(wp))
    # the FP32 form: density and p/(gamma-1) pass through; momenta and kinetic energy are the
    # products of the converted w plus the second differences of the point products
    r, a, b = [(1 + 2 * C24) * w0[:, i] - C24 * (wp[:, i] + wm[:, i]) for i in range(3)]
    prod = lambda x: (x[:, 0] * x[:, 1], x[:, 0] * x[:, 2], 0.5 * x[:, 0] * (x[:, 1] ** 2 + x[:, 2] ** 2))
    (m0x, m0y, e0), (mmx, mmy, em), (mpx, mpy, ep) = prod(w0), prod(wm), prod(wp)
    form = np.stack([w0[:, 0],
                     r * a + C24 * ((mpx - m0x) - (m0x - mmx)),
                     r * b + C24 * ((mpy - m0y) - (m0y - mmy)),
                     w0[:, 3] / (GAMMA - 1) + 0.5 * r * (a * a + b * b) + C24 * ((ep - e0) - (e0 - em))], axis=-1)
    assert np.max(np.abs(form - ref) / (np.abs(ref) + 1.0)) < 1e-14


def test_hllc_roe_terms_from_reciprocal_square_roots():
    # solvers.py:92-138: sqrt(rho) weights, c = sqrt(gamma p / rho), Roe-averaged c^2
    wl, wr = states(1000), states(1000)
    rl, pl, rr, pr = wl[:, 0], wl[:, 3], wr[:, 0], wr[:, 3]
    cl, cr = np.sqrt(GAMMA * pl / rl), np.sqrt(GAMMA * pr / rr)
    sl, sr = np.sqrt(rl), np.sqrt(rr)
    c2 = (sl * cl * cl + sr * cr * cr) / (sl + sr)
    il, ir = 1 / np.sqrt(rl), 1 / np.sqrt(rr)
    assert np.allclose(rl * il, sl, rtol=1e-15, atol=0)
    assert np.allclose(np.sqrt(GAMMA * pl) * il, cl, rtol=1e-15, atol=0)
    assert np.allclose(GAMMA * (pl * il + pr * ir) / (rl * il + rr * ir), c2, rtol=1e-14, atol=0)


def test_limiter_curvature_minimum_is_bit_exact_in_both_precisions():
    # min(C|a|, C|b|, C|c|) == C min(|a|, |b|, |c|) for C > 0: rounding is monotone
    for dtype in (np.float64, np.float32):
        x = RNG.standard_normal((3, 100000)).astype(dtype) * np.exp(RNG.uniform(-20, 20, (3, 100000))).astype(dtype)
        c = dtype(1.25)
        lhs = np.minimum(np.minimum(c * np.abs(x[0]), c * np.abs(x[1])), c * np.abs(x[2]))
        rhs = c * np.minimum(np.minimum(np.abs(x[0]), np.abs(x[1])), np.abs(x[2]))
        assert np.array_equal(lhs, rhs)


def test_euler_wave_speed_square_root_form():
    # max_speed: sqrt((a2 + sqrt(a2^2)) / 2) is sqrt(a2) for a2 >= 0
    a2 = np.abs(RNG.standard_normal(100000)) * np.exp(RNG.uniform(-30, 30, 100000))
    assert np.array_equal(0.5 * (a2 + np.sqrt(a2 * a2)), a2)


def test_flattening_blend_forms_agree():
    # ppm.py:67 with apply_flattener: f eta + w (1 - eta) == w + eta (f - w)
    f, w = RNG.uniform(-3, 3, 10000), RNG.uniform(-3, 3, 10000)
    eta = RNG.uniform(0, 1, 10000)
    assert np.max(np.abs((f * eta + w * (1 - eta)) - (w + eta * (f - w)))) < 1e-14
