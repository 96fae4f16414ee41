"""Interface Riemann fluxes of the oracle (test infrastructure only).

Inputs are face arrays of length N+1 along the sweep axis: ``w_plus`` /
``w_minus`` are the primitive states right / left of each interface (the
reference's ``wFs``), ``q_plus`` / ``q_minus`` their conservative forms
(``qFs``) and ``f_plus`` / ``f_minus`` the physical fluxes (``fluxFs``).

``label`` is the axis number the reference's ``calculate_Riemann_flux``
passes to the solver: the *iteration position* of the sweep (0 for the first
sweep of a step, 1 for the second), not necessarily the physical axis
(solvers.py:34-36,63).  HLLC and HLLD pick the normal velocity with it.
"""

import numpy as np

from .fvcore import divide, nsq, norm3, vdot


def llf(alpha, q_plus, q_minus, f_plus, f_minus):
    """Local Lax-Friedrichs with a per-interface speed (solvers.py:69-75)."""
    return .5 * (f_minus + f_plus) - .5 * ((q_plus - q_minus) * alpha[..., None])


def lax_wendroff(char_speed2_over_max, q_plus, q_minus, f_plus, f_minus):
    """Lax-Wendroff-type flux with a per-interface coefficient (solvers.py:79-88)."""
    return .5 * (f_minus + f_plus) - .5 * ((q_plus - q_minus) * char_speed2_over_max[..., None])


def hllc(label, gamma, w_plus, w_minus, q_plus, q_minus, f_plus, f_minus, physical=False):
    """HLLC (solvers.py:92-138) with the reference's quirks kept.

    * The normal velocity is component ``label+1``.
    * The star-state normal momentum is always written to component 1.
    * Where no wave condition holds (sL > 0) the flux is ``f_plus``.

    ``physical=True`` (not in the reference) is the textbook solver: ``label``
    is then the physical sweep axis, the star normal momentum goes to
    component ``label+1`` and the sL > 0 flux is ``f_minus``.
    """
    rL, uL, pL, QL = w_minus[..., 0], w_minus[..., label + 1], w_minus[..., 4], q_minus
    rR, uR, pR, QR = w_plus[..., 0], w_plus[..., label + 1], w_plus[..., 4], q_plus
    with np.errstate(invalid="ignore"):
        cL = np.sqrt(gamma * divide(pL, rL))
        cR = np.sqrt(gamma * divide(pR, rR))
        sqL, sqR = np.sqrt(rL), np.sqrt(rR)
        u_hat = divide(uL * sqL + uR * sqR, sqL + sqR)
        c2_hat = (divide(sqL * cL ** 2 + sqR * cR ** 2, sqL + sqR)
                  + .5 * ((uR - uL) ** 2) * divide(sqL * sqR, (sqL + sqR) ** 2))
        c_hat = np.sqrt(c2_hat)
    sL = np.minimum(uL - cL, u_hat - c_hat)
    sR = np.maximum(uR + cR, u_hat + c_hat)
    sM = divide(pR - pL + rL * uL * (sL - uL) - rR * uR * (sR - uR), rL * (sL - uL) - rR * (sR - uR))

    mom = label + 1 if physical else 1

    def star(rho, u, p, Q, s):
        coeff = divide(s - u, s - sM)
        Qs = Q * coeff[..., None]
        Qs[..., mom] = rho * coeff * sM
        Qs[..., 4] = Qs[..., 4] + coeff * (sM - u) * (rho * sM + divide(p, s - u))
        return Qs

    QLs = star(rL, uL, pL, QL, sL)
    QRs = star(rR, uR, pR, QR, sR)
    F = np.copy(f_minus if physical else f_plus)
    fLs = f_minus + (QLs - QL) * sL[..., None]
    fRs = f_plus + (QRs - QR) * sR[..., None]
    m = (sL <= 0) & (0 < sM)
    F[m] = fLs[m]
    m = (sM <= 0) & (0 <= sR)
    F[m] = fRs[m]
    m = sR < 0
    F[m] = f_plus[m]
    return F


def _fast_speed_bx(w, gamma, normal=0):
    """HLLD's fast speed; the 'normal' field is always B_x (solvers.py:144-153)."""
    rho, P, B = w[..., 0], w[..., 4], w[..., 5:8]
    with np.errstate(invalid="ignore"):
        cs = np.sqrt(divide(gamma * P, rho))
        ca = divide(norm3(B), np.sqrt(rho))
        cax = divide(B[..., normal], np.sqrt(rho))
        return np.sqrt(.5 * (cs ** 2 + ca ** 2 + np.sqrt(((cs ** 2 + ca ** 2) ** 2) - (4 * (cs ** 2) * (cax ** 2)))))


def hlld_textbook(a, gamma, Bn, w_plus, w_minus, q_plus, q_minus, f_plus, f_minus):
    """HLLD as published (Miyoshi & Kusano 2005, eqs. 38-51 and 59-67); not the reference's solver.

    The reference's calculate_HLLD_flux (solvers.py:142-232) departs from the
    paper in ways that make it blow up on the Orszag-Tang vortex within a few
    dozen steps: sR uses min(uL, uR), the star and double-star momenta are
    missing their density factors, the right Alfven speed has the wrong sign and
    the energy uses momenta in place of velocities.  This is the paper's solver,
    with one normal field ``Bn`` shared by both sides (the caller passes the mean
    of the two face states' normal fields).  A star state
    whose denominator rho (S - u)(S - S_M) - Bn^2 vanishes (relative 1e-10)
    keeps its transverse velocity and field (the paper's degenerate case).
    """
    o, p = (a + 1) % 3, (a + 2) % 3
    rL, uL, vL, wL, PL = w_minus[..., 0], w_minus[..., 1 + a], w_minus[..., 1 + o], w_minus[..., 1 + p], w_minus[..., 4]
    rR, uR, vR, wR, PR = w_plus[..., 0], w_plus[..., 1 + a], w_plus[..., 1 + o], w_plus[..., 1 + p], w_plus[..., 4]
    byL, bzL, byR, bzR = w_minus[..., 5 + o], w_minus[..., 5 + p], w_plus[..., 5 + o], w_plus[..., 5 + p]
    bn2 = Bn * Bn
    with np.errstate(invalid="ignore", divide="ignore"):
        def fast(r, P, by, bz):
            cs2 = divide(gamma * P, r)
            ca2 = divide((bn2 + by * by) + bz * bz, r)
            cx2 = divide(bn2, r)
            sm = cs2 + ca2
            return np.sqrt(.5 * (sm + np.sqrt(np.maximum(sm * sm - (4 * cs2) * cx2, 0.))))
        cf = np.maximum(fast(rL, PL, byL, bzL), fast(rR, PR, byR, bzR))
        sL = np.minimum(uL, uR) - cf
        sR = np.maximum(uL, uR) + cf
        ptL = PL + .5 * ((bn2 + byL * byL) + bzL * bzL)
        ptR = PR + .5 * ((bn2 + byR * byR) + bzR * bzR)
        dL, dR = sL - uL, sR - uR
        den = dR * rR - dL * rL
        sM = divide((((dR * rR) * uR - (dL * rL) * uL) - ptR) + ptL, den)
        pts = divide(((dR * rR) * ptL - (dL * rL) * ptR) + ((rL * rR) * (dR * dL)) * (uR - uL), den)

        def star(r, u, v, w, by, bz, E, pt, s, d):
            rs = r * divide(d, s - sM)
            rds = (r * d) * (s - sM)
            dn = rds - bn2
            degen = np.abs(dn) <= 1e-10 * (np.abs(rds) + bn2)
            g = divide(sM - u, dn)
            fac = divide((r * d) * d - bn2, dn)
            vs = np.where(degen, v, v - (Bn * by) * g)
            ws = np.where(degen, w, w - (Bn * bz) * g)
            bys = np.where(degen, by, by * fac)
            bzs = np.where(degen, bz, bz * fac)
            vb = (u * Bn + v * by) + w * bz
            vbs = (sM * Bn + vs * bys) + ws * bzs
            Es = divide(((d * E - pt * u) + pts * sM) + Bn * (vb - vbs), s - sM)
            return rs, vs, ws, bys, bzs, Es, vbs

        rsL, vsL, wsL, bysL, bzsL, EsL, vbsL = star(rL, uL, vL, wL, byL, bzL, q_minus[..., 4], ptL, sL, dL)
        rsR, vsR, wsR, bysR, bzsR, EsR, vbsR = star(rR, uR, vR, wR, byR, bzR, q_plus[..., 4], ptR, sR, dR)
        sqL, sqR = np.sqrt(rsL), np.sqrt(rsR)
        ssL = sM - divide(np.abs(Bn), sqL)
        ssR = sM + divide(np.abs(Bn), sqR)
        sg = np.sign(Bn)
        d2 = sqL + sqR
        vss = divide((sqL * vsL + sqR * vsR) + (bysR - bysL) * sg, d2)
        wss = divide((sqL * wsL + sqR * wsR) + (bzsR - bzsL) * sg, d2)
        byss = divide((sqL * bysR + sqR * bysL) + ((sqL * sqR) * (vsR - vsL)) * sg, d2)
        bzss = divide((sqL * bzsR + sqR * bzsL) + ((sqL * sqR) * (wsR - wsL)) * sg, d2)
        vbss = (sM * Bn + vss * byss) + wss * bzss
        EssL = EsL - (sqL * (vbsL - vbss)) * sg
        EssR = EsR + (sqR * (vbsR - vbss)) * sg

    def vec(r, v, w, E, by, bz, like):
        U = np.zeros_like(like)
        U[..., 0] = r
        U[..., 1 + a] = r * sM
        U[..., 1 + o] = r * v
        U[..., 1 + p] = r * w
        U[..., 4] = E
        U[..., 5 + a] = Bn
        U[..., 5 + o] = by
        U[..., 5 + p] = bz
        return U

    UsL = vec(rsL, vsL, wsL, EsL, bysL, bzsL, q_minus)
    UsR = vec(rsR, vsR, wsR, EsR, bysR, bzsR, q_plus)
    UssL = vec(rsL, vss, wss, EssL, byss, bzss, q_minus)
    UssR = vec(rsR, vss, wss, EssR, byss, bzss, q_plus)
    FsL = f_minus + (UsL - q_minus) * sL[..., None]
    FsR = f_plus + (UsR - q_plus) * sR[..., None]
    FssL = FsL + (UssL - UsL) * ssL[..., None]
    FssR = FsR + (UssR - UsR) * ssR[..., None]
    F = np.copy(f_minus)
    for m, G in (((sL <= 0) & (0 < ssL), FsL), ((ssL <= 0) & (0 < sM), FssL), ((sM <= 0) & (0 < ssR), FssR),
                 ((ssR <= 0) & (0 <= sR), FsR), (sR < 0, f_plus)):
        F[m] = G[m]
    return F


def hlld(label, gamma, wS_right, w_plus, w_minus, q_plus, q_minus, f_plus, f_minus, physical=False):
    """HLLD of Miyoshi & Kusano (solvers.py:142-232), reference quirks kept.

    ``wS_right`` is the cell-averaged primitive of the cell right of each
    interface (``add_boundary(wS)[1:]``, solvers.py:168); its component
    ``label+5`` is the normal field used in the star and double-star states.
    ``physical=True`` (not in the reference): ``label`` is the physical sweep
    axis and the solver is the published one (``hlld_textbook``) with the mean
    of the two face states' normal fields as B_n.
    """
    if physical:
        a = label % 3
        Bn = .5 * (w_minus[..., 5 + a] + w_plus[..., 5 + a])
        return hlld_textbook(a, gamma, Bn, w_plus, w_minus, q_plus, q_minus, f_plus, f_minus)
    a, o, p = label % 3, (label + 1) % 3, (label + 2) % 3
    rL, vL, pL, BL, QL = w_minus[..., 0], w_minus[..., 1:4], w_minus[..., 4], w_minus[..., 5:8], q_minus
    rR, vR, pR, BR, QR = w_plus[..., 0], w_plus[..., 1:4], w_plus[..., 4], w_plus[..., 5:8], q_plus
    Bn = wS_right[..., a + 5]
    uL, uR = vL[..., label], vR[..., label]

    nb = label if physical else 0
    cfL, cfR = _fast_speed_bx(w_minus, gamma, nb), _fast_speed_bx(w_plus, gamma, nb)
    sL = np.minimum(uL, uR) - np.maximum(cfL, cfR)
    sR = np.minimum(uL, uR) + np.maximum(cfL, cfR)
    sM = divide(pR - pL + rL * uL * (sL - uL) - rR * uR * (sR - uR) + .5 * (nsq(BR)) - .5 * (nsq(BL)),
                rL * (sL - uL) - rR * (sR - uR))

    rLs = rL * divide(sL - uL, sL - sM)
    rRs = rR * divide(sR - uR, sR - sM)
    with np.errstate(invalid="ignore"):
        sLs = sM - divide(BL[..., label], np.sqrt(rLs))
        sRs = sM - divide(BR[..., label], np.sqrt(rRs))

    p_star = divide(rL * (pR + .5 * nsq(BR)) * (sL - uL) - rR * (pL + .5 * nsq(BL)) * (sR - uR) + rR * rL * (sL - uL) * (sR - uR),
                    rL * (sL - uL) - rR * (sR - uR))

    def side(rho, v, B, u, s):
        den = rho * (s - u) * (s - sM) - Bn ** 2
        vy = v[..., o] - Bn * B[..., o] * divide(sM - u, den)
        vz = v[..., p] - Bn * B[..., p] * divide(sM - u, den)
        by = B[..., o] * divide(rho * (s - u) ** 2 - Bn ** 2, den)
        bz = B[..., p] * divide(rho * (s - u) ** 2 - Bn ** 2, den)
        return vy, vz, by, bz

    vyL, vzL, ByL, BzL = side(rL, vL, BL, uL, sL)
    vyR, vzR, ByR, BzR = side(rR, vR, BR, uR, sR)

    def star_state(Q, rho, rs, vy, vz, by, bz):
        Qs = np.zeros_like(Q)
        Qs[..., 0] = rs
        Qs[..., a + 1] = rho * sM
        Qs[..., o + 1] = rho * vy
        Qs[..., p + 1] = rho * vz
        Qs[..., a + 5] = np.copy(Q[..., a + 5])
        Qs[..., o + 5] = by
        Qs[..., p + 5] = bz
        return Qs

    QLs = star_state(QL, rL, rLs, vyL, vzL, ByL, BzL)
    QRs = star_state(QR, rR, rRs, vyR, vzR, ByR, BzR)
    QLs[..., 4] = divide(QL[..., 4] * (sL - uL) - uL * (pL + .5 * nsq(BL)) + p_star * sM
                         + Bn * (vdot(vL, BL) - vdot(QLs[..., 1:4], QLs[..., 5:8])), sL - sM)
    QRs[..., 4] = divide(QR[..., 4] * (sR - uR) - uR * (pR + .5 * nsq(BR)) + p_star * sM
                         + Bn * (vdot(vR, BR) - vdot(QRs[..., 1:4], QRs[..., 5:8])), sR - sM)

    fLs = np.copy(f_minus) + (QLs - QL) * sL[..., None]
    fRs = np.copy(f_plus) + (QRs - QR) * sR[..., None]

    with np.errstate(invalid="ignore"):
        sqLs, sqRs = np.sqrt(rLs), np.sqrt(rRs)
        sgn = np.sign(Bn)
        vy2 = divide(vyR * sqRs + vyL * sqLs + sgn * (ByL - ByR), sqLs + sqRs)
        vz2 = divide(vzR * sqRs + vzL * sqLs + sgn * (BzL - BzR), sqLs + sqRs)
        By2 = divide(ByL * sqRs + ByR * sqLs + sgn * (vyL - vyR) * np.sqrt(rRs * rLs), sqLs + sqRs)
        Bz2 = divide(BzL * sqRs + BzR * sqLs + sgn * (vzL - vzR) * np.sqrt(rRs * rLs), sqLs + sqRs)

    def dstar_state(Qs, rs):
        Q2 = np.zeros_like(Qs)
        Q2[..., 0] = rs
        Q2[..., a + 1] = sM
        Q2[..., o + 1] = vy2
        Q2[..., p + 1] = vz2
        Q2[..., a + 5] = np.copy(Qs[..., a + 5])
        Q2[..., o + 5] = By2
        Q2[..., p + 5] = Bz2
        return Q2

    QL2 = dstar_state(QLs, rLs)
    QR2 = dstar_state(QRs, rRs)
    QL2[..., 4] = np.copy(QLs[..., 4] - sqLs * sgn * (vdot(QLs[..., 1:4], QLs[..., 5:8]) - vdot(QL2[..., 1:4], QL2[..., 5:8])))
    QR2[..., 4] = np.copy(QRs[..., 4] - sqRs * sgn * (vdot(QRs[..., 1:4], QRs[..., 5:8]) - vdot(QR2[..., 1:4], QR2[..., 5:8])))

    fL2 = np.copy(f_minus) + (QL2 - QLs) * sLs[..., None]
    fR2 = np.copy(f_plus) + (QR2 - QRs) * sRs[..., None]

    F = np.copy(f_minus)
    m = (sL <= 0) & (0 < sLs)
    F[m] = fLs[m]
    m = (sLs <= 0) & (0 < sM)
    F[m] = fL2[m]
    m = (sM <= 0) & (0 < sRs)
    F[m] = fR2[m]
    m = (sRs <= 0) & (0 <= sR)
    F[m] = fRs[m]
    m = sR < 0
    F[m] = f_plus[m]
    return F
