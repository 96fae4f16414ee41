"""Constrained-transport pieces of the oracle for 2D MHD (test infrastructure only).

Restates num_methods/mag_field.py and the magnetic parts of
num_methods/evolvers.py.  Frames: ``P[0] = (0,1,2)`` (x sweep),
``P[1] = (1,0,2)`` (y sweep); a sweep's face array ``wF`` is indexed
``[i_sweep, i_transverse]``.
"""

import numpy as np

from .fvcore import gather, gather_range, divide, norm3, roe_average, avg_to_centre, centre_to_avg, max_speed_lapack, primitive_jacobian
from .recon import ppm_mc

PERM = {0: (0, 1, 2), 1: (1, 0, 2)}


def reconstruct_transverse(wF, bc):
    """PPM-mc of a sweep's face values along the transverse axis.

    mag_field.reconstruct_transverse (mag_field.py:11-65, 'ppm'/'mc').
    Returns (wD, wU) in the transposed frame ``[i_transverse, i_sweep]``.
    """
    ortho = np.copy(wF.transpose(1, 0, 2))
    wD, wU, _ = ppm_mc(ortho, bc)
    return wD, wU


def corner_speeds(wD, wU, gamma, bc, axis, solver_category, eig_mode):
    """Upwind speeds at the corners (mag_field.compute_corner.get_wavespeeds, :125-149)."""
    n = wD.shape[0]
    plus = gather_range(wD, 0, n + 1, bc)
    minus = gather_range(wU, -1, n + 1, bc)
    avg = roe_average(plus, minus)[1:]
    if solver_category == "hll":
        rho, v, P, B = avg[..., 0], avg[..., 1:4], avg[..., 4], avg[..., 5:8]
        vx, Bx = v[..., axis % 3], B[..., axis % 3]
        with np.errstate(invalid="ignore"):
            cs = np.sqrt(gamma * divide(P, rho))
            ca = divide(norm3(B), np.sqrt(rho))
            cax = divide(Bx, np.sqrt(rho))
            cf = np.sqrt(.5 * (cs ** 2 + ca ** 2 + np.sqrt(((cs ** 2 + ca ** 2) ** 2) - (4 * (cs ** 2) * (cax ** 2)))))
        a_plus = np.maximum(np.zeros_like(vx), vx + cf)
        a_minus = -np.minimum(np.zeros_like(vx), vx - cf)
        return a_plus, a_minus
    # Lax-type solvers: signed extreme eigenvalues of the Jacobian
    if eig_mode == "lapack":
        with np.errstate(all="ignore"):
            ev = np.linalg.eigvals(primitive_jacobian(avg, gamma, axis % 3))
        return np.max(ev, axis=-1).real, (-np.min(ev, axis=-1)).real
    rho, v, P, B = avg[..., 0], avg[..., 1:4], avg[..., 4], avg[..., 5:8]
    vn = v[..., axis % 3]
    with np.errstate(all="ignore"):
        a2 = (gamma * P) / rho
        b2 = (norm3(B) * norm3(B)) / rho
        bn2 = (B[..., axis % 3] * B[..., axis % 3]) / rho
        s = a2 + b2
        cf = np.sqrt(.5 * (s + np.sqrt(s * s - 4 * a2 * bn2)))
    return np.maximum(vn + cf, 0 * vn), -np.minimum(vn - cf, 0 * vn)


def compute_corner(sweeps, order, gamma, bc, solver_category, eig_mode):
    """Upwind corner electric field E_z (mag_field.compute_corner, :125-187).

    ``sweeps[a]['wTs']`` is the transverse reconstruction of sweep ``a``;
    ``order`` the physical axes in this step's iteration order.  The
    reference walks a 'swapped' permutation map, so which sweep supplies
    north/south and which speeds are called 'x' alternates with the step
    parity; that is kept.
    """
    a0, a1 = order
    swapped = [(a0, a1), (a1, a0)]  # (key axis, sweep whose data is read)
    alphas, mags = [], []
    for axis, s in swapped:
        wD, wU = sweeps[s]["wTs"]
        align = PERM[axis]
        ap, am = corner_speeds(wD, wU, gamma, bc, axis, solver_category, eig_mode)
        alphas.append([ap.transpose(align[:-1]), am.transpose(align[:-1])])
        mags.append([wD.transpose(align), wU.transpose(align)])
    [north, south], [east, west] = mags
    NE = .5 * (west[..., 2] + south[..., 2]) * south[..., 5] - .5 * (west[..., 1] + south[..., 1]) * west[..., 6]
    NW = .5 * (east[..., 2] + south[..., 2]) * south[..., 5] - .5 * (east[..., 1] + south[..., 1]) * east[..., 6]
    SE = .5 * (west[..., 2] + north[..., 2]) * north[..., 5] - .5 * (west[..., 1] + north[..., 1]) * west[..., 6]
    SW = .5 * (east[..., 2] + north[..., 2]) * north[..., 5] - .5 * (east[..., 1] + north[..., 1]) * east[..., 6]
    [ap_y, am_y], [ap_x, am_x] = alphas
    return (divide(ap_x * ap_y * SW + am_x * ap_y * SE + ap_x * am_y * NW + am_x * am_y * NE, (ap_x + am_x) * (ap_y + am_y))
            - divide(ap_y * am_y, ap_y + am_y) * (north[..., 5] - south[..., 5])
            + divide(ap_x * am_x, ap_x + am_x) * (east[..., 6] - west[..., 6]))


def corner_for_sweep(E, axis):
    """``fluxes[P[axis]]['mag_corner']`` as evolve_space stores it (evolvers.py:29-32)."""
    return np.copy(E.transpose(PERM[1 - axis][:-1]))


def induction_rates(mag_corners, dx, bc):
    """Magnetic rows of ``compute_L`` before the sign flip (evolvers.py:52-58).

    Returns {5: ..., 6: ...}: the flux differences that replace the B_x and
    B_y components of the summed hydro divergence.
    """
    out = {}
    for axis in (0, 1):
        Ec = mag_corners[axis]
        n = Ec.shape[0]
        padded = gather_range(Ec, -1, n + 2, bc)
        mag_flux = (-1) ** axis * np.diff(padded[1:], axis=0) / dx
        out[5 + axis] = mag_flux.transpose(PERM[1 - axis][:-1])
    return out


def inverse_reconstruct(grid, bc, centred=False):
    """Face-averaged B back to cell averages (mag_field.inverse_reconstruct, :191-210).

    Entry i of a face array is the face i+1/2.  The reference's 4-point
    interpolant of faces i-1/2 .. i+5/2 is centred on cell i+1, which moves B
    one cell along its own axis at every stage; that offset is kept unless
    ``centred``, which interpolates faces i-3/2 .. i+3/2 onto cell i (Felker &
    Stone 2018, eq. 39).
    """
    new = np.copy(grid)
    for axis in (0, 1):
        frame = grid.transpose(PERM[axis])
        fc = avg_to_centre(frame, bc, [1])
        if centred:
            cc = -1 / 16 * (gather(fc, -2, bc) + gather(fc, 1, bc)) + 9 / 16 * (gather(fc, -1, bc) + fc)
        else:
            cc = -1 / 16 * (gather(fc, -1, bc) + gather(fc, 2, bc)) + 9 / 16 * (fc + gather(fc, 1, bc))
        ca = centre_to_avg(cc, bc, [0, 1])
        new[..., 5 + axis] = ca.transpose(PERM[axis])[..., 5 + axis]
    return new


def divergence_B(grid, dx, bc):
    """Cell-centred central-difference div B of cell-averaged B (diagnostic; no reference counterpart)."""
    Bx, By = grid[..., 5], grid[..., 6]
    div = (gather(Bx, 1, bc, 0) - gather(Bx, -1, bc, 0)) / (2 * dx) + (gather(By, 1, bc, 1) - gather(By, -1, bc, 1)) / (2 * dx)
    return div
