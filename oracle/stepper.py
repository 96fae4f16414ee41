"""Space/time evolution of the oracle (test infrastructure only).

``evolve_space`` / ``evolve_time`` restate num_methods/evolvers.py:12-206 and
solvers.calculate_Riemann_flux (solvers.py:10-65); ``run`` restates the step
loop of astrea.core_run (astrea.py:44-85) without the HDF5 snapshots.

``order`` is the list of physical axes in the iteration order of the current
step: ``[0]`` in 1D, ``[0, 1]`` on even steps and ``[1, 0]`` on odd steps in
2D (core_run reverses its permutation map after every step, astrea.py:85).
"""

from dataclasses import dataclass, field

import numpy as np

from . import fvcore as fv
from . import recon, riemann, ct

PERM = {0: (0, 1, 2), 1: (1, 0, 2)}
HIGH_ORDER = ("ppm", "weno3", "weno5", "weno7")


@dataclass
class OracleConfig:
    """Canonical method choices (the reference's strings are mapped by the caller)."""
    dim: int = 1
    scheme: str = "plm"          # pcm | plm | ppm | weno3 | weno5 | weno7
    solver: str = "llf"          # llf | hllc | hlld
    integrator: str = "ssprk33"  # euler | rk4 | ssprk22 | ssprk33 | ssprk43 | ssprk53 | ssprk54 | ssprk104
    gamma: float = 1.4
    bc: str = "edge"             # edge (outflow) | wrap (periodic)
    dx: float = 1.0
    cfl: float = 0.8
    magnetic_2d: bool = False
    limiter: str = "minmod"      # PLM slope limiter: minmod | superbee
    eig: str = "lapack"          # lapack (as the reference) | analytic (as the kernels)
    compat: bool = True          # reference quirks in HLLC/HLLD (False: physical-axis solvers, not in the reference)
    ct_centred: bool = False     # constrained transport: face->cell interpolant centred on the cell (not the reference's)
    flatten: bool = False        # PPM flattening (parity unpinned)
    viscosity: bool = False      # PPM artificial viscosity (parity unpinned)
    av_alpha: float = .3
    av_beta: float = .3
    t_end: float = 0.2
    checkpoints: int = 1
    extra: dict = field(default_factory=dict)

    @property
    def solver_category(self):
        return "hll" if self.solver in ("hllc", "hlld") else "lax"

    @property
    def high_order(self):
        return self.scheme in HIGH_ORDER


def _frame(grid, axis, dim):
    return grid if dim == 1 else grid.transpose(PERM[axis])


def convert_conservative(q, cfg, axes):
    if cfg.high_order:
        return fv.ho_c2p(q, cfg.gamma, cfg.bc, axes)
    return fv.c2p(q, cfg.gamma)


def convert_primitive(w, cfg, axes):
    if cfg.high_order:
        return fv.ho_p2c(w, cfg.gamma, cfg.bc, axes)
    return fv.p2c(w, cfg.gamma)


def artificial_viscosity(wS, qf, axis, cfg):
    """Face viscous flux mu_{i+1/2} = alpha * nu * (q_{i+1} - q_i) (McCorquodale & Colella 2011 eq. 35-38).

    The reference's ``apply_artificial_viscosity`` (ppm.py:138-170) cannot
    run in 2D (it adds arrays of shapes (N+2,N) and (N,N)) and its result is
    never used.  This follows the paper it cites: lambda is h times the face
    velocity divergence (the normal velocity difference plus the quarter-sum of
    the transverse differences, eq. 35), nu = min(1, lambda^2 / (beta c_min^2))
    * lambda on compressive faces (eq. 36) and the viscous flux acts on the
    conserved differences (eq. 38).  ppm.py:157 multiplies lambda by dx once
    more, which makes the coefficient vanish as the grid is refined; that extra
    factor is left out.  Parity unpinned.
    """
    bc, g = cfg.bc, cfg.gamma
    vn = wS[..., axis + 1]
    lam = fv.gather(vn, 1, bc) - vn
    if cfg.dim == 2:
        vt = wS[..., (1 - axis) + 1]
        dvt = fv.gather(vt, 1, bc, 1) - fv.gather(vt, -1, bc, 1)
        lam = lam + .25 * (fv.gather(dvt, 1, bc) + dvt)
    with np.errstate(invalid="ignore"):
        cs = np.sqrt(fv.divide(g * wS[..., 4], wS[..., 0]))
    cmin = np.minimum(cs, fv.gather(cs, 1, bc))
    nu = np.minimum(1, fv.divide(lam ** 2, cfg.av_beta * cmin ** 2)) * lam
    nu[lam >= 0] = 0
    return cfg.av_alpha * (nu[..., None] * (fv.gather(qf, 1, bc) - qf))


def sweep(grid, cfg, axis, label):
    """One axis of evolve_space: reconstruction + Riemann flux (+ CT inputs).

    Returns a dict with the interface flux ``flux`` (sweep frame, N+1 along
    the sweep), ``eigmax``, the face value ``wF`` used for the magnetic
    re-assignment and, for 2D MHD, the transverse reconstruction ``wTs``.
    """
    g, bc, dim = cfg.gamma, cfg.bc, cfg.dim
    qf = _frame(grid, axis, dim)
    cell_axes = [0] if dim == 1 else [0, 1]
    face_axes = [] if dim == 1 else [1]
    wS = convert_conservative(qf, cfg, cell_axes)
    n = qf.shape[0]

    if cfg.scheme == "pcm":
        wL = wR = wF = wS
    elif cfg.scheme == "plm":
        wL, wR = recon.plm(wS, bc, cfg.limiter)
        wF = wR
    elif cfg.scheme == "ppm":
        wL, wR, wF = recon.ppm_mc(wS, bc, flatten_axis=axis if cfg.flatten else None)
        wF_transverse = recon.ppm_face(wS, bc)
    elif cfg.scheme.startswith("weno"):
        wL, wR = recon.weno(wS, bc, int(cfg.scheme[4:]))
        wF = wR
    else:
        raise ValueError(cfg.scheme)

    wp = fv.gather_range(wL, 0, n + 1, bc)
    wm = fv.gather_range(wR, -1, n + 1, bc)
    if cfg.scheme == "pcm":
        # pcm.py:85-101: conservative faces are the raw cell averages; speeds at cells
        qp = fv.gather_range(qf, 0, n + 1, bc)
        qm = fv.gather_range(qf, -1, n + 1, bc)
        y_cells = wS
    else:
        avg = fv.arith_average if cfg.scheme == "plm" else fv.roe_average
        y_cells = avg(wp[1:], wm[1:])
        qp = convert_primitive(wp, cfg, face_axes)
        qm = convert_primitive(wm, cfg, face_axes)
    fp, fm = fv.make_flux(wp, g, axis), fv.make_flux(wm, g, axis)
    loc = fv.max_speed(fv.gather_range(y_cells, -1, n + 2, bc), g, axis, cfg.eig)
    alpha = np.maximum(loc[:-1], loc[1:])
    eigmax = np.max(alpha)
    if cfg.solver == "lw":
        # solvers.py:79-88: the coefficient (sound speed)^2 / max|lambda| of each interface average,
        # paired like LLF's speeds.  'lapack' takes the reference's sound speed, the second unique
        # column of the whole eigenvalue array (np.unique(..., axis=-1)[..., 1]); 'analytic' the
        # entropy-wave eigenvalue v_n, which the kernels use
        y_pad = fv.gather_range(y_cells, -1, n + 2, bc)
        if cfg.eig == "lapack":
            with np.errstate(all="ignore"):
                ch = np.linalg.eigvals(fv.primitive_jacobian(y_pad, g, axis))
            ss = np.unique(ch, axis=-1)[..., 1]
            norm = fv.divide(ss ** 2, np.max(np.abs(ch), axis=-1))
        else:
            vn = y_pad[..., 1 + axis % 3]
            norm = fv.divide(vn * vn, loc)
        lw_coef = np.maximum(norm[:-1], norm[1:])
    wS_right = fv.gather_range(wS, 0, n + 1, bc)

    phys = not cfg.compat
    lab = axis if phys else label

    def solve(wp_, wm_, qp_, qm_, fp_, fm_):
        if cfg.solver == "llf":
            return riemann.llf(alpha, qp_, qm_, fp_, fm_)
        if cfg.solver == "lw":
            return riemann.lax_wendroff(lw_coef, qp_, qm_, fp_, fm_)
        if cfg.solver == "hllc":
            return riemann.hllc(lab, g, wp_, wm_, qp_, qm_, fp_, fm_, physical=phys)
        if cfg.solver == "hlld":
            return riemann.hlld(lab, g, wS_right, wp_, wm_, qp_, qm_, fp_, fm_, physical=phys)
        raise ValueError(cfg.solver)

    F_avg = solve(wp, wm, qp, qm, fp, fm)
    if dim == 2:
        c = lambda X: fv.avg_to_centre(X, bc, [1])
        F_c = solve(c(wp), c(wm), c(qp), c(qm), c(fp), c(fm))
        F = fv.flux_centre(F_c, F_avg, bc, 2)
    else:
        F = F_avg
    if cfg.viscosity and cfg.scheme == "ppm":
        mu = artificial_viscosity(wS, qf, axis, cfg)
        F = F + fv.gather_range(mu, -1, n + 1, bc)

    out = {"flux": F, "eigmax": eigmax, "wF": wF, "wS": wS}
    if cfg.magnetic_2d:
        out["wTs"] = ct.reconstruct_transverse(wF_transverse if cfg.scheme == "ppm" else wR, bc)
    return out


def evolve_space(grid, cfg, order):
    """evolvers.evolve_space (evolvers.py:12-34) for the given axis order."""
    fluxes = {}
    for label, axis in enumerate(order):
        fluxes[axis] = sweep(grid, cfg, axis, label)
    if cfg.magnetic_2d:
        E = ct.compute_corner(fluxes, order, cfg.gamma, cfg.bc, cfg.solver_category, cfg.eig)
        for axis in order:
            fluxes[axis]["mag_corner"] = ct.corner_for_sweep(E, axis)
        fluxes["E"] = E
    return fluxes


def compute_L(fluxes, cfg, order):
    """The spatial operator L = -sum_axes diff(F)/dx (+ induction rows) (evolvers.py:41-60)."""
    total = 0
    for axis in order:
        d = np.diff(fluxes[axis]["flux"], axis=0) / cfg.dx
        total = total + (d if cfg.dim == 1 else d.transpose(PERM[axis]))
    if cfg.magnetic_2d:
        rates = ct.induction_rates({a: fluxes[a]["mag_corner"] for a in (0, 1)}, cfg.dx, cfg.bc)
        total = np.copy(total)
        total[..., 5] = rates[5]
        total[..., 6] = rates[6]
    return -total


def evolve_time(grid, fluxes, dt, cfg, order):
    """evolvers.evolve_time (evolvers.py:38-206) for every integrator."""
    L = lambda fl: compute_L(fl, cfg, order)
    es = lambda k: evolve_space(k, cfg, order)
    refine = (lambda g: ct.inverse_reconstruct(g, cfg.bc, centred=cfg.ct_centred)) if cfg.magnetic_2d else (lambda g: g)

    L_zero = L(fluxes)
    if cfg.magnetic_2d:
        grid = np.copy(grid)
        for axis in order:
            grid[..., 5 + axis] = fluxes[axis]["wF"].transpose(PERM[axis])[..., 5 + axis]

    it = cfg.integrator
    if it == "ssprk104":
        k = np.copy(grid)
        fl = fluxes
        for _ in range(5):
            k = k + refine(1 / 6 * dt * L(fl))
            fl = es(k)
        k5 = refine(3 / 5 * grid + 6 / 15 * k + 1 / 15 * dt * L(fl))
        fl = es(k5)
        _k = np.copy(k5)
        for _ in range(4):
            _k = _k + refine(1 / 6 * dt * L(fl))
            fl = es(_k)
        return refine(-11 / 35 * grid + 5 / 7 * k5 + 3 / 5 * _k + 1 / 10 * dt * L(fl))
    if it == "ssprk54":
        k1 = refine(grid + .39175222657189 * dt * L_zero)
        f1 = es(k1)
        k2 = refine(.444370493651235 * grid + .555629506348765 * k1 + .368410593050371 * dt * L(f1))
        f2 = es(k2)
        k3 = refine(.620101851488403 * grid + .379898148511597 * k2 + .251891774271694 * dt * L(f2))
        f3 = es(k3)
        k4 = refine(.178079954393132 * grid + .821920045606868 * k3 + .544974750228521 * dt * L(f3))
        f4 = es(k4)
        return refine(.517231671970585 * k2 + .096059710526147 * k3 + .06369246866629 * dt * L(f3)
                      + .386708617503269 * k4 + .226007483236906 * dt * L(f4))
    if it == "ssprk53":
        k1 = refine(grid + .3772689151171 * dt * L_zero)
        f1 = es(k1)
        k2 = refine(k1 + .3772689151171 * dt * L(f1))
        f2 = es(k2)
        k3 = refine(.56656131914033 * grid + .43343868085967 * k2 + .16352294089771 * dt * L(f2))
        f3 = es(k3)
        k4 = refine(.09299483444413 * grid + .0000209036962 * k1 + .90698426185967 * k3
                    + .00071997378654 * dt * L_zero + .34217696850008 * dt * L(f3))
        f4 = es(k4)
        return refine(.0073613226092 * grid + .20127980325145 * k1 + .00182955389682 * k2 + .78952932024253 * k4
                      + (dt * (.0027771981946 * L_zero + .00001567934613 * L(f1) + .29786487010104 * L(f4))))
    if it == "ssprk43":
        k1 = refine(grid + .5 * dt * L_zero)
        f1 = es(k1)
        k2 = refine(k1 + .5 * dt * L(f1))
        f2 = es(k2)
        k3 = refine(1 / 6 * (4 * grid + 2 * k2 + dt * L(f2)))
        f3 = es(k3)
        return refine(k3 + .5 * dt * L(f3))
    if it == "ssprk33":
        k1 = refine(grid + dt * L_zero)
        f1 = es(k1)
        k2 = refine(.25 * (3 * grid + k1 + dt * L(f1)))
        f2 = es(k2)
        return refine(1 / 3 * (grid + 2 * k2 + 2 * dt * L(f2)))
    if it == "ssprk22":
        k1 = refine(grid + dt * L_zero)
        f1 = es(k1)
        return refine(.5 * (grid + k1 + dt * L(f1)))
    if it == "rk4":
        k1 = refine(grid + .5 * dt * L_zero)
        f1 = es(k1)
        k2 = refine(grid + .5 * dt * L(f1))
        f2 = es(k2)
        k3 = refine(grid + dt * L(f2))
        f3 = es(k3)
        return refine(grid + 1 / 6 * (dt * (L_zero + 2 * L(f1) + 2 * L(f2) + L(f3))))
    if it == "euler":
        return refine(grid + dt * L_zero)
    raise ValueError(it)


def initial_order(dim):
    return [0] if dim == 1 else [0, 1]


def timestep(fluxes, cfg, order):
    """``dt = cfl * min_axes(dx / eigmax)`` (astrea.py:70-71)."""
    return cfg.cfl * min([cfg.dx / fluxes[a]["eigmax"] for a in order])


def step(grid, cfg, t, idx, order):
    """One pass of the core_run loop body (astrea.py:66-85); returns (grid, t, idx, order, dt)."""
    chkpt = cfg.t_end / cfg.checkpoints
    fluxes = evolve_space(grid, cfg, order)
    dt = timestep(fluxes, cfg, order)
    if t + dt >= chkpt * idx:
        dt = chkpt * idx - t
        idx += 1
    grid = evolve_time(grid, fluxes, dt, cfg, order)
    return grid, t + dt, idx, order[::-1], dt


def run(grid, cfg, max_steps=None):
    """Advance to ``cfg.t_end`` like core_run (astrea.py:44-85); returns (grid, t, steps, dts)."""
    t, idx, order, n, dts = 0., 1, initial_order(cfg.dim), 0, []
    with np.errstate(all="ignore"):
        while t <= cfg.t_end:
            if t == cfg.t_end or (max_steps is not None and n >= max_steps):
                break
            grid, t, idx, order, dt = step(grid, cfg, t, idx, order)
            dts.append(dt)
            n += 1
    return grid, t, n, dts


def initialise(w_point, cfg):
    """Point primitives -> cell-averaged conservatives (constructor.initialise, :105-109)."""
    axes = list(range(cfg.dim))
    q = convert_primitive(w_point, cfg, axes)
    return fv.centre_to_avg(q, cfg.bc, axes)
