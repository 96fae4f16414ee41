"""Pin the CPU oracle against golden vectors produced by the reference itself.

The fixtures in tests/golden/ were written by tests/golden/make_golden.py,
which runs mervyzr/astrea's own evolve_space / evolve_time (and its limiter,
solver and conversion functions) in-process.  The oracle must reproduce
them: bit for bit where no eigenvalue solver is involved, and to 1e-13
(relative to the array's max magnitude) where the reference's LAPACK
eigenvalues enter (LLF speeds, dt), because LAPACK builds differ between
machines.
"""

import numpy as np
import pytest

from astrea_gb300 import config as C
from oracle import fvcore, recon, riemann, stepper
from tests import golden_io

TOL = 1e-13


def rel_err(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    scale = max(np.max(np.abs(b)), 1e-300)
    return float(np.max(np.abs(a - b)) / scale)


def cfg_from_meta(meta, eig="lapack"):
    return stepper.OracleConfig(
        dim=meta["dim"], scheme=C.scheme_of(meta["subgrid"]), solver=C.solver_of(meta["solver"]),
        integrator=C.integrator_of(meta["timestep"]), gamma=meta["gamma"], bc=meta["boundary"], dx=meta["dx"],
        cfl=meta["cfl"], magnetic_2d=meta["magnetic_2d"], eig=eig, t_end=meta["t_end"])


@pytest.mark.parametrize("name", golden_io.case_names())
def test_oracle_matches_reference_steps(name):
    g = golden_io.load(name)
    meta = g["meta"]
    cfg = cfg_from_meta(meta)
    q = g["q0"]
    t, idx, order = 0.0, 1, stepper.initial_order(cfg.dim)
    with np.errstate(all="ignore"):
        for s in range(meta["steps"]):
            if f"flux_s{s}_p0" in g:
                fl = stepper.evolve_space(q, cfg, order)
                for pos, axis in enumerate(order):
                    assert rel_err(fl[axis]["flux"], g[f"flux_s{s}_p{pos}"]) <= TOL, (name, s, pos)
                    assert abs(fl[axis]["eigmax"] - g[f"eigmax_s{s}_p{pos}"]) <= TOL * abs(g[f"eigmax_s{s}_p{pos}"])
                    if f"corner_s{s}_p{pos}" in g:
                        assert rel_err(fl[axis]["mag_corner"], g[f"corner_s{s}_p{pos}"]) <= TOL
            q, t, idx, order, dt = stepper.step(q, cfg, t, idx, order)
            assert abs(dt - g[f"dt_{s + 1}"]) <= TOL * g[f"dt_{s + 1}"], (name, s)
            assert rel_err(q, g[f"q_{s + 1}"]) <= TOL, (name, s, rel_err(q, g[f"q_{s + 1}"]))


def test_oracle_full_run_plain_config_n128():
    g = golden_io.load("sod1d_plm_lf_n128", prefix="full_")
    cfg = cfg_from_meta(g["meta"])
    q, t, n, _ = stepper.run(g["q0"], cfg)
    assert n == g["meta"]["steps"]
    assert t == g["t"]
    assert rel_err(q, g["qT"]) <= 1e-12


def test_oracle_initialise_matches_reference_sod():
    g = golden_io.load("sod1d_ppm_lf")
    cfg = cfg_from_meta(g["meta"])
    n = g["meta"]["cells"]
    dx = 1.0 / n
    x = np.linspace(0 - dx / 2, 1 + dx / 2, n + 2)[1:-1]
    w = np.zeros((n, 8))
    w[:] = [.125, 0, 0, 0, .1, 0, 0, 0]
    w[x <= .5] = [1, 0, 0, 0, 1, 0, 0, 0]
    assert np.array_equal(stepper.initialise(w, cfg), g["q0"])


class TestUnitFunctions:
    u = golden_io.load_units()

    @pytest.mark.parametrize("bc", ["edge", "wrap"])
    def test_slope_limiters(self, bc):
        w = self.u["w"]
        assert np.array_equal(recon.minmod(w, bc), self.u[f"minmod_{bc}"])
        with np.errstate(all="ignore"):
            assert np.array_equal(recon.superbee(w, bc), self.u[f"superbee_{bc}"])

    @pytest.mark.parametrize("bc", ["edge", "wrap"])
    def test_ppm_limiter(self, bc):
        wL, wR, _ = recon.ppm_mc(self.u["w"], bc)
        assert np.array_equal(wL, self.u[f"ppm_wL_{bc}"])
        assert np.array_equal(wR, self.u[f"ppm_wR_{bc}"])

    @pytest.mark.parametrize("bc", ["edge", "wrap"])
    @pytest.mark.parametrize("order", [3, 5, 7])
    def test_weno(self, bc, order):
        q = fvcore.p2c(self.u["w"], 1.4)
        wS = fvcore.ho_c2p(q, 1.4, bc, [0])
        assert np.array_equal(wS, self.u[f"weno{order}_wS_{bc}"])
        wL, wR = recon.weno(wS, bc, order)
        n = len(wS)
        assert np.array_equal(fvcore.gather_range(wL, 0, n + 1, bc), self.u[f"weno{order}_wp_{bc}"])
        assert np.array_equal(fvcore.gather_range(wR, -1, n + 1, bc), self.u[f"weno{order}_wm_{bc}"])

    def test_flux_roe_conversions(self):
        w = self.u["w"]
        for axis in (0, 1, 2):
            assert np.array_equal(fvcore.make_flux(w, 1.4, axis), self.u[f"flux_axis{axis}"])
        assert np.array_equal(fvcore.roe_average(w[1:], w[:-1]), self.u["roe"])
        assert np.array_equal(fvcore.p2c(w, 1.4), self.u["p2c"])
        assert np.array_equal(fvcore.c2p(self.u["p2c"], 1.4), self.u["c2p"])

    @pytest.mark.parametrize("label", [0, 1])
    def test_hllc_hlld(self, label):
        w = self.u["w"]
        wp, wm = w[1:], w[:-1]
        qp, qm = fvcore.p2c(wp, 1.4), fvcore.p2c(wm, 1.4)
        fp, fm = fvcore.make_flux(wp, 1.4, 0), fvcore.make_flux(wm, 1.4, 0)
        with np.errstate(all="ignore"):
            assert np.array_equal(riemann.hllc(label, 1.4, wp, wm, qp, qm, fp, fm), self.u[f"hllc_label{label}"], equal_nan=True)
            wS_right = fvcore.gather_range(w[:-2], 0, len(wp), "edge")
            assert np.array_equal(riemann.hlld(label, 1.4, wS_right, wp, wm, qp, qm, fp, fm), self.u[f"hlld_label{label}"], equal_nan=True)
