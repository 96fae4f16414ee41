"""The oracle's operation counter (oracle/flops.py): known answers, and the
counts of the benchmark workloads' steps."""

import numpy as np

from oracle import flops, stepper


def test_counter_known_answers():
    a = np.arange(10, dtype=np.float64).view(flops.Counted)
    with flops.counting() as tally:
        b = a * 2.0 + 1.0          # 20 operations
        c = np.sqrt(b) - a         # 20
        d = np.maximum(c, 0.0)     # comparisons do not count
        e = np.where(d > 1, d, a)  # selections do not count
        s = np.sum(e)              # a reduction: 9 additions
        np.divide(a, b, out=np.zeros_like(a), where=a > 4)  # 5 divisions
    assert isinstance(e, flops.Counted) and float(s) > 0
    assert tally.ops == 20 + 20 + 9 + 5


def test_headline_step_count():
    # one SSPRK3 step of the 2D shear layer (PPM + flattening + viscosity, textbook HLLC) on the
    # reference's 8-variable layout: about 10.6 thousand operations per cell-update
    n = 16
    x = flops.ops_per_cell_update(flops.shear_point(n), flops.headline_cfg(n))
    assert 10000 < x < 11500
    assert x == flops.ops_per_cell_update(flops.shear_point(n), flops.headline_cfg(n))


def test_sod_step_count():
    n = 256
    xs = (np.arange(n) + .5) / n
    w = np.zeros((n, 8))
    w[:, 0] = np.where(xs <= .5, 1.0, .125)
    w[:, 4] = np.where(xs <= .5, 1.0, .1)
    cfg = stepper.OracleConfig(dim=1, scheme="plm", solver="llf", integrator="ssprk33", gamma=1.4, bc="edge",
                               dx=1.0 / n, cfl=.8, eig="analytic", t_end=.2)
    x = flops.ops_per_cell_update(w, cfg)
    assert 900 < x < 1300
