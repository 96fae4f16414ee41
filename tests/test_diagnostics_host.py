"""Host part of the diagnostics: the Sod exact solution against the reference's (golden)."""

import os

import numpy as np

from astrea_gb300 import diagnostics

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "diagnostics.npz")


def test_sod_exact_matches_reference():
    g = np.load(GOLDEN)
    got = diagnostics.sod_exact(g["sod_w"], .2, float(g["sod_gamma"]), float(g["sod_start_pos"]),
                                float(g["sod_end_pos"]), float(g["sod_shock_pos"]))
    ref = g["sod_exact"]
    assert got.shape == ref.shape
    assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref))
