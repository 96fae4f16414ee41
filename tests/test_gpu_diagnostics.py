"""Device diagnostics (total variation, solution-error norms) against the reference's functions.

The golden file holds seeded primitive snapshots and the outputs of the
reference's calculate_TV and calculate_solution_error (L1, L2, max).  The
device reductions sum in a different order than NumPy, so the bar is 1e-12
relative per quantity (the quantities are sums of O(1e3) terms).
"""

import os

import numpy as np
import pytest
import torch

from astrea_gb300 import diagnostics
from astrea_gb300.solver import to_planes

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "diagnostics.npz")


def planes(w):
    return to_planes(w, 8, torch.float64, "cuda")


def close(a, b):
    return np.all(np.abs(a - b) <= 1e-12 * np.maximum(np.abs(b), 1e-300))


@pytest.mark.parametrize("name,dim", [("tv1", 1), ("tv2", 2)])
def test_total_variation(name, dim):
    g = np.load(GOLDEN)
    got = diagnostics.total_variation(planes(g[name + "_w"]), dim, float(g[name + "_gamma"]))
    assert close(got, g[name + "_tv"]), (got, g[name + "_tv"])


@pytest.mark.parametrize("name,dim", [("err1", 1), ("err2", 2)])
@pytest.mark.parametrize("norm", [1, 2, 99])
def test_solution_error(name, dim, norm):
    g = np.load(GOLDEN)
    got = diagnostics.solution_error(planes(g[name + "_w"]), planes(g[name + "_theo"]), dim,
                                     float(g[name + "_gamma"]), norm)
    assert close(got, g[f"{name}_norm{norm}"]), (got, g[f"{name}_norm{norm}"])
