"""Golden outputs of the reference's diagnostics (functions/analytic.py).

Run where a checkout of the reference (mervyzr/astrea) is available:

    python tests/golden/make_diag_golden.py --reference <path>   (or set ASTREA_REFERENCE)

Stores seeded primitive snapshots with the reference's calculate_TV,
calculate_solution_error (L1, L2 and max norms against the reference's own
initial state of the config) and calculate_Sod_analytical outputs.
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_golden import load_reference, make_sv, reference_path  # noqa: E402


def main():
    R = load_reference(reference_path())
    sys.path.insert(0, reference_path())
    from functions import analytic  # noqa: E402
    rng = np.random.default_rng(20261203)
    out = {}
    # total variation of a 1D and a 2D snapshot (positive density and pressure)
    for name, shape, dim in (("tv1", (48, 8), 1), ("tv2", (20, 20, 8), 2)):
        w = rng.uniform(-1, 1, shape)
        w[..., 0] = rng.uniform(.5, 2, shape[:-1])
        w[..., 4] = rng.uniform(.5, 2, shape[:-1])
        sv = make_sv(R, "sod", shape[0], dim, "plm", "lf", "ssprk(3,3)")
        out[name + "_w"] = w
        out[name + "_gamma"] = np.array(sv.gamma)
        out[name + "_tv"] = np.asarray(analytic.calculate_TV({0.0: w}, sv)[0.0], dtype=np.float64)
    # solution error of a perturbed sine state against the reference's initial state
    for name, config, dim, n in (("err1", "sin", 1, 64), ("err2", "gauss", 2, 24)):
        sv = make_sv(R, config, n, dim, "plm", "lf", "ssprk(3,3)")
        theo = R["constructor"].initialise(sv)
        w = theo * (1 + 1e-3 * rng.standard_normal(theo.shape))
        out[name + "_w"] = w
        out[name + "_theo"] = theo
        out[name + "_gamma"] = np.array(sv.gamma)
        for norm in (1, 2, 99):
            out[f"{name}_norm{norm}"] = np.asarray(analytic.calculate_solution_error(w, sv, norm), dtype=np.float64)
    # Sod exact solution at t = 0.2 on the 1D Sod initial state
    sv = make_sv(R, "sod", 128, 1, "plm", "lf", "ssprk(3,3)")
    g0 = R["constructor"].initialise(sv)
    out["sod_w"] = g0
    out["sod_exact"] = analytic.calculate_Sod_analytical(g0, .2, sv)
    for f in ("gamma", "start_pos", "end_pos", "shock_pos"):
        out["sod_" + f] = np.array(float(getattr(sv, f)))
    np.savez_compressed(os.path.join(HERE, "diagnostics.npz"), **out)
    print("wrote", len(out), "arrays")


if __name__ == "__main__":
    main()
