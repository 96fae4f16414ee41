#!/usr/bin/env python3
"""Oracle fixture of the full-size headline workload: two FP64 steps at 2048^2.

Usage:  python tests/golden/make_fullsize_golden.py [--n 2048] [--steps 2]

Runs the oracle (the NumPy restatement of the reference's step, test
infrastructure) on the shear-layer workload as bench.py defines it -- 2048^2
periodic, PPM with flattening and artificial viscosity, textbook HLLC
(physical labels), SSPRK3, CFL 0.8, closed-form wave speeds as the kernels
evaluate them -- for two steps (the second sweeps the axes in the other
order).  A full 2048^2 state is 134 MB per step, so the fixture keeps what a
comparison needs: per step the dt, the correctly rounded sum of every
stored plane, and the full rows and columns at the tile seams and at the
shear interfaces.  Takes a few minutes and ~20 GB of host memory.
"""

import argparse
import json
import math
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from bench import shear_layer  # noqa: E402
from oracle import stepper  # noqa: E402

# rows (axis-0 index) and columns (axis-1 index) kept per step: tile seams along and across
# both sweeps (tiles are 32 cells along a sweep, 8 or 15 rows across), the periodic wrap and
# the two shear interfaces (y = 0.25 and 0.75)
ROWS = [0, 1, 14, 15, 31, 32, 1023, 1024, 2046, 2047]
COLS = [0, 1, 14, 15, 31, 32, 511, 512, 1535, 1536, 2047]
VARS = [0, 1, 2, 4]  # the stored planes of 2D Euler: rho, m_x, m_y, E


def exact_sum(x):
    """The correctly rounded sum of an array (math.fsum), which compensated device sums approach."""
    return math.fsum(np.asarray(x, dtype=np.float64).ravel().tolist())


def config(n):
    return stepper.OracleConfig(dim=2, scheme="ppm", solver="hllc", integrator="ssprk33", gamma=1.4, bc="wrap",
                                dx=1.0 / n, cfl=0.8, eig="analytic", t_end=1.0, compat=False, flatten=True,
                                viscosity=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=2048)
    ap.add_argument("--steps", type=int, default=2)
    args = ap.parse_args()
    n = args.n
    cfg = config(n)
    t0 = time.time()
    q = stepper.initialise(shear_layer(n), cfg)
    out = {}
    t, idx, order = 0.0, 1, [0, 1]
    with np.errstate(all="ignore"):
        for k in range(args.steps):
            q, t, idx, order, dt = stepper.step(q, cfg, t, idx, order)
            out[f"dt_{k + 1}"] = np.float64(dt)
            out[f"sums_{k + 1}"] = np.array([exact_sum(q[..., v]) for v in VARS])
            out[f"rows_{k + 1}"] = q[ROWS][..., VARS]
            out[f"cols_{k + 1}"] = q[:, COLS][..., VARS]
            out[f"absmax_{k + 1}"] = np.abs(q[..., VARS]).max(axis=(0, 1))
            print(f"step {k + 1}: dt={dt:.17g}  {time.time() - t0:.0f} s", flush=True)
    meta = dict(n=n, steps=args.steps, rows=ROWS, cols=COLS, vars=VARS,
                workload="shear layer (bench.shear_layer), PPM + flattening + viscosity, textbook HLLC, SSPRK3, "
                         "CFL 0.8, periodic, closed-form wave speeds")
    out["meta"] = np.array(json.dumps(meta))
    np.savez_compressed(os.path.join(HERE, f"fullsize_shear{n}.npz"), **out)


if __name__ == "__main__":
    main()
