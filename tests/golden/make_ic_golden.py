"""Golden point primitives of the reference's test problems (constructor.initialise).

Run where a checkout of the reference (mervyzr/astrea) is available:

    python tests/golden/make_ic_golden.py --reference <path>   (or set ASTREA_REFERENCE)

For each (config, dimension, cells) it builds ``sim_variables`` with the
reference's own test table (static/tests.py) and calls its
``constructor.initialise`` (without the primitive -> conservative conversion),
whose result is the point primitive grid after its centre -> average step
(``fv.high_order_convert('cntr')``).  It stores that grid together with the
table's values (start/end/shock positions, left/right states, misc, boundary)
so that the GPU tests can rebuild the same ``sim_variables`` without the
reference.
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_golden import load_reference, make_sv, reference_path  # noqa: E402

CASES = [
    ("sod", 1, 64), ("sedov", 1, 64), ("shu-osher", 1, 64), ("sin", 1, 64), ("gauss", 1, 64), ("lin", 1, 64),
    ("lin mhd", 1, 64), ("sq", 1, 64), ("brio-wu", 1, 64), ("toro3", 1, 64),
    ("sod", 2, 24), ("sedov", 2, 24), ("gauss", 2, 24), ("khi", 2, 24), ("ivc", 2, 24), ("ll3", 2, 24),
    ("ll6", 2, 24), ("orszag-tang", 2, 24), ("rotor", 2, 24), ("mhd blast", 2, 24),
]


def main():
    R = load_reference(reference_path())
    out = {}
    for i, (config, dim, n) in enumerate(CASES):
        sv = make_sv(R, config, n, dim, "plm", "lf", "ssprk(3,3)")
        w = R["constructor"].initialise(sv, convert=False)
        key = f"c{i}"
        out[key + "_config"] = np.array(config)
        out[key + "_dim"] = np.array(dim)
        out[key + "_cells"] = np.array(n)
        out[key + "_gamma"] = np.array(sv.gamma)
        out[key + "_boundary"] = np.array(sv.boundary)
        for f in ("start_pos", "end_pos", "shock_pos"):
            out[key + "_" + f] = np.array(float(getattr(sv, f)))
        out[key + "_initial_left"] = np.asarray(sv.initial_left, dtype=np.float64)
        out[key + "_initial_right"] = np.asarray(sv.initial_right, dtype=np.float64)
        misc = sv.misc or {}
        for mk, mv in misc.items():
            out[key + "_misc_" + mk] = np.asarray(mv, dtype=np.float64)
        out[key + "_w"] = np.asarray(w, dtype=np.float64)
    np.savez_compressed(os.path.join(HERE, "initial_conditions.npz"), **out)
    print("wrote", len(CASES), "cases")


if __name__ == "__main__":
    main()
