"""Loading of the committed golden fixtures (tests/golden/*.npz)."""

import glob
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def case_names(prefix="case_"):
    return sorted(os.path.basename(p)[len(prefix):-4] for p in glob.glob(os.path.join(GOLDEN, prefix + "*.npz")))


def load(name, prefix="case_"):
    with np.load(os.path.join(GOLDEN, f"{prefix}{name}.npz")) as z:
        d = {k: z[k] for k in z.files}
    d["meta"] = json.loads(str(d["meta"]))
    return d


def load_units():
    with np.load(os.path.join(GOLDEN, "unit_functions.npz")) as z:
        return {k: z[k] for k in z.files}
