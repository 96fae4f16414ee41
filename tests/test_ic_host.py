"""Host side of the device initial conditions: name dispatch and the ABI struct."""

import ctypes
import os

import numpy as np

from astrea_gb300 import initial as I

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "initial_conditions.npz")


def test_config_names_map_like_constructor_initialise():
    assert I.kind_of("sod", 1) == (I.SPLIT, 0)
    assert I.kind_of("sedov", 1) == (I.SPLIT, 1)
    assert I.kind_of("sq", 1) == (I.SPLIT, 1)
    assert I.kind_of("shu-osher", 1) == (I.SHU, 0)
    assert I.kind_of("sine", 1) == (I.SINE, 0)
    assert I.kind_of("gauss", 1) == (I.GAUSS, 0)
    assert I.kind_of("lin", 1) == (I.LINEAR, 0)
    assert I.kind_of("lin mhd", 1) == (I.LINEAR_MHD, 0)
    assert I.kind_of("sedov", 2) == (I.RADIAL, 0)
    assert I.kind_of("mhd blast", 2) == (I.RADIAL, 0)
    assert I.kind_of("rotor", 2) == (I.RADIAL, 0)
    assert I.kind_of("gauss", 2) == (I.GAUSS, 0)
    assert I.kind_of("khi", 2) == (I.KHI, 0)
    assert I.kind_of("ivc", 2) == (I.VORTEX, 0)
    assert I.kind_of("ll3", 2) == (I.QUADRANT, 0)
    assert I.kind_of("orszag-tang", 2) == (I.OT, 0)
    assert I.kind_of("sod", 2) == (I.SPLIT, 0)


def test_ic_struct_layout():
    # 4 ints, 3 doubles, 4 x 8 doubles, 9 doubles (include/astrea_gb300.h)
    assert ctypes.sizeof(I.IC) == 4 * 4 + 8 * (3 + 32 + 9)
    assert I.IC.left.offset == 16 + 24


def test_golden_file_covers_every_kind():
    g = np.load(GOLDEN)
    kinds = {I.kind_of(str(g[f"c{i}_config"]), int(g[f"c{i}_dim"]))[0]
             for i in range(len([k for k in g.files if k.endswith("_config")]))}
    assert kinds == set(range(11))
