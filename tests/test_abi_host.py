"""CPU-side checks of the C ABI library and of the host-side configuration logic."""

import ctypes
import os
import re

import numpy as np
import pytest

from astrea_gb300 import _lib
from astrea_gb300 import config as C
from astrea_gb300.solver import RunConfig, pick_model, to_planes, from_planes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "astrea_gb300.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(astrea_[a-z_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(_lib.LIB_PATH):
        from astrea_gb300 import build
        build.build()
    return ctypes.CDLL(_lib.LIB_PATH)


def test_library_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 14
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(_lib.EXPORTS) <= set(names)


def test_version_and_error_string_without_gpu(lib):
    lib.astrea_version.restype = ctypes.c_int
    lib.astrea_last_error.restype = ctypes.c_char_p
    assert lib.astrea_version() >= 100
    assert isinstance(lib.astrea_last_error(), bytes)


def test_create_rejects_bad_config_before_touching_the_gpu():
    L = _lib.load()
    h = ctypes.c_void_p()
    bad = _lib.Cfg(dim=3, n0=64, n1=1, model=3, precision=64, gamma=1.4, dx=1.0, cfl=.5, t_end=1.0, checkpoints=1)
    assert L.astrea_create(ctypes.byref(bad), ctypes.byref(h)) == -1
    assert b"dim" in L.astrea_last_error()
    bad = _lib.Cfg(dim=2, n0=64, n1=64, model=3, precision=64, gamma=1.4, dx=1.0, cfl=.5, t_end=1.0, checkpoints=1)
    assert L.astrea_create(ctypes.byref(bad), ctypes.byref(h)) == -1
    bad = _lib.Cfg(dim=1, n0=64, n1=1, model=3, precision=16, gamma=1.4, dx=1.0, cfl=.5, t_end=1.0, checkpoints=1)
    assert L.astrea_create(ctypes.byref(bad), ctypes.byref(h)) == -1
    # PPM flattening with constrained transport
    bad = RunConfig(dim=2, n0=64, n1=64, model=8, scheme="ppm", solver="hlld", magnetic_2d=True, flatten=True).to_c()
    assert bad.flags == 2 | 4
    assert L.astrea_create(ctypes.byref(bad), ctypes.byref(h)) == -1
    assert b"flattening" in L.astrea_last_error()
    assert L.astrea_step(None, None, 1, None) == -6


@pytest.mark.parametrize("s,expect", [("ppm", "ppm"), ("parabolic", "ppm"), ("p", "ppm"), ("polynomial", "pcm"),
                                      ("plm", "plm"), ("linear", "plm"), ("l", "plm"), ("pcm", "pcm"), ("c", "pcm"),
                                      ("weno", "weno5"), ("weno3", "weno3"), ("weno-7", "weno7"), ("weno 5", "weno5")])
def test_subgrid_strings(s, expect):
    assert C.scheme_of(s) == expect


@pytest.mark.parametrize("s,expect", [("lf", "llf"), ("llf", "llf"), ("lax-wendroff", "llf"), ("lw", "lw"),
                                      ("hllc", "hllc"), ("c", "hllc"), ("hlld", "hlld"), ("d", "hlld")])
def test_solver_strings(s, expect):
    assert C.solver_of(s) == expect


@pytest.mark.parametrize("s,expect", [("ssprk(3,3)", "ssprk33"), ("ssprk33", "ssprk33"), ("ssprk(10,4)", "ssprk104"),
                                      ("ssprk5,4", "ssprk54"), ("ssprk(5,3)", "ssprk53"), ("ssprk43", "ssprk43"),
                                      ("ssprk22", "ssprk22"), ("rk4", "rk4"), ("runge-kutta", "rk4"),
                                      ("euler", "euler"), ("forward euler", "euler")])
def test_timestep_strings(s, expect):
    assert C.integrator_of(s) == expect


def test_handle_variables_derived_fields():
    d = C.handle_variables({"simulation_parameters": {"config": "Orszag-Tang", "cells": 65, "cfl": .4, "gamma": 5 / 3,
                                                      "dimension": 1},
                            "numerical_parameters": {"precision": "float64", "subgrid": "WENO5", "timestep": "SSPRK(3,3)",
                                                     "solver": "HLLD"}})
    assert d["cells"] == 64 and d["dimension"] == 2 and d["magnetic_2d"]
    assert d["permutations"] == {0: (0, 1, 2), 1: (1, 0, 2)} and d["ortho_axis"] == (1, 0, 2)
    assert d["solver_category"] == "hll"
    d = C.handle_variables({"config": "brio-wu", "solver": "hllc", "subgrid": "nonsense"})
    assert d["solver"] == "lf" and d["subgrid"] == "pcm"


def test_model_choice_and_layout_round_trip():
    import torch
    g = np.random.default_rng(0).standard_normal((6, 5, 8))
    g[..., 3] = 0
    g[..., 5:] = 0
    assert pick_model(2, "hllc", g) == 4
    assert pick_model(2, "hlld", g) == 8
    g2 = g.copy()
    g2[..., 6] = 1.0
    assert pick_model(2, "llf", g2) == 8
    p = to_planes(g, 4, torch.float64, "cpu")
    assert p.shape == (4, 6, 5)
    assert np.array_equal(from_planes(p, 4, 2).numpy(), g)


def test_runconfig_rejects_unprovided_methods():
    for s in ("os", "osher-solomon", "es", "entropy-stable"):
        with pytest.raises(C.ConfigError):
            C.solver_of(s)
    with pytest.raises(C.ConfigError):
        RunConfig(dim=1, n0=64, solver="roe").to_c()
    assert RunConfig(dim=1, n0=64, solver="lw").to_c().solver == 3  # Lax-Wendroff: ASTREA_LW
    with pytest.raises(C.ConfigError):
        RunConfig(dim=2, n0=64, n1=64, model=8, solver="hlld", integrator="rk4", magnetic_2d=True).to_c()
    # every integrator of the reference is provided without constrained transport
    for it in ("euler", "ssprk22", "ssprk33", "ssprk43", "ssprk53", "ssprk54", "ssprk104", "rk4"):
        assert RunConfig(dim=1, n0=64, integrator=it).to_c().integrator == C.INTEGRATOR[it]
