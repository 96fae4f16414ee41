"""Run configuration: the reference's ``.yml`` keys and accepted strings.

astrea reads its method choices as strings (``subgrid``, ``solver``,
``timestep`` ...) from ``parameters.yml`` and the CLI, validates them against
the accepted lists in ``static/.db.json`` and derives ``solver_category``,
``magnetic_2d``, ``permutations`` and ``ortho_axis``
(functions/generic.py:159-286).  This module accepts the same keys and the
same strings and maps them, at the boundary, onto the integer enums the C ABI
takes (``include/astrea_gb300.h``).  The string->method dispatch follows the
reference's own string tests, quirks included:

* ``subgrid``: ``startswith('w')`` -> WENO (order from the digits, default 5;
  schemes/weno.py:159-165); ``in ['ppm','parabolic','p']`` -> PPM;
  ``in ['plm','linear','l']`` -> PLM; anything else (including the accepted
  ``'polynomial'``) -> PCM (num_methods/evolvers.py:14-21).
* ``solver``: category ``hll``: ``endswith('d')`` -> HLLD else HLLC; category
  ``lax``: ``endswith('w')`` -> Lax-Wendroff else LLF (solvers.py:13-31).
  HLLC on a 1D magnetic config falls back to the default ``lf``
  (generic.py:266-269).
* ``timestep``: ``ssprk(r,o)`` register/order parsing of evolvers.py:79-81;
  ``startswith('r')`` -> RK4; else forward Euler.
"""

import itertools
from collections import namedtuple

import numpy as np

# accepted strings (static/.db.json)
CONFIG_CATEGORIES = {
    "shock": ["sod", "sod shock", "sod-shock", "blast", "sedov", "sedov blast", "sedov wave", "sedov-blast", "sedov-wave"],
    "special": ["shu-osher", "shu osher", "shu", "osher", "so", "toro1", "toro2", "toro3", "toro4", "toro5",
                "toro-1", "toro-2", "toro-3", "toro-4", "toro-5", "toro 1", "toro 2", "toro 3", "toro 4", "toro 5"],
    "interacting": ["slow", "slow-moving", "slow-moving shock", "slow shock", "slow-shock"],
    "smooth": ["sin", "sine", "sine wave", "sine-wave", "gaussian", "gauss", "linear", "lin", "linear mhd", "lin mhd",
               "linear-mhd", "lin-mhd"],
    "stationary": ["square", "sq", "square-wave", "square wave"],
    "magnetic": ["ryu-jones", "rj", "ryu", "jones", "brio-wu", "bw", "brio", "wu"],
    "magnetic-2D": ["orszag-tang", "orszag", "tang", "ot", "mhd rotor", "mhd-rotor", "rotor", "mhd blast", "mhd-blast",
                    "mhd blast wave", "mhd-blast-wave"],
    "2D": ["kelvin-helmholtz", "kelvin-helmholtz instability", "khi", "vortex", "isentropic-vortex", "isentropic vortex",
           "ivc"] + [f"ll{i}" for i in range(1, 20)] + [f"ll {i}" for i in range(1, 20)]
          + [f"lax-liu {i}" for i in range(1, 20)] + [f"lax-liu{i}" for i in range(1, 20)],
}
SUBGRID_ACCEPTED = ["pcm", "constant", "c", "plm", "linear", "l", "ppm", "parabolic", "polynomial", "p",
                    "weno", "weno3", "weno-3", "weno 3", "weno5", "weno-5", "weno 5", "weno7", "weno-7", "weno 7"]
TIMESTEP_ACCEPTED = ["euler", "forward", "forward-euler", "forward euler", "rk4", "runge-kutta", "runge kutta",
                     "runge kutta 4", "runge-kutta 4", "runge-kutta4",
                     "ssprk(2,2)", "ssprk22", "ssprk2,2", "ssprk(3,3)", "ssprk33", "ssprk3,3", "ssprk(4,3)", "ssprk43",
                     "ssprk4,3", "ssprk(5,3)", "ssprk53", "ssprk5,3", "ssprk(5,4)", "ssprk54", "ssprk5,4",
                     "ssprk(10,4)", "ssprk104", "ssprk10,4"]
SOLVER_CATEGORIES = {
    "lax": ["lf", "friedrich", "lax-friedrich", "llf", "local lax-friedrich", "lw", "lax-wendroff", "wendroff"],
    "hll": ["hllc", "c", "hlld", "d"],
    "complete": ["os", "osher", "solomon", "osher-solomon", "osher solomon", "es", "entropy", "entropy-stable"],
}
PRECISION_ACCEPTED = ["float", "float16", "float32", "float64"]
RUN_TYPE_ACCEPTED = ["s", "single", "m", "multiple", "multi", "many"]
DEFAULTS = {"config": "sod", "dimension": 1, "precision": "float64", "subgrid": "pcm", "timestep": "euler",
            "solver": "lf", "run_type": "single"}

# enums shared with include/astrea_gb300.h
SCHEME = {"pcm": 0, "plm": 1, "ppm": 2, "weno3": 3, "weno5": 4, "weno7": 5}
SOLVER = {"llf": 0, "hllc": 1, "hlld": 2, "lw": 3}
INTEGRATOR = {"euler": 0, "ssprk22": 1, "ssprk33": 2, "ssprk43": 3, "ssprk53": 4, "ssprk54": 5, "ssprk104": 6, "rk4": 7}
BOUNDARY = {"edge": 0, "wrap": 1}
LIMITER = {"minmod": 0, "superbee": 1}


class ConfigError(ValueError):
    pass


def config_category(config):
    for cat, names in CONFIG_CATEGORIES.items():
        if config in names:
            return cat
    raise ConfigError(f"unknown config {config!r}")


def solver_category(solver):
    for cat, names in SOLVER_CATEGORIES.items():
        if solver in names:
            return cat
    raise ConfigError(f"unknown solver {solver!r}")


def scheme_of(subgrid):
    """Canonical reconstruction name for a ``subgrid`` string (evolvers.py:14-21, weno.py:159-165)."""
    s = subgrid.lower()
    if s.startswith("w"):
        parts = s.split("weno")
        order = 5
        if len(parts) == 2:
            try:
                order = int(s.replace("-", "").split("weno")[-1])
            except ValueError:
                order = 5
        return f"weno{order}" if order in (3, 7) else "weno5"
    if s in ("ppm", "parabolic", "p"):
        return "ppm"
    if s in ("plm", "linear", "l"):
        return "plm"
    return "pcm"


def solver_of(solver, category=None):
    """Canonical Riemann solver for a ``solver`` string (solvers.py:13-31)."""
    s = solver.lower()
    category = category or solver_category(s)
    if category == "hll":
        return "hlld" if s.endswith("d") else "hllc"
    if category == "complete":
        raise ConfigError(f"solver {solver!r} (Osher-Solomon / entropy-stable) is not provided by astrea_gb300")
    return "lw" if s.endswith("w") else "llf"


def integrator_of(timestep):
    """Canonical integrator for a ``timestep`` string (evolvers.py:79-206)."""
    s = timestep.lower()
    if s.startswith("ssprk"):
        digits = s.replace(",", "").replace("(", "").replace(")", "").replace("ssprk", "")
        register, order = int(digits[:-1]), int(digits[-1])
        if order == 4:
            return "ssprk104" if register == 10 else "ssprk54"
        if order == 3:
            return {5: "ssprk53", 4: "ssprk43"}.get(register, "ssprk33")
        return "ssprk22"
    if s.startswith("r"):
        return "rk4"
    return "euler"


def high_order(subgrid):
    """4th-order prim<->cons conversions for WENO and PPM (generic.py:250-255)."""
    s = subgrid.lower()
    return s.startswith("w") or s in ("ppm", "parabolic", "p")


def permutations_for(dim):
    perms = [axes for axes in itertools.permutations(range(dim + 1)) if axes[-1] == dim]
    return {i: a for i, a in enumerate(perms)}, perms[-1]


def handle_variables(settings, overrides=None):
    """Validate ``.yml``-style settings and add the derived fields (generic.py:159-286).

    ``settings`` may be nested by section as in ``parameters.yml`` or flat.
    Invalid strings fall back to the reference's defaults, like the
    reference; unknown *supported-elsewhere* choices raise ConfigError.
    """
    flat = {}
    for k, v in settings.items():
        if isinstance(v, dict):
            flat.update(v)
        else:
            flat[k] = v
    flat.update(overrides or {})
    out = {}
    for k, v in flat.items():
        if k in ("live_plot", "take_snaps", "save_video", "save_plots", "save_file"):
            v = v if isinstance(v, bool) else False
        elif k in ("checkpoints", "dimension"):
            v = v if isinstance(v, int) else 1
        elif k == "cells":
            try:
                v = int(v) - int(v) % 2
            except (TypeError, ValueError):
                v = 128
        elif k in ("gamma", "cfl"):
            if not isinstance(v, float):
                v = 1.4 if k == "gamma" else .5
            if k == "gamma" and v == 1:
                v += float(np.finfo(flat.get("precision", "float64")).eps)
        elif isinstance(v, str):
            v = v.lower()
            accepted = {"subgrid": SUBGRID_ACCEPTED, "timestep": TIMESTEP_ACCEPTED, "precision": PRECISION_ACCEPTED,
                        "run_type": RUN_TYPE_ACCEPTED,
                        "solver": sum(SOLVER_CATEGORIES.values(), []),
                        "config": sum(CONFIG_CATEGORIES.values(), [])}.get(k)
            if accepted is not None and v not in accepted:
                v = DEFAULTS[k]
        out[k] = v
    for k, v in DEFAULTS.items():
        out.setdefault(k, v)
    out.setdefault("cells", 128)
    out.setdefault("cfl", .5)
    out.setdefault("gamma", 1.4)
    out.setdefault("checkpoints", 1)
    out["config_category"] = config_category(out["config"])
    out["solver_category"] = solver_category(out["solver"])
    out["magnetic_2d"] = out["config_category"] == "magnetic-2D"
    if "2D" in out["config_category"] and out["dimension"] != 2:
        out["dimension"] = 2
    out["permutations"], out["ortho_axis"] = permutations_for(out["dimension"])
    if out["solver_category"] == "hll" and out["solver"].endswith("c") and out["config"] in CONFIG_CATEGORIES["magnetic"]:
        out["solver"] = DEFAULTS["solver"]
        out["solver_category"] = solver_category(out["solver"])
    return out


def make_sim_variables(**fields):
    """A namedtuple with the given fields (the reference passes ``sim_variables`` this way)."""
    return namedtuple("simulation_variables", fields)(**fields)
