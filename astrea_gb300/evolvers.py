"""Drop-in replacement for the reference's num_methods/evolvers.py on the GPU.

``evolve_space(grid, sim_variables)`` and ``evolve_time(grid, fluxes, dt,
sim_variables)`` keep the reference signatures (evolvers.py:12, :38): ``grid``
is the (N, 8) or (N, N, 8) conservative array (NumPy or torch), the method is
chosen by the strings in ``sim_variables`` (subgrid, solver, timestep ...),
and the result has the reference's shapes:

* evolve_space -> ``{axes: {'flux': interface fluxes in the sweep frame,
  'eigmax': float}}`` keyed and ordered like ``sim_variables.permutations``;
* evolve_time  -> the updated grid.

``core_run``'s use of ``fluxes`` is only ``eigmax`` (astrea.py:70); the fluxes
of the initial state are recomputed on the device inside evolve_time (they are
a pure function of ``grid``), so ``fluxes`` may come from either evolver.

``simulate`` is the core_run loop (astrea.py:44-85) on the device without the
per-step HDF5 snapshot.
"""

import numpy as np
import torch

from . import config as C
from .solver import Solver, config_from_sim_variables, from_planes

_CACHE = {}


def _order(sv):
    if int(sv.dimension) == 1:
        return 0
    return 0 if list(sv.permutations.keys())[0] == 0 else 1


def _solver_for(grid, sv, precision=64):
    cfg = config_from_sim_variables(sv, precision=precision, grid=grid)
    key = tuple(sorted(cfg.__dict__.items()))
    s = _CACHE.get(key)
    if s is None:
        s = Solver(cfg)
        _CACHE[key] = s
    return s


def _like(x, ref):
    if isinstance(ref, np.ndarray):
        return x.detach().cpu().numpy()
    return x.to(device=ref.device) if isinstance(ref, torch.Tensor) else x


def _flux_aos(F, model, dim):
    # (nv, Ns+1, Nt) -> (Ns+1, Nt, 8); 1D -> (N+1, 8)
    return from_planes(F, model, dim)


def evolve_space(grid, sim_variables, precision=64):
    """Interface fluxes and max wave speeds of every axis (evolvers.py:12-34)."""
    s = _solver_for(grid, sim_variables, precision)
    s.load_conservative(grid)
    (f0, f1), eig = s.space(_order(sim_variables))
    out = {}
    for axis, axes in sim_variables.permutations.items():
        F = f0 if axis == 0 else f1
        out[axes] = {"flux": _like(_flux_aos(F, s.cfg.model, s.cfg.dim), grid), "eigmax": float(eig[axis])}
    return out


def evolve_time(grid, fluxes, dt, sim_variables, precision=64):
    """One Runge-Kutta step of size ``dt`` (evolvers.py:38-206)."""
    s = _solver_for(grid, sim_variables, precision)
    s.load_conservative(grid)
    s.time(float(dt), _order(sim_variables))
    return _like(s.conservative(), grid)


def simulate(sim_variables, grid0, precision=64, max_steps=None, graph=True):
    """Advance a conservative grid to sim_variables.t_end on the device (core_run without IO).

    Returns (final conservative grid like ``grid0``, clock dict).
    """
    cfg = config_from_sim_variables(sim_variables, precision=precision, grid=grid0)
    s = Solver(cfg)
    s.load_conservative(grid0)
    s.reset_clock(0.0, 1, _order(sim_variables))
    clock = s.run(max_steps=max_steps, graph=graph)
    return _like(s.conservative(), grid0), clock


__all__ = ["evolve_space", "evolve_time", "simulate", "C"]
