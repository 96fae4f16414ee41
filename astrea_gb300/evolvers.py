"""Drop-in replacement for the reference's num_methods/evolvers.py on the GPU.

``evolve_space(grid, sim_variables)`` and ``evolve_time(grid, fluxes, dt,
sim_variables)`` keep the reference signatures (evolvers.py:12, :38): ``grid``
is the (N, 8) or (N, N, 8) conservative array (NumPy or torch), the method is
chosen by the strings in ``sim_variables`` (subgrid, solver, timestep ...),
and the result has the reference's shapes:

* evolve_space -> ``{axes: {'flux': interface fluxes in the sweep frame,
  'eigmax': float}}`` keyed and ordered like ``sim_variables.permutations``;
  with ``sim_variables.magnetic_2d`` each entry also carries ``'face_avg'``
  (the sweep's face values in the sweep frame) and ``'mag_corner'`` (the
  corner electric field, transposed per axis as evolvers.py:28-32 stores it);
* evolve_time  -> the updated grid.

``core_run``'s use of ``fluxes`` is only ``eigmax`` (astrea.py:70); the fluxes
of the initial state are recomputed on the device inside evolve_time (they are
a pure function of ``grid``), so ``fluxes`` may come from either evolver.
With ``magnetic_2d``, evolve_time also does what the reference does to its
input (evolvers.py:73-76): the caller's ``grid`` has its B_x / B_y components
overwritten by the face-averaged values of ``fluxes[axes]['face_avg']``.

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
    magnetic = s.cfg.magnetic_2d
    if magnetic:
        (f0, f1), eig, faces, corner = s.space_ct(_order(sim_variables))
    else:
        (f0, f1), eig = s.space(_order(sim_variables))
    out = {}
    for axis, axes in sim_variables.permutations.items():
        F = f0 if axis == 0 else f1
        out[axes] = {"flux": _like(_flux_aos(F, s.cfg.model, s.cfg.dim), grid), "eigmax": float(eig[axis])}
        if magnetic:
            # face values in the sweep frame (data[axes]['wF']); the corner field as evolvers.py:28-32
            # stores it: its transpose for the axis-0 sweep, itself for the axis-1 sweep
            face = faces[axis].permute(1, 2, 0)
            out[axes]["face_avg"] = _like(face if axis == 0 else face.transpose(0, 1), grid)
            out[axes]["mag_corner"] = _like(corner.t() if axis == 0 else corner, grid)
    return out


def evolve_time(grid, fluxes, dt, sim_variables, precision=64):
    """One Runge-Kutta step of size ``dt`` (evolvers.py:38-206)."""
    s = _solver_for(grid, sim_variables, precision)
    s.load_conservative(grid)
    s.time(float(dt), _order(sim_variables))
    new = _like(s.conservative(), grid)
    if s.cfg.magnetic_2d:
        # the reference re-assigns the B components of its input grid to the face averages
        # (evolvers.py:73-76) before stepping; its caller sees that change
        for axis, axes in sim_variables.permutations.items():
            face = fluxes.get(axes, {}).get("face_avg")
            if face is not None:
                back = face.transpose(1, 0, 2) if isinstance(face, np.ndarray) else face.transpose(0, 1)
                grid[..., 5 + axis] = (face if axis == 0 else back)[..., 5 + axis]
    return new


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
