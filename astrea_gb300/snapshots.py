"""Snapshots of a run, written while the GPU keeps stepping (astrea.py:44-50, 151-175).

The reference saves the primitive grid before every step and at t_end into
an HDF5 file: one group per run (its access key) with the attributes
config, cells, cfl, gamma, dimension, subgrid, timestep and solver, and one
dataset per ``str(float(t))`` with the attribute ``t`` (gzip level 9); the
file carries ``datetime`` and ``seed``.  ``run_with_snapshots`` produces the
same sequence of snapshots without stopping the device:

* on the solver's stream: the conservative -> primitive kernel into one of two
  device buffers, then an asynchronous read of the device clock (t, steps,
  done) into page-locked memory, then the next ``every`` steps;
* on a copy stream, after the primitives are ready: the copy into one of two
  page-locked host buffers;
* on a writer thread, after that copy: the dataset is written.

Stores: ``HDF5Store`` writes the reference's layout with h5py where it is
installed; ``DirectoryStore`` writes the same groups, names and attributes as
a directory tree (``attrs.json``, ``<group>/attrs.json``, ``<group>/index.jsonl``
with one line per dataset in write order, and one ``.npy`` per dataset) where
it is not.
"""

import ctypes
import json
import os
import queue
import threading
from datetime import datetime

import numpy as np
import torch

from . import _lib
from .solver import MODEL_VARS, _stream


class DirectoryStore:
    """The reference's HDF5 layout as a directory tree (for hosts without h5py)."""

    def __init__(self, path, file_attrs=None):
        self.path = path
        os.makedirs(path, exist_ok=True)
        self._write_json(os.path.join(path, "attrs.json"), file_attrs or {})

    @staticmethod
    def _write_json(p, obj):
        tmp = p + ".tmp"
        with open(tmp, "w") as f:
            json.dump(obj, f, indent=1, sort_keys=True)
        os.replace(tmp, p)

    def create_group(self, key, attrs):
        os.makedirs(os.path.join(self.path, key), exist_ok=True)
        self._write_json(os.path.join(self.path, key, "attrs.json"), attrs)
        open(os.path.join(self.path, key, "index.jsonl"), "w").close()

    def write(self, key, name, array, attrs):
        # the array first, then its index line: a reader never sees a line without its data
        np.save(os.path.join(self.path, key, name + ".npy"), array)
        with open(os.path.join(self.path, key, "index.jsonl"), "a") as f:
            f.write(json.dumps({"name": name, "attrs": attrs}) + "\n")

    def close(self):
        pass


class HDF5Store:
    """The reference's file layout through h5py (gzip level 9, as astrea.py:48)."""

    def __init__(self, path, file_attrs=None):
        import h5py
        self.h5py = h5py
        self.path = path
        with h5py.File(path, "w") as f:
            for k, v in (file_attrs or {}).items():
                f.attrs[k] = v

    def create_group(self, key, attrs):
        with self.h5py.File(self.path, "a") as f:
            g = f.create_group(key)
            for k, v in attrs.items():
                g.attrs[k] = v

    def write(self, key, name, array, attrs):
        with self.h5py.File(self.path, "a") as f:
            d = f[key].create_dataset(name, data=array, compression="gzip", compression_opts=9)
            for k, v in attrs.items():
                d.attrs[k] = v

    def close(self):
        pass


def open_store(path, file_attrs=None):
    """An HDF5 store where h5py is installed, else a directory store at ``path`` (suffix .d)."""
    try:
        import h5py  # noqa: F401
        return HDF5Store(path, file_attrs)
    except ImportError:
        return DirectoryStore(path + ".d" if path.endswith((".h5", ".hdf5")) else path, file_attrs)


def read_directory_run(path, key):
    """[(name, attrs, array)] of one run of a ``DirectoryStore``, in write order."""
    with open(os.path.join(path, key, "index.jsonl")) as f:
        index = [json.loads(line) for line in f if line.strip()]
    return [(e["name"], e["attrs"], np.load(os.path.join(path, key, e["name"] + ".npy"))) for e in index]


def group_attrs(cfg, config="", subgrid=None, timestep=None, solver=None):
    """The run group's attributes (astrea.py:166-173) from a ``RunConfig``."""
    return {"config": config, "cells": int(cfg.n0), "cfl": float(cfg.cfl), "gamma": float(cfg.gamma),
            "dimension": int(cfg.dim), "subgrid": subgrid or cfg.scheme, "timestep": timestep or cfg.integrator,
            "solver": solver or cfg.solver}


def _reference_layout(planes, model, dim):
    nv, n0, n1 = planes.shape
    out = np.zeros((n0, n1, 8), dtype=planes.dtype)
    out[..., MODEL_VARS[model]] = np.transpose(planes, (1, 2, 0))
    return out[:, 0, :] if dim == 1 else out


def run_with_snapshots(solver, store, key, attrs=None, every=1, max_snapshots=None, graph=True):
    """Run ``solver`` from its current state to t_end, writing the primitive snapshot before
    every ``every`` steps and at the end into group ``key`` of ``store``.  Returns the list of
    (t, steps) of the snapshots written."""
    if every < 1:
        raise ValueError("every must be >= 1")
    cfg = solver.cfg
    store.create_group(key, attrs if attrs is not None else group_attrs(cfg))
    lib = solver.lib
    dev = [torch.empty_like(solver.state) for _ in range(2)]
    host = [torch.empty(solver.state.shape, dtype=solver.state.dtype).pin_memory() for _ in range(2)]
    t_h = [torch.zeros(1, dtype=torch.float64).pin_memory() for _ in range(2)]
    steps_h = [torch.zeros(1, dtype=torch.int32).pin_memory() for _ in range(2)]
    done_h = [torch.zeros(1, dtype=torch.int32).pin_memory() for _ in range(2)]
    free = [threading.Event(), threading.Event()]
    for f in free:
        f.set()
    copy_stream = torch.cuda.Stream(solver.state.device)
    jobs = queue.Queue()
    written, finished, failure = [], threading.Event(), []

    def writer():
        try:
            while True:
                job = jobs.get()
                if job is None:
                    return
                b, ready = job
                ready.synchronize()
                t, steps, done = float(t_h[b].item()), int(steps_h[b].item()), int(done_h[b].item())
                if not finished.is_set():
                    snap = _reference_layout(host[b].numpy(), cfg.model, cfg.dim)
                    store.write(key, str(float(t)), snap, {"t": float(t)})
                    written.append((t, steps))
                    if t >= cfg.t_end or done:
                        finished.set()
                free[b].set()
        except BaseException as e:  # surfaced by the caller
            failure.append(e)
            finished.set()
            for f in free:
                f.set()

    th = threading.Thread(target=writer, daemon=True)
    th.start()
    compute = torch.cuda.current_stream(solver.state.device)
    b, count = 0, 0
    try:
        while not finished.is_set() and (max_snapshots is None or count < max_snapshots):
            free[b].wait()
            if finished.is_set():
                break
            free[b].clear()
            _lib.check(lib.astrea_to_primitive(solver.handle, ctypes.c_void_p(solver.state.data_ptr()),
                                               ctypes.c_void_p(dev[b].data_ptr()), _stream()))
            _lib.check(lib.astrea_clock_async(solver.handle, ctypes.c_void_p(t_h[b].data_ptr()),
                                              ctypes.c_void_p(steps_h[b].data_ptr()),
                                              ctypes.c_void_p(done_h[b].data_ptr()), _stream()))
            ev = torch.cuda.Event()
            ev.record(compute)
            copy_stream.wait_event(ev)
            with torch.cuda.stream(copy_stream):
                host[b].copy_(dev[b], non_blocking=True)
                ready = torch.cuda.Event()
                ready.record(copy_stream)
            jobs.put((b, ready))
            count += 1
            solver.step(every, graph=graph)  # steps past t_end do nothing
            b ^= 1
    finally:
        jobs.put(None)
        th.join()
        torch.cuda.synchronize(solver.state.device)
        store.close()
    if failure:
        raise failure[0]
    return written


def new_file_attrs(seed=0):
    """The file's attributes (astrea.py:154-156)."""
    return {"datetime": datetime.now().strftime("%Y-%m-%d %H:%M:%S"), "seed": int(seed)}
