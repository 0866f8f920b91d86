"""``wsolve`` mirror (src/io.jl:118-133): integrate on the device and store every stride-th step.

The reference streams the selected components into HDF5 datasets extended along a trailing time
axis (io.jl:33-38, :68-79). HDF5 is not available here, so the same datasets (one per name in
``ustrs`` plus ``tstr``, shape (component shape..., nt)) are written to an ``.npz`` file; ``append``
concatenates onto an existing file, ``force`` overwrites.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import _capi as C
from .equation import ArrayPartition, ODEProblem


def integrate_record(model, u0: np.ndarray, t0: float, t1: float, stride: int = 1, max_records: int = 10000,
                     reltol=1e-6, abstol=1e-8, dt=1e-8, dtmax=np.inf, dtmin=1e-14, maxiters=10**9, alg="Tsit5"):
    """gbc_integrate_record: returns (u(t1), stats, t_records, u_records)."""
    u = np.ascontiguousarray(u0, dtype=np.float64).copy()
    o = C.SolverOpts(reltol, abstol, dt, dtmax if np.isfinite(dtmax) else 1e300, dtmin, maxiters, C.ALGS[alg])
    s = C.SolverStats()
    t_out = np.zeros(max_records)
    u_out = np.zeros(max_records * u.size)
    nrec = ctypes.c_longlong()
    rc = C.lib().gbc_integrate_record(model.h, C.ptr(u), float(t0), float(t1), ctypes.byref(o), int(stride),
                                      int(max_records), C.ptr(t_out), C.ptr(u_out), ctypes.byref(nrec), ctypes.byref(s))
    if rc < 0 and rc != -5:
        C.check(rc)
    k = nrec.value
    return u, s, t_out[:k], u_out[:k * u.size].reshape(k, u.size)


def wsolve(prob: ODEProblem, file: str, nstep: int, getu, ustrs, tstr: str, stride: int = 1, append: bool = False,
           force: bool = False, max_records: int = 10000, **solver):
    """Integrate ``prob`` on the device and save ``getu(u, t)`` every ``stride`` steps into ``file``.
    ``nstep`` (the reference's buffer length) is accepted for signature compatibility; the device
    keeps its own ring and the host drains it as it goes. Returns the final state."""
    assert tstr not in ustrs, f"Duplicate name of {tstr} in {ustrs}."
    if os.path.exists(file) and not (append or force):
        raise FileExistsError(f"{file} exists (use append=True or force=True)")
    u1, st, ts, us = integrate_record(prob.p, prob.u0.flat(), prob.tspan[0], prob.tspan[1], stride=stride,
                                      max_records=max_records, **solver)
    cols = {name: [] for name in ustrs}
    for k in range(len(ts)):
        parts = getu(ArrayPartition.like(prob.u0, us[k]), ts[k])
        assert len(parts) == len(ustrs), "Unmatched length between solution components and names."
        for name, p in zip(ustrs, parts):
            cols[name].append(np.asarray(p))
    data = {name: np.stack(v, axis=-1) for name, v in cols.items()}
    data[tstr] = np.asarray(ts)
    if append and os.path.exists(file):
        with np.load(file) as z:
            old = dict(z)
        data = {k: np.concatenate([old[k], v], axis=-1) for k, v in data.items()}
    with open(file, "wb") as f:
        np.savez(f, **data)
    return ArrayPartition.like(prob.u0, u1), st
