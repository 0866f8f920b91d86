"""Batched ensembles of independent fault-only cycle models (libgbcycle gbc_ensemble_*), with a
small autotuner for the per-model CTA size."""
from __future__ import annotations

import ctypes
import time

import numpy as np

from . import _capi as C


class Ensemble:
    """Many fault-only models (each the ODE of src/BEM/equation.jl:156-166) in one persistent
    launch with per-model Tsit5 step control."""

    def __init__(self, sizes):
        self.sizes = [(int(nx), int(nxi)) for nx, nxi in sizes]
        n = len(self.sizes)
        nx = (C.I * n)(*[s[0] for s in self.sizes])
        nxi = (C.I * n)(*[s[1] for s in self.sizes])
        h = ctypes.c_void_p()
        C.check(C.lib().gbc_ensemble_create(n, nx, nxi, ctypes.byref(h)))
        self.h = h
        self.n = n
        self.offsets = [int(C.lib().gbc_ensemble_state_offset(h, i)) for i in range(n)]
        self.state_len = int(C.lib().gbc_ensemble_state_len(h))
        self.block = 256

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            C.lib().gbc_ensemble_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self) -> int:
        return int(C.lib().gbc_ensemble_stream(self.h) or 0)

    def assemble(self, i, mf, lam, mu, ftype=0, nrept=2, buffer_ratio=0.0):
        k = C.Keep()
        fs = C.fault_struct(mf, k)
        C.check(C.lib().gbc_ensemble_assemble(self.h, i, ctypes.byref(fs), lam, mu, ftype, nrept, buffer_ratio))

    def set_gf(self, i, gf):
        g = np.asarray(gf)
        if np.iscomplexobj(g):
            flat = g.reshape(-1, order="F")
            buf = np.empty(2 * flat.size)
            buf[0::2], buf[1::2] = flat.real, flat.imag
            C.check(C.lib().gbc_ensemble_set_gf(self.h, i, C.GBC_GF11_DFT, C.ptr(buf)))
        else:
            C.check(C.lib().gbc_ensemble_set_gf(self.h, i, C.GBC_GF11_REAL, C.ptr(np.ascontiguousarray(g.reshape(-1, order="F")))))

    def set_fault_props(self, i, p):
        k = C.Keep()
        f = lambda a: k(np.asarray(a, dtype=np.float64).reshape(-1, order="F"))
        C.check(C.lib().gbc_ensemble_set_fault_props(self.h, i, f(p.a), f(p.b), f(p.L), f(p.σ), float(p.η), float(p.vpl),
                                                     float(p.f0), float(p.v0)))

    def set_block(self, threads: int):
        C.check(C.lib().gbc_ensemble_set_block(self.h, threads))
        self.block = threads

    def set_max_cluster(self, ctas: int):
        C.check(C.lib().gbc_ensemble_set_max_cluster(self.h, ctas))

    def set_regroup(self, on: bool):
        """Move the models still running to larger clusters as others finish (default on)."""
        C.check(C.lib().gbc_ensemble_set_regroup(self.h, int(bool(on))))

    @staticmethod
    def plan_clusters(npatch, done, steps_left, capacity):
        """The cluster size the regrouping gives each model (host only, no GPU): npatch[i] patches,
        done[i] finished, steps_left[i] steps left at the current step size; capacity[g] clusters of
        2**g CTAs the GPU holds at once (g = 0..4)."""
        npatch = np.ascontiguousarray(npatch, dtype=np.int32)
        n = npatch.size
        done = np.ascontiguousarray(np.broadcast_to(done, (n,)), dtype=np.int32)
        left = np.ascontiguousarray(np.broadcast_to(steps_left, (n,)), dtype=np.float64)
        cap = np.ascontiguousarray(capacity, dtype=np.int32)
        if cap.size != 5:
            raise ValueError("capacity holds the clusters of 1, 2, 4, 8 and 16 CTAs")
        out = np.zeros(n, dtype=np.int32)
        ip = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
        C.check(C.lib().gbc_ensemble_plan_clusters(n, ip(npatch), ip(done), C.ptr(left), ip(cap), ip(out)))
        return out

    def set_log_theta(self, on: bool):
        C.check(C.lib().gbc_ensemble_set_log_theta(self.h, int(bool(on))))

    def _opts(self, reltol, abstol, dt, dtmax, maxiters, alg="Tsit5"):
        return C.SolverOpts(reltol, abstol, dt, dtmax if np.isfinite(dtmax) else 1e300, 1e-14, maxiters, C.ALGS[alg])

    def integrate(self, u, t0, t1, reltol=1e-6, abstol=1e-8, dt=1e-8, dtmax=np.inf, maxiters=10**9, alg="Tsit5"):
        """Host state (concatenated (v, θ, δ) per model) from t0[i] to t1[i] with "Tsit5" or "VCABM5";
        returns (u, stats)."""
        u = np.ascontiguousarray(u, dtype=np.float64).copy()
        t0 = np.ascontiguousarray(np.broadcast_to(t0, (self.n,)), dtype=np.float64)
        t1 = np.ascontiguousarray(np.broadcast_to(t1, (self.n,)), dtype=np.float64)
        st = (C.SolverStats * self.n)()
        o = self._opts(reltol, abstol, dt, dtmax, maxiters, alg)
        rc = C.lib().gbc_ensemble_integrate(self.h, C.ptr(u), C.ptr(t0), C.ptr(t1), ctypes.byref(o), st)
        if rc < 0 and rc != -5:
            C.check(rc)
        return u, list(st)

    def integrate_dev(self, u_ptr, t0, t1, reltol=1e-6, abstol=1e-8, dt=1e-8, dtmax=np.inf, maxiters=10**9,
                      alg="Tsit5"):
        t0 = np.ascontiguousarray(np.broadcast_to(t0, (self.n,)), dtype=np.float64)
        t1 = np.ascontiguousarray(np.broadcast_to(t1, (self.n,)), dtype=np.float64)
        st = (C.SolverStats * self.n)()
        o = self._opts(reltol, abstol, dt, dtmax, maxiters, alg)
        rc = C.lib().gbc_ensemble_integrate_dev(self.h, ctypes.c_void_p(u_ptr), C.ptr(t0), C.ptr(t1), ctypes.byref(o), st)
        if rc < 0 and rc != -5:
            C.check(rc)
        return list(st)

    def autotune(self, u0, steps=200, candidates=(128, 256, 512), **solver):
        """Times the same fixed number of steps for every model (a horizon too long to reach,
        capped by maxiters) with each CTA size and keeps the fastest: per-step cost, not the mix of
        cheap and expensive steps in a short time window, decides."""
        solver = {k: v for k, v in solver.items() if k != "maxiters"}
        timings = {}
        for b in candidates:
            self.set_block(b)
            t0 = time.perf_counter()
            self.integrate(u0, 0.0, 1e15, maxiters=steps, **solver)
            timings[b] = time.perf_counter() - t0
        best = min(timings, key=timings.get)
        self.set_block(best)
        return best, timings
