"""Parameter sweeps on one geometry (libgbcycle gbc_sweep_*): variants of a viscoelastic model that
share its block-scaled BF16 Green's functions and differ in properties and initial state, integrated
together so that every right-hand side is one matrix product over all variants' states -- on the
tensor cores (engine "umma") or the FP32 pipe (engine "simt", each variant's sums in the single
model's order)."""
from __future__ import annotations

import ctypes
import time

import numpy as np

from . import _capi as C
from .equation import GB300Model, _fcol

ENGINES = {"simt": C.GBC_SWEEP_SIMT, "umma": C.GBC_SWEEP_UMMA}


class Sweep:
    """``nvariants`` copies of ``base`` (a GB300Model with mantle, in GBC_PREC_BF16, Green's
    functions and properties set). Each variant starts with the base's properties; ``base`` must
    outlive the sweep and keep its Green's functions."""

    def __init__(self, base: GB300Model, nvariants: int, engine: str = "umma"):
        h = ctypes.c_void_p()
        C.check(C.lib().gbc_sweep_create(base.h, int(nvariants), ctypes.byref(h)))
        self.h = h
        self.base = base
        self.n = int(nvariants)
        self.state_len = int(C.lib().gbc_sweep_state_len(h))
        self.set_engine(engine)

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            C.lib().gbc_sweep_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self) -> int:
        return int(C.lib().gbc_sweep_stream(self.h) or 0)

    def set_engine(self, engine: str):
        C.check(C.lib().gbc_sweep_set_engine(self.h, ENGINES[engine]))
        self.engine = engine

    def set_fault_product(self, on: bool):
        """Run the fault-fault block in the tensor-core product as well (engine "umma"; default off)."""
        C.check(C.lib().gbc_sweep_set_fault_product(self.h, int(bool(on))))

    def set_fault_props(self, k: int, p):
        """RateStateQuasiDynamicProperty of variant k."""
        for name in ("a", "b", "L", "σ"):
            if np.asarray(getattr(p, name)).size != self.base.N:
                raise ValueError(f"variant {k}: {name} must have {self.base.N} entries")
        keep = C.Keep()
        C.check(C.lib().gbc_sweep_set_fault_props(self.h, int(k), keep(_fcol(p.a)), keep(_fcol(p.b)), keep(_fcol(p.L)),
                                                  keep(_fcol(p.σ)), float(p.η), float(p.vpl), float(p.f0), float(p.v0)))

    def set_mantle_props(self, k: int, p):
        """PowerLawViscosityProperty (or a composite with the base's number of laws) of variant k."""
        keep = C.Keep()
        laws = p.piter if hasattr(p, "piter") else [p]
        gam = np.concatenate([np.asarray(q.γ, dtype=np.float64).ravel() for q in laws])
        nn = np.concatenate([np.asarray(q.n, dtype=np.float64).ravel() for q in laws])
        want = self.base.nlaws * self.base.ne
        if gam.size != want or nn.size != want:
            raise ValueError(f"variant {k}: {len(laws)} law(s) over {gam.size // max(len(laws), 1)} cells, the base model "
                             f"has {self.base.nlaws} over {self.base.ne}")
        d0 = np.asarray(p.dϵ0, dtype=np.float64)
        if d0.size != 6:
            raise ValueError("dϵ0 needs 6 components")
        C.check(C.lib().gbc_sweep_set_mantle_props(self.h, int(k), keep(gam), keep(nn), keep(d0)))

    def rhs(self, u: np.ndarray) -> np.ndarray:
        """du for all variants; u is (nvariants, state_len) of flat ArrayPartition states."""
        u = np.ascontiguousarray(u, dtype=np.float64).reshape(self.n, self.state_len)
        du = np.empty_like(u)
        C.check(C.lib().gbc_sweep_rhs(self.h, C.ptr(u), C.ptr(du)))
        return du

    def rhs_dev(self, u_ptr: int, du_ptr: int):
        """Same on device arrays of nvariants * state_len doubles (the sweep's stream, no sync)."""
        C.check(C.lib().gbc_sweep_rhs_dev(self.h, ctypes.c_void_p(u_ptr), ctypes.c_void_p(du_ptr)))

    def integrate(self, u: np.ndarray, t0: float, t1: float, reltol=1e-6, abstol=1e-8, dt=1e-8, dtmax=np.inf,
                  maxiters=10**9, alg="VCABM5"):
        """Every variant from t0 to t1 with its own step control; returns ((nvariants, state_len), stats)."""
        u = np.ascontiguousarray(u, dtype=np.float64).reshape(self.n, self.state_len).copy()
        o = C.SolverOpts(reltol, abstol, dt, dtmax if np.isfinite(dtmax) else 1e300, 1e-14, maxiters, C.ALGS[alg])
        st = (C.SolverStats * self.n)()
        rc = C.lib().gbc_sweep_integrate(self.h, C.ptr(u), float(t0), float(t1), ctypes.byref(o), st)
        if rc < 0 and rc != -5:
            C.check(rc)
        return u, list(st)

    def integrate_dev(self, u_ptr: int, t0: float, t1: float, reltol=1e-6, abstol=1e-8, dt=1e-8, dtmax=np.inf,
                      maxiters=10**9, alg="VCABM5"):
        """Same on a device array of nvariants * state_len doubles (runs on the sweep's stream)."""
        o = C.SolverOpts(reltol, abstol, dt, dtmax if np.isfinite(dtmax) else 1e300, 1e-14, maxiters, C.ALGS[alg])
        st = (C.SolverStats * self.n)()
        rc = C.lib().gbc_sweep_integrate_dev(self.h, ctypes.c_void_p(u_ptr), float(t0), float(t1), ctypes.byref(o), st)
        if rc < 0 and rc != -5:
            C.check(rc)
        return list(st)

    def autotune(self, u: np.ndarray, candidates=("umma", "simt"), reps: int = 5):
        """Times `reps` right-hand sides of all variants at the states u with each engine and keeps
        the fastest; returns (engine, {engine: seconds})."""
        timings = {}
        for eng in candidates:
            self.set_engine(eng)
            self.rhs(u)  # first call: staging buffers, kernel attributes
            t0 = time.perf_counter()
            for _ in range(reps):
                self.rhs(u)
            timings[eng] = time.perf_counter() - t0
        best = min(timings, key=timings.get)
        self.set_engine(best)
        return best, timings

    def error_word(self) -> int:
        return int(C.lib().gbc_sweep_error_word(self.h))
