"""``assemble`` and the ODE right-hand side on the GPU, mirroring src/BEM/equation.jl.

``assemble(gf, p, u0, tspan)`` (equation.jl:81-89) and
``assemble(gf₁₁, gf₁₂, gf₂₁, gf₂₂, pf, pa, u0, tspan)`` (equation.jl:141-154) return an
``ODEProblem`` whose ``f(du, u, p, t)`` runs the CUDA right-hand side through the C ABI. The
parameter ``p`` is a ``GB300Model``: the device-resident counterpart of the reference's
``(p, alloc, gf, se)`` / ``(pf, pa, alloc₁, alloc₂, gf₁₁, ..., se)`` tuples.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _capi as C
from .property import PowerLawViscosityProperty, RateStateQuasiDynamicProperty


class ArrayPartition:
    """Minimal stand-in for RecursiveArrayTools.ArrayPartition: ``x`` is a tuple of arrays."""

    def __init__(self, *parts):
        self.x = tuple(np.asarray(p, dtype=np.float64) for p in parts)

    def flat(self) -> np.ndarray:
        return np.concatenate([np.asarray(p).reshape(-1, order="F") for p in self.x])

    @classmethod
    def like(cls, other: "ArrayPartition", flat: np.ndarray) -> "ArrayPartition":
        out, off = [], 0
        for p in other.x:
            out.append(flat[off:off + p.size].reshape(p.shape, order="F"))
            off += p.size
        return cls(*out)

    def similar(self) -> "ArrayPartition":
        return ArrayPartition(*[np.zeros_like(p) for p in self.x])


def _fcol(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64).reshape(-1, order="F"))


class GB300Model:
    """Device-resident model: Green's functions, properties and scratch (libgbcycle handle)."""

    def __init__(self, nx: int, nξ: int, ne: int = 0):
        self.nx, self.nξ, self.ne = nx, nξ, ne
        self.N = nx * nξ
        self.dilatancy = False
        self.nlaws = 1
        h = ctypes.c_void_p()
        C.check(C.lib().gbc_model_create(nx, nξ, ne, ctypes.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            C.lib().gbc_model_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self) -> int:
        """The model's cudaStream_t as an integer handle."""
        return int(C.lib().gbc_model_stream(self.h) or 0)

    @property
    def state_len(self) -> int:
        return int(C.lib().gbc_model_state_len(self.h))

    def set_fault_props(self, p: RateStateQuasiDynamicProperty):
        k = C.Keep()
        C.check(C.lib().gbc_model_set_fault_props(self.h, k(_fcol(p.a)), k(_fcol(p.b)), k(_fcol(p.L)), k(_fcol(p.σ)),
                                                  float(p.η), float(p.vpl), float(p.f0), float(p.v0)))

    def set_mantle_props(self, p):
        """PowerLawViscosityProperty or CompositePowerLawViscosityProperty."""
        k = C.Keep()
        if hasattr(p, "piter"):
            gam = np.concatenate([np.asarray(q.γ, dtype=np.float64) for q in p.piter])
            nn = np.concatenate([np.asarray(q.n, dtype=np.float64) for q in p.piter])
            C.check(C.lib().gbc_model_set_mantle_props_composite(self.h, len(p.piter), k(gam), k(nn), k(p.dϵ0)))
            self.nlaws = len(p.piter)
            return
        C.check(C.lib().gbc_model_set_mantle_props(self.h, k(p.γ), k(p.n), k(p.dϵ0)))
        self.nlaws = 1

    def set_dilatancy(self, d):
        k = C.Keep()
        C.check(C.lib().gbc_model_set_dilatancy(self.h, k(_fcol(d.tp)), k(_fcol(d.ϵ)), k(_fcol(d.β)), k(_fcol(d.p0))))
        self.dilatancy = True

    def set_gf(self, which: int, gf):
        g = np.asarray(gf)
        if which == C.GBC_GF11_DFT or (which == C.GBC_GF11_REAL and np.iscomplexobj(g)):
            flat = g.reshape(-1, order="F")
            buf = np.empty(2 * flat.size)
            buf[0::2], buf[1::2] = flat.real, flat.imag
            C.check(C.lib().gbc_model_set_gf(self.h, C.GBC_GF11_DFT, C.ptr(buf)))
            return
        C.check(C.lib().gbc_model_set_gf(self.h, which, C.ptr(_fcol(g))))

    def assemble_gf(self, mf, ma, lam: float, mu: float, ftype=C.GBC_STRIKE_SLIP, nrept: int = 2,
                    buffer_ratio: float = 0.0, qtype="Gauss1"):
        """All Green's functions computed directly into device memory (no host round trip)."""
        from .greens import _ftype, _quad
        k = C.Keep()
        fs = C.fault_struct(mf, k)
        hs = C.hex_struct(ma, k) if ma is not None else None
        qc, qw = _quad(qtype)
        C.check(C.lib().gbc_model_assemble(self.h, ctypes.byref(fs), ctypes.byref(hs) if hs is not None else None,
                                           lam, mu, _ftype(ftype), nrept, buffer_ratio, k(qc), k(qw), len(qw)))

    def save_gf(self, file: str) -> None:
        """Write this model's Green's functions to a file; gf₁₁ as the real Toeplitz kernel, which
        the model holds exactly (the complex rFFT form of the reference also loads)."""
        from .persist import save_greens_functions
        g = {"gf11": self.export_gf(C.GBC_GF11_REAL)}
        if self.ne:
            g.update(gf12=self.export_gf(C.GBC_GF12), gf21=self.export_gf(C.GBC_GF21), gf22=self.export_gf(C.GBC_GF22))
        save_greens_functions(file, **g)

    def load_gf(self, file: str) -> None:
        """Set this model's Green's functions from a file written by save_gf (no assembly)."""
        from .persist import load_greens_functions
        g = load_greens_functions(file)
        which = {"gf12": C.GBC_GF12, "gf21": C.GBC_GF21, "gf22": C.GBC_GF22}
        for k, v in g.items():
            if k == "gf11":  # complex: the rFFT form of stress_greens_function(...; fourier=true)
                self.set_gf(C.GBC_GF11_DFT if np.iscomplexobj(v) else C.GBC_GF11_REAL, v)
            else:
                self.set_gf(which[k], v)

    def export_gf(self, which: int) -> np.ndarray:
        N, M = self.N, 6 * self.ne
        shape = {C.GBC_GF11_REAL: (self.nx, self.nξ, self.nξ), C.GBC_GF12: (M, N), C.GBC_GF21: (N, M),
                 C.GBC_GF22: (M, M)}
        if which == C.GBC_GF11_DFT:
            out = np.zeros(2 * self.nx * self.nξ * self.nξ)
            C.check(C.lib().gbc_model_export_gf(self.h, which, C.ptr(out)))
            return (out[0::2] + 1j * out[1::2]).reshape((self.nx, self.nξ, self.nξ), order="F")
        out = np.zeros(int(np.prod(shape[which])))
        C.check(C.lib().gbc_model_export_gf(self.h, which, C.ptr(out)))
        return out.reshape(shape[which], order="F")

    def export_gf_rows(self, which: int, rows) -> np.ndarray:
        """Chosen rows of GBC_GF12 / GBC_GF21 / GBC_GF22 in the reference layout's numbering
        (k*ne + j for stress component k at cell j; patch i for GF21): array (len(rows), columns)."""
        r = np.ascontiguousarray(rows, dtype=np.int32)
        cols = self.N if which == C.GBC_GF12 else 6 * self.ne
        out = np.zeros(r.size * cols)
        C.check(C.lib().gbc_model_export_gf_rows(self.h, which, r.size, r.ctypes.data_as(ctypes.POINTER(C.I)), C.ptr(out)))
        return out.reshape(r.size, cols)

    def set_precision(self, mode: int):
        C.check(C.lib().gbc_model_set_precision(self.h, mode))

    def set_log_theta(self, on: bool):
        C.check(C.lib().gbc_model_set_log_theta(self.h, int(bool(on))))

    def error_word(self) -> int:
        return int(C.lib().gbc_model_error_word(self.h))

    def clear_error_word(self) -> None:
        C.check(C.lib().gbc_model_clear_error_word(self.h))

    # -- right-hand side --------------------------------------------------------------------------
    def rhs(self, du: ArrayPartition, u: ArrayPartition, t: float = 0.0):
        n = len(u.x)
        ub = [np.ascontiguousarray(p.reshape(-1, order="F")) for p in u.x]
        db = [np.zeros(p.size) for p in u.x]
        up = (C.PD * n)(*[C.ptr(b) for b in ub])
        dp = (C.PD * n)(*[C.ptr(b) for b in db])
        C.check(C.lib().gbc_rhs(self.h, float(t), up, dp, n))
        for dst, src in zip(du.x, db):
            dst[...] = src.reshape(dst.shape, order="F")

    def rhs_flat(self, u: np.ndarray, t: float = 0.0) -> np.ndarray:
        """du for a flat host state (ArrayPartition order)."""
        N, E = self.N, 6 * self.ne
        sizes = ([N, N, N, N] if self.dilatancy else [N, N, N]) if self.ne == 0 else [N, N, E, E, N]
        u = np.ascontiguousarray(u, dtype=np.float64)
        parts = np.split(u, np.cumsum(sizes)[:-1])
        parts = [np.ascontiguousarray(p) for p in parts]
        outs = [np.zeros(s) for s in sizes]
        up = (C.PD * len(sizes))(*[C.ptr(b) for b in parts])
        dp = (C.PD * len(sizes))(*[C.ptr(b) for b in outs])
        C.check(C.lib().gbc_rhs(self.h, float(t), up, dp, len(sizes)))
        return np.concatenate(outs)

    def rhs_dev(self, u_ptr: int, du_ptr: int, t: float = 0.0):
        C.check(C.lib().gbc_rhs_dev(self.h, float(t), ctypes.c_void_p(u_ptr), ctypes.c_void_p(du_ptr)))

    def integrate(self, u: np.ndarray, t0: float, t1: float, reltol=1e-6, abstol=1e-8, dt=1e-8, dtmax=np.inf,
                  dtmin=1e-14, maxiters=10**9, alg="Tsit5"):
        """On-device Tsit5 or VCABM5 from t0 to t1; returns (u(t1), stats)."""
        u = np.ascontiguousarray(u, dtype=np.float64).copy()
        o = C.SolverOpts(reltol, abstol, dt, dtmax if np.isfinite(dtmax) else 1e300, dtmin, maxiters, C.ALGS[alg])
        s = C.SolverStats()
        rc = C.lib().gbc_integrate(self.h, C.ptr(u), float(t0), float(t1), ctypes.byref(o), ctypes.byref(s))
        if rc < 0 and rc != -5:
            C.check(rc)
        return u, s

    def integrate_dev(self, u_ptr: int, t0: float, t1: float, reltol=1e-6, abstol=1e-8, dt=1e-8, dtmax=np.inf,
                      dtmin=1e-14, maxiters=10**9, alg="Tsit5"):
        o = C.SolverOpts(reltol, abstol, dt, dtmax if np.isfinite(dtmax) else 1e300, dtmin, maxiters, C.ALGS[alg])
        s = C.SolverStats()
        rc = C.lib().gbc_integrate_dev(self.h, ctypes.c_void_p(u_ptr), float(t0), float(t1), ctypes.byref(o),
                                       ctypes.byref(s))
        if rc < 0 and rc != -5:
            C.check(rc)
        return s


@dataclass
class ODEProblem:
    """Counterpart of ODEProblem{true}(ode, u0, tspan, p)."""

    f: object
    u0: ArrayPartition
    tspan: tuple
    p: GB300Model


def _gpu_ode(du, u, p: GB300Model, t):
    p.rhs(du, u, t)


def assemble(*args, **kwargs) -> ODEProblem:
    """assemble(gf, p, u0, tspan), assemble(gf, p, dila, u0, tspan) (equation.jl:108-117) or
    assemble(gf₁₁, gf₁₂, gf₂₁, gf₂₂, pf, pa, u0, tspan)."""
    if len(args) == 5:
        gf, p, dila, u0, tspan = args
        nx, nξ = np.asarray(u0.x[0]).shape
        m = GB300Model(nx, nξ, 0)
        m.set_gf(C.GBC_GF11_DFT if np.iscomplexobj(gf) else C.GBC_GF11_REAL, gf)
        m.set_fault_props(p)
        m.set_dilatancy(dila)
        return ODEProblem(_gpu_ode, u0, tuple(tspan), m)
    if len(args) == 4:
        gf, p, u0, tspan = args
        nx, nξ = np.asarray(u0.x[0]).shape
        m = GB300Model(nx, nξ, 0)
        m.set_gf(C.GBC_GF11_DFT if np.iscomplexobj(gf) else C.GBC_GF11_REAL, gf)
        m.set_fault_props(p)
        return ODEProblem(_gpu_ode, u0, tuple(tspan), m)
    if len(args) == 8:
        gf11, gf12, gf21, gf22, pf, pa, u0, tspan = args
        nx, nξ = np.asarray(u0.x[0]).shape
        ne = np.asarray(u0.x[2]).shape[0]
        m = GB300Model(nx, nξ, ne)
        m.set_gf(C.GBC_GF11_DFT if np.iscomplexobj(gf11) else C.GBC_GF11_REAL, gf11)
        m.set_gf(C.GBC_GF12, gf12)
        m.set_gf(C.GBC_GF21, gf21)
        m.set_gf(C.GBC_GF22, gf22)
        m.set_fault_props(pf)
        m.set_mantle_props(pa)
        return ODEProblem(_gpu_ode, u0, tuple(tspan), m)
    raise TypeError("assemble: expected (gf, p, u0, tspan) or (gf11, gf12, gf21, gf22, pf, pa, u0, tspan)")


def solve(prob: ODEProblem, alg="Tsit5", reltol=1e-6, abstol=1e-8, dt=1e-8, dtmax=np.inf, maxiters=10**9):
    """solve(prob, alg; ...) (src/io.jl:125-130): integrates on the device with "Tsit5" or "VCABM5" (the
    reference's example solver) and returns (u(t_end) as ArrayPartition, stats)."""
    u, st = prob.p.integrate(prob.u0.flat(), prob.tspan[0], prob.tspan[1], reltol=reltol, abstol=abstol, dt=dt,
                             dtmax=dtmax, maxiters=maxiters, alg=alg)
    return ArrayPartition.like(prob.u0, u), st
