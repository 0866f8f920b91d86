"""ctypes front end of the CPU FP64 oracle (oracle/*.c).

TEST INFRASTRUCTURE ONLY: the FP64 reference the CUDA path is tested against. Only tests/, __graft_entry__.smoke()
and bench.py's CPU-baseline / reference arm import this module; the product never does.

Parity status: the Okada/strain-volume values are "parity unpinned" against the reference
(GeoGreensFunctions.jl, which holds them, is not vendored and publishes no golden vectors); the
restatement is pinned by physical identities and by the reference's own tests (test/BEM/tests.jl).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libgbc_oracle.so")
_lock = threading.Lock()
_lib = None

D = ctypes.c_double
PD = ctypes.POINTER(ctypes.c_double)
I = ctypes.c_int


class FaultMesh(ctypes.Structure):
    _fields_ = [("nx", I), ("nxi", I), ("x", PD), ("xi", PD), ("y", PD), ("z", PD),
                ("ax", PD), ("axi", PD), ("dx", D), ("dxi", D), ("dep", D), ("dip", D)]


class HexMesh(ctypes.Structure):
    _fields_ = [("ne", I)] + [(n, PD) for n in ("cx", "cy", "cz", "qx", "qy", "qz", "dx", "dy", "dz")]


class Model(ctypes.Structure):
    _fields_ = [("nx", I), ("nxi", I), ("ne", I), ("a", PD), ("b", PD), ("L", PD), ("sigma", PD),
                ("eta", D), ("vpl", D), ("f0", D), ("v0", D), ("gamma", PD), ("n", PD), ("nlaws", I),
                ("deps0", D * 6), ("tp", PD), ("deps", PD), ("beta", PD), ("p0", PD),
                ("gf11_dft", PD), ("gf12", PD), ("gf21", PD), ("gf22", PD)]


class FFTConv(ctypes.Structure):
    _fields_ = [("P", I), ("nx", I), ("nxi", I), ("H", PD)]


ALGS = {"Tsit5": 0, "VCABM5": 1}


class SolverOpts(ctypes.Structure):
    _fields_ = [("reltol", D), ("abstol", D), ("dt0", D), ("dtmax", D), ("dtmin", D),
                ("maxiters", ctypes.c_longlong), ("mantle", I), ("alg", I)]


class SolverStats(ctypes.Structure):
    _fields_ = [("naccept", ctypes.c_longlong), ("nreject", ctypes.c_longlong),
                ("nrhs", ctypes.c_longlong), ("t", D), ("dt", D), ("status", I)]


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc, OpenMP)."""
    srcs = [os.path.join(HERE, f) for f in ("okada_dc3d.c", "hex8_volume.c", "greens.c", "ode.c", "fastconv.c", "gbc_oracle.h", "Makefile")]
    stale = not os.path.exists(LIB_PATH) or any(os.path.getmtime(s) > os.path.getmtime(LIB_PATH) for s in srcs)
    if force or stale:
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(LIB_PATH)
            L.orc_dc3d.argtypes = [D] * 13 + [PD]
            L.orc_dc3d.restype = I
            L.orc_hex8_unit_stresses.argtypes = [PD] + [D] * 11
            L.orc_stress_vol_hex8.argtypes = [PD] + [D] * 9 + [PD, D, D]
            L.orc_gf_ff.argtypes = [ctypes.POINTER(FaultMesh), D, D, I, I, D, PD]
            L.orc_gf_ff_dft.argtypes = [I, I, PD, PD]
            L.orc_gf_fm.argtypes = [ctypes.POINTER(FaultMesh), ctypes.POINTER(HexMesh), D, D, I, I, D, PD, PD, I, PD]
            L.orc_gf_mf.argtypes = [ctypes.POINTER(HexMesh), ctypes.POINTER(FaultMesh), D, D, I, PD]
            L.orc_gf_mm.argtypes = [ctypes.POINTER(HexMesh), D, D, PD, PD, I, PD]
            PI = ctypes.POINTER(ctypes.c_int)
            L.orc_gf_fm_rows.argtypes = [ctypes.POINTER(FaultMesh), ctypes.POINTER(HexMesh), D, D, I, I, D, PD, PD, I, I,
                                         PI, PD]
            L.orc_gf_mf_rows.argtypes = [ctypes.POINTER(HexMesh), ctypes.POINTER(FaultMesh), D, D, I, I, PI, PD]
            L.orc_gf_mm_rows.argtypes = [ctypes.POINTER(HexMesh), D, D, PD, PD, I, I, PI, PD]
            L.orc_ode_fault.argtypes = [ctypes.POINTER(Model)] + [PD] * 5
            L.orc_ode_visco.argtypes = [ctypes.POINTER(Model)] + [PD] * 8
            L.orc_ode_dilatancy.argtypes = [ctypes.POINTER(Model)] + [PD] * 7
            L.orc_integrate.argtypes = [ctypes.POINTER(Model), PD, D, D, ctypes.POINTER(SolverOpts), ctypes.POINTER(SolverStats)]
            L.orc_integrate.restype = I
            L.orc_integrate_record.argtypes = [ctypes.POINTER(Model), PD, D, D, ctypes.POINTER(SolverOpts),
                                               ctypes.POINTER(SolverStats), I, ctypes.c_longlong, PD, PD,
                                               ctypes.POINTER(ctypes.c_longlong)]
            L.orc_integrate_record.restype = I
            L.orc_gl_table.argtypes = [I, PD, PD]
            L.orc_fftconv_init.argtypes = [ctypes.POINTER(Model), ctypes.POINTER(FFTConv)]
            L.orc_fftconv_init.restype = I
            L.orc_fftconv_free.argtypes = [ctypes.POINTER(FFTConv)]
            L.orc_dtau_dt_fft.argtypes = [ctypes.POINTER(FFTConv), ctypes.POINTER(Model), PD, PD]
            L.orc_integrate_many.argtypes = [ctypes.POINTER(ctypes.POINTER(Model)), I, ctypes.POINTER(PD), PD, PD,
                                             ctypes.POINTER(SolverOpts), ctypes.POINTER(SolverStats), I, I]
            L.orc_integrate_many.restype = I
            L.orc_num_threads.restype = I
            L.orc_dtau_dt.argtypes = [ctypes.POINTER(Model), PD, PD]
            L.orc_tsit5_tableau.argtypes = [PD, PD]
            L.orc_abm_coefficients.argtypes = [I, D, PD, PD, PD, PD]
            L.orc_abm_coefficients.restype = None
            _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(PD)


def _c(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class _Keep:
    """Holds numpy buffers alive while a ctypes struct points into them."""

    def __init__(self):
        self.bufs = []

    def __call__(self, a):
        a = _c(a)
        self.bufs.append(a)
        return _p(a)


def fault_struct(mf, keep):
    return FaultMesh(mf.nx, mf.nξ, keep(mf.x), keep(mf.ξ), keep(mf.y), keep(mf.z), keep(np.asarray(mf.ax).reshape(-1)),
                     keep(np.asarray(mf.aξ).reshape(-1)), mf.Δx, mf.Δξ, mf.dep, mf.dip)


def hex_struct(ma, keep):
    return HexMesh(ma.ne, *(keep(getattr(ma, n)) for n in ("cx", "cy", "cz", "qx", "qy", "qz", "Δx", "Δy", "Δz")))


def dc3d(x, y, z, alpha, depth, dip, al1, al2, aw1, aw2, d1, d2, d3):
    u = np.zeros(12)
    rc = lib().orc_dc3d(x, y, z, alpha, depth, dip, al1, al2, aw1, aw2, d1, d2, d3, _p(u))
    return u, rc


def hex8_unit_stresses(x, y, z, qx, qy, qz, T, L, W, mu, nu):
    out = np.zeros(36)
    lib().orc_hex8_unit_stresses(_p(out), x, y, z, qx, qy, qz, T, L, W, mu, nu)
    return out.reshape(6, 6)


def gf_ff(mf, lam, mu, ftype=0, nrept=2, buffer_ratio=0.0, fourier=False):
    keep = _Keep()
    st = np.zeros(mf.nx * mf.nξ * mf.nξ)
    fs = fault_struct(mf, keep)
    if lib().orc_gf_ff(ctypes.byref(fs), lam, mu, ftype, nrept, buffer_ratio, _p(st)) != 0:
        raise AssertionError("Argument `buffer_ratio` must be ≥ 0.")
    st = st.reshape((mf.nx, mf.nξ, mf.nξ), order="F")
    return gf_ff_dft(st) if fourier else st


def gf_ff_dft(st):
    nx, nxi, _ = st.shape
    src = _c(st.reshape(-1, order="F"))
    out = np.zeros(2 * src.size)
    lib().orc_gf_ff_dft(nx, nxi, _p(src), _p(out))
    return (out[0::2] + 1j * out[1::2]).reshape((nx, nxi, nxi), order="F")


def gf_fm(mf, ma, lam, mu, ftype=0, nrept=2, buffer_ratio=0.0, quad=None):
    keep = _Keep()
    qc, qw = quad if quad is not None else (np.zeros(3), np.ones(1))
    qc, qw = _c(qc), _c(qw)
    st = np.zeros(6 * ma.ne * mf.nx * mf.nξ)
    fs, hs = fault_struct(mf, keep), hex_struct(ma, keep)
    if lib().orc_gf_fm(ctypes.byref(fs), ctypes.byref(hs), lam, mu, ftype, nrept, buffer_ratio, _p(qc), _p(qw), len(qw), _p(st)) != 0:
        raise AssertionError("Argument `buffer_ratio` must be ≥ 0.")
    return st.reshape((6 * ma.ne, mf.nx * mf.nξ), order="F")


def gf_mf(ma, mf, lam, mu, ftype=0):
    keep = _Keep()
    st = np.zeros(6 * ma.ne * mf.nx * mf.nξ)
    fs, hs = fault_struct(mf, keep), hex_struct(ma, keep)
    lib().orc_gf_mf(ctypes.byref(hs), ctypes.byref(fs), lam, mu, ftype, _p(st))
    return st.reshape((mf.nx * mf.nξ, 6 * ma.ne), order="F")


def gf_mm(ma, lam, mu, quad=None):
    keep = _Keep()
    qc, qw = quad if quad is not None else (np.zeros(3), np.ones(1))
    qc, qw = _c(qc), _c(qw)
    st = np.zeros((6 * ma.ne) ** 2)
    hs = hex_struct(ma, keep)
    lib().orc_gf_mm(ctypes.byref(hs), lam, mu, _p(qc), _p(qw), len(qw), _p(st))
    return st.reshape((6 * ma.ne, 6 * ma.ne), order="F")


def _ints(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def gf_fm_rows(mf, ma, lam, mu, cells, ftype=0, nrept=2, buffer_ratio=0.0, quad=None):
    """Rows (k*ne + j for k in 0..5) of the fault->mantle Green's function for receiver cells j in
    `cells`: array (len(cells), 6, N)."""
    keep = _Keep()
    qc, qw = quad if quad is not None else (np.zeros(3), np.ones(1))
    qc, qw = _c(qc), _c(qw)
    r = _ints(cells)
    out = np.zeros(6 * r.size * mf.nx * mf.nξ)
    fs, hs = fault_struct(mf, keep), hex_struct(ma, keep)
    if lib().orc_gf_fm_rows(ctypes.byref(fs), ctypes.byref(hs), lam, mu, ftype, nrept, buffer_ratio, _p(qc), _p(qw),
                            len(qw), r.size, r.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), _p(out)) != 0:
        raise AssertionError("Argument `buffer_ratio` must be ≥ 0.")
    return out.reshape(r.size, 6, mf.nx * mf.nξ)


def gf_mf_rows(ma, mf, lam, mu, patches, ftype=0):
    """Rows of the mantle->fault Green's function for receiver patches: array (len(patches), 6ne)."""
    keep = _Keep()
    r = _ints(patches)
    out = np.zeros(r.size * 6 * ma.ne)
    fs, hs = fault_struct(mf, keep), hex_struct(ma, keep)
    lib().orc_gf_mf_rows(ctypes.byref(hs), ctypes.byref(fs), lam, mu, ftype, r.size,
                         r.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), _p(out))
    return out.reshape(r.size, 6 * ma.ne)


def gf_mm_rows(ma, lam, mu, cells, quad=None):
    """Rows (k*ne + j for k in 0..5) of the mantle-mantle Green's function for receiver cells j in
    `cells`: array (len(cells), 6, 6ne)."""
    keep = _Keep()
    qc, qw = quad if quad is not None else (np.zeros(3), np.ones(1))
    qc, qw = _c(qc), _c(qw)
    r = _ints(cells)
    out = np.zeros(r.size * 36 * ma.ne)
    hs = hex_struct(ma, keep)
    lib().orc_gf_mm_rows(ctypes.byref(hs), lam, mu, _p(qc), _p(qw), len(qw), r.size,
                         r.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), _p(out))
    return out.reshape(r.size, 6, 6 * ma.ne)


class OracleModel:
    """The reference's ODE parameter tuple (equation.jl:88,153) as an oracle model."""

    def __init__(self, gf11, pf, gf12=None, gf21=None, gf22=None, pa=None, dila=None):
        self.keep = _Keep()
        nx, nxi, _ = gf11.shape
        ne = 0 if gf12 is None else gf12.shape[0] // 6
        g = np.asarray(gf11)
        if not np.iscomplexobj(g):
            g = gf_ff_dft(g)
        gi = np.empty(2 * g.size)
        flat = g.reshape(-1, order="F")
        gi[0::2], gi[1::2] = flat.real, flat.imag
        null = ctypes.cast(None, PD)
        F = lambda a: self.keep(np.asarray(a, dtype=np.float64).reshape(-1, order="F"))
        if pa is not None and hasattr(pa, "piter"):  # CompositePowerLawViscosityProperty
            gam = np.concatenate([np.asarray(q.γ, dtype=np.float64) for q in pa.piter])
            nn = np.concatenate([np.asarray(q.n, dtype=np.float64) for q in pa.piter])
            nlaws = len(pa.piter)
        elif pa is not None:
            gam, nn, nlaws = pa.γ, pa.n, 1
        self.m = Model(nx, nxi, ne, F(pf.a), F(pf.b), F(pf.L), F(pf.σ),
                       pf.η, pf.vpl, pf.f0, pf.v0,
                       self.keep(gam) if pa is not None else null, self.keep(nn) if pa is not None else null,
                       nlaws if pa is not None else 1,
                       (D * 6)(*(pa.dϵ0 if pa is not None else np.zeros(6))),
                       F(dila.tp) if dila is not None else null, F(dila.ϵ) if dila is not None else null,
                       F(dila.β) if dila is not None else null, F(dila.p0) if dila is not None else null,
                       self.keep(gi),
                       self.keep(gf12.reshape(-1, order="F")) if gf12 is not None else null,
                       self.keep(gf21.reshape(-1, order="F")) if gf21 is not None else null,
                       self.keep(gf22.reshape(-1, order="F")) if gf22 is not None else null)
        self.N, self.ne = nx * nxi, ne
        self.dilatancy = dila is not None

    def ode(self, u):
        """du for the flat state in ArrayPartition order (v, θ, [ϵ, σ,] δ) or (v, θ, δ, 𝓅)."""
        u = _c(u)
        du = np.zeros_like(u)
        N, E = self.N, 6 * self.ne
        if self.dilatancy:
            lib().orc_ode_dilatancy(ctypes.byref(self.m), _p(u[:N]), _p(u[N:2 * N]), _p(u[3 * N:]), _p(du[:N]),
                                    _p(du[N:2 * N]), _p(du[2 * N:3 * N]), _p(du[3 * N:]))
            return du
        if self.ne == 0:
            lib().orc_ode_fault(ctypes.byref(self.m), _p(u[:N]), _p(u[N:2 * N]), _p(du[:N]), _p(du[N:2 * N]), _p(du[2 * N:]))
        else:
            v, th, sig = u[:N], u[N:2 * N], u[2 * N + E:2 * N + 2 * E]
            dv, dth, deps, dsig, dd = (np.zeros(N), np.zeros(N), np.zeros(E), np.zeros(E), np.zeros(N))
            lib().orc_ode_visco(ctypes.byref(self.m), _p(v), _p(th), _p(_c(sig)), _p(dv), _p(dth), _p(deps), _p(dsig), _p(dd))
            du = np.concatenate([dv, dth, deps, dsig, dd])
        return du

    def dtau_dt(self, v):
        """relative_velocity! + dτ_dt! (equation.jl:35-61) on a (nx, nξ) velocity."""
        v = _c(np.asarray(v).reshape(-1, order="F"))
        out = np.zeros_like(v)
        lib().orc_dtau_dt(ctypes.byref(self.m), _p(v), _p(out))
        return out

    def integrate(self, u0, t0, t1, reltol=1e-6, abstol=1e-8, dt0=1e-8, dtmax=np.inf, dtmin=1e-14, maxiters=10**9,
                  alg="Tsit5"):
        u = _c(u0).copy()
        o = SolverOpts(reltol, abstol, dt0, dtmax, dtmin, maxiters, 2 if self.dilatancy else (1 if self.ne else 0),
                       ALGS[alg])
        s = SolverStats()
        lib().orc_integrate(ctypes.byref(self.m), _p(u), t0, t1, ctypes.byref(o), ctypes.byref(s))
        return u, s


def dtau_dt_fft(om, v):
    """The traction rate of om.dtau_dt through the FFT variant (fastconv.c) used for timing."""
    c = FFTConv()
    if lib().orc_fftconv_init(ctypes.byref(om.m), ctypes.byref(c)) != 0:
        raise MemoryError("fftconv tables")
    v = _c(np.asarray(v).reshape(-1, order="F"))
    out = np.zeros_like(v)
    lib().orc_dtau_dt_fft(ctypes.byref(c), ctypes.byref(om.m), _p(v), _p(out))
    lib().orc_fftconv_free(ctypes.byref(c))
    return out


def integrate_many(models, u0s, t0, t1, reltol=1e-6, abstol=1e-8, dt0=1e-8, dtmax=np.inf, dtmin=1e-14,
                   maxiters=10**9, alg="Tsit5", fft=True, threads=None):
    """Independent fault-only or viscoelastic oracle models integrated in parallel, one model per
    host thread (orc_integrate_many); with fft the traction rate goes through the FFT variant.
    Returns (list of final states, list of stats)."""
    n = len(models)
    mantle = 1 if models[0].ne else 0
    us = [_c(u).copy() for u in u0s]
    ptrs = (PD * n)(*[_p(u) for u in us])
    mp = (ctypes.POINTER(Model) * n)(*[ctypes.pointer(om.m) for om in models])
    a0 = _c(np.broadcast_to(t0, (n,)))
    a1 = _c(np.broadcast_to(t1, (n,)))
    o = SolverOpts(reltol, abstol, dt0, dtmax, dtmin, maxiters, mantle, ALGS[alg])
    st = (SolverStats * n)()
    if lib().orc_integrate_many(mp, n, ptrs, _p(a0), _p(a1), ctypes.byref(o), st, int(bool(fft)),
                                int(threads or num_threads())) != 0:
        raise MemoryError("fftconv tables")
    return us, list(st)


def integrate_record(om, u0, t0, t1, stride, max_records, reltol=1e-6, abstol=1e-8, dt0=1e-8, dtmax=np.inf,
                     dtmin=1e-14, maxiters=10**9, alg="Tsit5"):
    """orc_integrate_record: returns (u(t1), stats, t_records, u_records)."""
    u = _c(u0).copy()
    o = SolverOpts(reltol, abstol, dt0, dtmax, dtmin, maxiters, 2 if om.dilatancy else (1 if om.ne else 0),
                   ALGS[alg])
    s = SolverStats()
    t_out = np.zeros(max_records)
    u_out = np.zeros(max_records * u.size)
    nrec = ctypes.c_longlong()
    lib().orc_integrate_record(ctypes.byref(om.m), _p(u), t0, t1, ctypes.byref(o), ctypes.byref(s), stride,
                               max_records, _p(t_out), _p(u_out), ctypes.byref(nrec))
    k = nrec.value
    return u, s, t_out[:k], u_out[:k * u.size].reshape(k, u.size)


def abm_coefficients(k, h, psi_prev):
    """orc_abm_coefficients: (psi[:k], beta[:k], g[:k+1]) of one VCABM step."""
    pp = np.zeros(5)
    pp[:len(psi_prev)] = psi_prev
    psi, beta, g = np.zeros(6), np.zeros(6), np.zeros(7)
    lib().orc_abm_coefficients(int(k), float(h), _p(pp), _p(psi), _p(beta), _p(g))
    return psi[:k], beta[:k], g[:k + 1]


def tsit5_tableau():
    a, e = np.zeros(42), np.zeros(7)
    lib().orc_tsit5_tableau(_p(a), _p(e))
    return a.reshape(7, 6), e


def gl_table(which):
    n = (4, 8, 12, 16)[which]
    x, w = np.zeros(n), np.zeros(n)
    lib().orc_gl_table(which, _p(x), _p(w))
    return x, w


def num_threads() -> int:
    return int(lib().orc_num_threads())
