"""Serving: continuous batching of cycle-simulation requests on one GPU (libgbcycle gbc_server_*).

``Server`` admits requests by HBM budget; fault-only requests share a persistent batch and
mantle requests run on their own streams, all with state kept on the device. ``run_stream``
replays a Poisson arrival process and reports per-request latency percentiles and the aggregate
simulated years per second.
"""
from __future__ import annotations

import ctypes
import threading
import time

import numpy as np

from . import _capi as C
from .mesh import gauss1_quadrature

PD = C.PD


class Request(ctypes.Structure):
    _fields_ = [("mf", ctypes.POINTER(C.FaultMesh)), ("ma", ctypes.POINTER(C.HexMesh)), ("lambda_", C.D), ("mu", C.D),
                ("ftype", C.I), ("nrept", C.I), ("buffer_ratio", C.D), ("a", PD), ("b", PD), ("L", PD), ("sigma", PD),
                ("eta", C.D), ("vpl", C.D), ("f0", C.D), ("v0", C.D), ("gamma", PD), ("n", PD), ("deps0", PD),
                ("qcoords", PD), ("qweights", PD), ("nq", C.I), ("u0", PD), ("t0", C.D), ("t1", C.D),
                ("precision", C.I), ("ne_opts_valid", C.I), ("opts", C.SolverOpts)]


class RequestResult(ctypes.Structure):
    _fields_ = [("id", ctypes.c_longlong), ("status", C.I), ("submit_s", C.D), ("admit_s", C.D), ("done_s", C.D),
                ("stats", C.SolverStats)]


class ServerInfo(ctypes.Structure):
    _fields_ = [("queued", C.I), ("batched", C.I), ("mantle", C.I), ("bytes_in_use", C.D), ("peak_bytes", C.D),
                ("iterations", ctypes.c_longlong), ("cache_entries", C.I), ("cache_bytes", C.D),
                ("cache_hits", ctypes.c_longlong), ("cache_misses", ctypes.c_longlong)]


def _sigs():
    L = C.lib()
    P = ctypes.c_void_p
    L.gbc_server_create.argtypes = [C.D, ctypes.POINTER(C.SolverOpts), ctypes.POINTER(P)]
    L.gbc_server_create.restype = C.I
    L.gbc_server_submit.argtypes = [P, ctypes.POINTER(Request), ctypes.POINTER(ctypes.c_longlong)]
    L.gbc_server_submit.restype = C.I
    L.gbc_server_wait.argtypes = [P, ctypes.c_longlong, PD, ctypes.POINTER(RequestResult)]
    L.gbc_server_wait.restype = C.I
    L.gbc_server_query.argtypes = [P, ctypes.POINTER(ServerInfo)]
    L.gbc_server_query.restype = C.I
    L.gbc_server_set_gf_cache.argtypes = [P, C.I]
    L.gbc_server_set_gf_cache.restype = C.I
    L.gbc_server_destroy.argtypes = [P]
    L.gbc_server_destroy.restype = None
    return L


class Server:
    def __init__(self, hbm_budget_gb=64.0, reltol=1e-6, abstol=1e-8, dt=1e-8, dtmax=1e300, maxiters=10**9,
                 alg="Tsit5"):
        L = _sigs()
        self.opts = C.SolverOpts(reltol, abstol, dt, dtmax, 1e-14, maxiters, C.ALGS[alg])
        h = ctypes.c_void_p()
        C.check(L.gbc_server_create(hbm_budget_gb * 2**30, ctypes.byref(self.opts), ctypes.byref(h)))
        self.h = h
        self._keep = {}
        self._sizes = {}
        self._lock = threading.Lock()

    def submit(self, cm, precision=C.GBC_PREC_BF16, quad=None, t0=0.0, t1=None) -> int:
        """Submit a workloads.CycleModel; returns the request id."""
        k = C.Keep()
        fs = C.fault_struct(cm.mf, k)
        f = lambda a: k(np.asarray(a, dtype=np.float64).reshape(-1, order="F"))
        r = Request()
        r.mf = ctypes.pointer(fs)
        r.lambda_, r.mu, r.ftype, r.nrept, r.buffer_ratio = cm.lam, cm.mu, 0, 2, 0.0
        p = cm.pf
        r.a, r.b, r.L, r.sigma = f(p.a), f(p.b), f(p.L), f(p.σ)
        r.eta, r.vpl, r.f0, r.v0 = p.η, p.vpl, p.f0, p.v0
        if cm.ma is not None:
            hs = C.hex_struct(cm.ma, k)
            r.ma = ctypes.pointer(hs)
            r.gamma, r.n, r.deps0 = f(cm.pa.γ), f(cm.pa.n), f(cm.pa.dϵ0)
            qc, qw = quad if quad is not None else gauss1_quadrature()
            r.qcoords, r.qweights, r.nq = f(qc), f(qw), len(qw)
        r.u0 = f(cm.u0)
        r.t0 = t0
        r.t1 = cm.horizon if t1 is None else t1
        r.precision = precision
        r.ne_opts_valid = 1
        r.opts = self.opts
        rid = ctypes.c_longlong()
        C.check(C.lib().gbc_server_submit(self.h, ctypes.byref(r), ctypes.byref(rid)))
        with self._lock:
            self._sizes[rid.value] = cm.u0.size
        return rid.value

    def wait(self, rid):
        with self._lock:
            n = self._sizes.pop(rid)
        u = np.zeros(n)
        res = RequestResult()
        rc = C.lib().gbc_server_wait(self.h, rid, C.ptr(u), ctypes.byref(res))
        if rc < 0 and rc != -5:
            C.check(rc)
        return u, res

    def set_gf_cache(self, enabled: bool):
        """Keep assembled Green's functions on the device across requests (default on)."""
        C.check(C.lib().gbc_server_set_gf_cache(self.h, int(bool(enabled))))

    def info(self) -> ServerInfo:
        i = ServerInfo()
        C.check(C.lib().gbc_server_query(self.h, ctypes.byref(i)))
        return i

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            C.lib().gbc_server_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def run_stream(server: Server, requests, rate_per_s: float, seed: int = 0, precision=C.GBC_PREC_BF16):
    """Submit requests at Poisson arrival times (rate per second), wait for all; returns a dict
    with per-request latencies (s), p50/p99, aggregate sim-yr/s and the makespan."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate_per_s, len(requests))
    ids = [None] * len(requests)
    t_start = time.perf_counter()

    def submitter():
        t = t_start
        for i, cm in enumerate(requests):
            t += gaps[i]
            dt = t - time.perf_counter()
            if dt > 0:
                time.sleep(dt)
            ids[i] = server.submit(cm, precision=precision)

    th = threading.Thread(target=submitter)
    th.start()
    th.join()
    results = [server.wait(rid) for rid in ids]
    makespan = time.perf_counter() - t_start
    lat = np.array([r.done_s - r.submit_s for _, r in results])
    years = sum(cm.horizon for cm in requests) / (365.0 * 86400.0)
    return {"latency_s": lat, "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "sim_yr_per_s": years / makespan, "makespan_s": makespan, "results": results,
            "status": sorted({r.status for _, r in results})}
