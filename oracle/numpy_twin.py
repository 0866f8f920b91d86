"""Numpy/scipy twin of the reference's CPU right-hand side.

TEST INFRASTRUCTURE ONLY: the second timed CPU baseline beside the C/OpenMP oracle. Only tests/ and
bench.py's CPU-baseline leg import this module; the product never does.

Where the C oracle restates the reference's loops, this twin keeps the reference's LIBRARY structure,
which is what its CPU time is made of (src/BEM/equation.jl):
  * relative_velocity! (:35-42) into a (2nx - 1, nξ) zero-padded buffer;
  * dτ_dt! (:44-61): real FFT along strike of the padded slip rates (FFTW's plan_rfft there,
    scipy.fft with all host threads here), the complex multiply-accumulate over source depth rows
    with the fourier-form kernel gf[i, j, l], the inverse real FFT, the first nx rows;
  * update_strain_rate! / relative_strain_rate! (:207-230) and the power laws (:285-292), vectorised;
  * the three matvecmul! GEMVs in the reference's order (:201-203) through numpy's BLAS;
  * update_fault! with the ageing law (:233-246, :279), vectorised.
The state is the flat ArrayPartition (v, θ, δ) or (v, θ, ϵ, σ, δ), column-major parts.
"""
from __future__ import annotations

import numpy as np
import scipy.fft as sfft


class NumpyTwin:
    """ode(du, u, p, t) of the reference (equation.jl:156-166 fault-only, :185-205 viscoelastic)."""

    def __init__(self, gf11, pf, gf12=None, gf21=None, gf22=None, pa=None, workers: int = -1):
        g = np.asarray(gf11)
        if not np.iscomplexobj(g):
            raise ValueError("gf11 must be the reference's fourier form (complex (nx, nξ, nξ))")
        self.nx, self.nxi = g.shape[0], g.shape[1]
        self.gf11 = np.ascontiguousarray(g)
        self.N = self.nx * self.nxi
        f = lambda a: np.asarray(a, dtype=np.float64).reshape(-1, order="F")
        self.a, self.b, self.L, self.sig = f(pf.a), f(pf.b), f(pf.L), f(pf.σ)
        self.eta, self.vpl, self.f0, self.v0 = float(pf.η), float(pf.vpl), float(pf.f0), float(pf.v0)
        self.workers = workers
        self.ne = 0
        if gf12 is not None:
            # row-major copies whatever layout arrives (the reference's arrays are column-major):
            # numpy's BLAS applies a row-major matrix 1.5x faster on the GB300 host's cores (10.0
            # against 14.8 ms per RHS of the 1000 + 2500 model), and timing both callers with one
            # layout keeps their samples comparable
            self.G12, self.G21, self.G22 = (np.ascontiguousarray(x, dtype=np.float64) for x in (gf12, gf21, gf22))
            self.ne = self.G12.shape[0] // 6
            laws = pa.piter if hasattr(pa, "piter") else [pa]
            self.gamma = [np.asarray(q.γ, dtype=np.float64) for q in laws]
            self.nexp = [np.asarray(q.n, dtype=np.float64) for q in laws]
            self.deps0 = np.asarray(pa.dϵ0, dtype=np.float64)
        self.pad = np.zeros((2 * self.nx - 1, self.nxi))

    def dtau_dt(self, relv: np.ndarray) -> np.ndarray:
        """dτ_dt! (equation.jl:44-61) for relative slip rates relv (nx, nξ); returns (nx, nξ)."""
        self.pad[: self.nx] = relv
        rdft = sfft.rfft(self.pad, axis=0, workers=self.workers)          # (nx, nξ)
        ddft = np.matmul(self.gf11, rdft[:, :, None])[:, :, 0]          # Σ_l gf[i,j,l] relv_dft[i,l]
        return sfft.irfft(ddft, n=2 * self.nx - 1, axis=0, workers=self.workers)[: self.nx]

    def ode(self, u: np.ndarray) -> np.ndarray:
        N, ne = self.N, self.ne
        M = 6 * ne
        u = np.asarray(u, dtype=np.float64)
        v, th = u[:N], u[N:2 * N]
        relvnp = v - self.vpl
        dtau = self.dtau_dt(relvnp.reshape((self.nx, self.nxi), order="F")).reshape(-1, order="F")
        parts = []
        if ne:
            s = u[2 * N + M:2 * N + 2 * M].reshape((ne, 6), order="F")
            skk = (s[:, 0] + s[:, 3] + s[:, 5]) / 3.0
            dev = np.stack([s[:, 0] - skk, s[:, 1], s[:, 2], s[:, 3] - skk, s[:, 4], s[:, 5] - skk], axis=1)
            tau = np.sqrt(dev[:, 0] ** 2 + dev[:, 3] ** 2 + dev[:, 5] ** 2 + 2 * (dev[:, 1] ** 2 + dev[:, 2] ** 2 + dev[:, 4] ** 2))
            fac = sum(g * tau ** n for g, n in zip(self.gamma, self.nexp))
            deps = (fac[:, None] * dev).reshape(-1, order="F")
            reldeps = (fac[:, None] * dev - self.deps0[None, :]).reshape(-1, order="F")
            dtau += self.G21 @ reldeps
            dsig = self.G12 @ relvnp
            dsig += self.G22 @ reldeps
            parts = [deps, dsig]
        psi1 = np.exp((self.f0 + self.b * np.log(self.v0 * np.maximum(0.0, th) / self.L)) / self.a) / (2 * self.v0)
        psi2 = self.sig * psi1 / np.hypot(1.0, v * psi1)
        dmu_dv = self.a * psi2
        dmu_dth = self.b / th * v * psi2
        dth = 1.0 - v * th / self.L
        dv = (dtau - dmu_dth * dth) / (dmu_dv + self.eta)
        return np.concatenate([dv, dth, *parts, v.copy()])
