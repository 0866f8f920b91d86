"""Seeded synthetic cycle models with the shapes of the headline workloads.

Random draws come from one splitmix64 stream (seeded) so CPU and GPU see identical inputs.
  * strike_slip_fault(): vertical strike-slip fault, 1 km cells, μ = λ = 3e10 Pa, Vs = 3044 m/s
    (η = μ/2Vs), σ = 50 MPa, b = 0.019, a = 0.015 at 2-8 km depth and 0.025 elsewhere,
    Vpl = 1e-9 m/s, initial v = Vpl and θ = Dc/Vpl (1 + 0.01 U(-1,1)).
  * strike_slip_with_mantle(): the same friction over a Maxwell mantle (η_v = 1e19 Pa s, so
    γ = 1/(2η_v), n = 0) spanning 10-30 km depth, with lognormal Dc (median 12 mm, σ_ln 0.3).
  * large_fault_with_mantle(): 256 x 16 patches at 0.5 km (4096) over 40 x 20 x 10 = 8000 cells
    (x over the fault length, y over 40 km centred, 10-30 km depth), same friction, 200 years.
  * serving_requests(): cycle-simulation requests with 500-4096 patches (10 rows, 1 km cells),
    an optional mantle of 0-4000 cells (a box under the fault, 10-30 km depth) and horizons of
    10-200 years; friction as in fault_ensemble().
  * fault_ensemble(): independent fault-only models with N ~ U[200, 2000] patches (10 rows of
    1 km cells, nx = round(N/10)); per model a - b ~ U(-0.006, 0.004) on the 2-8 km zone (a = 0.015
    there, 0.025 / b = 0.019 elsewhere), Dc lognormal (median 10 mm, σ_ln 0.3), σ ~ U(30, 80) MPa.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .mesh import BEMHex8Mesh, RectOkadaMesh, gen_hex8_box, gen_mesh
from .property import PowerLawViscosityProperty, RateStateQuasiDynamicProperty

YEAR = 365.0 * 86400.0   # the reference's year (src/vtk.jl:83)
MU = 3e10
VS = 3044.0
VPL = 1e-9


class SplitMix64:
    """splitmix64 (Steele, Lea & Flood 2014) -> uniform doubles in [0, 1)."""

    def __init__(self, seed: int):
        self.s = seed & 0xFFFFFFFFFFFFFFFF

    def next_u64(self) -> int:
        self.s = (self.s + 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF
        z = self.s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & 0xFFFFFFFFFFFFFFFF
        return z ^ (z >> 31)

    def uniform(self, n: int) -> np.ndarray:
        return np.array([(self.next_u64() >> 11) * (1.0 / 9007199254740992.0) for _ in range(n)])

    def normal(self, n: int) -> np.ndarray:
        u1, u2 = self.uniform(n), self.uniform(n)
        return np.sqrt(-2.0 * np.log1p(-u1)) * np.cos(2.0 * np.pi * u2)


@dataclass
class CycleModel:
    mf: RectOkadaMesh
    ma: BEMHex8Mesh | None
    pf: RateStateQuasiDynamicProperty
    pa: PowerLawViscosityProperty | None
    u0: np.ndarray          # flat state in ArrayPartition order
    horizon: float          # seconds
    lam: float = MU
    mu: float = MU
    name: str = ""

    @property
    def N(self) -> int:
        return self.mf.nx * self.mf.nξ

    @property
    def ne(self) -> int:
        return 0 if self.ma is None else self.ma.ne


def _friction(mf: RectOkadaMesh, rng: SplitMix64, dc_sigma_ln: float | None, dc_median: float = 0.012):
    depth = -np.tile(mf.z, (mf.nx, 1))
    a = np.where((depth >= 2e3) & (depth <= 8e3), 0.015, 0.025)
    b = np.full_like(a, 0.019)
    if dc_sigma_ln is None:
        L = np.full_like(a, dc_median)
    else:
        L = dc_median * np.exp(dc_sigma_ln * rng.normal(a.size)).reshape(a.shape, order="F")
    sig = np.full_like(a, 5e7)
    return RateStateQuasiDynamicProperty(a, b, L, sig, MU / (2 * VS), VPL, 0.6, 1e-6)


def strike_slip_fault(length=80e3, depth=10e3, cell=1e3, years=50.0, seed=1) -> CycleModel:
    mf = gen_mesh("RectOkada", length, depth, cell, cell, 90.0)
    rng = SplitMix64(seed)
    pf = _friction(mf, rng, None)
    N = mf.nx * mf.nξ
    th0 = pf.L.reshape(-1, order="F") / VPL * (1 + 0.01 * (2 * rng.uniform(N) - 1))
    u0 = np.concatenate([np.full(N, VPL), th0, np.zeros(N)])
    return CycleModel(mf, None, pf, None, u0, years * YEAR, name=f"fault {mf.nx}x{mf.nξ}")


def strike_slip_with_mantle(length=100e3, depth=10e3, cell=1e3, mantle_cells=(50, 10, 5), mantle_y=20e3,
                            mantle_top=-10e3, mantle_bottom=-30e3, eta_v=1e19, years=100.0, seed=1) -> CycleModel:
    mf = gen_mesh("RectOkada", length, depth, cell, cell, 90.0)
    nxm, nym, nzm = mantle_cells
    ma = gen_hex8_box(-length / 2, -mantle_y / 2, mantle_top, length, mantle_y, mantle_bottom - mantle_top, nxm, nym, nzm)
    rng = SplitMix64(seed)
    pf = _friction(mf, rng, 0.3)
    pa = PowerLawViscosityProperty(np.full(ma.ne, 1.0 / (2.0 * eta_v)), np.zeros(ma.ne), np.zeros(6))
    N, E = mf.nx * mf.nξ, 6 * ma.ne
    th0 = pf.L.reshape(-1, order="F") / VPL * (1 + 0.01 * (2 * rng.uniform(N) - 1))
    u0 = np.concatenate([np.full(N, VPL), th0, np.zeros(E), np.zeros(E), np.zeros(N)])
    return CycleModel(mf, ma, pf, pa, u0, years * YEAR, name=f"fault {mf.nx}x{mf.nξ} + mantle {ma.ne}")


def large_fault_with_mantle(years=200.0, seed=1) -> CycleModel:
    return strike_slip_with_mantle(length=128e3, depth=8e3, cell=0.5e3, mantle_cells=(40, 20, 10), mantle_y=40e3,
                                   mantle_top=-10e3, mantle_bottom=-30e3, years=years, seed=seed)


def fault_ensemble(n_models=256, years=50.0, seed=3, n_range=(200, 2000), nxi=10) -> list[CycleModel]:
    rng = SplitMix64(seed)
    out = []
    for m in range(n_models):
        N = n_range[0] + (n_range[1] - n_range[0]) * rng.uniform(1)[0]
        nx = max(2, int(round(N / nxi)))
        mf = gen_mesh("RectOkada", nx * 1e3, nxi * 1e3, 1e3, 1e3, 90.0)
        amb = -0.006 + 0.010 * rng.uniform(1)[0]
        sigma = 30e6 + 50e6 * rng.uniform(1)[0]
        depth = -np.tile(mf.z, (mf.nx, 1))
        vw = (depth >= 2e3) & (depth <= 8e3)
        a = np.where(vw, 0.015, 0.025)
        b = np.where(vw, 0.015 - amb, 0.019)
        L = 0.010 * np.exp(0.3 * rng.normal(mf.nx * mf.nξ)).reshape((mf.nx, mf.nξ), order="F")
        pf = RateStateQuasiDynamicProperty(a, b, L, np.full_like(a, sigma), MU / (2 * VS), VPL, 0.6, 1e-6)
        Nn = mf.nx * mf.nξ
        th0 = pf.L.reshape(-1, order="F") / VPL * (1 + 0.01 * (2 * rng.uniform(Nn) - 1))
        u0 = np.concatenate([np.full(Nn, VPL), th0, np.zeros(Nn)])
        out.append(CycleModel(mf, None, pf, None, u0, years * YEAR, name=f"ensemble member {m} ({mf.nx}x{mf.nξ})"))
    return out


def serving_requests(n_requests=32, seed=5, mantle_fraction=0.25, patch_range=(500, 4096), cell_range=(0, 4000),
                     year_range=(10.0, 200.0), geometries=None) -> list[CycleModel]:
    """With geometries = G, every request takes one of G seeded (patch count, mantle size) shapes,
    so requests repeat meshes (the case the server's Green's-function cache serves) while each
    draws its own friction, initial state and horizon."""
    rng = SplitMix64(seed)
    pool = None
    if geometries:
        pool = [(patch_range[0] + (patch_range[1] - patch_range[0]) * rng.uniform(1)[0],
                 rng.uniform(1)[0] < mantle_fraction,
                 max(1, int(cell_range[0] + (cell_range[1] - cell_range[0]) * rng.uniform(1)[0])))
                for _ in range(int(geometries))]
    out = []
    for r in range(n_requests):
        if pool is not None:
            N, with_mantle, ne_pick = pool[int(rng.uniform(1)[0] * len(pool)) % len(pool)]
        else:
            N = patch_range[0] + (patch_range[1] - patch_range[0]) * rng.uniform(1)[0]
        years = year_range[0] + (year_range[1] - year_range[0]) * rng.uniform(1)[0]
        member = fault_ensemble(n_models=1, years=years, seed=int(rng.next_u64() % 1000003), n_range=(N, N))[0]
        if (with_mantle if pool is not None else rng.uniform(1)[0] < mantle_fraction):
            ne_target = ne_pick if pool is not None else \
                max(1, int(cell_range[0] + (cell_range[1] - cell_range[0]) * rng.uniform(1)[0]))
            nz = 4
            nxy = max(1, int(round((ne_target / nz) ** 0.5)))
            L = member.mf.nx * 1e3
            ma = gen_hex8_box(-L / 2, -L / 4, -10e3, L, L / 2, -20e3, nxy, nxy, nz)
            pa = PowerLawViscosityProperty(np.full(ma.ne, 1.0 / (2.0 * 1e19)), np.zeros(ma.ne), np.zeros(6))
            Nn = member.N
            u0 = np.concatenate([member.u0[:2 * Nn], np.zeros(12 * ma.ne), member.u0[2 * Nn:]])
            member = CycleModel(member.mf, ma, member.pf, pa, u0, member.horizon, name=f"request {r} (+mantle {ma.ne})")
        else:
            member.name = f"request {r}"
        out.append(member)
    return out
