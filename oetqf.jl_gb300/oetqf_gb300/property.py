"""Fault and mantle properties, mirroring src/BEM/property.jl of Oetqf.jl."""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class RateStateQuasiDynamicProperty:
    """Regularized rate-and-state friction with radiation damping (property.jl:10-25)."""

    a: np.ndarray
    b: np.ndarray
    L: np.ndarray
    σ: np.ndarray
    η: float
    vpl: float
    f0: float = 0.6
    v0: float = 1e-6

    def __post_init__(self):
        self.a, self.b, self.L, self.σ = (np.asarray(v, dtype=np.float64) for v in (self.a, self.b, self.L, self.σ))
        assert self.a.shape == self.b.shape == self.L.shape == self.σ.shape
        assert self.f0 > 0
        assert self.v0 > 0
        assert self.η > 0
        assert self.vpl > 0


@dataclass
class PowerLawViscosityProperty:
    """dϵ/dt = γ σ' τⁿ with ``n`` = power - 1 (property.jl:34-41, equation.jl:285)."""

    γ: np.ndarray
    n: np.ndarray
    dϵ0: np.ndarray = field(default_factory=lambda: np.zeros(6))

    def __post_init__(self):
        self.γ = np.asarray(self.γ, dtype=np.float64)
        self.n = np.asarray(self.n, dtype=np.float64)
        self.dϵ0 = np.asarray(self.dϵ0, dtype=np.float64)
        assert len(self.dϵ0) == 6
        assert len(self.γ) == len(self.n)


def dϵ_dt(p: PowerLawViscosityProperty, i: int, σ: float, τ: float) -> float:
    """The viscosity law of src/BEM/equation.jl:285."""
    return p.γ[i] * σ * τ ** p.n[i]


@dataclass
class CompositePowerLawViscosityProperty:
    """A sum of power laws (property.jl:43-48): dϵ/dt = Σ_k γ_k σ' τ^{n_k} (equation.jl:286-292)."""

    piter: list
    dϵ0: np.ndarray = field(default_factory=lambda: np.zeros(6))

    def __post_init__(self):
        self.dϵ0 = np.asarray(self.dϵ0, dtype=np.float64)
        assert len(self.dϵ0) == 6


@dataclass
class DilatancyProperty:
    """Pore-pressure dilatancy (property.jl:27-32): tₚ diffusion time, ϵ dilatancy coefficient,
    β gouge compressibility, p₀ ambient pore pressure (each (nx, nξ))."""

    tp: np.ndarray
    ϵ: np.ndarray
    β: np.ndarray
    p0: np.ndarray

    def __post_init__(self):
        self.tp, self.ϵ, self.β, self.p0 = (np.asarray(v, dtype=np.float64) for v in (self.tp, self.ϵ, self.β, self.p0))
        assert self.tp.shape == self.ϵ.shape == self.β.shape == self.p0.shape


def dϵ_dt_composite(p: CompositePowerLawViscosityProperty, i: int, σ: float, τ: float) -> float:
    """equation.jl:286-292."""
    return sum(q.γ[i] * σ * τ ** q.n[i] for q in p.piter)
