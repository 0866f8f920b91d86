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


# ---- save_property / load_property (property.jl:70-107) ---------------------------------------
# Files hold one array per field under the reference's field names; BSON is not available here,
# so the container is numpy's .npz (written through an open handle: the name is kept as given).
_FIELDS = {  # reference field name -> attribute of this mirror (identifiers are NFKC-normalised)
    "RateStateQuasiDynamicProperty": ["a", "b", "L", "σ", "η", "vpl", "f₀", "v₀"],
    "PowerLawViscosityProperty": ["γ", "n", "dϵ₀"],
    "DilatancyProperty": ["tₚ", "ϵ", "β", "p₀"],
}
_ATTR = {"f₀": "f0", "v₀": "v0", "dϵ₀": "dϵ0", "tₚ": "tp", "p₀": "p0"}


def _attr(name: str) -> str:
    import unicodedata
    return unicodedata.normalize("NFKC", _ATTR.get(name, name))


def struct_to_dict(p) -> dict:
    """Field name -> value with the reference's names (property.jl:70-76)."""
    if isinstance(p, CompositePowerLawViscosityProperty):
        d = {"dϵ₀": np.asarray(p.dϵ0)}
        for k, q in enumerate(p.piter):
            for name, v in struct_to_dict(q).items():
                d[f"piter/{k}/{name}"] = v
        d["piter"] = np.asarray(len(p.piter))
        return d
    names = _FIELDS[type(p).__name__]
    return {name: np.asarray(getattr(p, _attr(name))) for name in names}


def save_property(file: str, *ps) -> None:
    """save_property(file, p...) (property.jl:78-85): the fields of every property, merged."""
    d = {}
    for p in ps:
        d.update(struct_to_dict(p))
    with open(file, "wb") as f:
        np.savez(f, **d)


def _from_dict(d: dict, name: str):
    def get(k):
        v = np.asarray(d[k])
        return float(v) if v.ndim == 0 else v.copy()
    if name == "RateStateQuasiDynamicProperty":
        return RateStateQuasiDynamicProperty(*[get(k) for k in _FIELDS[name]])
    if name == "PowerLawViscosityProperty":
        return PowerLawViscosityProperty(*[get(k) for k in _FIELDS[name]])
    if name == "DilatancyProperty":
        return DilatancyProperty(*[get(k) for k in _FIELDS[name]])
    if name == "CompositePowerLawViscosityProperty":
        piter = []
        for k in range(int(np.asarray(d["piter"]))):
            sub = {n: d[f"piter/{k}/{n}"] for n in _FIELDS["PowerLawViscosityProperty"]}
            piter.append(_from_dict(sub, "PowerLawViscosityProperty"))
        return CompositePowerLawViscosityProperty(piter, get("dϵ₀"))
    raise ValueError(f"unknown property type {name}")


def load_property(file_or_dict, name: str):
    """load_property(file, :Type) (property.jl:87-107): rebuild a property from its fields."""
    if isinstance(file_or_dict, dict):
        return _from_dict(file_or_dict, name)
    with np.load(file_or_dict) as z:
        return _from_dict({k: z[k] for k in z.files}, name)
