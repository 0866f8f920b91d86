"""Fault and mantle meshes, mirroring src/BEM/mesh.jl of Oetqf.jl.

``gen_mesh("RectOkada", ...)`` restates ``gen_mesh(Val(:RectOkada), x, ξ, Δx, Δξ, dip)``
(src/BEM/mesh.jl:39-56). The reference builds its hexahedral mantle mesh with gmsh
(``gen_gmsh_mesh`` + ``gen_mesh(Val(:BEMHex8Mesh), file)``, mesh.jl:95-187); gmsh is not part of
this project, so ``gen_hex8_box`` produces the same ``BEMHex8Mesh`` fields for the transfinite,
vertically extruded box that ``gen_gmsh_mesh`` describes (uniform in x and y, optional layer
heights ``rfzh`` in z). Elements are ordered x fastest, then y, then z (top layer first).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


def _count(length: float, step: float) -> int:
    r = length / step
    n = int(round(r))
    if abs(r - n) > 1e-9 * max(1.0, abs(r)):
        n = int(np.floor(r + 1e-12))
    return n


@dataclass
class RectOkadaMesh:
    """Uniform strike x down-dip grid of rectangular Okada cells (mesh.jl:5-21)."""

    x: np.ndarray       # centroids along strike (nx)
    Δx: float
    nx: int
    ax: np.ndarray      # (nx, 2) cell edges along strike
    ξ: np.ndarray       # centroids along down-dip (nξ), negative
    Δξ: float
    nξ: int
    aξ: np.ndarray      # (nξ, 2) cell edges along dip
    y: np.ndarray
    z: np.ndarray
    dep: float
    dip: float

    def __post_init__(self):
        assert len(self.x) == len(self.ax) == self.nx
        assert len(self.ξ) == len(self.aξ) == self.nξ == len(self.y) == len(self.z)

    @property
    def n(self) -> int:
        return self.nx * self.nξ


def sincosd(deg: float) -> tuple[float, float]:
    """sin and cos of an angle in degrees, exact at multiples of 90 (Julia's sind/cosd)."""
    r = float(np.fmod(deg, 360.0))
    if r < 0:
        r += 360.0
    k = int(np.floor(r / 90.0 + 0.5))
    t = np.deg2rad(r - 90.0 * k)
    st, ct = (0.0, 1.0) if t == 0.0 else (float(np.sin(t)), float(np.cos(t)))
    return [(st, ct), (ct, -st), (-st, -ct), (-ct, st)][k & 3]


def gen_mesh(kind: str, x: float, ξ: float, Δx: float, Δξ: float, dip: float) -> RectOkadaMesh:
    """``gen_mesh(Val(:RectOkada), x, ξ, Δx, Δξ, dip)`` (src/BEM/mesh.jl:39-56)."""
    if kind != "RectOkada":
        raise ValueError(f"unknown mesh kind {kind!r}; hex meshes come from gen_hex8_box")
    x, ξ, Δx, Δξ, dip = map(float, (x, ξ, Δx, Δξ, dip))
    nξ = _count(ξ - Δξ, Δξ) + 1
    ξi = -Δξ * np.arange(nξ) - Δξ / 2
    aξ = np.stack([ξi - Δξ / 2, ξi + Δξ / 2], axis=1)
    s, c = sincosd(dip)
    y, z = ξi * c, ξi * s
    nx = _count(x - Δx, Δx) + 1
    xi = -x / 2 + Δx / 2 + Δx * np.arange(nx)
    ax = np.stack([xi - Δx / 2, xi + Δx / 2], axis=1)
    return RectOkadaMesh(xi, Δx, nx, ax, ξi, Δξ, nξ, aξ, y, z, 0.0, dip)


@dataclass
class BEMHex8Mesh:
    """Hexahedral strain volumes (mesh.jl:58-72): centroids c*, source anchors q*, sizes Δ*."""

    cx: np.ndarray
    cy: np.ndarray
    cz: np.ndarray
    qx: np.ndarray
    qy: np.ndarray
    qz: np.ndarray
    Δx: np.ndarray
    Δy: np.ndarray
    Δz: np.ndarray
    θ: float = 0.0

    def __post_init__(self):
        shapes = {a.shape for a in (self.cx, self.cy, self.cz, self.qx, self.qy, self.qz,
                                    self.Δx, self.Δy, self.Δz)}
        assert len(shapes) == 1

    @property
    def ne(self) -> int:
        return int(self.cx.shape[0])


def gen_hex8_box(llx: float, lly: float, llz: float, dx: float, dy: float, dz: float,
                 nx: int, ny: int, nz: int, rfzh=None) -> BEMHex8Mesh:
    """Box [llx, llx+dx] x [lly, lly+dy] x (llz .. llz+dz) of nx*ny*nz hex cells.

    Same arguments as ``gen_gmsh_mesh(Val(:BEMHex8Mesh), ...)`` (mesh.jl:95-133) for a uniform
    transfinite x-y grid; ``dz`` is negative to extrude downward from the top face at ``llz``;
    ``rfzh`` are the (accumulated, normalised) layer heights. Fields follow the loader at
    mesh.jl:166-185: q = (cx, cy - Δy/2, cz + Δz/2).
    """
    if min(nx, ny, nz) < 1:
        raise ValueError("cell counts must be positive")
    xe = llx + dx * np.arange(nx + 1) / nx
    ye = lly + dy * np.arange(ny + 1) / ny
    h = np.ones(nz) if rfzh is None else np.asarray(rfzh, dtype=float)
    if h.shape != (nz,) or np.any(h <= 0):
        raise ValueError("rfzh must hold nz positive layer heights")
    cum = np.concatenate([[0.0], np.cumsum(h) / np.sum(h)])
    ze = llz + dz * cum
    X0, Y0, Z0 = np.meshgrid(xe[:-1], ye[:-1], ze[:-1], indexing="ij")
    X1, Y1, Z1 = np.meshgrid(xe[1:], ye[1:], ze[1:], indexing="ij")

    def flat(a):  # x fastest, then y, then z
        return np.ascontiguousarray(a.transpose(2, 1, 0).reshape(-1))

    cx, cy, cz = flat((X0 + X1) / 2), flat((Y0 + Y1) / 2), flat((Z0 + Z1) / 2)
    Dx, Dy, Dz = flat(np.abs(X1 - X0)), flat(np.abs(Y1 - Y0)), flat(np.abs(Z1 - Z0))
    return BEMHex8Mesh(cx, cy, cz, cx.copy(), cy - Dy / 2, cz + Dz / 2, Dx, Dy, Dz, 0.0)


def gauss1_quadrature():
    """The "Gauss1" hex rule after get_quadrature's normalisation (src/BEM/GF.jl:318-323)."""
    return np.zeros(3), np.ones(1)


def gauss_product_quadrature(order: int):
    """Tensor-product Gauss-Legendre hex rule, weights normalised to sum 1 (explicit
    ``(coords, weights)`` tuples are accepted by the reference at src/BEM/GF.jl:325-328)."""
    t, w = np.polynomial.legendre.leggauss(order)
    pts, wts = [], []
    for k in range(order):
        for j in range(order):
            for i in range(order):
                pts += [t[i], t[j], t[k]]
                wts.append(w[i] * w[j] * w[k])
    wts = np.asarray(wts)
    return np.asarray(pts), wts / wts.sum()


def gmsh_quadrature(etype: int, qtype: str):
    """gmsh_quadrature(etype, qtype) (src/BEM/GF.jl:300-316) for the hexahedron (Gmsh element type 5):
    the tensor-product Gauss-Legendre rule that integrates polynomials of the order named by
    "GaussN" exactly (ceil((N+1)/2) points per direction, as Gmsh builds it since 4.9), local
    coordinates on [-1, 1]^3 flattened (x, y, z) per point, weights summing to the element volume 8.
    Gmsh itself is not needed: only this element is on the path."""
    if etype != 5:
        raise NotImplementedError("only the 8-node hexahedron (Gmsh element type 5) is on this path")
    if not (isinstance(qtype, str) and qtype.startswith("Gauss") and qtype[5:].isdigit()):
        raise ValueError(f"unknown quadrature {qtype!r} (expected 'GaussN')")
    order = int(qtype[5:])
    n = max(1, (order + 2) // 2)
    coords, w = gauss_product_quadrature(n)
    return coords, w * 8.0


def get_quadrature(qtype):
    """get_quadrature (src/BEM/GF.jl:318-328): a "GaussN" name gives the hexahedron rule with
    weights normalised to sum 1; an explicit (coords, weights) tuple is checked and passed on."""
    if isinstance(qtype, str):
        c, w = gmsh_quadrature(5, qtype)
        return c, w / w.sum()
    coords, weights = qtype
    assert len(np.ravel(coords)) == 3 * len(np.ravel(weights)), "Wrong format of quadrature!"
    return qtype
