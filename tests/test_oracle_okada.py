"""Oracle dc3d (Okada 1992) pinned against known answers and physical identities.

The reference's dc3d lives in GeoGreensFunctions.jl (not vendored, no golden vectors), called at
src/BEM/GF.jl:49-53 and :156-160. These tests pin the C restatement by
  * 40-digit known answers (tests/golden/okada_golden.json, made by make_golden.py),
  * an independent formula set: Okada (1985) surface displacement,
  * an independent solution: Volterra's surface integral of Kelvin's full-space point-force solution
    (the deep limit of a finite rectangle),
  * equilibrium, the traction-free surface, the slip jump, far-field decay.
"""
import json
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden", "okada_golden.json")


def _stress(u, lam, mu):
    G = np.array([[u[3 + 3 * j + i] for j in range(3)] for i in range(3)])
    return lam * np.trace(G) * np.eye(3) + mu * (G + G.T)


def test_golden_okada92(oracle):
    g = json.load(open(GOLD))
    for p in g["dc3d_okada92"]:
        u, rc = oracle.dc3d(*p["args"])
        ref = np.asarray(p["u"])
        assert rc == 0
        np.testing.assert_allclose(u, ref, rtol=0, atol=1e-12 * np.abs(ref).max())


def test_golden_okada85_surface(oracle):
    g = json.load(open(GOLD))
    for p in g["surface_okada85"]:
        u, rc = oracle.dc3d(*p["args"])
        ref = np.asarray(p["u"])
        np.testing.assert_allclose(u[:3], ref, rtol=0, atol=1e-12 * np.abs(ref).max())


@pytest.mark.parametrize("dip", [90.0, 60.0, 41.0, 15.0])
@pytest.mark.parametrize("slip", [0, 1, 2])
def test_traction_free_surface(oracle, dip, slip):
    lam = mu = 1.0
    alpha = (lam + mu) / (lam + 2 * mu)
    rng = np.random.default_rng(7)
    disl = [0.0, 0.0, 0.0]
    disl[slip] = 1.0
    for _ in range(8):
        x, y = rng.uniform(-4, 4, 2)
        u, _ = oracle.dc3d(x, y, 0.0, alpha, 1.5, dip, -1, 2, -1.5, 0.3, *disl)
        s = _stress(u, lam, mu)
        assert np.abs(s[:, 2]).max() <= 1e-12 * np.abs(s).max()


@pytest.mark.parametrize("dip", [90.0, 33.0])
@pytest.mark.parametrize("slip", [0, 1, 2])
def test_equilibrium(oracle, dip, slip):
    """mu lap u + (lam + mu) grad div u = 0, from central differences of the exact gradient."""
    lam, mu = 2.0, 1.0
    alpha = (lam + mu) / (lam + 2 * mu)
    disl = [0.0, 0.0, 0.0]
    disl[slip] = 1.0
    rng = np.random.default_rng(11)
    h = 1e-4
    for _ in range(6):
        r = np.array([rng.uniform(-3, 3), rng.uniform(-3, 3), rng.uniform(-4, -0.3)])
        H = np.zeros((3, 3, 3))  # H[i, j, k] = d2 u_i / dx_j dx_k
        for k in range(3):
            e = np.zeros(3)
            e[k] = h
            up, _ = oracle.dc3d(*(r + e), alpha, 1.0, dip, -1, 2, -2, 0.3, *disl)
            um, _ = oracle.dc3d(*(r - e), alpha, 1.0, dip, -1, 2, -2, 0.3, *disl)
            for i in range(3):
                for j in range(3):
                    H[i, j, k] = (up[3 + 3 * j + i] - um[3 + 3 * j + i]) / (2 * h)
        res = mu * np.einsum("ijj->i", H) + (lam + mu) * np.einsum("jji->i", H)
        assert np.abs(res).max() <= 1e-6 * np.abs(H).max()


@pytest.mark.parametrize("dip", [90.0, 60.0, 20.0])
def test_slip_jump(oracle, dip):
    """u(+n) - u(-n) = U1 s + U2 d + U3 n across the fault, n = (0, -sin dip, cos dip)."""
    alpha = 2.0 / 3.0
    sd, cd = np.sin(np.deg2rad(dip)), np.cos(np.deg2rad(dip))
    n = np.array([0, -sd, cd])
    dvec = np.array([0, cd, sd])
    et0, xi0, c = -0.8, 0.4, 2.0
    p = np.array([xi0, et0 * cd, -c + et0 * sd])
    for disl in ([1, 0, 0], [0, 1, 0], [0, 0, 1], [0.3, -0.7, 0.2]):
        up, _ = oracle.dc3d(*(p + 1e-9 * n), alpha, c, dip, -1, 2, -1.5, 0.3, *disl)
        um, _ = oracle.dc3d(*(p - 1e-9 * n), alpha, c, dip, -1, 2, -1.5, 0.3, *disl)
        b = disl[0] * np.array([1, 0, 0]) + disl[1] * dvec + disl[2] * n
        np.testing.assert_allclose(up[:3] - um[:3], b, atol=1e-7)


def test_far_field_decay(oracle):
    """Stress of a finite source decays like r^-3."""
    mags = []
    for r in (1e3, 1e4):
        u, _ = oracle.dc3d(r, 0.7 * r, -0.5 * r, 2 / 3, 1.0, 60.0, -1, 1, -1, 1, 1.0, 0.5, 0.2)
        mags.append(np.abs(u[3:]).max())
    assert 900 < mags[0] / mags[1] < 1100


def test_vertical_branch_continuity(oracle):
    """The cos(dip) = 0 special forms of the I terms are the limit of the general ones."""
    for d in ([1, 0, 0], [0, 1, 0], [0, 0, 1]):
        u90, _ = oracle.dc3d(0.7, 1.3, -0.4, 2 / 3, 1.0, 90.0, -1, 1.5, -2, 0.3, *d)
        u89, _ = oracle.dc3d(0.7, 1.3, -0.4, 2 / 3, 1.0, 90.0 - 1e-3, -1, 1.5, -2, 0.3, *d)
        assert np.abs(u90[3:] - u89[3:]).max() <= 1e-4 * np.abs(u90[3:]).max()


def test_edge_and_above_surface(oracle):
    u, rc = oracle.dc3d(0.0, 0.0, 0.1, 2 / 3, 1.0, 90.0, -1, 1, -1, 0, 1, 0, 0)
    assert rc == 2 and not np.any(u)
    # receiver on the fault edge (q = 0, eta = 0 inside the strike range)
    u, rc = oracle.dc3d(0.0, 0.0, -1.0, 2 / 3, 1.0, 90.0, -1, 1, -1, 0, 1, 0, 0)
    assert rc == 1 and not np.any(u)


@pytest.mark.parametrize("dip", [90.0, 37.0])
@pytest.mark.parametrize("r", [(0.5, 0.7, 0.3), (1.4, -0.4, -0.2), (-0.6, 1.5, 1.0)])
def test_deep_rectangle_matches_the_kelvin_surface_integral(oracle, dip, r):
    """An independent pin of dc3d's displacement gradient: far below the free surface a finite
    rectangular dislocation tends to its full-space field, Volterra's surface integral of Kelvin's
    point-force solution, u_i,l = -int_S (C : sym(b n))_jk G_ij,kl dS with n = s x d (strike s,
    up-dip d) and b = U1 s + U2 d + U3 n -- formulas that share nothing with Okada's. At 16 km depth
    for a 2 x 1.5 rectangle the two agree to ~1e-12 (the gap scales as depth^-3)."""
    import os
    import sys
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    from test_oracle_hex8 import LAM as lam, MU as mu, _kelvin_grad2
    D = 16000.0
    sd, cd = np.sin(np.radians(dip)), np.cos(np.radians(dip))
    s_, d_ = np.array([1.0, 0.0, 0.0]), np.array([0.0, cd, sd])
    n_ = np.cross(s_, d_)
    al1, al2, aw1, aw2 = -1.0, 1.0, -0.8, 0.7
    g, w = np.polynomial.legendre.leggauss(12)

    def nodes(a, c, npan=16):
        e = np.linspace(a, c, npan + 1)
        m, h = (e[:-1] + e[1:]) / 2, (e[1:] - e[:-1]) / 2
        return (m[:, None] + h[:, None] * g[None, :]).ravel(), (h[:, None] * w[None, :]).ravel()

    (XI, WXI), (ET, WET) = nodes(al1, al2), nodes(aw1, aw2)
    P = (XI[:, None, None] * s_ + ET[None, :, None] * d_ + np.array([0.0, 0.0, -D])).reshape(-1, 3)
    Wt = (WXI[:, None] * WET[None, :]).ravel()
    x = np.array([r[0], r[1], r[2] - D])
    G2w = np.einsum("nijkl,n->ijkl", _kelvin_grad2(x[None, :] - P), Wt)
    alpha = (lam + mu) / (lam + 2 * mu)
    for U in np.eye(3):
        u, rc = oracle.dc3d(*x, alpha, D, dip, al1, al2, aw1, aw2, *U)
        assert rc == 0
        G = np.array([[u[3 + 3 * j + i] for j in range(3)] for i in range(3)])
        b = U[0] * s_ + U[1] * d_ + U[2] * n_
        eps = 0.5 * (np.outer(b, n_) + np.outer(n_, b))
        m = lam * np.trace(eps) * np.eye(3) + 2 * mu * eps
        K = -np.einsum("jk,ijkl->il", m, G2w)
        assert np.abs(G - K).max() <= 1e-11 * np.abs(G).max()
