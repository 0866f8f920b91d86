"""Oracle strain-volume stress (the quantity of GeoGreensFunctions.stress_vol_hex8!, called at
src/BEM/GF.jl:215-221, :277-283) pinned by elasticity identities and by independence of the
dislocation-stacking direction."""
import numpy as np
import pytest

MU, NU = 1.0, 0.25
LAM = 2 * MU * NU / (1 - 2 * NU)


def test_thin_plate_limit(oracle):
    """eps_xx in a thin, wide, deep plate normal to z: the plate is clamped in-plane, free
    across its thickness: sig_xx = -4 mu (lam + mu)/(lam + 2 mu), sig_yy = -2 lam mu/(lam + 2 mu)."""
    s = oracle.hex8_unit_stresses(0, 0, -5000, 0, -500, -4999.5, 1000, 1000, 1.0, MU, NU)
    assert s[0][0] == pytest.approx(-4 * MU * (LAM + MU) / (LAM + 2 * MU), rel=2e-3)
    assert s[0][3] == pytest.approx(-2 * LAM * MU / (LAM + 2 * MU), rel=2e-3)
    assert abs(s[0][5]) < 2e-3


def test_compatible_shear_is_stress_free(oracle):
    """Simple shear eps_xy in a thin plate normal to y is compatible: no stress."""
    s = oracle.hex8_unit_stresses(0, 0, -5000, 0, -0.5, -4500, 1000, 1.0, 1000, MU, NU)
    assert abs(s[1][1]) < 3e-3


@pytest.mark.parametrize("r", [(0.3, 2.0), (1.7, -0.4), (0.1, 0.2)])
def test_traction_free_surface(oracle, r):
    s = oracle.hex8_unit_stresses(r[0], r[1], 0.0, 0, 0, -1, 2, 2, 1.5, MU, NU)
    assert np.abs(s[:, [2, 4, 5]]).max() <= 1e-13 * np.abs(s).max()


def test_equilibrium(oracle):
    h = 1e-3
    idx = {(0, 0): 0, (0, 1): 1, (0, 2): 2, (1, 0): 1, (1, 1): 3, (1, 2): 4, (2, 0): 2, (2, 1): 4, (2, 2): 5}
    for r in [(0.5, 0.2, -1.0), (0.4, 0.6, -2.5), (3.0, 1.0, -4.0)]:
        g = np.zeros((6, 3, 6))
        for j, e in enumerate(np.eye(3)):
            sp = oracle.hex8_unit_stresses(*(np.array(r) + h * e), 0.1, -0.3, -2, 1.3, 1.7, 1.1, MU, NU)
            sm = oracle.hex8_unit_stresses(*(np.array(r) - h * e), 0.1, -0.3, -2, 1.3, 1.7, 1.1, MU, NU)
            g[:, j, :] = (sp - sm) / (2 * h)
        res = np.zeros((6, 3))
        for i in range(3):
            for j in range(3):
                res[:, i] += g[:, j, idx[(i, j)]]
        assert np.abs(res).max() <= 1e-5 * np.abs(g).max()


def test_face_traction_continuity(oracle):
    qx, qy, qz, T, L, W = 0.1, -0.3, -2, 1.3, 1.7, 1.1
    xf = qx + T / 2
    si = oracle.hex8_unit_stresses(xf - 1e-7, 0.2, -2.5, qx, qy, qz, T, L, W, MU, NU)
    so = oracle.hex8_unit_stresses(xf + 1e-7, 0.2, -2.5, qx, qy, qz, T, L, W, MU, NU)
    assert np.abs((si - so)[:, [0, 1, 2]]).max() < 1e-5
    # the in-plane stress jumps by the eigenstress contrast (eps_yy: sig_yy jumps)
    assert np.abs((si - so)[3, 3]) > 0.5


def test_self_stress_relaxes(oracle):
    """Inside its own deep cube a shear eigenstrain produces an opposing stress of order 2 mu."""
    s = oracle.hex8_unit_stresses(0, 0, -1000, 0, -0.5, -999.5, 1, 1, 1, MU, NU)
    assert -1.6 < s[1][1] < -0.8
    assert -2.6 < s[0][0] < -0.8


def _dc_grad(oracle, *args):
    u, _ = oracle.dc3d(*args)
    return np.array([[u[3 + 3 * j + i] for j in range(3)] for i in range(3)])


def _stress(G):
    e = 0.5 * (G + G.T)
    s = LAM * np.trace(G) * np.eye(3) + 2 * MU * e
    return np.array([s[0, 0], s[0, 1], s[0, 2], s[1, 1], s[1, 2], s[2, 2]])


def _composite(a, b, f, npan=24):
    xg, wg = np.polynomial.legendre.leggauss(16)
    edges = np.linspace(a, b, npan + 1)
    tot = 0
    for i in range(npan):
        m, h = (edges[i] + edges[i + 1]) / 2, (edges[i + 1] - edges[i]) / 2
        for t, w in zip(xg, wg):
            tot = tot + h * w * f(m + h * t)
    return tot


@pytest.mark.parametrize("r", [(2.5, 0.7, -1.0), (0.2, 0.3, -2.4), (-1.0, 3.0, -0.5)])
def test_stacking_direction_independence(oracle, r):
    """eps_yz, eps_xy, eps_xz recomputed from stacks of a different orientation (and a plain
    composite Gauss rule) agree with the oracle's adaptive panels."""
    x, y, z = r
    qx, qy, qz, T, L, W = 0.1, -0.3, -2, 1.3, 1.7, 1.1
    x1, x2, y1, y2, z1, z2 = qx - T / 2, qx + T / 2, qy, qy + L, qz - W, qz
    alpha = (LAM + MU) / (LAM + 2 * MU)
    Q = np.array([[0, 1, 0], [-1, 0, 0], [0, 0, 1]])
    ref = oracle.hex8_unit_stresses(x, y, z, qx, qy, qz, T, L, W, MU, NU)
    sc = np.abs(ref).max()
    a_yz = _stress(_composite(z1, z2, lambda s: _dc_grad(oracle, x, y, z, alpha, -s, 0.0, x1, x2, y1, y2, 0.0, 2.0, 0.0)))
    a_xy = _stress(_composite(x1, x2, lambda s: Q.T @ _dc_grad(oracle, y, s - x, z, alpha, 0.0, 90.0, y1, y2, z1, z2, 2.0, 0.0, 0.0) @ Q))
    a_xz = _stress(_composite(x1, x2, lambda s: Q.T @ _dc_grad(oracle, y, s - x, z, alpha, 0.0, 90.0, y1, y2, z1, z2, 0.0, 2.0, 0.0) @ Q))
    assert np.abs(a_yz - ref[4]).max() <= 1e-12 * sc
    assert np.abs(a_xy - ref[1]).max() <= 1e-12 * sc
    assert np.abs(a_xz - ref[2]).max() <= 1e-12 * sc


def test_gauss_legendre_table(oracle):
    for k, n in enumerate((4, 8, 12, 16)):
        x, w = oracle.gl_table(k)
        xr, wr = np.polynomial.legendre.leggauss(n)
        np.testing.assert_allclose(x, xr, atol=1e-15)
        np.testing.assert_allclose(w, wr, atol=1e-15)
