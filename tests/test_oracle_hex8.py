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


def _kelvin_grad2(r):
    """Second derivatives G_ij,kl of Kelvin's full-space point-force solution
    G_ij = [(3 - 4 nu) delta_ij / r + r_i r_j / r^3] / (16 pi mu (1 - nu)) at r = x - xi (..., 3)."""
    A = 1.0 / (16 * np.pi * MU * (1 - NU))
    d = np.eye(3)
    R = np.linalg.norm(r, axis=-1)[..., None, None, None, None]
    ri, rj = r[..., :, None, None, None], r[..., None, :, None, None]
    rk, rl = r[..., None, None, :, None], r[..., None, None, None, :]
    dij, dkl = d[:, :, None, None], d[None, None, :, :]
    dik, djl, djk, dil = d[:, None, :, None], d[None, :, None, :], d[None, :, :, None], d[:, None, None, :]
    t = -(3 - 4 * NU) * dij * (dkl / R ** 3 - 3 * rk * rl / R ** 5)
    t = t + dik * (djl / R ** 3 - 3 * rj * rl / R ** 5) + djk * (dil / R ** 3 - 3 * ri * rl / R ** 5)
    t = t - 3 * ((dil * rj * rk + djl * ri * rk + dkl * ri * rj) / R ** 5 - 5 * ri * rj * rk * rl / R ** 7)
    return A * t


def _kelvin_cuboid_unit_stresses(x, box, npan=4, ng=10):
    """Full-space stress outside a cuboid holding each unit eigenstrain (xx, xy, xz, yy, yz, zz; the
    shear ones as tensor components eps_ij = eps_ji = 1): u_i,l = -int_V (C:eps)_jk G_ij,kl dV
    (Mura's inclusion integral) by composite Gauss-Legendre, then sigma = C : grad u."""
    g, w = np.polynomial.legendre.leggauss(ng)

    def nodes(a, b):
        e = np.linspace(a, b, npan + 1)
        m, h = (e[:-1] + e[1:]) / 2, (e[1:] - e[:-1]) / 2
        return (m[:, None] + h[:, None] * g[None, :]).ravel(), (h[:, None] * w[None, :]).ravel()

    (X, WX), (Y, WY), (Z, WZ) = (nodes(*b) for b in box)
    P = np.stack(np.meshgrid(X, Y, Z, indexing="ij"), -1).reshape(-1, 3)
    Wt = (WX[:, None, None] * WY[None, :, None] * WZ[None, None, :]).ravel()
    G2w = np.einsum("nijkl,n->ijkl", _kelvin_grad2(x[None, :] - P), Wt)
    out = np.zeros((6, 6))
    for p, (a, b) in enumerate([(0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2)]):
        eps = np.zeros((3, 3))
        eps[a, b] = eps[b, a] = 1.0
        m = LAM * np.trace(eps) * np.eye(3) + 2 * MU * eps
        gu = -np.einsum("jk,ijkl->il", m, G2w)
        s = LAM * np.trace(gu) * np.eye(3) + MU * (gu + gu.T)
        out[p] = [s[0, 0], s[0, 1], s[0, 2], s[1, 1], s[1, 2], s[2, 2]]
    return out


@pytest.mark.parametrize("r", [(2.5, 0.7, -0.5), (0.2, 2.3, -0.4), (-1.0, 3.0, 1.0), (0.1, 0.5, -2.5)])
def test_deep_cuboid_matches_the_kelvin_volume_integral(oracle, r):
    """An independent pin of the strain-volume stress: far below the free surface the half-space
    solution tends to the full-space one, which is Mura's volume integral of Kelvin's point-force
    solution over the cuboid -- formulas that share nothing with the Okada dislocation planes the
    oracle stacks. At 16 km depth for a 1.3 x 1.7 x 1.1 cuboid the two agree to ~1e-12 (the gap
    scales as depth^-3: the surface's image term), receivers 0.4 to 2.5 from the faces, all six
    unit eigenstrains."""
    D = 16000.0
    qx, qy, qz, T, L, W = 0.1, -0.3, -D, 1.3, 1.7, 1.1
    box = ((qx - T / 2, qx + T / 2), (qy, qy + L), (qz - W, qz))
    x = np.array([r[0], r[1], r[2] - D])
    ref = oracle.hex8_unit_stresses(*x, qx, qy, qz, T, L, W, MU, NU)
    kv = _kelvin_cuboid_unit_stresses(x, box)
    assert np.abs(ref - kv).max() <= 1e-11 * np.abs(ref).max()
