"""Mesh generators against the reference's invariants (test/BEM/tests.jl:4-37)."""
import numpy as np
import pytest

from oetqf_gb300.mesh import gen_hex8_box, gen_mesh, sincosd


def test_rect_okada():
    msh = gen_mesh("RectOkada", 100.0, 50.0, 2.0, 2.0, 33.0)
    assert msh.nx == 50
    assert msh.nξ == 25
    assert msh.aξ[-1][0] == msh.ξ[-1] - msh.Δξ / 2
    s, c = sincosd(msh.dip)
    assert msh.y[-1] == msh.ξ[-1] * c
    assert msh.z[-1] == msh.ξ[-1] * s
    assert msh.x[-1] - msh.x[0] == pytest.approx(msh.Δx * (msh.nx - 1), rel=1e-15)


def test_rect_okada_shapes():
    m0 = gen_mesh("RectOkada", 80e3, 10e3, 1e3, 1e3, 90.0)
    assert (m0.nx, m0.nξ) == (80, 10)
    assert m0.ξ[0] == -500.0 and m0.aξ[0][1] == 0.0 and m0.z[-1] == -9500.0
    assert np.all(m0.y == 0.0)


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_hex8_box(seed):
    rng = np.random.default_rng(seed)
    llx, lly, llz = rng.random(3)
    dx, dy, dz = rng.random(3) * 5
    nx, ny, nz = rng.integers(2, 11, 3)
    me = gen_hex8_box(llx, lly, llz, dx, dy, -dz, nx, ny, nz)
    for x, tx in zip([me.cx, me.cy, me.cz], [nx, ny, nz]):
        assert len(np.unique(np.round(x, 6))) == tx
    np.testing.assert_allclose(me.cx, me.qx)
    np.testing.assert_allclose(me.cy - me.Δy / 2, me.qy)
    np.testing.assert_allclose(me.cz + me.Δz / 2, me.qz)
    assert np.max(me.cx + me.Δx / 2) == pytest.approx(llx + dx)
    assert np.min(me.cx - me.Δx / 2) == pytest.approx(llx)
    assert np.max(me.cy + me.Δy / 2) == pytest.approx(lly + dy)
    assert np.min(me.cy - me.Δy / 2) == pytest.approx(lly)
    assert np.max(me.cz + me.Δz / 2) == pytest.approx(llz)
    assert np.min(me.cz - me.Δz / 2) == pytest.approx(llz - dz)


def test_hex8_box_layers():
    me = gen_hex8_box(-40e3, -2.5e3, -8e3, 80e3, 5e3, -22e3, 4, 3, 3, rfzh=np.cumprod(np.ones(3) * 1.5))
    assert me.ne == 36
    np.testing.assert_allclose(np.sort(np.unique(np.round(me.Δz, 6))), np.sort(22e3 * np.array([1.5, 2.25, 3.375]) / 7.125))


def test_gmsh_quadrature_hex():
    """gmsh_quadrature(5, "GaussN") / get_quadrature (src/BEM/GF.jl:300-328): tensor-product rules that
    integrate monomials of total degree <= N exactly over [-1, 1]^3; get_quadrature normalises."""
    from oetqf_gb300 import get_quadrature, gmsh_quadrature
    for order in (1, 2, 3, 4, 5):
        c, w = gmsh_quadrature(5, f"Gauss{order}")
        pts = np.asarray(c).reshape(-1, 3)
        assert pts.shape[0] == len(w) and abs(w.sum() - 8.0) < 1e-13
        for a in range(order + 1):
            for b in range(order + 1 - a):
                for d in range(order + 1 - a - b):
                    exact = np.prod([0.0 if k % 2 else 2.0 / (k + 1) for k in (a, b, d)])
                    got = np.sum(w * pts[:, 0] ** a * pts[:, 1] ** b * pts[:, 2] ** d)
                    assert abs(got - exact) < 1e-12
        cn, wn = get_quadrature(f"Gauss{order}")
        assert abs(wn.sum() - 1.0) < 1e-14
    c1, w1 = get_quadrature("Gauss1")
    np.testing.assert_array_equal(np.asarray(c1).reshape(-1), np.zeros(3))
    with pytest.raises(NotImplementedError):
        gmsh_quadrature(4, "Gauss1")
    with pytest.raises(AssertionError):
        get_quadrature((np.zeros(4), np.ones(2)))
