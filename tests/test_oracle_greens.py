"""Green's-function assembly of the oracle against the reference's own tests and identities."""
import numpy as np
import pytest

from oetqf_gb300.mesh import gen_hex8_box, gen_mesh, gauss_product_quadrature
from oetqf_gb300.property import RateStateQuasiDynamicProperty


class _P:
    def __init__(self, nx, nxi, vpl):
        o = np.ones((nx, nxi))
        self.a, self.b, self.L, self.σ = o, o, o, o
        self.η, self.vpl, self.f0, self.v0 = 1.0, vpl, 0.6, 1e-6


@pytest.mark.parametrize("ftype", [0, 1])
def test_fft_conv_equals_dense_toeplitz(oracle, ftype):
    """test/BEM/tests.jl:39-61: rFFT convolution == dense Toeplitz contraction."""
    mf = gen_mesh("RectOkada", 100.0, 100.0, 10.0, 10.0, 41.0)
    gf1 = oracle.gf_ff(mf, 3e10, 3e10, ftype=ftype, fourier=True)
    gf2 = oracle.gf_ff(mf, 3e10, 3e10, ftype=ftype, fourier=False)
    gf3 = np.empty((mf.nx, mf.nξ, mf.nx, mf.nξ))
    for l in range(mf.nξ):
        for k in range(mf.nx):
            for j in range(mf.nξ):
                for i in range(mf.nx):
                    gf3[i, j, k, l] = gf2[abs(i - k), j, l]
    rng = np.random.default_rng(3)
    v = rng.random((mf.nx, mf.nξ))
    vpl = 0.1
    E = np.einsum("ijkl,kl->ij", gf3, v - vpl)
    m = oracle.OracleModel(gf1, _P(mf.nx, mf.nξ, vpl))
    dtau = m.dtau_dt(v).reshape((mf.nx, mf.nξ), order="F")
    np.testing.assert_allclose(dtau, E, rtol=1e-10, atol=1e-10 * np.abs(E).max())


def test_ff_toeplitz_translation(oracle):
    """The reference stores only the source in strike cell 1 (src/BEM/GF.jl:49-53) and relies on
    st[|i-k|, j, l] being the traction at x_i from cell k; check it against direct dc3d sums."""
    mf = gen_mesh("RectOkada", 20e3, 5e3, 1e3, 1e3, 90.0)
    lam = mu = 3e10
    st = oracle.gf_ff(mf, lam, mu, buffer_ratio=1.0, nrept=2)
    assert np.all(st[0, np.arange(mf.nξ), np.arange(mf.nξ)] < 0)   # self-stiffness opposes slip
    alpha = (lam + mu) / (lam + 2 * mu)
    lrept = 2.0 * mf.Δx * mf.nx
    for (i, k, j, l) in [(3, 11, 2, 4), (17, 5, 0, 0), (9, 9, 4, 1)]:
        acc = np.zeros(12)
        for p in range(-2, 3):
            u, _ = oracle.dc3d(mf.x[i], mf.y[j], mf.z[j], alpha, 0.0, 90.0, mf.ax[k][0] + p * lrept,
                               mf.ax[k][1] + p * lrept, mf.aξ[l][0], mf.aξ[l][1], 1.0, 0.0, 0.0)
            acc += u
        t = -mu * (acc[4] + acc[6])
        assert t == pytest.approx(st[abs(i - k), j, l], rel=1e-12, abs=1e-12 * np.abs(st).max())


def _small_pair():
    mf = gen_mesh("RectOkada", 100.0, 100.0, 10.0, 20.0, 90.0)
    ma = gen_hex8_box(-100.0, -50.0, -20.0, 200.0, 100.0, -30.0, 2, 3, 4)
    return mf, ma


def test_mantle_gf_shapes_and_selfterms(oracle):
    mf, ma = _small_pair()
    g12 = oracle.gf_fm(mf, ma, 1.0, 1.0)
    g21 = oracle.gf_mf(ma, mf, 1.0, 1.0)
    g22 = oracle.gf_mm(ma, 1.0, 1.0)
    ne, N = ma.ne, mf.nx * mf.nξ
    assert g12.shape == (6 * ne, N) and g21.shape == (N, 6 * ne) and g22.shape == (6 * ne, 6 * ne)
    assert np.all(np.isfinite(g12)) and np.all(np.isfinite(g21)) and np.all(np.isfinite(g22))
    d = np.diag(g22)
    assert np.all(d < 0)  # each unit strain relaxes its own stress component
    # src/BEM/GF.jl:291-294 prints the largest real eigenvalue; Gauss1 keeps it small
    ev = np.linalg.eigvals(g22)
    assert ev.real.max() < 0.05 * np.abs(ev.real).max()


def test_reciprocity_fault_mantle(oracle):
    """Mura reciprocity between a strike-slip patch and a strain volume:
    A * <traction on the patch from eps_p>  ==  V * c_p * <sigma_p in the cell from unit slip>,
    c_p = 2 for shear components; both sides integrated with product Gauss rules. This ties the
    Okada (fault->mantle) and strain-volume (mantle->fault) kernels to each other."""
    lam = mu = 1.0
    nu = lam / 2 / (lam + mu)
    alpha = (lam + mu) / (lam + 2 * mu)
    # one patch x in [0,1], z in [-1,0] on y = 0; one cell below and beside it
    cell = dict(qx=0.8, qy=0.4, qz=-1.3, T=0.9, L=0.7, W=0.8)
    tg, tw = np.polynomial.legendre.leggauss(8)
    lhs = np.zeros(6)
    for a, wa in zip(tg, tw):
        for b, wb in zip(tg, tw):
            x, z = 0.5 + 0.5 * a, -0.5 + 0.5 * b
            s = oracle.hex8_unit_stresses(x, 0.0, z, cell["qx"], cell["qy"], cell["qz"], cell["T"], cell["L"], cell["W"], mu, nu)
            lhs += 0.25 * wa * wb * (-s[:, 1])  # strike-slip traction, dip 90: -sigma_xy
    qc, qw = gauss_product_quadrature(8)
    rhs = np.zeros(6)
    V = cell["T"] * cell["L"] * cell["W"]
    for q in range(len(qw)):
        rx = cell["qx"] + qc[3 * q] * cell["T"] / 2
        ry = cell["qy"] + cell["L"] / 2 + qc[3 * q + 1] * cell["L"] / 2
        rz = cell["qz"] - cell["W"] / 2 + qc[3 * q + 2] * cell["W"] / 2
        u, _ = oracle.dc3d(rx, ry, rz, alpha, 0.0, 90.0, 0.0, 1.0, -1.0, 0.0, 1.0, 0.0, 0.0)
        G = np.array([[u[3 + 3 * j + i] for j in range(3)] for i in range(3)])
        S = lam * np.trace(G) * np.eye(3) + mu * (G + G.T)
        rhs += qw[q] * V * np.array([S[0, 0], 2 * S[0, 1], 2 * S[0, 2], S[1, 1], 2 * S[1, 2], S[2, 2]])
    np.testing.assert_allclose(lhs, rhs, rtol=1e-6, atol=1e-6 * np.abs(rhs).max())


def test_receiver_rows_equal_the_full_blocks(oracle):
    """The receiver-subset routines (used to check the 8000-cell mantle on the GPU) run the same
    loops as the full blocks: their rows are bit for bit the full blocks' rows."""
    from oetqf_gb300 import gen_hex8_box, gen_mesh
    mf = gen_mesh("RectOkada", 100.0, 100.0, 10.0, 20.0, 90.0)
    ma = gen_hex8_box(-100.0, -50.0, -20.0, 200.0, 100.0, -30.0, 2, 3, 4)
    g12, g21, g22 = oracle.gf_fm(mf, ma, 1.0, 1.0), oracle.gf_mf(ma, mf, 1.0, 1.0), oracle.gf_mm(ma, 1.0, 1.0)
    ne, cells, patches = ma.ne, [0, 5, 23], [0, 7, mf.nx * mf.nξ - 1]
    r12, r22 = oracle.gf_fm_rows(mf, ma, 1.0, 1.0, cells), oracle.gf_mm_rows(ma, 1.0, 1.0, cells)
    for a, j in enumerate(cells):
        for k in range(6):
            assert np.array_equal(r12[a, k], g12[k * ne + j])
            assert np.array_equal(r22[a, k], g22[k * ne + j])
    r21 = oracle.gf_mf_rows(ma, mf, 1.0, 1.0, patches)
    for a, i in enumerate(patches):
        assert np.array_equal(r21[a], g21[i])
