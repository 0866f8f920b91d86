"""Edge shapes against the FP64 oracle: a single depth row and odd row counts (the paired-row FFT of
the batched kernel), tiny strike lengths, and a one-cell mantle in every storage precision."""
import numpy as np
import pytest

from oetqf_gb300 import PowerLawViscosityProperty, RateStateQuasiDynamicProperty, gen_hex8_box, gen_mesh
from oetqf_gb300.workloads import YEAR

pytestmark = pytest.mark.gpu


def _props(mf, rng, mu=3e10):
    o = np.ones((mf.nx, mf.nξ))
    return RateStateQuasiDynamicProperty(0.015 * o, 0.019 * o, 0.012 * (1 + rng.random((mf.nx, mf.nξ))), 5e7 * o,
                                         mu / (2 * 3044.0), 1e-9, 0.6, 1e-6)


@pytest.mark.parametrize("nx,nxi", [(7, 1), (5, 3), (1, 2), (1, 1), (33, 5)])
def test_fault_shapes_rhs_and_ensemble(oracle, nx, nxi):
    from oetqf_gb300.ensemble import Ensemble
    from oetqf_gb300.equation import GB300Model
    mf = gen_mesh("RectOkada", 1e3 * nx, 1e3 * nxi, 1e3, 1e3, 90.0)
    assert (mf.nx, mf.nξ) == (nx, nxi)
    mu = 3e10
    rng = np.random.default_rng(nx * 10 + nxi)
    gf = oracle.gf_ff(mf, mu, mu, fourier=True)
    pf = _props(mf, rng)
    N = nx * nxi
    m = GB300Model(nx, nxi, 0)
    m.set_gf(1, gf)
    m.set_fault_props(pf)
    u = np.concatenate([1e-9 * np.exp(rng.uniform(-1, 4, N)), 0.012 / 1e-9 * np.exp(rng.uniform(-2, 1, N)), np.zeros(N)])
    ref = oracle.OracleModel(gf, pf).ode(u)
    np.testing.assert_allclose(m.rhs_flat(u), ref, rtol=1e-10, atol=1e-12 * np.abs(ref).max())
    th0 = pf.L.reshape(-1, order="F") / 1e-9 * (1 + 0.01 * rng.uniform(-1, 1, N))
    u0 = np.concatenate([np.full(N, 1e-9), th0, np.zeros(N)])
    T = 0.5 * YEAR
    e = Ensemble([(nx, nxi)])
    e.assemble(0, mf, mu, mu)
    e.set_fault_props(0, pf)
    for alg in ("Tsit5", "VCABM5"):
        ue, se = e.integrate(u0, 0.0, T, reltol=1e-8, abstol=1e-10, dt=1e-3, alg=alg)
        uc, sc = oracle.OracleModel(gf, pf).integrate(u0, 0.0, T, reltol=1e-8, abstol=1e-10, dt0=1e-3, alg=alg)
        assert se[0].status == 0 and se[0].t == T
        assert np.abs(ue[:N] - uc[:N]).max() / np.abs(uc[:N]).max() < 1e-5


@pytest.mark.parametrize("mode", [0, 1, 2, 3])
def test_one_cell_mantle(oracle, mode):
    from oetqf_gb300.equation import GB300Model
    mf = gen_mesh("RectOkada", 12e3, 4e3, 2e3, 1e3, 90.0)      # 6 x 4
    ma = gen_hex8_box(-6e3, -3e3, -6e3, 12e3, 6e3, -6e3, 1, 1, 1)
    mu = 3e10
    gfs = [oracle.gf_ff(mf, mu, mu, fourier=True), oracle.gf_fm(mf, ma, mu, mu), oracle.gf_mf(ma, mf, mu, mu),
           oracle.gf_mm(ma, mu, mu)]
    rng = np.random.default_rng(mode)
    pf = _props(mf, rng)
    pa = PowerLawViscosityProperty(np.full(1, 5e-20), np.zeros(1), np.zeros(6))
    N = mf.nx * mf.nξ
    m = GB300Model(mf.nx, mf.nξ, 1)
    for w, g in zip((1, 2, 3, 4), gfs):
        m.set_gf(w, g)
    m.set_fault_props(pf)
    m.set_mantle_props(pa)
    m.set_precision(mode)
    u = np.concatenate([1e-9 * np.exp(rng.uniform(-1, 4, N)), 0.012 / 1e-9 * np.exp(rng.uniform(-2, 1, N)),
                        np.zeros(6), 1e5 * rng.standard_normal(6), np.zeros(N)])
    du = m.rhs_flat(u)
    assert m.error_word() == 0
    ref = oracle.OracleModel(gfs[0], pf, *gfs[1:], pa).ode(u)
    rows = slice(2 * N + 6, 2 * N + 12)
    x = np.concatenate([u[:N] - 1e-9, ref[2 * N:2 * N + 6]])
    scale = np.abs(np.hstack([gfs[1], gfs[3]])) @ np.abs(x)
    tol = {0: 1e-12, 3: 1e-12, 1: 2 ** -8 * 1.05 + 2 ** -23, 2: 2 ** -11 * 1.05 + 2 ** -23}[mode]
    assert np.all(np.abs(du[rows] - ref[rows]) <= tol * scale + 1e-300)
    np.testing.assert_array_equal(du[2 * N + 12:], ref[2 * N + 12:])  # dδ = v
