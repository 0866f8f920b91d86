"""The numpy/scipy twin of the reference's CPU right-hand side (the second CPU baseline) against the
C oracle: the same ode, through the FFT convolution and BLAS GEMVs instead of direct sums."""
import numpy as np

from oetqf_gb300 import PowerLawViscosityProperty, RateStateQuasiDynamicProperty, gen_hex8_box, gen_mesh


def _fault(mf, mu, rng):
    o = np.ones((mf.nx, mf.nξ))
    return RateStateQuasiDynamicProperty(0.015 * o, 0.019 * o, 0.012 * (1 + rng.random((mf.nx, mf.nξ))), 5e7 * o,
                                         mu / (2 * 3044.0), 1e-9, 0.6, 1e-6)


def test_twin_fault_only_matches_oracle(oracle):
    from numpy_twin import NumpyTwin
    mf = gen_mesh("RectOkada", 40e3, 6e3, 2e3, 1e3, 90.0)
    mu = 3e10
    gf = oracle.gf_ff(mf, mu, mu, fourier=True)
    rng = np.random.default_rng(5)
    pf = _fault(mf, mu, rng)
    N = mf.nx * mf.nξ
    u = np.concatenate([1e-9 * np.exp(rng.uniform(-2, 6, N)), pf.L.reshape(-1, order="F") / 1e-9 * np.exp(rng.uniform(-1, 1, N)),
                        rng.standard_normal(N)])
    ref = oracle.OracleModel(gf, pf).ode(u)
    got = NumpyTwin(gf, pf).ode(u)
    for part in (slice(0, N), slice(N, 2 * N), slice(2 * N, 3 * N)):
        np.testing.assert_allclose(got[part], ref[part], rtol=1e-9, atol=1e-12 * np.abs(ref[part]).max())


def test_twin_viscoelastic_matches_oracle(oracle):
    from numpy_twin import NumpyTwin
    mf = gen_mesh("RectOkada", 40e3, 6e3, 2e3, 1e3, 90.0)
    ma = gen_hex8_box(-20e3, -6e3, -8e3, 40e3, 12e3, -12e3, 3, 2, 2)
    mu = 3e10
    gfs = [oracle.gf_ff(mf, mu, mu, fourier=True), oracle.gf_fm(mf, ma, mu, mu), oracle.gf_mf(ma, mf, mu, mu),
           oracle.gf_mm(ma, mu, mu)]
    rng = np.random.default_rng(9)
    pf = _fault(mf, mu, rng)
    pa = PowerLawViscosityProperty(np.full(ma.ne, 5e-25), np.ones(ma.ne), np.array([1e-15, 0, 0, 2e-15, 0, 0]))
    N, M = mf.nx * mf.nξ, 6 * ma.ne
    u = np.concatenate([1e-9 * np.exp(rng.uniform(-2, 6, N)), pf.L.reshape(-1, order="F") / 1e-9 * np.exp(rng.uniform(-1, 1, N)),
                        rng.standard_normal(M), 1e5 * rng.standard_normal(M), rng.standard_normal(N)])
    ref = oracle.OracleModel(gfs[0], pf, *gfs[1:], pa).ode(u)
    got = NumpyTwin(gfs[0], pf, *gfs[1:], pa).ode(u)
    for part in (slice(0, N), slice(N, 2 * N), slice(2 * N, 2 * N + M), slice(2 * N + M, 2 * N + 2 * M), slice(2 * N + 2 * M, None)):
        np.testing.assert_allclose(got[part], ref[part], rtol=1e-9, atol=1e-12 * np.abs(ref[part]).max())


def test_twin_composite_viscosity_matches_oracle(oracle):
    from numpy_twin import NumpyTwin

    from oetqf_gb300 import CompositePowerLawViscosityProperty
    mf = gen_mesh("RectOkada", 20e3, 4e3, 2e3, 1e3, 90.0)
    ma = gen_hex8_box(-10e3, -4e3, -6e3, 20e3, 8e3, -8e3, 2, 2, 2)
    mu = 3e10
    gfs = [oracle.gf_ff(mf, mu, mu, fourier=True), oracle.gf_fm(mf, ma, mu, mu), oracle.gf_mf(ma, mf, mu, mu),
           oracle.gf_mm(ma, mu, mu)]
    rng = np.random.default_rng(13)
    pf = _fault(mf, mu, rng)
    pa = CompositePowerLawViscosityProperty([PowerLawViscosityProperty(np.full(ma.ne, 5e-20), np.zeros(ma.ne), np.zeros(6)),
                                             PowerLawViscosityProperty(np.full(ma.ne, 1e-30), np.full(ma.ne, 2.0), np.zeros(6))],
                                            np.array([0.0, 1e-15, 0, 0, 0, 0]))
    N, M = mf.nx * mf.nξ, 6 * ma.ne
    u = np.concatenate([1e-9 * np.exp(rng.uniform(-2, 6, N)), pf.L.reshape(-1, order="F") / 1e-9 * np.exp(rng.uniform(-1, 1, N)),
                        np.zeros(M), 1e6 * rng.standard_normal(M), np.zeros(N)])
    ref = oracle.OracleModel(gfs[0], pf, *gfs[1:], pa).ode(u)
    got = NumpyTwin(gfs[0], pf, *gfs[1:], pa).ode(u)
    for part in (slice(0, N), slice(N, 2 * N), slice(2 * N, 2 * N + M), slice(2 * N + M, 2 * N + 2 * M), slice(2 * N + 2 * M, None)):
        np.testing.assert_allclose(got[part], ref[part], rtol=1e-9, atol=1e-12 * np.abs(ref[part]).max())
