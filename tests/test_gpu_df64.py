"""Double-float mantle Green's functions (GBC_PREC_DF64): FP32 pairs hi + lo with compensated
products and sums on the FP32 pipe.

Bar: FP64-equivalent. Each mantle-row result lies within 1e-12 * sum_j |G_ij x_j| of the FP64
oracle (the pair representation is exact to 2^-48 per operand; the compensated sums add ~n 2^-48
of sum |terms| over a lane's n terms), derivatives within 1e-10 relative, and the fault-only model
(no mantle GEMV) is bitwise the FP64 path."""
import numpy as np
import pytest

from oetqf_gb300 import PowerLawViscosityProperty, RateStateQuasiDynamicProperty, gen_hex8_box, gen_mesh

pytestmark = pytest.mark.gpu
DF64 = 3
ROW_TOL = 1e-12


def _props(mf, ne, rng, mu=3e10):
    o = np.ones((mf.nx, mf.nξ))
    pf = RateStateQuasiDynamicProperty(0.015 * o, 0.019 * o, 0.012 * (1 + rng.random((mf.nx, mf.nξ))), 5e7 * o,
                                       mu / (2 * 3044.0), 1e-9, 0.6, 1e-6)
    pa = PowerLawViscosityProperty(np.full(ne, 5e-20), np.zeros(ne), np.zeros(6))
    return pf, pa


def _model(mf, ne, gfs, pf, pa, mode):
    from oetqf_gb300.equation import GB300Model
    m = GB300Model(mf.nx, mf.nξ, ne)
    for w, g in zip((1, 2, 3, 4), gfs):
        m.set_gf(w, g)
    m.set_fault_props(pf)
    if ne:
        m.set_mantle_props(pa)
    m.set_precision(mode)
    return m


def _state(N, M, rng):
    v = 1e-9 * np.exp(rng.uniform(-2, 8, N))
    th = 0.012 / 1e-9 * np.exp(rng.uniform(-3, 1, N))
    sig = 1e5 * rng.standard_normal(M) * np.exp(rng.uniform(-8, 2, M))
    return np.concatenate([v, th, np.zeros(M), sig, np.zeros(N)])


def _check_rows(du, ref, gfs, u, N, M):
    deps = ref[2 * N:2 * N + M]
    x = np.concatenate([u[:N] - 1e-9, deps])
    Gm = np.hstack([gfs[1], gfs[3]])
    scale = np.abs(Gm) @ np.abs(x) + 1e-300
    err = np.abs(du[2 * N + M:2 * N + 2 * M] - ref[2 * N + M:2 * N + 2 * M])
    assert np.all(err <= ROW_TOL * scale), np.max(err / scale)
    np.testing.assert_array_equal(du[2 * N:2 * N + M], deps)          # strain rates are FP64 in both
    np.testing.assert_array_equal(du[2 * N + 2 * M:], ref[2 * N + 2 * M:])  # dδ = v
    return np.max(err / scale)


def test_df64_rhs_vs_fp64_oracle_physical(oracle):
    mf = gen_mesh("RectOkada", 70e3, 6e3, 2e3, 1e3, 90.0)   # 210 patches
    ma = gen_hex8_box(-35e3, -6e3, -8e3, 70e3, 12e3, -12e3, 3, 3, 3)
    mu = 3e10
    gfs = [oracle.gf_ff(mf, mu, mu, fourier=True), oracle.gf_fm(mf, ma, mu, mu), oracle.gf_mf(ma, mf, mu, mu),
           oracle.gf_mm(ma, mu, mu)]
    rng = np.random.default_rng(21)
    pf, pa = _props(mf, ma.ne, rng)
    N, M = mf.nx * mf.nξ, 6 * ma.ne
    m = _model(mf, ma.ne, gfs, pf, pa, DF64)
    m64 = _model(mf, ma.ne, gfs, pf, pa, 0)
    u = _state(N, M, rng)
    du = m.rhs_flat(u)
    assert m.error_word() == 0
    ref = oracle.OracleModel(gfs[0], pf, *gfs[1:], pa).ode(u)
    _check_rows(du, ref, gfs, u, N, M)
    # fault rows: FP64 Toeplitz + the double-float G21 part -> dv, dθ within 1e-10 of the oracle
    np.testing.assert_allclose(du[:N], ref[:N], rtol=1e-10, atol=1e-10 * np.abs(ref[:N]).max())
    np.testing.assert_allclose(du[N:2 * N], ref[N:2 * N], rtol=1e-14)
    # and the FP64 GPU path sees the same within the same bar
    d64 = m64.rhs_flat(u)
    np.testing.assert_allclose(du[:N], d64[:N], rtol=1e-10, atol=1e-10 * np.abs(d64[:N]).max())


@pytest.mark.parametrize("ne,seed", [(400, 1), (131, 2)])
def test_df64_rows_random_wide_range(oracle, ne, seed):
    """Random Green's functions spanning 12 decades, with tile counts above and below the SM count
    and an uneven split of tiles over the persistent grid."""
    mf = gen_mesh("RectOkada", 70e3, 6e3, 2e3, 1e3, 90.0)
    N, M = mf.nx * mf.nξ, 6 * ne
    rng = np.random.default_rng(seed)
    mu = 3e10

    def wide(shape):
        return mu * rng.standard_normal(shape) * np.exp(rng.uniform(-14, 14, shape))

    gf11 = oracle.gf_ff(mf, mu, mu, fourier=True)
    gfs = [gf11, wide((M, N)), wide((N, M)), wide((M, M))]
    pf, pa = _props(mf, ne, rng)
    m = _model(mf, ne, gfs, pf, pa, DF64)
    u = _state(N, M, rng)
    du = m.rhs_flat(u)
    assert m.error_word() == 0
    ref = oracle.OracleModel(gfs[0], pf, *gfs[1:], pa).ode(u)
    worst = _check_rows(du, ref, gfs, u, N, M)
    assert worst < ROW_TOL


def test_df64_fault_only_is_the_fp64_path(oracle):
    mf = gen_mesh("RectOkada", 40e3, 8e3, 1e3, 1e3, 90.0)
    mu = 3e10
    gf = oracle.gf_ff(mf, mu, mu, fourier=True)
    rng = np.random.default_rng(3)
    pf, _ = _props(mf, 0, rng)
    N = mf.nx * mf.nξ
    u = np.concatenate([1e-9 * np.exp(rng.uniform(0, 6, N)), 0.012 / 1e-9 * np.exp(rng.uniform(-2, 0, N)), np.zeros(N)])
    a = _model(mf, 0, [gf], pf, None, DF64).rhs_flat(u)
    b = _model(mf, 0, [gf], pf, None, 0).rhs_flat(u)
    np.testing.assert_array_equal(a, b)


def test_df64_integration_tracks_fp64(oracle):
    mf = gen_mesh("RectOkada", 70e3, 6e3, 2e3, 1e3, 90.0)
    ma = gen_hex8_box(-35e3, -6e3, -8e3, 70e3, 12e3, -12e3, 3, 3, 3)
    mu = 3e10
    gfs = [oracle.gf_ff(mf, mu, mu, fourier=True), oracle.gf_fm(mf, ma, mu, mu), oracle.gf_mf(ma, mf, mu, mu),
           oracle.gf_mm(ma, mu, mu)]
    rng = np.random.default_rng(11)
    pf, pa = _props(mf, ma.ne, rng)
    N, ne = mf.nx * mf.nξ, ma.ne
    th0 = pf.L.reshape(-1, order="F") / 1e-9 * (1 + 0.01 * rng.uniform(-1, 1, N))
    u0 = np.concatenate([np.full(N, 1e-9), th0, np.zeros(6 * ne), np.zeros(6 * ne), np.zeros(N)])
    T = 3.15e7
    u64, s64 = _model(mf, ne, gfs, pf, pa, 0).integrate(u0, 0.0, T, reltol=1e-8, abstol=1e-10, dt=1e-3)
    udf, sdf = _model(mf, ne, gfs, pf, pa, DF64).integrate(u0, 0.0, T, reltol=1e-8, abstol=1e-10, dt=1e-3)
    assert s64.status == 0 and sdf.status == 0
    rel = np.abs(udf[:N] - u64[:N]).max() / np.abs(u64[:N]).max()
    assert rel < 1e-8, rel
    np.testing.assert_allclose(udf[N:2 * N], u64[N:2 * N], rtol=1e-8)
