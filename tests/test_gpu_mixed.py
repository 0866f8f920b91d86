"""Block-scaled 16-bit mantle Green's functions (GBC_PREC_BF16 / GBC_PREC_F16).

Two bars: (1) the kernel computes exactly the block-scaled algorithm -- checked against a numpy
emulation of the same quantisation with FP32-accumulation tolerance; (2) the physical error
against the FP64 oracle stays inside the 16-bit rounding bound u * sum|G||x| per row."""
import numpy as np
import pytest

from oetqf_gb300 import PowerLawViscosityProperty, RateStateQuasiDynamicProperty, gen_hex8_box, gen_mesh

pytestmark = pytest.mark.gpu
QB = 128


def _round_bf16(x32: np.ndarray) -> np.ndarray:
    b = x32.astype(np.float32).view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) >> 16 << 16
    return b.astype(np.uint32).view(np.float32)


def _setup(oracle, seed=7, ne_cells=(3, 3, 3)):
    mf = gen_mesh("RectOkada", 70e3, 6e3, 2e3, 1e3, 90.0)   # 35 x 6 = 210 patches (N not a multiple of 32)
    ma = gen_hex8_box(-35e3, -6e3, -8e3, 70e3, 12e3, -12e3, *ne_cells)
    mu = 3e10
    gfs = [oracle.gf_ff(mf, mu, mu, fourier=True), oracle.gf_fm(mf, ma, mu, mu), oracle.gf_mf(ma, mf, mu, mu),
           oracle.gf_mm(ma, mu, mu)]
    rng = np.random.default_rng(seed)
    N, ne = mf.nx * mf.nξ, ma.ne
    o = np.ones((mf.nx, mf.nξ))
    pf = RateStateQuasiDynamicProperty(0.015 * o, 0.019 * o, 0.012 * (1 + rng.random((mf.nx, mf.nξ))), 5e7 * o,
                                       mu / (2 * 3044.0), 1e-9, 0.6, 1e-6)
    pa = PowerLawViscosityProperty(np.full(ne, 5e-20), np.zeros(ne), np.zeros(6))
    return mf, ma, gfs, pf, pa


def _model(mf, ma, gfs, pf, pa, mode):
    from oetqf_gb300.equation import GB300Model
    m = GB300Model(mf.nx, mf.nξ, ma.ne)
    for w, g in zip((1, 2, 3, 4), gfs):
        m.set_gf(w, g)
    m.set_fault_props(pf)
    m.set_mantle_props(pa)
    m.set_precision(mode)
    return m


def _emulate_rows(G, x, mode):
    """y = sum_blocks s * sum q x with the library's quantisation of one row-block-aligned matrix."""
    R, Cc = G.shape
    y = np.zeros(R)
    for rb in range(0, R, QB):
        for cb in range(0, Cc, QB):
            blk = G[rb:rb + QB, cb:cb + QB]
            amax = np.abs(blk).max()
            s = np.float32(amax / 32768.0) if amax > 0 else np.float32(1.0)
            v = (blk / np.float64(s)).astype(np.float32)
            q = _round_bf16(v) if mode == 1 else v.astype(np.float16).astype(np.float32)
            y[rb:rb + QB] += np.float64(s) * (q.astype(np.float64) @ x[cb:cb + QB].astype(np.float32).astype(np.float64))
    return y


@pytest.mark.parametrize("mode", [1, 2])
def test_mixed_rhs_is_the_block_scaled_algorithm(oracle, mode):
    mf, ma, gfs, pf, pa = _setup(oracle)
    m = _model(mf, ma, gfs, pf, pa, mode)
    N, ne = mf.nx * mf.nξ, ma.ne
    M = 6 * ne
    rng = np.random.default_rng(3)
    v = 1e-9 * np.exp(rng.uniform(-2, 8, N))
    th = 0.012 / 1e-9 * np.exp(rng.uniform(-3, 1, N))
    sig = 1e5 * rng.standard_normal(M)
    u = np.concatenate([v, th, np.zeros(M), sig, np.zeros(N)])
    du = m.rhs_flat(u)
    assert m.error_word() == 0
    # the mantle rows: [G12 | 0 | G22] x, emulated with the same block layout (npad columns of G12)
    npad = (N + 31) // 32 * 32
    deps = m.rhs_flat(u)[2 * N:2 * N + M]   # strain rates (FP64 in both paths)
    x = np.zeros(npad + M)
    x[:N] = v - pf.vpl
    x[npad:] = deps - np.repeat(pa.dϵ0, ne)
    G = np.zeros((M, npad + M))
    G[:, :N], G[:, npad:] = gfs[1], gfs[3]
    y = _emulate_rows(G, x, mode)
    got = du[2 * N + M:2 * N + 2 * M]
    bound = 2e-5 * (np.abs(G) @ np.abs(x)) + 1e-30
    assert np.all(np.abs(got - y) <= bound), np.max(np.abs(got - y) / bound)


@pytest.mark.parametrize("mode,u16", [(1, 2.0 ** -8), (2, 2.0 ** -11)])
def test_mixed_rhs_error_bound_vs_fp64_oracle(oracle, mode, u16):
    mf, ma, gfs, pf, pa = _setup(oracle, seed=9)
    m = _model(mf, ma, gfs, pf, pa, mode)
    N, ne = mf.nx * mf.nξ, ma.ne
    M = 6 * ne
    rng = np.random.default_rng(4)
    v = 1e-9 * np.exp(rng.uniform(-2, 8, N))
    th = 0.012 / 1e-9 * np.exp(rng.uniform(-3, 1, N))
    sig = 1e5 * rng.standard_normal(M)
    u = np.concatenate([v, th, np.zeros(M), sig, np.zeros(N)])
    du = m.rhs_flat(u)
    ref = oracle.OracleModel(gfs[0], pf, *gfs[1:], pa).ode(u)
    deps = ref[2 * N:2 * N + M]
    x = np.concatenate([v - pf.vpl, deps])
    Gm = np.hstack([gfs[1], gfs[3]])
    bound = 1.05 * (u16 + 2.0 ** -23) * (np.abs(Gm) @ np.abs(x)) + 1e-300
    err = np.abs(du[2 * N + M:2 * N + 2 * M] - ref[2 * N + M:2 * N + 2 * M])
    assert np.all(err <= bound), np.max(err / bound)
    np.testing.assert_array_equal(du[2 * N:2 * N + M], deps)          # strain rates stay FP64
    np.testing.assert_array_equal(du[2 * N + 2 * M:], ref[2 * N + 2 * M:])  # dδ = v


def test_mixed_fault_only_uses_fp32_toeplitz(oracle):
    from oetqf_gb300.equation import GB300Model
    mf = gen_mesh("RectOkada", 40e3, 8e3, 1e3, 1e3, 90.0)
    mu = 3e10
    gf = oracle.gf_ff(mf, mu, mu, fourier=True)
    o = np.ones((mf.nx, mf.nξ))
    pf = RateStateQuasiDynamicProperty(0.015 * o, 0.019 * o, 0.012 * o, 5e7 * o, mu / (2 * 3044.0), 1e-9, 0.6, 1e-6)
    m = GB300Model(mf.nx, mf.nξ, 0)
    m.set_gf(1, gf)
    m.set_fault_props(pf)
    m.set_precision(1)
    N = mf.nx * mf.nξ
    rng = np.random.default_rng(1)
    u = np.concatenate([1e-9 * np.exp(rng.uniform(0, 6, N)), 0.012 / 1e-9 * np.exp(rng.uniform(-2, 0, N)), np.zeros(N)])
    du = m.rhs_flat(u)
    ref = oracle.OracleModel(gf, pf).ode(u)
    dtau_ref = oracle.OracleModel(gf, pf).dtau_dt(u[:N])
    scale = np.abs(oracle.gf_ff(mf, mu, mu)).sum() * np.abs(u[:N] - 1e-9).max()
    # dv depends on dτ linearly through 1/(dμ/dv + η); FP32 accumulation error on dτ <= 1e-5 scale
    a = np.abs(du[:N] - ref[:N])
    assert np.all(a <= 1e-5 * scale / pf.η + 1e-9 * np.abs(ref[:N]))
    np.testing.assert_allclose(du[N:2 * N], ref[N:2 * N], rtol=1e-14)
    assert dtau_ref.shape == (N,)


@pytest.mark.parametrize("mode", [1, 2])
def test_log_theta_integration_tracks_fp64(oracle, mode):
    """Integrate 1 yr of loading from a perturbed state in FP64 and in the mixed path with ln θ:
    slip rates agree to the stated horizon error."""
    mf, ma, gfs, pf, pa = _setup(oracle, seed=11)
    N, ne = mf.nx * mf.nξ, ma.ne
    m64 = _model(mf, ma, gfs, pf, pa, 0)
    mm = _model(mf, ma, gfs, pf, pa, mode)
    mm.set_log_theta(True)
    rng = np.random.default_rng(5)
    th0 = pf.L.reshape(-1, order="F") / 1e-9 * (1 + 0.01 * rng.uniform(-1, 1, N))
    u0 = np.concatenate([np.full(N, 1e-9), th0, np.zeros(6 * ne), np.zeros(6 * ne), np.zeros(N)])
    T = 3.15e7
    u64, s64 = m64.integrate(u0, 0.0, T, reltol=1e-8, abstol=1e-10, dt=1e-3)
    umx, smx = mm.integrate(u0, 0.0, T, reltol=1e-8, abstol=1e-10, dt=1e-3)
    assert s64.status == 0 and smx.status == 0
    rel = np.abs(umx[:N] - u64[:N]).max() / np.abs(u64[:N]).max()
    assert rel < 1e-4, rel
    np.testing.assert_allclose(umx[N:2 * N], u64[N:2 * N], rtol=1e-4)
