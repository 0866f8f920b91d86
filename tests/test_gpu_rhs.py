"""GPU right-hand side and integrator against the oracle, through the C ABI."""
import numpy as np
import pytest

from oetqf_gb300 import (PowerLawViscosityProperty, RateStateQuasiDynamicProperty, gen_hex8_box, gen_mesh)

pytestmark = pytest.mark.gpu
RTOL = 1e-6


def _rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


def _fault(oracle, mesh=(10.0, 10.0, 2.0, 2.0, 90.0), seed=0):
    mf = gen_mesh("RectOkada", *mesh)
    gf = oracle.gf_ff(mf, 1.0, 1.0, buffer_ratio=1.0, fourier=True)
    rng = np.random.default_rng(seed)
    p = RateStateQuasiDynamicProperty(*[rng.random((mf.nx, mf.nξ)) for _ in range(4)], *rng.random(4))
    return mf, gf, p


def test_fft_conv_equals_dense_toeplitz_gpu(oracle):
    """test/BEM/tests.jl:39-61 on the GPU: the complex kernel goes in, the traction rate of the
    dense Toeplitz contraction comes out (read through dv with a = b = 0-free friction)."""
    from oetqf_gb300.equation import GB300Model
    mf = gen_mesh("RectOkada", 100.0, 100.0, 10.0, 10.0, 41.0)
    gf1 = oracle.gf_ff(mf, 3e10, 3e10, fourier=True)
    gf2 = oracle.gf_ff(mf, 3e10, 3e10, fourier=False)
    m = GB300Model(mf.nx, mf.nξ, 0)
    m.set_gf(1, gf1)
    st = m.export_gf(0)
    np.testing.assert_allclose(st, gf2, rtol=1e-9, atol=1e-9 * np.abs(gf2).max())


@pytest.mark.parametrize("mesh", [(10.0, 10.0, 2.0, 2.0, 90.0), (80e3, 10e3, 1e3, 1e3, 90.0), (9.0, 5.0, 1.0, 1.0, 60.0), (7.0, 1.0, 1.0, 1.0, 90.0)])
def test_rhs_fault_only(oracle, mesh):
    from oetqf_gb300 import ArrayPartition, assemble
    mf, gf, p = _fault(oracle, mesh)
    N = mf.nx * mf.nξ
    rng = np.random.default_rng(1)
    u0 = ArrayPartition(*[rng.random((mf.nx, mf.nξ)) for _ in range(3)])
    prob = assemble(gf, p, u0, (0.0, 1.0))
    du = u0.similar()
    prob.f(du, u0, prob.p, 1.0)
    ref = oracle.OracleModel(gf, p).ode(u0.flat())
    got = du.flat()
    for a, b in ((got[:N], ref[:N]), (got[N:2 * N], ref[N:2 * N]), (got[2 * N:], ref[2 * N:])):
        np.testing.assert_allclose(a, b, rtol=RTOL, atol=1e-12 * np.abs(b).max())


def _visco(oracle, seed=2):
    mf = gen_mesh("RectOkada", 100.0, 100.0, 10.0, 20.0, 90.0)
    ma = gen_hex8_box(-100.0, -50.0, -20.0, 200.0, 100.0, -30.0, 2, 3, 4)
    lam = mu = 1.0
    gfs = (oracle.gf_ff(mf, lam, mu, fourier=True), oracle.gf_fm(mf, ma, lam, mu), oracle.gf_mf(ma, mf, lam, mu),
           oracle.gf_mm(ma, lam, mu))
    rng = np.random.default_rng(seed)
    N, ne = mf.nx * mf.nξ, ma.ne
    pf = RateStateQuasiDynamicProperty(*[rng.random((mf.nx, mf.nξ)) for _ in range(4)], *rng.random(4))
    pa = PowerLawViscosityProperty(rng.random(ne), 3 * np.ones(ne), rng.random(6))
    return mf, ma, gfs, pf, pa


def test_rhs_viscoelastic(oracle):
    """test/BEM/tests.jl:84-110 with values: every ArrayPartition component against the oracle."""
    from oetqf_gb300 import ArrayPartition, assemble
    mf, ma, gfs, pf, pa = _visco(oracle)
    N, ne = mf.nx * mf.nξ, ma.ne
    rng = np.random.default_rng(3)
    u0 = ArrayPartition(rng.random((mf.nx, mf.nξ)), rng.random((mf.nx, mf.nξ)), rng.random((ne, 6)),
                        rng.random((ne, 6)), rng.random((mf.nx, mf.nξ)))
    prob = assemble(*gfs, pf, pa, u0, (0.0, 1.0))
    du = u0.similar()
    prob.f(du, u0, prob.p, 1.0)
    ref = oracle.OracleModel(gfs[0], pf, *gfs[1:], pa).ode(u0.flat())
    got = du.flat()
    bounds = np.cumsum([0, N, N, 6 * ne, 6 * ne, N])
    for k in range(5):
        a, b = got[bounds[k]:bounds[k + 1]], ref[bounds[k]:bounds[k + 1]]
        np.testing.assert_allclose(a, b, rtol=RTOL, atol=1e-12 * np.abs(b).max())


def test_device_assembly_matches_host_upload(oracle):
    from oetqf_gb300 import _capi as C
    from oetqf_gb300.equation import GB300Model
    mf, ma, gfs, pf, pa = _visco(oracle)
    m = GB300Model(mf.nx, mf.nξ, ma.ne)
    m.assemble_gf(mf, ma, 1.0, 1.0)
    for which, ref in ((C.GBC_GF12, gfs[1]), (C.GBC_GF21, gfs[2]), (C.GBC_GF22, gfs[3])):
        got = m.export_gf(which)
        np.testing.assert_allclose(got, ref, rtol=RTOL, atol=1e-12 * np.abs(ref).max())
    np.testing.assert_allclose(m.export_gf(C.GBC_GF11_REAL), oracle.gf_ff(mf, 1.0, 1.0), rtol=RTOL)


def test_rhs_dev_with_torch(oracle):
    torch = pytest.importorskip("torch")
    from oetqf_gb300.equation import GB300Model
    mf, ma, gfs, pf, pa = _visco(oracle)
    m = GB300Model(mf.nx, mf.nξ, ma.ne)
    m.assemble_gf(mf, ma, 1.0, 1.0)
    m.set_fault_props(pf)
    m.set_mantle_props(pa)
    rng = np.random.default_rng(4)
    u = rng.random(m.state_len)
    ut = torch.tensor(u, device="cuda:0")
    dut = torch.zeros_like(ut)
    torch.cuda.synchronize()
    m.rhs_dev(ut.data_ptr(), dut.data_ptr())
    ref = m.rhs_flat(u)
    torch.cuda.synchronize()
    import ctypes  # the dev call runs on the model stream: read back after a host RHS synchronised it
    got = dut.cpu().numpy()
    np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-14 * np.abs(ref).max())


def test_missing_state_is_an_error(oracle):
    from oetqf_gb300 import _capi as C
    from oetqf_gb300.equation import GB300Model
    m = GB300Model(4, 2, 0)
    with pytest.raises(C.GbcError) as e:
        m.rhs_flat(np.ones(24))
    assert e.value.code == -6


def _c0_like(oracle, nx_km=16.0):
    mf = gen_mesh("RectOkada", nx_km * 1e3, 4e3, 1e3, 1e3, 90.0)
    mu = 3e10
    N = mf.nx * mf.nξ
    depth = -np.tile(mf.z, (mf.nx, 1))
    a = np.where((depth >= 2e3) & (depth <= 8e3), 0.015, 0.025) * np.ones((mf.nx, mf.nξ))
    p = RateStateQuasiDynamicProperty(a, 0.019 * np.ones_like(a), 0.012 * np.ones_like(a), 5e7 * np.ones_like(a),
                                      mu / (2 * 3044.0), 1e-9, 0.6, 1e-9)
    gf = oracle.gf_ff(mf, mu, mu, fourier=True)
    rng = np.random.default_rng(5)
    u = np.concatenate([np.full(N, 1e-9), 0.012 / 1e-9 * (1 + 0.01 * rng.uniform(-1, 1, N)), np.zeros(N)])
    return mf, gf, p, u


def test_integrate_fault_only_matches_oracle(oracle):
    from oetqf_gb300.equation import GB300Model
    mf, gf, p, u = _c0_like(oracle)
    m = GB300Model(mf.nx, mf.nξ, 0)
    m.set_gf(1, gf)
    m.set_fault_props(p)
    T = 2 * 3.15e7
    u1, st = m.integrate(u, 0.0, T, reltol=1e-8, abstol=1e-12, dt=1e-3)
    assert st.status == 0 and st.t == T
    uc, sc = oracle.OracleModel(gf, p).integrate(u, 0.0, T, reltol=1e-8, abstol=1e-12, dt0=1e-3)
    assert abs(st.naccept - sc.naccept) <= 2
    assert _rel(u1, uc) < 1e-6


def test_integrate_viscoelastic_matches_oracle(oracle):
    from oetqf_gb300 import ArrayPartition
    from oetqf_gb300.equation import GB300Model
    mf = gen_mesh("RectOkada", 8e3, 4e3, 1e3, 1e3, 90.0)
    ma = gen_hex8_box(-8e3, -4e3, -6e3, 16e3, 8e3, -8e3, 4, 2, 2)
    mu = 3e10
    N, ne = mf.nx * mf.nξ, ma.ne
    o = np.ones((mf.nx, mf.nξ))
    pf = RateStateQuasiDynamicProperty(0.015 * o, 0.011 * o, 0.012 * o, 5e7 * o, mu / (2 * 3044.0), 1e-9, 0.6, 1e-9)
    pa = PowerLawViscosityProperty(np.full(ne, 1 / (2 * 1e19)), np.zeros(ne), np.zeros(6))
    m = GB300Model(mf.nx, mf.nξ, ne)
    m.assemble_gf(mf, ma, mu, mu)
    m.set_fault_props(pf)
    m.set_mantle_props(pa)
    gfs = [m.export_gf(w) for w in (1, 2, 3, 4)]
    om = oracle.OracleModel(gfs[0], pf, gfs[1], gfs[2], gfs[3], pa)
    u = np.concatenate([np.full(N, 1e-9), np.full(N, 0.012 / 1e-9), np.zeros(6 * ne), np.zeros(6 * ne), np.zeros(N)])
    T = 3.15e7
    u1, st = m.integrate(u, 0.0, T, reltol=1e-8, abstol=1e-10, dt=1e-3)
    uc, sc = om.integrate(u, 0.0, T, reltol=1e-8, abstol=1e-10, dt0=1e-3)
    assert st.status == 0
    assert _rel(u1, uc) < 1e-6


def test_rhs_dilatancy(oracle):
    """assemble(gf, p, dila, u0, tspan) (equation.jl:108-117) and its ode (:168-183) vs the oracle."""
    from oetqf_gb300 import ArrayPartition, DilatancyProperty, assemble
    mf, gf, p = _fault(oracle, seed=8)
    rng = np.random.default_rng(9)
    sh = (mf.nx, mf.nξ)
    dila = DilatancyProperty(*[rng.random(sh) for _ in range(4)])
    u0 = ArrayPartition(*[rng.random(sh) for _ in range(4)])
    prob = assemble(gf, p, dila, u0, (0.0, 1.0))
    du = u0.similar()
    prob.f(du, u0, prob.p, 1.0)
    ref = oracle.OracleModel(gf, p, dila=dila).ode(u0.flat())
    np.testing.assert_allclose(du.flat(), ref, rtol=RTOL, atol=1e-12 * np.abs(ref).max())


def test_integrate_dilatancy_matches_oracle(oracle):
    from oetqf_gb300 import DilatancyProperty
    from oetqf_gb300.equation import GB300Model
    mf = gen_mesh("RectOkada", 8e3, 4e3, 1e3, 1e3, 90.0)
    mu = 3e10
    N = mf.nx * mf.nξ
    o = np.ones((mf.nx, mf.nξ))
    pf = RateStateQuasiDynamicProperty(0.015 * o, 0.019 * o, 0.012 * o, 5e7 * o, mu / (2 * 3044.0), 1e-9, 0.6, 1e-6)
    dila = DilatancyProperty(1e5 * o, 1e-4 * o, 1e-9 * o, 1e7 * o)
    gf = oracle.gf_ff(mf, mu, mu, fourier=True)
    m = GB300Model(mf.nx, mf.nξ, 0)
    m.set_gf(1, gf)
    m.set_fault_props(pf)
    m.set_dilatancy(dila)
    rng = np.random.default_rng(2)
    u = np.concatenate([np.full(N, 1e-9), 0.012 / 1e-9 * (1 + 0.01 * rng.uniform(-1, 1, N)), np.zeros(N), np.full(N, 1e7)])
    T = 0.1 * 3.15e7
    u1, st = m.integrate(u, 0.0, T, reltol=1e-8, abstol=1e-10, dt=1e-3)
    uc, sc = oracle.OracleModel(gf, pf, dila=dila).integrate(u, 0.0, T, reltol=1e-8, abstol=1e-10, dt0=1e-3)
    assert st.status == 0 and sc.status == 0
    assert _rel(u1, uc) < 1e-6


@pytest.mark.parametrize("mode", [0, 1])
def test_rhs_composite_viscosity(oracle, mode):
    """CompositePowerLawViscosityProperty (property.jl:43-48, equation.jl:286-292) in FP64 and BF16."""
    from oetqf_gb300 import CompositePowerLawViscosityProperty
    from oetqf_gb300.equation import GB300Model
    mf, ma, gfs, pf, pa = _visco(oracle, seed=12)
    N, ne = mf.nx * mf.nξ, ma.ne
    rng = np.random.default_rng(13)
    laws = [PowerLawViscosityProperty(rng.random(ne), k * np.ones(ne), np.zeros(6)) for k in (0, 2)]
    pc = CompositePowerLawViscosityProperty(laws, rng.random(6))
    m = GB300Model(mf.nx, mf.nξ, ne)
    for w, g in zip((1, 2, 3, 4), gfs):
        m.set_gf(w, g)
    m.set_fault_props(pf)
    m.set_mantle_props(pc)
    m.set_precision(mode)
    u = rng.random(m.state_len)
    du = m.rhs_flat(u)
    ref = oracle.OracleModel(gfs[0], pf, *gfs[1:], pc).ode(u)
    np.testing.assert_allclose(du[2 * N:2 * N + 6 * ne], ref[2 * N:2 * N + 6 * ne], rtol=1e-12)
    if mode == 0:  # random friction inputs can overflow exp(); both sides must agree on those entries too
        np.testing.assert_allclose(du, ref, rtol=RTOL, atol=1e-12 * np.nanmax(np.abs(ref)), equal_nan=True)
