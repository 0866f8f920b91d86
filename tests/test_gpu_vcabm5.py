"""VCABM5 on the device (the reference example's integrator, examples/otf-with-mantle.jl:160-162)
against the oracle's restatement of the same method, and against Tsit5 at solver tolerance."""
import numpy as np
import pytest

from oetqf_gb300 import PowerLawViscosityProperty, RateStateQuasiDynamicProperty, gen_hex8_box, gen_mesh
from oetqf_gb300.workloads import YEAR, strike_slip_fault

pytestmark = pytest.mark.gpu


def _fault_model(cm, gf):
    from oetqf_gb300.equation import GB300Model
    m = GB300Model(cm.mf.nx, cm.mf.nξ, 0)
    m.set_gf(1, gf)
    m.set_fault_props(cm.pf)
    return m


def test_vcabm5_matches_oracle_method(oracle):
    """Same method, same steps: the device and the oracle accept and reject the same steps over a
    year of loading, and the states agree to round-off amplified by the step sequence."""
    cm = strike_slip_fault(length=40e3, depth=8e3, cell=1e3, years=1.0)
    gf = oracle.gf_ff(cm.mf, cm.lam, cm.mu, fourier=True)
    m = _fault_model(cm, gf)
    T = 1.0 * YEAR
    opts = dict(reltol=1e-8, abstol=1e-10)
    ug, sg = m.integrate(cm.u0, 0.0, T, dt=1e-3, alg="VCABM5", **opts)
    uc, sc = oracle.OracleModel(gf, cm.pf).integrate(cm.u0, 0.0, T, dt0=1e-3, alg="VCABM5", **opts)
    assert sg.status == 0 and sc.status == 0 and sg.t == T
    assert abs(sg.naccept - sc.naccept) <= 2 and abs(sg.nreject - sc.nreject) <= 2
    assert sg.nrhs == 2 * sg.naccept + sg.nreject + 1
    N = cm.N
    np.testing.assert_allclose(ug[:N], uc[:N], rtol=1e-7)
    np.testing.assert_allclose(ug[N:], uc[N:], rtol=1e-9)


def test_vcabm5_through_events_matches_tsit5(oracle):
    """50 years of the 80-km fault: VCABM5 and Tsit5 on the device see the same earthquakes."""
    from oetqf_gb300.io import integrate_record
    cm = strike_slip_fault(years=50.0)
    gf = oracle.gf_ff(cm.mf, cm.lam, cm.mu, fourier=True)
    m = _fault_model(cm, gf)
    N = cm.N
    onsets = {}
    for alg in ("Tsit5", "VCABM5"):
        u, st, ts, us = integrate_record(m, cm.u0, 0.0, 50 * YEAR, stride=1, max_records=200000, dt=1e-8,
                                         dtmax=0.2 * YEAR, alg=alg)
        assert st.status == 0
        vmax = us[:, :N].max(axis=1)
        onsets[alg] = ts[1:][(vmax[1:] > 1e-3) & (vmax[:-1] <= 1e-3)] / YEAR
        if alg == "VCABM5":
            assert st.nrhs < 0.6 * nrhs_tsit5  # PECE: two evaluations per step instead of six
        else:
            nrhs_tsit5 = st.nrhs
    assert len(onsets["Tsit5"]) == len(onsets["VCABM5"]) >= 5
    np.testing.assert_allclose(onsets["VCABM5"], onsets["Tsit5"], atol=0.02)


def _visco(oracle):
    mf = gen_mesh("RectOkada", 70e3, 6e3, 2e3, 1e3, 90.0)
    ma = gen_hex8_box(-35e3, -6e3, -8e3, 70e3, 12e3, -12e3, 3, 3, 3)
    mu = 3e10
    gfs = [oracle.gf_ff(mf, mu, mu, fourier=True), oracle.gf_fm(mf, ma, mu, mu), oracle.gf_mf(ma, mf, mu, mu),
           oracle.gf_mm(ma, mu, mu)]
    rng = np.random.default_rng(11)
    o = np.ones((mf.nx, mf.nξ))
    pf = RateStateQuasiDynamicProperty(0.015 * o, 0.019 * o, 0.012 * (1 + rng.random((mf.nx, mf.nξ))), 5e7 * o,
                                       mu / (2 * 3044.0), 1e-9, 0.6, 1e-6)
    pa = PowerLawViscosityProperty(np.full(ma.ne, 5e-20), np.zeros(ma.ne), np.zeros(6))
    N, ne = mf.nx * mf.nξ, ma.ne
    th0 = pf.L.reshape(-1, order="F") / 1e-9 * (1 + 0.01 * rng.uniform(-1, 1, N))
    u0 = np.concatenate([np.full(N, 1e-9), th0, np.zeros(6 * ne), np.zeros(6 * ne), np.zeros(N)])
    return mf, ma, gfs, pf, pa, u0


def _visco_model(mf, ma, gfs, pf, pa, mode):
    from oetqf_gb300.equation import GB300Model
    m = GB300Model(mf.nx, mf.nξ, ma.ne)
    for w, g in zip((1, 2, 3, 4), gfs):
        m.set_gf(w, g)
    m.set_fault_props(pf)
    m.set_mantle_props(pa)
    m.set_precision(mode)
    return m


def test_vcabm5_viscoelastic_and_mixed(oracle):
    """With a Maxwell mantle: VCABM5 (FP64) agrees with Tsit5 (FP64) at solver tolerance, and the
    block-scaled BF16 path with ln θ under VCABM5 stays within the mixed-precision bar."""
    mf, ma, gfs, pf, pa, u0 = _visco(oracle)
    N = mf.nx * mf.nξ
    T = 3.15e7
    opts = dict(reltol=1e-8, abstol=1e-10, dt=1e-3)
    u_t, s_t = _visco_model(mf, ma, gfs, pf, pa, 0).integrate(u0, 0.0, T, alg="Tsit5", **opts)
    u_a, s_a = _visco_model(mf, ma, gfs, pf, pa, 0).integrate(u0, 0.0, T, alg="VCABM5", **opts)
    mb = _visco_model(mf, ma, gfs, pf, pa, 1)
    mb.set_log_theta(True)
    u_b, s_b = mb.integrate(u0, 0.0, T, alg="VCABM5", **opts)
    assert s_t.status == 0 and s_a.status == 0 and s_b.status == 0
    assert np.abs(u_a[:N] - u_t[:N]).max() / np.abs(u_t[:N]).max() < 1e-6
    assert np.abs(u_b[:N] - u_t[:N]).max() / np.abs(u_t[:N]).max() < 1e-4
    # the oracle's VCABM5 on the same inputs (FP64 reference arithmetic)
    u_c, s_c = oracle.OracleModel(gfs[0], pf, *gfs[1:], pa).integrate(u0, 0.0, T, reltol=1e-8, abstol=1e-10,
                                                                       dt0=1e-3, alg="VCABM5")
    assert np.abs(u_a[:N] - u_c[:N]).max() / np.abs(u_c[:N]).max() < 1e-7
