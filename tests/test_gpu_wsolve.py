"""wsolve-style recorded histories (src/io.jl:22-133; test/tests.jl:1-42): record 0 is the initial
state, then every stride-th accepted step; the device recording matches the oracle's."""
import numpy as np
import pytest

from oetqf_gb300 import RateStateQuasiDynamicProperty, gen_mesh

pytestmark = pytest.mark.gpu


def _model(oracle):
    from oetqf_gb300.equation import GB300Model
    mf = gen_mesh("RectOkada", 8e3, 4e3, 1e3, 1e3, 90.0)
    mu = 3e10
    o = np.ones((mf.nx, mf.nξ))
    pf = RateStateQuasiDynamicProperty(0.015 * o, 0.019 * o, 0.012 * o, 5e7 * o, mu / (2 * 3044.0), 1e-9, 0.6, 1e-6)
    gf = oracle.gf_ff(mf, mu, mu, fourier=True)
    m = GB300Model(mf.nx, mf.nξ, 0)
    m.set_gf(1, gf)
    m.set_fault_props(pf)
    N = mf.nx * mf.nξ
    rng = np.random.default_rng(3)
    u = np.concatenate([np.full(N, 1e-9), 0.012 / 1e-9 * (1 + 0.01 * rng.uniform(-1, 1, N)), np.zeros(N)])
    return mf, gf, pf, m, u


@pytest.mark.parametrize("stride", [1, 3, 11])
def test_record_matches_oracle(oracle, stride):
    from oetqf_gb300.io import integrate_record
    mf, gf, pf, m, u = _model(oracle)
    T = 0.3 * 3.15e7
    kw = dict(reltol=1e-8, abstol=1e-10)
    u1, st, ts, us = integrate_record(m, u, 0.0, T, stride=stride, max_records=5000, dt=1e-3, **kw)
    uc, sc, tc, ucr = oracle.integrate_record(oracle.OracleModel(gf, pf), u, 0.0, T, stride, 5000, dt0=1e-3, **kw)
    assert st.status == 0 and sc.status == 0
    assert len(ts) == st.naccept // stride + 1          # test/tests.jl:190 semantics
    assert len(tc) == sc.naccept // stride + 1
    assert ts[0] == 0.0 and np.all(np.diff(ts) > 0)
    np.testing.assert_array_equal(us[0], u)
    # each record is the state a fresh device integration reaches at that time (same steps; the last
    # one is clamped to t1 - t, which can differ from the original dt in the last bit)
    for k in (1, len(ts) // 2, len(ts) - 1):
        uk, _ = m.integrate(u, 0.0, ts[k], dt=1e-3, **kw)
        np.testing.assert_allclose(uk, us[k], rtol=1e-13, atol=0)
    # the oracle's records agree to the integration tolerance (adaptive step sequences drift apart
    # by round-off in the cancelling error estimate, so times match only approximately)
    n = min(len(ts), len(tc))
    np.testing.assert_allclose(ts[:n], tc[:n], rtol=1e-3)
    np.testing.assert_allclose(us[:n], ucr[:n], rtol=1e-3, atol=1e-12 * np.abs(ucr).max())


def test_wsolve_file_and_append(oracle, tmp_path):
    from oetqf_gb300 import ArrayPartition
    from oetqf_gb300.equation import ODEProblem
    from oetqf_gb300.io import wsolve
    mf, gf, pf, m, u = _model(oracle)
    N = mf.nx * mf.nξ
    shape = (mf.nx, mf.nξ)
    u0 = ArrayPartition(u[:N].reshape(shape, order="F"), u[N:2 * N].reshape(shape, order="F"), u[2 * N:].reshape(shape, order="F"))
    getu = lambda u, t: (u.x[0], u.x[1], u.x[2])
    f = str(tmp_path / "out.npz")
    prob = ODEProblem(None, u0, (0.0, 0.1 * 3.15e7), m)
    ua, sta = wsolve(prob, f, 50, getu, ["v", "θ", "δ"], "t", stride=2)
    with np.load(f) as z:
        d = dict(z)
    assert d["v"].shape == (mf.nx, mf.nξ, len(d["t"]))
    assert len(d["t"]) == sta.naccept // 2 + 1
    prob2 = ODEProblem(None, ua, (0.15 * 3.15e7, 0.25 * 3.15e7), m)
    wsolve(prob2, f, 50, getu, ["v", "θ", "δ"], "t", stride=2, append=True)
    with np.load(f) as z:
        d2 = dict(z)
    assert len(d2["t"]) > len(d["t"]) and np.all(np.diff(d2["t"]) > 0)
    np.testing.assert_array_equal(d2["v"][..., :len(d["t"])], d["v"])
