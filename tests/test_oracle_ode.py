"""The oracle's right-hand side and integrator against the reference's tests
(test/BEM/tests.jl:63-110, :142-154) and published-method identities."""
import numpy as np
import pytest

from oetqf_gb300.mesh import gen_hex8_box, gen_mesh
from oetqf_gb300.property import PowerLawViscosityProperty, RateStateQuasiDynamicProperty, dϵ_dt


def test_viscosity_law():
    """test/BEM/tests.jl:142-149."""
    rng = np.random.default_rng(0)
    A, n, σ, τ = rng.random(4)
    p = PowerLawViscosityProperty([A], [n], rng.random(6))
    assert dϵ_dt(p, 0, σ, τ) == A * σ * τ ** n


def test_tsit5_order_conditions(oracle):
    a, e = oracle.tsit5_tableau()
    A = np.zeros((7, 7))
    for s in range(1, 7):
        A[s, :s] = a[s, :s]
    c = A.sum(axis=1)
    b = A[6]
    for k in range(5):
        assert b @ c**k == pytest.approx(1 / (k + 1), abs=1e-13)
    assert b @ A @ c == pytest.approx(1 / 6, abs=1e-13)
    assert b @ A @ A @ c == pytest.approx(1 / 24, abs=1e-13)
    assert (b * c) @ A @ c == pytest.approx(1 / 8, abs=1e-13)
    bh = b - e
    for k in range(4):
        assert bh @ c**k == pytest.approx(1 / (k + 1), abs=1e-13)
    assert e.sum() == pytest.approx(0.0, abs=1e-15)


def _fault_model(oracle, seed=0, mesh=(10.0, 10.0, 2.0, 2.0, 90.0), buffer_ratio=1.0):
    mf = gen_mesh("RectOkada", *mesh)
    gf = oracle.gf_ff(mf, 1.0, 1.0, buffer_ratio=buffer_ratio, fourier=True)
    rng = np.random.default_rng(seed)
    p = RateStateQuasiDynamicProperty(*[rng.random((mf.nx, mf.nξ)) for _ in range(4)], *rng.random(4))
    return mf, gf, p


def test_okada_assemble_runs(oracle):
    """test/BEM/tests.jl:63-71: the fault-only ode runs on random inputs."""
    mf, gf, p = _fault_model(oracle)
    m = oracle.OracleModel(gf, p)
    u0 = np.random.default_rng(1).random(3 * mf.nx * mf.nξ)
    du = m.ode(u0)
    assert du.shape == u0.shape and np.all(np.isfinite(du))
    np.testing.assert_array_equal(du[2 * mf.nx * mf.nξ:], u0[:mf.nx * mf.nξ])  # dδ = v


def test_viscoelastic_assemble_runs(oracle):
    """test/BEM/tests.jl:84-110 (gmsh box replaced by the structured box generator)."""
    mf = gen_mesh("RectOkada", 100.0, 100.0, 10.0, 20.0, 90.0)
    ma = gen_hex8_box(-100.0, -50.0, -20.0, 200.0, 100.0, -30.0, 2, 3, 4)
    lam = mu = 1.0
    gf11 = oracle.gf_ff(mf, lam, mu, fourier=True)
    gf12 = oracle.gf_fm(mf, ma, lam, mu)
    gf21 = oracle.gf_mf(ma, mf, lam, mu)
    gf22 = oracle.gf_mm(ma, lam, mu)
    rng = np.random.default_rng(2)
    N, ne = mf.nx * mf.nξ, ma.ne
    pf = RateStateQuasiDynamicProperty(*[rng.random((mf.nx, mf.nξ)) for _ in range(4)], *rng.random(4))
    pa = PowerLawViscosityProperty(rng.random(ne), 3 * np.ones(ne), rng.random(6))
    m = oracle.OracleModel(gf11, pf, gf12, gf21, gf22, pa)
    u0 = np.concatenate([rng.random(N), rng.random(N), rng.random(6 * ne), rng.random(6 * ne), rng.random(N)])
    du = m.ode(u0)
    assert du.shape == u0.shape and np.all(np.isfinite(du))
    # equation.jl:202-203 by hand
    sig = u0[2 * N + 6 * ne:2 * N + 12 * ne].reshape((ne, 6), order="F")
    skk = (sig[:, 0] + sig[:, 3] + sig[:, 5]) / 3
    dev = sig.copy()
    dev[:, [0, 3, 5]] -= skk[:, None]
    tau = np.sqrt(dev[:, 0]**2 + dev[:, 3]**2 + dev[:, 5]**2 + 2 * (dev[:, 1]**2 + dev[:, 2]**2 + dev[:, 4]**2))
    deps = pa.γ[:, None] * dev * tau[:, None] ** pa.n[:, None]
    np.testing.assert_allclose(du[2 * N:2 * N + 6 * ne], deps.reshape(-1, order="F"), rtol=1e-13)
    rel = (deps - pa.dϵ0[None, :]).reshape(-1, order="F")
    dsig = gf12 @ (u0[:N] - pf.vpl) + gf22 @ rel
    np.testing.assert_allclose(du[2 * N + 6 * ne:2 * N + 12 * ne], dsig, rtol=1e-10, atol=1e-12 * np.abs(dsig).max())


def test_friction_formula(oracle):
    """update_fault! (equation.jl:233-246) by hand on one model."""
    mf, gf, p = _fault_model(oracle, seed=5)
    m = oracle.OracleModel(gf, p)
    N = mf.nx * mf.nξ
    rng = np.random.default_rng(9)
    v, th = rng.random(N), rng.random(N)
    du = m.ode(np.concatenate([v, th, np.zeros(N)]))
    dtau = m.dtau_dt(v.reshape((mf.nx, mf.nξ), order="F"))
    a, b, L, s = (q.reshape(-1, order="F") for q in (p.a, p.b, p.L, p.σ))
    psi1 = np.exp((p.f0 + b * np.log(p.v0 * np.maximum(0, th) / L)) / a) / (2 * p.v0)
    psi2 = s * psi1 / np.hypot(1, v * psi1)
    dth = 1 - v * th / L
    dv = (dtau - b / th * v * psi2 * dth) / (a * psi2 + p.η)
    np.testing.assert_allclose(du[N:2 * N], dth, rtol=1e-14)
    np.testing.assert_allclose(du[:N], dv, rtol=1e-11)


def test_integrator_matches_scipy(oracle):
    """Tsit5 + PI control reproduces a tight scipy DOP853 solution of the same RHS."""
    scipy_integrate = pytest.importorskip("scipy.integrate")
    mf = gen_mesh("RectOkada", 8e3, 4e3, 1e3, 1e3, 90.0)
    mu = 3e10
    gf = oracle.gf_ff(mf, mu, mu, fourier=True)
    N = mf.nx * mf.nξ
    o = np.ones((mf.nx, mf.nξ))
    vpl = 1e-9
    p = RateStateQuasiDynamicProperty(0.015 * o, 0.019 * o, 0.012 * o, 5e7 * o, mu / (2 * 3044.0), vpl, 0.6, vpl)
    m = oracle.OracleModel(gf, p)
    th0 = 0.012 / vpl * (1 + 0.01 * np.linspace(-1, 1, N))
    u0 = np.concatenate([np.full(N, vpl), th0, np.zeros(N)])
    T = 3.15e7
    u1, st = m.integrate(u0, 0.0, T, reltol=1e-10, abstol=1e-14, dt0=1e-3)
    assert st.status == 0 and st.t == T
    ref = scipy_integrate.solve_ivp(lambda t, y: m.ode(y), (0.0, T), u0, method="DOP853", rtol=1e-12, atol=1e-16)
    np.testing.assert_allclose(u1, ref.y[:, -1], rtol=1e-7)


def test_composite_viscosity_law():
    """test/BEM/tests.jl:150-153."""
    from oetqf_gb300.property import CompositePowerLawViscosityProperty, dϵ_dt_composite
    rng = np.random.default_rng(1)
    A, n, σ, τ = rng.random(4)
    p = PowerLawViscosityProperty([A], [n], rng.random(6))
    A2, n2 = rng.random(2)
    p2 = PowerLawViscosityProperty([A2], [n2], rng.random(6))
    pc = CompositePowerLawViscosityProperty([p, p2], rng.random(6))
    assert dϵ_dt_composite(pc, 0, σ, τ) == A * σ * τ ** n + A2 * σ * τ ** n2


def test_okada_with_dilatancy_runs(oracle):
    """test/BEM/tests.jl:73-82 with values: update_fault_with_dilatancy! (equation.jl:248-276) by hand."""
    from oetqf_gb300.property import DilatancyProperty
    mf, gf, p = _fault_model(oracle, seed=3)
    rng = np.random.default_rng(4)
    sh = (mf.nx, mf.nξ)
    dila = DilatancyProperty(*[rng.random(sh) for _ in range(4)])
    m = oracle.OracleModel(gf, p, dila=dila)
    N = mf.nx * mf.nξ
    u = rng.random(4 * N)
    du = m.ode(u)
    assert np.all(np.isfinite(du))
    v, th, pp = u[:N], u[N:2 * N], u[3 * N:]
    f = lambda a: a.reshape(-1, order="F")
    a, b, L, s = f(p.a), f(p.b), f(p.L), f(p.σ)
    tp, ep, be, p0 = f(dila.tp), f(dila.ϵ), f(dila.β), f(dila.p0)
    dth = 1 - v * th / L
    dp = -(pp - p0) / tp + ep / be / th * dth
    af, bf = a / p.f0, b / p.f0
    vf, thf = np.maximum(0, v / p.v0), np.maximum(0, th * p.v0 / L)
    dtau = m.dtau_dt(v.reshape(sh, order="F"))
    dv = (dtau + p.f0 * dp * vf**af * thf**bf - p.f0 * (s - pp) * vf**af * thf**(bf - 1) * bf * p.v0 / L * dth) / \
         (p.f0 * (s - pp) * vf**(af - 1) * thf**bf * af / p.v0)
    np.testing.assert_allclose(du[N:2 * N], dth, rtol=1e-14)
    np.testing.assert_allclose(du[3 * N:], dp, rtol=1e-13)
    np.testing.assert_allclose(du[:N], dv, rtol=1e-10)
    np.testing.assert_array_equal(du[2 * N:3 * N], v)


def test_composite_viscoelastic_rhs(oracle):
    from oetqf_gb300.property import CompositePowerLawViscosityProperty
    mf = gen_mesh("RectOkada", 100.0, 100.0, 10.0, 20.0, 90.0)
    ma = gen_hex8_box(-100.0, -50.0, -20.0, 200.0, 100.0, -30.0, 2, 3, 4)
    gfs = (oracle.gf_ff(mf, 1.0, 1.0, fourier=True), oracle.gf_fm(mf, ma, 1.0, 1.0), oracle.gf_mf(ma, mf, 1.0, 1.0),
           oracle.gf_mm(ma, 1.0, 1.0))
    rng = np.random.default_rng(6)
    N, ne = mf.nx * mf.nξ, ma.ne
    pf = RateStateQuasiDynamicProperty(*[rng.random((mf.nx, mf.nξ)) for _ in range(4)], *rng.random(4))
    laws = [PowerLawViscosityProperty(rng.random(ne), k * np.ones(ne), np.zeros(6)) for k in (0, 2)]
    pc = CompositePowerLawViscosityProperty(laws, rng.random(6))
    u = rng.random(3 * N + 12 * ne)
    du = oracle.OracleModel(gfs[0], pf, *gfs[1:], pc).ode(u)
    sig = u[2 * N + 6 * ne:2 * N + 12 * ne].reshape((ne, 6), order="F")
    skk = (sig[:, 0] + sig[:, 3] + sig[:, 5]) / 3
    dev = sig.copy()
    dev[:, [0, 3, 5]] -= skk[:, None]
    tau = np.sqrt(dev[:, 0]**2 + dev[:, 3]**2 + dev[:, 5]**2 + 2 * (dev[:, 1]**2 + dev[:, 2]**2 + dev[:, 4]**2))
    f = sum(q.γ * tau ** q.n for q in laws)
    np.testing.assert_allclose(du[2 * N:2 * N + 6 * ne], (f[:, None] * dev).reshape(-1, order="F"), rtol=1e-13)


# ---- VCABM5 (the reference example's integrator, examples/otf-with-mantle.jl:160-162) -------------
def test_abm_weights_constant_step(oracle):
    """Equal steps: beta = 1 and g_j are the Adams-Bashforth backward-difference weights."""
    h = 0.37
    psi, beta, g = oracle.abm_coefficients(5, h, [h, 2 * h, 3 * h, 4 * h])
    np.testing.assert_allclose(psi, [h, 2 * h, 3 * h, 4 * h, 5 * h], rtol=1e-15)
    np.testing.assert_allclose(beta, np.ones(5), rtol=1e-15)
    np.testing.assert_allclose(g, [1, 1 / 2, 5 / 12, 3 / 8, 251 / 720, 95 / 288], rtol=1e-14)


def _divided(xs, fs):
    """Newton divided differences f[x0], f[x0,x1], ... of the points in the given order."""
    c = list(fs)
    out = [c[0]]
    for j in range(1, len(xs)):
        c = [(c[i + 1] - c[i]) / (xs[i + j] - xs[i]) for i in range(len(xs) - j)]
        out.append(c[0])
    return out


@pytest.mark.parametrize("k", [1, 2, 3, 4, 5])
def test_abm_variable_step_is_exact_on_polynomials(oracle, k):
    """With uneven history, the order-k predictor integrates polynomials of degree < k exactly over
    the step and the corrector those of degree <= k (Phi from divided differences, HNW III.5)."""
    rng = np.random.default_rng(k)
    xn = 2.0
    hist = xn - np.concatenate([[0.0], np.cumsum(rng.uniform(0.3, 1.2, k))])  # x_n, x_{n-1}, ...
    h = rng.uniform(0.2, 1.5)
    psi_prev = [xn - hist[i + 1] for i in range(k - 1)]
    psi, beta, g = oracle.abm_coefficients(k, h, psi_prev)
    for deg in range(k + 1):
        coef = rng.standard_normal(deg + 1)
        f = np.polynomial.Polynomial(coef)
        F = f.integ()
        dd = _divided(hist[:k], f(hist[:k]))
        phi = [np.prod(psi_prev[:j]) * dd[j] for j in range(k)]
        star = [beta[j] * phi[j] for j in range(k)]
        pred = h * sum(g[j] * star[j] for j in range(k))
        exact = F(xn + h) - F(xn)
        if deg < k:
            assert pred == pytest.approx(exact, rel=1e-11, abs=1e-11)
        phik = f(xn + h) - sum(star)
        corr = pred + h * g[k] * phik
        assert corr == pytest.approx(exact, rel=1e-10, abs=1e-10)


def test_vcabm5_matches_scipy(oracle):
    """VCABM5 at tight tolerance reproduces a tight scipy DOP853 solution of the same RHS."""
    scipy_integrate = pytest.importorskip("scipy.integrate")
    mf = gen_mesh("RectOkada", 8e3, 4e3, 1e3, 1e3, 90.0)
    mu = 3e10
    gf = oracle.gf_ff(mf, mu, mu, fourier=True)
    N = mf.nx * mf.nξ
    o = np.ones((mf.nx, mf.nξ))
    vpl = 1e-9
    p = RateStateQuasiDynamicProperty(0.015 * o, 0.019 * o, 0.012 * o, 5e7 * o, mu / (2 * 3044.0), vpl, 0.6, vpl)
    m = oracle.OracleModel(gf, p)
    th0 = 0.012 / vpl * (1 + 0.01 * np.linspace(-1, 1, N))
    u0 = np.concatenate([np.full(N, vpl), th0, np.zeros(N)])
    T = 3.15e7
    u1, st = m.integrate(u0, 0.0, T, reltol=1e-10, abstol=1e-14, dt0=1e-3, alg="VCABM5")
    assert st.status == 0 and st.t == T
    assert st.nrhs == 2 * st.naccept + st.nreject + 1  # PECE: two evaluations per accepted step
    ref = scipy_integrate.solve_ivp(lambda t, y: m.ode(y), (0.0, T), u0, method="DOP853", rtol=1e-12, atol=1e-16)
    np.testing.assert_allclose(u1, ref.y[:, -1], rtol=1e-7)


def test_vcabm5_viscoelastic_matches_scipy(oracle):
    """VCABM5 with a Maxwell mantle (state v, θ, ϵ, σ, δ) at tight tolerance against scipy DOP853."""
    scipy_integrate = pytest.importorskip("scipy.integrate")
    mf = gen_mesh("RectOkada", 8e3, 4e3, 1e3, 1e3, 90.0)
    ma = gen_hex8_box(-4e3, -4e3, -6e3, 8e3, 8e3, -6e3, 2, 2, 2)
    mu = 3e10
    gfs = (oracle.gf_ff(mf, mu, mu, fourier=True), oracle.gf_fm(mf, ma, mu, mu), oracle.gf_mf(ma, mf, mu, mu),
           oracle.gf_mm(ma, mu, mu))
    N, ne = mf.nx * mf.nξ, ma.ne
    o = np.ones((mf.nx, mf.nξ))
    vpl = 1e-9
    pf = RateStateQuasiDynamicProperty(0.015 * o, 0.019 * o, 0.012 * o, 5e7 * o, mu / (2 * 3044.0), vpl, 0.6, vpl)
    pa = PowerLawViscosityProperty(np.full(ne, 5e-20), np.zeros(ne), np.zeros(6))
    m = oracle.OracleModel(gfs[0], pf, *gfs[1:], pa)
    th0 = 0.012 / vpl * (1 + 0.01 * np.linspace(-1, 1, N))
    u0 = np.concatenate([np.full(N, vpl), th0, np.zeros(6 * ne), np.zeros(6 * ne), np.zeros(N)])
    T = 3.15e7
    u1, st = m.integrate(u0, 0.0, T, reltol=1e-10, abstol=1e-14, dt0=1e-3, alg="VCABM5")
    assert st.status == 0 and st.t == T
    ref = scipy_integrate.solve_ivp(lambda t, y: m.ode(y), (0.0, T), u0, method="DOP853", rtol=1e-12, atol=1e-16)
    np.testing.assert_allclose(u1[:N], ref.y[:N, -1], rtol=1e-7)
    np.testing.assert_allclose(u1[N:2 * N], ref.y[N:2 * N, -1], rtol=1e-7)
    np.testing.assert_allclose(u1[2 * N + 6 * ne:], ref.y[2 * N + 6 * ne:, -1], rtol=1e-6, atol=1e-6 * np.abs(ref.y[2 * N + 6 * ne:, -1]).max())


def test_fft_convolution_variant_equals_the_direct_transform(oracle):
    """The timed-baseline traction rate (radix-2 FFTs of length 2^k >= 2nx - 1) equals the
    checker's direct transforms of length 2nx - 1 (equation.jl:44-61) to round-off, for odd and
    even depth counts, and member-parallel integration changes nothing else."""
    from oetqf_gb300.workloads import YEAR, fault_ensemble
    ms = fault_ensemble(n_models=3, years=0.05, n_range=(60, 400), seed=41, nxi=7)
    oms = [oracle.OracleModel(oracle.gf_ff(m.mf, m.lam, m.mu, fourier=True), m.pf) for m in ms]
    rng = np.random.default_rng(3)
    for m, om in zip(ms, oms):
        v = m.pf.vpl * np.exp(rng.uniform(-2, 8, m.N))
        a, b = om.dtau_dt(v), oracle.dtau_dt_fft(om, v)
        assert np.abs(a - b).max() <= 1e-13 * np.abs(a).max()
    S = dict(reltol=1e-6, abstol=1e-8, dt0=1e-8, dtmax=0.2 * YEAR, alg="VCABM5")
    seq = [om.integrate(m.u0, 0.0, 0.05 * YEAR, **S) for m, om in zip(ms, oms)]
    par, st = oracle.integrate_many(oms, [m.u0 for m in ms], 0.0, 0.05 * YEAR, fft=False, threads=2, **S)
    for (u1, s1), u2, s2 in zip(seq, par, st):
        np.testing.assert_array_equal(u1, u2)
        assert s1.nrhs == s2.nrhs
    fast, st = oracle.integrate_many(oms, [m.u0 for m in ms], 0.0, 0.05 * YEAR, fft=True, threads=2, **S)
    for (u1, _), u2, s2 in zip(seq, fast, st):
        assert s2.status == 0
        assert np.abs(u1 - u2).max() <= 1e-9 * np.abs(u1).max()


def test_fft_convolution_variant_at_the_smallest_shapes(oracle):
    """The FFT variant at transform lengths 2 to 16 (nx = 1 to 4; one to five depth rows, odd and
    even) equals the direct transforms to round-off."""
    from oetqf_gb300 import RateStateQuasiDynamicProperty, gen_mesh
    for nx, nxi in [(1, 1), (1, 2), (2, 1), (2, 3), (3, 2), (4, 5)]:
        mf = gen_mesh("RectOkada", 1e3 * nx, 1e3 * nxi, 1e3, 1e3, 90.0)
        o = np.ones((nx, nxi))
        pf = RateStateQuasiDynamicProperty(0.015 * o, 0.019 * o, 0.012 * o, 5e7 * o, 4.9e6, 1e-9, 0.6, 1e-6)
        om = oracle.OracleModel(oracle.gf_ff(mf, 3e10, 3e10, fourier=True), pf)
        v = 1e-9 * np.exp(np.random.default_rng(nx * 7 + nxi).uniform(-2, 8, nx * nxi))
        a, b = om.dtau_dt(v), oracle.dtau_dt_fft(om, v)
        assert np.abs(a - b).max() <= 1e-14 * np.abs(a).max()
