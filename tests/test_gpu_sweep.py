"""Parameter sweeps on one geometry (gbc_sweep_*) against the single-model BF16 path.

The SIMT engine sums every variant in the single model's order, so each variant's right-hand side
and trajectory must equal a single model with that variant's properties bit for bit, while the
variants differ in friction, viscosity, initial state and step sequence."""
import numpy as np
import pytest

from oetqf_gb300 import PowerLawViscosityProperty, RateStateQuasiDynamicProperty, gen_hex8_box, gen_mesh

pytestmark = pytest.mark.gpu


def _geometry(oracle):
    mf = gen_mesh("RectOkada", 70e3, 6e3, 2e3, 1e3, 90.0)           # 35 x 6 = 210 patches
    ma = gen_hex8_box(-35e3, -6e3, -8e3, 70e3, 12e3, -12e3, 3, 3, 3)  # 27 cells
    mu = 3e10
    gfs = [oracle.gf_ff(mf, mu, mu, fourier=True), oracle.gf_fm(mf, ma, mu, mu), oracle.gf_mf(ma, mf, mu, mu),
           oracle.gf_mm(ma, mu, mu)]
    return mf, ma, gfs, mu


def _variant(mf, ma, mu, k, nonlinear=False):
    rng = np.random.default_rng(100 + k)
    o = np.ones((mf.nx, mf.nξ))
    pf = RateStateQuasiDynamicProperty((0.012 + 0.001 * k) * o, 0.019 * o, 0.012 * (1 + rng.random((mf.nx, mf.nξ))),
                                       (4e7 + 5e6 * k) * o, mu / (2 * 3044.0), 1e-9 * (1 + 0.1 * k), 0.6, 1e-6)
    n = float(k % 2) if nonlinear else 0.0
    gam = 5e-20 * (1 + 0.5 * k) / (1e5 ** n)
    pa = PowerLawViscosityProperty(np.full(ma.ne, gam), np.full(ma.ne, n), np.array([1e-16 * k, 0, 0, 0, 0, 0]))
    return pf, pa


def _state(mf, ma, pf, k, stressed=True):
    rng = np.random.default_rng(200 + k)
    N, M = mf.nx * mf.nξ, 6 * ma.ne
    v = 1e-9 * np.exp(rng.uniform(-2, 4, N)) if stressed else np.full(N, 1e-9)
    th = pf.L.reshape(-1, order="F") / 1e-9 * np.exp(rng.uniform(-1, 1, N) if stressed else 0.01 * rng.uniform(-1, 1, N))
    sig = 1e5 * rng.standard_normal(M) if stressed else np.zeros(M)
    return np.concatenate([v, th, np.zeros(M), sig, np.zeros(N)])


def _single(mf, ma, gfs, pf, pa):
    from oetqf_gb300 import _capi as C
    from oetqf_gb300.equation import GB300Model
    m = GB300Model(mf.nx, mf.nξ, ma.ne)
    for w, g in zip((1, 2, 3, 4), gfs):
        m.set_gf(w, g)
    m.set_fault_props(pf)
    m.set_mantle_props(pa)
    m.set_precision(C.GBC_PREC_BF16)
    return m


def _sweep(base, props, engine):
    from oetqf_gb300.sweep import Sweep
    sw = Sweep(base, len(props), engine=engine)
    for k, (pf, pa) in enumerate(props):
        sw.set_fault_props(k, pf)
        sw.set_mantle_props(k, pa)
    return sw


@pytest.mark.parametrize("K", [1, 5, 11])
def test_simt_rhs_equals_single_model(oracle, K):
    mf, ma, gfs, mu = _geometry(oracle)
    props = [_variant(mf, ma, mu, k, nonlinear=True) for k in range(K)]
    base = _single(mf, ma, gfs, *props[0])
    sw = _sweep(base, props, "simt")
    U = np.stack([_state(mf, ma, pf, k) for k, (pf, _) in enumerate(props)])
    DU = sw.rhs(U)
    assert sw.error_word() == 0
    for k, (pf, pa) in enumerate(props):
        ref = _single(mf, ma, gfs, pf, pa).rhs_flat(U[k])
        np.testing.assert_array_equal(DU[k], ref)


@pytest.mark.parametrize("alg", ["Tsit5", "VCABM5"])
def test_simt_integrate_equals_single_model(oracle, alg):
    """Every variant keeps its own step sequence (different properties, different steps) and ends
    bit for bit where a single model with its properties ends."""
    mf, ma, gfs, mu = _geometry(oracle)
    K = 3
    props = [_variant(mf, ma, mu, k) for k in range(K)]
    base = _single(mf, ma, gfs, *props[0])
    sw = _sweep(base, props, "simt")
    U0 = np.stack([_state(mf, ma, pf, k, stressed=False) for k, (pf, _) in enumerate(props)])
    T = 3.15e7
    opts = dict(reltol=1e-6, abstol=1e-8, dt=1e-3, alg=alg)
    U1, st = sw.integrate(U0, 0.0, T, **opts)
    assert sw.error_word() == 0
    steps = []
    for k, (pf, pa) in enumerate(props):
        u1, s1 = _single(mf, ma, gfs, pf, pa).integrate(U0[k], 0.0, T, **opts)
        assert st[k].status == 0 and s1.status == 0 and st[k].t == T
        assert (st[k].naccept, st[k].nreject, st[k].nrhs) == (s1.naccept, s1.nreject, s1.nrhs)
        np.testing.assert_array_equal(U1[k], u1)
        steps.append(st[k].naccept + st[k].nreject)
    assert len(set(steps)) > 1  # the variants really took different step sequences


def test_sweep_rejects_unsupported_bases(oracle):
    from oetqf_gb300 import _capi as C
    from oetqf_gb300.sweep import Sweep
    mf, ma, gfs, mu = _geometry(oracle)
    pf, pa = _variant(mf, ma, mu, 0)
    m = _single(mf, ma, gfs, pf, pa)
    for bad in (0, 65):
        with pytest.raises(C.GbcError):
            Sweep(m, bad)
    m.set_precision(C.GBC_PREC_F64)
    with pytest.raises(C.GbcError, match="BF16"):
        Sweep(m, 2)
    m.set_precision(C.GBC_PREC_BF16)
    sw = Sweep(m, 2, engine="simt")
    with pytest.raises(ValueError):
        sw.set_mantle_props(0, PowerLawViscosityProperty(np.ones(ma.ne + 1), np.zeros(ma.ne + 1), np.zeros(6)))
    # the base's Green's functions change: the sweep refuses to run on stale rows
    m.set_gf(4, gfs[3])
    with pytest.raises(C.GbcError, match="create the sweep again"):
        sw.rhs(np.zeros((2, sw.state_len)))
