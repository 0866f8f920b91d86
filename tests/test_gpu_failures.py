"""Failure detection without a GPU fault.

* A bounded pipeline wait that runs out: the failure-injection hook makes the 16-bit GEMV's
  producer issue no copies, so no barrier phase completes and every wait gives up (after a short,
  fixed number of polls). The right-hand side returns, the model's error word reads nonzero, and
  once the hook is off and the word cleared the next right-hand side equals a clean one bit for bit.
* A member whose initial state holds a NaN (injected on the host): the ensemble retires it with a
  failed status while every other member's result is bitwise the result of a clean run; the same
  for a serving request among clean ones.
The reference documents a return code for failed solves (src/io.jl:96-97)."""
import numpy as np
import pytest

from oetqf_gb300 import PowerLawViscosityProperty, RateStateQuasiDynamicProperty, gen_hex8_box, gen_mesh
from oetqf_gb300.workloads import YEAR, fault_ensemble

pytestmark = pytest.mark.gpu
SOLVER = dict(reltol=1e-6, abstol=1e-8, dt=1e-8, dtmax=0.2 * YEAR)


def _bf16_model(oracle):
    from oetqf_gb300 import _capi as C
    from oetqf_gb300.equation import GB300Model
    mf = gen_mesh("RectOkada", 60e3, 6e3, 2e3, 1e3, 90.0)
    ma = gen_hex8_box(-30e3, -6e3, -8e3, 60e3, 12e3, -12e3, 4, 3, 3)
    mu = 3e10
    m = GB300Model(mf.nx, mf.nξ, ma.ne)
    m.assemble_gf(mf, ma, mu, mu)
    o = np.ones((mf.nx, mf.nξ))
    m.set_fault_props(RateStateQuasiDynamicProperty(0.015 * o, 0.019 * o, 0.012 * o, 5e7 * o, mu / (2 * 3044.0),
                                                    1e-9, 0.6, 1e-6))
    m.set_mantle_props(PowerLawViscosityProperty(np.full(ma.ne, 5e-20), np.zeros(ma.ne), np.zeros(6)))
    m.set_precision(C.GBC_PREC_BF16)
    N, M = mf.nx * mf.nξ, 6 * ma.ne
    rng = np.random.default_rng(5)
    u = np.concatenate([1e-9 * np.exp(rng.uniform(-1, 3, N)), 0.012 / 1e-9 * np.exp(rng.uniform(-1, 1, N)),
                        np.zeros(M), 1e6 * rng.standard_normal(M), np.zeros(N)])
    return m, u


def test_pipeline_wait_runs_out_and_the_next_call_succeeds(oracle):
    from oetqf_gb300 import _capi as C
    m, u = _bf16_model(oracle)
    clean = m.rhs_flat(u)
    assert m.error_word() == 0
    C.check(C.lib().gbc_debug_pipeline_fault(1))
    try:
        m.rhs_flat(u)  # returns: every wait of the GEMV pipeline gives up
        assert m.error_word() == 1
    finally:
        C.check(C.lib().gbc_debug_pipeline_fault(0))
    m.clear_error_word()
    again = m.rhs_flat(u)
    assert m.error_word() == 0
    np.testing.assert_array_equal(again, clean)
    m.close()


def _ensemble(models):
    from oetqf_gb300.ensemble import Ensemble
    e = Ensemble([(mm.mf.nx, mm.mf.nξ) for mm in models])
    for i, mm in enumerate(models):
        e.assemble(i, mm.mf, mm.lam, mm.mu)
        e.set_fault_props(i, mm.pf)
    u0 = np.zeros(e.state_len)
    for i, mm in enumerate(models):
        u0[e.offsets[i]:e.offsets[i] + mm.u0.size] = mm.u0
    return e, u0


@pytest.mark.parametrize("alg", ["VCABM5", "Tsit5"])
def test_ensemble_retires_a_nan_member_and_the_rest_match_a_clean_run(alg):
    models = fault_ensemble(n_models=6, years=0.5, n_range=(150, 900), seed=23)
    e, u0 = _ensemble(models)
    e.set_log_theta(alg != "VCABM5")
    clean, st_clean = e.integrate(u0, 0.0, 0.5 * YEAR, alg=alg, **SOLVER)
    assert all(s.status == 0 for s in st_clean)
    bad = 2
    ub = u0.copy()
    ub[e.offsets[bad] + 3] = np.nan  # one slip rate of member 2
    got, st = e.integrate(ub, 0.0, 0.5 * YEAR, alg=alg, **SOLVER)
    e.close()
    assert st[bad].status == -5 and st[bad].t < 0.5 * YEAR
    for i in range(len(models)):
        if i == bad:
            continue
        assert st[i].status == 0
        part = slice(e.offsets[i], e.offsets[i] + models[i].u0.size)
        np.testing.assert_array_equal(got[part], clean[part])
        assert st[i].naccept == st_clean[i].naccept and st[i].nreject == st_clean[i].nreject


def test_serving_fails_a_nan_request_alone():
    from oetqf_gb300.serving import Server
    reqs = fault_ensemble(n_models=4, years=0.5, n_range=(200, 500), seed=29)
    s = Server(hbm_budget_gb=4.0, alg="VCABM5")
    clean = [s.wait(s.submit(r)) for r in reqs]
    s.close()
    assert all(r.status == 0 for _, r in clean)
    import copy
    poisoned = copy.copy(reqs[1])
    poisoned.u0 = reqs[1].u0.copy()
    poisoned.u0[0] = np.nan
    s = Server(hbm_budget_gb=4.0, alg="VCABM5")
    ids = [s.submit(r) for r in (reqs[0], poisoned, reqs[2], reqs[3])]
    out = [s.wait(i) for i in ids]
    s.close()
    assert out[1][1].status != 0
    for k in (0, 2, 3):
        assert out[k][1].status == 0
        np.testing.assert_array_equal(out[k][0], clean[k][0])
