"""Batched ensembles: many fault-only models of uneven size in one persistent launch."""
import numpy as np
import pytest

from oetqf_gb300.workloads import YEAR, fault_ensemble

pytestmark = pytest.mark.gpu


def _build(models, log_theta=True):
    from oetqf_gb300.ensemble import Ensemble
    e = Ensemble([(m.mf.nx, m.mf.nξ) for m in models])
    for i, m in enumerate(models):
        e.assemble(i, m.mf, m.lam, m.mu)
        e.set_fault_props(i, m.pf)
    e.set_log_theta(log_theta)
    u0 = np.zeros(e.state_len)
    for i, m in enumerate(models):
        u0[e.offsets[i]:e.offsets[i] + m.u0.size] = m.u0
    return e, u0


def test_ensemble_matches_fp64_oracle(oracle):
    models = fault_ensemble(n_models=6, n_range=(40, 300), seed=5)
    e, u0 = _build(models)
    T = 2 * YEAR
    u, st = e.integrate(u0, 0.0, T, reltol=1e-8, abstol=1e-10, dt=1e-3)
    assert all(s.status == 0 and s.t == T for s in st)
    for i, m in enumerate(models):
        gf = oracle.gf_ff(m.mf, m.lam, m.mu, fourier=True)
        uc, sc = oracle.OracleModel(gf, m.pf).integrate(m.u0, 0.0, T, reltol=1e-8, abstol=1e-10, dt0=1e-3)
        N = m.N
        ui = u[e.offsets[i]:e.offsets[i] + 3 * N]
        assert np.abs(ui[:N] - uc[:N]).max() / np.abs(uc[:N]).max() < 1e-4
        np.testing.assert_allclose(ui[N:2 * N], uc[N:2 * N], rtol=1e-4)


def test_alone_equals_in_the_mix():
    """A model integrated alone gives bitwise the same state as inside a batch of others."""
    models = fault_ensemble(n_models=8, n_range=(60, 400), seed=7)
    e, u0 = _build(models)
    T = 5 * YEAR
    u_mix, _ = e.integrate(u0, 0.0, T)
    for i in (0, 5):
        e1, u1 = _build([models[i]])
        ua, _ = e1.integrate(u1, 0.0, T)
        np.testing.assert_array_equal(ua, u_mix[e.offsets[i]:e.offsets[i] + 3 * models[i].N])


def test_per_model_horizons_and_blocks():
    models = fault_ensemble(n_models=5, n_range=(50, 250), seed=9)
    e, u0 = _build(models)
    t1 = np.array([0.5, 1.0, 2.0, 0.0, 3.0]) * YEAR
    outs = {}
    for b in (128, 256, 512):
        e.set_block(b)
        u, st = e.integrate(u0, 0.0, t1)
        assert [s.t for s in st] == list(t1)
        outs[b] = u
    np.testing.assert_array_equal(outs[128][e.offsets[3]:e.offsets[4]], u0[e.offsets[3]:e.offsets[4]])
    for b in (256, 512):  # the error norm is summed in a fixed order whatever the CTA size
        np.testing.assert_array_equal(outs[b], outs[128])


def test_cluster_split_models(oracle):
    """Models above 600 patches run on 2-8 CTA clusters; they agree with the one-CTA path and with
    the FP64 oracle."""
    models = fault_ensemble(n_models=3, n_range=(700, 700), seed=19) + fault_ensemble(n_models=1, n_range=(1300, 1300), seed=23) \
        + fault_ensemble(n_models=1, n_range=(2500, 2500), seed=29)
    T = 1 * YEAR
    e, u0 = _build(models)
    u8, st8 = e.integrate(u0, 0.0, T, reltol=1e-8, abstol=1e-10, dt=1e-3)
    e.set_max_cluster(1)
    u1, st1 = e.integrate(u0, 0.0, T, reltol=1e-8, abstol=1e-10, dt=1e-3)
    assert all(s.status == 0 for s in st8 + st1)
    np.testing.assert_array_equal(u8, u1)  # the trajectory does not depend on the cluster size
    for i in (0, 3):
        m = models[i]
        gf = oracle.gf_ff(m.mf, m.lam, m.mu, fourier=True)
        uc, _ = oracle.OracleModel(gf, m.pf).integrate(m.u0, 0.0, T, reltol=1e-8, abstol=1e-10, dt0=1e-3)
        N = m.N
        ui = u8[e.offsets[i]:e.offsets[i] + 3 * N]
        assert np.abs(ui[:N] - uc[:N]).max() / np.abs(uc[:N]).max() < 1e-4


def test_regrouping_keeps_trajectories():
    """Models with staggered horizons: as they finish, the rest move to larger clusters (2, 4, 8
    CTAs); every state is bitwise the same as without regrouping."""
    models = fault_ensemble(n_models=40, n_range=(100, 700), seed=31)
    e, u0 = _build(models)
    t1 = np.linspace(0.05, 1.5, len(models)) * YEAR
    e.set_regroup(False)
    ua, sa = e.integrate(u0, 0.0, t1)
    e.set_regroup(True)
    ub, sb = e.integrate(u0, 0.0, t1)
    assert [s.t for s in sb] == list(t1)
    assert [s.naccept for s in sa] == [s.naccept for s in sb]
    np.testing.assert_array_equal(ua, ub)


def test_vcabm5_ensemble(oracle):
    """VCABM5 inside the persistent launch: each member matches the oracle's VCABM5 (same method,
    FP32 convolution) and the state is bitwise independent of block size, cluster size and
    regrouping, as for Tsit5."""
    models = fault_ensemble(n_models=12, n_range=(100, 1300), seed=37)
    e, u0 = _build(models)
    T = 2 * YEAR
    t1 = np.linspace(0.3, 1.0, len(models)) * T
    u, st = e.integrate(u0, 0.0, t1, reltol=1e-8, abstol=1e-10, dt=1e-3, alg="VCABM5")
    assert all(s.status == 0 for s in st) and [s.t for s in st] == list(t1)
    assert all(s.nrhs == s.naccept + s.naccept + s.nreject + 1 for s in st)
    for i in (0, 5, 11):
        m = models[i]
        gf = oracle.gf_ff(m.mf, m.lam, m.mu, fourier=True)
        uc, sc = oracle.OracleModel(gf, m.pf).integrate(m.u0, 0.0, t1[i], reltol=1e-8, abstol=1e-10, dt0=1e-3,
                                                         alg="VCABM5")
        N = m.N
        ui = u[e.offsets[i]:e.offsets[i] + 3 * N]
        assert np.abs(ui[:N] - uc[:N]).max() / np.abs(uc[:N]).max() < 1e-4
    outs = []
    for block, maxc, rg in ((128, 1, False), (512, 8, True), (256, 2, True)):
        e.set_block(block)
        e.set_max_cluster(maxc)
        e.set_regroup(rg)
        outs.append(e.integrate(u0, 0.0, t1, reltol=1e-8, abstol=1e-10, dt=1e-3, alg="VCABM5")[0])
    np.testing.assert_array_equal(outs[0], u)
    np.testing.assert_array_equal(outs[1], u)
    np.testing.assert_array_equal(outs[2], u)
