"""Serving: continuous batching with HBM-budget admission; each result is the same alone and in
the mix (bitwise: every model's kernels and step control are independent of its neighbours)."""
import numpy as np
import pytest

from oetqf_gb300.workloads import YEAR, fault_ensemble, serving_requests

pytestmark = pytest.mark.gpu


def _mix():
    reqs = serving_requests(n_requests=6, seed=11, mantle_fraction=0.34, patch_range=(100, 600), cell_range=(8, 64),
                            year_range=(0.5, 2.0))
    assert any(r.ma is not None for r in reqs) and any(r.ma is None for r in reqs)
    return reqs


@pytest.mark.parametrize("alg", ["Tsit5", "VCABM5"])
def test_alone_equals_in_the_mix(alg):
    from oetqf_gb300.serving import Server, run_stream
    reqs = _mix()
    s = Server(hbm_budget_gb=8.0, alg=alg)
    out = run_stream(s, reqs, rate_per_s=50.0, seed=1)
    s.close()
    assert out["status"] == [0]
    for i in (0, 1, 2, 3, 4, 5):
        alone = Server(hbm_budget_gb=8.0, alg=alg)
        rid = alone.submit(reqs[i])
        u_alone, res = alone.wait(rid)
        alone.close()
        u_mix = out["results"][i][0]
        np.testing.assert_array_equal(u_alone, u_mix)
        assert res.stats.t == pytest.approx(reqs[i].horizon)


def test_budget_admission_limits_concurrency():
    from oetqf_gb300.serving import Server
    reqs = fault_ensemble(n_models=6, years=0.5, n_range=(300, 400), seed=13)
    budget_gb = 0.0004  # each request needs about 160 KB: two fit at a time
    s = Server(hbm_budget_gb=budget_gb)
    ids = [s.submit(r) for r in reqs]
    results = [s.wait(i) for i in ids]
    info = s.info()
    s.close()
    assert all(r.status == 0 for _, r in results)
    assert 0 < info.peak_bytes <= budget_gb * 2**30
    admits = sorted(r.admit_s for _, r in results)
    dones = sorted(r.done_s for _, r in results)
    assert admits[-1] >= dones[0]  # the last request waited for memory to free up


def test_server_matches_standalone_ensemble():
    from oetqf_gb300.ensemble import Ensemble
    from oetqf_gb300.serving import Server
    reqs = fault_ensemble(n_models=3, years=1.0, n_range=(80, 300), seed=17)
    s = Server(hbm_budget_gb=4.0)
    ids = [s.submit(r) for r in reqs]
    got = [s.wait(i)[0] for i in ids]
    s.close()
    e = Ensemble([(r.mf.nx, r.mf.nξ) for r in reqs])
    u0 = np.zeros(e.state_len)
    for i, r in enumerate(reqs):
        e.assemble(i, r.mf, r.lam, r.mu)
        e.set_fault_props(i, r.pf)
        u0[e.offsets[i]:e.offsets[i] + r.u0.size] = r.u0
    e.set_block(512)
    u, st = e.integrate(u0, 0.0, [r.horizon for r in reqs])
    for i, r in enumerate(reqs):
        np.testing.assert_array_equal(got[i], u[e.offsets[i]:e.offsets[i] + r.u0.size])


def _same_geometry(cm, scale):
    """The request cm with the same mesh and elastic constants, other friction and initial state."""
    import copy
    r = copy.deepcopy(cm)
    r.pf.a = r.pf.a * scale
    r.u0 = r.u0.copy()
    r.u0[:r.N] *= scale
    return r


def test_gf_cache_reuses_geometry_and_keeps_results():
    """Fault-only and mantle requests on one geometry: later requests hit the cache and give the
    bitwise result of a server that assembles every request itself."""
    from oetqf_gb300.serving import Server
    base = fault_ensemble(n_models=1, years=0.5, n_range=(200, 300), seed=19)[0]
    mant = serving_requests(n_requests=8, seed=23, mantle_fraction=1.0, patch_range=(100, 200), cell_range=(8, 27),
                            year_range=(0.2, 0.4))[0]
    assert mant.ma is not None
    reqs = [base, _same_geometry(base, 1.01), _same_geometry(base, 0.99), mant, _same_geometry(mant, 1.02)]
    out = {}
    for cache in (True, False):
        s = Server(hbm_budget_gb=8.0)
        s.set_gf_cache(cache)
        got = []
        for r in reqs:  # one at a time: a mantle model is reused only when idle
            got.append(s.wait(s.submit(r))[0])
        info = s.info()
        s.close()
        out[cache] = (got, info)
    got_c, info_c = out[True]
    got_n, info_n = out[False]
    for a, b in zip(got_c, got_n):
        np.testing.assert_array_equal(a, b)
    assert (info_c.cache_hits, info_c.cache_misses) == (3, 2)
    assert info_c.cache_entries == 2 and info_c.cache_bytes > 0
    assert info_n.cache_hits == 0 and info_n.cache_entries == 0


def test_gf_cache_evicts_idle_geometries_under_budget():
    from oetqf_gb300.serving import Server
    reqs = fault_ensemble(n_models=4, years=0.2, n_range=(300, 400), seed=29)
    budget = 0.00025  # 268 KB: a request (156-171 KB) and one or two idle geometries (54-57 KB each)
    s = Server(hbm_budget_gb=budget)
    for r in reqs:
        u, res = s.wait(s.submit(r))
        assert res.status == 0
    info = s.info()
    s.close()
    assert info.peak_bytes <= budget * 2**30
    assert info.cache_hits + info.cache_misses == 4
    assert info.cache_entries < info.cache_misses  # an idle geometry was evicted to admit a later one


def _fault_bytes(cm):
    """The server's charge for a fault-only request: its own buffers and its geometry's spectra."""
    nx, nxi = cm.mf.nx, cm.mf.nξ
    N, P = nx * nxi, 2
    while P < 2 * nx - 1:
        P *= 2
    own = 8 * 37 * N + 4096
    gf = 8 * (nx * nxi * nxi + 3 * nx + 4 * nxi) + 4 * nxi * nxi * (P // 2 + 1) + 512
    return own, gf


def test_waiting_request_does_not_empty_the_cache():
    """A head request that cannot fit even with every idle geometry evicted must evict nothing: a
    later request on a cached geometry, admitted around it, is a cache hit."""
    import dataclasses
    from oetqf_gb300.serving import Server
    ms = fault_ensemble(n_models=6, years=0.05, n_range=(300, 420), seed=29)
    ms = sorted(ms, key=lambda m: m.mf.nx)
    a, b, c = ms[0], ms[2], ms[-1]  # 31 x 10, 36 x 10 and 41 x 10 patches
    # steps of at most an hour: b (2 years, >= 17,520 steps) is still running while c and d arrive
    b = dataclasses.replace(b, horizon=2 * YEAR)
    own_a, gf_a = _fault_bytes(a)
    own_b, gf_b = _fault_bytes(b)
    own_c, gf_c = _fault_bytes(c)
    budget = own_b + gf_b + own_c + gf_c - 1024  # b and c never run together
    assert gf_a + own_b + gf_b + own_a <= budget  # a's geometry stays cached beside b, and d fits
    s = Server(hbm_budget_gb=budget / 2**30, dtmax=3600.0)
    _, ra = s.wait(s.submit(a))
    ib, ic, idd = s.submit(b), s.submit(c), s.submit(dataclasses.replace(a))
    rb, rc, rd = [s.wait(i)[1] for i in (ib, ic, idd)]
    info = s.info()
    s.close()
    assert all(r.status == 0 for r in (ra, rb, rc, rd))
    assert rd.admit_s < rc.admit_s and rc.admit_s >= rb.done_s  # c waited for b; d went around it
    assert (info.cache_hits, info.cache_misses) == (1, 3)
