"""The ensemble's regrouping plan (host only): which cluster size each running model gets so that
every CTA of the grouping is resident at once. Occupancies are the ones a GB300 reports for the
ensemble kernel (one-CTA models at 256 threads two per SM; 512-thread clusters holding their
spectra in shared memory, whose large sizes are limited by the GPCs)."""
import numpy as np
import pytest

from oetqf_gb300.ensemble import Ensemble

CAP = [304, 76, 36, 15, 7]  # clusters of 1, 2, 4, 8 and 16 CTAs resident at once


def _load(sizes, done, cap=CAP):
    idx = np.log2(sizes).astype(int)
    return sum(1.0 / cap[g] for g, d in zip(idx, done) if not d)


def test_every_grouping_is_resident():
    rng = np.random.default_rng(1)
    for n in (1, 2, 7, 9, 14, 40, 152, 256):
        N = rng.integers(200, 2001, n)
        done = np.zeros(n, np.int32)
        w = Ensemble.plan_clusters(N, done, rng.random(n) * 1e6, CAP)
        assert set(np.unique(w)) <= {1, 2, 4, 8, 16}
        assert _load(w, done) <= 1.0 + 1e-9


def test_the_last_model_takes_sixteen_ctas():
    w = Ensemble.plan_clusters([1540], [0], [1e5], CAP)
    assert list(w) == [16]


def test_small_models_stop_where_larger_clusters_no_longer_pay():
    # 400 patches: one CTA ~50 us a step, eight ~26 us, sixteen no faster
    w = Ensemble.plan_clusters([400], [0], [1e5], CAP)
    assert list(w) == [8]


def test_finished_models_take_nothing():
    w = Ensemble.plan_clusters([1500, 1500, 1500], [1, 0, 1], [0.0, 1e4, 0.0], CAP)
    assert list(w) == [1, 16, 1]


def test_the_stiff_tail_fits_without_a_second_wave():
    # fourteen long-running models of 640 to 1960 patches: nine 16-CTA clusters and five 8-CTA
    # clusters (152 SMs by count) would need two waves; the plan stays within the occupancy
    N = np.array([1540, 1960, 1580, 1520, 1560, 1380, 1620, 1310, 1630, 640, 1190, 690, 640, 670])
    w = Ensemble.plan_clusters(N, np.zeros(14, np.int32), np.full(14, 1e6), CAP)
    assert _load(w, np.zeros(14)) <= 1.0 + 1e-9
    assert (w >= 4).all()
    assert (w == 16).sum() <= 7
    # the largest model is never on a smaller cluster than a smaller one
    assert w[1] == w.max()


def test_sixteen_cta_clusters_unavailable():
    w = Ensemble.plan_clusters([1540, 1960], [0, 0], [1e5, 1e5], [304, 76, 36, 15, 0])
    assert list(w) == [8, 8]


def test_ties_go_to_the_models_with_more_steps_left():
    # eight equal models: all reach eight CTAs (8/15 of the GPU), then six of them fit sixteen; the
    # two with the fewest steps left stay on eight
    left = np.array([5e3, 9e5, 1e3, 7e5, 8e5, 6e5, 4e5, 3e5])
    w = Ensemble.plan_clusters(np.full(8, 1500), np.zeros(8, np.int32), left, CAP)
    assert list(w) == [8, 16, 8, 16, 16, 16, 16, 16]


def test_many_models_stay_on_one_cta():
    # 304 running models fill the one-CTA slots: nobody moves up
    w = Ensemble.plan_clusters(np.full(304, 2000), np.zeros(304, np.int32), np.ones(304), CAP)
    assert (w == 1).all()


def test_invalid_capacity_rejected():
    with pytest.raises(Exception):
        Ensemble.plan_clusters([1000], [0], [1.0], [304, -1, 36, 15, 7])
    with pytest.raises(ValueError):
        Ensemble.plan_clusters([1000], [0], [1.0], [304, 76])


def test_plan_entry_point_checks_its_arguments():
    import ctypes
    from oetqf_gb300 import _capi as C
    L = C.lib()
    ip = ctypes.POINTER(ctypes.c_int)
    null_i = ctypes.cast(None, ip)
    null_d = ctypes.cast(None, ctypes.POINTER(ctypes.c_double))
    assert L.gbc_ensemble_plan_clusters(-1, null_i, null_i, null_d, null_i, null_i) < 0
    assert L.gbc_ensemble_plan_clusters(2, null_i, null_i, null_d, null_i, null_i) < 0
    assert L.gbc_ensemble_plan_clusters(0, null_i, null_i, null_d, null_i, null_i) < 0  # no capacities
    cap = (ctypes.c_int * 5)(304, 76, 36, 15, 7)
    assert L.gbc_ensemble_plan_clusters(0, null_i, null_i, null_d, cap, null_i) == 0  # nothing to plan
