"""The sweep's fault rows on the tensor cores (gbc_sweep_set_fault_product): the dense fault-fault
block as exact hi/mid/lo BF16 planes in the tcgen05 product, against the SIMT engine's FP32
Toeplitz rows (K = 1, 5, 20: the 3 x 16 and 3 x 32-column instantiations) and over a one-year
VCABM5 window against single models."""
import numpy as np
import pytest

from test_gpu_sweep import _geometry, _single, _state, _sweep, _variant

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("K", [1, 5, 20])
def test_fault_product_rhs_matches_simt(oracle, K):
    mf, ma, gfs, mu = _geometry(oracle)
    props = [_variant(mf, ma, mu, k % 7, nonlinear=True) for k in range(K)]
    base = _single(mf, ma, gfs, *props[0])
    U = np.stack([_state(mf, ma, pf, k) for k, (pf, _) in enumerate(props)])
    ref = _sweep(base, props, "simt").rhs(U)
    sw = _sweep(base, props, "umma")
    sw.set_fault_product(True)
    DU = sw.rhs(U)
    assert sw.error_word() == 0
    N = mf.nx * mf.nξ
    for k in range(K):
        dv = np.abs(DU[k, :N] - ref[k, :N]).max() / np.abs(ref[k, :N]).max()
        assert dv < 1e-5, (k, dv)
        np.testing.assert_array_equal(DU[k, N:2 * N], ref[k, N:2 * N])
        np.testing.assert_array_equal(DU[k, -N:], ref[k, -N:])  # dδ = v


def test_fault_product_integrate_close_to_single_models(oracle):
    mf, ma, gfs, mu = _geometry(oracle)
    K = 3
    props = [_variant(mf, ma, mu, k) for k in range(K)]
    base = _single(mf, ma, gfs, *props[0])
    sw = _sweep(base, props, "umma")
    sw.set_fault_product(True)
    U0 = np.stack([_state(mf, ma, pf, k, stressed=False) for k, (pf, _) in enumerate(props)])
    T = 3.15e7
    U1, st = sw.integrate(U0, 0.0, T, reltol=1e-6, abstol=1e-8, dt=1e-3, alg="VCABM5")
    N = mf.nx * mf.nξ
    for k, (pf, pa) in enumerate(props):
        u1, s1 = _single(mf, ma, gfs, pf, pa).integrate(U0[k], 0.0, T, reltol=1e-6, abstol=1e-8, dt=1e-3, alg="VCABM5")
        assert st[k].status == 0
        assert np.abs(U1[k, :N] - u1[:N]).max() / np.abs(u1[:N]).max() < 1e-4
