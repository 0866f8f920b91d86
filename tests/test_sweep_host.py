"""The Python side of gbc_sweep on CPU: argument checks before any library call, the law-major
flattening of composite viscosities, the (variants, state) shapes and the solver options handed to
the C ABI. The library is replaced by a recording stand-in (no device)."""
import ctypes

import numpy as np
import pytest

from oetqf_gb300 import (CompositePowerLawViscosityProperty, PowerLawViscosityProperty,
                         RateStateQuasiDynamicProperty)


class _Lib:
    """Records the calls the wrapper makes and answers like the library would."""

    def __init__(self, state_len):
        self.calls = []
        self.state_len = state_len

    def __getattr__(self, name):
        def call(*args):
            self.calls.append((name, args))
            # gbc_sweep_create leaves the handle null, so that a later __del__ (after the stand-in is
            # gone) never hands a fake handle to the real library
            if name == "gbc_sweep_state_len":
                return self.state_len
            if name in ("gbc_sweep_rhs",):
                u = np.ctypeslib.as_array(args[1], shape=(self._k * self.state_len,))
                du = np.ctypeslib.as_array(args[2], shape=(self._k * self.state_len,))
                du[:] = 2.0 * u
            if name == "gbc_sweep_integrate":
                st = args[5]
                for k in range(self._k):
                    st[k].naccept, st[k].t = 10 + k, args[3]
            return 0
        return call


class _Base:
    def __init__(self, nx, nxi, ne, nlaws=1):
        self.h = ctypes.c_void_p(99)
        self.nx, self.nξ, self.ne, self.N, self.nlaws = nx, nxi, ne, nx * nxi, nlaws


@pytest.fixture
def fake(monkeypatch):
    from oetqf_gb300 import _capi as C
    from oetqf_gb300 import sweep as S
    lib = _Lib(state_len=3 * 6 + 12 * 4)
    monkeypatch.setattr(C, "lib", lambda: lib)
    monkeypatch.setattr(S.C, "lib", lambda: lib)
    return lib, S


def _pf(nx, nxi, s=1.0):
    o = np.ones((nx, nxi))
    return RateStateQuasiDynamicProperty(0.015 * o, 0.019 * o, 0.012 * o, 5e7 * s * o, 4.9e6, 1e-9, 0.6, 1e-6)


def test_create_engine_and_shapes(fake):
    lib, S = fake
    lib._k = 3
    sw = S.Sweep(_Base(3, 2, 4), 3)
    assert sw.engine == "umma" and sw.state_len == 3 * 6 + 12 * 4
    assert ("gbc_sweep_set_engine", (sw.h, S.ENGINES["umma"])) in [(n, a) for n, a in lib.calls]
    sw.set_engine("simt")
    assert lib.calls[-1][1][1] == S.ENGINES["simt"] == 0
    U = np.arange(3 * sw.state_len, dtype=float)
    DU = sw.rhs(U)
    assert DU.shape == (3, sw.state_len)
    np.testing.assert_array_equal(DU.ravel(), 2 * U)


def test_property_checks_before_the_library(fake):
    lib, S = fake
    lib._k = 2
    base = _Base(3, 2, 4)
    sw = S.Sweep(base, 2)
    n0 = len(lib.calls)
    with pytest.raises(ValueError):
        sw.set_fault_props(0, _pf(4, 2))                  # 8 patches, the base has 6
    with pytest.raises(ValueError):
        sw.set_mantle_props(1, PowerLawViscosityProperty(np.ones(5), np.zeros(5), np.zeros(6)))
    assert len(lib.calls) == n0                           # nothing reached the C ABI
    sw.set_fault_props(1, _pf(3, 2, 2.0))
    name, args = lib.calls[-1]
    assert name == "gbc_sweep_set_fault_props" and args[1] == 1 and args[6:] == (4.9e6, 1e-9, 0.6, 1e-6)
    sig = np.ctypeslib.as_array(args[5], shape=(6,))
    np.testing.assert_array_equal(sig, np.full(6, 1e8))


def test_composite_laws_flattened_law_major(fake):
    lib, S = fake
    lib._k = 1
    base = _Base(3, 2, 4, nlaws=2)
    sw = S.Sweep(base, 1)
    p = CompositePowerLawViscosityProperty([PowerLawViscosityProperty(np.arange(4.0), np.zeros(4), np.zeros(6)),
                                            PowerLawViscosityProperty(10 + np.arange(4.0), np.ones(4), np.zeros(6))],
                                           np.array([1.0, 2, 3, 4, 5, 6]))
    sw.set_mantle_props(0, p)
    name, args = lib.calls[-1]
    gam = np.ctypeslib.as_array(args[2], shape=(8,))
    nn = np.ctypeslib.as_array(args[3], shape=(8,))
    d0 = np.ctypeslib.as_array(args[4], shape=(6,))
    np.testing.assert_array_equal(gam, [0, 1, 2, 3, 10, 11, 12, 13])
    np.testing.assert_array_equal(nn, [0, 0, 0, 0, 1, 1, 1, 1])
    np.testing.assert_array_equal(d0, [1, 2, 3, 4, 5, 6])
    with pytest.raises(ValueError):  # one law where the base has two
        sw.set_mantle_props(0, PowerLawViscosityProperty(np.ones(4), np.zeros(4), np.zeros(6)))


def test_integrate_passes_options_and_returns_stats(fake):
    lib, S = fake
    lib._k = 2
    sw = S.Sweep(_Base(3, 2, 4), 2)
    U0 = np.zeros((2, sw.state_len))
    U1, st = sw.integrate(U0, 0.0, 5.0, reltol=1e-7, dtmax=np.inf, alg="Tsit5")
    name, args = lib.calls[-1]
    assert name == "gbc_sweep_integrate" and args[2:4] == (0.0, 5.0)
    o = args[4]._obj
    assert o.reltol == 1e-7 and o.dtmax == 1e300 and o.alg == 0
    assert [s.naccept for s in st] == [10, 11] and st[1].t == 5.0
    assert U1.shape == (2, sw.state_len)
