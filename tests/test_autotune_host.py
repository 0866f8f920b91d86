"""The host autotuners on CPU: the ensemble's CTA size (Ensemble.autotune) and the sweep's product
engine (Sweep.autotune) keep the configuration whose timed runs were fastest and leave it set. The
library is replaced by a stand-in whose calls take a configuration-dependent time."""
import ctypes
import time

import numpy as np
import pytest


class _TimedLib:
    def __init__(self, cost):
        self.cost = cost          # {configuration value: seconds per call}
        self.current = None
        self.calls = []

    def __getattr__(self, name):
        def call(*args):
            self.calls.append((name, args))
            if name in ("gbc_ensemble_set_block", "gbc_sweep_set_engine"):
                self.current = args[1]
            if name in ("gbc_ensemble_integrate", "gbc_sweep_rhs"):
                time.sleep(self.cost[self.current])
            if name == "gbc_ensemble_state_offset":
                return 0
            if name in ("gbc_ensemble_state_len", "gbc_sweep_state_len"):
                return 4
            return 0
        return call


def test_ensemble_autotune_keeps_fastest_block(monkeypatch):
    from oetqf_gb300 import _capi as C
    from oetqf_gb300 import ensemble as E
    lib = _TimedLib({128: 0.004, 256: 0.001, 512: 0.003})
    monkeypatch.setattr(C, "lib", lambda: lib)
    e = E.Ensemble([(4, 2)])
    best, tim = e.autotune(np.zeros(4), steps=7, candidates=(128, 256, 512))
    assert best == 256 and e.block == 256 and set(tim) == {128, 256, 512}
    assert lib.calls[-1][0] == "gbc_ensemble_set_block" and lib.calls[-1][1][1] == 256
    # every candidate ran the same fixed step count (maxiters), not a horizon
    runs = [a for n, a in lib.calls if n == "gbc_ensemble_integrate"]
    assert len(runs) == 3 and all(a[4]._obj.maxiters == 7 for a in runs)
    e.h = ctypes.c_void_p()  # no destroy through the stand-in


def test_sweep_autotune_keeps_fastest_engine(monkeypatch):
    from oetqf_gb300 import _capi as C
    from oetqf_gb300 import sweep as S

    class Base:
        h, N, ne, nlaws = ctypes.c_void_p(7), 1, 0, 1

    lib = _TimedLib({S.ENGINES["umma"]: 0.001, S.ENGINES["simt"]: 0.004})
    monkeypatch.setattr(C, "lib", lambda: lib)
    sw = S.Sweep(Base(), 2)
    best, tim = sw.autotune(np.zeros((2, 4)), reps=3)
    assert best == "umma" and sw.engine == "umma" and tim["umma"] < tim["simt"]
    lib.cost = {S.ENGINES["umma"]: 0.004, S.ENGINES["simt"]: 0.001}
    best, _ = sw.autotune(np.zeros((2, 4)), reps=3)
    assert best == "simt" and sw.engine == "simt" and lib.current == S.ENGINES["simt"]
