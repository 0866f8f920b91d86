"""The C-ABI library without a GPU: it builds, loads, exports every symbol include/gbcycle.h
declares, and fails loudly (no CPU fallback) when no device is present."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, "include", "gbcycle.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(gbc_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_the_boundary():
    names = _declared()
    for n in ("gbc_stress_gf_ff", "gbc_stress_gf_fm", "gbc_stress_gf_mf", "gbc_stress_gf_mm", "gbc_model_create",
              "gbc_rhs", "gbc_rhs_dev", "gbc_integrate", "gbc_last_error"):
        assert n in names


def test_library_exports_every_declared_symbol():
    from oetqf_gb300 import _capi as C
    L = C.lib()
    for n in _declared():
        assert hasattr(L, n), n


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="checks the no-GPU error path")
def test_no_cpu_fallback_without_gpu():
    from oetqf_gb300 import _capi as C
    h = ctypes.c_void_p()
    rc = C.lib().gbc_model_create(4, 2, 0, ctypes.byref(h))
    assert rc == -2 and not h.value
    assert "no CUDA device" in C.last_error()
    from oetqf_gb300 import gen_mesh, stress_greens_function
    with pytest.raises(C.GbcError):
        stress_greens_function(gen_mesh("RectOkada", 4.0, 2.0, 1.0, 1.0, 90.0), 1.0, 1.0)


def test_invalid_arguments_rejected_before_device_use():
    from oetqf_gb300 import _capi as C
    h = ctypes.c_void_p()
    assert C.lib().gbc_model_create(0, 2, 0, ctypes.byref(h)) == -1
    assert C.lib().gbc_model_create(2, 2, -1, ctypes.byref(h)) == -1


def test_failure_injection_hook_checks_its_mode_before_any_device_use():
    from oetqf_gb300 import _capi as C
    assert C.lib().gbc_debug_pipeline_fault(7) == -1
    assert "mode" in C.last_error()


def test_julia_binding_calls_only_declared_symbols():
    """The Julia glue (no Julia toolchain here) binds only entry points the header declares and the
    library exports."""
    from oetqf_gb300 import _capi as C
    src = open(os.path.join(ROOT, "oetqf.jl_gb300", "julia", "OetqfGB300.jl")).read()
    called = set(re.findall(r"ccall\(\(:(gbc_[a-z0-9_]+), libgbc\)", src))
    assert {"gbc_rhs", "gbc_integrate", "gbc_sweep_integrate", "gbc_ensemble_integrate"} <= called
    declared = set(_declared())
    L = C.lib()
    for n in called:
        assert n in declared, n
        assert hasattr(L, n), n


_NULL_CALLS = r'''
import ctypes, sys
sys.path[:0] = [sys.argv[1]]
from oetqf_gb300 import _capi as C
from oetqf_gb300 import serving
L = C.lib()
serving._sigs()
zero = {ctypes.c_int: 0, ctypes.c_longlong: 0, ctypes.c_size_t: 0, ctypes.c_long: 0, ctypes.c_double: 0.0,
        ctypes.c_float: 0.0}
for name in sys.argv[2:]:
    f = getattr(L, name)
    if f.argtypes is None:
        continue
    print(name, flush=True)
    f(*[zero.get(a) for a in f.argtypes])
print("done", flush=True)
'''


def test_every_entry_point_survives_null_and_zero_arguments():
    """Each declared entry point called with null pointers and zero sizes returns (an error code, or
    nothing for the destroy functions) instead of crashing: arguments are checked before use. Host
    only: where a GPU is present the calls could reach device work, so the probe does not run."""
    if _has_gpu():
        pytest.skip("host-only probe of the argument checks")
    import subprocess
    import sys
    names = _declared()
    p = subprocess.run([sys.executable, "-c", _NULL_CALLS, os.path.join(ROOT, "oetqf.jl_gb300"), *names],
                       capture_output=True, text=True, timeout=300)
    lines = p.stdout.split()
    assert p.returncode == 0 and lines[-1] == "done", f"crashed after {lines[-1:]}: {p.stderr[-500:]}"
