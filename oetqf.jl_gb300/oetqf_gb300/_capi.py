"""ctypes binding of libgbcycle.so (include/gbcycle.h). No CPU fallback: loading fails loudly when
the library is missing, and calls fail with GbcError when there is no GPU."""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

D = ctypes.c_double
PD = ctypes.POINTER(ctypes.c_double)
I = ctypes.c_int
LL = ctypes.c_longlong

GBC_STRIKE_SLIP, GBC_DIP_SLIP = 0, 1
GBC_PREC_F64, GBC_PREC_BF16, GBC_PREC_F16, GBC_PREC_DF64 = 0, 1, 2, 3
GBC_GF11_REAL, GBC_GF11_DFT, GBC_GF12, GBC_GF21, GBC_GF22 = 0, 1, 2, 3, 4
GBC_SWEEP_SIMT, GBC_SWEEP_UMMA = 0, 1
ERRORS = {-1: "EINVAL", -2: "ENODEV", -3: "ECUDA", -4: "ENOMEM", -5: "ESOLVER", -6: "ESTATE"}


class GbcError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"gbcycle {ERRORS.get(code, code)}: {msg}")
        self.code = code


class FaultMesh(ctypes.Structure):
    _fields_ = [("nx", I), ("nxi", I), ("x", PD), ("xi", PD), ("y", PD), ("z", PD), ("ax", PD), ("axi", PD),
                ("dx", D), ("dxi", D), ("dep", D), ("dip", D)]


class HexMesh(ctypes.Structure):
    _fields_ = [("ne", I)] + [(n, PD) for n in ("cx", "cy", "cz", "qx", "qy", "qz", "dx", "dy", "dz")]


class SolverOpts(ctypes.Structure):
    _fields_ = [("reltol", D), ("abstol", D), ("dt0", D), ("dtmax", D), ("dtmin", D), ("maxiters", LL), ("alg", I)]


GBC_ALG_TSIT5, GBC_ALG_VCABM5 = 0, 1
ALGS = {"Tsit5": GBC_ALG_TSIT5, "VCABM5": GBC_ALG_VCABM5}


class SolverStats(ctypes.Structure):
    _fields_ = [("naccept", LL), ("nreject", LL), ("nrhs", LL), ("t", D), ("dt", D), ("status", I)]


_lib = None


def lib():
    """Load libgbcycle.so (built in-tree on first use)."""
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        P = ctypes.c_void_p
        sig = {
            "gbc_stress_gf_ff": [ctypes.POINTER(FaultMesh), D, D, I, I, I, D, PD],
            "gbc_stress_gf_fm": [ctypes.POINTER(FaultMesh), ctypes.POINTER(HexMesh), D, D, I, PD, PD, I, I, D, PD],
            "gbc_stress_gf_mf": [ctypes.POINTER(HexMesh), ctypes.POINTER(FaultMesh), D, D, I, PD],
            "gbc_stress_gf_mm": [ctypes.POINTER(HexMesh), D, D, PD, PD, I, PD],
            "gbc_model_create": [I, I, I, ctypes.POINTER(P)],
            "gbc_model_set_fault_props": [P, PD, PD, PD, PD, D, D, D, D],
            "gbc_model_set_mantle_props": [P, PD, PD, PD],
            "gbc_model_set_mantle_props_composite": [P, I, PD, PD, PD],
            "gbc_model_set_dilatancy": [P, PD, PD, PD, PD],
            "gbc_model_set_gf": [P, I, PD],
            "gbc_model_assemble": [P, ctypes.POINTER(FaultMesh), ctypes.POINTER(HexMesh), D, D, I, I, D, PD, PD, I],
            "gbc_model_export_gf": [P, I, PD],
            "gbc_model_export_gf_rows": [P, I, I, ctypes.POINTER(I), PD],
            "gbc_model_set_precision": [P, I],
            "gbc_rhs": [P, D, ctypes.POINTER(PD), ctypes.POINTER(PD), I],
            "gbc_rhs_dev": [P, D, P, P],
            "gbc_integrate": [P, PD, D, D, ctypes.POINTER(SolverOpts), ctypes.POINTER(SolverStats)],
            "gbc_integrate_dev": [P, P, D, D, ctypes.POINTER(SolverOpts), ctypes.POINTER(SolverStats)],
            "gbc_integrate_record": [P, PD, D, D, ctypes.POINTER(SolverOpts), I, LL, PD, PD, ctypes.POINTER(LL),
                                     ctypes.POINTER(SolverStats)],
            "gbc_last_error": [ctypes.c_char_p, ctypes.c_size_t],
            "gbc_model_set_log_theta": [P, I],
            "gbc_model_error_word": [P],
            "gbc_ensemble_create": [I, ctypes.POINTER(I), ctypes.POINTER(I), ctypes.POINTER(P)],
            "gbc_ensemble_set_gf": [P, I, I, PD],
            "gbc_ensemble_assemble": [P, I, ctypes.POINTER(FaultMesh), D, D, I, I, D],
            "gbc_ensemble_set_fault_props": [P, I, PD, PD, PD, PD, D, D, D, D],
            "gbc_ensemble_set_block": [P, I],
            "gbc_ensemble_set_log_theta": [P, I],
            "gbc_ensemble_set_max_cluster": [P, I],
            "gbc_ensemble_set_regroup": [P, I],
            "gbc_ensemble_plan_clusters": [I, ctypes.POINTER(I), ctypes.POINTER(I), PD, ctypes.POINTER(I),
                                           ctypes.POINTER(I)],
            "gbc_hex_mesh_grid": [ctypes.POINTER(HexMesh), ctypes.POINTER(I), ctypes.POINTER(I), ctypes.POINTER(I)],
            "gbc_ensemble_integrate": [P, PD, PD, PD, ctypes.POINTER(SolverOpts), ctypes.POINTER(SolverStats)],
            "gbc_ensemble_integrate_dev": [P, P, PD, PD, ctypes.POINTER(SolverOpts), ctypes.POINTER(SolverStats)],
            "gbc_sweep_create": [P, I, ctypes.POINTER(P)],
            "gbc_sweep_set_fault_props": [P, I, PD, PD, PD, PD, D, D, D, D],
            "gbc_sweep_set_mantle_props": [P, I, PD, PD, PD],
            "gbc_sweep_set_engine": [P, I],
            "gbc_sweep_set_fault_product": [P, I],
            "gbc_sweep_rhs": [P, PD, PD],
            "gbc_sweep_rhs_dev": [P, P, P],
            "gbc_sweep_integrate": [P, PD, D, D, ctypes.POINTER(SolverOpts), ctypes.POINTER(SolverStats)],
            "gbc_sweep_integrate_dev": [P, P, D, D, ctypes.POINTER(SolverOpts), ctypes.POINTER(SolverStats)],
            "gbc_sweep_error_word": [P],
            "gbc_probe_fp64_fma": [P, I, I, LL, P, PD],
            "gbc_model_clear_error_word": [P],
            "gbc_debug_pipeline_fault": [I],
        }
        for name, args in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = I
        L.gbc_model_destroy.argtypes = [P]
        L.gbc_model_destroy.restype = None
        L.gbc_model_state_len.argtypes = [P]
        L.gbc_model_state_len.restype = LL
        L.gbc_kernel_launches.restype = LL
        L.gbc_rhs_visco_noalloc.argtypes = [I, I, I, P, P, ctypes.c_size_t, P, ctypes.c_size_t, P, P, P, P, D, D, D, D,
                                            P, P, PD, P, P, P]
        L.gbc_rhs_visco_noalloc.restype = I
        L.gbc_ensemble_destroy.argtypes = [P]
        L.gbc_ensemble_destroy.restype = None
        L.gbc_ensemble_state_len.argtypes = [P]
        L.gbc_ensemble_state_len.restype = LL
        L.gbc_ensemble_state_offset.argtypes = [P, I]
        L.gbc_ensemble_state_offset.restype = LL
        L.gbc_ensemble_stream.argtypes = [P]
        L.gbc_ensemble_stream.restype = P
        L.gbc_sweep_destroy.argtypes = [P]
        L.gbc_sweep_destroy.restype = None
        L.gbc_sweep_state_len.argtypes = [P]
        L.gbc_sweep_state_len.restype = LL
        L.gbc_sweep_stream.argtypes = [P]
        L.gbc_sweep_stream.restype = P
        L.gbc_model_stream.argtypes = [P]
        L.gbc_model_stream.restype = P
        L.gbc_version.restype = ctypes.c_char_p
        _lib = L
    return _lib


def last_error() -> str:
    buf = ctypes.create_string_buffer(1024)
    lib().gbc_last_error(buf, 1024)
    return buf.value.decode(errors="replace")


def check(rc: int) -> int:
    if rc < 0:
        raise GbcError(rc, last_error())
    return rc


def ptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(PD)


class Keep:
    def __init__(self):
        self.bufs = []

    def __call__(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        self.bufs.append(a)
        return ptr(a)


def fault_struct(mf, keep: Keep) -> FaultMesh:
    return FaultMesh(mf.nx, mf.nξ, keep(mf.x), keep(mf.ξ), keep(mf.y), keep(mf.z), keep(np.asarray(mf.ax).reshape(-1)),
                     keep(np.asarray(mf.aξ).reshape(-1)), float(mf.Δx), float(mf.Δξ), float(mf.dep), float(mf.dip))


def hex_struct(ma, keep: Keep) -> HexMesh:
    return HexMesh(ma.ne, *(keep(getattr(ma, n)) for n in ("cx", "cy", "cz", "qx", "qy", "qz", "Δx", "Δy", "Δz")))


def hex_mesh_grid(ma):
    """(nX, nY, nZ) when the mesh is a complete grid of equal cells (the mantle-mantle assembly then
    evaluates once per horizontal offset and layer pair), else None. Host-only."""
    k = Keep()
    h = hex_struct(ma, k)
    nx, ny, nz = I(), I(), I()
    ok = lib().gbc_hex_mesh_grid(ctypes.byref(h), ctypes.byref(nx), ctypes.byref(ny), ctypes.byref(nz))
    return (nx.value, ny.value, nz.value) if ok else None


def kernel_launches() -> int:
    return int(lib().gbc_kernel_launches())


def library_path() -> str:
    return os.path.realpath(_build.LIB)
