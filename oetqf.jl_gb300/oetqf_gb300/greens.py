"""``stress_greens_function`` on the GPU, mirroring the four methods of src/BEM/GF.jl."""
from __future__ import annotations

import ctypes

import numpy as np

from . import _capi as C
from .mesh import BEMHex8Mesh, RectOkadaMesh


class StrikeSlip:  # src/BEM/GF.jl:4
    code = C.GBC_STRIKE_SLIP


class DipSlip:  # src/BEM/GF.jl:5
    code = C.GBC_DIP_SLIP


def _ftype(ftype) -> int:
    if isinstance(ftype, int):
        return ftype
    if isinstance(ftype, type):
        ftype = ftype()
    return ftype.code


def _quad(qtype):
    if qtype is None or (isinstance(qtype, str) and qtype == "Gauss1"):
        return np.zeros(3), np.ones(1)
    if isinstance(qtype, str):  # "GaussN": the hexahedron rule, weights normalised (GF.jl:318-323)
        from .mesh import get_quadrature
        qtype = get_quadrature(qtype)
    coords, weights = (np.asarray(q, dtype=np.float64).reshape(-1) for q in qtype)
    if len(coords) != 3 * len(weights):
        raise AssertionError("Wrong format of quadrature!")
    return coords, weights


def stress_greens_function(*args, ftype=StrikeSlip, fourier: bool = True, nrept: int = 2, buffer_ratio: float = 0.0,
                           qtype="Gauss1", checkeigvals: bool = False):
    """Dispatches like the reference on the argument types:

    (mf, λ, μ)       -> fault-fault (GF.jl:31), complex (nx,nξ,nξ) when fourier else real
    (mf, ma, λ, μ)   -> fault->mantle (GF.jl:123), (6ne, N)
    (ma, mf, λ, μ)   -> mantle->fault (GF.jl:194), (N, 6ne)
    (ma, λ, μ)       -> mantle-mantle (GF.jl:250), (6ne, 6ne)
    """
    L = C.lib()
    keep = C.Keep()
    ft = _ftype(ftype)
    if buffer_ratio < 0:
        raise AssertionError("Argument `buffer_ratio` must be ≥ 0.")
    if len(args) == 3 and isinstance(args[0], RectOkadaMesh):
        mf, lam, mu = args
        fs = C.fault_struct(mf, keep)
        n = mf.nx * mf.nξ * mf.nξ
        out = np.zeros(2 * n if fourier else n)
        C.check(L.gbc_stress_gf_ff(ctypes.byref(fs), lam, mu, ft, int(bool(fourier)), nrept, buffer_ratio, C.ptr(out)))
        if fourier:
            return (out[0::2] + 1j * out[1::2]).reshape((mf.nx, mf.nξ, mf.nξ), order="F")
        return out.reshape((mf.nx, mf.nξ, mf.nξ), order="F")
    if len(args) == 4 and isinstance(args[0], RectOkadaMesh) and isinstance(args[1], BEMHex8Mesh):
        mf, ma, lam, mu = args
        qc, qw = _quad(qtype)
        fs, hs = C.fault_struct(mf, keep), C.hex_struct(ma, keep)
        out = np.zeros(6 * ma.ne * mf.nx * mf.nξ)
        C.check(L.gbc_stress_gf_fm(ctypes.byref(fs), ctypes.byref(hs), lam, mu, ft, keep(qc), keep(qw), len(qw), nrept,
                                   buffer_ratio, C.ptr(out)))
        return out.reshape((6 * ma.ne, mf.nx * mf.nξ), order="F")
    if len(args) == 4 and isinstance(args[0], BEMHex8Mesh):
        ma, mf, lam, mu = args
        fs, hs = C.fault_struct(mf, keep), C.hex_struct(ma, keep)
        out = np.zeros(6 * ma.ne * mf.nx * mf.nξ)
        C.check(L.gbc_stress_gf_mf(ctypes.byref(hs), ctypes.byref(fs), lam, mu, ft, C.ptr(out)))
        return out.reshape((mf.nx * mf.nξ, 6 * ma.ne), order="F")
    if len(args) == 3 and isinstance(args[0], BEMHex8Mesh):
        ma, lam, mu = args
        qc, qw = _quad(qtype)
        hs = C.hex_struct(ma, keep)
        out = np.zeros((6 * ma.ne) ** 2)
        C.check(L.gbc_stress_gf_mm(ctypes.byref(hs), lam, mu, keep(qc), keep(qw), len(qw), C.ptr(out)))
        st = out.reshape((6 * ma.ne, 6 * ma.ne), order="F")
        if checkeigvals:
            print("Maximum real part of eigval is: %.4f" % np.linalg.eigvals(st).real.max())
        return st
    raise TypeError("stress_greens_function: unsupported argument types")
