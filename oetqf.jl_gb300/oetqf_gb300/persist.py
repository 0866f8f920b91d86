"""Green's-function files: the assembled arrays under the dataset names the reference's example
uses (``gf₁₁``, ``gf₁₂``, ``gf₂₁``, ``gf₂₂``; examples/otf-with-mantle.jl:44-56), so a model can be
rebuilt without assembly. HDF5 is not available here: the container is numpy's ``.npz``, written
through an open handle so the file keeps the name it was given. ``gf₁₁`` is stored in the form
it was given (the complex rFFT of the circulant embedding, or the real Toeplitz kernel)."""
from __future__ import annotations

import numpy as np

NAMES = {"gf11": "gf₁₁", "gf12": "gf₁₂", "gf21": "gf₂₁", "gf22": "gf₂₂"}


def save_greens_functions(file: str, gf11=None, gf12=None, gf21=None, gf22=None) -> None:
    d = {NAMES[k]: np.asarray(v) for k, v in (("gf11", gf11), ("gf12", gf12), ("gf21", gf21), ("gf22", gf22))
         if v is not None}
    if not d:
        raise ValueError("no Green's function given")
    with open(file, "wb") as f:
        np.savez(f, **d)


def load_greens_functions(file: str) -> dict:
    """Returns {"gf11": ..., "gf12": ..., ...} for the datasets present in the file."""
    inv = {v: k for k, v in NAMES.items()}
    with np.load(file) as z:
        return {inv[k]: z[k].copy() for k in z.files if k in inv}
