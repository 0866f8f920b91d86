"""Structured mantle boxes (host-side detection of a complete grid of equal cells, which the
mantle-mantle assembly evaluates once per horizontal offset and layer pair). CPU only."""
import copy

import numpy as np

from oetqf_gb300 import gen_hex8_box

FIELDS = ("cx", "cy", "cz", "qx", "qy", "qz", "Δx", "Δy", "Δz")


def _grid(ma):
    from oetqf_gb300 import _capi as C
    return C.hex_mesh_grid(ma)


def _subset(ma, idx):
    mb = copy.deepcopy(ma)
    for f in FIELDS:
        setattr(mb, f, np.asarray(getattr(ma, f), dtype=float)[idx].copy())
    return mb


def test_complete_box_and_shuffled_order():
    ma = gen_hex8_box(-30e3, -25e3, -10e3, 60e3, 50e3, -25e3, 5, 4, 3)
    assert _grid(ma) == (5, 4, 3)
    perm = np.random.default_rng(0).permutation(ma.ne)
    assert _grid(_subset(ma, perm)) == (5, 4, 3)
    one_layer = gen_hex8_box(-30e3, -25e3, -10e3, 60e3, 50e3, -5e3, 5, 4, 1)
    assert _grid(one_layer) == (5, 4, 1)


def test_broken_grids_use_the_pair_kernel():
    ma = gen_hex8_box(-30e3, -25e3, -10e3, 60e3, 50e3, -25e3, 5, 4, 3)
    mb = _subset(ma, np.arange(ma.ne))
    mb.cx[7] += 1e-6 * mb.Δx[7]
    mb.qx[7] += 1e-6 * mb.Δx[7]
    assert _grid(mb) is None                                   # a cell off the grid
    assert _grid(_subset(ma, np.arange(1, ma.ne))) is None     # a missing cell
    mc = _subset(ma, np.arange(ma.ne))
    mc.Δz[3] *= 1.5
    assert _grid(mc) is None                                   # unequal cells
    assert _grid(gen_hex8_box(-1e3, -1e3, -2e3, 2e3, 3e3, -4e3, 2, 3, 4)) is None  # keys not fewer than pairs / 4
