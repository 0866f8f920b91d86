"""GPU Green's functions (libgbcycle) against the FP64 oracle: 1e-6 relative per entry with an
absolute floor of 1e-12 * max|row| (the FP64-mode bar)."""
import numpy as np
import pytest

from oetqf_gb300 import gen_hex8_box, gen_mesh, gauss_product_quadrature

pytestmark = pytest.mark.gpu
RTOL = 1e-6


def _close(gpu, cpu, axis=None):
    gpu, cpu = np.asarray(gpu), np.asarray(cpu)
    # 1e-12 * max|row|; rows that vanish by symmetry hold only round-off, hence the tiny global term
    if axis is None:
        floor = 1e-12 * np.abs(cpu).max()
    else:
        floor = 1e-12 * np.abs(cpu).max(axis=axis, keepdims=True) + 1e-13 * np.abs(cpu).max()
    err = np.abs(gpu - cpu) - (RTOL * np.abs(cpu) + floor)
    assert np.all(err <= 0), f"max excess {err.max()} (max rel {np.abs(gpu - cpu).max() / np.abs(cpu).max():.3e})"


@pytest.mark.parametrize("dip,ftype,br", [(90.0, 0, 0.0), (90.0, 0, 1.0), (41.0, 0, 0.0), (41.0, 1, 0.5), (33.0, 1, 0.0)])
def test_gf_ff(oracle, dip, ftype, br):
    from oetqf_gb300 import stress_greens_function
    mf = gen_mesh("RectOkada", 100.0, 100.0, 10.0, 10.0, dip)
    g = stress_greens_function(mf, 3e10, 3e10, ftype=ftype, fourier=False, buffer_ratio=br)
    c = oracle.gf_ff(mf, 3e10, 3e10, ftype=ftype, buffer_ratio=br)
    _close(g, c)
    gd = stress_greens_function(mf, 3e10, 3e10, ftype=ftype, fourier=True, buffer_ratio=br)
    cd = oracle.gf_ff_dft(c)
    # the embedding is symmetric: the imaginary parts are round-off, so the floor is taken on |X|
    floor = 1e-12 * np.abs(cd).max()
    assert np.all(np.abs(gd - cd) <= RTOL * np.abs(cd) + floor)


def test_gf_ff_config0_mesh(oracle):
    from oetqf_gb300 import stress_greens_function
    mf = gen_mesh("RectOkada", 80e3, 10e3, 1e3, 1e3, 90.0)
    g = stress_greens_function(mf, 3e10, 3e10, fourier=False)
    c = oracle.gf_ff(mf, 3e10, 3e10)
    _close(g, c)


def _pair():
    mf = gen_mesh("RectOkada", 100.0, 100.0, 10.0, 20.0, 90.0)
    ma = gen_hex8_box(-100.0, -50.0, -20.0, 200.0, 100.0, -30.0, 2, 3, 4)
    return mf, ma


@pytest.mark.parametrize("quad", ["Gauss1", "Gauss2"])
def test_gf_fm(oracle, quad):
    from oetqf_gb300 import stress_greens_function
    mf, ma = _pair()
    q = None if quad == "Gauss1" else gauss_product_quadrature(2)
    g = stress_greens_function(mf, ma, 1.0, 1.0, qtype=q if q is not None else "Gauss1", buffer_ratio=1.0)
    c = oracle.gf_fm(mf, ma, 1.0, 1.0, buffer_ratio=1.0, quad=q)
    _close(g, c, axis=1)


@pytest.mark.parametrize("ftype", [0, 1])
def test_gf_mf(oracle, ftype):
    from oetqf_gb300 import stress_greens_function
    mf, ma = _pair()
    g = stress_greens_function(ma, mf, 1.0, 1.0, ftype=ftype)
    c = oracle.gf_mf(ma, mf, 1.0, 1.0, ftype=ftype)
    _close(g, c, axis=1)


@pytest.mark.parametrize("quad", ["Gauss1", "Gauss2"])
def test_gf_mm(oracle, quad):
    from oetqf_gb300 import stress_greens_function
    _, ma = _pair()
    q = None if quad == "Gauss1" else gauss_product_quadrature(2)
    g = stress_greens_function(ma, 1.0, 1.0, qtype=q if q is not None else "Gauss1")
    c = oracle.gf_mm(ma, 1.0, 1.0, quad=q)
    _close(g, c, axis=1)


def test_gf_fault_touching_mantle(oracle):
    """Fault receivers sitting on mantle cell faces (y = 0) and 0.5 km above the mantle top:
    the strain-volume stacks refine toward the receiver."""
    from oetqf_gb300 import stress_greens_function
    mf = gen_mesh("RectOkada", 8e3, 10e3, 1e3, 1e3, 90.0)
    ma = gen_hex8_box(-4e3, -4e3, -10e3, 8e3, 8e3, -8e3, 4, 4, 2)
    g = stress_greens_function(ma, mf, 3e10, 3e10)
    c = oracle.gf_mf(ma, mf, 3e10, 3e10)
    _close(g, c, axis=1)
    g = stress_greens_function(mf, ma, 3e10, 3e10)
    c = oracle.gf_fm(mf, ma, 3e10, 3e10)
    _close(g, c, axis=1)


def test_invalid_buffer_ratio():
    from oetqf_gb300 import _capi as C, stress_greens_function
    mf = gen_mesh("RectOkada", 10.0, 10.0, 2.0, 2.0, 90.0)
    with pytest.raises(AssertionError):
        stress_greens_function(mf, 1.0, 1.0, buffer_ratio=-1.0)


def test_gf_mm_structured_box_uses_offsets(oracle):
    """A complete grid of equal cells takes the one-evaluation-per-(offset, layers) path: it matches the
    oracle at the FP64-mode bar and the direct pair kernel (reached by moving one cell off the grid)
    on every entry that does not involve the moved cell."""
    import copy
    from oetqf_gb300 import stress_greens_function
    ma = gen_hex8_box(-30e3, -25e3, -10e3, 60e3, 50e3, -25e3, 6, 5, 3)   # 90 cells, 891 keys
    g = stress_greens_function(ma, 3e10, 3e10)
    c = oracle.gf_mm(ma, 3e10, 3e10)
    _close(g, c, axis=1)
    mb = copy.deepcopy(ma)
    mb.cx = np.array(mb.cx, dtype=float)
    mb.qx = np.array(mb.qx, dtype=float)
    shift = 1e-7 * mb.Δx[0] if hasattr(mb, "Δx") else 1e-7 * np.asarray(mb.dx)[0]
    mb.cx[0] += shift
    mb.qx[0] += shift
    from oetqf_gb300 import _capi as C
    assert C.hex_mesh_grid(ma) == (6, 5, 3) and C.hex_mesh_grid(mb) is None  # the two paths are compared
    gd = stress_greens_function(mb, 3e10, 3e10)
    ne = ma.ne
    keep_r = np.array([(r % ne) != 0 for r in range(6 * ne)])
    keep_c = np.array([(c_ % ne) != 0 for c_ in range(6 * ne)])
    a, b = g[np.ix_(keep_r, keep_c)], gd[np.ix_(keep_r, keep_c)]
    np.testing.assert_allclose(a, b, rtol=1e-12, atol=1e-12 * np.abs(b).max())
