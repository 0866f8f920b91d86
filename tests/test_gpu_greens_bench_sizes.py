"""Device-assembled Green's functions at the benchmark's own sizes against the FP64 oracle.

The 1000-patch fault over the 2500-cell Maxwell mantle (the fault-mantle benchmark model) is
compared entry by entry: every entry of the three mantle blocks (15000 x 1000, 1000 x 15000 and
15000 x 15000) and one right-hand side built from the oracle's own Green's functions. The
4096-patch fault over the 8000-cell mantle (the mixed-precision model; its 48000 x 48000 block is
18 GB) is compared on receiver rows: the four horizontal corner cells of every layer and a few
interior cells, each against every source. Both mantles are complete grids of equal cells, so the
device builds the mantle-mantle block from one evaluation per (horizontal offset, layer pair); the
corner receivers reach every offset sign, the largest |dx| and |dy| and every layer pair, i.e.
every key of that table. Bar: 1e-6 relative per entry with an absolute floor of 1e-12 * max|row|
(+1e-13 * max|block| for rows that vanish by symmetry), the FP64-mode bar of the other tests
(reference: src/BEM/GF.jl:123-296)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
RTOL = 1e-6


def _excess(gpu, cpu):
    """Per-entry excess over the bar, rows along the last axis."""
    gpu, cpu = np.asarray(gpu), np.asarray(cpu)
    floor = 1e-12 * np.abs(cpu).max(axis=-1, keepdims=True) + 1e-13 * np.abs(cpu).max()
    return np.abs(gpu - cpu) - (RTOL * np.abs(cpu) + floor)


def _check(gpu, cpu, what):
    e = _excess(gpu, cpu)
    rel = np.abs(gpu - cpu).max() / np.abs(cpu).max()
    assert np.all(e <= 0), f"{what}: max excess {e.max():.3e} (max diff / max entry {rel:.3e})"


def _device_model(cm):
    from oetqf_gb300.equation import GB300Model
    m = GB300Model(cm.mf.nx, cm.mf.nξ, cm.ne)
    m.assemble_gf(cm.mf, cm.ma, cm.lam, cm.mu)
    m.set_fault_props(cm.pf)
    m.set_mantle_props(cm.pa)
    return m


@pytest.fixture(scope="module")
def c1(oracle):
    from oetqf_gb300 import _capi as C
    from oetqf_gb300.workloads import strike_slip_with_mantle
    cm = strike_slip_with_mantle()
    m = _device_model(cm)
    dev = {w: m.export_gf(w) for w in (C.GBC_GF12, C.GBC_GF21, C.GBC_GF22)}
    orc = {C.GBC_GF12: oracle.gf_fm(cm.mf, cm.ma, cm.lam, cm.mu), C.GBC_GF21: oracle.gf_mf(cm.ma, cm.mf, cm.lam, cm.mu),
           C.GBC_GF22: oracle.gf_mm(cm.ma, cm.lam, cm.mu)}
    yield cm, m, dev, orc
    m.close()


def test_structured_box_path_is_taken():
    """The bench mantles are complete grids, so their mantle-mantle blocks come from the key table."""
    from oetqf_gb300 import _capi as C
    from oetqf_gb300.workloads import large_fault_with_mantle, strike_slip_with_mantle
    assert C.hex_mesh_grid(strike_slip_with_mantle().ma) == (50, 10, 5)
    assert C.hex_mesh_grid(large_fault_with_mantle().ma) == (40, 20, 10)


@pytest.mark.parametrize("which", ["gf12", "gf21", "gf22"])
def test_fault_mantle_1000x2500_every_entry(c1, which):
    from oetqf_gb300 import _capi as C
    cm, m, dev, orc = c1
    w = {"gf12": C.GBC_GF12, "gf21": C.GBC_GF21, "gf22": C.GBC_GF22}[which]
    _check(dev[w], orc[w], which)


def test_fault_mantle_1000x2500_rhs_on_oracle_greens_functions(c1, oracle):
    """One right-hand side of the benchmark model: the device (its own assembly) against the oracle
    model built from the oracle's Green's functions, at a state away from steady sliding."""
    from oetqf_gb300 import _capi as C
    cm, m, dev, orc = c1
    N, ne = cm.N, cm.ne
    rng = np.random.default_rng(11)
    u = cm.u0.copy()
    u[:N] = cm.pf.vpl * np.exp(rng.uniform(-1.0, 3.0, N))
    u[N:2 * N] *= np.exp(rng.uniform(-0.5, 0.5, N))
    u[2 * N + 6 * ne:2 * N + 12 * ne] = 1e6 * rng.standard_normal(6 * ne)
    gf11 = oracle.gf_ff(cm.mf, cm.lam, cm.mu, fourier=True)
    om = oracle.OracleModel(gf11, cm.pf, orc[C.GBC_GF12], orc[C.GBC_GF21], orc[C.GBC_GF22], cm.pa)
    ref = om.ode(u)
    got = m.rhs_flat(u)
    bounds = np.cumsum([0, N, N, 6 * ne, 6 * ne, N])
    for k, name in enumerate(("v", "θ", "ϵ", "σ", "δ")):
        a, b = got[bounds[k]:bounds[k + 1]], ref[bounds[k]:bounds[k + 1]]
        np.testing.assert_allclose(a, b, rtol=RTOL, atol=1e-12 * np.abs(b).max(), err_msg=name)


def _corner_and_interior_cells(ma):
    """The four horizontal corner cells of every layer plus the cells nearest the box centre in
    the top and bottom layers."""
    cx, cy, cz = np.asarray(ma.cx), np.asarray(ma.cy), np.asarray(ma.cz)
    cells = []
    for z in np.unique(cz):
        lay = np.flatnonzero(cz == z)
        for fx in (np.min, np.max):
            for fy in (np.min, np.max):
                sel = lay[(cx[lay] == fx(cx[lay])) & (cy[lay] == fy(cy[lay]))]
                cells.append(int(sel[0]))
    for z in (cz.max(), cz.min()):
        lay = np.flatnonzero(cz == z)
        d = (cx[lay] - cx.mean()) ** 2 + (cy[lay] - cy.mean()) ** 2
        cells.append(int(lay[np.argmin(d)]))
    return sorted(set(cells))


def test_fault_mantle_4096x8000_receiver_rows(oracle):
    from oetqf_gb300 import _capi as C
    from oetqf_gb300.workloads import large_fault_with_mantle
    cm = large_fault_with_mantle()
    ne, nx, nxi = cm.ne, cm.mf.nx, cm.mf.nξ
    cells = _corner_and_interior_cells(cm.ma)
    assert len(cells) == 4 * 10 + 2
    rows = np.array([k * ne + j for j in cells for k in range(6)])
    patches = [0, nx - 1, nx * (nxi - 1), nx * nxi - 1, nx * (nxi // 2) + nx // 2]
    m = _device_model(cm)
    try:
        g22 = m.export_gf_rows(C.GBC_GF22, rows)
        g12 = m.export_gf_rows(C.GBC_GF12, rows)
        g21 = m.export_gf_rows(C.GBC_GF21, patches)
    finally:
        m.close()
    o22 = oracle.gf_mm_rows(cm.ma, cm.lam, cm.mu, cells).reshape(len(rows), -1)
    o12 = oracle.gf_fm_rows(cm.mf, cm.ma, cm.lam, cm.mu, cells).reshape(len(rows), -1)
    o21 = oracle.gf_mf_rows(cm.ma, cm.mf, cm.lam, cm.mu, patches)
    _check(g22, o22, "gf22 rows")
    _check(g12, o12, "gf12 rows")
    _check(g21, o21, "gf21 rows")
