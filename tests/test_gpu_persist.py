"""A model rebuilt from a Green's-function file (GB300Model.save_gf / load_gf) evaluates the same
right-hand side, bit for bit, as the model whose device assembly wrote the file."""
import numpy as np
import pytest

from oetqf_gb300.workloads import strike_slip_with_mantle

pytestmark = pytest.mark.gpu


def test_saved_greens_functions_rebuild_the_model(tmp_path):
    from oetqf_gb300.equation import GB300Model
    cm = strike_slip_with_mantle(length=20e3, depth=6e3, cell=2e3, mantle_cells=(5, 2, 2), mantle_y=8e3, years=1.0)
    a = GB300Model(cm.mf.nx, cm.mf.nξ, cm.ne)
    a.assemble_gf(cm.mf, cm.ma, cm.lam, cm.mu)
    f = str(tmp_path / "gf.h5")
    a.save_gf(f)
    b = GB300Model(cm.mf.nx, cm.mf.nξ, cm.ne)
    b.load_gf(f)
    for m in (a, b):
        m.set_fault_props(cm.pf)
        m.set_mantle_props(cm.pa)
    rng = np.random.default_rng(0)
    u = cm.u0.copy()
    u[:cm.N] *= np.exp(rng.uniform(-1, 3, cm.N))
    np.testing.assert_array_equal(a.rhs_flat(u), b.rhs_flat(u))
