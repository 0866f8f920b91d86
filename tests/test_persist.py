"""save_property / load_property (property.jl:70-107) and Green's-function files: exact round
trips under the reference's field and dataset names."""
import numpy as np
import pytest

from oetqf_gb300 import (CompositePowerLawViscosityProperty, DilatancyProperty, PowerLawViscosityProperty,
                         RateStateQuasiDynamicProperty, load_greens_functions, load_property, save_greens_functions,
                         save_property)


def _rs(rng, n=12):
    return RateStateQuasiDynamicProperty(rng.random((4, 3)), rng.random((4, 3)), rng.random((4, 3)),
                                         1e7 * rng.random((4, 3)), 4.9e6, 1e-9, 0.55, 2e-6)


def _eq(p, q):
    assert type(p) is type(q)
    for f in p.__dataclass_fields__:
        a, b = getattr(p, f), getattr(q, f)
        if isinstance(a, list):
            for x, y in zip(a, b):
                _eq(x, y)
        else:
            np.testing.assert_array_equal(np.asarray(a), np.asarray(b))


def test_property_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    rs = _rs(rng)
    pl = PowerLawViscosityProperty(rng.random(5), np.array([0.0, 1, 2, 3, 2.5]), rng.random(6))
    cp = CompositePowerLawViscosityProperty([pl, PowerLawViscosityProperty(rng.random(5), np.zeros(5))], rng.random(6))
    dl = DilatancyProperty(rng.random(12), rng.random(12), rng.random(12), rng.random(12))
    for p in (rs, pl, cp, dl):
        f = tmp_path / "p.bson"
        save_property(str(f), p)
        assert f.exists()  # the given name is kept
        _eq(p, load_property(str(f), type(p).__name__))


def test_property_merged_file_uses_reference_names(tmp_path):
    rng = np.random.default_rng(1)
    rs, dl = _rs(rng), DilatancyProperty(rng.random(12), rng.random(12), rng.random(12), rng.random(12))
    f = str(tmp_path / "both.bson")
    save_property(f, rs, dl)  # property.jl:82-85 merges the field dictionaries
    with np.load(f) as z:
        assert set(z.files) == {"a", "b", "L", "σ", "η", "vpl", "f₀", "v₀", "tₚ", "ϵ", "β", "p₀"}
    _eq(rs, load_property(f, "RateStateQuasiDynamicProperty"))
    _eq(dl, load_property(f, "DilatancyProperty"))
    with pytest.raises(ValueError):
        load_property(f, "NoSuchProperty")


def test_greens_function_file_round_trip(tmp_path):
    rng = np.random.default_rng(2)
    g11 = rng.standard_normal((8, 3, 3)) + 1j * rng.standard_normal((8, 3, 3))
    g12, g21, g22 = rng.standard_normal((12, 24)), rng.standard_normal((24, 12)), rng.standard_normal((12, 12))
    f = str(tmp_path / "gf.h5")
    save_greens_functions(f, gf11=g11, gf12=g12, gf21=g21, gf22=g22)
    with np.load(f) as z:
        assert set(z.files) == {"gf₁₁", "gf₁₂", "gf₂₁", "gf₂₂"}
    g = load_greens_functions(f)
    for k, v in (("gf11", g11), ("gf12", g12), ("gf21", g21), ("gf22", g22)):
        np.testing.assert_array_equal(g[k], v)
    save_greens_functions(f, gf11=g11.real.copy())
    assert list(load_greens_functions(f)) == ["gf11"]
    with pytest.raises(ValueError):
        save_greens_functions(f)
