"""wsolve's file side (src/io.jl:22-133 mirror) on CPU: the datasets per name with the time axis
last, the reference's argument checks, append and force. The device recording call is replaced by
a stand-in that returns known records."""
import numpy as np
import pytest


def _prob():
    from oetqf_gb300.equation import ArrayPartition, ODEProblem
    u0 = ArrayPartition(np.arange(6.0).reshape(3, 2), np.arange(6.0).reshape(3, 2) + 10, np.zeros((3, 2)))
    return ODEProblem(None, u0, (0.0, 5.0), object())


def _fake_record(t0, n_rec, n):
    def rec(model, u0, a, b, stride=1, max_records=10000, **kw):
        ts = t0 + np.arange(n_rec, dtype=float)
        us = np.stack([u0 + k for k in range(n_rec)])
        return us[-1], {"status": 0}, ts, us
    return rec


def test_wsolve_datasets_time_last_and_append(tmp_path, monkeypatch):
    from oetqf_gb300 import io
    prob = _prob()
    n = prob.u0.flat().size
    f = str(tmp_path / "out.npz")
    getu = lambda u, t: (u.x[0], u.x[1])  # noqa: E731  (v and θ, as the reference's handler)
    monkeypatch.setattr(io, "integrate_record", _fake_record(0.0, 4, n))
    u1, st = io.wsolve(prob, f, 100, getu, ["v", "θ"], "t")
    with np.load(f) as z:
        assert set(z.files) == {"v", "θ", "t"}
        assert z["v"].shape == (3, 2, 4) and z["t"].shape == (4,)
        np.testing.assert_array_equal(z["v"][..., 2], prob.u0.x[0] + 2)
        np.testing.assert_array_equal(z["θ"][..., 3], prob.u0.x[1] + 3)
    with pytest.raises(FileExistsError):
        io.wsolve(prob, f, 100, getu, ["v", "θ"], "t")
    monkeypatch.setattr(io, "integrate_record", _fake_record(10.0, 2, n))
    io.wsolve(prob, f, 100, getu, ["v", "θ"], "t", append=True)
    with np.load(f) as z:
        assert z["v"].shape == (3, 2, 6)
        np.testing.assert_array_equal(z["t"], [0, 1, 2, 3, 10, 11])
    io.wsolve(prob, f, 100, getu, ["v", "θ"], "t", force=True)
    with np.load(f) as z:
        assert z["t"].shape == (2,)
    with pytest.raises(AssertionError):
        io.wsolve(prob, str(tmp_path / "x.npz"), 100, getu, ["v", "t"], "t")   # duplicate name (io.jl)
    with pytest.raises(AssertionError):
        io.wsolve(prob, str(tmp_path / "y.npz"), 100, getu, ["v"], "t")        # unmatched lengths
