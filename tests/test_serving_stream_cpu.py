"""run_stream's host logic on CPU with a stand-in server: Poisson submission in arrival order,
latency percentiles from the server's own timestamps, aggregate simulated years over the makespan."""
import types

import numpy as np


class _FakeServer:
    def __init__(self):
        self.submitted, self.t = [], 0.0

    def submit(self, cm, precision=None):
        rid = len(self.submitted)
        self.submitted.append(cm)
        return rid

    def wait(self, rid):
        res = types.SimpleNamespace(submit_s=float(rid), done_s=float(rid) + 1.0 + rid, status=0)
        return np.zeros(1), res


def test_run_stream_aggregates():
    from oetqf_gb300.serving import run_stream
    year = 365.0 * 86400.0
    reqs = [types.SimpleNamespace(horizon=(k + 1) * year) for k in range(5)]
    srv = _FakeServer()
    out = run_stream(srv, reqs, rate_per_s=1e4, seed=3)
    assert srv.submitted == reqs                       # arrival order kept
    np.testing.assert_allclose(out["latency_s"], [1, 2, 3, 4, 5])
    assert out["p50_s"] == 3.0 and abs(out["p99_s"] - 4.96) < 1e-12
    assert out["status"] == [0]
    assert abs(out["sim_yr_per_s"] * out["makespan_s"] - 15.0) < 1e-9   # 1 + 2 + ... + 5 years
