"""bench.py's clock sampler: median SM clock under load, the maximum, and the throttle reasons
that were active during the timed region (parsed from nvidia-smi CSV lines)."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


class _Proc:
    def terminate(self):
        pass

    def wait(self):
        pass


def test_clock_samples_and_reasons(tmp_path):
    sys.path.insert(0, ROOT)
    import bench
    c = bench.Clocks(0)
    c.path = str(tmp_path / "clocks.csv")
    with open(c.path, "w") as f:
        f.write("0, 2070, 2070, 900.1, 0x0, Not Active, Not Active, Not Active, Not Active\n")
        f.write("0, 1980, 2070, 1390.0, 0x4, Not Active, Not Active, Not Active, Active\n")
        f.write("0, 2070, 2070, 1200.0, 0x0, Not Active, Not Active, Not Active, Not Active\n")
        f.write("garbage line\n")
    c.proc = _Proc()
    c.f = open(os.devnull, "w")
    out = c.stop()
    assert out["sm_mhz"] == 2070.0 and out["sm_max_mhz"] == 2070.0 and out["samples"] == 3
    assert out["reasons"] == ["sw_power_cap"]
    assert not os.path.exists(c.path)
    assert bench.Clocks(0).stop()["reasons"] == ["nvidia-smi unavailable"]   # never started
