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


def test_gemv_traffic_scaled_from_the_small_capture():
    """The default line's roofline traffic: DRAM bytes per algorithmic byte of the captured 1000 + 2500
    launch (within 1 % of one: every row streamed once) times the 4096 + 8000 launch's bytes."""
    import bench
    tr, ab = bench.NCU_GEMV_TMA_SMALL
    assert 1.0 <= tr / ab < 1.01
    traffic, src = bench.gemv_tma_traffic(5394432000)
    assert traffic == round(5394432000 * tr / ab) and 5394432000 < traffic < 1.01 * 5394432000
    assert "scaled" in src
