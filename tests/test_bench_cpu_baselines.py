"""bench.py's two CPU baselines on the 800-patch fault with tiny budgets: the oracle's bounded
integration sample and the numpy/scipy twin's bounded RHS sample carry the fields of the bench line
and scale to the same horizon."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cpu_baselines_fault_only():
    sys.path.insert(0, ROOT)
    import bench
    cm = bench.workload("fault-800-f64")
    ob, (pack, how, total) = bench.cpu_oracle_sample(cm, "fault-800-f64", "VCABM5", budget_s=0.3)
    assert ob["kind"] == "port" and ob["unit"] == "sim-yr/s" and ob["value"] > 0 and ob["cores"] >= 1
    assert total == bench.RHS_FOR_HORIZON[("fault-800-f64", "VCABM5")] and how == "exact"
    tw = bench.cpu_twin_sample(cm, pack, how, total, budget_s=0.3)
    assert tw["kind"] == "port" and tw["value"] > 0 and "numpy/scipy twin" in tw["sample"]
    assert str(total) in tw["sample"] and str(total) in ob["sample"]
