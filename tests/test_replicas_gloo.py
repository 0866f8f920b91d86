"""The N > 1 path of bench.py: replicas only (no data-path collective). Two CPU ranks over gloo
check the max-over-ranks timing and the whole-job aggregate, and the reference arm under
torch.distributed.run prints from rank 0 alone."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as tdist
    sys.path.insert(0, ROOT)
    import bench
    tdist.init_process_group("gloo", rank=rank, world_size=world)
    ms = bench.max_over_ranks(tdist, 100.0 * (rank + 1), "cpu")
    v = bench.replica_throughput(world, 2.0, ms)
    tdist.barrier()
    with open(out + f".{rank}", "w") as f:
        json.dump({"ms": ms, "value": v}, f)
    tdist.destroy_process_group()


def test_max_over_ranks_and_aggregate_gloo(tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    out = str(tmp_path / "r")
    mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
    for r in range(2):
        d = json.load(open(out + f".{r}"))
        assert d["ms"] == 200.0                 # the slower rank's time on every rank
        assert d["value"] == pytest.approx(2 * 2.0 / 0.2)


def test_reference_arm_under_torchrun_prints_once():
    env = dict(os.environ, GBC_BENCH_BACKEND="gloo", OMP_NUM_THREADS="2")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(_free_port()), os.path.join(ROOT, "bench.py"), "--impl", "reference",
           "--workload", "fault-800-f64", "--steps", "1", "--warmup", "0", "--cpu-budget", "1", "--gpus", "2"]
    p = subprocess.run(cmd, env=env, capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [l for l in p.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["e2e"]["h2d_bytes_per_step"] == 0
