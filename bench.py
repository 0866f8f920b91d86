"""Benchmark: simulated years per second of earthquake-cycle models on one GB300.

Default line (the headline metric, batched mixed precision against the plain FP64 GPU path): 256
independent fault-only models (patch counts U[200, 2000], per-model a - b, Dc, sigma; seeded
splitmix64 synthetic inputs) integrated together by the persistent ensemble kernel (FP32 FFT
convolution in shared memory, FP64 friction, theta state, stages and error norm; VCABM5 with the
reference example's settings) over a fixed window of the horizon, as one batched call (the models
never wait for each other); `ms_per_step` is that time divided by --steps. Warm-up integrates W
short windows (0.01 yr) untimed. `value` keeps the state in HBM (gbc_ensemble_integrate_dev);
`e2e` repeats the window through the host-buffer call gbc_ensemble_integrate (pinned host state in,
final state out). The same line measures the plain FP64 GPU path on every one of the 256 models
over the same window (each model alone through gbc_integrate, one after another), the slip-rate
differences between the arms and the FP64 oracle, and, as sub-objects, the FP64 and 16-bit
mantle GEMVs against their rooflines (the FP64 pipe peak is measured in the same run), the
tensor-core sweep and a serving stream. Other workloads: --workload.

--impl reference integrates the same 256 models over the same window on the host cores with the
C/OpenMP FP64 oracle (the reference's algorithm restated in C, its FFT convolution through radix-2
transforms; one model per host thread). Under torchrun each rank integrates an independent
replica (the path does not shard).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import tempfile
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "oetqf.jl_gb300"))

import numpy as np  # noqa: E402

from oetqf_gb300.workloads import (YEAR, fault_ensemble, large_fault_with_mantle, serving_requests,  # noqa: E402
                                   strike_slip_fault, strike_slip_with_mantle)

SOLVER = dict(reltol=1e-6, abstol=1e-8, dt=1e-8, dtmax=0.2 * YEAR)
# Right-hand-side evaluations each integrator takes over a workload's horizon, as counted by the
# device integrator (the oracle restates the same methods and controllers and takes the same steps
# over the horizons the parity tests cover: 28543 and 12381 for the 800-patch fault, counted by
# both); used to turn a bounded CPU sample into sim-yr/s.
RHS_FOR_HORIZON = {("fault-mantle-1000x2500-f64", "Tsit5"): 6 * 42388 + 1,
                   ("fault-mantle-1000x2500-f64", "VCABM5"): 138710,
                   ("fault-800-f64", "Tsit5"): 28543, ("fault-800-f64", "VCABM5"): 12381}
WORKLOADS = ["fault-mantle-1000x2500-f64", "fault-800-f64"]
# DRAM bytes (read + write) of one launch of the dominant kernel, read from an ncu capture of the
# same workload (dram__bytes_read.sum + dram__bytes_write.sum); reported as `traffic` with its
# source, since a live bench run cannot read hardware counters
NCU_TRAFFIC = {"fault-mantle-1000x2500-f64": 2044237000 + 2987264,
               "fault-mantle-1000x2500-f64-df64": 2081574000 + 3372032}
# the 16-bit row GEMV (k_gemv_tma) in an ncu capture on the 1000-patch + 2500-cell model: DRAM bytes
# (read + write) and the algorithmic bytes of its 16128 x 16128 16-bit rows. A 4096 + 8000 launch
# (5.39 GB) is above the capture size rule; its traffic is reported at the same ratio, since the
# kernel streams every row once whatever the model's size.
NCU_GEMV_TMA_SMALL = (520460000 + 3330000, 16128 * 16128 * 2)


def gemv_tma_traffic(bytes_per_launch):
    """(DRAM bytes of one k_gemv_tma launch of that many algorithmic bytes, how it was obtained)."""
    tr, ab = NCU_GEMV_TMA_SMALL
    return (round(bytes_per_launch * tr / ab),
            f"k_gemv_tma's DRAM bytes per algorithmic byte in an ncu capture on the 1000 + 2500 model ({tr / ab:.4f}), "
            "scaled to this launch's bytes (too large to capture)")
# the headline ensemble: window of the horizon integrated by every arm (all 256 models)
ENSEMBLE_WINDOW_YR = 8.0
# the loading phase before the ensemble's first events (the earliest starts after 3 years)
SHORT_HORIZON_YR = 3.0


def workload(name):
    if name == "fault-mantle-1000x2500-f64":
        return strike_slip_with_mantle()
    if name == "fault-800-f64":
        return strike_slip_fault()
    raise SystemExit(f"unknown workload {name}")


def rhs_bytes(cm) -> int:
    N, E = cm.N, 6 * cm.ne
    gf = (E * (N + E) + N * E) * 8 + cm.mf.nx * cm.mf.nξ ** 2 * 8
    state = (3 * N + 2 * E) * 8 * 2
    return gf + state


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), f"gbc_clocks_{os.getpid()}.csv")

    def start(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits", "-lms", "200",
                                          "-i", str(self.idx)], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        self.f.close()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx = float(p[2])
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.remove(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return None, 0, 1
    import torch.distributed as tdist
    tdist.init_process_group("nccl" if os.environ.get("GBC_BENCH_BACKEND", "nccl") == "nccl" else "gloo")
    return tdist, tdist.get_rank(), ws


def max_over_ranks(tdist, value: float, device: str) -> float:
    """The slowest rank's time: every replica integrates its own model, so the job ends with the last."""
    if tdist is None:
        return value
    import torch
    t = torch.tensor([value], device=device, dtype=torch.float64)
    tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(world_size: int, sim_years_per_rank: float, ms_max: float) -> float:
    """Whole-job sim-yr/s: every rank integrates its own replica over the same horizon."""
    return world_size * sim_years_per_rank / (ms_max / 1e3)


def cpu_oracle_model(cm, gfs=None):
    """The workload on the FP64 oracle. With gfs=None (no GPU on this path) the mantle Green's
    functions are stand-ins of the right shapes and scale: fault->mantle exact from the oracle,
    mantle->fault from it by Betti/Mura reciprocity (area/volume weighted transpose), mantle-mantle
    as its diagonal self-relaxation stored dense. The timed arithmetic -- dense FP64 GEMVs over
    every entry plus the friction update -- does not depend on the values."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    gf11 = O.gf_ff(cm.mf, cm.lam, cm.mu, fourier=True)
    if not cm.ne:
        return O, O.OracleModel(gf11, cm.pf), "exact", (gf11,)
    if gfs is not None:
        return O, O.OracleModel(gf11, cm.pf, *gfs, cm.pa), "exact (exported from the device assembly)", (gf11, *gfs)
    g12 = O.gf_fm(cm.mf, cm.ma, cm.lam, cm.mu)
    vol = np.tile(cm.ma.Δx * cm.ma.Δy * cm.ma.Δz, 6) * np.repeat([1.0, 2, 2, 1, 2, 1], cm.ne)
    area = cm.mf.Δx * cm.mf.Δξ
    g21 = np.ascontiguousarray((g12 * vol[:, None]).T / area)
    g22 = np.diag(np.full(6 * cm.ne, -cm.mu))
    return (O, O.OracleModel(gf11, cm.pf, g12, g21, g22, cm.pa), "stand-in mantle values (timing is value-independent)",
            (gf11, g12, g21, g22))


def cpu_oracle_sample(cm, name, alg, gfs=None, budget_s=20.0, nrhs_horizon=None):
    """Times the oracle (all host threads) over a bounded number of steps of the full-size workload
    with the same integrator and scales by the RHS evaluations that integrator takes for the whole
    horizon (from the table, or as counted on the device in the same run)."""
    O, om, how, pack = cpu_oracle_model(cm, gfs)
    t0 = time.perf_counter()
    om.ode(cm.u0)
    t_rhs = time.perf_counter() - t0
    per_step = 6.0 if alg == "Tsit5" else 2.0
    steps = int(min(1500, max(3, budget_s / (per_step * max(t_rhs, 1e-6)))))
    t0 = time.perf_counter()
    _, st = om.integrate(cm.u0, 0.0, cm.horizon, reltol=SOLVER["reltol"], abstol=SOLVER["abstol"], dt0=SOLVER["dt"],
                         maxiters=steps, alg=alg)
    wall = time.perf_counter() - t0
    per_rhs = wall / max(st.nrhs, 1)
    total_rhs = RHS_FOR_HORIZON.get((name, alg), nrhs_horizon)
    total = per_rhs * total_rhs
    out = {"value": (cm.horizon / YEAR) / total, "unit": "sim-yr/s", "cores": O.num_threads(), "kind": "port",
           "sample": f"{st.naccept + st.nreject} {alg} steps ({st.nrhs} RHS) of the full-size workload on the "
                     f"C/OpenMP FP64 oracle ({per_rhs * 1e3:.2f} ms/RHS, Green's functions: {how}), scaled to the "
                     f"{total_rhs} RHS evaluations the same integrator takes for {cm.horizon / YEAR:.0f} yr"}
    return out, (pack, how, total_rhs)


def cpu_twin_sample(cm, pack, how, total_rhs, budget_s=8.0):
    """The numpy/scipy twin of the reference's RHS (FFT convolution, BLAS GEMVs, vectorised friction;
    oracle/numpy_twin.py) timed over a bounded number of right-hand sides on all host threads and
    scaled to the RHS evaluations of the whole horizon (integrator overhead not included)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from numpy_twin import NumpyTwin
    tw = NumpyTwin(pack[0], cm.pf, *pack[1:], cm.pa) if cm.ne else NumpyTwin(pack[0], cm.pf)
    tw.ode(cm.u0)
    t0 = time.perf_counter()
    tw.ode(cm.u0)
    t1 = time.perf_counter() - t0
    n = int(min(500, max(3, budget_s / max(t1, 1e-6))))
    t0 = time.perf_counter()
    for _ in range(n):
        tw.ode(cm.u0)
    per_rhs = (time.perf_counter() - t0) / n
    return {"value": (cm.horizon / YEAR) / (per_rhs * total_rhs), "unit": "sim-yr/s", "cores": os.cpu_count(),
            "kind": "port",
            "sample": f"{n} right-hand sides of the full-size workload on the numpy/scipy twin of the reference's "
                      f"library structure (scipy.fft convolution, numpy BLAS GEMVs; {per_rhs * 1e3:.2f} ms/RHS, Green's "
                      f"functions: {how}), scaled to the {total_rhs} RHS evaluations of the horizon; integrator "
                      f"overhead not included"}


def run_reference(args):
    """The reference's CPU path on the host cores: the C/OpenMP oracle (the reference's loops, with its
    integrator) and the numpy/scipy twin (the reference's FFT + BLAS structure, right-hand sides only),
    each a bounded sample per step scaled to the horizon; the line reports the faster of the two."""
    tdist, rank, ws = dist()
    if rank != 0:
        return
    cm = workload(args.workload)
    share = args.cpu_budget / max(args.steps, 1) / 2
    oracle_vals, twin_vals = [], []
    for _ in range(args.steps):
        ob, (pack, how, total) = cpu_oracle_sample(cm, args.workload, args.alg, budget_s=share)
        oracle_vals.append(ob)
        twin_vals.append(cpu_twin_sample(cm, pack, how, total, budget_s=share))
    vo = statistics.median([x["value"] for x in oracle_vals])
    vt = statistics.median([x["value"] for x in twin_vals])
    base, other = (dict(twin_vals[0]), dict(oracle_vals[0])) if vt > vo else (dict(oracle_vals[0]), dict(twin_vals[0]))
    v = max(vo, vt)
    base["value"] = v
    other["value"] = min(vo, vt)
    line = {"metric": "sim-yr/s", "value": v, "unit": "sim-yr/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": (cm.horizon / YEAR) / v / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded splitmix64)", "impl": "reference",
            "config": {"workload": args.workload, "fault_patches": cm.N, "mantle_cells": cm.ne,
                       "horizon_yr": cm.horizon / YEAR, "solver": f"{args.alg} reltol 1e-6 abstol 1e-8 dt0 1e-8 s dtmax 0.2 yr"},
            "cpu_baseline": base, "cpu_baseline_other": other,
            "e2e": {"value": v, "unit": "sim-yr/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_gpu(args):
    import torch
    from oetqf_gb300 import _capi as C
    from oetqf_gb300.equation import GB300Model

    tdist, rank, ws = dist()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    cm = workload(args.workload)
    if args.years:
        cm.horizon = args.years * YEAR
    H = cm.horizon
    t_asm = time.perf_counter()
    m = GB300Model(cm.mf.nx, cm.mf.nξ, cm.ne)
    m.assemble_gf(cm.mf, cm.ma, cm.lam, cm.mu)
    m.set_fault_props(cm.pf)
    if cm.ne:
        m.set_mantle_props(cm.pa)
    if args.storage == "df64":
        m.set_precision(C.GBC_PREC_DF64)
    t_asm = time.perf_counter() - t_asm
    stream = torch.cuda.ExternalStream(m.stream)
    u = torch.tensor(cm.u0, device="cuda")
    if args.profile_rhs:
        if args.profile_precision != "f64":
            m.set_precision({"bf16": C.GBC_PREC_BF16, "f16": C.GBC_PREC_F16, "df64": C.GBC_PREC_DF64}[args.profile_precision])
        du = torch.zeros_like(u)
        for _ in range(args.profile_rhs):
            m.rhs_dev(u.data_ptr(), du.data_ptr())
        torch.cuda.synchronize()
        print(json.dumps({"profile_rhs": args.profile_rhs, "assembly_s": t_asm}))
        return
    # warm-up: W short windows from the initial state
    for _ in range(args.warmup):
        u.copy_(torch.tensor(cm.u0, device="cuda"))
        torch.cuda.synchronize()
        m.integrate_dev(u.data_ptr(), 0.0, 0.01 * YEAR, alg=args.alg, **SOLVER)
    u.copy_(torch.tensor(cm.u0, device="cuda"))
    torch.cuda.synchronize()
    K = args.steps
    edges = np.linspace(0.0, H, K + 1)
    clocks = Clocks(local)
    clocks.start()
    if tdist:
        tdist.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = C.kernel_launches()
    e0.record(stream)
    naccept = nreject = nrhs = 0
    for k in range(K):
        st = m.integrate_dev(u.data_ptr(), float(edges[k]), float(edges[k + 1]), alg=args.alg, **SOLVER)
        if st.status != 0:
            raise SystemExit(f"integration failed in window {k}: status {st.status}")
        naccept += st.naccept
        nreject += st.nreject
        nrhs += st.nrhs
    e1.record(stream)
    e1.synchronize()
    torch.cuda.synchronize()
    if tdist:
        tdist.barrier()
    ms = e0.elapsed_time(e1)
    launches = C.kernel_launches() - launches0
    clk = clocks.stop()
    ms = max_over_ranks(tdist, ms, "cuda")
    sim_yr = H / YEAR
    value = replica_throughput(ws, sim_yr, ms)
    # roofline of the dominant kernel (the row GEMV + friction launch): CUDA events on the model stream
    du = torch.zeros_like(u)
    R = 30
    for _ in range(3):
        m.rhs_dev(u.data_ptr(), du.data_ptr())
    r0, r1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    r0.record(stream)
    for _ in range(R):
        m.rhs_dev(u.data_ptr(), du.data_ptr())
    r1.record(stream)
    r1.synchronize()
    rhs_ms = r0.elapsed_time(r1) / R
    pk, psrc = peaks()
    peak = pk["hbm_gbs"]
    achieved = rhs_bytes(cm) / (rhs_ms / 1e3) / 1e9
    traffic = NCU_TRAFFIC.get(args.workload + ("-df64" if args.storage == "df64" else ""))
    df64_line = None
    if cm.ne and args.storage == "f64":
        # the FP64-accurate double-float storage, one RHS timed the same way (the FP64 pipe bounds
        # the FP64 GEMV; the FP32-pair GEMV is bound by HBM)
        m.set_precision(C.GBC_PREC_DF64)
        for _ in range(3):
            m.rhs_dev(u.data_ptr(), du.data_ptr())
        d0, d1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        d0.record(stream)
        for _ in range(R):
            m.rhs_dev(u.data_ptr(), du.data_ptr())
        d1.record(stream)
        d1.synchronize()
        dms = d0.elapsed_time(d1) / R
        m.set_precision(C.GBC_PREC_F64)
        da = rhs_bytes(cm) / (dms / 1e3) / 1e9
        df64_line = {"kernel": "k_prologue_mixed + k_gemv_df64 (one RHS)", "rhs_ms": dms, "achieved": da, "peak": peak,
                     "unit": "GB/s", "frac": da / peak, "speedup_vs_f64_rhs": rhs_ms / dms,
                     "run": "python bench.py --storage df64"}
    err_vs_f64 = None
    if args.storage == "df64":
        # slip-rate agreement with the plain FP64 path over one year from the initial state
        from oetqf_gb300.equation import GB300Model as _M
        ref = _M(cm.mf.nx, cm.mf.nξ, cm.ne)
        ref.assemble_gf(cm.mf, cm.ma, cm.lam, cm.mu)
        ref.set_fault_props(cm.pf)
        ref.set_mantle_props(cm.pa)
        ua, _ = ref.integrate(cm.u0, 0.0, YEAR, alg=args.alg, **SOLVER)
        ub, _ = m.integrate(cm.u0, 0.0, YEAR, alg=args.alg, **SOLVER)
        err_vs_f64 = float(np.abs(ub[:cm.N] - ua[:cm.N]).max() / np.abs(ua[:cm.N]).max())
        del ref
    # e2e: the same horizon through the host-buffer C-ABI call (pinned host state, H2D + D2H per window)
    uh = torch.tensor(cm.u0).pin_memory()
    un = uh.numpy()
    torch.cuda.synchronize()
    x0, x1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    x0.record(stream)
    for k in range(K):
        out, st = m.integrate(un, float(edges[k]), float(edges[k + 1]), alg=args.alg, **SOLVER)
        un[:] = out
    x1.record(stream)
    x1.synchronize()
    e2e_ms = x0.elapsed_time(x1)
    if rank != 0:
        return
    line = {"metric": "sim-yr/s", "value": value, "unit": "sim-yr/s", "n_gpus": ws, "steps": K, "warmup": args.warmup,
            "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if args.storage == "f64" else "f32x2 (double-float pairs, FP64-accurate)",
            "data": "synthetic (seeded splitmix64)",
            "config": {"workload": args.workload, "fault_patches": cm.N, "mantle_cells": cm.ne, "horizon_yr": sim_yr,
                       "precision": "f64" if args.storage == "f64" else
                       "mantle + fault rows as FP32 pairs (hi + lo), compensated FP32 dot products, FP64 results and friction",
                       "solver": f"{args.alg} reltol 1e-6 abstol 1e-8 dt0 1e-8 s dtmax 0.2 yr (the reference example's "
                                 "settings, examples/otf-with-mantle.jl:160-162)",
                       "rhs_evals": nrhs,
                       "l2": "inputs larger than L2 (Green's functions read every RHS)", "parallelism": "replicas",
                       "rk_steps": naccept + nreject, "rk_rejected": nreject, "assembly_s": round(t_asm, 3)},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": traffic, "rhs_ms": rhs_ms,
                         "kernel": "k_prologue + k_rows (one RHS)" if args.storage == "f64" else
                         "k_prologue_mixed + k_gemv_df64 (one RHS)",
                         "bytes_per_launch": rhs_bytes(cm), "peak_source": psrc,
                         "traffic_source": "ncu capture of this workload"},
            "e2e": {"value": sim_yr / (e2e_ms / 1e3), "unit": "sim-yr/s", "h2d_bytes_per_step": int(cm.u0.nbytes),
                    "d2h_bytes_per_step": int(cm.u0.nbytes)},
            "clocks": clk, "gpu_launches": launches}
    if df64_line:
        line["roofline_df64"] = df64_line
    if err_vs_f64 is not None:
        line["max_slip_rate_rel_err_vs_f64_1yr"] = err_vs_f64
    if not args.no_cpu:
        gfs = tuple(m.export_gf(w) for w in (C.GBC_GF12, C.GBC_GF21, C.GBC_GF22)) if cm.ne else None
        line["cpu_baseline"], (pack, how, total_rhs) = cpu_oracle_sample(cm, args.workload, args.alg, gfs=gfs,
                                                                         budget_s=args.cpu_budget, nrhs_horizon=nrhs)
        line["cpu_baseline_twin"] = cpu_twin_sample(cm, pack, how, total_rhs)
    print(json.dumps(line), flush=True)


def _peak():
    return peaks()[0]["hbm_gbs"]


def _base_line(metric_value, args, n_gpus, extra_cfg, ms, dtype):
    return {"metric": "sim-yr/s", "value": metric_value, "unit": "sim-yr/s", "n_gpus": n_gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": dtype, "data": "synthetic (seeded splitmix64)", "config": extra_cfg}


def run_mixed_large(args):
    """4096 patches + 8000 cells: block-scaled 16-bit Green's functions vs FP64 over a window."""
    import torch
    from oetqf_gb300 import _capi as C
    from oetqf_gb300.equation import GB300Model
    cm = large_fault_with_mantle()
    years = args.years or 20.0
    m = GB300Model(cm.mf.nx, cm.mf.nξ, cm.ne)
    t_asm = time.perf_counter()
    m.assemble_gf(cm.mf, cm.ma, cm.lam, cm.mu)
    t_asm = time.perf_counter() - t_asm
    m.set_fault_props(cm.pf)
    m.set_mantle_props(cm.pa)
    stream = torch.cuda.ExternalStream(m.stream)
    mode = C.GBC_PREC_BF16 if args.precision == "bf16" else C.GBC_PREC_F16
    N, E = cm.N, 6 * cm.ne
    out = {}
    # the 16-bit arm integrates ln θ under Tsit5; VCABM5 integrates θ itself (as the ensemble does)
    mixed_lt = args.alg != "VCABM5"
    for name, md, lt in (("f64", C.GBC_PREC_F64, False), ("df64", C.GBC_PREC_DF64, False), (args.precision, mode, mixed_lt)):
        m.set_precision(md)
        m.set_log_theta(lt)
        u = torch.tensor(cm.u0, device="cuda")
        du = torch.zeros_like(u)
        for _ in range(max(args.warmup, 3)):
            m.rhs_dev(u.data_ptr(), du.data_ptr())
        r0, r1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        r0.record(stream)
        for _ in range(20):
            m.rhs_dev(u.data_ptr(), du.data_ptr())
        r1.record(stream)
        r1.synchronize()
        rhs_ms = r0.elapsed_time(r1) / 20
        edges = np.linspace(0.0, years * YEAR, args.steps + 1)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        steps = 0
        for k in range(args.steps):
            st = m.integrate_dev(u.data_ptr(), float(edges[k]), float(edges[k + 1]), alg=args.alg, **SOLVER)
            steps += st.naccept + st.nreject
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        out[name] = {"rhs_ms": rhs_ms, "ms": ms, "v": u[:N].cpu().numpy(), "steps": steps,
                     "bytes": (E * (N + E) + N * E) * (8 if md in (C.GBC_PREC_F64, C.GBC_PREC_DF64) else 2)}
    v64, vmx = out["f64"]["v"], out[args.precision]["v"]
    err = float(np.abs(vmx - v64).max() / np.abs(v64).max())
    mx = out[args.precision]
    peak = _peak()
    ach = mx["bytes"] / (mx["rhs_ms"] / 1e3) / 1e9
    line = _base_line(years / (mx["ms"] / 1e3), args, 1,
                      {"workload": f"fault-mantle-4096x8000-{args.precision}", "fault_patches": N, "mantle_cells": cm.ne,
                       "window_yr": years, "assembly_s": round(t_asm, 2), "rk_steps": mx["steps"], "solver": args.alg,
                       "storage": f"{args.precision} with FP32 scale per 128x128 block, FP32 accumulate; FP32 Toeplitz (shared memory); FP64 friction, "
                                  f"{'ln-theta' if mixed_lt else 'theta'} state, error norm",
                       "l2": "inputs larger than L2"}, mx["ms"] / args.steps, args.precision)
    traffic, tsrc = gemv_tma_traffic(mx["bytes"])
    line["roofline"] = {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                        "traffic": traffic, "traffic_source": tsrc,
                        "kernel": "k_gemv_tma (TMA cp.async.bulk.tensor pipeline) + k_prologue_mixed + k_fault_rows_smem",
                        "rhs_ms": mx["rhs_ms"], "bytes_per_launch": mx["bytes"]}
    line["fp64_gpu"] = {"value": years / (out["f64"]["ms"] / 1e3), "rhs_ms": out["f64"]["rhs_ms"], "rk_steps": out["f64"]["steps"]}
    line["speedup_vs_fp64_gpu"] = line["value"] / line["fp64_gpu"]["value"]
    line["max_slip_rate_rel_err_vs_fp64"] = err
    d = out["df64"]
    line["df64"] = {"value": years / (d["ms"] / 1e3), "rhs_ms": d["rhs_ms"], "rk_steps": d["steps"],
                    "achieved_GBps": d["bytes"] / (d["rhs_ms"] / 1e3) / 1e9,
                    "max_slip_rate_rel_err_vs_fp64": float(np.abs(d["v"] - v64).max() / np.abs(v64).max()),
                    "storage": "FP32 pairs (hi + lo), compensated FP32 dot products, FP64 results and friction"}
    print(json.dumps(line), flush=True)


SWEEP_GEOMETRY = {"sweep-4096x8000": large_fault_with_mantle, "sweep-1000x2500": strike_slip_with_mantle}


def sweep_measure(K, engine, years, steps, alg, warmup=3, fault_product=False, geometry="sweep-4096x8000",
                  profile_rhs=0, base=None):
    """Property variants of a viscoelastic model sharing its block-scaled BF16 Green's functions
    (gbc_sweep) over a window, and the single-model BF16 path on variant 0 over the same window in
    the same run. Returns the measurements (times from CUDA events on the sweep's and the model's
    streams). With profile_rhs > 0 only that many right-hand sides of all variants run (for ncu)."""
    import torch
    from oetqf_gb300 import _capi as C
    from oetqf_gb300.equation import GB300Model
    from oetqf_gb300.property import PowerLawViscosityProperty, RateStateQuasiDynamicProperty
    from oetqf_gb300.sweep import Sweep
    if base is not None:  # an assembled BF16 model of the same geometry (kept open for the caller)
        m, cm = base
    else:
        cm = SWEEP_GEOMETRY[geometry]()
        m = GB300Model(cm.mf.nx, cm.mf.nξ, cm.ne)
        m.assemble_gf(cm.mf, cm.ma, cm.lam, cm.mu)
        m.set_fault_props(cm.pf)
        m.set_mantle_props(cm.pa)
        m.set_precision(C.GBC_PREC_BF16)
    N, E = cm.N, 6 * cm.ne
    props, u0s = [], []
    for k in range(K):  # normal stress, state distance and mantle viscosity vary across the variants
        s_k, l_k = 1.0 + 0.05 * k, 1.0 + 0.1 * k
        pf = RateStateQuasiDynamicProperty(cm.pf.a, cm.pf.b, cm.pf.L * l_k, cm.pf.σ * s_k, cm.pf.η, cm.pf.vpl,
                                           cm.pf.f0, cm.pf.v0)
        pa = PowerLawViscosityProperty(cm.pa.γ * (1.0 + 0.25 * k), cm.pa.n, cm.pa.dϵ0)
        u = cm.u0.copy()
        u[N:2 * N] *= l_k
        props.append((pf, pa))
        u0s.append(u)
    sw = Sweep(m, K, engine=engine)
    if fault_product:
        sw.set_fault_product(True)
    for k, (pf, pa) in enumerate(props):
        sw.set_fault_props(k, pf)
        sw.set_mantle_props(k, pa)
    stream = torch.cuda.ExternalStream(sw.stream)
    U = torch.tensor(np.stack(u0s), device="cuda")
    DU = torch.zeros_like(U)
    if profile_rhs:
        for _ in range(profile_rhs):
            sw.rhs_dev(U.data_ptr(), DU.data_ptr())
        torch.cuda.synchronize()
        err = sw.error_word()
        sw.close()
        if base is None:
            m.close()
        return {"profile_rhs": profile_rhs, "error_word": err}
    for _ in range(max(warmup, 3)):
        sw.rhs_dev(U.data_ptr(), DU.data_ptr())
    r0, r1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    r0.record(stream)
    for _ in range(20):
        sw.rhs_dev(U.data_ptr(), DU.data_ptr())
    r1.record(stream)
    r1.synchronize()
    rhs_ms = r0.elapsed_time(r1) / 20
    edges = np.linspace(0.0, years * YEAR, steps + 1)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    rk = np.zeros(K, dtype=np.int64)
    for i in range(steps):
        st = sw.integrate_dev(U.data_ptr(), float(edges[i]), float(edges[i + 1]), alg=alg, **SOLVER)
        rk += np.array([s.naccept + s.nreject for s in st])
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    if sw.error_word() != 0:
        raise RuntimeError("sweep pipeline wait timed out")
    stream1 = torch.cuda.ExternalStream(m.stream)
    u = torch.tensor(u0s[0], device="cuda")
    torch.cuda.synchronize()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(stream1)
    for i in range(steps):
        m.integrate_dev(u.data_ptr(), float(edges[i]), float(edges[i + 1]), alg=alg, **SOLVER)
    f1.record(stream1)
    f1.synchronize()
    ms1 = f0.elapsed_time(f1)
    v_sw, v_1 = U[0, :N].cpu().numpy(), u[:N].cpu().numpy()
    matrix_bytes = (E * (N + E) + N * E) * 2
    if fault_product:  # the three BF16 planes of the dense fault-fault block
        matrix_bytes += 6 * ((N + 127) // 128 * 128) ** 2
    reads = 1 if engine == "umma" else (K + 7) // 8
    sw.close()
    if base is None:
        m.close()
    return {"value": K * years / (ms / 1e3), "ms": ms, "rhs_ms": rhs_ms, "single_value": years / (ms1 / 1e3),
            "rk_steps": [int(x) for x in rk], "err": float(np.abs(v_sw - v_1).max() / np.abs(v_1).max()),
            "bytes": matrix_bytes * reads, "N": N, "ne": cm.ne}


def run_sweep(args):
    """Property variants of the 4096-patch + 8000-cell model sharing its block-scaled BF16 Green's
    functions (gbc_sweep): aggregate sim-yr/s over a window against the single-model BF16 path."""
    years = args.years or 20.0
    K = args.variants
    r = sweep_measure(K, args.engine, years, args.steps, args.alg, args.warmup, args.fault_product, args.workload,
                      args.profile_rhs)
    if args.profile_rhs:
        print(json.dumps(r), flush=True)
        return
    peak = _peak()
    ach = r["bytes"] / (r["rhs_ms"] / 1e3) / 1e9
    line = _base_line(r["value"], args, 1,
                      {"workload": f"{args.workload}-bf16-K{K}", "variants": K, "engine": args.engine,
                       "fault_rows": "tensor-core product (hi/mid/lo BF16 planes)" if args.fault_product else "FP32 Toeplitz per variant",
                       "fault_patches": r["N"], "mantle_cells": r["ne"], "window_yr": years, "solver": args.alg,
                       "rk_steps_per_variant": r["rk_steps"],
                       "variants_differ_in": "normal stress (+5%/variant), state distance L (+10%), mantle viscosity (+25%)",
                       "storage": "BF16 with FP32 scale per 128x128 block shared by all variants; FP32 Toeplitz; FP64 friction, theta state",
                       "l2": "inputs larger than L2"}, r["ms"] / args.steps, "bf16")
    line["roofline"] = {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                        "traffic": None, "kernel": f"k_sw_gemm_{args.engine} + k_sw_prologue + "
                        f"{'k_sw_friction' if args.fault_product else 'k_sw_fault_rows'} (one RHS of all variants)",
                        "rhs_ms": r["rhs_ms"], "bytes_per_launch": r["bytes"]}
    line["single_model"] = {"value": r["single_value"], "unit": "sim-yr/s"}
    line["speedup_vs_single_model"] = line["value"] / r["single_value"]
    line["variant0_max_slip_rate_rel_diff_vs_single_model"] = r["err"]
    print(json.dumps(line), flush=True)


def run_ensemble_profile(args):
    """Short ensemble runs for ncu captures of the persistent kernel: 0.01 yr of the 256 models, or
    with --profile-member i that model of the headline ensemble alone (regrouped onto the largest
    cluster it may use, as the slowest models run once the others have finished) for
    --profile-steps integrator steps."""
    from oetqf_gb300.ensemble import Ensemble
    years = 0.01 if args.profile_member < 0 else ENSEMBLE_WINDOW_YR
    models = fault_ensemble(n_models=256, years=years)
    if args.profile_member >= 0:
        models = [models[args.profile_member]]
    e = Ensemble([(mm.mf.nx, mm.mf.nξ) for mm in models])
    for i, mm in enumerate(models):
        e.assemble(i, mm.mf, mm.lam, mm.mu)
        e.set_fault_props(i, mm.pf)
    u0 = np.zeros(e.state_len)
    for i, mm in enumerate(models):
        u0[e.offsets[i]:e.offsets[i] + mm.u0.size] = mm.u0
    if args.profile_member >= 0:
        e.set_log_theta(args.alg != "VCABM5")
        e.set_block(512)
        u, st = e.integrate(u0, 0.0, 1e15, maxiters=args.profile_steps, alg=args.alg, **SOLVER)
    else:
        e.set_block(256)
        u, st = e.integrate(u0, 0.0, 0.01 * YEAR, alg=args.alg, **SOLVER)
    print(json.dumps({"profile_ensemble": True, "models": len(models), "steps": int(sum(s.naccept + s.nreject for s in st))}))


def run_serving(args):
    from oetqf_gb300.serving import Server, run_stream
    reqs = serving_requests(n_requests=args.requests)
    s = Server(hbm_budget_gb=args.hbm_budget_gb, alg=args.alg)
    out = run_stream(s, reqs, rate_per_s=20.0, seed=1)
    info = s.info()
    s.close()
    lat = out["latency_s"]
    line = _base_line(out["sim_yr_per_s"], args, 1, {"workload": "serving-poisson-20rps", "requests": len(reqs),
                                                     "mantle_requests": sum(r.ma is not None for r in reqs),
                                                     "hbm_budget_gb": args.hbm_budget_gb, "peak_bytes": info.peak_bytes,
                                                     "batch_iterations": info.iterations, "makespan_s": out["makespan_s"],
                                                     "solver": args.alg},
                      out["makespan_s"] * 1e3 / len(reqs), "f32+f64 / bf16")
    line["latency_s"] = {"p50": out["p50_s"], "p99": out["p99_s"], "max": float(lat.max())}
    line["gf_cache"] = {"hits": info.cache_hits, "misses": info.cache_misses, "resident_entries": info.cache_entries,
                        "resident_bytes": info.cache_bytes}
    line["status"] = out["status"]
    print(json.dumps(line), flush=True)


# ---- peaks ----------------------------------------------------------------------------------
FALLBACK_PEAKS = {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}


def peaks():
    """The machine's measured copy bandwidth and BF16 GEMM rate, else the stated fallback."""
    try:
        d = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        return {k: float(d[k]) for k in FALLBACK_PEAKS if k in d}, "measured (MEASURED_PEAKS.json)"
    except Exception:
        return dict(FALLBACK_PEAKS), "fallback (MEASURED_PEAKS.json absent: 6.8 TB/s, 1.9 PFLOP/s)"


def fp64_fma_peak(torch, C, reps=3):
    """FP64 FMA throughput of this GPU (FLOP/s), from gbc_probe_fp64_fma timed with CUDA events on
    the stream it runs on: 8 CTAs of 256 threads per SM, 8 independent chains per thread."""
    import ctypes
    blocks = torch.cuda.get_device_properties(0).multi_processor_count * 8
    out = torch.empty(blocks * 256, dtype=torch.float64, device="cuda")
    st = torch.cuda.current_stream()
    flops = ctypes.c_double()
    h = ctypes.c_void_p(st.cuda_stream)
    C.check(C.lib().gbc_probe_fp64_fma(ctypes.c_void_p(out.data_ptr()), blocks, 256, 512, h, ctypes.byref(flops)))
    best = 0.0
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        C.check(C.lib().gbc_probe_fp64_fma(ctypes.c_void_p(out.data_ptr()), blocks, 256, 16384, h, ctypes.byref(flops)))
        e1.record(st)
        e1.synchronize()
        best = max(best, flops.value / (e0.elapsed_time(e1) / 1e3))
    return best


# ---- the headline: 256-model ensemble vs the plain FP64 GPU path --------------------------------
def ensemble_of(models):
    from oetqf_gb300.ensemble import Ensemble
    e = Ensemble([(mm.mf.nx, mm.mf.nξ) for mm in models])
    for i, mm in enumerate(models):
        e.assemble(i, mm.mf, mm.lam, mm.mu)
        e.set_fault_props(i, mm.pf)
    u0 = np.zeros(e.state_len)
    for i, mm in enumerate(models):
        u0[e.offsets[i]:e.offsets[i] + mm.u0.size] = mm.u0
    return e, u0


def fp64_arm(models, years, alg, torch):
    """Every model alone through the plain FP64 single-model path (gbc_integrate_dev on its own
    stream), one after another, over [0, years]; each call bracketed by CUDA events on the model's
    stream (the host's graph capture and relaunch loop fall inside the bracket). Returns the total
    milliseconds, per-model final states, step counts and statuses."""
    from oetqf_gb300.equation import GB300Model
    total_ms, finals, steps, status = 0.0, [], [], []
    for mm in models:
        g = GB300Model(mm.mf.nx, mm.mf.nξ, 0)
        g.assemble_gf(mm.mf, None, mm.lam, mm.mu)
        g.set_fault_props(mm.pf)
        u = torch.tensor(mm.u0, device="cuda")
        s = torch.cuda.ExternalStream(g.stream)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        st = g.integrate_dev(u.data_ptr(), 0.0, years * YEAR, alg=alg, **SOLVER)
        e1.record(s)
        e1.synchronize()
        total_ms += e0.elapsed_time(e1)
        finals.append(u.cpu().numpy())
        steps.append(int(st.naccept + st.nreject))
        status.append(int(st.status))
        g.close()
    return total_ms, finals, steps, status


def short_horizon_errors(models, u_short, offs, alg, torch):
    """Slip rates of every model after the loading phase (SHORT_HORIZON_YR): the batched form and the
    plain FP64 GPU path against the FP64 oracle (FFT convolution, all host threads)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    _, f_short, _, _ = fp64_arm(models, SHORT_HORIZON_YR, alg, torch)
    oms = [O.OracleModel(O.gf_ff(mm.mf, mm.lam, mm.mu, fourier=True), mm.pf) for mm in models]
    orc, st = O.integrate_many(oms, [mm.u0 for mm in models], 0.0, SHORT_HORIZON_YR * YEAR, reltol=SOLVER["reltol"],
                               abstol=SOLVER["abstol"], dt0=SOLVER["dt"], dtmax=SOLVER["dtmax"], alg=alg, fft=True)
    eb, ef = [], []
    for i, mm in enumerate(models):
        ref = orc[i][:mm.N]
        eb.append(float(np.abs(u_short[offs[i]:offs[i] + mm.N] - ref).max() / np.abs(ref).max()))
        ef.append(float(np.abs(f_short[i][:mm.N] - ref).max() / np.abs(ref).max()))
    return {"at": f"{SHORT_HORIZON_YR:g} yr (the loading phase), every model, max |v - v_oracle| / max |v_oracle|",
            "batched_vs_oracle": {"max": max(eb), "median": float(np.median(eb))},
            "fp64_gpu_vs_oracle": {"max": max(ef), "median": float(np.median(ef))},
            "oracle_failed": int(sum(1 for x in st if x.status != 0))}


def run_headline(args):
    import ctypes
    import torch
    from oetqf_gb300 import _capi as C

    tdist, rank, ws = dist()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    years = args.years or ENSEMBLE_WINDOW_YR
    alg = args.alg
    models = fault_ensemble(n_models=256, years=years)
    n = len(models)
    t_asm = time.perf_counter()
    e, u0 = ensemble_of(models)
    t_asm = time.perf_counter() - t_asm
    # VCABM5 integrates θ itself (as the reference and the oracle do); Tsit5 runs on ln θ
    log_theta = alg != "VCABM5"
    e.set_log_theta(log_theta)
    best, tim = e.autotune(u0, steps=200, alg=alg, **SOLVER)
    stream = torch.cuda.ExternalStream(e.stream)
    for _ in range(args.warmup):
        e.integrate(u0, 0.0, 0.01 * YEAR, alg=alg, **SOLVER)
    K = args.steps
    u = torch.tensor(u0, device="cuda")
    torch.cuda.synchronize()
    clocks = Clocks(local)
    clocks.start()
    if tdist:
        tdist.barrier()
    torch.cuda.synchronize()
    launches0 = C.kernel_launches()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    # the window as one batched call: every model runs at its own pace and none waits for another
    # (K synchronised sub-windows would make the models meet at every edge, each sub-window lasting
    # as long as its slowest model: 5x the time on this workload); K divides the timed region
    st = e.integrate_dev(u.data_ptr(), 0.0, years * YEAR, alg=alg, **SOLVER)
    e1.record(stream)
    e1.synchronize()
    torch.cuda.synchronize()
    if tdist:
        tdist.barrier()
    ms = e0.elapsed_time(e1)
    launches = C.kernel_launches() - launches0
    clk = clocks.stop()
    steps = np.array([x.naccept + x.nreject for x in st], dtype=np.int64)
    rejects = np.array([x.nreject for x in st], dtype=np.int64)
    bad = [i for i, x in enumerate(st) if x.status != 0]
    if bad:
        raise SystemExit(f"ensemble members {bad[:8]} failed")
    ms = max_over_ranks(tdist, ms, "cuda")
    value = replica_throughput(ws, n * years, ms)
    u_ens = u.cpu().numpy()
    # e2e: the same window through the host-buffer call (pinned host state in, final state out)
    uh = torch.tensor(u0).pin_memory()
    un = uh.numpy()
    o = e._opts(SOLVER["reltol"], SOLVER["abstol"], SOLVER["dt"], SOLVER["dtmax"], 10**9, alg)
    torch.cuda.synchronize()
    x0, x1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    x0.record(stream)
    t0a, t1a = np.zeros(n), np.full(n, years * YEAR)
    sts = (C.SolverStats * n)()
    C.check(C.lib().gbc_ensemble_integrate(e.h, C.ptr(un), C.ptr(t0a), C.ptr(t1a), ctypes.byref(o), sts))
    x1.record(stream)
    x1.synchronize()
    e2e_ms = x0.elapsed_time(x1)
    e2e_same = bool(np.array_equal(un, u_ens))
    offs = list(e.offsets)
    # the loading phase before the first events (every model), for the short-horizon comparison
    u_s = torch.tensor(u0, device="cuda")
    e.integrate_dev(u_s.data_ptr(), 0.0, SHORT_HORIZON_YR * YEAR, alg=alg, **SOLVER)
    u_short = u_s.cpu().numpy()
    e.close()
    if rank != 0:
        return
    line = {"metric": "sim-yr/s", "value": value, "unit": "sim-yr/s", "n_gpus": ws, "steps": K, "warmup": args.warmup,
            "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32+f64", "data": "synthetic (seeded splitmix64)"}
    line["config"] = {"workload": "ensemble-256-fault-only", "models": n,
                      "patches_total": int(sum(mm.N for mm in models)),
                      "patch_range": [int(min(mm.N for mm in models)), int(max(mm.N for mm in models))],
                      "window_yr": years,
                      "steps": f"the window is integrated by one batched call; ms_per_step = that time / {K}",
                      "solver": f"{alg} reltol 1e-6 abstol 1e-8 dt0 1e-8 s dtmax 0.2 yr (examples/otf-with-mantle.jl:160-162)",
                      "precision": "FP32 rFFT convolution in shared memory; FP64 friction, " +
                                   ("ln-theta" if log_theta else "theta") + " state, stages, error norm",
                      "cta_threads": best, "assembly_s": round(t_asm, 2),
                      "rk_steps_min_mean_max": [int(steps.min()), float(steps.mean()), int(steps.max())],
                      "rk_rejected": int(rejects.sum()),
                      "slowest_member": {"index": int(np.argmax(steps)), "patches": int(models[int(np.argmax(steps))].N),
                                         "steps": int(steps.max()),
                                         "us_per_step": ms * 1e3 / float(steps.max())},
                      "l2": "per-model state and spectra are L2-resident (a few MB in all); no flush between steps",
                      "parallelism": "replicas"}
    line["e2e"] = {"value": ws * n * years / (e2e_ms / 1e3), "unit": "sim-yr/s",
                   "h2d_bytes_per_step": int(u0.nbytes) // K, "d2h_bytes_per_step": int(u0.nbytes) // K,
                   "call": "gbc_ensemble_integrate (pinned host state in, final state out: one call for the window)",
                   "final_state_equals_device_run": e2e_same}
    line["clocks"] = clk
    line["gpu_launches"] = launches
    # the plain FP64 GPU path on every model over the same window
    f_ms, finals, f_steps, f_status = fp64_arm(models, years, alg, torch)
    fp64_value = n * years / (f_ms / 1e3)
    errs = np.array([float(np.abs(u_ens[offs[i]:offs[i] + mm.N] - finals[i][:mm.N]).max() /
                           np.abs(finals[i][:mm.N]).max()) for i, mm in enumerate(models)])
    line["fp64_gpu"] = {"value": fp64_value, "unit": "sim-yr/s", "ms": f_ms, "models": n, "window_yr": years,
                        "how": "each model alone through the plain FP64 single-model path (gbc_integrate_dev: FP64 "
                               "Toeplitz rows, FP64 friction, the same VCABM5), one after another, CUDA events around "
                               "each call",
                        "rk_steps_total": int(sum(f_steps)), "failed": int(sum(1 for x in f_status if x != 0))}
    line["speedup_vs_fp64_gpu"] = value / fp64_value
    line["slip_rate_rel_diff_vs_fp64_gpu"] = {
        "at": f"window end ({years:g} yr), every model: max |v_batched - v_fp64| / max |v_fp64| (after the first "
              f"events the cycles are chaotic: any rounding difference grows, for the FP64 path as well, see "
              f"slip_rate_rel_diff_vs_fp64_oracle)",
        "max": float(errs.max()), "median": float(np.median(errs)), "p90": float(np.percentile(errs, 90)),
        "models_within_1e-4": int((errs <= 1e-4).sum())}
    line["slip_rate_rel_diff_short_horizon"] = short_horizon_errors(models, u_short, offs, alg, torch)
    pk, psrc = peaks()
    fpk = fp64_fma_peak(torch, C)
    line["fp64_peak"] = {"value": fpk / 1e12, "unit": "TFLOP/s", "how": "gbc_probe_fp64_fma, CUDA events, this run"}
    if not args.no_sub and ws == 1:
        # the matvec kernels against their bounds, measured in the same run
        try:
            line["fault_mantle_1000x2500"] = sub_fault_mantle_f64(torch, C, fpk, pk, psrc)
        except Exception as exc:
            line["fault_mantle_1000x2500"] = {"error": f"{type(exc).__name__}: {exc}"[:300]}
        try:
            line["fault_mantle_4096x8000"] = sub_mixed_4096(torch, C, pk, psrc, alg, sweep=not args.no_sweep)
        except Exception as exc:
            line["fault_mantle_4096x8000"] = {"error": f"{type(exc).__name__}: {exc}"[:300]}
        mx = line.get("fault_mantle_4096x8000", {}).get("bf16")
        if mx:
            traffic, tsrc = gemv_tma_traffic(mx["bytes_per_rhs"])
            line["roofline"] = {"bound": "hbm", "achieved": mx["achieved"], "peak": mx["peak"], "unit": "GB/s",
                                "frac": mx["frac"], "traffic": traffic, "traffic_source": tsrc,
                                "kernel": mx["kernel"], "rhs_ms": mx["rhs_ms"],
                                "bytes_per_launch": mx["bytes_per_rhs"], "peak_source": psrc,
                                "note": "the 16-bit mantle GEMV of the mixed-precision form; the ensemble kernel "
                                        "itself is bound by the latency of its dependent phases (its spectra and "
                                        "state stay in shared memory and L2), so no HBM or tensor roofline applies to it"}
    if not args.no_serving and ws == 1:
        try:
            line["serving"] = sub_serving(args)
        except Exception as exc:
            line["serving"] = {"error": f"{type(exc).__name__}: {exc}"[:300]}
    if not args.no_cpu and ws == 1:
        cb, done = cpu_ensemble_sample(models, years, alg)
        line["cpu_baseline"] = cb
        oe, of = [], []
        for i, uo in done.items():
            if uo is None:
                continue
            mm = models[i]
            ref = uo[:mm.N]
            oe.append(float(np.abs(u_ens[offs[i]:offs[i] + mm.N] - ref).max() / np.abs(ref).max()))
            of.append(float(np.abs(finals[i][:mm.N] - ref).max() / np.abs(ref).max()))
        if oe:
            line["slip_rate_rel_diff_vs_fp64_oracle"] = {
                "at": f"window end ({years:g} yr), the sampled models that reached it on the oracle",
                "models": len(oe), "batched": {"max": max(oe), "median": float(np.median(oe))},
                "fp64_gpu": {"max": max(of), "median": float(np.median(of))}}
    print(json.dumps(line), flush=True)


def sub_fault_mantle_f64(torch, C, fp64_peak, pk, psrc):
    """The 1000-patch + 2500-cell model (FP64 Green's functions, 2.04 GB read per RHS): the FP64 row
    GEMV (k_prologue + k_rows) against the measured FP64 FMA peak and against HBM, and the FP64-accurate
    double-float GEMV (k_gemv_df64) against HBM; CUDA events on the model's stream, 30 RHS each."""
    from oetqf_gb300.equation import GB300Model
    cm = strike_slip_with_mantle()
    m = GB300Model(cm.mf.nx, cm.mf.nξ, cm.ne)
    t = time.perf_counter()
    m.assemble_gf(cm.mf, cm.ma, cm.lam, cm.mu)
    t = time.perf_counter() - t
    m.set_fault_props(cm.pf)
    m.set_mantle_props(cm.pa)
    stream = torch.cuda.ExternalStream(m.stream)
    u = torch.tensor(cm.u0, device="cuda")
    du = torch.zeros_like(u)

    def rhs_ms(R=30):
        for _ in range(3):
            m.rhs_dev(u.data_ptr(), du.data_ptr())
        r0, r1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        r0.record(stream)
        for _ in range(R):
            m.rhs_dev(u.data_ptr(), du.data_ptr())
        r1.record(stream)
        r1.synchronize()
        return r0.elapsed_time(r1) / R

    N, E = cm.N, 6 * cm.ne
    entries = E * (N + E) + N * E + N * N   # mantle rows, mantle->fault rows, Toeplitz sum (one FMA each)
    f64 = rhs_ms()
    m.set_precision(C.GBC_PREC_DF64)
    df = rhs_ms()
    m.close()
    b = rhs_bytes(cm)
    ach, achd = b / (f64 / 1e3) / 1e9, b / (df / 1e3) / 1e9
    flops = 2.0 * entries / (f64 / 1e3)
    return {"workload": "fault-mantle-1000x2500-f64", "assembly_s": round(t, 2), "bytes_per_rhs": b,
            "f64": {"kernel": "k_prologue + k_rows (one RHS)", "rhs_ms": f64, "bound": "fp64",
                    "achieved_tflops": flops / 1e12, "peak_tflops": fp64_peak / 1e12, "frac": flops / fp64_peak,
                    "peak_source": "measured in this run (gbc_probe_fp64_fma, CUDA events)",
                    "hbm": {"achieved": ach, "peak": pk["hbm_gbs"], "unit": "GB/s", "frac": ach / pk["hbm_gbs"],
                            "peak_source": psrc},
                    "traffic": NCU_TRAFFIC["fault-mantle-1000x2500-f64"], "traffic_source": "ncu capture of this workload"},
            "df64": {"kernel": "k_prologue_mixed + k_gemv_df64 (one RHS)", "rhs_ms": df, "bound": "hbm", "achieved": achd,
                     "peak": pk["hbm_gbs"], "unit": "GB/s", "frac": achd / pk["hbm_gbs"], "peak_source": psrc,
                     "traffic": NCU_TRAFFIC["fault-mantle-1000x2500-f64-df64"],
                     "traffic_source": "ncu capture of this workload"}}


def sub_mixed_4096(torch, C, pk, psrc, alg, sweep=True):
    """The 4096-patch + 8000-cell model: the block-scaled BF16 GEMV (k_gemv_tma, 5.394 GB per RHS)
    against HBM, and on the same assembled Green's functions the 32-variant tensor-core sweep
    (k_sw_gemm_umma, fault rows on the tensor cores too) over a 20-year window against the
    single-model BF16 path."""
    from oetqf_gb300.equation import GB300Model
    cm = large_fault_with_mantle()
    m = GB300Model(cm.mf.nx, cm.mf.nξ, cm.ne)
    t = time.perf_counter()
    m.assemble_gf(cm.mf, cm.ma, cm.lam, cm.mu)
    t = time.perf_counter() - t
    m.set_fault_props(cm.pf)
    m.set_mantle_props(cm.pa)
    m.set_precision(C.GBC_PREC_BF16)
    stream = torch.cuda.ExternalStream(m.stream)
    u = torch.tensor(cm.u0, device="cuda")
    du = torch.zeros_like(u)
    for _ in range(3):
        m.rhs_dev(u.data_ptr(), du.data_ptr())
    r0, r1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    r0.record(stream)
    for _ in range(20):
        m.rhs_dev(u.data_ptr(), du.data_ptr())
    r1.record(stream)
    r1.synchronize()
    rms = r0.elapsed_time(r1) / 20
    N, E = cm.N, 6 * cm.ne
    b = (E * (N + E) + N * E) * 2
    ach = b / (rms / 1e3) / 1e9
    out = {"workload": "fault-mantle-4096x8000-bf16", "assembly_s": round(t, 2),
           "bf16": {"kernel": "k_prologue_mixed + k_gemv_tma + k_fault_rows_smem (one RHS)", "rhs_ms": rms,
                    "bytes_per_rhs": b, "bound": "hbm", "achieved": ach, "peak": pk["hbm_gbs"], "unit": "GB/s",
                    "frac": ach / pk["hbm_gbs"], "peak_source": psrc}}
    if sweep:
        try:
            r = sweep_measure(32, "umma", 20.0, 1, alg, fault_product=True, base=(m, cm))
            ach = r["bytes"] / (r["rhs_ms"] / 1e3) / 1e9
            out["sweep"] = {"workload": "sweep-4096x8000-bf16-K32", "variants": 32, "engine": "tcgen05",
                            "fault_rows": "tensor-core product (exact hi/mid/lo BF16 planes)", "window_yr": 20.0,
                            "value": r["value"], "unit": "sim-yr/s (all variants)", "single_model_bf16": r["single_value"],
                            "speedup_vs_single_model": r["value"] / r["single_value"],
                            "rhs_ms_all_variants": r["rhs_ms"],
                            "rhs_roofline": {"achieved": ach, "peak": pk["hbm_gbs"], "unit": "GB/s",
                                             "frac": ach / pk["hbm_gbs"], "peak_source": psrc,
                                             "bytes": r["bytes"]},
                            "rk_steps_per_variant_min_max": [min(r["rk_steps"]), max(r["rk_steps"])],
                            "variant0_max_slip_rate_rel_diff_vs_single_model": r["err"]}
        except Exception as exc:
            out["sweep"] = {"error": f"{type(exc).__name__}: {exc}"[:300]}
    m.close()
    return out


def cpu_ensemble_sample(models, years, alg, budget_steps=40000, every=16):
    """A bounded sample of the ensemble workload on the host cores: every `every`-th model over the
    same window with the C/OpenMP FP64 oracle (FFT convolution, one model per host thread), each
    capped at budget_steps steps. Returns (cpu_baseline dict, {model index: final state or None})."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    idx = list(range(0, len(models), every))
    oms = [O.OracleModel(O.gf_ff(models[i].mf, models[i].lam, models[i].mu, fourier=True), models[i].pf) for i in idx]
    t0 = time.perf_counter()
    finals, st = O.integrate_many(oms, [models[i].u0 for i in idx], 0.0, years * YEAR, reltol=SOLVER["reltol"],
                                  abstol=SOLVER["abstol"], dt0=SOLVER["dt"], dtmax=SOLVER["dtmax"], alg=alg,
                                  maxiters=budget_steps, fft=True)
    wall = time.perf_counter() - t0
    sim = sum(s.t for s in st) / YEAR
    done = {i: (f if s.status == 0 else None) for i, f, s in zip(idx, finals, st)}
    cores = O.num_threads()
    return ({"value": sim / wall, "unit": "sim-yr/s", "cores": cores, "kind": "port",
             "sample": f"{len(idx)} of the 256 models (every {every}th) over the same {years:g}-yr window on the "
                       f"C/OpenMP FP64 oracle (FFT convolution, one model per host thread, {alg}), each capped at "
                       f"{budget_steps} steps: {sum(1 for s in st if s.status == 0)} reached the window end, "
                       f"{sim:.2f} sim-yr in {wall:.1f} s"}, done)


def sub_serving(args, n_requests=200):
    """A Poisson stream (20 requests/s) of fault and fault+mantle requests drawn from 8 geometries
    (so the Green's-function cache is exercised), horizons of 1 to 4 years."""
    from oetqf_gb300.serving import Server, run_stream
    reqs = serving_requests(n_requests=n_requests, geometries=8, year_range=(1.0, 4.0))
    s = Server(hbm_budget_gb=args.hbm_budget_gb, alg=args.alg)
    out = run_stream(s, reqs, rate_per_s=20.0, seed=1)
    info = s.info()
    s.close()
    lat = out["latency_s"]
    return {"workload": "serving-poisson-20rps-8-geometries", "requests": len(reqs),
            "mantle_requests": sum(r.ma is not None for r in reqs), "horizon_yr_range": [1.0, 4.0],
            "value": out["sim_yr_per_s"], "unit": "sim-yr/s (aggregate)", "makespan_s": out["makespan_s"],
            "latency_s": {"p50": out["p50_s"], "p99": out["p99_s"], "max": float(lat.max())},
            "gf_cache": {"hits": info.cache_hits, "misses": info.cache_misses},
            "peak_bytes": info.peak_bytes, "batch_iterations": info.iterations, "status": out["status"]}


def run_reference_ensemble(args):
    """The reference arm of the headline: the same 256 models over the same window on the host cores
    with the C/OpenMP FP64 oracle (the reference's ode and integrator restated in C; its traction-rate
    convolution through radix-2 FFTs, as the reference applies it through FFTW; one model per host
    thread, each thread taking the next model when done). Measured end to end, nothing scaled."""
    tdist, rank, ws = dist()
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    years = args.years or ENSEMBLE_WINDOW_YR
    alg = args.alg
    models = fault_ensemble(n_models=256, years=years)
    n = len(models)
    oms = [O.OracleModel(O.gf_ff(mm.mf, mm.lam, mm.mu, fourier=True), mm.pf) for mm in models]
    S = dict(reltol=SOLVER["reltol"], abstol=SOLVER["abstol"], dt0=SOLVER["dt"], dtmax=SOLVER["dtmax"], alg=alg, fft=True)
    for _ in range(args.warmup):
        O.integrate_many(oms, [mm.u0 for mm in models], 0.0, 0.01 * YEAR, **S)
    K = args.steps
    t0 = time.perf_counter()
    states, st = O.integrate_many(oms, [mm.u0 for mm in models], 0.0, years * YEAR, **S)
    wall = time.perf_counter() - t0
    steps = sum(s.naccept + s.nreject for s in st)
    bad = [i for i, s in enumerate(st) if s.status != 0]
    if bad:
        raise SystemExit(f"oracle models {bad[:8]} failed")
    v = n * years / wall
    cores = O.num_threads()
    line = {"metric": "sim-yr/s", "value": v, "unit": "sim-yr/s", "n_gpus": ws, "steps": K, "warmup": args.warmup,
            "ms_per_step": wall * 1e3 / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded splitmix64)", "impl": "reference",
            "config": {"workload": "ensemble-256-fault-only", "models": n,
                       "patches_total": int(sum(mm.N for mm in models)),
                       "patch_range": [int(min(mm.N for mm in models)), int(max(mm.N for mm in models))],
                       "window_yr": years,
                       "steps": f"the window is integrated by one batched call; ms_per_step = that time / {K}",
                       "solver": f"{alg} reltol 1e-6 abstol 1e-8 dt0 1e-8 s dtmax 0.2 yr (examples/otf-with-mantle.jl:160-162)"},
            "cpu_baseline": {"value": v, "unit": "sim-yr/s", "cores": cores, "kind": "port",
                             "sample": f"all {n} models over the whole {years:g}-yr window in one call on the "
                                       f"C/OpenMP FP64 oracle ({alg}, FFT convolution, one model per host thread): "
                                       f"{steps} steps in {wall:.1f} s, nothing scaled"},
            "e2e": {"value": v, "unit": "sim-yr/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gbcycle", choices=["gbcycle", "reference"])
    ap.add_argument("--workload", default="ensemble-256",
                    choices=["ensemble-256"] + WORKLOADS + ["fault-mantle-4096x8000-mixed", "serving", "ensemble-profile",
                                                           "sweep-4096x8000", "sweep-1000x2500"])
    ap.add_argument("--precision", default="bf16", choices=["bf16", "f16"])
    ap.add_argument("--alg", default=None, choices=["VCABM5", "Tsit5"],
                    help="integrator (default: VCABM5, the reference example's solver; with it the state holds θ; "
                         "Tsit5 runs the 16-bit and ensemble workloads on ln θ)")
    ap.add_argument("--requests", type=int, default=32)
    ap.add_argument("--hbm-budget-gb", type=float, default=64.0)
    ap.add_argument("--cpu-budget", type=float, default=20.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-sub", action="store_true", help="default line: skip the GEMV / sweep sub-measurements")
    ap.add_argument("--no-serving", action="store_true", help="default line: skip the serving-stream sub-measurement")
    ap.add_argument("--profile-rhs", type=int, default=0, help="run N right-hand sides only (for ncu captures)")
    ap.add_argument("--years", type=float, default=0.0,
                    help="override the window (default line: %g yr) or a workload's horizon" % ENSEMBLE_WINDOW_YR)
    ap.add_argument("--profile-precision", default="f64", choices=["f64", "bf16", "f16", "df64"])
    ap.add_argument("--profile-member", type=int, default=-1,
                    help="ensemble-profile: that model of the headline ensemble alone")
    ap.add_argument("--profile-steps", type=int, default=2000, help="ensemble-profile: integrator steps")
    ap.add_argument("--variants", type=int, default=32, help="property variants of the sweep workload")
    ap.add_argument("--engine", default="umma", choices=["simt", "umma"], help="product engine of the sweep workload")
    ap.add_argument("--fault-product", action="store_true", help="sweep workload: fault-fault rows on the tensor cores too")
    ap.add_argument("--no-sweep", action="store_true", help="default line: skip the shared-geometry sweep sub-measurement")
    ap.add_argument("--storage", default="f64", choices=["f64", "df64"],
                    help="mantle Green's functions of the fault-mantle workloads: FP64, or FP32 pairs (FP64-accurate)")
    args = ap.parse_args()
    if args.alg is None:
        args.alg = "Tsit5" if args.workload == "ensemble-profile" else "VCABM5"
    if args.impl == "reference":
        if args.workload == "ensemble-256":
            run_reference_ensemble(args)
        else:
            run_reference(args)
    elif args.workload == "fault-mantle-4096x8000-mixed":
        run_mixed_large(args)
    elif args.workload == "ensemble-256":
        run_headline(args)
    elif args.workload == "ensemble-profile":
        run_ensemble_profile(args)
    elif args.workload == "serving":
        run_serving(args)
    elif args.workload.startswith("sweep-"):
        run_sweep(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
