"""Benchmark of the H2-matrix kernel matvec on one GB300 (or N replicas).

Workload (the configuration the headline metric is quoted on): n = 1e6 points
i.i.d. uniform in [0,1]^3 (numpy default_rng(0)), Matern-3/2 kernel l = 0.5,
Chebyshev tensor-product interpolation p = 4 (q = 125 nodes), eta = 0.8,
leaf size 128, R = 32 right-hand sides ~ N(0,1).  One step = one H2 matvec
of all 32 right-hand sides in mixed precision (FP32 near field and coupling,
FP64 final combination).  Metric: n * R / time ("n*RHS/s", higher is better).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun (N > 1) every rank runs an independent replica of the
workload on its own GPU (weak scaling, no data-path collective); the step
time is the maximum over ranks.  ``--impl reference`` times the CPU FP64
restatement of the reference's matvec (the oracle; the reference itself
cannot be built here) on all host cores, rank 0 only.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "H2 matvecs/sec (n·RHS/s) at n=1e6, mixed-precision batched vs FP64 GPU at 1e-5 rel err"
UNIT = "n*RHS/s"
SMS = 152
FP32_LANES_PER_SM = 128


def workload_config(args):
    return {
        "workload": (f"H2 matvec, n={args.n} uniform [0,1]^3 (seed 0), MATERN32 l=0.5, "
                     f"p=4 (q=125), eta=0.8, leaf 128, R={args.rhs} ~N(0,1), precision mixed"),
        "n": args.n, "rhs": args.rhs, "kernel": "MATERN32", "l": 0.5, "degree": 4,
        "eta": 0.8, "min_leaf": 128, "precision": "mixed",
        "l2": "inputs larger than L2 (x: n*R FP64 = 256 MB) and a 512 MB L2 flush between steps",
    }


def make_problem(args):
    rng = np.random.default_rng(0)
    P = rng.random((3, args.n))
    X = rng.standard_normal((args.n, args.rhs))
    return P, X


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_id: str):
        self.gpu_id = gpu_id
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", self.gpu_id],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        out, _ = self.proc.communicate(timeout=10)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def gpu_smi_id(torch, dev) -> str:
    try:
        p = torch.cuda.get_device_properties(dev)
        bus = getattr(p, "pci_bus_id", None)
        dom = getattr(p, "pci_domain_id", 0)
        pdev = getattr(p, "pci_device_id", 0)
        if bus is not None:
            return f"{dom:08X}:{bus:02X}:{pdev:02X}.0"
    except Exception:
        pass
    return str(dev.index or 0)


def max_over_ranks(ms: float, dist=None, device=None) -> float:
    """Step time of the slowest rank (the contract's max over ranks)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return ms
    import torch
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(units_per_replica: float, ms: float, world: int) -> float:
    """Whole-job throughput of ``world`` independent replicas (weak scaling)."""
    return world * units_per_replica / (ms * 1e-3)


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    P, X = make_problem(args)
    import oracle
    O = oracle.OraclePlan(P, None, 4, 0.8, 128)
    stride = args.ref_stride
    t_tr = None
    times = []
    total = None
    for step in range(args.warmup + args.steps):
        if t_tr is None:
            t0 = time.perf_counter()
            O.action(1, 0.5, X, bucket_stride=1 << 30, nthreads=threads)
            t_tr = time.perf_counter() - t0
        t0 = time.perf_counter()
        _, work = O.action(1, 0.5, X, bucket_stride=stride, nthreads=threads)
        dt = time.perf_counter() - t0
        if total is None:
            total = O.near_pairs + O.q ** 2 * O.n_far
        frac = (work[0] + work[1]) / total
        t_full = t_tr + max(dt - t_tr, 0.0) / frac
        if step >= args.warmup:
            times.append(t_full)
    t_full = statistics.median(times)
    value = args.n * args.rhs / t_full
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_full * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": workload_config(args),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": (f"each step: oracle FP64 CPU restatement (the reference "
                                    f"needs Eigen, absent here) on every {stride}th column "
                                    f"bucket ({frac:.3%} of the pair work) + full upward/"
                                    f"downward passes, extrapolated; median of {args.steps}")},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=1_000_000)
    ap.add_argument("--rhs", type=int, default=32)
    ap.add_argument("--cpu-stride", type=int, default=8)
    ap.add_argument("--ref-stride", type=int, default=32)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.impl == "reference":
        return run_reference(args)

    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)

    from fmca_gb300 import CovarianceKernel, H2Matrix
    P, X = make_problem(args)
    t0 = time.perf_counter()
    H = H2Matrix(CovarianceKernel("MATERN32", 0.5), P, P, 4, 0.8, min_leaf=128,
                 precision="mixed")
    t_plan = time.perf_counter() - t0
    info = H.info
    Xd = torch.tensor(X, device=dev)  # FP64, n x R row-major
    Y = torch.empty_like(Xd)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)

    def barrier():
        torch.cuda.synchronize(dev)
        if dist is not None:
            dist.barrier()

    # warm-up (also uploads the plan)
    for _ in range(args.warmup):
        H.matvec(Xd, Y)
    barrier()
    H.set_profiling(True)
    sampler = ClockSampler(gpu_smi_id(torch, dev))
    sampler.start()
    time.sleep(0.3)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    stage_tot = None
    launches = 0
    barrier()
    for k in range(args.steps):
        flush.zero_()
        ev[k][0].record()
        H.matvec(Xd, Y)
        ev[k][1].record()
        st, nl = H.profile()
        launches += nl
        stage_tot = st if stage_tot is None else {s: stage_tot[s] + st[s] for s in st}
    barrier()
    clocks = sampler.stop()
    H.set_profiling(False)
    ms = max_over_ranks(sum(a.elapsed_time(b) for a, b in ev) / args.steps, dist, dev)
    value = replica_throughput(args.n * args.rhs, ms, world)
    stage_ms = {s: v / args.steps for s, v in stage_tot.items()}
    H.check_device_error()

    # end to end through the public API: pinned FP64 host buffers, H2D + matvec + D2H
    Xh = torch.tensor(X).pin_memory()
    Yh = torch.empty_like(Xh).pin_memory()
    for _ in range(3):
        H.action(Xh, out=Yh)
    barrier()
    e2e_t = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        yh = H.action(Xh, out=Yh)
        e2e_t.append(time.perf_counter() - t0)
    e2e_ms = max_over_ranks(statistics.median(e2e_t) * 1e3, dist, dev)
    e2e_value = replica_throughput(args.n * args.rhs, e2e_ms, world)
    assert yh.shape == (args.n, args.rhs)

    # accuracy against the plain FP64 GPU H2 product (the 5x denominator)
    fp64 = None
    if not args.no_fp64:
        Y64 = torch.empty_like(Xd)
        H.matvec(Xd, Y64, precision="fp64")
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        H.matvec(Xd, Y64, precision="fp64")
        e1.record()
        barrier()
        ms64 = e0.elapsed_time(e1)
        H.matvec(Xd, Y)
        barrier()
        err = float((torch.linalg.norm(Y - Y64) / torch.linalg.norm(Y64)).item())
        fp64 = {"ms_per_step": ms64, "value": args.n * args.rhs / (ms64 * 1e-3),
                "mixed_rel_err_vs_fp64": err, "speedup_mixed_vs_fp64": ms64 / ms}

    # roofline of the dominant kernel (near-field ksum): FP32 FMA work 2 R N_nf
    near_flops = 2.0 * args.rhs * info["near_pairs"]
    t_near = stage_ms["near"] * 1e-3
    achieved = near_flops / t_near / 1e12
    sm_mhz = clocks.get("sm_mhz") or 2070.0
    peak = SMS * FP32_LANES_PER_SM * 2 * sm_mhz * 1e6 / 1e12
    roofline = {
        "bound": "fp32", "kernel": "ksum near field (FP32 CUDA cores)",
        "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
        "traffic": None,
        "work": f"2*R*N_nf = {near_flops:.4g} FP32 flops per launch (N_nf = {info['near_pairs']} pairs)",
        "peak_source": ("FP32 FMA issue peak 152 SMs x 128 lanes x 2 flops at the median SM "
                        "clock sampled during the timed region (MEASURED_PEAKS.json has no "
                        "FP32 CUDA-core figure)"),
        "stage_ms": stage_ms,
    }

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        total = info["near_pairs"] + info["q"] ** 2 * info["far_blocks"]
        import oracle
        threads = os.cpu_count() or 1
        t0 = time.perf_counter()
        O = oracle.OraclePlan(P, None, 4, 0.8, 128)
        t_build = time.perf_counter() - t0
        t0 = time.perf_counter()
        O.action(1, 0.5, X, bucket_stride=1 << 30, nthreads=threads)
        t_tr = time.perf_counter() - t0
        t0 = time.perf_counter()
        _, work = O.action(1, 0.5, X, bucket_stride=args.cpu_stride, nthreads=threads)
        t_s = time.perf_counter() - t0
        frac = (work[0] + work[1]) / total
        t_full = t_tr + max(t_s - t_tr, 0.0) / frac
        cpu = {"value": args.n * args.rhs / t_full, "unit": UNIT, "cores": threads,
               "kind": "port",
               "sample": (f"oracle FP64 CPU restatement of the reference matvec (OpenMP, "
                          f"{threads} threads): every {args.cpu_stride}th column bucket "
                          f"({frac:.3%} of the pair work) + full upward/downward passes on "
                          f"the full workload took {t_s:.1f} s; extrapolated full matvec "
                          f"{t_full:.1f} s (passes alone {t_tr:.1f} s, plan build "
                          f"{t_build:.1f} s untimed)")}
        del O

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic", "config": workload_config(args),
            "e2e": {"value": e2e_value, "unit": UNIT,
                    "h2d_bytes_per_step": int(Xh.numel() * 8),
                    "d2h_bytes_per_step": int(args.n * args.rhs * 8),
                    "ms_per_step": e2e_ms},
            "gpu_launches": launches,
            "roofline": roofline, "cpu_baseline": cpu, "clocks": clocks, "fp64_gpu": fp64,
            "plan": {"build_s": t_plan, "far_blocks": info["far_blocks"],
                     "near_blocks": info["near_blocks"], "near_pairs": info["near_pairs"],
                     "clusters": info["row_clusters"]},
        }
        print(json.dumps(line))
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
