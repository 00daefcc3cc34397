"""Benchmark of the H2-matrix kernel matvec on one GB300 (or N replicas).

Workload (the configuration the headline metric is quoted on): n = 1e6 points
i.i.d. uniform in [0,1]^3 (numpy default_rng(0)), Matern-3/2 kernel l = 0.5,
Chebyshev tensor-product interpolation p = 4 (q = 125 nodes), eta = 0.8,
leaf size 128, R = 32 right-hand sides ~ N(0,1).  One step = one H2 matvec
of all 32 right-hand sides in mixed precision (near field and coupling as
tensor-core kernel sums on FP16 hi/lo splits with FP32 accumulation, tree
passes in FP32, FP64 final combination).  Metric: n * R / time ("n*RHS/s",
higher is better).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun (N > 1) every rank runs an independent replica of the
workload on its own GPU (weak scaling, no data-path collective); the step
time is the maximum over ranks.  ``--impl reference`` times the CPU FP64
restatement of the reference's matvec (the oracle; the reference itself
cannot be built here) on all host cores, rank 0 only: one full product,
then one part of the product per step (a row subtree of the cluster tree
with exactly the work the full product spends on it), so that no number is
extrapolated.  The default run also computes the full FP64 oracle product
once and reports the GPU results' error against it.
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
# point pairs per clock per SM on the special-function unit: every pair costs
# one sqrt.approx (16 results per clock per SM) and one ex2.approx (32 per
# clock on GB300) on one pipe, 32 / 3 pairs per clock (measured by
# tests/test_sfu_rates.py)
SFU_PAIRS_PER_CLK = 32.0 / 3.0
# DRAM bytes (read + write) of one near-field kernel-sum launch of the default
# workload: a fixed figure from one ncu capture of the current kernel
# (dram__bytes_read.sum + dram__bytes_write.sum), not measured by this script
NEAR_DRAM_BYTES_PER_LAUNCH = 2.671359e9 + 0.151429e9
# parts of the CPU reference's product per timed step (a level of the
# cluster tree with this many clusters)
REF_PARTS = 16


def _measured_peak(key, fallback):
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)[key]), "of measured"
    except (OSError, KeyError, ValueError):
        return fallback, "of fallback"  # figures of an earlier GB300 measurement


BF16_TFLOPS, BF16_SOURCE = _measured_peak("bf16_tflops", 1900.0)
HBM_GBS, HBM_SOURCE = _measured_peak("hbm_gbs", 6800.0)


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
    """The CPU FP64 restatement of the reference's matvec on all host cores:
    one full product (warm-up, also timed and reported), then one part of the
    product per step, rotating over the REF_PARTS row subtrees of one tree
    level (oracle_action_part: exactly the work the full product spends on
    those rows, plus the small shared work of the levels above).  value =
    rows computed x R / time, summed over the timed steps: nothing is
    extrapolated."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    P, X = make_problem(args)
    import oracle
    t0 = time.perf_counter()
    O = oracle.OraclePlan(P, None, 4, 0.8, 128)
    t_build = time.perf_counter() - t0
    O.set_keep(True)
    t0 = time.perf_counter()
    Y, _ = O.action(1, 0.5, X, nthreads=threads)
    t_full = time.perf_counter() - t0
    Yp = np.zeros_like(Y, order="F")
    times, units = [], 0.0
    for step in range(args.warmup - 1 + args.steps):
        t0 = time.perf_counter()
        (b, cnt), _ = O.action_part(1, 0.5, X, Yp, step % REF_PARTS, REF_PARTS, nthreads=threads)
        dt = time.perf_counter() - t0
        if step >= args.warmup - 1:
            times.append(dt)
            units += cnt * args.rhs
    rows = O.perm(0)
    exact = bool(np.array_equal(Yp[rows[b:b + cnt]], Y[rows[b:b + cnt]]))
    value = units / sum(times)
    ms = 1e3 * sum(times) / len(times)
    sample = (f"oracle FP64 CPU restatement of the reference matvec (the reference needs Eigen, "
              f"absent here; OpenMP, {threads} threads). Warm-up: one full product, "
              f"{t_full:.1f} s = {args.n * args.rhs / t_full:.4g} n*RHS/s. Each step: one of "
              f"{REF_PARTS} parts (a row subtree with its column subtree's upward pass, every "
              f"block of its rows and its downward pass; about {100 / REF_PARTS:.1f}% of the "
              f"work; its blocks in one OpenMP loop over its row clusters, every row summed in "
              f"the full product's column-bucket order), rows x R computed / time, no "
              f"extrapolation; the last part's rows equal the full product's: {exact}")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": workload_config(args),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "full_product": {"seconds": t_full, "value": args.n * args.rhs / t_full,
                         "plan_build_s": t_build},
    }
    print(json.dumps(line))
    return 0


def _events_ms(torch, fn, steps, flush=None):
    """Mean device time of fn() over steps, CUDA events on the current stream."""
    times = []
    for _ in range(steps):
        if flush is not None:
            flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        fn()
        b.record()
        b.synchronize()
        times.append(a.elapsed_time(b))
    return sum(times) / len(times)


def plan_build_on_gpu(H, P, p, eta, leaf, dev):
    """The same plan with the cluster tree sorted and the block pattern built
    on the GPU (fmca_plan_create_gpu): its build time (two runs, the second
    counts; the first warms up the device) and whether it equals the
    host-built plan."""
    import torch
    from fmca_gb300 import H2Matrix
    torch.cuda.synchronize(dev)
    times = []
    for _ in range(2):
        t0 = time.perf_counter()
        G = H2Matrix(H.cov, P, P, p, eta, min_leaf=leaf, precision="mixed", build="gpu")
        times.append(time.perf_counter() - t0)
    same = (G.info == H.info and np.array_equal(G.rindices(), H.rindices()) and
            all(np.array_equal(a, b) for k in (0, 1) for a, b in zip(G.blocks(k), H.blocks(k))))
    return {"build_s": times[-1], "trees_on_gpu": G.trees_on_gpu,
            "pattern_on_gpu": G.pattern_on_gpu, "equals_host_plan": bool(same)}


def run_c3(args, torch, dev):
    """Batching: 64 clouds, n log-uniform in [2e3, 2e5], 3-D Gaussian mixture
    (8 components, sigma 0.05, centres U[0,1]^3 per cloud), GAUSSIAN l = 0.2,
    p = 3, eta = 0.8, 8 right-hand sides each, float32.  One CUDA-graph
    launch of the batched plan against per-instance launches."""
    from fmca_gb300 import CovarianceKernel, H2Matrix
    rng = np.random.default_rng(0)
    clouds = []
    for _ in range(64):
        n = int(np.exp(rng.uniform(np.log(2e3), np.log(2e5))))
        centres = rng.random((8, 3))
        comp = rng.integers(0, 8, n)
        clouds.append((centres[comp] + 0.05 * rng.standard_normal((n, 3))).T.copy())
    cov = CovarianceKernel("GAUSSIAN", 0.2)
    t0 = time.perf_counter()
    B = H2Matrix.batched(cov, clouds, 3, 0.8, precision="mixed")
    t_plan = time.perf_counter() - t0
    N, R = B.rows(), 8
    X = torch.tensor(rng.standard_normal((N, R)), dtype=torch.float32, device=dev)
    Y = torch.empty_like(X)
    B.set_autotune(not args.no_autotune)
    B.matvec(X, Y)  # tunes (outside the graph capture)
    g = B.graph(X, Y)
    for _ in range(args.warmup):
        g.launch()
    ms_graph = _events_ms(torch, g.launch, args.steps)
    # stage times of the batched product (CUDA events between the stages of
    # ordinary launches, averaged over the timed steps)
    B.set_profiling(True)
    stage_tot = None
    for _ in range(args.steps):
        B.matvec(X, Y)
        st, _ = B.profile()
        stage_tot = st if stage_tot is None else {k: stage_tot[k] + st[k] for k in st}
    B.set_profiling(False)
    stage_ms = {k: v / args.steps for k, v in stage_tot.items()}
    singles = [H2Matrix(cov, P, P, 3, 0.8, precision="mixed") for P in clouds]
    xs = [X[B.offsets[i]:B.offsets[i + 1]] for i in range(64)]
    ys = [torch.empty_like(x) for x in xs]
    for S in singles:
        S.set_autotune(not args.no_autotune)

    def each():
        for S, x, y in zip(singles, xs, ys):
            S.matvec(x, y)
    for _ in range(args.warmup):
        each()
    ms_each = _events_ms(torch, each, args.steps)
    err = max(float((torch.linalg.norm(Y[B.offsets[i]:B.offsets[i + 1]] - ys[i]) /
                     torch.linalg.norm(ys[i])).item()) for i in range(64))
    # the batched result against the FP64 oracle, cloud by cloud, on the
    # eight smallest clouds (a reduced batch the CPU finishes in seconds)
    import oracle
    small = sorted(range(64), key=lambda i: clouds[i].shape[1])[:8]
    Yh, Xh = Y.double().cpu().numpy(), X.double().cpu().numpy()
    err_or = 0.0
    for i in small:
        a, b = B.offsets[i], B.offsets[i + 1]
        Yo, _ = oracle.OraclePlan(clouds[i], None, 3, 0.8, 0).action(3, 0.2, Xh[a:b])
        err_or = max(err_or, float(np.linalg.norm(Yh[a:b] - Yo) / np.linalg.norm(Yo)))
    return {
        "metric": "batched H2 matvecs/sec (n·RHS/s), 64 clouds, one CUDA-graph launch",
        "value": N * R / (ms_graph * 1e-3), "unit": UNIT, "ms_per_step": ms_graph,
        "per_instance": {"value": N * R / (ms_each * 1e-3), "ms_per_step": ms_each,
                         "launch": "64 plans, one matvec each, back to back"},
        "speedup_graph_vs_per_instance": ms_each / ms_graph,
        "stage_ms": stage_ms,
        "max_rel_diff_batched_vs_single": err,
        "max_rel_err_vs_fp64_oracle": {"value": err_or, "clouds": [int(clouds[i].shape[1])
                                                                  for i in small]},
        "dtype": "f32", "data": "synthetic",
        "autotune": B.tuned_config(R),
        "config": {"workload": "C3: 64 clouds, n log-uniform [2e3, 2e5], Gaussian mixture, "
                               "GAUSSIAN l=0.2, p=3, eta=0.8, R=8, float32",
                   "total_points": int(N), "far_blocks": B.info["far_blocks"],
                   "near_pairs": B.info["near_pairs"], "plan_build_s": t_plan},
    }


def run_c4(args, torch, dev):
    """Differentiation: n = 2e5 on S^2, MATERN52 l = 0.3, sigma2 = 1, p = 4,
    eta = 0.8, leaf 96 (125 in effect); gradient of y^T K x w.r.t. l, sigma2
    and X, x and y ~ N(0,1) float32; FP64 adjoint, central differences
    (h = 1e-4) and the mixed-precision adjoint."""
    from fmca_gb300 import CovarianceKernel, H2Matrix
    rng = np.random.default_rng(0)
    n = 200000
    P = rng.standard_normal((3, n))
    P /= np.linalg.norm(P, axis=0)
    x = rng.standard_normal((n, 1))
    y = rng.standard_normal((n, 1))
    H = H2Matrix(CovarianceKernel("MATERN52", 0.3, sigma2=1.0), P, P, 4, 0.8, min_leaf=96)
    x64, y64 = torch.tensor(x, device=dev), torch.tensor(y, device=dev)
    x32, y32 = x64.float(), y64.float()
    ref = H.adjoint(x64, y64, precision="fp64")
    # the adjoint uses the launch shapes a matvec of its key tuned
    H.set_autotune(not args.no_autotune)
    H.matvec(x32, precision="mixed")
    for _ in range(args.warmup):
        H.adjoint(x32, y32, precision="mixed")
    ms_mixed = _events_ms(torch, lambda: H.adjoint(x32, y32, precision="mixed"), args.steps)
    ms_fp64 = _events_ms(torch, lambda: H.adjoint(x64, y64, precision="fp64"), 2)
    out = H.adjoint(x32, y32, precision="mixed")
    v64 = ref["values"].cpu().numpy()
    v32 = out["values"].cpu().numpy()
    d64 = ref["dX"].cpu().numpy()
    d32 = out["dX"].double().cpu().numpy()

    def f(l=0.3, Pn=None):
        if Pn is not None:
            H.update_points(Pn)
        H.cov.l = l
        v = float((y64 * H.matvec(x64, precision="fp64")).sum())
        H.cov.l = 0.3
        return v
    h = 1e-4
    fd_l = (f(0.3 * (1 + h)) - f(0.3 * (1 - h))) / (2 * 0.3 * h)
    fd_err = [abs(v64[1] - fd_l) / abs(fd_l)]
    for _ in range(3):
        i, d = int(rng.integers(0, n)), int(rng.integers(0, 3))
        Pp, Pm = P.copy(), P.copy()
        Pp[d, i] += h
        Pm[d, i] -= h
        fd = (f(Pn=Pp) - f(Pn=Pm)) / (2 * h)
        H.update_points(P)
        fd_err.append(abs(d64[i, d] - fd) / max(1.0, abs(fd)))
    return {
        "metric": "H2 adjoint (f, df/dl, df/dsigma2, df/dX) evaluations/sec (n·RHS/s)",
        "value": n / (ms_mixed * 1e-3), "unit": UNIT, "ms_per_step": ms_mixed,
        "fp64": {"ms_per_step": ms_fp64, "value": n / (ms_fp64 * 1e-3)},
        "mixed_rel_err_vs_fp64": {"f": abs(v32[0] - v64[0]) / abs(v64[0]),
                                  "df_dl": abs(v32[1] - v64[1]) / abs(v64[1]),
                                  "df_dsigma2": abs(v32[2] - v64[2]) / abs(v64[2]),
                                  "df_dX": float(np.linalg.norm(d32 - d64) / np.linalg.norm(d64))},
        "fp64_vs_central_differences_h1e-4": {"max_rel_err": max(fd_err), "checks": fd_err},
        "dtype": "f32", "data": "synthetic", "autotune": H.tuned_config(1, "mixed"),

        "config": {"workload": "C4: n=2e5 on S^2, MATERN52 l=0.3 sigma2=1, p=4, eta=0.8, "
                               "leaf 96 (125 effective), x,y ~ N(0,1) float32",
                   "far_blocks": H.info["far_blocks"], "near_pairs": H.info["near_pairs"]},
    }


def run_c5(args, torch, dev):
    """Combined GP hyperparameter step: n = 2e6 in [0,1]^2 with the first
    coordinate scaled by 4, EXPONENTIAL l = 0.1, p = 5 (36 nodes), eta = 0.6,
    leaf 128, 64 Rademacher probes z: K z and z^T (dK/dl) z in one adjoint
    call, mixed precision against FP64."""
    from fmca_gb300 import CovarianceKernel, H2Matrix
    rng = np.random.default_rng(0)
    n = 2000000
    P = rng.random((2, n))
    P[0] *= 4
    z = rng.choice([-1.0, 1.0], size=(n, 64))
    t0 = time.perf_counter()
    H = H2Matrix(CovarianceKernel("EXPONENTIAL", 0.1), P, P, 5, 0.6, min_leaf=128)
    t_plan = time.perf_counter() - t0
    gpu_build = None if args.no_gpu_build else plan_build_on_gpu(H, P, 5, 0.6, 128, dev)
    z32 = torch.tensor(z, dtype=torch.float32, device=dev)
    z64 = z32.double()

    def step(zz, prec):
        return H.adjoint(zz, zz, precision=prec, want_dX=False, want_Kx=True)
    H.set_autotune(not args.no_autotune)
    H.matvec(z32, precision="mixed")  # tunes the key the adjoint uses
    for _ in range(args.warmup):
        step(z32, "mixed")
    ms_mixed = _events_ms(torch, lambda: step(z32, "mixed"), args.steps)
    ms_fp64 = _events_ms(torch, lambda: step(z64, "fp64"), 1)
    a = step(z32, "mixed")
    b = step(z64, "fp64")
    va, vb = a["values"].cpu().numpy(), b["values"].cpu().numpy()
    kz_err = float((torch.linalg.norm(a["Kx"].double() - b["Kx"]) /
                    torch.linalg.norm(b["Kx"])).item())
    return {
        "metric": "GP hyperparameter step (K z and z^T dK/dl z, 64 probes) n·RHS/s",
        "value": n * 64 / (ms_mixed * 1e-3), "unit": UNIT, "ms_per_step": ms_mixed,
        "fp64": {"ms_per_step": ms_fp64, "value": n * 64 / (ms_fp64 * 1e-3),
                 "speedup_mixed_vs_fp64": ms_fp64 / ms_mixed},
        "autotune": H.tuned_config(64, "mixed"),
        "mixed_rel_err_vs_fp64": {"Kz": kz_err,
                                  "zKz": abs(va[0] - vb[0]) / abs(vb[0]),
                                  "z_dKdl_z": abs(va[1] - vb[1]) / abs(vb[1])},
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": "C5: n=2e6 in [0,4]x[0,1], EXPONENTIAL l=0.1, p=5 (q=36), "
                               "eta=0.6, leaf 128, 64 Rademacher probes",
                   "far_blocks": H.info["far_blocks"], "near_pairs": H.info["near_pairs"],
                   "plan_build_s": t_plan, "gpu_tree_build": gpu_build},
    }


def run_other_config(args):
    import torch
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    fn = {"c3": run_c3, "c4": run_c4, "c5": run_c5}[args.config]
    sampler = ClockSampler(gpu_smi_id(torch, dev))
    sampler.start()
    line = fn(args, torch, dev)
    line["clocks"] = sampler.stop()
    line.update({"n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
                 "higher_is_better": True, "scaling": "weak", "vs_baseline": None})
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
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-autotune", action="store_true",
                    help="default launch shapes instead of the autotuner's")
    ap.add_argument("--no-gpu-build", action="store_true",
                    help="skip timing the plan build on the GPU")
    ap.add_argument("--no-assembled", action="store_true",
                    help="skip the assembled (stored-block) product of the workload")
    ap.add_argument("--config", choices=["c2", "c3", "c4", "c5"], default="c2",
                    help="c2 (default): the headline workload; c3 batching, c4 gradients, "
                         "c5 GP step (one JSON line each, not the headline)")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.impl == "reference":
        return run_reference(args)
    if args.config != "c2":
        return run_other_config(args)

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
    gpu_build = None if args.no_gpu_build else plan_build_on_gpu(H, P, 4, 0.8, 128, dev)
    Xd = torch.tensor(X, device=dev)  # FP64, n x R row-major
    Y = torch.empty_like(Xd)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    # the autotuner measures the launch shapes on the first warm-up matvec
    # (untimed) and every later matvec reuses them
    H.set_autotune(not args.no_autotune)

    def barrier():
        torch.cuda.synchronize(dev)
        if dist is not None:
            dist.barrier()

    # warm-up (also uploads the plan and tunes)
    for _ in range(args.warmup):
        H.matvec(Xd, Y)
    barrier()
    tuned = H.tuned_config(args.rhs)
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

    # the assembled H2 matrix of the workload (computeH2Matrix): FP32 blocks
    # stored in HBM and streamed by every product (fmca_matvec_assembled);
    # with one right-hand side the stream is bound by HBM bandwidth
    asm = None
    if not args.no_assembled:
        need = H.assembled_bytes("fp32")
        free = torch.cuda.mem_get_info(dev)[0]
        if need + (8 << 30) > free:
            asm = {"skipped": f"{need / 1e9:.1f} GB of stored blocks do not fit next to "
                              f"the {free / 1e9:.1f} GB free"}
        else:
            barrier()
            t0 = time.perf_counter()
            H.computeH2Matrix("fp32")
            barrier()
            t_asm = time.perf_counter() - t0
            Ya = torch.empty_like(Xd)
            x1 = Xd[:, :1].contiguous()
            y1 = torch.empty_like(x1)

            def timed(fn, reps=5):
                fn()
                out = []
                for _ in range(reps):
                    flush.zero_()
                    e0, e1 = (torch.cuda.Event(enable_timing=True),
                              torch.cuda.Event(enable_timing=True))
                    e0.record()
                    fn()
                    e1.record()
                    torch.cuda.synchronize(dev)
                    out.append(e0.elapsed_time(e1))
                return statistics.median(out)

            ms_a32 = timed(lambda: H.mul(Xd, Ya))
            ms_a1 = timed(lambda: H.mul(x1, y1))
            H.check_device_error()
            ref = Y64 if fp64 is not None else Y
            err = float((torch.linalg.norm(Ya - ref) / torch.linalg.norm(ref)).item())
            asm = {"precision": "fp32", "stored_bytes": need, "assemble_s": t_asm,
                   "ms_per_step": ms_a32, "value": args.n * args.rhs / (ms_a32 * 1e-3),
                   "rel_err_vs_fp64" if fp64 is not None else "rel_err_vs_mixed": err,
                   "r1_ms_per_step": ms_a1,
                   "r1_roofline": {"bound": "hbm", "achieved": need / (ms_a1 * 1e-3) / 1e9,
                                   "peak": HBM_GBS, "unit": "GB/s",
                                   "frac": need / (ms_a1 * 1e-3) / 1e9 / HBM_GBS,
                                   "peak_source": f"MEASURED_PEAKS.json hbm_gbs, {HBM_SOURCE}",
                                   "work": "every stored block value read once per product"}}
            del Ya, x1, y1
            H.release_assembled()

    # roofline of the dominant kernel, the near-field kernel sum (ksum_um_kernel):
    # every point pair costs one square root and one exponential on
    # the special-function unit, the busiest unit of the kernel; the tensor
    # cores run 2 products per 16 sources (N = 64 and N = 32 columns, 192
    # flops per pair at R = 32)
    pairs = float(info["near_pairs"])
    t_near = stage_ms["near"] * 1e-3
    sm_mhz = clocks.get("sm_mhz") or 2070.0
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    sfu_peak = sms * SFU_PAIRS_PER_CLK * sm_mhz * 1e6 / 1e9
    sfu_achieved = pairs / t_near / 1e9
    tensor_flops = 2.0 * (2 * args.rhs + args.rhs) * pairs
    roofline = {
        "bound": "sfu", "kernel": "ksum_um_kernel, near field (tcgen05 products, SFU kernel values)",
        "achieved": sfu_achieved, "peak": sfu_peak, "unit": "Gpair/s", "frac": sfu_achieved / sfu_peak,
        "traffic": NEAR_DRAM_BYTES_PER_LAUNCH,
        "work": (f"N_nf = {info['near_pairs']} point pairs per launch, one sqrt and one "
                 "exp2 each"),
        "peak_source": (f"special-function unit: {SFU_PAIRS_PER_CLK:.2f} pairs/clock/SM (sqrt "
                        "16 and ex2 32 results/clock/SM on one pipe, measured by "
                        f"tests/test_sfu_rates.py) x {sms} SMs at the median SM clock sampled "
                        "during the timed region (the SFU has no entry in MEASURED_PEAKS.json)"),
        "traffic_source": ("fixed figure, not measured by this run: ncu "
                           "dram__bytes_read.sum + dram__bytes_write.sum of one near-field launch "
                           "of this workload, captured once with the current kernel"),
        "tensor": {"achieved": tensor_flops / t_near / 1e12, "peak": BF16_TFLOPS,
                   "unit": "TFLOP/s", "frac": tensor_flops / t_near / 1e12 / BF16_TFLOPS,
                   "work": "192 executed FP16 tensor flops per pair (3 products x 32 columns x 2)",
                   "peak_source": f"MEASURED_PEAKS.json bf16_tflops (cuBLAS burst), {BF16_SOURCE}"},
        "stage_ms": stage_ms,
    }

    # the full FP64 oracle product on the host cores: the CPU baseline
    # (timed, not extrapolated) and the reference the GPU results are
    # checked against at this size
    cpu, vs_oracle = None, None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        import oracle
        threads = os.cpu_count() or 1
        t0 = time.perf_counter()
        O = oracle.OraclePlan(P, None, 4, 0.8, 128)
        t_build = time.perf_counter() - t0
        t0 = time.perf_counter()
        Y_or, _ = O.action(1, 0.5, X, nthreads=threads)
        t_full = time.perf_counter() - t0
        cpu = {"value": args.n * args.rhs / t_full, "unit": UNIT, "cores": threads,
               "kind": "port",
               "sample": (f"one full product of this workload by the oracle FP64 CPU "
                          f"restatement of the reference matvec (OpenMP, {threads} threads): "
                          f"{t_full:.1f} s (plan build {t_build:.1f} s, not timed)")}
        yo = torch.tensor(Y_or, device=dev)
        H.matvec(Xd, Y)
        barrier()
        vs_oracle = {"mixed_rel_err": float((torch.linalg.norm(Y - yo) /
                                             torch.linalg.norm(yo)).item())}
        if fp64 is not None:
            vs_oracle["fp64_rel_err"] = float((torch.linalg.norm(Y64 - yo) /
                                               torch.linalg.norm(yo)).item())
        del O, yo

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
            "vs_fp64_oracle": vs_oracle, "autotune": tuned, "assembled": asm,
            "plan": {"build_s": t_plan, "gpu_tree_build": gpu_build,
                     "far_blocks": info["far_blocks"],
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
