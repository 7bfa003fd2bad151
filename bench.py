#!/usr/bin/env python
"""FP64-accurate GEMM throughput on GB300: Ozaki BF16 split vs native FP64.

Workload (default): C = A * B, M = N = K = 8192, float64, A and B from the emulated-FP64
configuration (sign * U[1,2) * 2^(e_line + e_elem), e_line in [-30, 30] per row of A /
column of B, e_elem in [-8, 8] per element; seeded, synthetic), slice count chosen per
problem by the library (slices = 0) to meet its normwise tolerance.

One JSON line (rank 0):
  value      FP64-equivalent TFLOP/s (2*M*N*K / time) of gb_gemm_f64 in Ozaki mode, inputs
             resident in HBM, whole job over all ranks (replicas: each rank its own GEMM)
  e2e        the same through the C ABI with host buffers: pinned H2D of A and B, the call,
             D2H of C, all inside the timed region
  roofline   the slice-product tensor-core kernel: BF16 tensor flops per launch / its
             CUDA-event duration (library tracing layer, on the launching stream), against
             the measured BF16 dense peak
  native     the native FP64 kernel on the same inputs (TFLOP/s) and both normwise errors
             against near-exact sampled dot products
  cpu_baseline  jmul!'s register-tiled FMA chain (the oracle port) on the host cores
--impl reference times that CPU port alone on the same configuration.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (os.path.join(ROOT, "jblas.jl_gb300"), os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "FP64-accurate GEMM TFLOP/s, Ozaki split vs native FP64 on GB300 at stated rel. error"


def parse_args():
    p = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["gbblas", "reference"], default="gbblas")
    p.add_argument("--size", type=int, default=8192)
    p.add_argument("--slices", type=int, default=0, help="0 = automatic (library tolerance)")
    p.add_argument("--no-native", action="store_true", help="skip the native FP64 comparison")
    p.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    p.add_argument("--cpu-seconds", type=float, default=12.0, help="target length of the CPU sample")
    return p.parse_args()


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except (OSError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def committed_traffic(workload):
    """DRAM bytes per launch of the slice-product kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "ozaki_slice_mma_%s.txt" % workload)
    try:
        with open(path) as f:
            for line in f:
                if line.startswith("dram_bytes_per_launch_full_size:"):
                    return float(line.split(":", 1)[1].split()[0])
    except OSError:
        pass
    return None


class ClockSampler:
    """nvidia-smi clock / throttle-reason samples while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.dev = device_index
        self.proc = None
        self.path = os.path.join(ROOT, "gpurun_out", "clocks_bench_%d.csv" % os.getpid())

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.fh, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.fh.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, parts[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "samples": len(sm),
                "reasons": sorted(reasons)}


def cpu_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_sample(A, B, target_s, threads):
    """Time jmul!'s register-tiled chain on a column sample of A*B; TFLOP/s and description."""
    import oracle
    n = A.shape[0]
    K = A.shape[1]
    cols = max(6, min(B.shape[1], 48))
    t0 = time.perf_counter()
    oracle.jmul_tiled(A, np.asfortranarray(B[:, :cols]), nthreads=threads)
    dt = time.perf_counter() - t0
    cols = int(min(B.shape[1], max(6, cols * target_s / max(dt, 1e-6))))
    cols -= cols % 6 if cols > 6 else 0
    Bs = np.asfortranarray(B[:, :cols])
    t0 = time.perf_counter()
    oracle.jmul_tiled(A, Bs, nthreads=threads)
    dt = time.perf_counter() - t0
    flops = 2.0 * n * K * cols
    return flops / dt / 1e12, "C[:, :%d] of the %dx%dx%d product (%.3g flop), %.2f s" % (cols, n, K, B.shape[1],
                                                                                      flops, dt), cols, dt


def normwise_err(Cres, A, B, rows, cols, hi, lo):
    d = (Cres[rows, cols] - hi) - lo
    scale = np.sqrt(Cres.size / rows.size)
    return float(np.linalg.norm(d) * scale / (np.linalg.norm(A) * np.linalg.norm(B)))


def reference_arm(args, rank, world):
    """The reference's CPU algorithm (oracle port of jmul!) timed on the host cores."""
    if rank != 0:
        return 0
    from gbblas import workloads
    import oracle
    n = args.size
    A = np.asfortranarray(workloads.ozaki_matrix(n, n, per="row", stream=1))
    B = np.asfortranarray(workloads.ozaki_matrix(n, n, per="col", stream=2))
    threads = cpu_cores()
    per_step_s = 3.0
    _, _, cols, _ = cpu_sample(A, B, per_step_s, threads)
    Bs = np.asfortranarray(B[:, :cols])
    for _ in range(args.warmup):
        oracle.jmul_tiled(A, Bs, nthreads=threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        oracle.jmul_tiled(A, Bs, nthreads=threads)
    dt = (time.perf_counter() - t0) / args.steps
    flops = 2.0 * n * n * cols
    v = flops / dt / 1e12
    sample = "each step C[:, :%d] of the %d^3 product (%.3g flop) on %d threads" % (cols, n, flops, threads)
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "TFLOP/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "gemm_fp64_%d^3" % n, "M": n, "N": n, "K": n,
                   "distribution": "sign*U[1,2)*2^(e_line+e_elem), e_line in [-30,30], e_elem in [-8,8]",
                   "algorithm": "jmul! FMA chain, register-tiled (oracle port; Julia reference cannot run)"},
        "cpu_baseline": {"value": v, "unit": "TFLOP/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": v, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return reference_arm(args, rank, world)

    import torch
    import gbblas
    from gbblas import workloads
    import __graft_entry__  # noqa: F401  (path setup only)

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    def max_over_ranks(x):
        if dist is None:
            return x
        t = torch.tensor([x], dtype=torch.float64, device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    n = args.size
    M = N = K = n
    flops = 2.0 * M * N * K
    A_h = np.asfortranarray(workloads.ozaki_matrix(M, K, per="row", stream=1 + 2 * rank))
    B_h = np.asfortranarray(workloads.ozaki_matrix(K, N, per="col", stream=2 + 2 * rank))

    def pinned_colmajor(X):
        t = torch.from_numpy(np.ascontiguousarray(X.T)).pin_memory()
        return t  # (cols, rows) row-major == column-major (rows, cols)

    A_pin, B_pin = pinned_colmajor(A_h), pinned_colmajor(B_h)
    C_pin = torch.empty((N, M), dtype=torch.float64).pin_memory()
    A_d = A_pin.to(dev).t()
    B_d = B_pin.to(dev).t()
    C_d = torch.empty((N, M), dtype=torch.float64, device=dev).t()
    stream = torch.cuda.current_stream(dev)

    # warm-up (also fixes the slice plan the library picks for these inputs)
    bound = None
    for _ in range(args.warmup):
        _, bound = gbblas.gemm_(C_d, A_d, B_d, mode="ozaki", slices=args.slices, return_bound=True)
    torch.cuda.synchronize()
    gbblas.check_device_status()
    C_oz = np.asfortranarray(C_d.cpu().numpy())

    # ---------------------------------------------------------------- timed: device-resident
    clocks = ClockSampler(torch.cuda.current_device()) if rank == 0 else None
    if clocks:
        clocks.start()
    counts0 = gbblas.launch_counts()
    barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with gbblas.profile() as prof:
        ev0.record(stream)
        for _ in range(args.steps):
            gbblas.gemm_(C_d, A_d, B_d, mode="ozaki", slices=args.slices)
        ev1.record(stream)
        torch.cuda.synchronize()
    barrier()
    counts1 = gbblas.launch_counts()
    clk = clocks.stop() if clocks else None
    ms_step = max_over_ranks(ev0.elapsed_time(ev1) / args.steps)
    gbblas.check_device_status()
    launches = sum(counts1.get(k, 0) - counts0.get(k, 0) for k in counts1)
    value = world * flops / (ms_step * 1e-3) / 1e12

    # ---------------------------------------------------------------- timed: end to end
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    A_e = torch.empty_like(A_pin, device=dev)
    B_e = torch.empty_like(B_pin, device=dev)
    e0.record(stream)
    for _ in range(args.steps):
        A_e.copy_(A_pin, non_blocking=True)
        B_e.copy_(B_pin, non_blocking=True)
        gbblas.gemm_(C_d, A_e.t(), B_e.t(), mode="ozaki", slices=args.slices)
        C_pin.copy_(C_d.t(), non_blocking=True)
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    ms_e2e = max_over_ranks(e0.elapsed_time(e1) / args.steps)
    e2e_value = world * flops / (ms_e2e * 1e-3) / 1e12

    plan = None
    line = None
    if rank == 0:
        plan = gbblas.last_ozaki_plan()   # the plan the automatic slice choice used
        mma_ms = prof.ms.get("ozaki_slice_mma", float("nan")) / max(1, prof.launches.get("ozaki_slice_mma", 1))
        peaks, peak_src = load_peaks()
        timed_s = ms_step * args.steps / 1e3
        peak_key = "bf16_tflops_sustained" if timed_s >= 1.0 else "bf16_tflops"
        achieved = plan["flops_tensor"] / (mma_ms * 1e-3) / 1e12
        traffic = committed_traffic("%d" % n)

        # ------------------------------------------------------------ accuracy and native
        import oracle
        g = np.random.default_rng(12345)
        rows, cols = g.integers(0, M, 4096), g.integers(0, N, 4096)
        hi, lo, _ = oracle.dot2_entries(A_h, B_h, rows, cols)
        err_oz = normwise_err(C_oz, A_h, B_h, rows, cols, hi, lo)
        native = None
        if not args.no_native:
            Cn = torch.empty_like(C_d.t()).t()
            gbblas.gemm_(Cn, A_d, B_d, mode="native")
            torch.cuda.synchronize()
            n0, n1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            n0.record(stream)
            gbblas.gemm_(Cn, A_d, B_d, mode="native")
            n1.record(stream)
            torch.cuda.synchronize()
            nat_ms = n0.elapsed_time(n1)
            C_nat = np.asfortranarray(Cn.cpu().numpy())
            err_nat = normwise_err(C_nat, A_h, B_h, rows, cols, hi, lo)
            native = {"tflops": flops / (nat_ms * 1e-3) / 1e12, "ms": nat_ms, "normwise_err": err_nat,
                      "ozaki_speedup": (flops / (ms_step * 1e-3) / 1e12) / (flops / (nat_ms * 1e-3) / 1e12)}
        cpu = None
        if not args.no_cpu and world == 1:
            threads = cpu_cores()
            v, sample, _, _ = cpu_sample(A_h, B_h, args.cpu_seconds, threads)
            cpu = {"value": v, "unit": "TFLOP/s", "cores": threads, "kind": "port", "sample": sample}

        line = {
            "metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "ozaki_fp64_gemm_%d^3" % n, "M": M, "N": N, "K": K,
                       "distribution": "sign*U[1,2)*2^(e_line+e_elem), e_line in [-30,30] per row/col, "
                                       "e_elem in [-8,8]",
                       "slices": plan["slices"], "bits": plan["bits"], "slice_products": plan["products"],
                       "accumulation_groups": plan["groups"], "alpha": 1.0, "beta": 0.0,
                       "parallelism": "replicas" if world > 1 else "single",
                       "l2": "inputs larger than L2 (512 MiB per operand)"},
            "accuracy": {"normwise_err": err_oz, "bound": bound,
                         "metric": "||C - C_ref||_F / (||A||_F ||B||_F), 4096 sampled entries vs Dot2"},
            "native_fp64": native,
            "roofline": {"bound": "tensor", "achieved": achieved, "peak": peaks[peak_key], "unit": "TFLOP/s",
                         "frac": achieved / peaks[peak_key], "traffic": traffic,
                         "kernel": "ozaki_slice_mma", "ms_per_launch": mma_ms,
                         "peak_source": "%s %s" % (peak_src, peak_key),
                         "work": "BF16 tensor flops per launch = slice_products * 2*M*N*ceil(K/64)*64"},
            "kernel_ms_per_step": {k: v / args.steps for k, v in prof.ms.items()},
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": "TFLOP/s", "ms_per_step": ms_e2e,
                    "h2d_bytes_per_step": int(A_pin.numel() * 8 + B_pin.numel() * 8),
                    "d2h_bytes_per_step": int(C_pin.numel() * 8)},
            "gpu_launches": launches,
            "clocks": clk,
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
