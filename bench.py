#!/usr/bin/env python
"""FP64-accurate GEMM throughput on GB300: Ozaki emulation on BF16 tensor cores vs native FP64.

Workload (default): C = A * B, M = N = K = 8192, float64, A and B from the emulated-FP64
configuration (sign * U[1,2) * 2^(e_line + e_elem), e_line in [-30, 30] per row of A /
column of B, e_elem in [-8, 8] per element; seeded, synthetic), emulated by the CRT method
(--method crt: exact integer product of t-bit scaled operands from BF16 residue products
modulo n coprime moduli) or by digit slices (--method slices); moduli / slices and t chosen
per problem by the library (slices = 0) to meet its normwise tolerance.

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
import datetime
import json
import os
import statistics
import subprocess
import tempfile
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
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["gbblas", "reference"], default="gbblas")
    p.add_argument("--size", type=int, default=8192)
    p.add_argument("--mnk", type=str, default=None, help="M,N,K override of --size (profiling cases)")
    p.add_argument("--slices", type=int, default=0,
                   help="digit slices (slice method) or moduli (crt method); 0 = automatic (library tolerance)")
    p.add_argument("--method", choices=["crt", "slices"], default="crt",
                   help="FP64 emulation: residue products + Chinese remainder theorem, or digit slices")
    p.add_argument("--no-alt", action="store_true", help="skip timing the other emulation method")
    p.add_argument("--no-native", action="store_true", help="skip the native FP64 comparison")
    p.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    p.add_argument("--ring", type=int, default=8,
                   help="depth of the end-to-end pipeline's ring of device input / output buffers")
    p.add_argument("--cpu-seconds", type=float, default=12.0, help="target length of the CPU sample")
    p.add_argument("--workload", choices=["ozaki", "ozaki_sweep", "native", "f32_tc", "grouped", "adjoint",
                                          "semiring"],
                   default="ozaki",
                   help="ozaki: the headline (default); ozaki_sweep: error and TFLOP/s by slice / moduli count; "
                        "native: FP64/FP32 sweep; f32_tc: FP32 on tensor cores; grouped: 4096 uneven problems; adjoint: fused dA/dB; "
                        "semiring: (min, +) and relatives")
    return p.parse_args()


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except (OSError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def committed_traffic(method, n):
    """DRAM bytes per launch of the tensor-core product kernel from the committed ncu summary: the
    4096 x 4096 x 8192 capture scaled to n^3 by the pair tiles one launch processes (only n = 8192
    is recorded there)."""
    name = {"crt": "ozaki_crt_launch_list_4096x4096x8192.md", "slices": "ozaki_slices_launch_list_4096x4096x8192.md"}
    path = os.path.join(ROOT, "profiles", name.get(method, ""))
    try:
        with open(path) as f:
            for line in f:
                if line.startswith("dram_bytes_per_launch_scaled_%d:" % n):
                    return float(line.split(":", 1)[1].split()[0])
    except OSError:
        pass
    return None


class ClockSampler:
    """nvidia-smi clock / throttle-reason samples while the timed region runs."""

    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.dev = device_index
        self.proc = None
        self.window = None   # host wall-clock (start, end) of the timed region
        self.path = os.path.join(tempfile.gettempdir(), "gbblas_clocks_%d.csv" % os.getpid())

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=self.fh, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)

    def mark_start(self):
        self.window = (time.time(), None)

    def mark_end(self):
        if self.window:
            self.window = (self.window[0], time.time())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.fh.close()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 10:
                    continue
                try:
                    ts = datetime.datetime.strptime(parts[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
                    rows.append((ts, float(parts[2]), float(parts[3]),
                                 {nm for nm, v in zip(names, parts[6:10]) if v.lower() == "active"}))
                except ValueError:
                    continue
        if not rows:
            return None
        scope = "whole run"
        if self.window and self.window[1]:
            inside = [r for r in rows if self.window[0] - 0.05 <= r[0] <= self.window[1] + 0.05]
            if inside:
                rows, scope = inside, "timed region"
        sm = [r[1] for r in rows]
        reasons = set().union(*(r[3] for r in rows))
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(r[2] for r in rows), "samples": len(rows),
                "scope": scope, "reasons": sorted(reasons)}


def cpu_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_sample(A, B, target_s, threads, runs=5):
    """Time jmul!'s register-tiled chain (the tile pick_kernel_size gives for this host's register
    file) on a column sample of A*B: `runs` timed runs of a sample sized to target_s / runs
    seconds each; TFLOP/s of the median run, description, columns, seconds of the median run.
    The sample's result is checked against the scalar chain on 64 entries (the port must compute
    jmul!'s arithmetic, not only take its time)."""
    import oracle
    n = A.shape[0]
    K = A.shape[1]
    tr, tc = oracle.host_tile(np.float64)
    cols = max(tc, min(B.shape[1], 8 * tc))
    t0 = time.perf_counter()
    oracle.jmul_tiled(A, np.asfortranarray(B[:, :cols]), nthreads=threads)
    dt = time.perf_counter() - t0
    cols = int(min(B.shape[1], max(tc, cols * target_s / runs / max(dt, 1e-6))))
    cols -= cols % tc
    Bs = np.asfortranarray(B[:, :cols])
    times = []
    for _ in range(runs):
        t0 = time.perf_counter()
        out = oracle.jmul_tiled(A, Bs, nthreads=threads)
        times.append(time.perf_counter() - t0)
    dt = statistics.median(times)
    g = np.random.default_rng(5)
    ri, ci = g.integers(0, n, 64), g.integers(0, cols, 64)
    if not np.array_equal(out[ri, ci].view(np.uint64), oracle.chain_entries(A, Bs, ri, ci).view(np.uint64)):
        raise RuntimeError("CPU baseline result differs from jmul!'s chain")
    flops = 2.0 * n * K * cols
    return flops / dt / 1e12, ("C[:, :%d] of the %dx%dx%d product (%.3g flop), median of %d runs %.2f s "
                               "(%s s), %dx%d register tile") % (
        cols, n, K, B.shape[1], flops, runs, dt, ", ".join("%.2f" % x for x in times), tr, tc), cols, dt


def reference_shape_timing():
    """jmul! at the one shape the reference publishes a time for: D 16x14 = A 16x32 * X 32x14
    Float64, minimum 127.921 ns (test/runtests.jl:103-116, single thread).  The port on one
    core, with this host's pick_kernel_size tile (remainder rows and columns by the scalar
    chain) and with one 16x14 tile covering D, as the reference's benchmark kernel did."""
    import oracle
    g = np.random.default_rng(16)
    A = np.asfortranarray(g.standard_normal((16, 32)))
    X = np.asfortranarray(g.standard_normal((32, 14)))
    flops = 2.0 * 16 * 32 * 14
    out = {"shape": "16x32x14 (M x K x N)", "reference_min_ns": 127.921,
           "reference_gflops": flops / 127.921}
    for name, tile in (("host_tile", None), ("tile_16x14", (16, 14))):
        ns = oracle.time_jmul_tiled(A, X, tile=tile)
        out[name] = {"tile": list(tile or oracle.host_tile(np.float64)), "min_ns": ns, "gflops": flops / ns}
    return out


def normwise_err(Cres, A, B, rows, cols, hi, lo):
    d = (Cres[rows, cols] - hi) - lo
    scale = np.sqrt(Cres.size / rows.size)
    return float(np.linalg.norm(d) * scale / (np.linalg.norm(A) * np.linalg.norm(B)))


def componentwise_err(Cres, rows, cols, hi, lo, ab):
    """max over the sampled entries of |C - C_ref|_ij / (|A||B|)_ij."""
    d = np.abs((Cres[rows, cols] - hi) - lo)
    ok = ab > 0
    return float(np.max(d[ok] / ab[ok])) if ok.any() else 0.0


def headline_config(M, N, K, world):
    """The workload both arms run (identical dicts): sizes, input distribution, alpha/beta."""
    square = M == N == K
    return {"workload": ("ozaki_fp64_gemm_%d^3" % M) if square else "ozaki_fp64_gemm_%dx%dx%d" % (M, N, K),
            "M": M, "N": N, "K": K,
            "distribution": "sign*U[1,2)*2^(e_line+e_elem), e_line in [-30,30] per row/col, e_elem in [-8,8]",
            "alpha": 1.0, "beta": 0.0, "parallelism": "replicas" if world > 1 else "single",
            "l2": "inputs larger than L2 (%d MiB per operand)" % (M * K * 8 // 2 ** 20)}


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
    _, _, cols, _ = cpu_sample(A, B, per_step_s, threads, runs=1)
    Bs = np.asfortranarray(B[:, :cols])
    for _ in range(args.warmup):
        oracle.jmul_tiled(A, Bs, nthreads=threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        oracle.jmul_tiled(A, Bs, nthreads=threads)
    dt = (time.perf_counter() - t0) / args.steps
    flops = 2.0 * n * n * cols
    v = flops / dt / 1e12
    tr, tc = oracle.host_tile(np.float64)
    sample = "each step C[:, :%d] of the %d^3 product (%.3g flop) on %d threads, %dx%d register tile" % (
        cols, n, flops, threads, tr, tc)
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "TFLOP/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": headline_config(n, n, n, world),
        "algorithm": "jmul! FMA chain, register-tiled (oracle port; the Julia reference cannot run)",
        "cpu_baseline": {"value": v, "unit": "TFLOP/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": v, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def pipeline_timeline(e0, up_ev, comp_ev, down_ev, nbuf, host_enqueue_ms):
    """Per-step timeline of the end-to-end ring (ms from the start event): for each step the
    compute stream's idle time before it and what it waited on — its upload, the previous
    step's compute, the download that frees its ring slot, or the host (the launch arrived
    after every dependency had finished).  Also the uploads' overlap with compute."""
    T = lambda ev: (e0.elapsed_time(ev[0]), e0.elapsed_time(ev[1]))   # noqa: E731
    up, comp, down = [T(x) for x in up_ev], [T(x) for x in comp_ev], [T(x) for x in down_ev]
    steps = len(comp)
    waited = {"upload": 0, "previous_compute": 0, "ring_download": 0, "host": 0}
    idle, rows = [], []
    for i in range(steps):
        deps = {"upload": up[i][1], "previous_compute": comp[i - 1][1] if i else 0.0}
        if i >= nbuf:
            deps["ring_download"] = down[i - nbuf][1]
        cause = max(deps, key=deps.get)
        if comp[i][0] - deps[cause] > 0.05:
            cause = "host"
        waited[cause] += 1
        gap = comp[i][0] - (comp[i - 1][1] if i else 0.0)
        if i:
            idle.append(gap)
        rows.append({"step": i, "upload": [round(up[i][0], 3), round(up[i][1], 3)],
                     "compute": [round(comp[i][0], 3), round(comp[i][1], 3)],
                     "download": [round(down[i][0], 3), round(down[i][1], 3)],
                     "compute_idle_before_ms": round(gap, 3), "waited_on": cause,
                     "host_enqueued_ms": round(host_enqueue_ms[i], 3)})
    # milliseconds of upload time that ran while some compute interval was active
    overlap = 0.0
    for a, z in up:
        for c0, c1 in comp:
            overlap += max(0.0, min(z, c1) - max(a, c0))
    up_total = sum(z - a for a, z in up)
    # every step after the first whose compute waited more than 0.5 ms, with its upload's length
    stalls = [{"step": r["step"], "idle_ms": r["compute_idle_before_ms"], "waited_on": r["waited_on"],
               "upload_ms": round(up[r["step"]][1] - up[r["step"]][0], 3)}
              for r in rows[1:] if r["compute_idle_before_ms"] > 0.5]
    return {"compute_idle_ms_median": statistics.median(idle) if idle else 0.0,
            "compute_idle_ms_total": sum(idle), "waited_on": waited,
            "upload_overlapped_with_compute_frac": overlap / up_total if up_total else 0.0,
            "upload_ms_max": round(max(z - a for a, z in up), 3) if up else 0.0,
            "stalls": stalls, "steps": rows[:8]}


def _event_ms(fn, steps, stream):
    import torch
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def _side_line(args, metric, value, unit, ms, config, extra):
    line = {"metric": metric, "value": value, "unit": unit, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "data": "synthetic", "config": config}
    line.update(extra)
    print(json.dumps(line), flush=True)


def _native_sample_error(A, B, alpha, beta, dt, samples=1024):
    """Errors of one fresh call C = alpha A B + beta C0 against Dot2 on sampled entries:
    normwise ||dC|| sqrt(MN/s) / (|alpha| ||A||_F ||B||_F + |beta| ||C0||_F) and componentwise
    max |dC|_ij / (|alpha| (|A||B|)_ij + |beta| |C0|_ij) (FP64 references for both dtypes)."""
    import torch
    import gbblas
    import oracle
    M, K = A.shape
    N = B.shape[1]
    g = np.random.default_rng(M + 3 * N + 7 * K)
    rows, cols = g.integers(0, M, samples), g.integers(0, N, samples)
    C0 = (torch.rand((N, M), dtype=dt, device=A.device) * 2 - 1).t()
    C1 = C0.clone()
    gbblas.gemm_(C1, A, B, alpha, beta)
    torch.cuda.synchronize()
    ri, ci = torch.from_numpy(rows).to(A.device), torch.from_numpy(cols).to(A.device)
    As = np.asfortranarray(A[ri, :].double().cpu().numpy())
    Bs = np.asfortranarray(B[:, ci].double().cpu().numpy())
    idx = np.arange(samples)
    hi, lo, ab = oracle.dot2_entries(As, Bs, idx, idx)
    c0 = C0[ri, ci].double().cpu().numpy()
    got = C1[ri, ci].double().cpu().numpy()
    d = np.abs((got - alpha * hi) - (alpha * lo + beta * c0))
    na = float(torch.linalg.norm(A.double()))
    nb = float(torch.linalg.norm(B.double()))
    nc = float(torch.linalg.norm(C0.double()))
    normwise = float(np.linalg.norm(d) * np.sqrt(M * N / samples) / (abs(alpha) * na * nb + abs(beta) * nc))
    den = abs(alpha) * ab + abs(beta) * np.abs(c0)
    ok = den > 0
    comp = float(np.max(d[ok] / den[ok])) if ok.any() else 0.0
    return {"normwise_err": normwise, "componentwise_err": comp}


def workload_native(args):
    """Native FP64 / FP32 GEMM sweep (square 1024..16384, 16384x64x16384, 64x16384x16384), alpha = 1.5, beta = 0.5, uniform[-1, 1)."""
    import torch
    import gbblas
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    shapes = [(n, n, n) for n in (1024, 2048, 4096, 8192, 16384)] + [(16384, 64, 16384), (64, 16384, 16384)]
    rows = []
    for dt in (torch.float64, torch.float32):
        for (M, N, K) in shapes:
            if dt == torch.float64 and M * N * K > 8192 ** 3 and args.steps > 1:
                steps = 1
            else:
                steps = args.steps
            A = torch.rand((K, M), dtype=dt, device=dev).t() * 2 - 1
            B = torch.rand((N, K), dtype=dt, device=dev).t() * 2 - 1
            C = torch.rand((N, M), dtype=dt, device=dev).t() * 2 - 1
            A, B, C = (x.t().contiguous().t() for x in (A, B, C))
            gbblas.gemm_(C, A, B, 1.5, 0.5)
            torch.cuda.synchronize()
            ms = _event_ms(lambda: gbblas.gemm_(C, A, B, 1.5, 0.5), steps, stream)
            err = _native_sample_error(A, B, 1.5, 0.5, dt)
            rows.append({"dtype": str(dt).replace("torch.", ""), "M": M, "N": N, "K": K, "ms": ms,
                         "tflops": 2.0 * M * N * K / (ms * 1e-3) / 1e12, **err})
            del A, B, C
    f64 = [r for r in rows if r["dtype"] == "float64" and r["M"] == r["N"] == r["K"] == 8192][0]
    pk = gbblas.measure_fma_peaks()
    for r in rows:
        r["frac_of_measured_pipe"] = r["tflops"] / pk["fp64_tflops" if r["dtype"] == "float64" else "fp32_tflops"]
    _side_line(args, "native FP64 GEMM TFLOP/s (CUDA cores, jmul! FMA order)", f64["tflops"], "TFLOP/s",
               f64["ms"], {"workload": "native_gemm_sweep", "alpha": 1.5, "beta": 0.5,
                           "headline_shape": "f64 8192^3"},
               {"dtype": "f64", "sweep": rows, "fma_peaks": pk,
                "roofline": {"bound": "fp64_pipe", "achieved": f64["tflops"], "peak": pk["fp64_tflops"],
                             "unit": "TFLOP/s", "frac": f64["tflops"] / pk["fp64_tflops"],
                             "peak_source": "measured DFMA register loop (gb_measure_fma_peaks)"}})
    return 0


# Instructions per output element and k of each semiring's mainloop step, and the share of
# them on the 64-lane min/max (ALU) pipe; the rest (add, mul) issue on the 128-lane FMA pipe.
# Paired steps fold two k into one three-input min/max (float: all; int32: max-min, min-max).
_SR_INSTR = {("float32", "min_plus"): (1.5, 0.5), ("float32", "max_plus"): (1.5, 0.5),
             ("float32", "max_times"): (1.5, 0.5), ("float32", "max_min"): (1.5, 1.5),
             ("float32", "min_max"): (1.5, 1.5), ("int32", "max_min"): (1.5, 1.5),
             ("int32", "min_max"): (1.5, 1.5)}


def _sr_bound(dtype, sr, sms, mhz):
    """Issue bound in 1e12 semiring multiply-adds (M N K) per second: each SM issues 4 x 32
    lanes per clock, and min/max run on a 64-lane pipe."""
    if dtype == "float64":
        return None
    instr, alu = _SR_INSTR.get((dtype, sr), (2.0, 1.0))
    per_clk = min(128.0 / instr, 64.0 / alu)
    return sms * per_clk * mhz * 1e6 / 1e12


def workload_semiring(args):
    """Semiring GEMM sweep (no counterpart in the reference's code; jBLAS names min-plus algebra
    as the use of its Vec fallback, src/jBLAS.jl:10): every semiring in float32 and int32 at
    8192^3 and float64 at 4096^3, A, B uniform, each checked bit for bit against the oracle on
    32 x 32 sampled outputs."""
    import torch
    import gbblas
    import oracle
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    clocks = ClockSampler(0)
    rows = []
    clocks.start()
    clocks.mark_start()
    for dt, n in ((torch.float32, 8192), (torch.int32, 8192), (torch.float64, 4096)):
        if dt == torch.int32:
            A = torch.randint(-10**6, 10**6, (n, n), dtype=dt, device=dev).t()
            B = torch.randint(-10**6, 10**6, (n, n), dtype=dt, device=dev).t()
        else:
            A = (torch.rand((n, n), dtype=dt, device=dev) * 200 - 100).t()
            B = (torch.rand((n, n), dtype=dt, device=dev) * 200 - 100).t()
        C = torch.empty((n, n), dtype=dt, device=dev).t()
        g = np.random.default_rng(n)
        ri = np.sort(g.choice(n, 32, replace=False))
        ci = np.sort(g.choice(n, 32, replace=False))
        As = np.asfortranarray(A[torch.as_tensor(ri, device=dev), :].cpu().numpy())
        Bs = np.asfortranarray(B[:, torch.as_tensor(ci, device=dev)].cpu().numpy())
        steps = max(1, min(args.steps, 3)) if dt == torch.float64 else args.steps
        for sr in ("min_plus", "max_plus", "max_min", "min_max", "max_times"):
            gbblas.gemm_semiring_(C, A, B, sr)
            torch.cuda.synchronize()
            ms = _event_ms(lambda: gbblas.gemm_semiring_(C, A, B, sr), steps, stream)
            got = C[torch.as_tensor(ri, device=dev)][:, torch.as_tensor(ci, device=dev)].cpu().numpy()
            ref = oracle.semiring_gemm(As, Bs, sr, dtype=As.dtype)
            same = bool(np.array_equal(got, ref))
            rows.append({"dtype": str(dt).replace("torch.", ""), "semiring": sr, "n": n, "ms": ms,
                         "tera_mnk_per_s": n ** 3 / (ms * 1e-3) / 1e12, "sampled_bit_exact": same})
        del A, B, C
    clocks.mark_end()
    clk = clocks.stop() or {}
    mhz = clk.get("sm_mhz") or 2070.0
    for r in rows:
        bound = _sr_bound(r["dtype"], r["semiring"], sms, mhz)
        r["issue_bound"] = bound
        r["frac"] = r["tera_mnk_per_s"] / bound if bound else None
    head = [r for r in rows if r["dtype"] == "float32" and r["semiring"] == "min_plus"][0]
    _side_line(args, "semiring GEMM 1e12 (min,+) multiply-adds/s, float32 8192^3", head["tera_mnk_per_s"],
               "T(min,+)/s", head["ms"],
               {"workload": "semiring_gemm_sweep", "inputs": "uniform [-100, 100) / int32 [-1e6, 1e6)",
                "headline_shape": "f32 min_plus 8192^3"},
               {"dtype": "f32", "sweep": rows, "clocks": clk,
                "roofline": {"bound": "issue", "achieved": head["tera_mnk_per_s"], "peak": head["issue_bound"],
                             "unit": "T(min,+)/s", "frac": head["frac"],
                             "peak_source": "%d SMs x 128 lanes/clk / 1.5 instructions per element x %.0f MHz "
                                            "(median SM clock sampled during the sweep)" % (sms, mhz)}})
    return 0


def workload_grouped(args):
    """4096 problems, m, n, k log-uniform in [8, 512], one persistent grouped launch in a
    CUDA graph with autotuned tiles, against a loop of plain per-problem launches."""
    import torch
    import gbblas
    from gbblas import grouped, workloads
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    sizes = [tuple(int(x) for x in r) for r in workloads.grouped_sizes(4096)]
    out = {}
    for dt in (torch.float64, torch.float32):
        As, Bs, Cs = [], [], []
        for m, n, k in sizes:
            As.append((torch.rand((k, m), dtype=dt, device=dev) * 2 - 1).t())
            Bs.append((torch.rand((n, k), dtype=dt, device=dev) * 2 - 1).t())
            Cs.append(torch.empty((n, m), dtype=dt, device=dev).t())
        plan = grouped.GroupedGemm(As, Bs, Cs)
        flops = plan.flops()
        default_ms = _event_ms(plan.run, max(1, args.steps), stream)
        cache = os.path.join(tempfile.gettempdir(), "gbblas_grouped_tuning_%d.json" % os.getpid())
        tuning, class_ms = grouped.autotune(plan, reps=3, cache=cache)
        plan.tuning = tuning
        graph = plan.capture()
        for _ in range(args.warmup):
            graph.replay()
        torch.cuda.synchronize()
        graph_ms = _event_ms(graph.replay, args.steps, stream)

        def loop():
            for A, B, C in zip(As, Bs, Cs):
                gbblas.gemm_(C, A, B)
        loop()
        torch.cuda.synchronize()
        loop_ms = _event_ms(loop, 1, stream)            # eager: 4096 C-ABI calls from the host
        g2 = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g2):
            loop()                                      # the same 4096 launches, replayed as a graph
        g2.replay()
        torch.cuda.synchronize()
        loop_graph_ms = _event_ms(g2.replay, args.steps, stream)
        out[str(dt).replace("torch.", "")] = {
            "flops": flops, "graph_ms": graph_ms, "graph_tflops": flops / (graph_ms * 1e-3) / 1e12,
            "default_tuning_ms": default_ms, "loop_ms": loop_ms, "loop_graph_ms": loop_graph_ms,
            "loop_graph_tflops": flops / (loop_graph_ms * 1e-3) / 1e12,
            "speedup_vs_loop_graph": loop_graph_ms / graph_ms, "tuning": tuning.as_list(),
            "class_ms": class_ms}
        del g2
        del As, Bs, Cs, plan, graph
    f64 = out["float64"]
    pk = gbblas.measure_fma_peaks()
    out["float32"]["frac_of_measured_fp32_pipe"] = out["float32"]["graph_tflops"] / pk["fp32_tflops"]
    _side_line(args, "grouped FP64 GEMM TFLOP/s, 4096 uneven problems, one persistent launch in a CUDA graph",
               f64["graph_tflops"], "TFLOP/s", f64["graph_ms"],
               {"workload": "grouped_4096_loguniform_8_512", "count": 4096, "alpha": 1.0, "beta": 0.0},
               {"dtype": "f64", "results": out, "fma_peaks": pk,
                "roofline": {"bound": "fp64_pipe", "achieved": f64["graph_tflops"], "peak": pk["fp64_tflops"],
                             "unit": "TFLOP/s", "frac": f64["graph_tflops"] / pk["fp64_tflops"],
                             "peak_source": "measured DFMA register loop (gb_measure_fma_peaks)"},
            "gpu_launches": 2 * args.steps})
    return 0


def workload_ozaki_sweep(args):
    """Emulated FP64 at 8192^3 on the sign*U[1,2)*2^(e_line+e_elem) inputs, by slice and moduli
    count: digit slices s = 3..8 (BF16 digit products, FP32 accumulation) and the automatic s;
    CRT moduli n = 8..16 and the automatic n; native FP64 beside them.  Per plan: TFLOP/s
    (FP64-equivalent 2MNK over the CUDA-event step time), the a-priori bound the call returns,
    and the normwise error against binary128 dot products on a 64 x 64 grid of outputs."""
    import torch
    import gbblas
    import oracle
    from gbblas import workloads
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    n = args.size
    A = np.asfortranarray(workloads.ozaki_matrix(n, n, per="row", stream=1))
    B = np.asfortranarray(workloads.ozaki_matrix(n, n, per="col", stream=2))
    g = np.random.default_rng(77)
    r = np.sort(g.choice(n, 64, replace=False))
    c = np.sort(g.choice(n, 64, replace=False))
    ii, jj = (x.ravel() for x in np.meshgrid(np.arange(64), np.arange(64), indexing="ij"))
    hi, lo = oracle.quad_entries(np.asfortranarray(A[r, :]), np.asfortranarray(B[:, c]), ii, jj)
    na, nb = float(np.linalg.norm(A)), float(np.linalg.norm(B))

    def dev_cm(x):
        return torch.from_numpy(np.ascontiguousarray(x.T)).to(dev).t()
    Ad, Bd = dev_cm(A), dev_cm(B)
    del A, B
    C = torch.empty((n, n), dtype=torch.float64, device=dev).t()
    rt, ct = torch.as_tensor(r, device=dev), torch.as_tensor(c, device=dev)
    flops = 2.0 * n ** 3

    def err_of():
        got = C[rt][:, ct].cpu().numpy()[ii, jj]
        return float(np.linalg.norm((got - hi) - lo) * np.sqrt(n * n / ii.size) / (na * nb))

    rows = []
    cases = [("native", 0)] + [("ozaki", s) for s in (3, 4, 5, 6, 7, 8, 0)] + \
            [("ozaki_crt", m) for m in (8, 9, 10, 11, 12, 13, 14, 15, 16, 0)]
    for mode, cnt in cases:
        steps = 1 if mode == "native" else args.steps
        _, bound = gbblas.gemm_(C, Ad, Bd, mode=mode, slices=cnt, return_bound=True)
        torch.cuda.synchronize()
        gbblas.check_device_status()
        err = err_of()
        plan = gbblas.last_ozaki_plan() if mode != "native" else None
        ms = _event_ms(lambda: gbblas.gemm_(C, Ad, Bd, mode=mode, slices=cnt), steps, stream)
        row = {"method": {"native": "native_fp64", "ozaki": "slices", "ozaki_crt": "crt"}[mode],
               "requested": cnt if mode != "native" else None, "ms": ms,
               "tflops": flops / (ms * 1e-3) / 1e12, "bound": bound, "normwise_err": err}
        if plan:
            row.update({"slices_or_moduli": plan["slices"], "bits": plan["bits"],
                        "tensor_products": plan["products"]})
        rows.append(row)
    auto = [x for x in rows if x["method"] == "crt" and x["requested"] == 0][0]
    _side_line(args, "FP64-accurate GEMM TFLOP/s by slice and moduli count, 8192^3", auto["tflops"], "TFLOP/s",
               auto["ms"], {"workload": "ozaki_fp64_gemm_%d^3_sweep" % n, "M": n, "N": n, "K": n,
                            "distribution": "sign*U[1,2)*2^(e_line+e_elem), e_line in [-30,30] per row/col, "
                                            "e_elem in [-8,8]"},
               {"dtype": "f64", "sweep": rows,
                "error_metric": "||C - C_ref||_F / (||A||_F ||B||_F) estimated on a 64 x 64 output grid against "
                                "binary128 dot products"})
    return 0


def workload_f32_tc(args):
    """FP32 GEMM at 8192^3 on N(0,1) inputs: the tensor-core term modes (BF16X3: 3 BF16 products,
    BF16X6: 6) beside the bit-exact native FP32 mode; TFLOP/s (useful 2MNK flops), componentwise
    error max |C - C_ref| / (|A||B|) on a 64 x 64 output grid against Dot2, and the MMA kernel's
    BF16 tensor rate (products x 2MNK over its CUDA-event time) against the measured peak."""
    import torch
    import gbblas
    import oracle
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    n = args.size
    gen = torch.Generator(device=dev).manual_seed(8192)
    A = torch.randn((n, n), generator=gen, dtype=torch.float32, device=dev).t()
    B = torch.randn((n, n), generator=gen, dtype=torch.float32, device=dev).t()
    C = torch.empty((n, n), dtype=torch.float32, device=dev).t()
    g = np.random.default_rng(9)
    r = np.sort(g.choice(n, 64, replace=False))
    c = np.sort(g.choice(n, 64, replace=False))
    rt, ct = torch.as_tensor(r, device=dev), torch.as_tensor(c, device=dev)
    ii, jj = (x.ravel() for x in np.meshgrid(np.arange(64), np.arange(64), indexing="ij"))
    hi, lo, ab = oracle.dot2_entries(np.asfortranarray(A[rt].double().cpu().numpy()),
                                     np.asfortranarray(B[:, ct].double().cpu().numpy()), ii, jj)
    peaks, src = load_peaks()
    flops = 2.0 * n ** 3
    rows = []
    from gbblas import tuning
    cls = tuning.size_class(n, n)
    # the FP32 epilogue's two store paths, same bits: direct stores and TMA stores of C
    epilogue = {}
    for mode in ("bf16x3", "bf16x6"):
        for tma in (0, 1):
            tuning.set_tuning("f32", cls, {"engine": 2, "band": 8, "tma_store": tma})
            gbblas.gemm_(C, A, B, mode=mode)
            torch.cuda.synchronize()
            with gbblas.profile() as prof:
                ms_t = _event_ms(lambda: gbblas.gemm_(C, A, B, mode=mode), args.steps, stream)
            epilogue["%s_%s" % (mode, "tma_store" if tma else "direct")] = {
                "ms": ms_t, "mma_ms": prof.ms.get("f32_mma", float("nan")) / max(1, prof.launches.get("f32_mma", 1))}
    tuning.set_tuning("f32", cls, None)
    tuned, tuned_ms = tuning.autotune("f32", n, n, n, reps=3, install=False)
    for mode, products in (("native", 0), ("bf16x3", 3), ("bf16x6", 6)):
        steps = max(1, min(args.steps, 3)) if mode == "native" else args.steps
        for _ in range(max(1, args.warmup if mode != "native" else 1)):
            gbblas.gemm_(C, A, B, mode=mode)
        torch.cuda.synchronize()
        got = C[rt][:, ct].double().cpu().numpy()[ii, jj]
        err = float(np.max(np.abs((got - hi) - lo) / ab))
        with gbblas.profile() as prof:
            ms = _event_ms(lambda: gbblas.gemm_(C, A, B, mode=mode), steps, stream)
        row = {"mode": mode, "ms": ms, "tflops": flops / (ms * 1e-3) / 1e12, "componentwise_err": err,
               "kernel_ms_per_step": {k: v / steps for k, v in prof.ms.items()}}
        if products:
            mma_ms = prof.ms.get("f32_mma", float("nan")) / max(1, prof.launches.get("f32_mma", 1))
            tensor = products * 2.0 * n * n * (-(-n // 64) * 64)
            row["roofline"] = {"bound": "tensor", "achieved": tensor / (mma_ms * 1e-3) / 1e12,
                               "peak": peaks["bf16_tflops"], "unit": "TFLOP/s",
                               "frac": tensor / (mma_ms * 1e-3) / 1e12 / peaks["bf16_tflops"],
                               "peak_source": "%s bf16_tflops" % src, "kernel": "f32_mma", "ms_per_launch": mma_ms}
        rows.append(row)
    head = [x for x in rows if x["mode"] == "bf16x6"][0]
    _side_line(args, "FP32 GEMM TFLOP/s on tensor cores (BF16 term products), 8192^3", head["tflops"], "TFLOP/s",
               head["ms"], {"workload": "f32_gemm_%d^3" % n, "M": n, "N": n, "K": n, "inputs": "N(0,1)",
                            "alpha": 1.0, "beta": 0.0},
               {"dtype": "f32", "modes": rows, "roofline": head["roofline"], "epilogue_store_paths": epilogue,
                "autotuned": {"tuning": tuned.as_dict(), "ms_bf16x3": tuned_ms},
                "error_metric": "max |C - C_ref|_ij / (|A||B|)_ij on a 64 x 64 output grid against Dot2"})
    return 0


def workload_adjoint(args):
    """Adjoint: loss = sum(W .* (A*B)), A 4096x2048, B 2048x4096, W 4096x4096 N(0,1) float32:
    dA = W B^T and dB = A^T W in one launch (3xBF16 split, FP32 accumulation)."""
    import torch
    import gbblas
    from gbblas import workloads
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    M, K, N = 4096, 2048, 4096

    def dev_cm(x):
        return torch.from_numpy(np.ascontiguousarray(x.T)).to(dev).t()
    A = dev_cm(workloads.normal(M, K, stream=51))
    B = dev_cm(workloads.normal(K, N, stream=52))
    W = dev_cm(workloads.normal(M, N, stream=53))
    dA = torch.empty((K, M), dtype=torch.float32, device=dev).t()
    dB = torch.empty((N, K), dtype=torch.float32, device=dev).t()
    from gbblas import tuning
    cls = tuning.size_class(M, M)
    store_paths = {}
    for tma in (1, 0):   # the default (direct stores) last: its profile is the reported one
        tuning.set_tuning("adjoint", cls, {"engine": 2, "band": 8, "tma_store": tma})
        for _ in range(args.warmup):
            gbblas.gemm_adjoint_(dA, dB, A, B, W)
        torch.cuda.synchronize()
        with gbblas.profile() as prof:
            ms = _event_ms(lambda: gbblas.gemm_adjoint_(dA, dB, A, B, W), args.steps, stream)
        store_paths["tma_store" if tma else "direct"] = {
            "ms": ms, "mma_ms": prof.ms.get("adjoint_mma", float("nan")) / max(1, prof.launches.get("adjoint_mma", 1))}
    tuning.set_tuning("adjoint", cls, None)
    useful = 2 * 2.0 * M * N * K
    tensor = 3 * useful
    mma_ms = prof.ms.get("adjoint_mma", float("nan")) / max(1, prof.launches.get("adjoint_mma", 1))
    peaks, src = load_peaks()
    achieved = tensor / (mma_ms * 1e-3) / 1e12
    _side_line(args, "adjoint dA = dC*B^T and dB = A^T*dC (one launch) TFLOP/s", useful / (ms * 1e-3) / 1e12,
               "TFLOP/s", ms, {"workload": "adjoint_4096x2048x4096_f32", "M": M, "K": K, "N": N,
                                "split": "3xBF16, FP32 accumulation"},
               {"dtype": "f32", "kernel_ms_per_step": {k: v / args.steps for k, v in prof.ms.items()},
                "epilogue_store_paths": store_paths,
                "roofline": {"bound": "tensor", "achieved": achieved, "peak": peaks["bf16_tflops"], "unit": "TFLOP/s",
                             "frac": achieved / peaks["bf16_tflops"], "peak_source": "%s bf16_tflops" % src,
                             "work": "BF16 tensor flops = 3 products x 2 outputs x 2*M*N*K"}})
    return 0


def main():
    args = parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return reference_arm(args, rank, world)
    if args.workload != "ozaki":
        import __graft_entry__  # noqa: F401  (path setup only)
        if rank != 0:
            return 0
        return {"native": workload_native, "grouped": workload_grouped, "adjoint": workload_adjoint,
                "semiring": workload_semiring, "ozaki_sweep": workload_ozaki_sweep,
                "f32_tc": workload_f32_tc}[args.workload](args)

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

    from gbblas import replicas

    def max_over_ranks(x):
        return replicas.job_time_and_throughput(x, 0.0, device=dev)[0] if dist is not None else x

    n = args.size
    M = N = K = n
    if args.mnk:
        M, N, K = (int(x) for x in args.mnk.split(","))
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

    mode = "ozaki_crt" if args.method == "crt" else "ozaki"
    # warm-up (also fixes the plan the library picks for these inputs)
    bound = None
    for _ in range(args.warmup):
        _, bound = gbblas.gemm_(C_d, A_d, B_d, mode=mode, slices=args.slices, return_bound=True)
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
        if clocks:
            clocks.mark_start()
        ev0.record(stream)
        for _ in range(args.steps):
            gbblas.gemm_(C_d, A_d, B_d, mode=mode, slices=args.slices)
        ev1.record(stream)
        torch.cuda.synchronize()
        if clocks:
            clocks.mark_end()
    barrier()
    counts1 = gbblas.launch_counts()
    clk = clocks.stop() if clocks else None
    ms_step = max_over_ranks(ev0.elapsed_time(ev1) / args.steps)
    gbblas.check_device_status()
    launches = sum(counts1.get(k, 0) - counts0.get(k, 0) for k in counts1)
    value = world * flops / (ms_step * 1e-3) / 1e12

    # ---------------------------------------------------------------- timed: end to end
    # Every step copies its inputs host -> device (pinned) and its result device -> host.
    # Uploads and downloads run on their own streams (the two copy directions overlap) into a
    # ring of NBUF device input/output buffers: uploads run up to NBUF - 1 steps ahead of the
    # compute and downloads trail it, so the host link's jitter (it is shared with the node's
    # other GPUs) does not stall the compute (a serving pipeline with a queue of NBUF).  An
    # upload may end up to about (NBUF - 1) compute steps minus its own length late before the
    # compute waits for it: 27 ms with 4 buffers at 8192^3, 70 ms with 8 (12 GiB of buffers).
    NBUF = max(2, args.ring)
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    up_stream, down_stream = torch.cuda.Stream(dev), torch.cuda.Stream(dev)
    A_e = [torch.empty_like(A_pin, device=dev) for _ in range(NBUF)]
    B_e = [torch.empty_like(B_pin, device=dev) for _ in range(NBUF)]
    C_e = [torch.empty((N, M), dtype=torch.float64, device=dev) for _ in range(NBUF)]
    up_done = [torch.cuda.Event() for _ in range(NBUF)]
    comp_done = [torch.cuda.Event() for _ in range(NBUF)]
    down_done = [torch.cuda.Event() for _ in range(NBUF)]

    def run_pipeline(steps):
        """Enqueues `steps` pipelined steps; returns their (start, end) event pairs per stage
        and the host time at which each step's compute was enqueued."""
        up_ev, comp_ev, down_ev = ([(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                                    for _ in range(steps)] for _ in range(3))
        up_stream.wait_stream(stream)
        down_stream.wait_stream(stream)

        def upload(i):
            b = i % NBUF
            with torch.cuda.stream(up_stream):
                if i >= NBUF:
                    up_stream.wait_event(comp_done[b])       # buffer b's previous compute is done
                up_ev[i][0].record(up_stream)
                A_e[b].copy_(A_pin, non_blocking=True)
                B_e[b].copy_(B_pin, non_blocking=True)
                up_ev[i][1].record(up_stream)
                up_done[b].record(up_stream)

        host_t0 = time.perf_counter()
        host_enqueue_ms = []
        for i in range(min(NBUF - 1, steps)):
            upload(i)
        for i in range(steps):
            b = i % NBUF
            if i + NBUF - 1 < steps:
                upload(i + NBUF - 1)
            host_enqueue_ms.append((time.perf_counter() - host_t0) * 1e3)
            stream.wait_event(up_done[b])
            if i >= NBUF:
                stream.wait_event(down_done[b])              # C_e[b] of step i - NBUF has been read
            comp_ev[i][0].record(stream)
            gbblas.gemm_(C_e[b].t(), A_e[b].t(), B_e[b].t(), mode=mode, slices=args.slices)
            comp_ev[i][1].record(stream)
            comp_done[b].record(stream)
            with torch.cuda.stream(down_stream):
                down_stream.wait_event(comp_done[b])
                down_ev[i][0].record(down_stream)
                C_pin.copy_(C_e[b], non_blocking=True)
                down_ev[i][1].record(down_stream)
                down_done[b].record(down_stream)
        stream.wait_stream(up_stream)
        stream.wait_stream(down_stream)
        return up_ev, comp_ev, down_ev, host_enqueue_ms

    # warm-up: the same pipeline, untimed (the ring buffers' first copies are slow: the first
    # upload into a fresh device buffer measured 55 ms instead of 5 ms)
    run_pipeline(max(args.warmup, NBUF))
    torch.cuda.synchronize()
    # NWIN timed windows of `steps` steps each; the window with the median time is reported, all
    # of them beside it.  The host link is shared with the node's other GPUs: single copies were
    # seen to take 20-95 ms instead of 3-5 ms when other traffic ran, which one window of 20
    # steps cannot absorb; the median of five windows is the typical one, and every window is in
    # the line.
    NWIN = 5
    windows = []
    for _ in range(NWIN):
        barrier()
        pipe_prof = gbblas.profile()
        pipe_prof.__enter__()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        up_ev, comp_ev, down_ev, host_enqueue_ms = run_pipeline(args.steps)
        e1.record(stream)
        torch.cuda.synchronize()
        pipe_prof.__exit__(None, None, None)
        barrier()
        windows.append({"ms": max_over_ranks(e0.elapsed_time(e1) / args.steps), "prof": pipe_prof,
                        "ev": (e0, up_ev, comp_ev, down_ev, host_enqueue_ms)})
    order = sorted(range(NWIN), key=lambda w: windows[w]["ms"])
    med = windows[order[NWIN // 2]]
    ms_e2e = med["ms"]
    pipe_prof = med["prof"]
    e0, up_ev, comp_ev, down_ev, host_enqueue_ms = med["ev"]
    e2e_value = world * flops / (ms_e2e * 1e-3) / 1e12
    e2e_windows = [world * flops / (w["ms"] * 1e-3) / 1e12 for w in windows]
    comp_in_pipeline = statistics.median(a.elapsed_time(z) for a, z in comp_ev)
    up_in_pipeline = statistics.median(a.elapsed_time(z) for a, z in up_ev)
    down_in_pipeline = statistics.median(a.elapsed_time(z) for a, z in down_ev)
    timeline = pipeline_timeline(e0, up_ev, comp_ev, down_ev, NBUF, host_enqueue_ms)
    copy_stream = up_stream

    # the blocking host-buffer entry point (the reference's own calling pattern: host operands
    # in, host result out, one call at a time), on the same pinned buffers
    host_api = None
    if rank == 0:
        A_hv, B_hv, C_hv = A_pin.numpy().T, B_pin.numpy().T, C_pin.numpy().T   # column-major views
        gbblas.gemm_host(C_hv, A_hv, B_hv, mode=mode, slices=args.slices)     # warm-up
        t_calls = []
        for _ in range(3):
            t0 = time.perf_counter()
            gbblas.gemm_host(C_hv, A_hv, B_hv, mode=mode, slices=args.slices)
            t_calls.append(time.perf_counter() - t0)
        ms_host = statistics.median(t_calls) * 1e3
        host_api = {"value": flops / (ms_host * 1e-3) / 1e12, "unit": "TFLOP/s", "ms_per_call": ms_host,
                    "what": "one blocking gb_gemm_f64_host call per step on pinned host buffers: upload of A "
                            "and B, the product, download of C, no overlap between calls (median of 3, host "
                            "wall clock)"}

    # the host link alone: one step's uploads and download on the copy stream, no compute
    c0, c1, c2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    with torch.cuda.stream(copy_stream):
        c0.record(copy_stream)
        A_e[0].copy_(A_pin, non_blocking=True)
        B_e[0].copy_(B_pin, non_blocking=True)
        c1.record(copy_stream)
        C_pin.copy_(C_e[0], non_blocking=True)
        c2.record(copy_stream)
    torch.cuda.synchronize()
    h2d_gbs = (A_pin.numel() + B_pin.numel()) * 8 / (c0.elapsed_time(c1) * 1e-3) / 1e9
    d2h_gbs = C_pin.numel() * 8 / (c1.elapsed_time(c2) * 1e-3) / 1e9

    plan = gbblas.last_ozaki_plan()   # the plan the automatic choice used
    # The residue products alone: the same calls in one column panel, so that nothing runs
    # beside the tensor-core kernel (in the timed steps the split of the next panel and the
    # reconstruction of the previous one share its SMs).
    mma_alone = None
    if rank == 0 and args.method == "crt" and not args.mnk:
        from gbblas import tuning
        cls = tuning.size_class(M, N)
        saved = tuning.get_tuning("ozaki_crt", cls)
        tuning.set_tuning("ozaki_crt", cls, dict(saved.as_dict(), panels=1))
        try:
            for _ in range(2):
                gbblas.gemm_(C_d, A_d, B_d, mode=mode, slices=args.slices)
            torch.cuda.synchronize()
            with gbblas.profile() as prof_alone:
                for _ in range(5):
                    gbblas.gemm_(C_d, A_d, B_d, mode=mode, slices=args.slices)
                torch.cuda.synchronize()
        finally:
            tuning.set_tuning("ozaki_crt", cls, saved)
        mma_alone = prof_alone.ms.get("ozaki_slice_mma", float("nan")) / max(1, prof_alone.launches.get(
            "ozaki_slice_mma", 1))
    crt_tuned = None
    if rank == 0 and args.method == "crt" and not args.mnk:
        from gbblas import tuning
        t_best, t_ms = tuning.autotune("ozaki_crt", M, N, K, reps=2, install=False)
        crt_tuned = {"tuning": t_best.as_dict(), "ms_15_moduli": t_ms,
                     "default": tuning.get_tuning("ozaki_crt", tuning.size_class(M, N)).as_dict()}
    alt = None
    if not args.no_alt:
        # the other emulation method on the same inputs (automatic plan), for comparison
        alt_mode = "ozaki" if mode == "ozaki_crt" else "ozaki_crt"
        C_alt = torch.empty_like(C_d.t()).t()
        for _ in range(2):
            _, alt_bound = gbblas.gemm_(C_alt, A_d, B_d, mode=alt_mode, return_bound=True)
        alt_plan = gbblas.last_ozaki_plan()
        torch.cuda.synchronize()
        a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a0.record(stream)
        for _ in range(args.steps):
            gbblas.gemm_(C_alt, A_d, B_d, mode=alt_mode)
        a1.record(stream)
        torch.cuda.synchronize()
        alt_ms = a0.elapsed_time(a1) / args.steps
        alt = {"method": "slices" if alt_mode == "ozaki" else "crt", "value": flops / (alt_ms * 1e-3) / 1e12,
               "ms_per_step": alt_ms, "bound": alt_bound, "slices_or_moduli": alt_plan["slices"],
               "bits": alt_plan["bits"], "tensor_products": alt_plan["products"]}
        C_alt_h = np.asfortranarray(C_alt.cpu().numpy())
        del C_alt
    line = None
    if rank == 0:
        # a CRT call in column panels launches the residue products once per panel: the
        # algorithmic work and the DRAM traffic of one launch are the call's divided by that
        launches_per_call = max(1, round(prof.launches.get("ozaki_slice_mma", args.steps) / args.steps))
        mma_ms = prof.ms.get("ozaki_slice_mma", float("nan")) / max(1, prof.launches.get("ozaki_slice_mma", 1))
        peaks, peak_src = load_peaks()
        timed_s = ms_step * args.steps / 1e3
        peak_key = "bf16_tflops_sustained" if timed_s >= 1.0 else "bf16_tflops"
        achieved = plan["flops_tensor"] / launches_per_call / (mma_ms * 1e-3) / 1e12
        traffic = committed_traffic(args.method, n) if not args.mnk else None
        if traffic is not None:
            traffic /= launches_per_call

        # ------------------------------------------------------------ accuracy and native
        import oracle
        g = np.random.default_rng(12345)
        rows, cols = g.integers(0, M, 4096), g.integers(0, N, 4096)
        # reference values: binary128 dot products; sum |a||b| from the Dot2 pass
        _, _, ab = oracle.dot2_entries(A_h, B_h, rows, cols)
        hi, lo = oracle.quad_entries(A_h, B_h, rows, cols)
        err_oz = normwise_err(C_oz, A_h, B_h, rows, cols, hi, lo)
        cerr_oz = componentwise_err(C_oz, rows, cols, hi, lo, ab)
        if alt is not None:
            alt["normwise_err"] = normwise_err(C_alt_h, A_h, B_h, rows, cols, hi, lo)
            alt["componentwise_err"] = componentwise_err(C_alt_h, rows, cols, hi, lo, ab)
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
            cerr_nat = componentwise_err(C_nat, rows, cols, hi, lo, ab)
            pk = gbblas.measure_fma_peaks()
            native = {"tflops": flops / (nat_ms * 1e-3) / 1e12, "ms": nat_ms, "normwise_err": err_nat,
                      "fp64_pipe_tflops_measured": pk["fp64_tflops"],
                      "frac_of_measured_fp64": flops / (nat_ms * 1e-3) / 1e12 / pk["fp64_tflops"],
                      "componentwise_err": cerr_nat,
                      "ozaki_speedup": (flops / (ms_step * 1e-3) / 1e12) / (flops / (nat_ms * 1e-3) / 1e12)}
        cpu = None
        if not args.no_cpu and world == 1:
            threads = cpu_cores()
            v, sample, _, _ = cpu_sample(A_h, B_h, args.cpu_seconds, threads)
            # the reference itself is single-threaded: the same port on one core, a shorter sample
            v1, sample1, _, _ = cpu_sample(A_h, B_h, max(2.0, args.cpu_seconds / 4), 1)
            cpu = {"value": v, "unit": "TFLOP/s", "cores": threads, "kind": "port", "sample": sample,
                   "single_core": {"value": v1, "cores": 1, "sample": sample1},
                   "reference_shape": reference_shape_timing()}

        line = {
            "metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": headline_config(M, N, K, world),
            "plan": {"method": args.method,
                     **({"moduli": plan["slices"], "integer_bits": plan["bits"],
                         "residue_products": plan["products"]} if args.method == "crt" else
                        {"slices": plan["slices"], "bits": plan["bits"], "slice_products": plan["products"],
                         "accumulation_groups": plan["groups"]}),
                     "k_chunk": plan["k_chunk"]},
            "accuracy": {"normwise_err": err_oz, "bound": bound, "componentwise_err": cerr_oz,
                         "metric": "||C - C_ref||_F / (||A||_F ||B||_F), 4096 sampled entries against "
                                   "binary128 dot products; componentwise: max |C - C_ref|_ij / (|A||B|)_ij "
                                   "on the same entries"},
            "native_fp64": native,
            "roofline": {"bound": "tensor", "achieved": achieved, "peak": peaks[peak_key], "unit": "TFLOP/s",
                         "frac": achieved / peaks[peak_key], "traffic": traffic,
                         "traffic_source": "ncu dram__bytes_read.sum + write.sum of a 4096x4096x8192 launch "
                                           "scaled by the pair tiles one launch processes (profiles/, a lower "
                                           "bound at 8192^3)",
                         "kernel": "ozaki_slice_mma", "ms_per_launch": mma_ms,
                         "launches_per_call": launches_per_call,
                         "alone": None if mma_alone is None else {
                             "ms_per_launch": mma_alone,
                             "achieved": plan["flops_tensor"] / (mma_alone * 1e-3) / 1e12,
                             "frac": plan["flops_tensor"] / (mma_alone * 1e-3) / 1e12 / peaks[peak_key],
                             "note": "the same calls in one column panel (5 calls after the timed steps): "
                                     "the residue products with nothing running beside them"},
                         "peak_source": "%s %s" % (peak_src, peak_key),
                         "work": "BF16 tensor flops per launch = %s * 2*M*N*ceil(K/64)*64 / launches_per_call"
                                 % ("moduli" if args.method == "crt" else "slice_products")},
            "other_method": alt,
            "tc_autotune": crt_tuned,
            "kernel_ms_per_step": {k: v / args.steps for k, v in prof.ms.items()},
            "kernel_ms_note": ("CUDA-event time of each kernel kind per step; with column panels the split of "
                               "the next panel and the reconstruction of the previous one run beside the "
                               "residue products, so the kinds can sum to more than ms_per_step"),
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": "TFLOP/s", "ms_per_step": ms_e2e,
                    "pipeline": f"{NBUF}-deep ring: uploads run up to {NBUF - 1} steps ahead, the download of step i "
                                "overlaps step i+1; the timed steps start with an empty pipeline (the first upload and the last "
                                "download are not overlapped), after an untimed warm-up pass of the same pipeline",
                    "h2d_GBps": h2d_gbs, "d2h_GBps": d2h_gbs,
                    "compute_ms_in_pipeline": comp_in_pipeline,
                    "upload_ms_in_pipeline": up_in_pipeline, "download_ms_in_pipeline": down_in_pipeline,
                    "kernel_ms_in_pipeline": {k: v / args.steps for k, v in pipe_prof.ms.items()},
                    "timeline": timeline, "windows_tflops": e2e_windows,
                    "windows": "median of 5 timed windows of `steps` steps (all five listed)",
                    "h2d_bytes_per_step": int(A_pin.numel() * 8 + B_pin.numel() * 8),
                    "d2h_bytes_per_step": int(C_pin.numel() * 8)},
            "host_api": host_api,
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
