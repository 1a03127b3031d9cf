#!/usr/bin/env python3
"""Benchmark of the CAPS Strassen multiply on GB300 (one JSON line on rank 0).

Metric: effective TFLOP/s (2 n^3 / t) of the split-form Strassen multiply at
n = 16384, r = 3 (uniform[-1,1) float64 inputs, seeded), with the plain FP64
(DMMA) Strassen of the same multiply timed beside it and the error of both
measured on sampled entries against a binary128 (numpy longdouble on aarch64)
classical product.

  value     device-resident: A, B, C already in HBM, K multiplies timed with
            CUDA events on the launching stream (each matrix is 2 GiB, far
            above the 129 MB L2, so nothing is served from L2 across steps)
  e2e       the same through the host entry point: pinned host A, B copied in,
            C copied out, inside the timed region
  roofline  the dominant kernel (the split GEMM of the scheme that ran:
            crt_gemm_kernel for residues, split_gemm_kernel for digits):
            its tensor flops per launch / its average launch time (CUDA events,
            same stream)
  cpu_baseline  the oracle restatement of the reference's CPU path (OpenMP +
            OpenBLAS dgemm): one whole multiply of the same workload, timed

--impl reference times the reference's CPU path alone (the oracle port on the
host cores), as the reference arm.  N > 1 GPUs (torchrun) run independent
replicas: the multiply does not shard across GPUs on this path.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

os.environ.setdefault("OMP_WAIT_POLICY", "passive")  # before any OpenMP runtime starts

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "effective TFLOP/s (2n³/t) at n=16384: split-INT8 vs FP64 Strassen, same error"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=16384)
    ap.add_argument("--nrec", type=int, default=3)
    ap.add_argument("--pattern", default=None, help="default: the library's choice")
    ap.add_argument("--slices", type=int, default=0)
    ap.add_argument("--scheme", default="auto", choices=["auto", "digits", "residues"],
                    help="split-form operand cut (auto: from the data)")
    ap.add_argument("--operand-bits", type=int, default=-1,
                    help="residue operand-bit cap: -1 = the library's accuracy-gated choice per leaf size "
                         "(55, 52 or 48), 0 = 55, else 1..55")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-wide", action="store_true", help="skip the wide-range (u*2^k) error check")
    ap.add_argument("--samples", type=int, default=256, help="entries checked against binary128")
    ap.add_argument("--workload", default="split16384",
                    choices=["split16384", "plain8192", "batched512", "int32768", "chol16384", "rect"],
                    help="split16384: the headline (n=16384, r=3, split vs FP64); plain8192: FP64 Strassen "
                         "n=8192 r=3 'ddd'; batched512: 512 uneven multiplies; int32768: n=32768 r=4 'bbdd' "
                         "integers under a 120 GB budget; chol16384: the Cholesky subproject's update "
                         "C = C - A B^T, n=16384, r=3; rect: the rectangular subproject's rectMM, "
                         "16384 x 8192 times 8192 x 12288, r=2 'dd'")
    return ap.parse_args()


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("nccl" if args.impl == "ours" else "gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x: float, world: int, device: str = "cuda") -> float:
    """Slowest rank's time (replicas: every rank runs its own multiplies)."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(units_per_rank: float, world: int, seconds_max: float) -> float:
    """Whole-job rate: the units all ranks processed over the slowest rank's time."""
    return world * units_per_rank / seconds_max


# ----------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = os.path.join("/tmp", "caps_clocks_%d_%d.csv" % (os.getpid(), index))

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None:
            return None
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            for line in open(self.path):
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 8:
                    continue
                try:
                    sm.append(float(parts[0]))
                    mx.append(float(parts[1]))
                except ValueError:
                    continue
                for nm, v in zip(names, parts[4:8]):
                    if v.lower().startswith("active"):
                        reasons.add(nm)
        except OSError:
            return None
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ----------------------------------------------------------------- peaks
def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(p))
        return d, "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def profiled_traffic(kernel="split_gemm_kernel"):
    """dram bytes per GEMM launch from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", "%s_n16384.md" % kernel)
    try:
        for line in open(p):
            if line.strip().startswith("traffic_bytes_per_launch:"):
                return float(line.split(":", 1)[1].strip())
    except OSError:
        pass
    return None


# ----------------------------------------------------------------- error
def pinned_copy_bandwidth(h, d, stream, reps=3):
    """Plain pinned host<->device copy rates (GB/s) of one input matrix on
    this box, reported beside the e2e figure, which they bound."""
    import torch
    out = {}
    for name, dst, src in (("h2d", d, h), ("d2h", h, d)):
        dst.copy_(src, non_blocking=True)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            dst.copy_(src, non_blocking=True)
        e1.record(stream)
        torch.cuda.synchronize()
        out[name] = reps * h.numel() * 8 / (e0.elapsed_time(e1) / 1e3) / 1e9
    return out


def sampled_error(C_cm, A_cm, B_cm, n, samples, seed=7):
    """Max elementwise |C - C_ref| / (|A||B|) and normwise over sampled entries;
    C_ref from binary128 (numpy longdouble) dot products."""
    import numpy as np
    rng = np.random.default_rng(seed)
    rows = rng.integers(0, n, samples)
    cols = rng.integers(0, n, samples)
    ld = np.longdouble
    Am, Bm, Cm = A_cm.reshape(n, n), B_cm.reshape(n, n), C_cm.reshape(n, n)  # [col][row]
    ew, num, den = 0.0, 0.0, 0.0
    for i, j in zip(rows, cols):
        a = np.ascontiguousarray(Am[:, i])  # row i of A
        b = Bm[j]                           # column j of B
        ref = np.dot(a.astype(ld), b.astype(ld))
        ab = float(np.dot(np.abs(a), np.abs(b)))
        c = Cm[j, i]
        d = float(ld(c) - ref)
        ew = max(ew, abs(d) / ab if ab > 0 else abs(d))
        num += d * d
        den += float(ref) ** 2
    return {"max_elementwise_rel": ew, "normwise_rel": (num / den) ** 0.5 if den > 0 else 0.0,
            "samples": int(samples), "reference_precision_bits": int(np.finfo(ld).nmant + 1)}


# ----------------------------------------------------------------- CPU leg
def cpu_setup(n, seed=11):
    """Threads, OpenBLAS leaves and seeded uniform[-1,1) inputs for the oracle
    port of the reference CPU path (randombenchmark.cpp:19-22 draws the same
    distribution)."""
    import numpy as np
    from oracle import oracle
    cores = os.cpu_count() or 1
    oracle.build()
    blas = oracle.use_blas(True, threads=cores)
    oracle.set_threads(cores)
    rng = np.random.default_rng(seed)
    A = rng.uniform(-1, 1, n * n)
    B = rng.uniform(-1, 1, n * n)
    return oracle, A, B, cores, blas


def cpu_whole_multiplies(n, nrec, count, seed=11):
    """Seconds of each of `count` whole n x n, nrec-level 'd'*nrec multiplies
    of the oracle port of the reference CPU path (OpenMP sums, OpenBLAS dgemm
    leaves), timed as randombenchmark.cpp:89-93 times multiply(): a timer
    read on each side of the call.  One rank runs 'd' steps: a 'b' step
    needs more than one rank."""
    oracle, A, B, cores, blas = cpu_setup(n, seed)
    times = []
    for _ in range(count):
        t0 = time.perf_counter()
        oracle.multiply(A, B, n, nrec, 1, "d" * nrec)
        times.append(time.perf_counter() - t0)
    return times, cores, blas


def cpu_sample_model(n, nrec, seed=11):
    """Cross-check only: the top level's sums and C combination timed in full
    plus one of its seven subproducts (n/2, nrec-1) timed in full; a whole
    multiply takes about t_top + 7 t_sub."""
    import numpy as np
    oracle, A, B, cores, blas = cpu_setup(n, seed)
    C = np.empty(n * n)
    t_top, t_sub = oracle.multiply_sample(A, B, C, n, nrec, 1, "d" * nrec, child=1)
    return {"t_top_s": t_top, "t_sub_s": t_sub, "t_model_s": t_top + 7 * t_sub,
            "model": "t_top + 7 t_sub (top-level sums and combination + one of seven subproducts)"}


def cpu_sample_text(n, nrec, count, cores, blas):
    return ("oracle restatement of the reference CPU path (OpenMP sums, %s dgemm leaves, OMP_WAIT_POLICY=passive, "
            "%d threads): %d whole multiplies n=%d r=%d pattern '%s', each timed around the call"
            % ("OpenBLAS" if blas else "loop", cores, count, n, nrec, "d" * nrec))


def run_reference(args, world, rank):
    if rank != 0:
        return
    n, r = args.n, args.nrec
    times, cores, blas = cpu_whole_multiplies(n, r, args.warmup + args.steps)
    timed = times[args.warmup:]
    model = cpu_sample_model(n, r)  # cross-check of the earlier sampled estimate
    t = sum(timed) / len(timed)
    val = 2.0 * n ** 3 / t / 1e12
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": val, "unit": "TFLOP/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "CAPS Strassen multiply n=%d r=%d, reference CPU path (one rank)" % (n, r),
                   "n": n, "nrec": r, "pattern": "d" * r, "inputs": "uniform[-1,1) seeded"},
        "step_ms": [x * 1e3 for x in timed], "warmup_ms": [x * 1e3 for x in times[:args.warmup]],
        "sample_model": model,
        "cpu_baseline": {"value": val, "unit": "TFLOP/s", "cores": cores, "kind": "port",
                         "sample": cpu_sample_text(n, r, len(timed), cores, blas)},
        "e2e": {"value": val, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


# ----------------------------------------------------------------- GPU legs
def common_line(metric, value, args, world, ms, config, **extra):
    d = {"metric": metric, "value": value, "unit": "TFLOP/s", "n_gpus": world, "steps": args.steps,
         "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
         "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": config}
    d.update(extra)
    return d


def run_plain8192(args, world, rank, local):
    """FP64 Strassen n=8192, r=3, 'ddd' on DMMA (uniform[-1,1) inputs)."""
    import torch
    import caps_gb300 as cg
    dev = torch.device("cuda", local)
    n, r, pat = 8192, 3, "ddd"
    d = cg.MatDescriptor.make(n, r)
    g = torch.Generator(device=dev)
    g.manual_seed(2)
    A = torch.rand(n * n, dtype=torch.float64, device=dev, generator=g) * 2 - 1
    B = torch.rand(n * n, dtype=torch.float64, device=dev, generator=g) * 2 - 1
    C = torch.empty_like(A)
    for _ in range(args.warmup):
        cg.multiply(A, B, C, d, pat, form="plain")
    torch.cuda.synchronize()
    barrier(world)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        e0.record()
        for _ in range(args.steps):
            cg.multiply(A, B, C, d, pat, form="plain")
        e1.record()
        torch.cuda.synchronize()
    t = max_over_ranks(e0.elapsed_time(e1) / 1e3 / args.steps, world)
    if rank == 0:
        def cm(x):
            y = torch.empty_like(x)
            cg.from_caps_layout(x, y, d)
            torch.cuda.synchronize()
            return y.cpu().numpy()
        err = sampled_error(cm(C), cm(A), cm(B), n, args.samples)
        print(json.dumps(common_line("effective TFLOP/s (2n³/t), FP64 Strassen n=8192 r=3 'ddd'",
                                     world * 2.0 * n ** 3 / t / 1e12, args, world, t * 1e3,
                                     {"workload": "plain FP64 Strassen n=8192 r=3 ddd (DMMA base case)", "n": n,
                                      "nrec": r, "pattern": pat, "form": "plain",
                                      "inputs": "uniform[-1,1) seeded"},
                                     error=err, clocks=clk.summary(),
                                     gpu_launches=cg.counters()["kernel_launches"] * args.steps)), flush=True)


def run_rect(args, world, rank, local):
    """The rectangular subproject's rectMM on one rank (rect-class/rectmm.cpp):
    A 16384 x 8192 times B 8192 x 12288, r = 2 'dd', divisions (2,1,1)(1,3,1):
    six base products of 8192 x 8192 by 8192 x 4096 on FP64 DMMA, the whole
    product (every divk is 1, and divm or divn is 1 at each level)."""
    import numpy as np
    import torch
    import caps_gb300 as cg
    from fractions import Fraction
    dev = torch.device("cuda", local)
    m, n, k, r, patt, div = 16384, 12288, 8192, 2, "dd", [2, 1, 1, 1, 3, 1]
    g = torch.Generator(device=dev)
    g.manual_seed(41 + rank)
    A = torch.rand(m * k, dtype=torch.float64, device=dev, generator=g) * 2 - 1
    B = torch.rand(k * n, dtype=torch.float64, device=dev, generator=g) * 2 - 1
    C = torch.zeros(m * n, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    for _ in range(max(args.warmup, 3)):
        cg.rect_mm(A, B, C, m, n, k, r, patt, div, stream=stream.cuda_stream)
    torch.cuda.synchronize()
    launches = cg.counters()["kernel_launches"]
    barrier(world)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            cg.rect_mm(A, B, C, m, n, k, r, patt, div, stream=stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize()
    t = max_over_ranks(e0.elapsed_time(e1) / 1e3 / args.steps, world)
    if rank != 0:
        return
    # the layout: A rows in two column-major halves, B column-major, C in
    # (row half, column third) blocks of 8192 x 4096, column-major
    hA, hB, hC = A.cpu().numpy(), B.cpu().numpy(), C.cpu().numpy()
    rng = np.random.default_rng(5)
    worst = 0.0
    for _ in range(16):
        i, j = int(rng.integers(0, m)), int(rng.integers(0, n))
        ai = hA[(i // 8192) * 8192 * k:][: 8192 * k].reshape(k, 8192)[:, i % 8192]
        bj = hB[j * k:(j + 1) * k]
        cij = hC[((i // 8192) * 3 + j // 4096) * 8192 * 4096 + (j % 4096) * 8192 + i % 8192]
        exact = sum(Fraction(float(a)) * Fraction(float(b)) for a, b in zip(ai, bj))
        absdot = float(np.abs(ai) @ np.abs(bj))
        worst = max(worst, abs(float(Fraction(float(cij)) - exact)) / absdot)
    cpu = None
    if not args.no_cpu:
        from oracle import oracle
        cores = os.cpu_count() or 1
        oracle.build()
        blas = oracle.use_blas(True, threads=cores)
        oracle.set_threads(cores)
        try:
            tc0 = time.perf_counter()
            oracle.rect_mm(hA, hB, hC, m, n, k, r, patt, div)
            tcpu = time.perf_counter() - tc0
        finally:
            oracle.use_blas(False)
        cpu = {"value": 2.0 * m * n * k / tcpu / 1e12, "unit": "TFLOP/s", "cores": cores, "kind": "port",
               "sample": "one whole rectMM of the same shape: the oracle's restatement of the one-rank walk, "
                         "%s dgemm at the base blocks, %d threads (%.2f s)" % ("OpenBLAS" if blas else "loop",
                                                                                cores, tcpu)}
    flops = 2.0 * m * n * k
    peak = 1.13  # the FP64 pipe's rate at 2.07 GHz, from the DMMA capture (profiles/dmma_gemm_kernel_n4096.md)
    print(json.dumps(common_line(
        "effective TFLOP/s (2mnk/t), rectMM 16384x8192 * 8192x12288, r=2 'dd'", world * flops / t / 1e12, args,
        world, t * 1e3,
        {"workload": "the rectangular subproject's rectMM on one rank, m=16384 n=12288 k=8192, r=2 'dd', "
                     "divisions (2,1,1)(1,3,1), FP64 DMMA base case", "m": m, "n": n, "k": k, "nrec": r,
         "pattern": patt, "divisions": div, "inputs": "uniform[-1,1) seeded (torch.Generator)"},
        error={"max_elementwise_rel": worst, "samples": 16, "reference": "exact rational dot products"},
        roofline={"bound": "tensor", "kernel": "dmma_gemm_kernel", "achieved": flops / t / 1e12, "peak": peak,
                  "unit": "TFLOP/s", "frac": flops / t / 1e12 / peak,
                  "peak_source": "FP64 (DMMA) pipe rate at 2.07 GHz, from profiles/dmma_gemm_kernel_n4096.md",
                  "traffic": None},
        cpu_baseline=cpu, gpu_launches=launches * args.steps, clocks=clk.summary())), flush=True)


def run_batched512(args, world, rank, local):
    """512 independent multiplies, n log-uniform over {448, 896, 1792, 3584}."""
    import numpy as np
    import torch
    import caps_gb300 as cg
    dev = torch.device("cuda", local)
    rng = np.random.default_rng(5)
    sizes = [int(x) for x in rng.choice([448, 896, 1792, 3584], 512)]
    g = torch.Generator(device=dev)
    g.manual_seed(5 + rank)
    As = [torch.rand(n * n, dtype=torch.float64, device=dev, generator=g) * 2 - 1 for n in sizes]
    Bs = [torch.rand(n * n, dtype=torch.float64, device=dev, generator=g) * 2 - 1 for n in sizes]
    Cs = [torch.empty(n * n, dtype=torch.float64, device=dev) for n in sizes]
    eff = sum(2.0 * n ** 3 for n in sizes)
    res = {}
    for form in ("split", "plain"):
        steps = args.steps if form == "split" else 1
        for _ in range(max(1, args.warmup if form == "split" else 1)):  # first call tunes and captures
            cg.multiply_batched(As, Bs, Cs, sizes, form=form)
        barrier(world)
        with ClockSampler(local) as clk:
            t0 = time.perf_counter()
            for _ in range(steps):
                cg.multiply_batched(As, Bs, Cs, sizes, form=form)  # synchronises
            t = max_over_ranks((time.perf_counter() - t0) / steps, world)
        res[form] = {"value": world * eff / t / 1e12, "ms_per_step": t * 1e3, "steps": steps,
                     "graph_kernels": cg.counters()["kernel_launches"], "clocks": clk.summary()}
        if rank == 0:  # error of three instances against binary128
            res[form]["error"] = {
                str(sizes[i]): sampled_error(Cs[i].cpu().numpy(), As[i].cpu().numpy(), Bs[i].cpu().numpy(),
                                             sizes[i], 64) for i in range(3)}
    if rank == 0:
        counts = {str(n): sizes.count(n) for n in sorted(set(sizes))}
        print(json.dumps(common_line("effective TFLOP/s (sum 2n³ / t), 512 uneven multiplies",
                                     res["split"]["value"], args, world, res["split"]["ms_per_step"],
                                     {"workload": "512 independent multiplies, n over {448,896,1792,3584}",
                                      "sizes": counts, "form": "split", "inputs": "uniform[-1,1) seeded",
                                      "execution": "per-size autotuned depth/pattern/scheme, CUDA graph replay"},
                                     split=res["split"], plain_fp64=res["plain"],
                                     split_vs_plain=res["split"]["value"] / res["plain"]["value"],
                                     autotune=cg.autotune_table(), clocks=res["split"]["clocks"],
                                     gpu_launches=res["split"]["graph_kernels"] * args.steps)), flush=True)


def run_int32768(args, world, rank, local):
    """n=32768, r=4, 'bbdd', integers in [-1024, 1024], 120 GB workspace budget."""
    import numpy as np
    import torch
    import caps_gb300 as cg
    dev = torch.device("cuda", local)
    n, r, pat = 32768, 4, "bbdd"
    budget = 120000 * 2 ** 20
    d = cg.MatDescriptor.make(n, r)
    g = torch.Generator(device=dev)
    g.manual_seed(9)
    A = torch.randint(-1024, 1025, (n * n,), dtype=torch.int32, device=dev, generator=g).to(torch.float64)
    B = torch.randint(-1024, 1025, (n * n,), dtype=torch.int32, device=dev, generator=g).to(torch.float64)
    C = torch.empty_like(A)
    res = {}
    for form in ("split", "plain"):
        steps = args.steps if form == "split" else 1
        sch = args.scheme if form == "split" else "auto"
        cg.multiply(A, B, C, d, pat, form=form, workspace_limit=budget, scheme=sch)
        torch.cuda.synchronize()
        cg.set_phase_timing(True)
        t_tot, add_t, add_b = 0.0, 0.0, 0
        for _ in range(steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            cg.multiply(A, B, C, d, pat, form=form, workspace_limit=budget, scheme=sch)
            e1.record()
            torch.cuda.synchronize()
            c = cg.counters()
            t_tot += e0.elapsed_time(e1) / 1e3
            add_t += c["time_add"]
            add_b += c["add_bytes"]
        cg.set_phase_timing(False)
        t = t_tot / steps
        # bit-exactness on sampled entries: exact int64 dot products
        y = torch.empty_like(C)
        cg.from_caps_layout(C, y, d)
        Ac, Bc = torch.empty_like(A), torch.empty_like(B)
        cg.from_caps_layout(A, Ac, d)
        cg.from_caps_layout(B, Bc, d)
        rng = np.random.default_rng(1)
        rows, cols = rng.integers(0, n, 64), rng.integers(0, n, 64)
        Am = Ac.view(n, n)  # [col][row]
        Bm = Bc.view(n, n)
        Cm = y.view(n, n)
        exact = 0
        for i, j in zip(rows, cols):
            ref = int((Am[:, i].to(torch.int64) * Bm[j].to(torch.int64)).sum().item())
            exact += int(float(Cm[j, i].item()) == float(ref))
        del y, Ac, Bc
        cnt = cg.counters()
        res[form] = {"value": 2.0 * n ** 3 / t / 1e12, "ms_per_step": t * 1e3, "steps": steps,
                     "bit_exact_sampled": "%d/64" % exact, "leaf_gemm_ms": cnt["time_leaf_gemm"] * 1e3,
                     "split_moduli": cnt["split_moduli"], "split_slices": cnt["split_slices"],
                     "additions_hbm_gbs": add_b / add_t / 1e9 if add_t > 0 else None,
                     "workspace_bytes": cg.counters()["workspace_peak_bytes"]}
    if rank == 0:
        print(json.dumps(common_line("effective TFLOP/s (2n³/t), n=32768 r=4 'bbdd' integers",
                                     res["split"]["value"], args, world, res["split"]["ms_per_step"],
                                     {"workload": "Strassen n=32768 r=4 bbdd, integer inputs [-1024,1024], "
                                                  "-m 120000 (MB) budget", "n": n, "nrec": r, "pattern": pat,
                                      "form": "split"},
                                     split=res["split"], plain_fp64=res["plain"],
                                     split_vs_plain=res["split"]["value"] / res["plain"]["value"])), flush=True)


def chol_sampled_error(out_cm, C0_cm, A_cm, B_cm, n, samples, seed=7):
    """C = C0 - A B^T on sampled entries: max |C - C_ref| / (|C0| + |A||B^T|)
    and normwise; C_ref in binary128 (numpy longdouble)."""
    import numpy as np
    rng = np.random.default_rng(seed)
    ld = np.longdouble
    Am, Bm = A_cm.reshape(n, n), B_cm.reshape(n, n)  # [col][row]
    Om, Cm = out_cm.reshape(n, n), C0_cm.reshape(n, n)
    ew, num, den = 0.0, 0.0, 0.0
    for i, j in zip(rng.integers(0, n, samples), rng.integers(0, n, samples)):
        a, b = np.ascontiguousarray(Am[:, i]), np.ascontiguousarray(Bm[:, j])  # rows i of A, j of B
        ref = ld(Cm[j, i]) - np.dot(a.astype(ld), b.astype(ld))
        scale = abs(float(Cm[j, i])) + float(np.dot(np.abs(a), np.abs(b)))
        d = float(ld(Om[j, i]) - ref)
        ew = max(ew, abs(d) / scale if scale > 0 else abs(d))
        num += d * d
        den += float(ref) ** 2
    return {"max_elementwise_rel": ew, "normwise_rel": (num / den) ** 0.5 if den > 0 else 0.0,
            "samples": int(samples)}


def run_chol16384(args, world, rank, local):
    """The Cholesky subproject's trailing update C = C - A B^T (cholesky/mult.h:6,
    mult.cpp:11-137 on one rank) at n=16384 in its recursive layout with r=3,
    uniform[-1,1) inputs: -B^T formed on the device, the product by the split
    Strassen multiply, one scale-add pass."""
    import numpy as np
    import torch
    import caps_gb300 as cg
    dev = torch.device("cuda", local)
    n, r = 16384, 3
    desc = cg.MatDescriptor.make(n, r)
    g = torch.Generator(device=dev)
    g.manual_seed(31 + rank)
    A, B, C0 = (torch.rand(n * n, dtype=torch.float64, device=dev, generator=g) * 2 - 1 for _ in range(3))
    C = C0.clone()
    stream = torch.cuda.current_stream(dev)
    hA, hB, hC = (torch.empty(n * n, dtype=torch.float64, pin_memory=True) for _ in range(3))
    hA.copy_(A)
    hB.copy_(B)
    hC.copy_(C0)

    def step():
        cg.chol_mult(C, A, B, n, r, 1.0, form="split", stream=stream.cuda_stream, scheme=args.scheme,
                     operand_bits=args.operand_bits)

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    cg.set_phase_timing(True)
    gemm_t, gemm_launches, gemm_m3, launches = 0.0, 0, 0.0, 0
    barrier(world)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            step()
            c = cg.counters()
            gemm_t += c["time_leaf_gemm"]
            gemm_launches += c["leaf_gemm_launches"]
            gemm_m3 += c["leaf_gemm_m3"]
            launches += c["kernel_launches"] + 2  # the transpose and the scale-add
        e1.record(stream)
        torch.cuda.synchronize()
    cg.set_phase_timing(False)
    t = max_over_ranks(e0.elapsed_time(e1) / 1e3 / args.steps, world)
    moduli = cg.counters()["split_moduli"]
    pattern = cg.resolve_pattern(desc, None, form="split")
    gate = [e for e in cg.autotune_table() if e["leaf_gate"] and e["n"] == n >> r]
    bits_used = (gate[-1]["operand_bits"] if gate else 55) if args.operand_bits < 0 else (args.operand_bits or 55)

    # e2e: the host entry point with pinned host buffers (A, B, C in; C out)
    nA, nB, nC = hA.numpy(), hB.numpy(), hC.numpy()
    cg.chol_mult(nC, nA, nB, n, r, 1.0, form="split", scheme=args.scheme, operand_bits=args.operand_bits)
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        cg.chol_mult(nC, nA, nB, n, r, 1.0, form="split", scheme=args.scheme, operand_bits=args.operand_bits)
    t_e2e = max_over_ranks((time.perf_counter() - t0) / args.steps, world)
    if rank != 0:
        return
    # accuracy of one update from the seeded C0
    C.copy_(C0)
    step()
    torch.cuda.synchronize()

    def colmajor(x):
        y = torch.empty_like(x)
        cg.from_caps_layout(x, y, desc)
        torch.cuda.synchronize()
        return y.cpu().numpy()
    err = chol_sampled_error(colmajor(C), colmajor(C0), colmajor(A), colmajor(B), n, args.samples)
    peaks, peak_src = measured_peaks()
    per_launch_flops = 2.0 * moduli * gemm_m3 / max(gemm_launches, 1)
    per_launch_s = gemm_t / max(gemm_launches, 1)
    achieved = per_launch_flops / per_launch_s / 1e12 if per_launch_s > 0 else 0.0
    peak = float(peaks.get("bf16_tflops_sustained", peaks.get("bf16_tflops", 1700.0)))
    cpu = None
    if not args.no_cpu:
        # the reference's path at n=16384, r=3 is multDFS down to 512 base
        # updates of 2048 (r = 0: no repack), each one dgemm('N','T')
        from oracle import oracle
        cores = os.cpu_count() or 1
        oracle.build()
        blas = oracle.use_blas(True, threads=cores)
        oracle.set_threads(cores)
        rng = np.random.default_rng(12)
        m = 2048
        a, b, c0 = (rng.uniform(-1, 1, m * m) for _ in range(3))
        oracle.chol_mult(c0, a, b, m, 0, 1.0)
        reps = 3
        tb0 = time.perf_counter()
        for _ in range(reps):
            oracle.chol_mult(c0, a, b, m, 0, 1.0)
        t_base = (time.perf_counter() - tb0) / reps
        cpu = {"value": 2.0 * n ** 3 / (512 * t_base) / 1e12, "unit": "TFLOP/s", "cores": cores, "kind": "port",
               "sample": "oracle restatement of cholesky mult() (one rank, %s dgemm, %d threads): one base "
                         "update of 2048 (r = 0) timed %d times (%.3f s each); the n=16384 r=3 update is "
                         "512 of them (multDFS), value = 2n^3 / (512 t_base)" % (
                             "OpenBLAS" if blas else "loop", cores, reps, t_base)}
    print(json.dumps(common_line(
        "effective TFLOP/s (2n³/t), Cholesky update C = C - A B^T, n=16384 r=3", world * 2.0 * n ** 3 / t / 1e12,
        args, world, t * 1e3,
        {"workload": "cholesky mult() C = C - A B^T, n=16384, r=3 recursive layout, split form "
                     "(residues modulo %d moduli)" % moduli, "n": n, "nrec": r, "pattern": pattern,
         "form": "split", "alpha": 1.0, "inputs": "float64 uniform[-1,1) seeded (torch.Generator)",
         "operand_bits": bits_used, "operand_bits_choice": "library's accuracy-gated choice per leaf size"
         if args.operand_bits < 0 else "fixed by --operand-bits",
         "l2": "inputs larger than L2 (each matrix 2 GiB vs 129 MB L2)"},
        error=err,
        roofline={"bound": "tensor", "kernel": "crt_gemm_kernel" if moduli else "split_gemm_kernel",
                  "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak if peak else None,
                  "traffic": profiled_traffic("crt_gemm_kernel" if moduli else "split_gemm_kernel"),
                  "peak_source": "%s bf16_tflops_sustained" % peak_src, "launches": gemm_launches,
                  "avg_launch_ms": per_launch_s * 1e3},
        cpu_baseline=cpu,
        e2e={"value": world * 2.0 * n ** 3 / t_e2e / 1e12, "unit": "TFLOP/s", "h2d_bytes_per_step": 3 * n * n * 8,
             "d2h_bytes_per_step": n * n * 8, "ms_per_step": t_e2e * 1e3,
             "api": "caps_chol_mult_host, pinned host buffers"},
        gpu_launches=launches, clocks=clk.summary())), flush=True)


def main():
    args = parse()
    world, rank, local = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, world, rank)
        return
    if args.workload != "split16384":
        import torch
        torch.cuda.set_device(local)
        from caps_gb300 import build as cbuild
        if not os.path.exists(cbuild.LIB):
            cbuild.build()
        {"plain8192": run_plain8192, "batched512": run_batched512, "int32768": run_int32768,
         "chol16384": run_chol16384, "rect": run_rect}[args.workload](
            args, world, rank, local)
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return
    import numpy as np
    import torch
    from caps_gb300 import build as cbuild
    if not os.path.exists(cbuild.LIB):
        cbuild.build()
    import caps_gb300 as cg

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    n, r = args.n, args.nrec
    desc = cg.MatDescriptor.make(n, r)
    pattern = args.pattern or cg.resolve_pattern(desc, None, form="split", workspace_limit=96 << 30)
    g = torch.Generator(device=dev)
    g.manual_seed(1234 + rank)
    A = torch.rand(n * n, dtype=torch.float64, device=dev, generator=g) * 2 - 1
    B = torch.rand(n * n, dtype=torch.float64, device=dev, generator=g) * 2 - 1
    C = torch.empty_like(A)
    stream = torch.cuda.current_stream(dev)
    # host copies of the inputs for the e2e leg, pinned while host memory is fresh
    hA = torch.empty(n * n, dtype=torch.float64, pin_memory=True)
    hB = torch.empty(n * n, dtype=torch.float64, pin_memory=True)
    hC = torch.empty(n * n, dtype=torch.float64, pin_memory=True)
    hA.copy_(A)
    hB.copy_(B)

    def step(form, c=C):
        cg.multiply(A, B, c, desc, pattern, form=form, slices=args.slices, stream=stream.cuda_stream,
                    scheme=args.scheme, operand_bits=args.operand_bits)

    # ---- headline: split form, device resident
    for _ in range(max(args.warmup, 3)):
        step("split")
    torch.cuda.synchronize()
    cg.set_phase_timing(True)
    gemm_t, gemm_launches, gemm_m3, launches = 0.0, 0, 0.0, 0
    add_t, add_b = 0.0, 0
    barrier(world)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            step("split")
            c = cg.counters()
            gemm_t += c["time_leaf_gemm"]
            gemm_launches += c["leaf_gemm_launches"]
            gemm_m3 += c["leaf_gemm_m3"]
            launches += c["kernel_launches"]
            add_t += c["time_add"]
            add_b += c["add_bytes"]
        e1.record(stream)
        torch.cuda.synchronize()
    barrier(world)
    cg.set_phase_timing(False)
    t_split = max_over_ranks(e0.elapsed_time(e1) / 1e3 / args.steps, world)
    cnt = cg.counters()
    peaks0, _ = measured_peaks()
    hbm_peak = float(peaks0.get("hbm_gbs", 6800.0))
    # the layout reorder (communication.cpp:612-704) both ways on the same
    # matrices: 16 bytes moved per element, CUDA events on the stream
    tmp, back = torch.empty_like(A), torch.empty_like(A)
    cg.from_caps_layout(A, tmp, desc, stream=stream.cuda_stream)
    r0, r1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    r0.record(stream)
    for _ in range(3):
        cg.from_caps_layout(A, tmp, desc, stream=stream.cuda_stream)
        cg.to_caps_layout(tmp, back, desc, stream=stream.cuda_stream)
    r1.record(stream)
    torch.cuda.synchronize()
    reorder_gbs = 6 * 16.0 * n * n / (r0.elapsed_time(r1) / 1e3) / 1e9
    reorder_roundtrip_exact = bool(torch.equal(back, A))
    del tmp, back
    memory_kernels = {
        "reorder": {"gbs": reorder_gbs, "frac_of_hbm_copy": reorder_gbs / hbm_peak,
                    "round_trip_exact": reorder_roundtrip_exact,
                    "bytes_per_element": 16, "what": "column-major <-> CAPS layout, n=%d, both directions" % n},
        "sums": {"gbs": add_b / add_t / 1e9 if add_t > 0 else None,
                 "frac_of_hbm_copy": (add_b / add_t / 1e9 / hbm_peak) if add_t > 0 else None,
                 "what": "Strassen operand sums and C combinations of the timed multiplies (algorithmic bytes "
                         "read + written / their kernels' CUDA-event time)"},
        "hbm_copy_gbs": hbm_peak}
    s_used, nd_used, moduli = cnt["split_slices"], cnt["split_diagonals"], cnt["split_moduli"]
    # the operand bits the residues ran with, and how they were chosen
    leaf_gate = [t for t in cg.autotune_table() if t["leaf_gate"] and t["n"] == n >> r]
    if args.operand_bits < 0:
        bits_used = leaf_gate[-1]["operand_bits"] if leaf_gate else 55
        bits_how = ("library's choice for leaves of %d: the fewest bits among 55/52/48 that ran faster and "
                    "whose leaf product was no less accurate than the FP64 DMMA leaf's on uniform and "
                    "wide-range inputs (%d faster cap(s) rejected)"
                    % (n >> r, leaf_gate[-1]["gate_rejected"] if leaf_gate else 0))
    else:
        bits_used, bits_how = (args.operand_bits or 55), "fixed by --operand-bits"
    value = replica_throughput(2.0 * n ** 3 / 1e12, world, t_split)

    # ---- e2e through the host entry point (pinned host buffers).  Timed
    # before the error checks below: their multi-GiB pageable host copies
    # leave host memory fragmented, and pinned copies made after them ran at
    # a fraction of the bandwidth measured right after start-up.
    nA, nB, nC = hA.numpy(), hB.numpy(), hC.numpy()
    copy_bw = pinned_copy_bandwidth(hA, A, stream)
    # the call a user makes: no pattern, the library's choice for host arrays
    # (a top-level 'd' step whose subproducts overlap the copies)
    e2e_pattern = cg.resolve_pattern(desc, None, form="split", workspace_limit=96 << 30)
    cg.multiply(nA, nB, nC, desc, None, form="split", slices=args.slices, scheme=args.scheme,
                    operand_bits=args.operand_bits)
    barrier(world)
    e2e_steps = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ts = time.perf_counter()
        cg.multiply(nA, nB, nC, desc, None, form="split", slices=args.slices, scheme=args.scheme,
                    operand_bits=args.operand_bits)
        e2e_steps.append((time.perf_counter() - ts) * 1e3)
    t_e2e = max_over_ranks((time.perf_counter() - t0) / args.steps, world)
    # the copy rates again: on a shared host they can drop while the leg runs
    copy_bw_after = pinned_copy_bandwidth(hA, A, stream)
    # one more call with timing events on the copy stream: where its time goes
    cg.set_phase_timing(True)
    ts = time.perf_counter()
    cg.multiply(nA, nB, nC, desc, None, form="split", slices=args.slices, scheme=args.scheme,
                    operand_bits=args.operand_bits)
    tl_wall = (time.perf_counter() - ts) * 1e3
    cg.set_phase_timing(False)
    tc = cg.counters()
    e2e_timeline = {"wall_ms": tl_wall, "first_inputs_ms": tc["host_first_inputs"] * 1e3,
                    "all_inputs_ms": tc["host_all_inputs"] * 1e3, "compute_end_ms": tc["host_compute_end"] * 1e3,
                    "copy_back_end_ms": tc["host_copy_back_end"] * 1e3,
                    "meaning": "device times from the call's start: the first inputs Q1 waits for on the device "
                               "(the first sub-quadrants of A11 and B11), all inputs on the device, last kernel "
                               "done, last C quadrant on the host"}
    barrier(world)

    # ---- plain FP64 Strassen of the same multiply, and the errors of both
    out = {}
    if rank == 0:
        def colmajor(x):
            y = torch.empty_like(x)
            cg.from_caps_layout(x, y, desc)
            torch.cuda.synchronize()
            return y.cpu().numpy()
        A_cm, B_cm = colmajor(A), colmajor(B)
        err_split = sampled_error(colmajor(C), A_cm, B_cm, n, args.samples)
        plain = None
        if not args.no_plain:
            Cp = torch.empty_like(A)
            step("plain", Cp)
            torch.cuda.synchronize()
            p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            p0.record(stream)
            step("plain", Cp)
            p1.record(stream)
            torch.cuda.synchronize()
            t_plain = p0.elapsed_time(p1) / 1e3
            err_plain = sampled_error(colmajor(Cp), A_cm, B_cm, n, args.samples)
            plain = {"value": 2.0 * n ** 3 / t_plain / 1e12, "ms_per_step": t_plain * 1e3, "steps": 1,
                     "error": err_plain, "pattern": pattern}
            del Cp
        out["split_error"] = err_split
        out["plain"] = plain
        del A_cm, B_cm
        if not args.no_wide:
            # config 3b: a = u 2^k, u uniform[-1,1), k uniform integer in [-20, 20]
            gw = torch.Generator(device=dev)
            gw.manual_seed(4)
            Aw = (torch.rand(n * n, dtype=torch.float64, device=dev, generator=gw) * 2 - 1) * torch.exp2(
                torch.randint(-20, 21, (n * n,), device=dev, generator=gw).to(torch.float64))
            Bw = (torch.rand(n * n, dtype=torch.float64, device=dev, generator=gw) * 2 - 1) * torch.exp2(
                torch.randint(-20, 21, (n * n,), device=dev, generator=gw).to(torch.float64))
            Cw = torch.empty_like(Aw)
            Aw_cm, Bw_cm = colmajor(Aw), colmajor(Bw)
            wide = {}
            for form in (("split",) if args.no_plain else ("split", "plain")):
                cg.multiply(Aw, Bw, Cw, desc, pattern, form=form, slices=args.slices, stream=stream.cuda_stream,
                            scheme=args.scheme, operand_bits=args.operand_bits)
                torch.cuda.synchronize()
                wide[form] = sampled_error(colmajor(Cw), Aw_cm, Bw_cm, n, args.samples)
                if form == "split":
                    wc = cg.counters()
                    wide["split_slices"], wide["split_moduli"] = wc["split_slices"], wc["split_moduli"]
            out["wide"] = wide
            del Aw, Bw, Cw, Aw_cm, Bw_cm
        out["copy_bw_late"] = pinned_copy_bandwidth(hA, A, stream)

    if rank == 0:
        peaks, peak_src = measured_peaks()
        pairs = cg.digit_pairs(s_used, nd_used) if not moduli else 0
        products = moduli if moduli else pairs  # tensor-core products per leaf
        gemm_kernel = "crt_gemm_kernel" if moduli else "split_gemm_kernel"
        unit_of_work = ("modular products: %d moduli x 2 m^3 per leaf" % moduli if moduli else
                        "digit-pair products: %d pairs x 2 m^3 per leaf" % pairs)
        per_launch_flops = 2.0 * products * gemm_m3 / max(gemm_launches, 1)
        per_launch_s = gemm_t / max(gemm_launches, 1)
        achieved = per_launch_flops / per_launch_s / 1e12 if per_launch_s > 0 else 0.0
        peak = float(peaks.get("bf16_tflops_sustained", peaks.get("bf16_tflops", 1700.0)))
        traffic = profiled_traffic(gemm_kernel)
        cpu = None
        if not args.no_cpu:
            try:
                times, cores, blas = cpu_whole_multiplies(n, r, 1)
                cpu = {"value": 2.0 * n ** 3 / times[0] / 1e12, "unit": "TFLOP/s", "cores": cores, "kind": "port",
                       "sample": cpu_sample_text(n, r, 1, cores, blas), "seconds": times[0]}
            except Exception as ex:  # the baseline is reported, never required
                cpu = {"value": None, "unit": "TFLOP/s", "cores": os.cpu_count(), "kind": "port",
                       "sample": "failed: %s" % ex}
        plain = out.get("plain")
        line = {
            "metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_split * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "CAPS Strassen multiply C=A*B, n=%d, r=%d, split base case (%s)" % (
                           n, r, "residues modulo %d moduli" % moduli if moduli else "%d digits" % s_used),
                       "n": n, "nrec": r, "pattern": pattern, "form": "split",
                       "scheme": "residues" if moduli else "digits", "moduli": moduli, "slices": s_used,
                       "operand_bits": bits_used if moduli else None, "operand_bits_choice": bits_how,
                       "diagonals": nd_used, "digit_pairs": pairs,
                       "inputs": "float64 uniform[-1,1) seeded (torch.Generator), CAPS layout",
                       "l2": "inputs larger than L2 (each matrix 2 GiB vs 129 MB L2)",
                       "parallelism": "replicas x%d" % world},
            "split_vs_plain": (value / world) / plain["value"] if plain else None,
            "plain_fp64": plain,
            "error": {"split": out.get("split_error"), "plain": plain["error"] if plain else None,
                      "wide_range_inputs": out.get("wide"),
                      "definition": "max over sampled (i,j) of |C_ij - C_ref_ij| / (|A||B|)_ij, and "
                                    "||C - C_ref||_2 / ||C_ref||_2 over the same entries; C_ref = binary128 dot"},
            "roofline": {"bound": "tensor", "kernel": gemm_kernel, "achieved": achieved, "peak": peak,
                         "unit": "TFLOP/s", "frac": achieved / peak if peak else None, "traffic": traffic,
                         "peak_source": "%s bf16_tflops_sustained (of %s)" % (peak_src, peak_src),
                         "flops_per_launch": per_launch_flops, "launches": gemm_launches,
                         "avg_launch_ms": per_launch_s * 1e3,
                         "unit_of_work": unit_of_work},
            "cpu_baseline": cpu,
            "memory_kernels": memory_kernels,
            "e2e": {"value": world * 2.0 * n ** 3 / t_e2e / 1e12, "unit": "TFLOP/s",
                    "h2d_bytes_per_step": 2 * n * n * 8, "d2h_bytes_per_step": n * n * 8,
                    "ms_per_step": t_e2e * 1e3, "step_ms": e2e_steps, "timeline": e2e_timeline,
                    "pinned_copy_gbs": copy_bw,
                    "pinned_copy_gbs_after_e2e": copy_bw_after,
                    "pinned_copy_gbs_after_error_checks": out.get("copy_bw_late"),
                    "api": "caps_multiply_host, pinned host buffers, no pattern given: top level 'd' + %s "
                           "with copies overlapped (its first subproduct a 'd' step too, started on the first "
                           "sub-quadrants of A11 and B11)" % e2e_pattern[1:]},
            "gpu_launches": launches,
            "clocks": clk.summary(),
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
