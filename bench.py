#!/usr/bin/env python
"""Benchmark of the Schwarz smoother hot path (SchwarzPreconditioner::vmult) on GB300.

Workload (the configuration the headline metric is quoted on): 3D Poisson, SIPG DG Q4 on the
unit cube with 64^3 Cartesian cells (32,768,000 DoFs), additive vertex-patch Schwarz smoother
(250,047 patches of 10^3 DoFs, 8 tiled colors), FP32 gather / fast-diagonalization / scatter
into FP64 vectors, relaxation 0.15.  One step = one vmult.  Inputs: f ~ U[-1,1] per DoF from
numpy's Philox generator (seed 0), synthetic -- there is no dataset in this domain.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun (N > 1) every rank runs an independent replica on its own GPU (the smoother
does not shard on one level; value = DoFs of all ranks / max time).  The reference arm times
the CPU oracle port (the reference itself needs deal.II, absent here) with all host threads.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import shutil
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "smoother DoF/s (SchwarzPreconditioner::vmult; CG+MG solve s to 1e-8 rel. residual and FP32 vs FP64 in 'solve')"


# (BX, BY, BZ, pencils per thread[, a warp per patch]) of the streamed kernel's six work
# decompositions, for k = 4
VARIANT_SHAPES = ["4,4,8,4", "4,4,8,5", "4,4,4,4", "4,4,16,4", "4,4,8,4,true", "4,4,4,4,true"]


def stream_kernel_name(k1, v):
    """Kernel name of decomposition v of the streamed smoother (pencil or plane passes)."""
    if v in (6, 7):
        return f"plane_kernel<PCfg<{k1},8,{8 if v == 6 else 4}>>"
    return f"stream_kernel<SCfg<{k1},{VARIANT_SHAPES[v]}>>"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--dim", type=int, default=3)
    ap.add_argument("--degree", type=int, default=4)
    ap.add_argument("--cells", type=int, default=64)
    ap.add_argument("--precision", choices=["fp32", "fp64"], default="fp32")
    ap.add_argument("--omega", type=float, default=0.15)
    ap.add_argument("--no-solve", action="store_true")
    ap.add_argument("--no-distorted", action="store_true")
    ap.add_argument("--no-c0ip", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--batch-problems", type=int, default=512)
    ap.add_argument("--distortion", type=float, default=0.15)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--kernel", choices=["auto", "color", "stream"], default="auto")
    ap.add_argument("--stream-variant", type=int, default=-1,
                    help="run this decomposition of the streamed kernel instead of the autotuned one "
                         "(profiling; also skips the FP64 arm)")
    ap.add_argument("--level-kernels", action="store_true",
                    help="time only the level operator (FP64, FP32) and the transfers on the "
                         "--cells level (also the command the operator profile captures)")
    ap.add_argument("--precision-sweep", action="store_true",
                    help="only the CG + V-cycle solve of the --cells level with FP32 smoothers on all "
                         "levels but one, which computes in FP64 (each level in turn), next to "
                         "all-FP32 and all-FP64: iterations and seconds, one JSON line")
    ap.add_argument("--no-dgq3-2d", action="store_true",
                    help="skip the 2D SIPG DGQ3 64^2 section (both penalty modes)")
    ap.add_argument("--profile-case", choices=["mapped", "perpatch", "k5", "cg2d", "cg2d_eager", "cg3dk5_eager",
                                               "c0ip", "mlp", "host"],
                    help="run one small workload of a secondary kernel three times and exit (the "
                         "commands the ncu profiles capture): mapped = mapped SIPG operator on a "
                         "distorted 3D DGQ3 24^3 level; perpatch = FP32 smoother on per-patch 1-D "
                         "problems (distorted 3D DGQ3 56^3, surrogate widths), streamed decomposition 4 "
                         "and the per-color kernel; k5 = FP32 smoother on 3D DGQ5 40^3 (Cartesian), "
                         "streamed decomposition 2 and the per-color kernel; cg2d = CG + V-cycle on 2D SIPG DGQ3 64^2 (2 root "
                         "cells, damping 0.25, dense coarse solve), one solve after a warm-up solve (cg2d_eager: the same "
                         "without CUDA graphs, every kernel launched from the host); cg3dk5_eager = the "
                         "same for 3D SIPG DGQ5 32^3 with FP32 smoothers (the batch's largest problems); c0ip = C0IP FE_Q(3) 512^2 operator and "
                         "FP32 Bilaplacian-FD smoother; mlp = one training epoch of the "
                         "87 -> 3 x 64 -> 108 network on 119,164 samples; host = the FP32 "
                         "smoother between pinned host buffers on 3D DGQ4 64^3")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def workload(args):
    n, k, dim = args.cells, args.degree, args.dim
    N = n ** dim * (k + 1) ** dim
    P = (n - 1) ** dim
    nl = 2 * (k + 1)
    flops_per_patch = 4 * dim * nl ** (dim + 1) + 2 * nl ** dim
    return dict(N=N, P=P, n1d=nl, flops_per_patch=flops_per_patch,
                flops=P * flops_per_patch, bytes=N * 16)


def workload_name(args, W):
    """config.workload of both arms (the same string, so that their lines compare)."""
    n, k = args.cells, args.degree
    prec = "FP32" if args.precision == "fp32" else "FP64"
    return (f"additive vertex-patch Schwarz vmult, 3D SIPG DGQ{k}, {n}^3 cells, {W['N']} DoFs, "
            f"{W['P']} patches of {W['n1d']}^3, {prec} smoother / FP64 vectors")


def philox_src(N, seed):
    import numpy as np
    return np.random.Generator(np.random.Philox(seed)).uniform(-1.0, 1.0, N)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 100 ms (recipe's clocks line)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None
        self.t0 = self.t1 = None

    def start(self):
        if not shutil.which("nvidia-smi"):
            return
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        self.proc = subprocess.Popen(
            ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu=timestamp,{self.FIELDS}",
             "--format=csv,noheader,nounits", "-lms", "100"],
            stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        time.sleep(0.3)

    def mark(self, which):
        setattr(self, which, time.time())

    def stop(self):
        if not self.proc:
            return None
        time.sleep(0.15)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 10:
                continue
            try:
                rows.append(dict(sm=float(parts[2]), smax=float(parts[3]), active=parts[5],
                                 hw=parts[6], hwt=parts[7], swt=parts[8], pcap=parts[9]))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return None
        # samples taken while the timed loop ran (the last ones if it was shorter than 100 ms)
        n_timed = max(1, min(len(rows), int((self.t1 - self.t0) / 0.1) + 2)) if self.t0 else len(rows)
        sel = rows[-(n_timed + 1):-1] if len(rows) > n_timed else rows
        reasons = set()
        for r in sel:
            for key, name in (("hw", "hw_slowdown"), ("hwt", "hw_thermal_slowdown"),
                              ("swt", "sw_thermal_slowdown"), ("pcap", "sw_power_cap")):
                if r[key].lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(r["sm"] for r in sel), "sm_max_mhz": max(r["smax"] for r in sel),
                "reasons": sorted(reasons), "samples": len(sel)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


def ncu_traffic(dim, k):
    """DRAM bytes per vmult of the streamed kernel plus its fix-up pass at 64^3 cells, from the
    committed ncu summary (each captured on its own at 48^3 and scaled by DoFs)."""
    path = os.path.join(ROOT, "profiles", f"stream_kernel_{dim}d_k{k}_48cubed.md")
    if not os.path.exists(path):
        return None
    total, found = 0.0, False
    for line in open(path):
        m = re.match(r"\s*(fixup_)?dram_bytes_per_launch_full_size:\s*([0-9.eE+]+)", line)
        if m:
            total += float(m.group(2))
            found = True
    return total if found else None


def cpu_baseline(args, W):
    """The reference's CPU path restated with SIMD macro patches (oracle/simd_baseline.c: 8 FP64
    lanes per macro patch, lane-wise eigenvectors, FMA, OpenMP over the macro patches of a
    color), FP64: full vmults of the same workload on all host threads (a few seconds), and a
    bounded sample (1/16 of the patches, all colors) on one thread."""
    from oracle import oracle as O
    O.build()
    import numpy as np
    threads = O.simd_num_threads()
    n = args.cells
    h = O.SimdSchwarzHandle(args.dim, args.degree, (n,) * args.dim, patch_variant=1, omega=args.omega)
    src = philox_src(W["N"], args.seed)
    dst = np.zeros_like(src)
    h.apply(dst, src)  # warm-up (page-in)
    reps, t0 = 0, time.perf_counter()
    while True:
        h.apply(dst, src)
        reps += 1
        el = time.perf_counter() - t0
        if el > 8.0 or reps >= 5:
            break
    per = el / reps
    P = h.n_patches
    part = max(1, P // 16)
    O.simd_set_num_threads(1)
    t0 = time.perf_counter()
    h.apply_range(0, part, dst, src)
    one = (time.perf_counter() - t0) * P / part
    O.simd_set_num_threads(threads)
    h.close()
    return {"value": W["N"] / per, "unit": "DoF/s", "cores": threads, "kind": "port",
            "sample": f"{reps} full FP64 vmults of the same 3D DGQ{args.degree} {n}^3 workload, "
                      f"{per:.3f} s each, {threads} OpenMP threads; SIMD restatement of the "
                      f"reference's CPU path (macro patches of 8 FP64 lanes, FMA)",
            "single_core": {"value": W["N"] / one, "unit": "DoF/s", "cores": 1,
                            "sample": f"patches 0..{part} of {P} on one thread, scaled to a vmult "
                                      f"({one:.2f} s)"}}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    W = workload(args)
    from oracle import oracle as O
    O.build()
    import numpy as np
    n = args.cells
    h = O.SimdSchwarzHandle(args.dim, args.degree, (n,) * args.dim, patch_variant=1, omega=args.omega)
    src = philox_src(W["N"], args.seed)
    dst = np.zeros_like(src)
    # one step = a bounded sample: 1/8 of the patches (about one color's worth) per step
    P = h.n_patches
    chunk = max(1, P // 8)
    steps, warm = args.steps, args.warmup
    for i in range(warm):
        h.apply_range((i * chunk) % P, min(P, (i * chunk) % P + chunk), dst, src)
    t0 = time.perf_counter()
    done = 0
    for i in range(steps):
        b = (i * chunk) % P
        e = min(P, b + chunk)
        h.apply_range(b, e, dst, src)
        done += e - b
    el = time.perf_counter() - t0
    h.close()
    value = W["N"] * (done / P) / el
    threads = O.simd_num_threads()
    line = {"metric": METRIC, "value": value, "unit": "DoF/s", "n_gpus": args.gpus, "steps": steps,
            "warmup": warm, "ms_per_step": 1e3 * el / steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": workload_name(args, W), "sample_per_step": f"{chunk} of {P} patches"},
            "cpu_baseline": {"value": value, "unit": "DoF/s", "cores": threads, "kind": "port",
                             "sample": f"{steps} steps of {chunk} patches (1/8 of a vmult) each, "
                                       f"SIMD restatement of the reference's CPU path (macro "
                                       f"patches of 8 FP64 lanes, FMA), {threads} OpenMP threads"},
            "e2e": {"value": value, "unit": "DoF/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args):
    import numpy as np
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    import tpss_gb300 as tpss
    W = workload(args)
    n, k, dim = args.cells, args.degree, args.dim
    prec = tpss.Precision.fp32 if args.precision == "fp32" else tpss.Precision.fp64
    sh = tpss.SubdomainHandler(tpss.SubdomainHandler.AdditionalData(
        dim=dim, degree=k, n_cells=(n,) * dim, patch_variant=tpss.PatchVariant.vertex))
    p = tpss.SchwarzPreconditioner()
    variant = {"auto": 0, "color": 1, "stream": 2}[args.kernel]
    forced = args.stream_variant >= 0
    p.initialize(sh, None, tpss.SchwarzPreconditioner.AdditionalData(
        relaxation=args.omega, precision=prec, kernel_variant=2 if forced else variant,
        stream_variant=max(0, args.stream_variant)))
    # the column-streamed kernel runs for 3D vertex patches in FP32 with k <= 4
    streamed = forced or (args.kernel == "stream" or (args.kernel == "auto" and prec == tpss.Precision.fp32
                                                      and dim == 3 and k <= 4))
    n_colors = sh.n_colors()
    launches_per_step = 2 if streamed else n_colors  # stream + fix-up, or one per color
    src_h = philox_src(W["N"], args.seed + rank)
    src = torch.tensor(src_h, dtype=torch.float64, device="cuda")
    dst = torch.empty_like(src)
    stream = torch.cuda.current_stream()
    # the library's autotuner picks the work decomposition of the kernel for this level
    if forced:
        tuned, tuned_ms = args.stream_variant, []
    else:
        tuned, tuned_ms = p.autotune(dst, src, reps=5)

    def barrier():
        if dist is not None:
            dist.barrier()

    clocks = ClockSampler(local)
    clocks.start()
    for _ in range(args.warmup):
        p.vmult(dst, src)
    td0 = p.get_time_data()
    barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks.mark("t0")
    e0.record(stream)
    for _ in range(args.steps):
        p.vmult(dst, src)
    e1.record(stream)
    torch.cuda.synchronize()
    clocks.mark("t1")
    barrier()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1) / args.steps
    td1 = p.get_time_data()
    t_max = ms
    if dist is not None:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_max = float(t.item())
    value = world * W["N"] / (t_max * 1e-3)

    # dominant kernel: the fused color kernel, timed by the library's "Apply inverses" CUDA
    # events on the launching stream (colors launched back to back)
    apply_s = td1[1].time - td0[1].time
    apply_calls = td1[1].n_calls - td0[1].n_calls
    P = W["P"]
    if streamed:
        # one streamed launch (+ a small fix-up) per vmult covers all patches; the timed
        # region includes the fix-up
        per_launch = apply_s / max(1, apply_calls)
        units_per_launch = P
        bytes_launch = W["bytes"]  # compulsory: read src, write dst once (8 B + 8 B per DoF)
    else:
        per_launch = apply_s / max(1, apply_calls * n_colors)
        units_per_launch = P / n_colors
        bytes_launch = units_per_launch * W["n1d"] ** dim * 24  # gather src + RMW dst
    flops_launch = units_per_launch * W["flops_per_patch"]
    hbm_peak, hbm_kind = measured_peaks()
    fma_peak = tpss_fma_peak(tpss, prec)
    achieved_gbs = bytes_launch / per_launch / 1e9
    achieved_tf = flops_launch / per_launch / 1e12
    traffic = ncu_traffic(dim, k) if streamed else None
    if traffic is not None:
        # the committed figure is for 64^3 cells (scaled from a 48^3 capture by DoFs); traffic
        # grows with the DoFs of the level
        traffic *= W["N"] / (64 ** 3 * (k + 1) ** 3)
    roofline = {"bound": "hbm", "achieved": achieved_gbs, "peak": hbm_peak, "unit": "GB/s",
                "frac": achieved_gbs / hbm_peak, "traffic": traffic,
                "peak_source": f"{hbm_kind} (MEASURED_PEAKS.json hbm_gbs)",
                "kernel": (f"{stream_kernel_name(k + 1, tuned)} + fixup_list_kernel" if streamed
                           else f"schwarz_color_kernel<{args.precision},3,2,{k + 1}>"),
                "per_launch_ms": per_launch * 1e3,
                "algorithmic_bytes_per_launch": bytes_launch,
                "traffic_source": ("ncu dram__bytes_read.sum + dram__bytes_write.sum of stream_kernel and of "
                                   "fixup_list_kernel, each captured at 48^3 and scaled by DoFs "
                                   "(profiles/stream_kernel_3d_k4_48cubed.md)") if traffic is not None else None,
                "binding": "fp32 FMA pipe (CUDA cores)" if prec == tpss.Precision.fp32 else "fp64 FMA pipe",
                "compute": {"achieved": achieved_tf, "peak": fma_peak / 1e12, "unit": "TFLOP/s",
                            "frac": achieved_tf * 1e12 / fma_peak,
                            "peak_source": "measured in this run (tpss_diag_fma_peak)",
                            "algorithmic_flops_per_launch": flops_launch,
                            "executed_flops_per_launch": executed_fd_flops(n, k, dim) if dim == 3 else None,
                            "executed_frac": (executed_fd_flops(n, k, dim) / per_launch / fma_peak
                                              if dim == 3 else None)}}

    out = {"metric": METRIC, "value": value, "unit": "DoF/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": t_max, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32" if prec == tpss.Precision.fp32 else "f64",
           "data": "synthetic (f ~ U[-1,1] per DoF, numpy Philox seed %d)" % args.seed,
           "config": {"workload": workload_name(args, W),
                      "dim": dim, "degree": k, "cells_per_direction": n, "n_dofs": W["N"],
                      "n_patches": P, "n_colors": n_colors, "relaxation": args.omega,
                      "l2": "inputs larger than L2 (src and dst 262 MB each)",
                      "autotuned_variant": tuned, "autotune_ms_per_variant": tuned_ms,
                      "parallelism": "replicas" if world > 1 else "single GPU"},
           "gpu_launches": args.steps * launches_per_step,
           "roofline": roofline, "clocks": clk}

    if not args.no_e2e:
        out["e2e"] = e2e(tpss, p, src_h, args, W, world, dist)
    if prec == tpss.Precision.fp32 and not forced:
        out["fp64"] = fp64_arm(tpss, sh, src, src_h, args, W, world, dist)
    if not args.no_solve:
        out["operator"] = operator_time(tpss, sh, src, W)
        out["solve"] = solve_times(tpss, args)
    if not args.no_dgq3_2d:
        out["dgq3_2d"] = dgq3_2d_section(tpss, args)
    if not args.no_distorted:
        out["distorted"] = distorted_section(tpss, args)
    if not args.no_c0ip:
        out["c0ip"] = c0ip_section(tpss, args)
    if not args.no_batch:
        out["batch"] = batch_section(tpss, args)
    if rank == 0 and not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline(args, W)
    if rank == 0:
        print(json.dumps(out), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def tpss_fma_peak(tpss, prec):
    import ctypes as C
    v = C.c_double(0.0)
    tpss._lib.check(tpss.load().tpss_diag_fma_peak(prec, 1 << 16, C.byref(v), None))
    v2 = C.c_double(0.0)
    tpss._lib.check(tpss.load().tpss_diag_fma_peak(prec, 1 << 16, C.byref(v2), None))
    return max(v.value, v2.value)


def e2e(tpss, p, src_h, args, W, world, dist):
    """Same metric through the C ABI with host buffers: tpss_precond_vmult_host copies src
    in, applies the smoother and copies dst out (pinned buffers, copies overlapping the kernel)."""
    import torch
    N = W["N"]
    h_src = torch.tensor(src_h, dtype=torch.float64).pin_memory()
    h_dst = torch.empty(N, dtype=torch.float64).pin_memory()
    stream = torch.cuda.current_stream()
    steps = max(3, min(args.steps, 50))

    def step():
        # SchwarzPreconditioner::vmult on host vectors through the C ABI: the library copies
        # src in and dst out, pipelined with the streamed kernel along z
        p.vmult_host(h_dst, h_src)

    for _ in range(3):
        step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    if dist is not None:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    return {"value": world * N / (ms * 1e-3), "unit": "DoF/s", "h2d_bytes_per_step": N * 8,
            "d2h_bytes_per_step": N * 8, "ms_per_step": ms, "steps": steps}


def executed_fd_flops(n, k, dim):
    """Floating-point operations the FD kernels execute per vmult on the Cartesian n^dim level:
    per patch and direction a forward and a backward pass over n1^(dim-1) pencils, 2 h^2
    multiply-adds plus n1 additions per pencil where the 1-D problem is mirror-symmetric (the
    even/odd split, h = n1/2: interior vertices), n1^2 multiply-adds elsewhere; one
    reciprocal multiplication per patch DoF and one damping multiplication."""
    n1, h = 2 * (k + 1), k + 1
    pencils = n1 ** (dim - 1)
    sym_frac = max(0, n - 3) / max(1, n - 1)  # vertex positions 2..n-2 of 1..n-1 per direction
    per_dir = 2 * pencils * (sym_frac * (2 * 2 * h * h + n1) + (1 - sym_frac) * 2 * n1 * n1)
    return (n - 1) ** dim * (dim * per_dir + 2 * n1 ** dim)


def fp64_arm(tpss, sh, src, src_h, args, W, world, dist):
    """The FP64 smoother on the same level (the precision of the reference's arithmetic): device
    DoF/s, e2e through tpss_precond_vmult_host (copy in, vmult, copy out), and the roofline of the
    FP64 pipe that binds it (executed operations / measured FP64 FMA peak)."""
    import torch
    p = tpss.SchwarzPreconditioner()
    p.initialize(sh, None, tpss.SchwarzPreconditioner.AdditionalData(relaxation=args.omega,
                                                                     precision=tpss.Precision.fp64))
    dst = torch.empty_like(src)
    chosen, tuned_ms = p.autotune(dst, src, reps=2)
    for _ in range(3):
        p.vmult(dst, src)
    torch.cuda.synchronize()
    steps = 10
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        p.vmult(dst, src)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    ex = executed_fd_flops(args.cells, args.degree, args.dim)
    peak = tpss_fma_peak(tpss, tpss.Precision.fp64)
    ee = e2e(tpss, p, src_h, argparse.Namespace(steps=5), W, world, dist)
    return {"value": world * W["N"] / (ms * 1e-3), "unit": "DoF/s", "ms_per_step": ms, "steps": steps,
            "kernel": f"schwarz_color_kernel<double,3,2,{args.degree + 1}> x {sh.n_colors()} colors",
            "autotuned_variant": chosen, "autotune_ms_per_variant": tuned_ms,
            "e2e": ee,
            "roofline": {"bound": "fp64 pipe", "achieved": ex / (ms * 1e-3) / 1e12, "peak": peak / 1e12,
                         "unit": "TFLOP/s", "frac": ex / (ms * 1e-3) / peak,
                         "peak_source": "measured in this run (tpss_diag_fma_peak, FP64)",
                         "executed_flops_per_vmult": ex,
                         "algorithmic_dense_flops_per_vmult": W["flops"],
                         "hbm_frac": W["bytes"] / (ms * 1e-3) / 1e9 / measured_peaks()[0]}}


def operator_time(tpss, sh, src, W):
    """FP64 matrix-free SIPG operator (MF::Operator::vmult) on the same level: the residual
    inside every smoothing step and CG iteration."""
    import torch
    op = tpss.LaplaceOperator(sh, 1.0)
    dst = torch.empty_like(src)
    for _ in range(3):
        op.vmult(dst, src)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 10
    e0.record()
    for _ in range(reps):
        op.vmult(dst, src)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    # the same product in FP32 arithmetic (the level operator of a single-precision V-cycle)
    for _ in range(3):
        op.vmult_fp32(dst, src)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(reps):
        op.vmult_fp32(dst, src)
    e1.record()
    torch.cuda.synchronize()
    ms32 = e0.elapsed_time(e1) / reps
    k, dim = sh.get_additional_data().degree, sh.get_additional_data().dim
    cells = W["N"] // (k + 1) ** dim
    npt = k + 1
    # multiply-adds per cell of the evaluation the kernel performs: per direction and pencil the
    # own 1-D block (np^2) and two neighbour couplings with unit face-value vectors (2 np + 2
    # each); mass contractions shared between the direction terms (2 in 2D, 5 in 3D, np^2 per
    # pencil)
    mass_passes = 2 if dim == 2 else 5
    fma_cell = npt ** (dim - 1) * (dim * npt * npt + mass_passes * npt * npt + dim * 2 * (2 * npt + 2))
    return {"ms": ms, "dof_per_s": W["N"] / (ms * 1e-3),
            "fp64_tflops": 2 * fma_cell * cells / (ms * 1e-3) / 1e12,
            "algorithmic_fma_per_cell": fma_cell, "fp32_ms": ms32,
            "fp32_tflops": 2 * fma_cell * cells / (ms32 * 1e-3) / 1e12}


def solve_times(tpss, args):
    """CG + GMG solve to 1e-8 relative residual, FP32 vs FP64 smoother (same workload mesh,
    one root cell, 7 levels, dense coarse solve, V-cycle captured in a CUDA graph)."""
    import torch
    res = {}
    n, k, dim = args.cells, args.degree, args.dim
    N = n ** dim * (k + 1) ** dim
    f = torch.tensor(philox_src(N, args.seed), dtype=torch.float64, device="cuda")
    for name, prec, opp in (("fp32", tpss.Precision.fp32, tpss.Precision.fp64),
                            ("fp32_vcycle", tpss.Precision.fp32, tpss.Precision.fp32),
                            ("fp64", tpss.Precision.fp64, tpss.Precision.fp64)):
        mg = tpss.MultigridSolver(dim, k, 1, n, relaxation=args.omega, precision=prec,
                                  coarse_solver=1, use_graph=True, vcycle_precision=opp, autotune=True)
        u = torch.zeros_like(f)
        mg.vmult(u, f)  # warm-up: graph capture
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        it, hist = mg.solve(u, f, rel_tol=1e-8)
        torch.cuda.synchronize()
        el = time.perf_counter() - t0
        res[name] = {"seconds": el, "iterations": it, "final_rel_residual": float(hist[-1] / hist[0])}
        del mg
    res["fp32_over_fp64_time"] = res["fp32"]["seconds"] / res["fp64"]["seconds"]
    res["fp32_vcycle_over_fp64_time"] = res["fp32_vcycle"]["seconds"] / res["fp64"]["seconds"]
    res["workload"] = (f"CG + V-cycle (1 pre/1 post additive vertex-patch Schwarz step, omega "
                       f"{args.omega}), 3D SIPG DGQ{k} {n}^3, f ~ U[-1,1], to 1e-8 rel. residual; "
                       f"fp32: FP32 smoothers; fp32_vcycle: FP32 smoothers and FP32 level operators "
                       f"in the V-cycle (outer CG and coarse solve FP64); fp64: all FP64; smoother "
                       f"kernel decompositions autotuned per level at setup (outside the timed solve)")
    return res


def dgq3_2d_section(tpss, args):
    """2D SIPG DGQ3 on 64^2 cells (65,536 DoFs), additive vertex patches of 8 x 8 DoFs, FP64 as
    stated (damping 0.5, penalty 2(k+1)^2/h) and with the reference's penalty: smoother
    milliseconds and DoF/s, lambda_max(P A) of the finest level, CG + V-cycle (2 root cells,
    6 levels, dense coarse solve, graphs) to 1e-8 at damping 0.5 and at the reference's 0.25."""
    import torch
    dim, k, nrep, n = 2, 3, 2, 64
    N = n ** dim * (k + 1) ** dim
    f = torch.tensor(philox_src(N, args.seed), dtype=torch.float64, device="cuda")
    sh = tpss.SubdomainHandler(tpss.SubdomainHandler.AdditionalData(dim=dim, degree=k, n_cells=(n, n),
                                                                     patch_variant=1))
    out = {"workload": "2D SIPG DGQ3 64^2 cells, 65536 DoFs, additive vertex patches (8x8 DoFs, 4 colors), "
                       "f ~ U[-1,1]; CG + V-cycle (1 pre/1 post smoothing step) to 1e-8, 2 root cells, "
                       "dense coarse solve"}
    for pen_name, mode in (("kp1sq", tpss.Penalty.kp1sq), ("reference", tpss.Penalty.reference)):
        r = {}
        for prec_name, prec in (("fp64", tpss.Precision.fp64), ("fp32", tpss.Precision.fp32)):
            p = tpss.SchwarzPreconditioner()
            p.initialize(sh, None, tpss.SchwarzPreconditioner.AdditionalData(
                relaxation=0.5, precision=prec, penalty_mode=mode))
            d = torch.empty_like(f)
            for _ in range(10):
                p.vmult(d, f)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(200):
                p.vmult(d, f)
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / 200
            r[f"smoother_{prec_name}_ms"] = ms
            r[f"smoother_{prec_name}_dof_per_s"] = N / (ms * 1e-3)
        probe = tpss.MultigridSolver(dim, k, nrep, n, relaxation=0.5, coarse_solver=1,
                                     auto_relaxation=True, penalty_mode=mode)
        r["lambda_max_PA_finest"] = probe.relaxation(probe.n_levels - 1)[1]
        del probe
        for om in (0.5, 0.25):
            for prec_name, prec in (("fp64", tpss.Precision.fp64), ("fp32", tpss.Precision.fp32)):
                mg = tpss.MultigridSolver(dim, k, nrep, n, relaxation=om, precision=prec, coarse_solver=1,
                                          use_graph=True, penalty_mode=mode)
                u = torch.zeros_like(f)
                mg.vmult(u, f)  # graph capture
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                try:
                    it, hist = mg.solve(u, f, rel_tol=1e-8, max_iter=100)
                    torch.cuda.synchronize()
                    res = {"seconds": time.perf_counter() - t0, "iterations": it,
                           "final_rel_residual": float(hist[-1] / hist[0])}
                except tpss.TPSSNotConverged:
                    torch.cuda.synchronize()
                    res = {"converged": False, "max_iter": 100,
                           "why": "damping x lambda_max(P A) > 2: the smoother amplifies and the V-cycle "
                                  "is indefinite (the oracle does not converge either)"}
                r[f"solve_damping{om}_{prec_name}"] = res
                del mg
        out[pen_name] = r
    return out


def distorted_section(tpss, args):
    """Distorted 3D DGQ3 32^3 level (interior vertices moved by `distortion` x the shortest
    edge in random directions, as the reference's distort_random): train the learned local
    solver's network on the ~200k patches of seven other meshes, then solve CG + V-cycle to 1e-8 with
    surrogate (FP64, FP32), Kronecker-sum-fitted, rank-2 Kronecker (KSVD), learned and exact
    (FP32) local solvers; measured local inverse errors of the separable solvers."""
    import numpy as np
    import torch
    from tpss_gb300.mesh import distorted_cube
    dim, k, n, fac = 3, 3, 32, args.distortion
    out = {"workload": f"3D SIPG DGQ{k} {n}^3 distorted mesh (vertices moved {fac} x shortest edge), "
                       f"CG + V-cycle to 1e-8, additive vertex patches, damping 0.15 scaled per level by "
                       f"8 / (1.05 lambda_max(P A)), dense coarse solve, smoother kernel decompositions "
                       f"autotuned per level at setup"}
    t0 = time.perf_counter()
    xs, ys = [], []
    for seed in range(100, 107):
        X = distorted_cube(dim, [n] * dim, seed, fac)
        sh = tpss.SubdomainHandler(tpss.SubdomainHandler.AdditionalData(
            dim=dim, degree=k, n_cells=(n,) * dim, patch_variant=tpss.PatchVariant.vertex, vertex_coords=X))
        op = tpss.LaplaceOperator(sh)
        xs.append(tpss.learned_features(sh))
        ys.append(tpss.learned_targets(sh, op))
        del op, sh
    torch.cuda.synchronize()
    x, y = torch.cat(xs), torch.cat(ys)
    t1 = time.perf_counter()
    m = tpss.MLP(x.shape[1], y.shape[1], n_hidden=64, n_hidden_layers=3, seed=1)
    l0 = m.loss(x, y)
    hist = m.train(x, y, epochs=40, batch=256, lr=1e-3, seed=2)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    out["training"] = {"patches": int(x.shape[0]), "inputs": int(x.shape[1]), "outputs": int(y.shape[1]),
                       "network": "3 x 64 tanh, Adam lr 1e-3, batch 256, 40 epochs",
                       "data_seconds": t1 - t0, "train_seconds": t2 - t1,
                       "loss_initial": l0, "loss_final": float(hist[-1])}
    X = distorted_cube(dim, [n] * dim, 7, fac)
    N = n ** dim * (k + 1) ** dim
    f = torch.tensor(philox_src(N, args.seed), dtype=torch.float64, device="cuda")
    fp64, fp32 = tpss.Precision.fp64, tpss.Precision.fp32
    # measured local inverse error ||A_j^-1 - B_j||_F / ||A_j^-1||_F of every local solver on
    # a sample of 512 patches spread over the finest level (exact FP64 inverses on the GPU)
    sh = tpss.SubdomainHandler(tpss.SubdomainHandler.AdditionalData(
        dim=dim, degree=k, n_cells=(n,) * dim, patch_variant=tpss.PatchVariant.vertex, vertex_coords=X))
    op = tpss.LaplaceOperator(sh)
    P = sh.n_subdomains()
    first = P // 3
    errs = {}
    for name, ls, model in (("surrogate", tpss.LocalSolver.fd, None), ("ksum", tpss.LocalSolver.ksum, None),
                            ("ksvd", tpss.LocalSolver.ksvd, None), ("learned", tpss.LocalSolver.learned, m)):
        p = tpss.SchwarzPreconditioner()
        p.initialize(sh, op, tpss.SchwarzPreconditioner.AdditionalData(relaxation=0.15, local_solver=ls,
                                                                       model=model))
        e = tpss.local_inverse_error(p, op, first, 512)
        errs[name] = {"mean": float(e.mean()), "median": float(np.median(e)), "max": float(e.max())}
        del p
    out["local_inverse_error"] = dict(errs, sample=f"patches {first}..{first + 511} of {P}",
                                      measure="||A_j^-1 - B_j||_F / ||A_j^-1||_F, A_j exact (FP64 inverse)")
    del op, sh
    runs = (("surrogate_fp64", tpss.LocalSolver.fd, fp64, None, fp64),
            ("surrogate_fp32", tpss.LocalSolver.fd, fp32, None, fp64),
            ("ksum_fp32", tpss.LocalSolver.ksum, fp32, None, fp64),
            ("ksvd_fp32", tpss.LocalSolver.ksvd, fp32, None, fp64),
            ("learned_fp32", tpss.LocalSolver.learned, fp32, m, fp64),
            ("learned_fp32_vcycle", tpss.LocalSolver.learned, fp32, m, fp32),
            ("exact_fp32", tpss.LocalSolver.exact, fp32, None, fp64))
    for name, ls, prec, model, vprec in runs:
        ts = time.perf_counter()
        mg = tpss.MultigridSolver(dim, k, 2, n, relaxation=0.15, precision=prec, coarse_solver=1,
                                  use_graph=True, vertex_coords=X, local_solver=ls, model=model,
                                  auto_relaxation=True, vcycle_precision=vprec, autotune=True)
        torch.cuda.synchronize()
        setup = time.perf_counter() - ts
        u = torch.zeros_like(f)
        mg.vmult(u, f)  # warm-up: graph capture
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        try:
            it, h = mg.solve(u, f, rel_tol=1e-8, max_iter=300)
            torch.cuda.synchronize()
            out[name] = {"setup_seconds": setup, "seconds": time.perf_counter() - t0, "iterations": it,
                         "damping_per_level": [round(mg.relaxation(l)[0], 5) for l in range(1, mg.n_levels)]}
        except tpss.TPSSNotConverged:
            out[name] = {"setup_seconds": setup, "iterations": "not converged in 300"}
        del mg
    b = out["surrogate_fp64"]
    for name in ("learned_fp32", "learned_fp32_vcycle"):
        a = out[name]
        if "seconds" in a and "seconds" in b:
            out[f"{name}_over_surrogate_fp64_time"] = a["seconds"] / b["seconds"]
    return out


def c0ip_section(tpss, args):
    """2D clamped C0IP biharmonic, FE_Q(3), 256^2 cells (588,289 interior nodes): smoother
    throughput and CG + V-cycle to 1e-8 with the FP32 fast-diagonalization local solver (patch
    matrix without the mixed term, a rank-2 Kronecker sum) against FP64 exact local inverses."""
    import torch
    k, n = 3, 256
    N = (n * k - 1) ** 2
    f = torch.tensor(philox_src(N, args.seed), dtype=torch.float64, device="cuda")
    out = {"workload": f"2D C0IP biharmonic FE_Q({k}) {n}^2 cells, {N} DoFs, additive vertex patches "
                       f"of {(2 * k - 1) ** 2} nodes, damping 0.25, CG + V-cycle to 1e-8, dense coarse solve"}
    for name, ls, prec in (("fd_fp32", tpss.LocalSolver.fd, tpss.Precision.fp32),
                           ("fd_fp64", tpss.LocalSolver.fd, tpss.Precision.fp64),
                           ("exact_fp64", tpss.LocalSolver.exact, tpss.Precision.fp64)):
        P = tpss.C0IPBiharmonic(k, 2, n, local_solver=ls, precision=prec, relaxation=0.25)
        d = torch.empty_like(f)
        for _ in range(3):
            P.smooth(d, f)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(20):
            P.smooth(d, f)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / 20
        u = torch.zeros_like(f)
        P.solve(u, f, rel_tol=0.5, max_iter=200)  # warm-up: captures the V-cycle graph
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        it, hist = P.solve(u, f, rel_tol=1e-8, max_iter=200)
        torch.cuda.synchronize()
        out[name] = {"smoother_ms": ms, "smoother_dof_per_s": N / (ms * 1e-3),
                     "solve_seconds": time.perf_counter() - t0, "iterations": it}
        del P
    out["fd_fp32_over_exact_fp64_time"] = out["fd_fp32"]["solve_seconds"] / out["exact_fp64"]["solve_seconds"]
    return out


def batch_section(tpss, args):
    """Many independent Poisson SIPG problems (dimension 2/3, degree 2..7 and mesh 8^d..64^d drawn
    from the seed; a draw beyond the per-problem or the total DoF cap is rejected and drawn again;
    one root cell, dense coarse solve, V-cycles in CUDA graphs, kernel decompositions chosen by the
    autotuner per level shape, FP32 smoothers, FP64 CG) solved as one batch (every problem's
    device-side CG loop launched once on one of 64 streams), against solving them one after the
    other with the single-problem solver (the same device loops, one synchronization each)."""
    import numpy as np
    import torch
    cap_total, cap_problem = 96_000_000, 8_000_000
    problems, rejected = tpss.draw_batch_problems(args.batch_problems, args.seed + 4, cap_total, cap_problem)
    for pr in problems:
        pr["precision"] = tpss.Precision.fp32
    t0 = time.perf_counter()
    b = tpss.BatchSolver(problems, n_streams=64)
    fs = [torch.tensor(philox_src(n, args.seed + i), dtype=torch.float64, device="cuda")
          for i, n in enumerate(b.n_dofs)]
    us = [torch.empty_like(f) for f in fs]
    b.solve(us, fs)  # warm-up: captures every problem's V-cycle graph
    torch.cuda.synchronize()
    setup = time.perf_counter() - t0
    t0 = time.perf_counter()
    its = b.solve(us, fs)
    torch.cuda.synchronize()
    t_batch = time.perf_counter() - t0
    # the same problems one after the other through the single-problem solver objects
    mgs = []
    for i in range(len(problems)):
        h = tpss._lib.C.c_void_p()
        tpss.check(tpss.load().tpss_batch_problem(b._h, i, tpss._lib.C.byref(h)))
        mgs.append(h)
    t0 = time.perf_counter()
    hist = np.zeros(201)
    it_c = tpss._lib.C.c_int(0)
    for h, u, f, n in zip(mgs, us, fs, b.n_dofs):
        tpss.check(tpss.load().tpss_mg_cg_solve(h, tpss._ptr(u, n), tpss._ptr(f, n), 1e-8, 1e-14, 200,
                                                tpss._lib.C.byref(it_c),
                                                hist.ctypes.data_as(tpss._lib.C.POINTER(tpss._lib.C.c_double)),
                                                None))
    torch.cuda.synchronize()
    t_seq = time.perf_counter() - t0
    total = int(sum(b.n_dofs))
    shapes = sorted({(p["dim"], p["degree"], p["n_cells_fine"]) for p in problems})
    return {"workload": f"{len(problems)} independent 2D/3D SIPG Poisson problems, DGQ2..7, 8^d..64^d cells, "
                        f"{total} DoFs in total, CG + V-cycle to 1e-8 each, FP32 smoothers",
            "problems": len(problems), "total_dofs": total,
            "draw": {"seed": args.seed + 4, "max_dofs_total": cap_total, "max_dofs_problem": cap_problem,
                     "rejected_draws": rejected, "distinct_shapes": len(shapes),
                     "largest": max(shapes, key=lambda s: (s[2] * (s[1] + 1)) ** s[0])},
            "batch_seconds": t_batch, "sequential_seconds": t_seq,
            "dofs_solved_per_s": total / t_batch, "batch_speedup": t_seq / t_batch,
            "iterations_mean": float(np.mean(its)), "iterations_max": int(np.max(its)),
            "setup_seconds": setup}


def level_kernels(args):
    """Level operator (FP64 and FP32 arithmetic) and DG prolongation / restriction from the
    half-size level, on random vectors of the --cells level: milliseconds per application
    (CUDA events, warmed up), one JSON line."""
    import torch
    import tpss_gb300 as tpss
    dim, k, n = args.dim, args.degree, args.cells
    nd = (k + 1) ** dim
    sh = tpss.SubdomainHandler(tpss.SubdomainHandler.AdditionalData(dim=dim, degree=k, n_cells=(n,) * dim,
                                                                     patch_variant=1))
    op = tpss.LaplaceOperator(sh, 1.0)
    g = torch.Generator(device="cuda").manual_seed(args.seed)
    x = torch.rand(sh.n_dofs(), dtype=torch.float64, device="cuda", generator=g) * 2 - 1
    y = torch.empty_like(x)
    ncc = (n // 2,) * dim
    coarse = torch.rand((n // 2) ** dim * nd, dtype=torch.float64, device="cuda", generator=g) * 2 - 1
    fns = {"operator_fp64": lambda: op.vmult(y, x), "operator_fp32": lambda: op.vmult_fp32(y, x),
           "prolongate_add": lambda: tpss.prolongate_add(dim, k, ncc, x, coarse),
           "restrict_add": lambda: tpss.restrict_add(dim, k, ncc, coarse, x)}
    out = {"workload": f"{dim}D SIPG DGQ{k} {n}^{dim} cells, {sh.n_dofs()} DoFs; transfers from {n // 2}^{dim}"}
    for name, fn in fns.items():
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        out[name + "_ms"] = e0.elapsed_time(e1) / args.steps
    print(json.dumps(out))


def precision_sweep(args):
    """Where the FP32 smoothers' extra CG iterations come from: the solve of solve_times (one root
    cell, dense coarse solve, graphs) with FP32 smoothers everywhere, FP64 everywhere, and FP32
    except one level l (l = 1 .. L) that computes in FP64."""
    import numpy as np
    import torch
    import tpss_gb300 as tpss
    n, k, dim = args.cells, args.degree, args.dim
    N = n ** dim * (k + 1) ** dim
    f = torch.tensor(philox_src(N, args.seed), dtype=torch.float64, device="cuda")
    nl = n.bit_length()  # levels 0 .. L with 1, 2, .., n cells per direction
    cases = [("all_fp32", tpss.Precision.fp32, 0), ("all_fp64", tpss.Precision.fp64, 0)]
    cases += [(f"fp64_level_{l}", tpss.Precision.fp32, 1 << l) for l in range(1, nl)]
    out = {"workload": f"CG + V-cycle, 3D SIPG DGQ{k} {n}^3, f ~ U[-1,1] seed {args.seed}, damping "
                       f"{args.omega}, to 1e-8; level 0 is the coarse level (dense solve)"}
    for name, prec, mask in cases:
        mg = tpss.MultigridSolver(dim, k, 1, n, relaxation=args.omega, precision=prec, coarse_solver=1,
                                  use_graph=True, fp64_level_mask=mask)
        u = torch.zeros_like(f)
        mg.vmult(u, f)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        it, hist = mg.solve(u, f, rel_tol=1e-8)
        torch.cuda.synchronize()
        out[name] = {"iterations": it, "seconds": time.perf_counter() - t0,
                     "residual_1e-4_at": int(np.argmax(hist / hist[0] < 1e-4)),
                     "final_rel_residual": float(hist[-1] / hist[0])}
        del mg
    print(json.dumps(out))


def profile_case(args):
    """One small workload of a secondary kernel, run three times (--profile-case)."""
    import torch
    import tpss_gb300 as tpss
    from tpss_gb300.mesh import distorted_cube

    name = args.profile_case
    if name == "mapped":
        # FP64 operator of a distorted level: cell blocks + matrix-free face couplings
        n, k = 24, 3
        X = distorted_cube(3, [n] * 3, 7, 0.15)
        sh = tpss.SubdomainHandler(tpss.SubdomainHandler.AdditionalData(
            dim=3, degree=k, n_cells=(n,) * 3, vertex_coords=X))
        op = tpss.LaplaceOperator(sh)
        x = torch.rand(sh.n_dofs(), dtype=torch.float64, device="cuda")
        y = torch.empty_like(x)
        for _ in range(3):
            op.vmult(y, x)
    elif name == "perpatch":
        # streamed FP32 smoother on per-patch 1-D problems against the per-color kernel (src and
        # dst 90 MB each: together larger than L2)
        n, k = 56, 3
        X = distorted_cube(3, [n] * 3, 7, 0.15)
        sh = tpss.SubdomainHandler(tpss.SubdomainHandler.AdditionalData(
            dim=3, degree=k, n_cells=(n,) * 3, vertex_coords=X))
        x = torch.rand(sh.n_dofs(), dtype=torch.float64, device="cuda")
        y = torch.empty_like(x)
        ms = {}
        for label, kv in (("streamed_variant4", 2), ("per_color", 1)):
            p = tpss.SchwarzPreconditioner()
            p.initialize(sh, None, tpss.SchwarzPreconditioner.AdditionalData(
                relaxation=0.15, precision=tpss.Precision.fp32, kernel_variant=kv, stream_variant=4))
            for _ in range(3):
                p.vmult(y, x)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(10):
                p.vmult(y, x)
            e1.record()
            torch.cuda.synchronize()
            ms[label] = e0.elapsed_time(e1) / 10
            del p
        print(json.dumps({"profile_case": name, "n_dofs": sh.n_dofs(), "ms_per_vmult": ms}))
    elif name == "k5":
        # degree-5 streamed smoother (4 x 2 vertex columns) against the per-color kernel (src and
        # dst 110 MB each: together larger than L2)
        sh = tpss.SubdomainHandler(tpss.SubdomainHandler.AdditionalData(dim=3, degree=5, n_cells=(40,) * 3))
        x = torch.rand(sh.n_dofs(), dtype=torch.float64, device="cuda")
        y = torch.empty_like(x)
        ms = {}
        for label, kv in (("streamed_variant2", 2), ("per_color", 1)):
            p = tpss.SchwarzPreconditioner()
            p.initialize(sh, None, tpss.SchwarzPreconditioner.AdditionalData(
                relaxation=0.15, precision=tpss.Precision.fp32, kernel_variant=kv, stream_variant=2))
            for _ in range(3):
                p.vmult(y, x)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(10):
                p.vmult(y, x)
            e1.record()
            torch.cuda.synchronize()
            ms[label] = e0.elapsed_time(e1) / 10
            del p
        print(json.dumps({"profile_case": name, "n_dofs": sh.n_dofs(), "ms_per_vmult": ms}))
    elif name in ("cg2d", "cg2d_eager"):
        # small-problem latency: every kernel of a 65,536-DoF solve (20 iterations)
        mg = tpss.MultigridSolver(2, 3, 2, 64, relaxation=0.25, precision=tpss.Precision.fp64,
                                  coarse_solver=1, use_graph=name == "cg2d")
        f = torch.rand(mg.n_dofs(), dtype=torch.float64, device="cuda") * 2 - 1
        u = torch.zeros_like(f)
        mg.solve(u, f, rel_tol=1e-8)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        it, _ = mg.solve(u, f, rel_tol=1e-8)
        torch.cuda.synchronize()
        print(json.dumps({"profile_case": name, "iterations": it, "seconds": time.perf_counter() - t0}))
    elif name == "cg3dk5_eager":
        mg = tpss.MultigridSolver(3, 5, 1, 32, precision=tpss.Precision.fp32, coarse_solver=1, use_graph=False,
                                  autotune=True)
        f = torch.rand(mg.n_dofs(), dtype=torch.float64, device="cuda") * 2 - 1
        u = torch.zeros_like(f)
        t0 = time.perf_counter()
        it, _ = mg.solve(u, f, rel_tol=1e-8)
        torch.cuda.synchronize()
        print(json.dumps({"profile_case": name, "iterations": it, "seconds": time.perf_counter() - t0}))
    elif name == "c0ip":
        P = tpss.C0IPBiharmonic(3, 2, 512, local_solver=tpss.LocalSolver.fd, precision=tpss.Precision.fp32)
        x = torch.rand(P.n_dofs(), dtype=torch.float64, device="cuda")
        y = torch.empty_like(x)
        for _ in range(3):
            P.vmult(y, x)
            P.smooth(y, x)
    elif name == "mlp":
        m = tpss.MLP(87, 108, 64, 3, seed=1)
        x = torch.rand(119164, 87, device="cuda")
        t = torch.rand(119164, 108, device="cuda")
        m.train(x, t, epochs=1, batch=256)
    elif name == "host":
        sh = tpss.SubdomainHandler(tpss.SubdomainHandler.AdditionalData(dim=3, degree=4, n_cells=(64,) * 3))
        p = tpss.SchwarzPreconditioner()
        p.initialize(sh, None, tpss.SchwarzPreconditioner.AdditionalData(relaxation=0.15,
                                                                         precision=tpss.Precision.fp32))
        N = sh.n_dofs()
        h_src = torch.rand(N, dtype=torch.float64).pin_memory()
        h_dst = torch.empty(N, dtype=torch.float64).pin_memory()
        for _ in range(3):
            p.vmult_host(h_dst, h_src)
    torch.cuda.synchronize()
    print(json.dumps({"profile_case": name, "done": True}))


def main():
    args = parse()
    if args.steps < 1 or args.warmup < 3:
        raise SystemExit("need --steps >= 1 and --warmup >= 3")
    if args.profile_case:
        profile_case(args)
    elif args.precision_sweep:
        precision_sweep(args)
    elif args.level_kernels:
        level_kernels(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
