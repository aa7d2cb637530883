#!/usr/bin/env python
"""Benchmark of the BD step for the mesoscale chromatin fiber on GB300.

One "step" is one full predictor-corrector BD step (RPY tensor, Cholesky,
noise displacement, two force passes, two moves) of the 50-nucleosome fiber
with 44-bp linkers and a linker histone on every nucleosome (3N = 11,700),
with seeded MT19937 noise.  Inputs are resident in HBM for `value`; `e2e`
runs the same steps through the reference-facing call (host noise in, host
copies of the state out, as main_cuda does).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--config 0..4] [--precision fp64|mixed]

Multi-GPU: replicas only (independent fibers, one per rank, no collective in
the step); rank 0 prints the max-over-ranks time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "BD steps/s vs plain FP64 on 1 GB300 at <=1e-6 rel. error; replica-steps/s"
# dram__bytes_read.sum + dram__bytes_write.sum / algorithmic bytes of one
# k_chol_step launch under ncu (the fourth of a factorisation: panel 3 beside
# the K = 384 bulk update by panels 0-2, 3N = 11,700: 1,015.5 MB of DRAM
# traffic for 1,024.6 MB algorithmic)
NCU_TRAFFIC_PER_ALG_BYTE = 1015.5 / 1024.6
# largest 3N for which the GPU line's CPU baseline times complete oracle steps
CPU_STEP_MAX_M = 20000


def peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0, "fallback": True}


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu, self.rows, self.proc = gpu, [], None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self) -> dict:
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        sm = [float(r[1]) for r in self.rows if len(r) > 8 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 8 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows if len(r) > 8 for k in range(4) if r[5 + k] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(sm)}


def max_over_ranks(x: float) -> float:
    """Max of a per-rank scalar over the process group (identity without one)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_rate(ms_per_step_max: float, world: int) -> float:
    """Whole-job replica-steps/s: every rank advances its own fiber one step."""
    return world * 1000.0 / ms_per_step_max


def fp64_peak_tflops() -> float:
    """cuBLAS DGEMM rate on this GPU (8192^3, best of 3): the FP64 roofline
    denominator (MEASURED_PEAKS.json carries HBM and BF16 figures only)."""
    import torch
    n = 8192
    a = torch.randn(n, n, device="cuda", dtype=torch.float64)
    b = torch.randn(n, n, device="cuda", dtype=torch.float64)
    a @ b
    torch.cuda.synchronize()
    best = float("inf")
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        a @ b
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1) * 1e-3)
    del a, b
    torch.cuda.empty_cache()
    return 2.0 * n ** 3 / best / 1e12


def fp64_comparison(fib, rr_d, p_d, host, args, local, stream, krylov=False) -> dict:
    """Plain FP64 step (CUDA graph, same fiber, same noise) timed like the
    headline, and the relative displacement error of one mixed step against
    one FP64 step from the same state: max |dr_mixed - dr_fp64| / max |dr_fp64|
    over r, r_t and r_lh.  With the Krylov noise both sides use it (FP64:
    relative change 1e-10)."""
    import torch
    from brownian_dynamics_cuda_gb300 import NOISE_KRYLOV, PREC_FP64, PREC_MIXED, Context

    def mode(c, tol):
        if krylov:
            c.set_noise_mode(NOISE_KRYLOV, tol, 128)
        return c
    steps = max(2, min(args.steps, 5))
    c64 = mode(Context(fib, precision=PREC_FP64, use_graph=True, device=local, stream=stream.cuda_stream), 1e-10)
    with torch.cuda.stream(stream):
        for i in range(args.warmup):
            c64.step_device(rr_d[i].data_ptr(), p_d[i].data_ptr())
        stream.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for i in range(steps):
            c64.step_device(rr_d[args.warmup + i % args.steps].data_ptr(), p_d[args.warmup + i % args.steps].data_ptr())
        e1.record(stream)
        stream.synchronize()
    ms64 = e0.elapsed_time(e1) / steps
    c64.close()
    a = mode(Context(fib, precision=PREC_FP64, device=local), 1e-10)
    b = mode(Context(fib, precision=PREC_MIXED, device=local), args.krylov_tol)
    rr, p = host[0]
    a.step(rr, p)
    b.step(rr, p)
    num = den = 0.0
    for k in ("r", "r_t", "r_lh"):
        if fib.state[k].size == 0:
            continue
        d64 = a.get(k) - fib.state[k]
        dm = b.get(k) - fib.state[k]
        num = max(num, float(np.abs(dm - d64).max()))
        den = max(den, float(np.abs(d64).max()))
    a.close()
    b.close()
    return {"fp64_steps_per_s": 1000.0 / ms64, "fp64_ms_per_step": ms64, "fp64_steps_timed": steps,
            "rel_displacement_err": num / den, "tolerance": 1e-6}


def library_bar(fib, local, dpotrf: bool) -> dict:
    """The library bar for the factorisation phase: cuSOLVER's potrf through
    torch.linalg.cholesky (cusolverDnXpotrf) on this fiber's own FP64 RPY
    tensor (3N <= 20,000; above that a synthetic SPD matrix of the same size,
    since the timing does not depend on the values), in FP32 (the accuracy
    class of the mixed factor) and FP64 (what func_cuda.cu:3526-3529 calls).
    Measurement only: the product never calls it."""
    import torch
    from brownian_dynamics_cuda_gb300 import PREC_FP64, Context
    torch.backends.cuda.preferred_linalg_library("cusolver")
    m = fib.m
    if m <= 20000:
        c = Context(fib, precision=PREC_FP64, device=local)
        D = torch.tensor(c.diffusion_tensor(), device="cuda")
        c.close()
        src = "the fiber's FP64 RPY tensor"
    else:
        g = torch.Generator(device="cuda").manual_seed(0)
        X = torch.randn(m, 64, device="cuda", dtype=torch.float64, generator=g)
        D = X @ X.T / 64 + 2.0 * torch.eye(m, device="cuda", dtype=torch.float64)
        del X
        src = "synthetic SPD matrix of the same size"
    out = {"input": src, "3N": m}
    legs = [("cusolver_spotrf_ms", torch.float32, 5)] + ([("cusolver_dpotrf_ms", torch.float64, 2)] if dpotrf else [])
    for key, dt, reps in legs:
        A = D.to(dt)
        torch.linalg.cholesky(A)
        torch.cuda.synchronize()
        best = float("inf")
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            Lc = torch.linalg.cholesky(A)
            e1.record()
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1))
            del Lc
        out[key] = best
        del A
    del D
    torch.cuda.empty_cache()
    return out


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def make_fiber(cfg: int, seed: int):
    from brownian_dynamics_cuda_gb300.fiber_gen import config, make_fiber as mk
    d = tempfile.mkdtemp(prefix="bdfiber_")
    spec = config(cfg, seed=seed)
    return mk(spec, d), spec


def oracle_fiber(cfg: int, seed: int):
    """The workload's input files read by the oracle's restatement of the
    reference readers (oracle/ref_loader.py): the CPU legs load no product
    library."""
    from brownian_dynamics_cuda_gb300.fiber_gen import config, write_fiber
    from oracle import ref_loader
    d = tempfile.mkdtemp(prefix="bdfiber_ref_")
    spec = config(cfg, seed=seed)
    return ref_loader.load(d, **write_fiber(spec, d)), spec


def cpu_steps(fib, threads: int, warmup: int, steps: int, seed: int = 1000) -> dict:
    """Complete BD steps of the CPU oracle (oracle/bd_oracle.cpp, the
    reference's func.cpp step restated): RPY assembly, the reference's full
    Cholesky, rd = s2dt L p, both force passes and both moves, with the
    reference's MT19937 noise.  The assembly, the Cholesky (bit for bit the
    reference's row loop, column-blocked over `threads`) and rd run on
    `threads` host threads; the force passes on one, as in the reference."""
    from oracle.pyoracle import Oracle, OracleNoise, set_threads
    set_threads(threads)
    o = Oracle(fib)
    gen = OracleNoise(seed)
    times = []
    for i in range(warmup + steps):
        rr, p = gen.step(i, fib.arrays["r_var"], fib.m)
        t = time.perf_counter()
        o.step(rr, p)
        if i >= warmup:
            times.append(time.perf_counter() - t)
    total = float(np.sum(times))
    return {"steps_timed": steps, "total_s": total, "step_s": total / max(steps, 1),
            "sample": f"{steps} complete oracle steps of the full fiber (3N = {fib.m}) after {warmup} untimed: "
                      f"RPY assembly, the reference Cholesky (func.cpp:806-836; same factor bit for bit, "
                      f"column-blocked on {threads} threads), rd, two force passes (1 thread) and two moves; "
                      f"nothing extrapolated"}


def run_reference(args):
    """The reference's CPU path on this host's cores: complete steps of the
    oracle port (oracle/_ref is not built on the GPU host), the fiber read by
    the oracle's own restatement of the reference readers."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    fib, spec = oracle_fiber(args.config, 1)
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    s = cpu_steps(fib, threads, args.warmup, args.steps)
    wall = time.perf_counter() - t0
    v = 1.0 / s["step_s"]
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "steps/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": s["step_s"] * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded fiber generator)",
            "config": {"workload": spec.name, "n_D": fib.n_D, "3N": fib.m, "precision": "fp64",
                       "timed_s": s["total_s"], "wall_s": wall},
            "cpu_baseline": {"value": v, "unit": "steps/s", "cores": threads, "kind": "port", "sample": s["sample"]},
            "e2e": {"value": v, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch
    from brownian_dynamics_cuda_gb300 import NOISE_KRYLOV, PREC_FP64, PREC_MIXED, Context, Noise
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    prec = PREC_MIXED if args.precision == "mixed" else PREC_FP64
    fib, spec = make_fiber(args.config, 1 + rank)
    stream = torch.cuda.Stream()
    freq = args.frequency_rp
    ctx = Context(fib, precision=prec, use_graph=True, frequency_RP=freq, device=local, stream=stream.cuda_stream)
    krylov = args.noise == "krylov"

    def noise_mode(c, tol=None):
        if krylov:
            c.set_noise_mode(NOISE_KRYLOV, tol or args.krylov_tol, 128)
        return c
    noise_mode(ctx)
    n3, m = 3 * fib.sizes["n"], fib.m
    nsteps = args.warmup + args.steps
    noise = Noise(1000 + rank)
    host = [noise.step(i, fib.arrays["r_var"], m) for i in range(nsteps)]
    rr_d = torch.tensor(np.stack([h[0] for h in host]), device="cuda", dtype=torch.float64)
    p_d = torch.tensor(np.stack([h[1] for h in host]), device="cuda", dtype=torch.float64)

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    with torch.cuda.stream(stream):
        for i in range(args.warmup):
            ctx.step_device(rr_d[i].data_ptr(), p_d[i].data_ptr())
        stream.synchronize()
        # per-phase times of one eager step (events on the context's stream)
        ctx.phase_times()
        ph_ctx = noise_mode(Context(fib, precision=prec, use_graph=False, device=local, stream=stream.cuda_stream))
        ph_ctx.phase_times()
        ph_ctx.step_device(rr_d[0].data_ptr(), p_d[0].data_ptr())
        phases = ph_ctx.phase_times()
        ph_ctx_stats = ph_ctx.krylov_stats() if krylov else None
        kt = ph_ctx.kernel_time()
        kbytes = ph_ctx.kernel_bytes()
        ph_ctx.close()
        barrier()
        torch.cuda.synchronize()
        clk = ClockSampler(local)
        clk.start()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for i in range(args.warmup, nsteps):
            ctx.step_device(rr_d[i].data_ptr(), p_d[i].data_ptr())
        e1.record(stream)
        stream.synchronize()
        torch.cuda.synchronize()
        barrier()
        clocks = clk.stop()
    ms = max_over_ranks(e0.elapsed_time(e1) / args.steps)
    value = replica_rate(ms, world)
    launches = ctx.launch_count() * args.steps
    # e2e: reference-facing call with host buffers (noise H2D, r_lh D2H every
    # step, full state D2H on sampling steps every 100 steps)
    e2e_ctx = noise_mode(Context(fib, precision=prec, use_graph=True, frequency_RP=freq, device=local,
                                 stream=stream.cuda_stream))
    pin = lambda a: torch.from_numpy(a).pin_memory().numpy()  # noqa: E731
    rr_h = [pin(h[0]) for h in host]
    p_h = [pin(h[1]) for h in host]
    out = {k: pin(np.zeros(v)) for k, v in (("r", n3), ("a", n3), ("b", n3), ("c", n3),
                                              ("r_t", max(3 * fib.sizes["n_tail"], 1)),
                                              ("r_lh", max(3 * fib.sizes["n_LH"], 1)))}
    freq = 100
    for i in range(args.warmup):
        e2e_ctx.step_reference(i, 1 << 30, freq, rr_h[i], p_h[i], out)
    barrier()
    t0 = time.perf_counter()
    for i in range(args.warmup, nsteps):
        e2e_ctx.step_reference(i, 1 << 30, freq, rr_h[i], p_h[i], out)
    torch.cuda.synchronize()
    barrier()
    e2e_s = max_over_ranks((time.perf_counter() - t0) / args.steps)
    h2d = (n3 + m) * 8
    d2h = 8 + 3 * fib.sizes["n_LH"] * 8 + (4 * n3 + 3 * fib.sizes["n_tail"]) * 8 / freq
    # roofline of the dominant kernel
    pk = peaks()
    chol_ms = float(phases[1])
    chol_flop = m ** 3 / 3.0
    if krylov:
        it, ch = ph_ctx_stats
        byt = it * 8.0 * m * (m + 1) / 2  # the lower triangle of D read once per iteration (8 B per entry)
        rd_ms = float(phases[2])
        achieved = byt / (rd_ms * 1e-3) / 1e9
        roof = {"bound": "hbm", "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
                "frac": achieved / pk["hbm_gbs"], "traffic": None,
                "kernel": ("k_rpy_mv (matrix-free FP32 RPY products, no tensor read: bytes below are those the "
                           "stored tensor would cost)" if prec == PREC_MIXED else
                           "k_symv_tiles + k_symv_sum (products with the stored FP64 tensor)") +
                          " of the Lanczos noise, %d iterations, last relative change %.1e" % (it, ch),
                "algorithmic_bytes_per_step": byt, "rd_phase_ms": rd_ms,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)"}
    elif prec == PREC_FP64:
        fp64_peak = fp64_peak_tflops()
        roof = {"bound": "fp64", "achieved": chol_flop / (chol_ms * 1e-3) / 1e12, "peak": fp64_peak,
                "unit": "TFLOP/s", "frac": None, "traffic": None,
                "kernel": "FP64 Cholesky phase (k_potrf_diag + k_trsm_panel + k_syrk_update), (3N)^3/3 flop",
                "peak_source": "cuBLAS DGEMM 8192^3 measured in this run (no FP64 entry in MEASURED_PEAKS.json)"}
        roof["frac"] = roof["achieved"] / roof["peak"]
    else:
        ms_k, nk, flop_k = kt
        byt = kbytes
        achieved = byt / (ms_k * 1e-3) / 1e9 if ms_k > 0 else None
        roof = {"bound": "hbm", "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
                "frac": achieved / pk["hbm_gbs"] if achieved else None,
                "traffic": byt * NCU_TRAFFIC_PER_ALG_BYTE,
                "traffic_source": "DRAM read+write per algorithmic byte of one ncu capture "
                                  "of k_chol_step at 3N = 11,700, times this step's algorithmic bytes",
                "kernel": "k_chol_step (every launch of the mixed factorisation: next panel in its own CTAs beside "
                          "tcgen05 column and bulk trailing updates of one or two panels, double-float tile "
                          "read-modify-write), %d launches/step, avg %.3f ms" % (nk, ms_k / max(nk, 1)),
                "algorithmic_bytes_per_step": byt,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)",
                "tensor_tflops_issued": flop_k / (ms_k * 1e-3) / 1e12 if ms_k > 0 else None,
                "tensor_frac_of_bf16_sustained": (flop_k / (ms_k * 1e-3) / 1e12 /
                                                  pk.get("bf16_tflops_sustained", pk["bf16_tflops"]))
                if ms_k > 0 else None,
                "chol_phase_ms": chol_ms, "chol_fp32_equiv_tflops": chol_flop / (chol_ms * 1e-3) / 1e12}
    # the plain FP64 step on the same fiber and noise: the metric's reference
    # point, and the mixed step's displacement error against it
    vs64 = None
    if prec == PREC_MIXED and not args.no_fp64:
        vs64 = fp64_comparison(fib, rr_d, p_d, host, args, local, stream, krylov)
        if world > 1:
            vs64["fp64_steps_per_s"] = replica_rate(max_over_ranks(1000.0 / vs64["fp64_steps_per_s"]), world)
        vs64["speedup_vs_fp64"] = value / vs64["fp64_steps_per_s"]
    lib = None
    if rank == 0 and not args.no_library_bar:
        lib = library_bar(fib, local, dpotrf=fib.m <= 20000)
        lib["ours_chol_phase_ms"] = float(phases[1])
        if "cusolver_spotrf_ms" in lib:
            lib["spotrf_over_ours"] = lib["cusolver_spotrf_ms"] / float(phases[1])
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        if fib.m <= CPU_STEP_MAX_M:
            ofib, _ = oracle_fiber(args.config, 1)
            threads = os.cpu_count() or 1
            s = cpu_steps(ofib, threads, 0, 2)
            cpu = {"value": 1.0 / s["step_s"], "unit": "steps/s", "cores": threads, "kind": "port",
                   "sample": s["sample"]}
        else:
            cpu = {"value": None, "unit": "steps/s", "cores": None, "kind": "port",
                   "sample": f"not run: one complete oracle step at 3N = {fib.m} takes minutes (O((3N)^3) Cholesky)"}
    if rank == 0:
        names = ["rpy", "chol", "rd", "forces1", "move1", "frames", "forces2", "move2+frames", "total"]
        line = {"metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64" if prec == PREC_FP64 else "bf16x3+f64",
                "data": "synthetic (seeded fiber generator, reference file formats)",
                "config": {"workload": spec.name, "n_D": fib.n_D, "3N": m, "precision": args.precision,
                           "frequency_RP": args.frequency_rp, "noise": args.noise,
                           "parallelism": f"replicas x{world}", "l2": "inputs larger than L2 (D is %.2f GB)" %
                                                                         (m * m * 8 / 1e9)},
                "e2e": {"value": world / e2e_s, "unit": "steps/s", "h2d_bytes_per_step": h2d,
                        "d2h_bytes_per_step": d2h},
                "gpu_launches": launches, "clocks": clocks, "roofline": roof, "vs_fp64": vs64,
                "phases_ms": dict(zip(names, [round(float(x), 4) for x in phases])),
                "library_bar": lib, "cpu_baseline": cpu}
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def mixed_schedule_bytes(m: int, kT: int = 128, triple_min: int = 40, pair_min: int = 24) -> float:
    """Algorithmic HBM bytes of one mixed factorisation of a 3N = m tensor: the
    schedule of bdk::potrf_mixed (one launch per panel; three panels per bulk
    pass while 40 tile rows remain, two while 24 do), 16 B (double-float read +
    write) per element of the panel's column and of every trailing tile a bulk
    pass updates.  Equals the library's own count (bd_kernel_bytes; 12.70 GB at
    3N = 11,700)."""
    nt = -(-m // kT)
    kb = lambda k: m - k * kT if m - k * kT < kT else kT  # noqa: E731

    def elems(j0, j1):
        e = 0.0
        for J in range(j0, min(j1, nt)):
            cols = kb(J)
            e += cols * (m - J * kT) - cols * (cols - 1) / 2
        return e

    total = 0.0

    def launch(pn, jobs):
        nonlocal total
        total += 16.0 * (m - pn * kT) * kb(pn)
        for mode, jlo in jobs:
            n = nt - jlo
            if n > 0:
                total += 16.0 * elems(jlo, jlo + 1 if mode == "col" else nt)

    launch(0, [])
    k = 0
    while k + 1 < nt:
        if nt - (k + 4) >= triple_min:
            launch(k + 1, [("col", k + 2)])
            launch(k + 2, [("col", k + 3)])
            launch(k + 3, [("tri", k + 4)])
            k += 3
        elif nt - (k + 3) >= pair_min:
            launch(k + 1, [("col", k + 2)])
            launch(k + 2, [("tri", k + 3)])
            k += 2
        else:
            launch(k + 1, [("tri", k + 2)])
            k += 1
    return total


def batch_fp64_comparison(fibers, host, d_rr, d_p, local, stream, passes_list=(3, 1)) -> dict:
    """The plain FP64 GPU step on the same replicas and noise: one FP64 batch
    step from the start states (its displacements kept), two timed FP64 batch
    steps (CUDA graph, CUDA events); then, for each mixed schedule (at most
    `passes` panels per trailing pass; 3 is the default), one mixed batch step
    from the same start states — every replica's relative displacement error
    max |dr_mixed - dr_fp64| / max |dr_fp64| over r, r_t, r_lh — and two timed
    mixed steps of that schedule."""
    import torch
    from brownian_dynamics_cuda_gb300 import PREC_FP64, PREC_MIXED, Batch
    R = len(fibers)
    rr0, p0 = [h[0][0] for h in host], [h[0][1] for h in host]
    keys = ("r", "r_t", "r_lh")

    def timed(b, steps=2):
        with torch.cuda.stream(stream):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for s in range(1, 1 + steps):
                b.step_device([x[s].data_ptr() for x in d_rr], [x[s].data_ptr() for x in d_p])
            e1.record(stream)
            stream.synchronize()
        return e0.elapsed_time(e1) / steps

    b64 = Batch(fibers, precision=PREC_FP64, use_graph=True, device=local, stream=stream.cuda_stream)
    b64.step(rr0, p0)
    ref = [{k: c.get(k) - f.state[k] for k in keys if f.state[k].size} for c, f in zip(b64.contexts, fibers)]
    ms64 = timed(b64)
    b64.close()
    out = {"fp64_replica_steps_per_s": R * 1000.0 / ms64, "fp64_ms_per_step": ms64, "fp64_steps_timed": 2,
           "tolerance": 1e-6}
    for passes in passes_list:
        bm = Batch(fibers, precision=PREC_MIXED, use_graph=True, device=local, stream=stream.cuda_stream)
        bm.set_mixed_passes(passes)
        bm.step(rr0, p0)
        errs = []
        for c, f, d64 in zip(bm.contexts, fibers, ref):
            num = max(float(np.abs((c.get(k) - f.state[k]) - d64[k]).max()) for k in d64)
            den = max(float(np.abs(d64[k]).max()) for k in d64)
            errs.append(num / den)
        ms = timed(bm)
        bm.close()
        leg = {"replica_steps_per_s": R * 1000.0 / ms, "ms_per_step": ms, "rel_displacement_err_max": max(errs),
               "rel_displacement_err_median": float(np.median(errs)),
               "replicas_over_tolerance": int(sum(e > 1e-6 for e in errs))}
        out[f"mixed_passes{passes}"] = leg
        if passes == 3:
            out["rel_displacement_err_max"] = leg["rel_displacement_err_max"]
            out["rel_displacement_err_median"] = leg["rel_displacement_err_median"]
    return out


def batch_cpu_sample(dirs, budget_s: float = 15.0) -> dict:
    """Complete oracle steps of the replicas in order (one each, the fibers
    read by the oracle's reader restatement) until `budget_s` of CPU time;
    replica-steps/s over the replicas done."""
    from oracle import ref_loader
    from oracle.pyoracle import Oracle, OracleNoise, set_threads
    threads = os.cpu_count() or 1
    set_threads(threads)
    done, total, ms = 0, 0.0, []
    for i, (d, files) in enumerate(dirs):
        fib = ref_loader.load(d, **files)
        o = Oracle(fib)
        rr, p = OracleNoise(1000 + i).step(0, fib.arrays["r_var"], fib.m)
        t = time.perf_counter()
        o.step(rr, p)
        total += time.perf_counter() - t
        done += 1
        ms.append(fib.m)
        if total >= budget_s:
            break
    return {"value": done / total, "unit": "replica-steps/s", "cores": threads, "kind": "port",
            "sample": f"one complete oracle step of each of the first {done} replicas (3N {min(ms)}-{max(ms)}), "
                      f"{total:.1f} s; RPY, the reference Cholesky (bit for bit, column-blocked on {threads} "
                      f"threads), rd, two force passes, two moves"}


def run_batch(args):
    """Config 2: replicas of uneven size and salt (nucleosomes 12-48, linkers
    20-60 bp, 50/100/150 mM) advanced together through bd_batch_* (one CUDA
    graph per batch step); metric replica-steps/s.  Beside it: the batched
    factorisation's roofline (phase times of one eager step), the plain FP64
    batch on the same replicas (rate and every replica's displacement error),
    and complete CPU oracle steps of a bounded sample of the replicas."""
    import torch
    from brownian_dynamics_cuda_gb300 import PREC_FP64, PREC_MIXED, Batch, Fiber, Noise
    from brownian_dynamics_cuda_gb300.fiber_gen import config, write_fiber
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    prec = PREC_MIXED if args.precision == "mixed" else PREC_FP64
    dirs = []
    for i in range(args.replicas):
        d = tempfile.mkdtemp(prefix="bdrep_")
        dirs.append((d, write_fiber(config(2, seed=1 + rank, replica=i), d)))
    fibers = [Fiber.load(d, **files) for d, files in dirs]
    stream = torch.cuda.Stream()
    b = Batch(fibers, precision=prec, use_graph=True, device=local, stream=stream.cuda_stream)
    nsteps = max(args.warmup + args.steps, 3)
    gens = [Noise(1000 + i) for i in range(len(fibers))]
    host = [[g.step(s, f.arrays["r_var"], f.m) for s in range(nsteps)] for g, f in zip(gens, fibers)]
    d_rr = [[torch.tensor(h[s][0], device="cuda") for s in range(nsteps)] for h in host]
    d_p = [[torch.tensor(h[s][1], device="cuda") for s in range(nsteps)] for h in host]
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        for s in range(args.warmup):
            b.step_device([x[s].data_ptr() for x in d_rr], [x[s].data_ptr() for x in d_p])
        stream.synchronize()
        clk = ClockSampler(local)
        clk.start()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for s in range(args.warmup, args.warmup + args.steps):
            b.step_device([x[s].data_ptr() for x in d_rr], [x[s].data_ptr() for x in d_p])
        e1.record(stream)
        stream.synchronize()
        clocks = clk.stop()
    ms = max_over_ranks(e0.elapsed_time(e1) / args.steps)
    value = world * len(fibers) * 1000.0 / ms
    launches = b.launch_count() * args.steps
    # e2e: host noise per replica per step through bd_batch_step
    t0 = time.perf_counter()
    for s in range(args.warmup, args.warmup + args.steps):
        b.step([h[s][0] for h in host], [h[s][1] for h in host])
    e2e_s = max_over_ranks((time.perf_counter() - t0) / args.steps)
    # the run with every replica's noise drawn on the device (bd_batch_run_device:
    # one noise launch per step for all replicas, one host wait at the end)
    b.run_device(1, 4242)  # creates the generators
    t0 = time.perf_counter()
    b.run_device(args.steps, 4242)
    dev_run_s = max_over_ranks((time.perf_counter() - t0) / args.steps)
    h2d = sum((3 * f.sizes["n"] + f.m) * 8 for f in fibers)
    sizes = [f.m for f in fibers]
    # phases of one eager step (timing on: no graph), for the roofline
    b.phase_times()
    b.step([h[0][0] for h in host], [h[0][1] for h in host])
    ph = b.phase_times()
    roof = None
    if prec == PREC_MIXED and ph[1] > 0:
        pk = peaks()
        byt = sum(mixed_schedule_bytes(m) for m in sizes)
        achieved = byt / (ph[1] * 1e-3) / 1e9
        roof = {"bound": "hbm", "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
                "frac": achieved / pk["hbm_gbs"], "traffic": byt * NCU_TRAFFIC_PER_ALG_BYTE,
                "traffic_source": "DRAM read+write per algorithmic byte of one ncu capture of k_chol_step at "
                                  "3N = 11,700, times this batch's algorithmic bytes",
                "kernel": "k_chol_step_multi (every replica's mixed factorisation, launch i carrying step i of "
                          "every replica's schedule), phase time of one eager batch step",
                "algorithmic_bytes_per_step": byt, "factorisation_phase_ms": float(ph[1]),
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)"}
    b.close()
    vs64 = None
    if prec == PREC_MIXED and not args.no_fp64:
        vs64 = batch_fp64_comparison(fibers, host, d_rr, d_p, local, stream)
        vs64["speedup_vs_fp64"] = value / (world * vs64["fp64_replica_steps_per_s"])
    cpu = batch_cpu_sample(dirs) if rank == 0 and world == 1 and not args.no_cpu else None
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "replica-steps/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64" if prec == PREC_FP64 else "bf16x3+f64",
                "data": "synthetic (seeded fiber generator, reference file formats)",
                "config": {"workload": "cfg2_replicas", "replicas": len(fibers), "3N_min": min(sizes),
                           "3N_max": max(sizes), "3N_sum": sum(sizes), "precision": args.precision,
                           "parallelism": f"replicas x{world}", "l2": "inputs larger than L2"},
                "e2e": {"value": world * len(fibers) / e2e_s, "unit": "replica-steps/s", "h2d_bytes_per_step": h2d,
                        "d2h_bytes_per_step": 8 * len(fibers)},
                "device_noise_run": {"value": world * len(fibers) / dev_run_s, "unit": "replica-steps/s",
                                     "api": "bd_batch_run_device (host wall clock over the timed steps)"},
                "gpu_launches": launches, "clocks": clocks, "roofline": roof, "vs_fp64": vs64,
                "phases_ms": {"positions+tensors": float(ph[0]), "factorisation": float(ph[1]),
                              "forces+moves": float(ph[2])},
                "cpu_baseline": cpu}
        print(json.dumps(line), flush=True)


def run_adjoint(args):
    """--config 3, the 24-nucleosome fiber with 30-bp linkers and no linker
    histone: gradient of the 200-step rollout observable (mean over the
    final 50 states of the squared end-to-end distance plus the radius of
    gyration) with respect to the stretch, bend and twist moduli and the
    Debye length, by bd_adjoint (reverse mode, checkpoints every 20 steps,
    FP32-class forward on a mixed-precision context).  One "step" of this
    workload is one gradient evaluation (forward sweep + checkpointed
    reverse sweep); metric: gradient evaluations/s.  With --fd the FP64
    central-difference gradient (steps of 1e-4 relative) is computed too and
    the relative error reported."""
    import torch
    from brownian_dynamics_cuda_gb300 import PREC_FP64, PREC_MIXED, Context, Noise
    from brownian_dynamics_cuda_gb300.fiber_gen import config, make_fiber as mk
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    spec = config(3, seed=1 + rank)
    fib = mk(spec, tempfile.mkdtemp(prefix="bdadj_"))
    nsteps, window, ck = 200, 50, 20
    gen = Noise(1)
    rows = [gen.step(s, fib.arrays["r_var"], fib.m) for s in range(nsteps)]
    rr = np.array([r[0] for r in rows])
    p = np.array([r[1] for r in rows])
    ctx = Context(fib, precision=PREC_MIXED if args.precision == "mixed" else PREC_FP64, device=local)
    for _ in range(args.warmup):
        ctx.adjoint(rr, p, window, ck)
    torch.cuda.synchronize()
    clk = ClockSampler(local)
    clk.start()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        loss, grad = ctx.adjoint(rr, p, window, ck)
    dt = max_over_ranks((time.perf_counter() - t0) / args.steps)
    clocks = clk.stop()
    launches = ctx.adjoint_launches()
    t0 = time.perf_counter()
    ctx.rollout_loss(rr, p, window)
    fwd = time.perf_counter() - t0
    fd = None
    if args.fd and rank == 0:
        c64 = Context(fib, precision=PREC_FP64, device=local)
        sc = fib.scalars
        th = np.array([sc["h"], sc["g"], sc["s"], 1.0 / sc["debye"]])
        g = np.zeros(4)
        for k in range(4):
            d = 1e-4 * th[k]
            tp, tm = th.copy(), th.copy()
            tp[k] += d
            tm[k] -= d
            c64.set_moduli(*tp)
            lp = c64.rollout_loss(rr, p, window)
            c64.set_moduli(*tm)
            lm = c64.rollout_loss(rr, p, window)
            g[k] = (lp - lm) / (2 * d)
        fd = {"grad_fd64": g.tolist(), "rel_err": float(np.max(np.abs(grad - g)) / np.max(np.abs(g)))}
        c64.close()
    if rank == 0:
        h2d = (rr.size + p.size) * 8
        line = {"metric": "adjoint gradient evaluations/s (200-step rollout, 4 parameters)",
                "value": world / dt, "unit": "gradients/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": dt * 1000.0, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32 (adjoint pair sums, RPY, Cholesky backward) + f64 (angle terms)",
                "data": "synthetic (seeded fiber generator, reference file formats)",
                "config": {"workload": spec.name, "n_D": fib.n_D, "3N": fib.m, "rollout_steps": nsteps,
                           "window": window, "checkpoint_every": ck, "precision": args.precision,
                           "forward_rollout_ms": fwd * 1000.0, "l2": "inputs larger than L2 (D: 60 MB FP32 x4)"},
                "e2e": {"value": world / dt, "unit": "gradients/s", "h2d_bytes_per_step": h2d,
                        "d2h_bytes_per_step": 5 * 8},
                "gpu_launches": launches, "clocks": clocks, "roofline": None, "cpu_baseline": None,
                "loss": loss, "grad": grad.tolist(), "fd_check": fd}
        print(json.dumps(line), flush=True)
    ctx.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None, help="timed steps (default 5; 10 for config 4)")
    ap.add_argument("--warmup", type=int, default=None, help="warm-up steps (default 3; 10 for config 4)")
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--config", type=int, default=1)
    ap.add_argument("--precision", choices=["fp64", "mixed"], default="mixed")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--replicas", type=int, default=256, help="config 2: number of replicas")
    ap.add_argument("--frequency-rp", type=int, default=None,
                    help="rebuild and refactor D every k steps (default 1; 10 for config 4)")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 comparison leg of the mixed run")
    ap.add_argument("--no-library-bar", action="store_true", help="skip the cuSOLVER potrf timing leg")
    ap.add_argument("--noise", choices=["cholesky", "krylov"], default="cholesky",
                    help="noise displacement: the reference's L p, or D^{1/2} p by Lanczos (non-parity fast mode)")
    ap.add_argument("--krylov-tol", type=float, default=1e-6, help="Lanczos stopping tolerance (relative change)")
    ap.add_argument("--fd", action="store_true", help="with --config 3 (rollout gradient): also the FP64 central-difference gradient")
    args = ap.parse_args()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        sys.exit(f"bench.py --gpus {args.gpus}: launch one process per GPU, e.g. python -m torch.distributed.run "
                 f"--nnodes=1 --nproc-per-node {args.gpus} --master-addr 127.0.0.1 bench.py --gpus {args.gpus}")
    big = args.config == 4
    args.frequency_rp = args.frequency_rp or (10 if big else 1)
    args.steps = args.steps if args.steps is not None else (10 if big else 5)
    args.warmup = args.warmup if args.warmup is not None else (10 if big else 3)
    if args.impl == "reference":
        run_reference(args)
    elif args.config == 2:
        run_batch(args)
    elif args.config == 3:
        run_adjoint(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
