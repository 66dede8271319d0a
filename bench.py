"""Benchmark of the sketching hot path on GB300.

Headline workload (one "step" = one sketch): B = S A with S a 4096 x 2^20 uniform dense
operator (seed RNGState(3)) generated inside the kernel, A a 2^20 x 1024 FP32 row-major matrix
with singular values decaying geometrically from 1 to 1e-6 (random orthogonal factors from a
seeded QR), d = 4096.  Reported as TFLOP/s of 2*d*m*n, for the tensor-core path (S and A
rounded to BF16, FP32 accumulation) when the library provides it, next to the plain FP32
path on the same GPU.  Secondary: the 1024 x 2^20 SASO (8 nonzeros per column) sketch of a
2^20 x 256 N(0,1) matrix, reported in GB/s against the measured HBM copy bandwidth.

python bench.py [--gpus 1] [--steps K] [--warmup W] [--impl ours|reference]
The GPU path is measured on one GPU only: the sketch needs no exchange between GPUs and the
benchmark runs no replicas, so ``--gpus N`` with N > 1 (or a torchrun launch with
WORLD_SIZE > 1) is refused with exit status 2.
The reference arm (``--impl reference``) runs on the host cores of rank 0 only.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "S·A sketch time and roofline fraction: BF16-TC fused vs FP32 plain, same GPU"
# DRAM bytes per launch of the BF16 tensor-core sketch at the headline size, from one ncu capture
# at m = 2^17 (344.7 MB read, 83.4 MB written) with the reads scaled by 8 to m = 2^20 (they
# grow with m; the partial-sum writes do not).
HEADLINE_TRAFFIC_BYTES = 8 * 344.7e6 + 83.4e6
D_SK, M_SK, N_SK = 4096, 1 << 20, 1024
SASO_D, SASO_M, SASO_N, SASO_K = 1024, 1 << 20, 256, 8


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return p["hbm_gbs"], p["bf16_tflops"], p.get("bf16_tflops_sustained"), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, 1900.0, 1700.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 50 ms while running."""

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4)
                          if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.rows)}


# ----------------------------------------------------------------------------- workload
def _cholesky_qr2(torch, G):
    """Orthonormal columns spanning G (tall, well conditioned): CholeskyQR2 (Fukaya, Nakatsukasa,
    Yanagisawa, Yamamoto 2014) -- Q = G R^-1 twice, with the small Gram matrix factored on the
    host in FP64 and the products on the GPU in FP32 (TF32 off)."""
    import numpy as np
    Q = G
    for _ in range(2):
        W = (Q.T @ Q).double().cpu().numpy()
        R = np.linalg.cholesky(W).T  # W = R^T R
        Q = Q @ torch.from_numpy(np.linalg.inv(R)).to(device=Q.device, dtype=Q.dtype)
    return Q


def make_precision_input(torch, device):
    """A = U diag(sigma) V^T, 2^20 x 1024 FP32 row-major, sigma_i = 10^(-6 i / 1023); U from
    CholeskyQR2 of a seeded 2^20 x 1024 Gaussian matrix (torch seed 0), V the Q factor of a
    seeded 1024 x 1024 Gaussian matrix (torch seed 1, Householder QR in FP64 on the host)."""
    import numpy as np
    torch.backends.cuda.matmul.allow_tf32 = False
    g0 = torch.Generator(device=device).manual_seed(0)
    g1 = torch.Generator(device=device).manual_seed(1)
    U = _cholesky_qr2(torch, torch.randn(M_SK, N_SK, generator=g0, device=device))
    Vh = torch.randn(N_SK, N_SK, generator=g1, device=device, dtype=torch.float64).cpu().numpy()
    V = torch.from_numpy(np.linalg.qr(Vh)[0]).to(device)
    sigma = torch.logspace(0, -6, N_SK, dtype=torch.float64, device=device)
    A = (U * sigma.float()) @ V.T.float()
    return A.contiguous(), U


def event_time(torch, fn, steps, warmup, stream):
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    start = torch.cuda.Event(enable_timing=True)
    stop = torch.cuda.Event(enable_timing=True)
    start.record(stream)
    for _ in range(steps):
        fn()
    stop.record(stream)
    torch.cuda.synchronize()
    return start.elapsed_time(stop) / steps


# ----------------------------------------------------------------------------- CPU baseline
def cpu_precision_sample(rows: int, A_host):
    """The reference's CPU path on a row block of the operator: the oracle's OpenMP port of
    fill_dense_unpacked (the 4096 x 2^20 uniform operator, rows [0, rows)) followed by an
    OpenBLAS SGEMM -- what the reference does (materialise the submatrix, blas::gemm)."""
    import ctypes as C

    import numpy as np

    from oracle.oracle import Oracle, State, find_cblas
    orc = Oracle()
    blas, sgemm, _ = find_cblas()
    t0 = time.perf_counter()
    Sblk, _ = orc.fill_dense_unpacked(0, 1, D_SK, M_SK, 1, 1, rows, M_SK, 0, 0,
                                      State.from_key(3))
    B = np.zeros((rows, N_SK), np.float32)
    if sgemm:
        fn = C.CFUNCTYPE(None, C.c_int, C.c_int, C.c_int, C.c_int64, C.c_int64, C.c_int64,
                         C.c_float, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_float,
                         C.c_void_p, C.c_int64)(sgemm)
        fn(101, 111, 111, rows, N_SK, M_SK, 1.0, Sblk.ctypes.data, M_SK, A_host.ctypes.data,
           N_SK, 0.0, B.ctypes.data, N_SK)
    else:
        B[:] = Sblk.reshape(rows, M_SK) @ A_host
    return time.perf_counter() - t0


# ----------------------------------------------------------------------------- main
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-rows", type=int, default=128,
                    help="operator rows of the bounded CPU-baseline sample")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batched", action="store_true",
                    help="skip the 512-problem batching measurement (about 15 s)")
    ap.add_argument("--precision", default="bf16", choices=["bf16", "fp8"],
                    help="tensor-core operand precision for the lowp-small case")
    ap.add_argument("--tile-config", type=int, default=5,
                    help="batching tile configuration for the batched-small case")
    ap.add_argument("--m-log2", type=int, default=17,
                    help="log2 of m for the dense small cases")
    ap.add_argument("--case", default="full",
                    choices=["full", "lowp-small", "plain-small", "saso", "convert-small",
                             "batched", "batched-small", "dense-fp64-small", "more-rows",
                             "autograd-small"],
                    help="full: the benchmark line; the others run one kernel family on a "
                         "smaller case (for profilers) and print a short JSON line")
    args = ap.parse_args()

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        return run_reference(args, rank, world)
    if world > 1 or args.gpus != 1:
        return refuse_multi_gpu(args, rank, world)
    if args.case != "full":
        return run_case(args)

    import torch

    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    from randblas_gb300 import build as rbuild
    rbuild.build()
    import randblas_gb300 as rb
    from randblas_gb300 import lowp
    stream = torch.cuda.current_stream()
    hbm, bf16_burst, bf16_sus, peak_kind = peaks()

    A, U = make_precision_input(torch, device)
    S = rb.DenseSkOp(rb.DenseDist(D_SK, M_SK, rb.ScalarDist.Uniform), rb.RNGState(3))
    B = torch.empty(D_SK, N_SK, device=device)
    flops = 2.0 * D_SK * M_SK * N_SK

    have_lowp = lowp.available()

    def plain():
        rb.sketch_general(rb.Layout.RowMajor, rb.Op.NoTrans, rb.Op.NoTrans, D_SK, N_SK, M_SK,
                          1.0, S, A, N_SK, 0.0, B, N_SK)

    def fused():
        lowp.sketch_lowp(rb.Layout.RowMajor, rb.Op.NoTrans, rb.Op.NoTrans, D_SK, N_SK, M_SK,
                         1.0, S, 0, 0, A, N_SK, 0.0, B, N_SK)

    headline = fused if have_lowp else plain
    # plain FP32 path on the same GPU (fewer steps: it is the slow arm)
    plain_steps = max(1, min(args.steps, 3))
    ms_plain = event_time(torch, plain, plain_steps, 1, stream)

    lib = rb.lib()
    launches0 = lib.rbg_kernel_launches()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        ms = event_time(torch, headline, args.steps, args.warmup, stream)
    launches = (lib.rbg_kernel_launches() - launches0)
    per_step_launches = launches / (args.steps + args.warmup)
    gpu_launches = int(round(per_step_launches * args.steps))
    # per-kernel times from a second pass with the library's event profiling on (its events
    # are kept out of the timed steps above)
    rb.profile.enable(True)
    event_time(torch, headline, args.steps, 1, stream)
    prof = rb.profile.read()
    rb.profile.enable(False)

    # accuracy of the headline result against an FP64 oracle on sampled row blocks
    headline()
    torch.cuda.synchronize()
    rel_err = sampled_rel_err(torch, rb, S, A, B, device)

    # the same sketch with FP8 e4m3 operands (a second precision form of this path)
    fp8 = None
    if have_lowp:
        def fused_fp8():
            lowp.sketch_lowp(rb.Layout.RowMajor, rb.Op.NoTrans, rb.Op.NoTrans, D_SK, N_SK, M_SK,
                             1.0, S, 0, 0, A, N_SK, 0.0, B, N_SK, precision=lowp.FP8_E4M3)
        rb.profile.enable(True)
        ms8 = event_time(torch, fused_fp8, args.steps, args.warmup, stream)
        prof8 = rb.profile.read()
        rb.profile.enable(False)
        fp8 = {"ms_per_step": round(ms8, 4), "TFLOP/s": round(flops / (ms8 * 1e-3) / 1e12, 1),
               "speedup_vs_fp32_plain": round(ms_plain / ms8, 2),
               "rel_frobenius_err_vs_fp64": sampled_rel_err(torch, rb, S, A, B, device),
               "kernels_ms": {k: round(v["ms"] / max(1, v["launches"]), 4)
                              for k, v in prof8.items()}}

    # subspace-embedding distortion of the headline operator on range(A) = range(U):
    # extreme singular values of S U / sqrt(d) (FP64 SVD on the host)
    distortion = embedding_distortion(torch, rb, lowp, have_lowp, S, U, device)
    del U

    # roofline of the dominant kernel
    main_kernel = max(prof, key=lambda k: prof[k]["ms"]) if prof else None
    if main_kernel:
        kms = prof[main_kernel]["ms"] / max(1, prof[main_kernel]["launches"])
        achieved = flops / (kms * 1e-3) / 1e12
    else:
        kms, achieved = ms, flops / (ms * 1e-3) / 1e12
    peak = bf16_burst if have_lowp else derived_fp32_peak(torch, clk.summary())
    roofline = {"bound": "tensor", "achieved": round(achieved, 1), "peak": round(peak, 1),
                "unit": "TFLOP/s", "frac": round(achieved / peak, 4),
                "traffic": HEADLINE_TRAFFIC_BYTES if have_lowp else None,
                "traffic_note": "ncu capture at m=2^17 scaled to m=2^20" if have_lowp else None,
                "kernel": main_kernel, "kernel_ms": round(kms, 4),
                "peak_source": ("bf16 burst, " + peak_kind) if have_lowp else
                "FP32 CUDA-core peak derived as SMs x 128 lanes x 2 x median SM clock"}

    # secondary rows: SASO sketch (HBM-bound), the small FP64 dense sketch, the
    # differentiation path and the batching path
    saso = bench_saso(torch, rb, device, args, stream, hbm)
    more_rows = bench_more_rows(torch, rb, device, stream, hbm)
    small = bench_small_fp64(torch, rb, device, stream)
    autograd_row = bench_autograd(torch, rb, device, stream, bf16_sus)
    batched_row = None if args.no_batched else bench_batched(torch, rb, device, args, stream)

    # end to end through the C ABI with host buffers
    e2e = None
    A_host = None
    if not args.no_e2e or not args.no_cpu:
        A_host = A.cpu().pin_memory() if not args.no_e2e else A.cpu()
    if not args.no_e2e:
        e2e = bench_e2e(torch, rb, lowp, have_lowp, S, A_host, args, stream, flops, device)

    cpu = None
    if not args.no_cpu:
        t = cpu_precision_sample(args.cpu_rows, A_host.numpy())
        full_s = t * D_SK / args.cpu_rows
        cpu = {"value": round(flops / full_s / 1e12, 5), "unit": "TFLOP/s",
               "cores": os.cpu_count(), "kind": "port",
               "sample": f"operator rows [0,{args.cpu_rows}) of 4096 (oracle OpenMP fill + "
                         f"OpenBLAS SGEMM), {t:.2f} s, scaled by {D_SK // args.cpu_rows}",
               "ms_per_sketch": round(full_s * 1e3, 1), "host": host_info()}

    value = flops / (ms * 1e-3) / 1e12
    line = {
        "metric": METRIC, "value": round(value, 2), "unit": "TFLOP/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "bf16" if have_lowp else "f32", "data": "synthetic",
        "config": headline_config(),
        "path": "bf16 tensor-core fused" if have_lowp else "fp32 plain",
        "kernels_ms": {k: round(v["ms"] / max(1, v["launches"]), 4) for k, v in prof.items()},
        "a_spectrum": "singular values 1 -> 1e-6 (random orthogonal factors)",
        "l2": "inputs larger than L2 (A is 4.3 GB)",
        "fp32_plain": {"ms_per_step": round(ms_plain, 3),
                       "TFLOP/s": round(flops / (ms_plain * 1e-3) / 1e12, 2)},
        "speedup_vs_fp32_plain": round(ms_plain / ms, 2),
        "rel_frobenius_err_vs_fp64": rel_err,
        "embedding_distortion": distortion, "fp8_e4m3": fp8,
        "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
        "gpu_launches": gpu_launches, "clocks": clk.summary(), "saso": saso,
        "dense_fp64_small": small, "autograd": autograd_row, "batched": batched_row,
        "more_rows": more_rows,
    }
    print(json.dumps(line))


def headline_config():
    """The workload both arms measure (the reference arm's A has another spectrum, which does
    not change the CPU path's cost)."""
    return {"workload": "uniform DenseDist 4096 x 2^20 (seed RNGState(3)) left sketch of a "
                        "2^20 x 1024 FP32 row-major matrix",
            "d": D_SK, "m": M_SK, "n": N_SK, "parallelism": "one GPU"}


def host_info():
    """CPU model, logical cores and RAM of this host (for the CPU baseline's record)."""
    model = None
    try:
        with open("/proc/cpuinfo") as f:
            for ln in f:
                if ln.lower().startswith("model name"):
                    model = ln.split(":", 1)[1].strip()
                    break
    except OSError:
        pass
    if model is None:
        try:
            out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
            for ln in out.splitlines():
                if ln.strip().lower().startswith("model name"):
                    model = ln.split(":", 1)[1].strip()
                    break
        except (OSError, subprocess.SubprocessError):
            pass
    try:
        ram = os.sysconf("SC_PAGE_SIZE") * os.sysconf("SC_PHYS_PAGES") / 2 ** 30
    except (ValueError, OSError):
        ram = None
    return {"cpu_model": model, "logical_cores": os.cpu_count(),
            "ram_gib": round(ram, 1) if ram else None}


def refuse_multi_gpu(args, rank, world):
    """The GPU arm measures one GPU; no multi-GPU launch of it is offered: every rank exits with
    status 2, rank 0 saying why on stderr."""
    if rank == 0:
        sys.stderr.write(json.dumps({
            "metric": METRIC, "error": "bench.py measures one GPU only",
            "requested_gpus": max(args.gpus, world),
            "why": "the benchmark measures the single-GPU sketch; it runs no replicas"}) + "\n")
    sys.exit(2)


def sampled_rel_err(torch, rb, S, A, B, device):
    """Relative Frobenius error of B = S A on four 64-row blocks against an FP64 product with
    the FP64 operator rows from fill_dense_unpacked."""
    err_num, err_den = 0.0, 0.0
    for r0 in (0, 1024, 2048, 4032):
        Sblk = torch.empty(64 * M_SK, dtype=torch.float64, device=device)
        rb.fill_dense_unpacked(rb.Layout.RowMajor, S.dist, 64, M_SK, r0, 0, Sblk, S.seed_state)
        ref = Sblk.view(64, M_SK) @ A.double()
        err_num += float((B[r0:r0 + 64].double() - ref).norm() ** 2)
        err_den += float(ref.norm() ** 2)
        del Sblk, ref
    return (err_num / err_den) ** 0.5


def embedding_distortion(torch, rb, lowp, have_lowp, S, U, device):
    """max(sigma_max - 1, 1 - sigma_min) of S U / sqrt(d) for the headline path (and the plain
    FP32 path): S is an approximate isometry on range(U) after the 1/sqrt(d) scaling (uniform
    entries have unit variance)."""
    import numpy as np
    out = {}
    paths = [("plain_fp32", None)]
    if have_lowp:
        paths += [("bf16_tc", lowp.BF16), ("fp8_e4m3_tc", lowp.FP8_E4M3)]
    for name, prec in paths:
        SU = torch.empty(D_SK, N_SK, device=device)
        if prec is not None:
            lowp.sketch_lowp(rb.Layout.RowMajor, rb.Op.NoTrans, rb.Op.NoTrans, D_SK, N_SK, M_SK,
                             1.0, S, 0, 0, U, N_SK, 0.0, SU, N_SK, precision=prec)
        else:
            rb.sketch_general(rb.Layout.RowMajor, rb.Op.NoTrans, rb.Op.NoTrans, D_SK, N_SK,
                              M_SK, 1.0, S, U, N_SK, 0.0, SU, N_SK)
        sv = np.linalg.svd(SU.double().cpu().numpy() / np.sqrt(D_SK), compute_uv=False)
        out[name] = {"sigma_max": float(sv[0]), "sigma_min": float(sv[-1]),
                     "distortion": float(max(sv[0] - 1.0, 1.0 - sv[-1]))}
        del SU
    return out


def bench_small_fp64(torch, rb, device, stream):
    """The reference's CPU-runnable dense case: Gaussian 200 x 10000 operator (seeded after a
    10000 x 50 uniform A from Philox key 0), FP64, column-major; latency of one sketch."""
    d, m, n = 200, 10000, 50
    A = torch.empty(m * n, dtype=torch.float64, device=device)
    nxt = rb.fill_dense_unpacked(rb.Layout.RowMajor, rb.DenseDist(50, 10000, rb.ScalarDist.Uniform),
                                 50, 10000, 0, 0, A, rb.RNGState(0))
    S = rb.DenseSkOp(rb.DenseDist(d, m), nxt, dtype=torch.float64)
    B = torch.empty(d * n, dtype=torch.float64, device=device)

    def step():
        rb.sketch_general(rb.Layout.ColMajor, rb.Op.NoTrans, rb.Op.NoTrans, d, n, m, 1.0, S, A,
                          m, 0.0, B, d)
    ms = event_time(torch, step, 20, 3, stream)
    return {"workload": "Gaussian 200 x 10000, A 10000 x 50 FP64 column-major",
            "us_per_sketch": round(ms * 1e3, 1),
            "GFLOP/s": round(2.0 * d * m * n / (ms * 1e-3) / 1e9, 1)}


def bench_autograd(torch, rb, device, stream, bf16_peak):
    """Forward + backward of ||S A - B||_F^2 through the autograd Function, Gaussian
    2048 x 2^18 operator (RNGState(5)), A 2^18 x 512: FP32 plain path and BF16 tensor cores."""
    from randblas_gb300 import autograd
    d, m, n = 2048, 1 << 18, 512
    S = rb.DenseSkOp(rb.DenseDist(d, m, rb.ScalarDist.Gaussian), rb.RNGState(5))
    g = torch.Generator(device=device).manual_seed(5)
    A0 = torch.randn(m, n, device=device, generator=g)
    Bt = torch.randn(d, n, device=device, generator=g)
    out = {"workload": "Gaussian 2048 x 2^18, A 2^18 x 512, loss ||S A - B||^2, fwd + bwd"}
    flops = 2 * 2.0 * d * m * n
    for name, prec, dt in (("fp32_plain", None, torch.float32), ("bf16_tc", "bf16", torch.float32),
                           ("bf16_tc_bf16_input", "bf16", torch.bfloat16)):
        # a fresh leaf for every variant (A0.to(float32) would return A0 itself, which would
        # then require grad and put a cast into the next variant's graph)
        A = A0.to(dt, copy=True).requires_grad_(True)

        def step():
            A.grad = None
            loss = ((autograd.sketch(S, A, precision=prec) - Bt) ** 2).sum()
            loss.backward()
        # steady state: ten steps after three warm-ups (the FP32 form takes ~37 ms a step)
        ms = event_time(torch, step, 10, 3, stream)
        out[name] = {"ms_fwd_bwd": round(ms, 3), "TFLOP/s": round(flops / (ms * 1e-3) / 1e12, 1)}
        if prec is not None and dt == torch.float32:
            out[name + "_graphed"] = autograd_graphed(torch, autograd, S, A, Bt, flops, stream)
    return out


def bench_autograd_small(torch, rb, device, args, stream):
    """The differentiation workload's BF16 forward + backward (Gaussian 2048 x m operator,
    RNGState(5), A m x 512 FP32) at m = 2^m_log2, with the per-kernel device times."""
    from randblas_gb300 import autograd
    d, m, n = 2048, 1 << args.m_log2, 512
    S = rb.DenseSkOp(rb.DenseDist(d, m, rb.ScalarDist.Gaussian), rb.RNGState(5))
    g = torch.Generator(device=device).manual_seed(5)
    A = torch.randn(m, n, device=device, generator=g).requires_grad_(True)
    Bt = torch.randn(d, n, device=device, generator=g)

    def step():
        A.grad = None
        ((autograd.sketch(S, A, precision="bf16") - Bt) ** 2).sum().backward()
    rb.profile.enable(True)
    ms = event_time(torch, step, args.steps, args.warmup, stream)
    prof = rb.profile.read()
    rb.profile.enable(False)
    return {"d": d, "m": m, "n": n, "ms_fwd_bwd": round(ms, 4),
            "TFLOP/s": round(4.0 * d * m * n / (ms * 1e-3) / 1e12, 1),
            "kernels_ms": {k: round(v["ms"] / max(1, v["launches"]), 4) for k, v in prof.items()}}


def autograd_graphed(torch, autograd, S, A, Bt, flops, stream):
    """The same forward + backward captured once in a CUDA graph and replayed: the device time
    of the step without host time between launches (A.grad is the graph's static output)."""
    try:
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            for _ in range(3):
                A.grad = None
                ((autograd.sketch(S, A, precision="bf16") - Bt) ** 2).sum().backward()
        torch.cuda.current_stream().wait_stream(side)
        graph = torch.cuda.CUDAGraph()
        A.grad = None
        with torch.cuda.graph(graph, capture_error_mode="relaxed"):
            ((autograd.sketch(S, A, precision="bf16") - Bt) ** 2).sum().backward()
        static_grad = A.grad
        ms = event_time(torch, graph.replay, 10, 3, stream)
        A.grad = None
        ((autograd.sketch(S, A, precision="bf16") - Bt) ** 2).sum().backward()
        same = bool(torch.equal(static_grad, A.grad))
        return {"ms_fwd_bwd": round(ms, 3), "TFLOP/s": round(flops / (ms * 1e-3) / 1e12, 1),
                "grad_equals_eager": same}
    except Exception as e:  # capture is a measurement aid, not part of the product path
        torch.cuda.synchronize()
        return {"error": str(e).splitlines()[0][:160]}


def derived_fp32_peak(torch, clocks):
    props = torch.cuda.get_device_properties(torch.cuda.current_device())
    mhz = clocks.get("sm_mhz") or 2070.0
    return props.multi_processor_count * 128 * 2 * mhz * 1e6 / 1e12


def bench_saso(torch, rb, device, args, stream, hbm):
    m, d, n = SASO_M, SASO_D, SASO_N
    A = torch.empty(m * n, dtype=torch.float32, device=device)
    nxt = rb.fill_dense(rb.DenseDist(m, n, rb.ScalarDist.Gaussian, rb.Axis.Short), A,
                        rb.RNGState(0))
    S = rb.SparseSkOp(rb.SparseDist(d, m, SASO_K), nxt)
    B = torch.empty(d * n, dtype=torch.float32, device=device)

    def step():
        rb.sketch_general(rb.Layout.RowMajor, rb.Op.NoTrans, rb.Op.NoTrans, d, n, m, 1.0, S, A,
                          n, 0.0, B, n)
    rb.profile.enable(True)
    ms = event_time(torch, step, args.steps, args.warmup, stream)
    prof = rb.profile.read()
    rb.profile.enable(False)
    algo = 4.0 * m * n + 4.0 * d * n
    out = {"workload": "SASO 1024 x 2^20, 8 nnz/col, sampled in the sketch; A 2^20 x 256 FP32",
           "ms_per_step": round(ms, 4), "GB/s": round(algo / (ms * 1e-3) / 1e9, 1),
           "frac_of_hbm": round(algo / (ms * 1e-3) / 1e9 / hbm, 4),
           "kernels_ms": {k: round(v["ms"] / max(1, v["launches"]), 4) for k, v in prof.items()}}
    del A, B
    return out


def bench_more_rows(torch, rb, device, stream, hbm):
    """Further rows of the hot path, each timed alone with CUDA events: fill_sparse of the
    1024 x 2^20 SASO operator (8 per column), the SASO sketch of a 2^20 x 256 matrix with that
    operator pre-filled (its COO arrays read from HBM), sketch_vector with the 4096 x 2^20 uniform
    operator, random_csr of a 2^17 x 512 matrix with 5 expected nonzeros per row, and
    sketch_sparse of a Gaussian 1024 x 2^17 operator against that matrix."""
    out = {}
    m, d, n, k = SASO_M, SASO_D, SASO_N, SASO_K
    A = torch.empty(m * n, dtype=torch.float32, device=device)
    nxt = rb.fill_dense(rb.DenseDist(m, n, rb.ScalarDist.Gaussian, rb.Axis.Short), A,
                        rb.RNGState(0))
    D = rb.SparseDist(d, m, k)
    S = rb.SparseSkOp(D, nxt)
    nnz = D.full_nnz
    S.rows = torch.empty(nnz, dtype=torch.int64, device=device)
    S.cols = torch.empty(nnz, dtype=torch.int64, device=device)
    S.vals = torch.empty(nnz, dtype=torch.float32, device=device)
    ms = event_time(torch, lambda: rb.fill_sparse(S), 10, 3, stream)
    written = nnz * (8 + 8 + 4)
    out["fill_sparse"] = {
        "workload": "SASO 1024 x 2^20, 8 nnz/col, int64 indices, FP32 values",
        "ms": round(ms, 4), "G_entries/s": round(nnz / (ms * 1e-3) / 1e9, 1),
        "GB/s_written": round(written / (ms * 1e-3) / 1e9, 1),
        "frac_of_hbm": round(written / (ms * 1e-3) / 1e9 / hbm, 4)}
    B = torch.empty(d * n, dtype=torch.float32, device=device)

    def step():
        rb.sketch_general(rb.Layout.RowMajor, rb.Op.NoTrans, rb.Op.NoTrans, d, n, m, 1.0, S, A,
                          n, 0.0, B, n)
    rb.profile.enable(True)
    ms = event_time(torch, step, 10, 3, stream)
    prof = rb.profile.read()
    rb.profile.enable(False)
    algo = 4.0 * m * n + 4.0 * d * n + written
    out["saso_prefilled"] = {
        "workload": "SASO 1024 x 2^20 sketch of a 2^20 x 256 FP32 matrix after fill_sparse: "
                    "COO operator read from HBM",
        "ms": round(ms, 4), "GB/s": round(algo / (ms * 1e-3) / 1e9, 1),
        "frac_of_hbm": round(algo / (ms * 1e-3) / 1e9 / hbm, 4),
        "kernels_ms": {kk: round(v["ms"] / max(1, v["launches"]), 4) for kk, v in prof.items()}}
    del A, B, S

    Sv = rb.DenseSkOp(rb.DenseDist(D_SK, M_SK, rb.ScalarDist.Uniform), rb.RNGState(3))
    g = torch.Generator(device=device).manual_seed(7)
    x = torch.randn(M_SK, device=device, generator=g)
    y = torch.empty(D_SK, device=device)
    ms = event_time(torch, lambda: rb.sketch_vector(rb.Op.NoTrans, D_SK, M_SK, 1.0, Sv, 0, 0, x,
                                                    1, 0.0, y, 1), 5, 2, stream)
    entries = D_SK * M_SK
    out["sketch_vector"] = {
        "workload": "uniform 4096 x 2^20 operator (RNGState(3)) times a 2^20 FP32 vector",
        "ms": round(ms, 4), "G_operator_entries/s": round(entries / (ms * 1e-3) / 1e9, 1),
        "GFLOP/s": round(2.0 * entries / (ms * 1e-3) / 1e9, 1)}
    del x, y

    ds, ms_, ns, per_row = 1024, 1 << 17, 512, 5
    gen = lambda: rb.random_csr(ms_, ns, per_row / ns, rb.RNGState(11), dtype=torch.float32)
    ms = event_time(torch, gen, 5, 2, stream)
    Acsr, _ = gen()
    nnz_csr = Acsr.vals.numel()
    out["random_csr"] = {
        "workload": "random_csr(2^17, 512, density 5/512, RNGState(11)): FP32 values, int64 "
                    "indices, structure drawn on the GPU, nnz read back, arrays written",
        "ms": round(ms, 4), "nnz": nnz_csr,
        "M_nonzeros/s": round(nnz_csr / (ms * 1e-3) / 1e6, 1)}
    Sg = rb.DenseSkOp(rb.DenseDist(ds, ms_, rb.ScalarDist.Gaussian), rb.RNGState(5))
    Bs = torch.empty(ds * ns, device=device)
    ms = event_time(torch, lambda: rb.sketch_sparse(rb.Layout.RowMajor, rb.Op.NoTrans,
                                                    rb.Op.NoTrans, ds, ns, ms_, 1.0, Sg, 0, 0,
                                                    Acsr, 0.0, Bs, ns), 5, 2, stream)
    out["sketch_sparse"] = {
        "workload": "Gaussian 1024 x 2^17 operator (RNGState(5)) times that 2^17 x 512 CSR "
                    "matrix; the operator is generated inside the SpMM (the reference fills it "
                    "first)",
        "ms": round(ms, 4), "GFLOP/s": round(2.0 * ds * nnz_csr / (ms * 1e-3) / 1e9, 1)}
    return out


def batched_workload(torch, rb, device, count=512):
    """512 left sketches: m log-uniform in [2^12, 2^18], n uniform in [16, 512], d = 4n
    (numpy default_rng(0)); A_i N(0,1) FP32 row-major from fill_dense with key 1000 + i;
    Gaussian operators with chained states starting at RNGState(4)."""
    import numpy as np
    from randblas_gb300 import batched
    rng = np.random.default_rng(0)
    ms = np.round(2.0 ** rng.uniform(12, 18, count)).astype(int)
    ns = rng.integers(16, 513, count)
    probs, state = [], rb.RNGState(4)
    for i in range(count):
        d, n, m = 4 * int(ns[i]), int(ns[i]), int(ms[i])
        A = torch.empty(m, n, device=device)
        rb.fill_dense(rb.DenseDist(m, n, rb.ScalarDist.Gaussian, rb.Axis.Short), A.view(-1),
                      rb.RNGState(1000 + i))
        S = rb.DenseSkOp(rb.DenseDist(d, m, rb.ScalarDist.Gaussian), state)
        state = S.next_state
        probs.append(batched.BatchProblem(S, A, torch.empty(d, n, device=device), d, n, m))
    return probs


# n classes of the batching workload for the per-class breakdown (FLOPs grow as n^2 m)
BATCH_CLASSES = ((16, 64), (65, 128), (129, 256), (257, 512))
FP32_SIMT_TFLOPS = 152 * 128 * 2 * 2.07e9 / 1e12  # FFMA lanes x 2 FLOP x max SM clock


def bench_batched(torch, rb, device, args, stream, tune=True):
    """The 512-problem batch three ways: 512 separate plain launches, one persistent launch
    with the library's default tiles, and one with the autotuner's tiles (tuned before the
    timed region; the tuning time is reported).  Then each n class on its own, batched and
    as separate launches, with its fraction of the FP32 FFMA peak."""
    import tempfile
    import time
    from randblas_gb300 import batched
    probs = batched_workload(torch, rb, device)
    flops = sum(2.0 * p.d * p.n * p.m for p in probs)

    def separate(ps):
        for p in ps:
            rb.sketch_general(rb.Layout.RowMajor, rb.Op.NoTrans, rb.Op.NoTrans, p.d, p.n, p.m,
                              1.0, p.S, p.A, p.n, 0.0, p.B, p.n)
    steps = max(1, min(args.steps, 3))
    ms_sep = event_time(torch, lambda: separate(probs), steps, 1, stream)
    res = {"workload": "512 Gaussian left sketches, m log-uniform [2^12, 2^18], n uniform "
                       "[16, 512], d = 4n, FP32", "gflop": round(flops / 1e9, 1),
           "separate_plain_launches": {"ms": round(ms_sep, 2),
                                       "TFLOP/s": round(flops / ms_sep / 1e9, 2)}}
    tuned_plan, tuner = None, None
    if tune:
        # per-class choices, then checked against the library's choices on this batch
        cache = os.path.join(tempfile.mkdtemp(prefix="rbg_tiles_"), "tiles.json")
        tuner = batched.Autotuner(cache_path=cache)
        t0 = time.perf_counter()
        for p in probs:
            p.tile_config = 0
        tuned_plan = tuner.tune_batch(probs)
        torch.cuda.synchronize()
        res["autotune_s"] = round(time.perf_counter() - t0, 1)
        tuned_cfg = [p.tile_config for p in probs]
    variants = [("default_tiles", None)] + ([("autotuned", tuned_plan)] if tune else [])
    for name, tp in variants:
        if tp is None:
            for p in probs:
                p.tile_config = 0
            plan = batched.BatchedPlan(probs)
        else:
            for p, c in zip(probs, tuned_cfg):
                p.tile_config = c
            plan = tp
        graph = plan.capture()
        ms = event_time(torch, graph.replay, steps, 1, stream)
        res[name] = {"ms": round(ms, 2), "TFLOP/s": round(flops / ms / 1e9, 2),
                     "speedup_vs_separate": round(ms_sep / ms, 2),
                     "work_items": plan.info()["work_items"]}
        shapes = {}
        for p in probs:
            key = "x".join(str(x) if x else "all" for x in batched.tile_shape(p.tile_config)) \
                if p.tile_config \
                else "library"
            shapes[key] = shapes.get(key, 0) + 1
        res[name]["tiles"] = shapes
        plan.close()
    per_class = {}
    for lo, hi in BATCH_CLASSES:
        sub = [p for p in probs if lo <= p.n <= hi]
        if not sub:
            continue
        fl = sum(2.0 * p.d * p.n * p.m for p in sub)
        for p in sub:
            p.tile_config = 0
        plan = batched.BatchedPlan(sub, tuner=tuner)
        graph = plan.capture()
        ms_b = event_time(torch, graph.replay, steps, 1, stream)
        plan.close()
        ms_s = event_time(torch, lambda: separate(sub), steps, 1, stream)
        per_class[f"n{lo}-{hi}"] = {
            "problems": len(sub), "gflop_share": round(fl / flops, 3),
            "batched_TFLOP/s": round(fl / ms_b / 1e9, 2),
            "separate_TFLOP/s": round(fl / ms_s / 1e9, 2),
            "batched_frac_fp32_peak": round(fl / ms_b / 1e9 / FP32_SIMT_TFLOPS, 3)}
    res["per_class"] = per_class
    res["fp32_peak_TFLOP/s"] = round(FP32_SIMT_TFLOPS, 1)
    return res


def bench_batched_small(torch, rb, device, args, stream):
    """The batching workload's dominant class at a size a full profiler capture handles: 48
    Gaussian problems, n uniform in [257, 512], d = 4n, m = 2^15, all on tile configuration
    --tile-config (5: row blocks)."""
    import numpy as np
    from randblas_gb300 import batched
    rng = np.random.default_rng(0)
    probs, state = [], rb.RNGState(4)
    for _ in range(48):
        n = int(rng.integers(257, 513))
        d, m = 4 * n, 1 << 15
        A = torch.randn(m, n, device=device)
        S = rb.DenseSkOp(rb.DenseDist(d, m, rb.ScalarDist.Gaussian), state)
        state = S.next_state
        probs.append(batched.BatchProblem(S, A, torch.empty(d, n, device=device), d, n, m,
                                          tile_config=args.tile_config))
    flops = sum(2.0 * p.d * p.n * p.m for p in probs)
    plan = batched.BatchedPlan(probs)
    ms = event_time(torch, plan.execute, max(1, args.steps), args.warmup, stream)
    plan.close()
    return {"workload": "48 Gaussian sketches, n in [257, 512], d = 4n, m = 2^15",
            "tile_config": args.tile_config, "ms": round(ms, 3),
            "TFLOP/s": round(flops / ms / 1e9, 2)}


def bench_e2e(torch, rb, lowp, have_lowp, S, A_host, args, stream, flops, device):
    """Same sketch through the public API with host buffers.  Precision path: A and B stay in
    pinned host memory and are passed to the call itself (its A conversion pass reads A over
    the host link; B is written in place).  Plain path: copy A in, sketch, copy B back."""
    B_host = torch.empty(D_SK, N_SK, pin_memory=True)
    if not have_lowp:
        A_dev = torch.empty(M_SK, N_SK, device=device)
        B_dev = torch.empty(D_SK, N_SK, device=device)

    def step():
        if have_lowp:
            lowp.sketch_lowp(rb.Layout.RowMajor, rb.Op.NoTrans, rb.Op.NoTrans, D_SK, N_SK, M_SK,
                             1.0, S, 0, 0, A_host, N_SK, 0.0, B_host, N_SK)
            return
        A_dev.copy_(A_host, non_blocking=True)
        rb.sketch_general(rb.Layout.RowMajor, rb.Op.NoTrans, rb.Op.NoTrans, D_SK, N_SK, M_SK,
                          1.0, S, A_dev, N_SK, 0.0, B_dev, N_SK)
        B_host.copy_(B_dev, non_blocking=True)
    # three warm-up steps: the first calls on a freshly pinned buffer can take 1.3-3x longer;
    # up to ten timed steps (single calls of 60-110 ms appear now and then on the host link).
    # The value is the mean over the steps; each step's own time is recorded beside it.
    steps = max(1, min(args.steps, 10))
    for _ in range(3):
        step()
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
    ev[0].record(stream)
    for t in range(steps):
        step()
        ev[t + 1].record(stream)
    torch.cuda.synchronize()
    per = sorted(ev[t].elapsed_time(ev[t + 1]) for t in range(steps))
    ms = ev[0].elapsed_time(ev[steps]) / steps
    return {"value": round(flops / (ms * 1e-3) / 1e12, 2), "unit": "TFLOP/s",
            "ms_per_step": round(ms, 3), "h2d_bytes_per_step": M_SK * N_SK * 4,
            "d2h_bytes_per_step": D_SK * N_SK * 4,
            "step_ms_median": round(per[len(per) // 2], 3), "step_ms_max": round(per[-1], 3)}


def run_case(args):
    """One kernel family on a smaller case: 4096 x 2^m_log2 uniform operator against a
    2^m_log2 x 1024 FP32 matrix (default 2^17: 512 MiB, larger than L2) for the dense paths;
    the full SASO workload for the sparse path."""
    import torch

    import randblas_gb300 as rb
    from randblas_gb300 import build as rbuild
    from randblas_gb300 import lowp
    rbuild.build()
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream()
    out = {"case": args.case}
    if args.case == "saso":
        out.update(bench_saso(torch, rb, dev, args, stream, peaks()[0]))
    elif args.case == "batched":
        out.update(bench_batched(torch, rb, dev, args, stream))
    elif args.case == "batched-small":
        out.update(bench_batched_small(torch, rb, dev, args, stream))
    elif args.case == "more-rows":
        out.update(bench_more_rows(torch, rb, dev, stream, peaks()[0]))
    elif args.case == "autograd-small":
        out.update(bench_autograd_small(torch, rb, dev, args, stream))
    elif args.case == "dense-fp64-small":
        rb.profile.enable(True)
        out.update(bench_small_fp64(torch, rb, dev, stream))
        out["kernels_ms"] = {k: round(v["ms"] / max(1, v["launches"]), 4)
                             for k, v in rb.profile.read().items()}
        rb.profile.enable(False)
    else:
        m = 1 << args.m_log2
        S = rb.DenseSkOp(rb.DenseDist(D_SK, m, rb.ScalarDist.Uniform), rb.RNGState(3))
        A = torch.randn(m, N_SK, device=dev)
        B = torch.empty(D_SK, N_SK, device=dev)
        if args.case == "lowp-small":
            prec = lowp.FP8_E4M3 if args.precision == "fp8" else lowp.BF16

            def step():
                lowp.sketch_lowp(rb.Layout.RowMajor, rb.Op.NoTrans, rb.Op.NoTrans, D_SK, N_SK, m,
                                 1.0, S, 0, 0, A, N_SK, 0.0, B, N_SK, precision=prec)
        elif args.case == "convert-small":
            def step():
                # the same call with a 1-row operator: the A conversion dominates
                lowp.sketch_lowp(rb.Layout.RowMajor, rb.Op.NoTrans, rb.Op.NoTrans, 1, N_SK, m,
                                 1.0, S, 0, 0, A, N_SK, 0.0, B, N_SK)
        else:
            def step():
                rb.sketch_general(rb.Layout.RowMajor, rb.Op.NoTrans, rb.Op.NoTrans, D_SK, N_SK, m,
                                  1.0, S, A, N_SK, 0.0, B, N_SK)
        rb.profile.enable(True)
        ms = event_time(torch, step, args.steps, args.warmup, stream)
        prof = rb.profile.read()
        rb.profile.enable(False)
        out.update({"d": D_SK, "m": m, "n": N_SK, "ms_per_step": round(ms, 4),
                    "TFLOP/s": round(2.0 * D_SK * m * N_SK / (ms * 1e-3) / 1e12, 1),
                    "kernels_ms": {k: round(v["ms"] / max(1, v["launches"]), 4)
                                   for k, v in prof.items()}})
    print(json.dumps(out))


def run_reference(args, rank, world):
    """The reference's CPU path (the oracle's OpenMP port of the operator fill plus OpenBLAS
    SGEMM, as RandBLAS materialises the submatrix and calls blas::gemm), each step a bounded
    row block of the same workload, extrapolated to the full sketch."""
    if rank != 0:
        return
    import numpy as np
    rng = np.random.default_rng(0)
    # the CPU arm needs A on the host; the exact singular spectrum does not change its cost
    A_host = rng.standard_normal((M_SK, N_SK), dtype=np.float32)
    for _ in range(max(0, min(args.warmup, 1))):
        cpu_precision_sample(16, A_host)
    times = [cpu_precision_sample(args.cpu_rows, A_host) for _ in range(args.steps)]
    t = statistics.median(times)
    full_s = t * D_SK / args.cpu_rows
    flops = 2.0 * D_SK * M_SK * N_SK
    value = flops / full_s / 1e12
    line = {"impl": "reference", "metric": METRIC, "value": round(value, 5), "unit": "TFLOP/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(full_s * 1e3, 1), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": headline_config(),
            "path": "CPU: operator fill + OpenBLAS SGEMM (RandBLAS's materialise-then-gemm)",
            "a_spectrum": "N(0,1) entries (the cost does not depend on the values)",
            "cpu_baseline": {"value": round(value, 5), "unit": "TFLOP/s",
                             "cores": os.cpu_count(), "kind": "port",
                             "sample": f"operator rows [0,{args.cpu_rows}) per step, scaled by "
                                       f"{D_SK // args.cpu_rows}", "host": host_info()},
            "e2e": {"value": round(value, 5), "unit": "TFLOP/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


if __name__ == "__main__":
    main()
