#!/usr/bin/env python
"""CAQR benchmark on GB300: the reference's 2D QR (QR_2D) of one square matrix.

Workload (the configuration the headline metric is quoted on): n = 16384,
float64, A = U diag(sigma) V^T with U, V Haar-orthogonal (Mezzadri's
Q*diag(sign(diag R)) of Gaussian draws from numpy PCG64(seed=1), U drawn
first), sigma log-spaced from 1 to 1e-6, panel width b = 128: every panel is
factored by TSQR + Householder reconstruction and the trailing matrix is
updated with A -= Y T^T (Y^T A).

One step = restore A from the device-resident input (2 GiB D2D copy) + one
full factorization.  The 2 GiB input is larger than L2 (129 MB), so no flush
is needed between steps.  Metric: FP64-equivalent TFLOP/s = (4/3 n^3) / step
time (the reference's own GFlops formula 2mk^2 - 2/3 k^3 at m = k,
bench/QR/bench_qr_2d.cxx:85-87).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl candmc|reference]

N > 1 (torchrun) runs N independent replicas (the factorization of one
matrix is not sharded across GPUs here), value = N * flops / max time.
`--impl reference` times the reference's own single-rank call sequence
(dgeqrf, dorgqr, signed LU, dtrsm, dgemm: oracle/reference_lapack.py) on the
host cores with all BLAS threads, on a bounded n = 8192 sample.
"""
import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

FP64_PEAK_GF = 1170.0   # measured DFMA rate of this GB300 (chip-wide microbenchmark)


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["candmc", "reference"], default="candmc")
    p.add_argument("--n", type=int, default=16384)
    p.add_argument("--b", type=int, default=128)
    p.add_argument("--form", choices=["fp64", "ozaki"], default="ozaki")
    p.add_argument("--entry", choices=["pipe", "qr2d"], default="pipe",
                   help="QR_2D_pipe (lookahead, the reference tests' default) or QR_2D")
    p.add_argument("--sigma-min", type=float, default=1e-6)
    p.add_argument("--seed", type=int, default=1)
    p.add_argument("--ref-n", type=int, default=8192, help="bounded CPU sample size")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    return p.parse_args()


def flops(n):
    return 4.0 / 3.0 * float(n) ** 3


# ----------------------------------------------------------------- inputs
def make_input_gpu(n, seed, sigma_min, device):
    """A = U diag(sigma) V^T, U and V Haar from PCG64(seed) (U first), on the GPU."""
    import ctypes

    import torch
    # torch loads its CUDA linear-algebra library lazily by bare name; load it
    # by path first so the lookup also succeeds under a profiler's injection.
    linalg = os.path.join(os.path.dirname(torch.__file__), "lib", "libtorch_cuda_linalg.so")
    if os.path.exists(linalg):
        ctypes.CDLL(linalg, mode=ctypes.RTLD_GLOBAL)
    rng = np.random.default_rng(seed)
    mats = []
    for _ in range(2):
        G = torch.from_numpy(rng.standard_normal((n, n))).to(device)
        Q, R = torch.linalg.qr(G)
        Q *= torch.sign(torch.diagonal(R))[None, :]
        mats.append(Q)
        del G, R
    U, V = mats
    s = torch.logspace(0, np.log10(sigma_min), n, dtype=torch.float64, device=device)
    A = (U * s[None, :]) @ V.t()
    del U, V
    torch.cuda.synchronize()
    return A.t().contiguous().t()   # column-major


# ----------------------------------------------------------------- clocks
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    NAMES = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]

    def __init__(self, gpu_id):
        self.proc = None
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(gpu_id)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=10)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, smax, reasons, power = [], [], set(), []
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
                power.append(float(f[3]))
            except ValueError:
                continue
            for name, v in zip(self.NAMES, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        top = max(sm)
        loaded = [x for x in sm if x >= 0.5 * top] or sm
        return {"sm_mhz": statistics.median(loaded), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm),
                "power_w_max": max(power) if power else None}


def gpu_id_for_smi(local_rank):
    vis = os.environ.get("CUDA_VISIBLE_DEVICES")
    if vis:
        ids = [x.strip() for x in vis.split(",") if x.strip()]
        if local_rank < len(ids):
            return ids[local_rank]
    return str(local_rank)


# ----------------------------------------------------------------- helpers
def traffic_from_profile(name):
    """Per-launch DRAM bytes recorded by the committed ncu summary, if present."""
    path = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(path):
        return None
    m = re.search(r"traffic_per_launch_bytes\s*[:=]\s*([0-9.eE+]+)", open(path).read())
    return float(m.group(1)) if m else None


def sampled_backward_error(cm, A0, YR, b, ncols=64, seed=0):
    """||Q^T A0[:, S] - R[:, S]||_F / ||A0[:, S]||_F over a random column sample S.

    Q^T is applied panel by panel with update_A (T from Y^T Y, qr_2d.cxx:22-60),
    the reference tests' residual restricted to sampled columns.
    """
    import torch
    n = A0.shape[0]
    rng = np.random.default_rng(seed)
    S = torch.from_numpy(np.sort(rng.choice(n, size=min(ncols, n), replace=False))).to(A0.device)
    X = A0[:, S].t().contiguous().t()
    for r0 in range(0, n, b):
        bb = min(b, n - r0)
        if n - r0 <= 0:
            break
        cm.update_A(YR[r0:, r0:r0 + bb], X[r0:, :], bb, None)
    R = torch.triu(YR)[:, S]
    torch.cuda.synchronize()
    return float(torch.linalg.norm(X - R) / torch.linalg.norm(A0[:, S]))


# ----------------------------------------------------------------- reference arm
def run_reference(args, world, rank):
    if rank != 0:
        return 0
    from oracle import fixtures as fx
    from oracle import reference_lapack as rl
    n = args.ref_n
    rng = np.random.default_rng(args.seed)
    A0 = np.asfortranarray(fx.svd_matrix(n, n, args.seed, args.sigma_min)) if n <= 4096 else \
        np.asfortranarray(rng.standard_normal((n, n)))
    times = []
    for it in range(args.warmup + args.steps):
        A = A0.copy(order="F")
        t0 = time.perf_counter()
        rl.QR_2D_lapack(A, args.b)
        dt = time.perf_counter() - t0
        if it >= args.warmup:
            times.append(dt)
    tot = sum(times)
    val = flops(n) * len(times) / tot / 1e12
    cores = rl.blas_threads()
    line = {
        "impl": "reference",
        "metric": "CAQR TFLOP/s (FP64-equivalent, 4/3 n^3 per factorization)",
        "value": val, "unit": "TFLOP/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * tot / len(times), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"CAQR QR_2D n={args.n} b={args.b} float64 (timed on a bounded "
                               f"n={n} sample on the host cores)",
                   "n": args.n, "b": args.b, "sample_n": n, "form": "reference LAPACK call sequence",
                   "parallelism": "host BLAS threads"},
        "cpu_baseline": {"value": val, "unit": "TFLOP/s", "cores": cores, "kind": "port",
                         "sample": f"QR_2D_lapack n={n} (bounded sample of the n={args.n} workload; "
                                   "Gaussian input above n=4096)"},
        "e2e": {"value": val, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def cpu_baseline(args):
    from oracle import reference_lapack as rl
    n = min(args.ref_n, args.n)
    rng = np.random.default_rng(args.seed)
    A0 = np.asfortranarray(rng.standard_normal((n, n)))
    rl.QR_2D_lapack(A0.copy(order="F")[: n // 4, : n // 4].copy(order="F"), args.b)  # warm-up
    A = A0.copy(order="F")
    t0 = time.perf_counter()
    rl.QR_2D_lapack(A, args.b)
    dt = time.perf_counter() - t0
    return {"value": flops(n) / dt / 1e12, "unit": "TFLOP/s", "cores": rl.blas_threads(),
            "kind": "port",
            "sample": f"reference QR_2D call sequence on LAPACK/BLAS (scipy OpenBLAS), n={n}, "
                      f"b={args.b}, Gaussian input, one factorization ({dt:.1f} s)"}


# ----------------------------------------------------------------- main
def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, world, rank)

    import torch
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)

    from candmc_gb300 import build as _build
    _build.build()
    import candmc_gb300 as cm
    from candmc_gb300 import _abi
    lib = cm.lib()

    n, b = args.n, args.b
    A0 = make_input_gpu(n, args.seed + rank * 1000 if world > 1 else args.seed, args.sigma_min, dev)
    A = torch.empty_like(A0.t()).t()
    prec = args.form

    qr = cm.QR_2D_pipe if args.entry == "pipe" else cm.QR_2D

    def step():
        A.copy_(A0)
        qr(A, b, precision=prec)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()

    # dominant kernel class of this form, timed live on its launching stream
    dom = {"fp64": ["gemm_tn", "gemm_nn"], "ozaki": ["oz_tn", "oz_nn"]}[prec]
    mask = 0
    for c in dom:
        mask |= 1 << _abi.KCLASS[c]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(gpu_id_for_smi(local))
    launches0 = lib.candmc_launch_count()
    lib.candmc_profile_begin(mask)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        step()
    e1.record()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    ms = e0.elapsed_time(e1)
    launches = lib.candmc_launch_count() - launches0
    import ctypes
    nc = _abi.NKCLASS
    kms = (ctypes.c_double * nc)()
    kwork = (ctypes.c_double * nc)()
    kl = (ctypes.c_longlong * nc)()
    lib.candmc_profile_end(nc, kms, kwork, kl)
    clk = clocks.stop()
    t_max = ms
    if dist:
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_max = float(t.item())
    value = world * flops(n) * args.steps / (t_max / 1e3) / 1e12

    dom_ms = sum(kms[_abi.KCLASS[c]] for c in dom)
    dom_work = sum(kwork[_abi.KCLASS[c]] for c in dom)
    dom_l = sum(kl[_abi.KCLASS[c]] for c in dom)
    achieved = dom_work / (dom_ms / 1e3) / 1e12 if dom_ms > 0 else None
    if prec == "fp64":
        roof = {"bound": "fp64", "achieved": achieved, "peak": FP64_PEAK_GF / 1e3,
                "unit": "TFLOP/s", "frac": achieved / (FP64_PEAK_GF / 1e3) if achieved else None,
                "traffic": traffic_from_profile("gemm_f64_caqr_n16384.md"),
                "kernel": "k_gemm_f64 (Y^T A split-K partials and A -= Y Z)",
                "launches": dom_l, "share_of_step": dom_ms / ms if ms else None,
                "peak_source": "DFMA microbenchmark on this GB300 (FP64 is not in MEASURED_PEAKS.json); "
                               "FP64 is neither the HBM nor the tensor roof"}
    else:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) \
            if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
        # Each FP64 product is emulated by 28 BF16 slice products (7 slices,
        # pairs i + j <= 6), so the emulated-FP64 roof is the BF16 roof / 28;
        # `achieved` counts algorithmic FP64 flops (2 m n k per contraction).
        pk_bf16 = peaks.get("bf16_tflops_sustained", 1700.0)
        pk = pk_bf16 / 28.0
        roof = {"bound": "tensor", "achieved": achieved, "peak": pk, "unit": "TFLOP/s",
                "frac": achieved / pk if achieved else None,
                "bf16_issued_tflops": achieved * 28.0 if achieved else None,
                "traffic": traffic_from_profile("ozaki_gemm_caqr_n16384.md"),
                "kernel": "k_oz_mma (Ozaki BF16 slice contractions on tcgen05, Y^T A and A -= Y Z)",
                "launches": dom_l, "share_of_step": dom_ms / ms if ms else None,
                "peak_source": "MEASURED_PEAKS.json bf16_tflops_sustained / 28 slice products "
                               "(of measured)"}

    # accuracy of the last factorization
    bwd = sampled_backward_error(cm, A0, A, b)

    # end-to-end through the host-pointer C ABI (pinned host buffers)
    e2e = None
    if not args.no_e2e:
        src = torch.empty((n, n), dtype=torch.float64, pin_memory=True)
        src.copy_(A0.t())                 # row-major (n x n) of A^T == column-major A
        work = torch.empty((n, n), dtype=torch.float64, pin_memory=True)
        host_view = work.numpy().T        # Fortran-ordered view
        tt = 0.0
        for it in range(1 + args.steps):
            work.copy_(src)
            t0 = time.perf_counter()
            cm.QR_2D(host_view, b, precision=prec)
            dt = time.perf_counter() - t0
            if it >= 1:
                tt += dt
        e2e = {"value": world * flops(n) * args.steps / tt / 1e12, "unit": "TFLOP/s",
               "h2d_bytes_per_step": 8 * n * n, "d2h_bytes_per_step": 8 * n * n}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_baseline(args)

    if rank == 0:
        line = {
            "metric": "CAQR TFLOP/s (FP64-equivalent, 4/3 n^3 per factorization)",
            "value": value, "unit": "TFLOP/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if prec == "fp64" else "f64 (emulated: bf16 Ozaki slices, fp32 accumulate)",
            "data": "synthetic",
            "config": {"workload": f"CAQR QR_2D n={n} b={b} float64, A=U diag(logspace(0,"
                                   f"{np.log10(args.sigma_min):.0f},n)) V^T, U,V Haar (PCG64 seed {args.seed})",
                       "n": n, "b": b, "form": prec, "parallelism": f"replicas x{world}",
                       "l2": "input 2 GiB > L2 129 MB, no flush needed"},
            "clocks": clk,
            "e2e": e2e,
            "gpu_launches": launches,
            "roofline": roof,
            "cpu_baseline": cpu,
            "accuracy": {"backward_error_sampled": bwd, "columns": 64,
                         "bound": 1e-13},
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
