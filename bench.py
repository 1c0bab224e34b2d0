#!/usr/bin/env python
"""Benchmarks of the CANDMC QR hot path on GB300.

Default workload (the configuration the headline metric is quoted on):
`caqr` -- the reference's 2D QR of one square matrix, n = 16384, float64,
A = U diag(sigma) V^T with U, V Haar-orthogonal (Mezzadri's Q*diag(sign(diag
R)) of Gaussian draws from numpy PCG64(seed=1), U drawn first), sigma
log-spaced from 1 to 1e-6, panel width b = 128: every panel is factored by
TSQR + Householder reconstruction and the trailing matrix is updated with
A -= Y T^T (Y^T A).  One step = restore A from the device-resident input
(2 GiB D2D copy) + one full factorization; the 2 GiB input is larger than L2
(129 MB), so no flush is needed between steps.  Metric: FP64-equivalent
TFLOP/s = (4/3 n^3) / step time (the reference's GFlops formula
2mk^2 - 2/3 k^3 at m = k, bench/QR/bench_qr_2d.cxx:85-87).  The line also
carries the whole-matrix backward error and orthogonality of the timed
factorization, and, each with its own step count, `fp64_form` (the plain FP64
form on the same matrix), `tsqr_hr`, `forms`, `batched` and `serve` (the
workloads below).

Other workloads (`--workload`), one JSON line each in the same format:
  tsqr_hr  TSQR-HR of one 8192 x 64 N(0,1) panel (seed 0): hh_recon_qr,
           L2 flushed between steps.
  forms    precision forms of CAQR at m = 32768, n = 16384 (U, V Haar from
           seed 2, sigma to 1e-10 and to 1e-3): QR_2D_pipe in the ozaki, fp32
           and fp64 forms, then least squares with 16 N(0,1) right-hand sides
           refined in FP64.
  batched  4096 uneven least-squares problems in one batched call (m
           log-uniform in [256, 262144], n in {8,16,32,64,128}), autotuned,
           CUDA-graph replay; metric solves/s.
  serve    the least-squares request server under Poisson arrivals (seed 4)
           at 1k..50k requests/s, m log-uniform in [512, 1048576], n in
           {16,32,64,128,256}; FP32 CAQR + FP64 refinement; p50/p99 latency
           and solves/s beside the plain FP64 one-request-at-a-time path.

    python bench.py [--workload W] [--gpus N] [--steps K] [--warmup W] [--impl candmc|reference]

N > 1 (torchrun) runs N independent replicas (the problems are not sharded
across GPUs), value = N * work / max time.  `--impl reference` times the
reference's own CPU path on the host cores: for caqr, full QR_2D
factorizations of the same n = 16384 matrix (the compiled reference where it
was built from its sources, oracle/_ref; elsewhere its LAPACK call sequence
replayed on the same OpenBLAS, oracle/reference_lapack.py, which gives
bitwise-equal results); its warm-up steps factor a leading block only.
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
WORKLOADS = ("caqr", "tsqr_hr", "forms", "batched", "serve")


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--workload", choices=WORKLOADS, default="caqr")
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["candmc", "reference"], default="candmc")
    p.add_argument("--m", type=int, default=None)
    p.add_argument("--n", type=int, default=None)
    p.add_argument("--b", type=int, default=None)
    p.add_argument("--form", choices=["fp64", "ozaki", "fp32"], default=None)
    p.add_argument("--forms", default="ozaki,fp32")
    p.add_argument("--entry", choices=["pipe", "qr2d"], default="pipe",
                   help="QR_2D_pipe (lookahead, the reference tests' default) or QR_2D")
    p.add_argument("--sigma-min", type=float, default=1e-6)
    p.add_argument("--seed", type=int, default=None)
    p.add_argument("--ref-n", type=int, default=8192, help="bounded CPU sample size (caqr)")
    p.add_argument("--count", type=int, default=None, help="problems (batched) / requests per rate (serve)")
    p.add_argument("--rates", default="1000,2000,5000,10000,20000,50000")
    p.add_argument("--workers", type=int, default=12)
    p.add_argument("--budget-gb", type=float, default=120.0)
    p.add_argument("--no-graph", action="store_true")
    p.add_argument("--no-tune", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-f32", action="store_true", help="batched: skip the float32-input measurement")
    p.add_argument("--no-extra-forms", action="store_true", help="batched: skip the plain-FP64 comparison")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-extra", action="store_true",
                   help="caqr: skip the fp64-form, TSQR-HR and precision-form legs")
    p.add_argument("--cpu-seconds", type=float, default=15.0)
    return p.parse_args()


_T0 = time.time()


def log(msg):
    """Progress on stderr (the JSON line alone goes to stdout)."""
    print(f"[bench {time.time() - _T0:7.1f}s] {msg}", file=sys.stderr, flush=True)


def flops(n):
    return 4.0 / 3.0 * float(n) ** 3


def qr_flops(m, n):
    return 2.0 * m * n * n - 2.0 / 3.0 * float(n) ** 3


# ----------------------------------------------------------------- inputs
def _preload_linalg():
    """torch loads its CUDA linear-algebra library lazily by bare name; load it
    by path first so the lookup also succeeds under a profiler's injection."""
    import ctypes

    import torch
    linalg = os.path.join(os.path.dirname(torch.__file__), "lib", "libtorch_cuda_linalg.so")
    if os.path.exists(linalg):
        ctypes.CDLL(linalg, mode=ctypes.RTLD_GLOBAL)


def haar_gpu(rng, rows, cols, device):
    """Haar-distributed orthonormal columns (rows x cols): Q diag(sign(diag R))
    of a Gaussian matrix drawn from rng (row-major draws), QR on the GPU."""
    import torch
    G = torch.from_numpy(rng.standard_normal((rows, cols))).to(device)
    Q, R = torch.linalg.qr(G)
    Q *= torch.sign(torch.diagonal(R))[None, :]
    del G, R
    return Q


def make_input_gpu(n, seed, sigma_min, device, m=None):
    """A = U diag(sigma) V^T (m x n, default square), U and V Haar from
    PCG64(seed) (U first), sigma log-spaced from 1 to sigma_min; column-major."""
    import torch
    _preload_linalg()
    m = m or n
    rng = np.random.default_rng(seed)
    U = haar_gpu(rng, m, n, device)
    V = haar_gpu(rng, n, n, device)
    s = torch.logspace(0, np.log10(sigma_min), n, dtype=torch.float64, device=device)
    A = (U * s[None, :]) @ V.t()
    del U, V
    torch.cuda.synchronize()
    return A.t().contiguous().t(), rng


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


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    return json.load(open(path)) if os.path.exists(path) else {}


def full_accuracy(cm, A0, YR, b, precision="fp64", cols=None, orth_cols=None, seed=0):
    """Backward error ||Q^T A0 - R||_F / ||A0||_F and orthogonality
    ||Q Q^T - I||_F of the factor held in YR, computed on the GPU.

    Q^T is applied panel by panel with update_A (T from Y^T Y, qr_2d.cxx:22-60)
    to [E | A0], E holding unit vectors, in the given arithmetic form: that
    gives rows of Q explicitly and Q^T A0 at once (the reference tests' two
    criteria, test_qr_2d.cxx:285-301 and test_bitree_tsqr.cxx:370-427).  By
    default over every column of A0 and every row of Q; with cols / orth_cols,
    over that many sampled columns of A0 / rows of Q (the Gram block of the
    sampled rows against I).  Q Q^T is formed in FP64.
    """
    import torch
    m, n = YR.shape
    rng = np.random.default_rng(seed)
    qrows = np.arange(m) if orth_cols is None else np.sort(rng.choice(m, size=orth_cols, replace=False))
    acols = np.arange(n) if cols is None else np.sort(rng.choice(n, size=cols, replace=False))
    nq, na = len(qrows), len(acols)
    dev_ = A0.device
    X = torch.zeros((nq + na, m), dtype=torch.float64, device=dev_).t()
    X[torch.from_numpy(qrows).to(dev_), torch.arange(nq, device=dev_)] = 1.0
    ac = torch.from_numpy(acols).to(dev_)
    X[:, nq:] = A0[:, ac]
    for r0 in range(0, min(m, n), b):
        bb = min(b, n - r0)
        cm.update_A(YR[r0:, r0:r0 + bb], X[r0:, :], bb, None, precision=precision)
    R = torch.triu(YR)[:, ac]
    bwd = float(torch.linalg.norm(X[:, nq:] - R) / torch.linalg.norm(A0[:, ac]))
    Qc = X[:, :nq]                      # Q^T e_j = row j of Q, as columns
    G = Qc.t() @ Qc
    G.diagonal().sub_(1.0)
    orth = float(torch.linalg.norm(G))
    del X, G
    torch.cuda.synchronize()
    return bwd, orth


class Ctx:
    """What every workload needs: the library, the device, the process group."""

    def __init__(self, args):
        import torch
        self.args = args
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        torch.cuda.set_device(self.local)
        self.dev = torch.device("cuda", self.local)
        self.dist = None
        if self.world > 1:
            import torch.distributed as dist
            dist.init_process_group("nccl", device_id=self.dev)
            self.dist = dist
        from candmc_gb300 import build as _build
        _build.build()
        import candmc_gb300 as cm
        from candmc_gb300 import _abi
        self.cm, self.abi, self.lib = cm, _abi, cm.lib()

    def barrier(self):
        if self.dist:
            self.dist.barrier()

    def max_over_ranks(self, x):
        if not self.dist:
            return x
        import torch
        t = torch.tensor([x], device=self.dev, dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def timed(self, step, steps, classes=(), flush=None):
        """Run `steps` steps inside the timed region: barrier + synchronize on
        both sides, CUDA events on the launching (current) stream, clocks
        sampled throughout, kernel classes timed live.  With `flush`, the L2
        flush runs before each step outside the per-step event pair."""
        import ctypes

        import torch
        mask = 0
        for c in classes:
            mask |= 1 << self.abi.KCLASS[c]
        self.barrier()
        torch.cuda.synchronize()
        clocks = ClockSampler(gpu_id_for_smi(self.local))
        l0 = self.lib.candmc_launch_count()
        self.lib.candmc_profile_begin(mask)
        if flush is None:
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(steps):
                step()
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1)
        else:
            pairs = []
            for _ in range(steps):
                flush()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record()
                step()
                e1.record()
                pairs.append((e0, e1))
            torch.cuda.synchronize()
            ms = sum(a.elapsed_time(b) for a, b in pairs)
        self.barrier()
        launches = self.lib.candmc_launch_count() - l0
        nc = self.abi.NKCLASS
        kms = (ctypes.c_double * nc)()
        kwork = (ctypes.c_double * nc)()
        kl = (ctypes.c_longlong * nc)()
        self.lib.candmc_profile_end(nc, kms, kwork, kl)
        clk = clocks.stop()
        prof = {c: (kms[self.abi.KCLASS[c]], kwork[self.abi.KCLASS[c]], kl[self.abi.KCLASS[c]])
                for c in classes}
        return self.max_over_ranks(ms), launches, prof, clk


def kernel_time_shares(ctx, step):
    """Share of each kernel class in the summed kernel time of one extra,
    untimed step profiled on every class (the normalisation of an ncu launch
    list, so the two can be compared)."""
    import ctypes

    import torch
    names = list(ctx.abi.KCLASS)
    mask = 0
    for c in names:
        mask |= 1 << ctx.abi.KCLASS[c]
    torch.cuda.synchronize()
    ctx.lib.candmc_profile_begin(mask)
    step()
    torch.cuda.synchronize()
    nc = ctx.abi.NKCLASS
    kms = (ctypes.c_double * nc)()
    kwork = (ctypes.c_double * nc)()
    kl = (ctypes.c_longlong * nc)()
    ctx.lib.candmc_profile_end(nc, kms, kwork, kl)
    tot = sum(kms[ctx.abi.KCLASS[c]] for c in names)
    return {c: kms[ctx.abi.KCLASS[c]] / tot for c in names if tot > 0}


def fp64_roof(prof, classes, kernel, step_ms):
    ms = sum(prof[c][0] for c in classes)
    work = sum(prof[c][1] for c in classes)
    launches = sum(prof[c][2] for c in classes)
    achieved = work / (ms / 1e3) / 1e12 if ms > 0 else None
    return {"bound": "fp64", "achieved": achieved, "peak": FP64_PEAK_GF / 1e3, "unit": "TFLOP/s",
            "frac": achieved / (FP64_PEAK_GF / 1e3) if achieved else None, "traffic": None,
            "kernel": kernel, "launches": launches, "share_of_step": ms / step_ms if step_ms else None,
            "peak_source": "DFMA microbenchmark on this GB300 (FP64 is not in MEASURED_PEAKS.json); "
                           "FP64 is neither the HBM nor the tensor roof"}


def base_line(args, ctx, metric, value, unit, ms_per_step, dtype, config, higher=True):
    return {"metric": metric, "value": value, "unit": unit, "n_gpus": ctx.world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": higher,
            "scaling": "weak", "vs_baseline": None, "dtype": dtype, "data": "synthetic", "config": config}


# ----------------------------------------------------------------- CPU legs
def _cpu_ls_task(task):
    """One least-squares problem by the reference call sequence, single BLAS
    thread (run inside a spawned worker); returns the solve's seconds."""
    m, n, seed = task
    from oracle import reference_lapack as rl
    rng = np.random.default_rng(seed)
    A = np.asfortranarray(rng.standard_normal((m, n)))
    b = rng.standard_normal((m, 1))
    t0 = time.perf_counter()
    rl.ls_solve_lapack(A, b, 128)
    return time.perf_counter() - t0


def cpu_ls_rate(tasks, seconds):
    """Solves/s of the reference call sequence over `tasks` (m, n, seed), one
    single-threaded process per host core, stopping after ~`seconds` of
    solve time per core; generation is excluded from the timed solves."""
    import multiprocessing as mp
    cores = os.cpu_count() or 1
    old = os.environ.get("OPENBLAS_NUM_THREADS")
    os.environ["OPENBLAS_NUM_THREADS"] = "1"
    try:
        with mp.get_context("spawn").Pool(cores) as pool:
            done, total = 0, 0.0
            it = pool.imap(_cpu_ls_task, tasks, chunksize=1)
            for dt in it:
                done += 1
                total += dt
                if total / cores >= seconds:
                    pool.terminate()
                    break
    finally:
        if old is None:
            os.environ.pop("OPENBLAS_NUM_THREADS", None)
        else:
            os.environ["OPENBLAS_NUM_THREADS"] = old
    return done / (total / cores), done, cores


def cpu_caqr_sample(A0h, b):
    """One full factorization of the same matrix by the reference's CPU path:
    the compiled reference (oracle/_ref) where it was built, else its LAPACK
    call sequence replayed on the same OpenBLAS (bitwise-equal to it;
    tests/test_oracle_ref.py).  Returns (seconds, kind, threads)."""
    from oracle import ref
    from oracle import reference_lapack as rl
    A = np.array(A0h, order="F")
    t0 = time.perf_counter()
    if ref.available():
        ref.QR_2D(A, b)
        kind = "reference"
    else:
        rl.QR_2D_lapack(A, b)
        kind = "port"
    return time.perf_counter() - t0, kind, rl.blas_threads()


def cpu_tsqr_hr(args, m, b, reps=None):
    from oracle import reference_lapack as rl
    A0 = np.asfortranarray(np.random.default_rng(0).standard_normal((m, b)))
    Af = A0.copy(order="F").reshape(-1, order="F")
    rl.hh_recon_qr_lapack(Af, m, 0, m, b)
    times = []
    t_end = time.perf_counter() + args.cpu_seconds
    while (reps is None and time.perf_counter() < t_end) or (reps is not None and len(times) < reps):
        Af = A0.copy(order="F").reshape(-1, order="F")
        t0 = time.perf_counter()
        rl.hh_recon_qr_lapack(Af, m, 0, m, b)
        times.append(time.perf_counter() - t0)
    return qr_flops(m, b) * len(times) / sum(times) / 1e9, len(times), rl.blas_threads()


# ----------------------------------------------------------------- reference arm
def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    world = int(os.environ.get("WORLD_SIZE", "1"))
    wl = args.workload
    line = {"impl": "reference", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "scaling": "weak", "vs_baseline": None, "data": "synthetic", "higher_is_better": True}
    if wl == "caqr":
        A0 = caqr_input_host(args)
        from oracle import ref
        from oracle import reference_lapack as rl
        use_ref = ref.available()
        nw = max(512, (args.n // 8) // args.b * args.b)
        for _ in range(args.warmup):      # warm-up: the leading block only (pages in, starts BLAS threads)
            W = np.array(A0[:nw, :nw], order="F")
            ref.QR_2D(W, args.b) if use_ref else rl.QR_2D_lapack(W, args.b)
        times = []
        for _ in range(args.steps):
            dt, kind, cores = cpu_caqr_sample(A0, args.b)
            times.append(dt)
            log(f"reference step {len(times)}: {dt:.1f} s")
        tot = sum(times)
        val = flops(args.n) * len(times) / tot / 1e12
        line.update({
            "metric": "CAQR TFLOP/s (FP64-equivalent, 4/3 n^3 per factorization)",
            "value": val, "unit": "TFLOP/s", "ms_per_step": 1e3 * tot / len(times), "dtype": "f64",
            "config": caqr_config(args),
            "cpu_baseline": {"value": val, "unit": "TFLOP/s", "cores": cores, "kind": kind,
                             "sample": f"{len(times)} full QR_2D factorizations of the same n={args.n} matrix "
                                       f"({'compiled reference' if kind == 'reference' else 'the reference call sequence replayed on the same OpenBLAS, bitwise-equal to the compiled reference'}); "
                                       f"warm-up steps factor the leading {nw} x {nw} block"}})
    elif wl == "tsqr_hr":
        gf, reps, cores = cpu_tsqr_hr(args, args.m, args.b, reps=args.warmup + args.steps)
        line.update({"metric": "TSQR-HR GFLOP/s (2mb^2 - 2/3 b^3 per panel)", "value": gf,
                     "unit": "GFLOP/s", "ms_per_step": qr_flops(args.m, args.b) / gf / 1e6, "dtype": "f64",
                     "config": {"workload": f"hh_recon_qr {args.m}x{args.b} N(0,1) seed 0"},
                     "cpu_baseline": {"value": gf, "unit": "GFLOP/s", "cores": cores, "kind": "port",
                                      "sample": f"hh_recon_qr_lapack x{reps}"}})
    elif wl in ("batched", "serve"):
        if wl == "batched":
            sizes = batched_sizes(args.count, seed=3)
            tasks = [(m, n, 1000 + i) for i, (m, n) in enumerate(sizes)]
            metric = "batched least squares solves/s"
        else:
            trace = serve_trace(args, args.count, max(float(r) for r in args.rates.split(",")))
            tasks = [(m, n, 2000 + i) for i, (_, m, n) in enumerate(trace)]
            metric = "least-squares requests solves/s (CPU per-request path)"
        rate, done, cores = cpu_ls_rate(tasks, args.cpu_seconds * max(1, args.steps))
        line.update({"metric": metric, "value": rate, "unit": "solves/s", "ms_per_step": 1e3 / rate,
                     "dtype": "f64", "config": {"workload": wl, "sample_problems": done},
                     "cpu_baseline": {"value": rate, "unit": "solves/s", "cores": cores, "kind": "port",
                                      "sample": f"first {done} problems of the workload, reference call "
                                                "sequence, one single-threaded process per core"}})
    else:
        print(json.dumps({"impl": "reference", "unavailable": f"no CPU reference arm for workload {wl}; "
                          "its CPU baseline is the caqr arm"}), flush=True)
        return 0
    line["e2e"] = {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0}
    print(json.dumps(line), flush=True)
    return 0


# ----------------------------------------------------------------- caqr (default)
def caqr_config(args):
    """The workload, identical in both arms (this one and --impl reference)."""
    return {"workload": f"CAQR n={args.n} b={args.b} float64, A=U diag(logspace(0,"
                        f"{np.log10(args.sigma_min):.0f},n)) V^T, U,V Haar (PCG64 seed {args.seed}, "
                        "QR of the Gaussian draws on the GPU)",
            "n": args.n, "b": args.b, "seed": args.seed, "sigma_min": args.sigma_min,
            "l2": f"input {8.0 * args.n * args.n / 2**30:.1f} GiB "
                  + ("> L2 129 MB, no flush needed" if 8.0 * args.n * args.n > 129e6 else "(< L2)")}


def caqr_input_host(args):
    """The benchmark matrix as a Fortran-ordered host array: the same bytes
    the GPU arm factors (generated on the GPU when one is present)."""
    try:
        import torch
        if torch.cuda.is_available():
            A0, _ = make_input_gpu(args.n, args.seed, args.sigma_min, torch.device("cuda", 0))
            h = np.asfortranarray(A0.cpu().numpy())
            del A0
            torch.cuda.empty_cache()
            return h
    except ImportError:
        pass
    from oracle import fixtures as fx
    return np.asfortranarray(fx.svd_matrix(args.n, args.n, args.seed, args.sigma_min))


def caqr_form_run(ctx, A0, A, b, form, entry, steps, warmup):
    """warm-up + timed factorizations of A0 (restored into A each step) in one form."""
    import torch
    cm = ctx.cm
    qr = cm.QR_2D_pipe if entry == "pipe" else cm.QR_2D

    def step():
        A.copy_(A0)
        qr(A, b, precision=form)

    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    dom = {"fp64": ["gemm_tn", "gemm_nn"], "ozaki": ["oz_tn", "oz_nn"], "fp32": ["f32"]}[form]
    t_max, launches, prof, clk = ctx.timed(step, steps, dom)
    return step, dom, t_max, launches, prof, clk


def wl_caqr(args, ctx):
    import torch
    cm = ctx.cm
    n, b, prec = args.n, args.b, args.form
    A0, _ = make_input_gpu(n, args.seed + ctx.rank * 1000 if ctx.world > 1 else args.seed,
                           args.sigma_min, ctx.dev)
    A = torch.empty_like(A0.t()).t()
    step, dom, t_max, launches, prof, clk = caqr_form_run(ctx, A0, A, b, prec, args.entry, args.steps,
                                                          args.warmup)
    value = ctx.world * flops(n) * args.steps / (t_max / 1e3) / 1e12
    dom_ms = sum(prof[c][0] for c in dom)
    dom_work = sum(prof[c][1] for c in dom)
    dom_l = sum(prof[c][2] for c in dom)
    achieved = dom_work / (dom_ms / 1e3) / 1e12 if dom_ms > 0 else None
    if prec == "ozaki":
        # Each FP64 product is emulated by 28 BF16 slice products (7 slices,
        # pairs i + j <= 6), so the emulated-FP64 roof is the BF16 roof / 28;
        # `achieved` counts algorithmic FP64 flops (2 m n k per contraction).
        pk_bf16 = measured_peaks().get("bf16_tflops_sustained", 1700.0)
        pk = pk_bf16 / 28.0
        roof = {"bound": "tensor", "achieved": achieved, "peak": pk, "unit": "TFLOP/s",
                "frac": achieved / pk if achieved else None,
                "bf16_issued_tflops": achieved * 28.0 if achieved else None,
                "traffic": traffic_from_profile("ozaki_gemm_caqr_n16384.md"),
                "kernel": "k_oz_mma (Ozaki BF16 slice contractions on tcgen05, Y^T A and A -= Y Z; "
                          "the b x b operator product T^T Z is counted under 'small')",
                "launches": dom_l, "share_of_step": dom_ms / t_max if t_max else None,
                "peak_source": "MEASURED_PEAKS.json bf16_tflops_sustained / 28 slice products "
                               "(of measured)"}
    elif prec == "fp32":
        # the FP32 form: 6 BF16 slice products (3 slices, pairs i + j <= 2)
        pk = measured_peaks().get("bf16_tflops_sustained", 1700.0) / 6.0
        roof = {"bound": "tensor", "achieved": achieved, "peak": pk, "unit": "TFLOP/s",
                "frac": achieved / pk if achieved else None, "traffic": None,
                "kernel": "k_oz_mma<., 3> (FP32 form: 3 BF16 slices on tcgen05)", "launches": dom_l,
                "share_of_step": dom_ms / t_max if t_max else None,
                "peak_source": "MEASURED_PEAKS.json bf16_tflops_sustained / 6 slice products (of measured)"}
    else:
        roof = fp64_roof(prof, dom, "k_gemm_f64 (Y^T A split-K partials and A -= Y Z)", t_max)
        roof["traffic"] = traffic_from_profile("gemm_f64_caqr_n16384.md")

    log(f"caqr {prec}: {t_max / args.steps:.1f} ms/step")
    shares = kernel_time_shares(ctx, step)
    roof["share_of_kernel_time"] = sum(shares.get(c, 0.0) for c in dom)
    # accuracy of the last timed factorization, over the whole matrix, checked in FP64
    bwd, orth = full_accuracy(cm, A0, A, b, precision="fp64")
    accuracy = {"backward_error": bwd, "orthogonality": orth, "bound": 1e-13,
                "how": "||Q^T A - R||_F/||A||_F and ||Q Q^T - I||_F over the whole matrix; Q^T applied "
                       "to [I | A] panel by panel in FP64 on the GPU, Q Q^T formed in FP64"}

    log(f"caqr accuracy: backward {bwd:.2e}, orthogonality {orth:.2e}")
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
        e2e = {"value": ctx.world * flops(n) * args.steps / tt / 1e12, "unit": "TFLOP/s",
               "h2d_bytes_per_step": 8 * n * n, "d2h_bytes_per_step": 8 * n * n,
               "entry": "candmc_QR_2D_host (host pointers: copy in, lookahead factorization, copy out)"}
        del src, work

    log("caqr e2e done")
    extra = {}
    if not args.no_extra and ctx.world == 1:
        extra["fp64_form"] = caqr_fp64_leg(args, ctx, A0, A)
        log("fp64 form leg done")
        extra["tsqr_hr"] = tsqr_hr_leg(args, ctx)
        log("tsqr_hr leg done")
        extra["forms"] = forms_leg(args, ctx)
        log("forms leg done")
        extra["batched"] = batched_leg(args, ctx)
        log("batched leg done")
        extra["serve"] = serve_leg(args, ctx)
        log("serve leg done")

    cpu = None
    if ctx.rank == 0 and ctx.world == 1 and not args.no_cpu:
        A0h = np.asfortranarray(A0.cpu().numpy())
        dt, kind, cores = cpu_caqr_sample(A0h, b)
        cpu = {"value": flops(n) / dt / 1e12, "unit": "TFLOP/s", "cores": cores, "kind": kind,
               "sample": f"one full QR_2D factorization of the same n={n} matrix ({dt:.1f} s; "
                         + ("compiled reference" if kind == "reference" else
                            "the reference's LAPACK call sequence replayed on the same OpenBLAS, "
                            "bitwise-equal to the compiled reference") + ")"}
        del A0h
        log("cpu baseline done")
    dtype = {"fp64": "f64", "ozaki": "f64 (emulated: bf16 Ozaki slices, fp32 accumulate)",
             "fp32": "f64 panels, fp32 trailing-update contractions"}[prec]
    line = base_line(args, ctx, "CAQR TFLOP/s (FP64-equivalent, 4/3 n^3 per factorization)", value,
                     "TFLOP/s", t_max / args.steps, dtype, caqr_config(args))
    line.update({"variant": {"form": prec, "entry": "QR_2D_pipe" if args.entry == "pipe" else "QR_2D",
                             "parallelism": f"replicas x{ctx.world}"},
                 "clocks": clk, "e2e": e2e, "gpu_launches": launches, "roofline": roof,
                 "cpu_baseline": cpu, "accuracy": accuracy})
    line.update(extra)
    return line


def caqr_fp64_leg(args, ctx, A0, A, steps=2, warmup=1):
    """The plain FP64 form on the same matrix: TFLOP/s and accuracy."""
    _, dom, t_max, launches, prof, clk = caqr_form_run(ctx, A0, A, args.b, "fp64", args.entry, steps, warmup)
    roof = fp64_roof(prof, dom, "k_gemm_f64", t_max)
    bwd, orth = full_accuracy(ctx.cm, A0, A, args.b, precision="fp64")
    return {"value": flops(args.n) * steps / (t_max / 1e3) / 1e12, "unit": "TFLOP/s", "steps": steps,
            "warmup": warmup, "ms_per_step": t_max / steps, "gpu_launches": launches,
            "dominant_kernel_fp64_frac": roof["frac"], "clocks": clk,
            "accuracy": {"backward_error": bwd, "orthogonality": orth, "how": "as the headline's"}}


# ----------------------------------------------------------------- tsqr_hr
def wl_tsqr_hr(args, ctx):
    import torch
    cm = ctx.cm
    m, b = args.m, args.b
    A0h = np.random.default_rng(0).standard_normal((m, b))
    A0 = cm.colmajor(torch.from_numpy(A0h).to(ctx.dev))
    A = cm.colmajor(A0.clone())
    W = cm.empty_colmajor(b, b, ctx.dev)
    T = cm.empty_colmajor(b, b, ctx.dev)
    flush_buf = torch.empty(512 << 20, dtype=torch.uint8, device=ctx.dev)   # 512 MB > L2

    def step():
        A.copy_(A0)
        cm.hh_recon_qr(A, W, T)

    def flush():
        flush_buf.add_(1)

    for _ in range(args.warmup):
        flush()
        step()
    torch.cuda.synchronize()
    classes = ["panel_leaf", "panel_y", "small", "gemm_tn", "gemm_nn", "reduce"]
    t_max, launches, prof, clk = ctx.timed(step, args.steps, classes, flush=flush)
    f = qr_flops(m, b)
    value = ctx.world * f * args.steps / (t_max / 1e3) / 1e9
    roof = fp64_roof(prof, ["panel_leaf", "panel_y"],
                     "k_hr6_pipe (pipelined TSQR tree) or k_hr4_leaf_tree, + k_hr4_form_y (reconstruction, Y)",
                     t_max)
    roof["traffic"] = traffic_from_profile("tsqr_hr_panel_8192x64.md")
    shares = kernel_time_shares(ctx, step)
    roof["share_of_kernel_time"] = shares.get("panel_leaf", 0.0) + shares.get("panel_y", 0.0)
    hbm = measured_peaks().get("hbm_gbs", 6778.0)
    bytes_alg = 16.0 * m * b
    roof["hbm"] = {"achieved_gbs": bytes_alg * args.steps / (t_max / 1e3) / 1e9, "peak_gbs": hbm,
                   "frac": bytes_alg * args.steps / (t_max / 1e3) / 1e9 / hbm,
                   "note": "algorithmic bytes 16 m b (read A, write Y) per step"}
    # accuracy of the last step
    Yh = A.cpu().numpy()
    Th = T.cpu().numpy()
    Y = np.tril(Yh, -1)
    Y[np.arange(b), np.arange(b)] = 1.0
    R = np.triu(Yh[:b])
    QR = np.vstack([R, np.zeros((m - b, b))])
    QR = QR - Y @ (Th @ (Y.T @ QR))
    bwd = float(np.linalg.norm(QR - A0h) / np.linalg.norm(A0h))
    E = np.eye(m, b) - Y @ (Th @ Y[:b].T)
    orth = float(np.linalg.norm(E.T @ E - np.eye(b)))

    e2e = None
    if not args.no_e2e:
        pin = torch.empty((b, m), dtype=torch.float64, pin_memory=True)
        hv = pin.numpy().T
        Wh = np.zeros((b, b), order="F")
        Th2 = np.zeros((b, b), order="F")
        tt, reps = 0.0, 0
        for it in range(args.warmup + max(args.steps, 20)):
            hv[:] = A0h
            t0 = time.perf_counter()
            cm.hh_recon_qr(hv, Wh, Th2)
            dt = time.perf_counter() - t0
            if it >= args.warmup:
                tt += dt
                reps += 1
        e2e = {"value": ctx.world * f * reps / tt / 1e9, "unit": "GFLOP/s",
               "h2d_bytes_per_step": 8 * m * b, "d2h_bytes_per_step": 8 * (m * b + 2 * b * b)}
    cpu = None
    if ctx.rank == 0 and ctx.world == 1 and not args.no_cpu:
        gf, reps, cores = cpu_tsqr_hr(args, m, b)
        cpu = {"value": gf, "unit": "GFLOP/s", "cores": cores, "kind": "port",
               "sample": f"hh_recon_qr call sequence (dgeqrf, dorgqr, signed LU, dtrsm) on {m}x{b}, "
                         f"{reps} runs in ~{args.cpu_seconds:.0f} s"}
    line = base_line(args, ctx, "TSQR-HR GFLOP/s (2mb^2 - 2/3 b^3 per panel)", value, "GFLOP/s",
                     t_max / args.steps, "f64",
                     {"workload": f"hh_recon_qr {m}x{b} float64 N(0,1) (PCG64 seed 0)", "m": m, "b": b,
                      "parallelism": f"replicas x{ctx.world}",
                      "l2": "512 MB buffer written between steps (input 4 MB < L2)"})
    line.update({"clocks": clk, "e2e": e2e, "gpu_launches": launches, "roofline": roof,
                 "cpu_baseline": cpu,
                 "accuracy": {"backward_error": bwd, "orthogonality": orth, "bound": 1e-13}})
    return line


# ----------------------------------------------------------------- forms
def wl_forms(args, ctx):
    import torch
    cm = ctx.cm
    m, n, b = args.m, args.n, args.b
    forms = [f for f in args.forms.split(",") if f]
    _preload_linalg()
    rng = np.random.default_rng(args.seed)
    U = haar_gpu(rng, m, n, ctx.dev)
    V = haar_gpu(rng, n, n, ctx.dev)
    B = cm.colmajor(torch.from_numpy(rng.standard_normal((m, 16))).to(ctx.dev))
    cases = []
    head = None
    total_launches = 0
    clk_all = []
    for smin in (1e-10, 1e-3):
        s = torch.logspace(0, np.log10(smin), n, dtype=torch.float64, device=ctx.dev)
        A0 = cm.colmajor((U * s[None, :]) @ V.t())
        A = torch.empty_like(A0.t()).t()
        # the FP64 oracle of the least-squares solutions: the plain FP64 form
        x64, st64 = cm.ls_solve(A0, B, b, precision="fp64", max_refine=20)
        r64 = float(torch.linalg.norm(B - A0 @ x64))
        for form in forms:
            _, dom, t_max, launches, prof, clk = caqr_form_run(ctx, A0, A, b, form, "pipe", args.steps,
                                                               args.warmup)
            total_launches += launches
            clk_all.append(clk)
            tf = qr_flops(m, n) * args.steps / (t_max / 1e3) / 1e12
            bwd, orth = full_accuracy(cm, A0, A, b, precision="fp64", cols=256, orth_cols=256)
            dom_ms = sum(prof[c][0] for c in dom)
            dom_tf = sum(prof[c][1] for c in dom) / (dom_ms / 1e3) / 1e12 if dom_ms else None
            # least squares, 16 right-hand sides, FP64 refinement
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            X, st = cm.ls_solve(A0, B, b, precision=form, max_refine=20)
            e1.record()
            torch.cuda.synchronize()
            ls_ms = e0.elapsed_time(e1)
            Rr = B - A0 @ X
            opt = float(torch.linalg.norm(A0.t() @ Rr) / (torch.linalg.norm(A0) * torch.linalg.norm(Rr)))
            rec = {"sigma_min": smin, "form": form, "qr_tflops": tf, "qr_ms": t_max / args.steps,
                   "dominant_kernel_tflops": dom_tf, "backward_error_256_cols": bwd,
                   "orthogonality_256_rows": orth,
                   "ls_ms": ls_ms, "refine_steps": st["steps"], "last_correction": st["last_change"],
                   "normal_eq_residual": opt,
                   "x_rel_diff_vs_fp64": float(torch.linalg.norm(X - x64) / torch.linalg.norm(x64)),
                   "resid_rel_diff_vs_fp64": abs(float(torch.linalg.norm(Rr)) - r64) / r64}
            cases.append(rec)
            if smin == 1e-10 and form == forms[0]:
                head = (tf, t_max / args.steps, form, prof, dom)
            del X, Rr
        del A0, A, x64
    tf, ms, form, prof, dom = head
    roof = None
    if form == "ozaki":
        pk = measured_peaks().get("bf16_tflops_sustained", 1700.0) / 28.0
        dom_ms = sum(prof[c][0] for c in dom)
        ach = sum(prof[c][1] for c in dom) / (dom_ms / 1e3) / 1e12 if dom_ms else None
        roof = {"bound": "tensor", "achieved": ach, "peak": pk, "unit": "TFLOP/s",
                "frac": ach / pk if ach else None, "traffic": None,
                "kernel": "k_oz_mma", "peak_source": "bf16_tflops_sustained / 28 (of measured)"}
    line = base_line(args, ctx, "CAQR TFLOP/s by precision form (FP64-equivalent, 2mn^2 - 2/3 n^3)",
                     tf * ctx.world, "TFLOP/s", ms, f"{form} trailing update, f64 panels",
                     {"workload": f"CAQR {m}x{n} b={b}, A=U diag(logspace(0,-10|-3,n)) V^T, U,V Haar "
                                  f"(PCG64 seed {args.seed}); LS with 16 N(0,1) RHS refined in FP64",
                      "m": m, "n": n, "b": b, "forms": forms, "headline": f"{form} at sigma_min 1e-10",
                      "l2": "input 4 GiB > L2"})
    line.update({"clocks": clk_all[0] if clk_all else None, "clocks_all": clk_all, "e2e": None,
                 "gpu_launches": total_launches, "roofline": roof, "cpu_baseline": None, "cases": cases,
                 "accuracy_how": "backward error ||Q^T A_S - R_S||_F/||A_S||_F over 256 sampled columns S "
                                 "and ||(Q Q^T - I)_RR||_F over 256 sampled rows R, Q^T applied in FP64; "
                                 "LS errors against the plain FP64 form's solution"})
    return line


def _sub_args(args, **kw):
    import copy
    a = copy.copy(args)
    for k, v in kw.items():
        setattr(a, k, v)
    return a


def tsqr_hr_leg(args, ctx):
    """TSQR-HR of the 8192 x 64 N(0,1) seed-0 panel, as `--workload tsqr_hr`."""
    a = _sub_args(args, m=8192, b=64, seed=0, steps=20, warmup=5, no_e2e=True, cpu_seconds=5.0)
    ln = wl_tsqr_hr(a, ctx)
    return {k: ln[k] for k in ("metric", "value", "unit", "steps", "warmup", "ms_per_step", "config",
                               "roofline", "accuracy", "cpu_baseline", "clocks", "gpu_launches")}


def batched_leg(args, ctx):
    """The 4096 uneven least-squares problems, as `--workload batched` with
    two timed steps (autotuned, CUDA-graph replay)."""
    a = _sub_args(args, count=4096, seed=3, steps=2, warmup=1, cpu_seconds=10.0)
    ln = wl_batched(a, ctx)
    return {k: ln[k] for k in ("metric", "value", "unit", "steps", "warmup", "ms_per_step", "config",
                               "roofline", "accuracy", "e2e", "cpu_baseline", "clocks", "gpu_launches",
                               "fp64_form", "float32_inputs")}


def serve_leg(args, ctx):
    """The request server under Poisson arrivals at 1k..50k requests/s, as
    `--workload serve` with 200 requests per rate."""
    a = _sub_args(args, count=200, seed=4, form="fp32", cpu_seconds=10.0)
    ln = wl_serve(a, ctx)
    return {k: ln[k] for k in ("metric", "value", "unit", "config", "latency", "fp64_per_request", "server",
                               "accuracy", "e2e", "cpu_baseline", "clocks", "gpu_launches")}


def forms_leg(args, ctx):
    """The precision forms at m = 32768, n = 16384 (seed 2), as `--workload forms`
    with two timed steps per form."""
    a = _sub_args(args, m=32768, n=16384, b=128, seed=2, steps=2, warmup=1, forms="ozaki,fp32")
    ln = wl_forms(a, ctx)
    return {k: ln[k] for k in ("metric", "value", "unit", "steps", "warmup", "ms_per_step", "config",
                               "roofline", "cases", "accuracy_how", "clocks", "gpu_launches")}


# ----------------------------------------------------------------- batched
def batched_sizes(count, seed=3, m_lo=256, m_hi=262144, widths=(8, 16, 32, 64, 128)):
    """(m_i, n_i) per problem: PCG64 streams from SeedSequence(seed).spawn(count),
    m_i = round(exp(U(ln m_lo, ln m_hi))), n_i uniform over widths, m_i >= n_i."""
    out = []
    for ss in np.random.SeedSequence(seed).spawn(count):
        r = np.random.default_rng(ss)
        m = int(round(np.exp(r.uniform(np.log(m_lo), np.log(m_hi)))))
        n = int(r.choice(widths))
        out.append((max(m, n), n))
    return out


def wl_batched(args, ctx):
    import torch
    cm = ctx.cm
    count = args.count
    sizes = batched_sizes(count, seed=3)
    al = 32                                     # 256-byte aligned problem starts
    offA, offB, ta, tb = [], [], 0, 0
    for m, n in sizes:
        offA.append(ta)
        offB.append(tb)
        ta += (m * n + al - 1) // al * al
        tb += (m + al - 1) // al * al
    g = torch.Generator(device=ctx.dev)
    g.manual_seed(3)
    A0 = torch.randn(ta, dtype=torch.float64, device=ctx.dev, generator=g)
    B0 = torch.randn(tb, dtype=torch.float64, device=ctx.dev, generator=g)
    Ap, Bp = A0.clone(), B0.clone()
    As = [Ap[o:o + m * n].view(n, m).t() for o, (m, n) in zip(offA, sizes)]
    Bs = [Bp[o:o + m].view(1, m).t() for o, (m, n) in zip(offB, sizes)]
    xidx = torch.cat([torch.arange(o, o + n) for o, (m, n) in zip(offB, sizes)]).to(ctx.dev)

    tuned = {"nstreams": 16, "leaf_rows": 64, "source": "default"}
    if not args.no_tune:
        from candmc_gb300 import autotune
        ns = min(512, count)

        def make_batch():
            sA = [a.clone().t().contiguous().t() for a in As[:ns]]
            sB = [bb.clone() for bb in Bs[:ns]]
            for a, o, (m, n) in zip(sA, offA, sizes):
                a.copy_(A0[o:o + m * n].view(n, m).t())
            for bb, o, (m, n) in zip(sB, offB, sizes):
                bb.copy_(B0[o:o + m].view(1, m).t())
            return sA, sB
        best, trials = autotune.tune_batched(make_batch, [m for m, _ in sizes[:ns]],
                                             [n for _, n in sizes[:ns]])
        tuned = dict(best, source=f"autotune on the first {ns} problems", trials=len(trials))
    cm.set_tuning("leaf_rows", tuned["leaf_rows"])
    use_graph = not args.no_graph

    def step():
        Ap.copy_(A0)
        Bp.copy_(B0)
        cm.batched_ls(As, Bs, nstreams=tuned["nstreams"], use_graph=use_graph)

    cm.batched_ls(As, Bs, nstreams=tuned["nstreams"])   # eager run first (kernel attributes)
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    classes = ["panel_leaf", "panel_y", "small", "gemm_tn", "gemm_nn", "reduce"]
    t_max, launches, prof, clk = ctx.timed(step, args.steps, classes)
    solves = ctx.world * count * args.steps / (t_max / 1e3)
    # plain FP64 beside the chosen form: the same problems with the panels'
    # half-panel updates on the FP64 pipe (batched_form 0)
    fp64_form = None
    if not args.no_extra_forms:
        cm.set_tuning("batched_form", 0)
        try:
            step()
            torch.cuda.synchronize()
            t64, l64, _, _ = ctx.timed(step, args.steps, [])
            fp64_form = {"value": ctx.world * count * args.steps / (t64 / 1e3), "unit": "solves/s",
                         "ms_per_step": t64 / args.steps, "gpu_launches": l64,
                         "form": "half-panel updates on the FP64 pipe (batched_form 0)"}
        finally:
            cm.set_tuning("batched_form", 1)
        step()                                   # the chosen form's result for the accuracy check
    f = sum(qr_flops(m, n) for m, n in sizes)
    by = sum(16.0 * m * n for m, n in sizes)
    roof = fp64_roof(prof, ["panel_leaf", "panel_y"], "k_hr6_pipe / k_hr4_leaf_tree + k_hr4_form_y", t_max)
    hbm = measured_peaks().get("hbm_gbs", 6778.0)
    roof["step_fp64_tflops"] = f * args.steps / (t_max / 1e3) / 1e12
    if roof["achieved"] is None:
        # graph replays bypass the per-launch timers: use the whole step
        roof["achieved"] = roof["step_fp64_tflops"]
        roof["frac"] = roof["achieved"] / roof["peak"]
        roof["note"] = ("CUDA-graph replay: per-class kernel timers do not fire; achieved = FP64 "
                        "flops (sum of 2 m n^2 - 2/3 n^3) over the whole step")
    roof["hbm"] = {"achieved_gbs": by * args.steps / (t_max / 1e3) / 1e9, "peak_gbs": hbm,
                   "frac": by * args.steps / (t_max / 1e3) / 1e9 / hbm,
                   "note": "algorithmic bytes 16 m n per problem (read A, write Y)"}
    # accuracy on a sample of problems against LAPACK lstsq (numpy), and no
    # device-side failure recorded by the batched calls
    torch.cuda.synchronize()
    cm.batched_status()
    rs = np.random.default_rng(0)
    small = [i for i, (m, n) in enumerate(sizes) if m <= 65536]
    errs = []
    for i in rs.choice(small, size=min(12, len(small)), replace=False):
        m, n = sizes[i]
        Ah = A0[offA[i]:offA[i] + m * n].view(n, m).t().cpu().numpy()
        bh = B0[offB[i]:offB[i] + m].cpu().numpy()
        xo = np.linalg.lstsq(Ah, bh, rcond=None)[0]
        x = Bp[offB[i]:offB[i] + n].cpu().numpy()
        errs.append(float(np.linalg.norm(x - xo) / np.linalg.norm(xo)))

    e2e = None
    if not args.no_e2e:
        try:
            hA = torch.empty(ta, dtype=torch.float64, pin_memory=True)
            hB = torch.empty(tb, dtype=torch.float64, pin_memory=True)
            hA.copy_(A0)
            hB.copy_(B0)
            hx = torch.empty(xidx.numel(), dtype=torch.float64, pin_memory=True)
            tt = 0.0
            for it in range(1 + args.steps):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                Ap.copy_(hA, non_blocking=True)
                Bp.copy_(hB, non_blocking=True)
                cm.batched_ls(As, Bs, nstreams=tuned["nstreams"], use_graph=use_graph)
                hx.copy_(Bp[xidx], non_blocking=True)
                torch.cuda.synchronize()
                if it >= 1:
                    tt += time.perf_counter() - t0
            e2e = {"value": ctx.world * count * args.steps / tt, "unit": "solves/s",
                   "h2d_bytes_per_step": 8 * (ta + tb), "d2h_bytes_per_step": 8 * xidx.numel()}
            del hA, hB
        except RuntimeError as ex:
            e2e = {"value": None, "unit": "solves/s", "h2d_bytes_per_step": 8 * (ta + tb),
                   "d2h_bytes_per_step": 8 * xidx.numel(), "error": str(ex)[:200]}
    f32 = None
    if not args.no_f32:
        del As, Bs, Ap, Bp                       # the FP64 copies: room for the float32 run's work area
        torch.cuda.empty_cache()
        f32 = batched_f32_inputs(args, ctx, sizes, A0, B0, offA, offB, ta, tb, tuned, use_graph)
    cpu = None
    if ctx.rank == 0 and ctx.world == 1 and not args.no_cpu:
        tasks = [(m, n, 1000 + i) for i, (m, n) in enumerate(sizes)]
        rate, done, cores = cpu_ls_rate(tasks, args.cpu_seconds)
        cpu = {"value": rate, "unit": "solves/s", "cores": cores, "kind": "port",
               "sample": f"first {done} problems (same size distribution), reference call sequence "
                         "(hh_recon_qr + update_A on [A|b] + dtrsm), one single-threaded process per core"}
    line = base_line(args, ctx, "batched least squares solves/s", solves, "solves/s", t_max / args.steps,
                     "f64",
                     {"workload": f"{count} LS problems, m log-uniform [256, 262144], n in "
                                  "{8,16,32,64,128}, A,b ~ N(0,1) on the device (Philox seed 3)",
                      "problems": count, "tuning": tuned, "graph": use_graph,
                      "form": "half-panel updates and Gram products of panels >= 8192 rows in emulated FP64 on tcgen05 "
                              "(batched_form 1), everything else FP64",
                      "l2": f"inputs {8 * ta / 1e9:.0f} GB > L2"})
    line.update({"clocks": clk, "e2e": e2e, "gpu_launches": launches, "roofline": roof, "cpu_baseline": cpu,
                 "accuracy": {"x_rel_err_vs_lstsq_max": max(errs) if errs else None, "sampled": len(errs),
                              "bound": 1e-12},
                 "fp64_form": fp64_form, "float32_inputs": f32})
    return line


def batched_f32_inputs(args, ctx, sizes, A0, B0, offA, offB, ta, tb, tuned, use_graph):
    """The same problems stored as float32 (A0, B0 rounded), solved by
    batched_ls_f32 (widened to FP64 on the device, FP64 solve, x rounded to
    float32): device-resident solves/s, and end to end with the float32 inputs
    copied from pinned host memory each step (half the FP64 host traffic)."""
    import torch
    cm = ctx.cm
    count = len(sizes)
    A32 = torch.empty(ta, dtype=torch.float32, device=ctx.dev)
    B32 = torch.empty(tb, dtype=torch.float32, device=ctx.dev)
    A32.copy_(A0)
    As = [A32[o:o + m * n].view(n, m).t() for o, (m, n) in zip(offA, sizes)]
    Bs = [B32[o:o + m].view(1, m).t() for o, (m, n) in zip(offB, sizes)]
    xidx = torch.cat([torch.arange(o, o + n) for o, (m, n) in zip(offB, sizes)]).to(ctx.dev)

    def step():
        B32.copy_(B0)
        cm.batched_ls_f32(As, Bs, nstreams=tuned["nstreams"], use_graph=use_graph)

    step()                                        # grows the FP64 work area
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    t_max, launches, _, _ = ctx.timed(step, args.steps, [])
    out = {"value": ctx.world * count * args.steps / (t_max / 1e3), "unit": "solves/s",
           "ms_per_step": t_max / args.steps, "gpu_launches": launches}
    torch.cuda.synchronize()
    cm.batched_status()
    rs = np.random.default_rng(1)
    small = [i for i, (m, n) in enumerate(sizes) if m <= 65536]
    errs = []
    for i in rs.choice(small, size=min(8, len(small)), replace=False):
        m, n = sizes[i]
        Ah = A32[offA[i]:offA[i] + m * n].view(n, m).t().double().cpu().numpy()
        bh = B0[offB[i]:offB[i] + m].float().double().cpu().numpy()
        xo = np.linalg.lstsq(Ah, bh, rcond=None)[0]
        x = B32[offB[i]:offB[i] + n].double().cpu().numpy()
        errs.append(float(np.linalg.norm(x - xo) / np.linalg.norm(xo)))
    out["accuracy"] = {"x_rel_err_vs_lstsq_of_the_float32_data_max": max(errs) if errs else None,
                       "sampled": len(errs), "bound": 2e-7}
    if not args.no_e2e:
        try:
            hA = torch.empty(ta, dtype=torch.float32, pin_memory=True)
            hB = torch.empty(tb, dtype=torch.float32, pin_memory=True)
            hA.copy_(A32)
            hB.copy_(B0)
            hx = torch.empty(xidx.numel(), dtype=torch.float32, pin_memory=True)
            tt = 0.0
            for it in range(1 + args.steps):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                A32.copy_(hA, non_blocking=True)
                B32.copy_(hB, non_blocking=True)
                cm.batched_ls_f32(As, Bs, nstreams=tuned["nstreams"], use_graph=use_graph)
                hx.copy_(B32[xidx], non_blocking=True)
                torch.cuda.synchronize()
                if it >= 1:
                    tt += time.perf_counter() - t0
            out["e2e"] = {"value": ctx.world * count * args.steps / tt, "unit": "solves/s",
                          "h2d_bytes_per_step": 4 * (ta + tb), "d2h_bytes_per_step": 4 * xidx.numel()}
            del hA, hB
        except RuntimeError as ex:
            out["e2e"] = {"value": None, "error": str(ex)[:200]}
    del A32, B32
    return out


# ----------------------------------------------------------------- serve
def serve_trace(args, count, rate):
    from candmc_gb300.serve import poisson_trace
    return poisson_trace(count, rate, seed=4, m_lo=512, m_hi=1048576, widths=(16, 32, 64, 128, 256))


def wl_serve(args, ctx):
    import torch
    cm = ctx.cm
    from candmc_gb300.serve import LSServer, latency_summary, replay
    M, N = 1048576, 256
    ss = np.random.SeedSequence(4).spawn(3)
    pools = []
    for k in range(2):
        t = torch.empty((N, M), dtype=torch.float64, pin_memory=True)
        np.random.default_rng(ss[k]).standard_normal(out=t.numpy())
        pools.append(t.numpy().T)                # Fortran view M x N
    tb = torch.empty(M, dtype=torch.float64, pin_memory=True)
    np.random.default_rng(ss[2]).standard_normal(out=tb.numpy())
    bpool = tb.numpy()

    def inputs(i, m, n):
        return pools[i % 2][:m, :n], bpool[:m]

    rates = [float(r) for r in args.rates.split(",")]
    budget = args.budget_gb * 1e9
    form = args.form
    results = []
    clk, launches = None, 0
    with LSServer(budget_bytes=budget, workers=args.workers, precision=form) as srv:
        warm = serve_trace(args, 24, 1e6)
        replay(srv, warm, inputs)
        for k, rate in enumerate(rates):
            trace = serve_trace(args, args.count, rate)
            torch.cuda.synchronize()
            sampler = ClockSampler(gpu_id_for_smi(ctx.local)) if k == len(rates) - 1 else None
            l0 = ctx.lib.candmc_launch_count()
            xs, infos = replay(srv, trace, inputs)
            launches += ctx.lib.candmc_launch_count() - l0
            if sampler:
                clk = sampler.stop()
            summ = latency_summary(infos)
            summ["rate"] = rate
            summ["peak_in_flight"] = srv.stats()["peak_in_flight"]
            results.append(summ)
        st = srv.stats()
    # accuracy on sampled requests of the last trace against LAPACK lstsq (numpy)
    errs = []
    for i, (_, m, n) in enumerate(trace):
        if m <= 65536 and len(errs) < 12:
            A, bvec = inputs(i, m, n)
            xo = np.linalg.lstsq(np.asarray(A), bvec, rcond=None)[0]
            errs.append(float(np.linalg.norm(xs[i] - xo) / np.linalg.norm(xo)))
    # plain FP64 per-request path on the same (highest-rate) trace
    with LSServer(budget_bytes=budget, workers=1, precision="fp64") as srv:
        replay(srv, serve_trace(args, 8, 1e6), inputs)
        _, infos64 = replay(srv, trace, inputs)
    base = latency_summary(infos64)
    cpu = None
    if ctx.rank == 0 and ctx.world == 1 and not args.no_cpu:
        tasks = [(m, n, 2000 + i) for i, (_, m, n) in enumerate(trace)]
        rate, done, cores = cpu_ls_rate(tasks, args.cpu_seconds)
        cpu = {"value": rate, "unit": "solves/s", "cores": cores, "kind": "port",
               "sample": f"first {done} requests of the trace, reference call sequence, one "
                         "single-threaded process per core (throughput only)"}
    top = results[-1]
    mean_in = float(np.mean([8.0 * (m * n + m) for _, m, n in trace]))
    mean_out = float(np.mean([8.0 * n for _, m, n in trace]))
    line = base_line(args, ctx, "least-squares requests solves/s (continuous batching, refined to 1e-12)",
                     top["solves_per_s"] * ctx.world, "solves/s", 1e3 / top["solves_per_s"],
                     f"{form} trailing update, f64 panels and refinement",
                     {"workload": "Poisson arrivals (seed 4), m log-uniform [512, 1048576], n in "
                                  "{16,32,64,128,256}, A,b ~ N(0,1) host buffers",
                      "requests_per_rate": args.count, "rates": rates, "workers": args.workers,
                      "budget_gb": args.budget_gb, "form": form})
    line.update({"clocks": clk, "gpu_launches": launches,
                 "e2e": {"value": top["solves_per_s"] * ctx.world, "unit": "solves/s",
                         "h2d_bytes_per_step": mean_in, "d2h_bytes_per_step": mean_out,
                         "note": "every request is copied in from host memory and x copied back"},
                 "latency": results, "fp64_per_request": base,
                 "server": {"peak_bytes_reserved": st["peak_bytes_reserved"],
                            "peak_in_flight": st["peak_in_flight"]},
                 "roofline": None, "cpu_baseline": cpu,
                 "accuracy": {"x_rel_err_vs_lstsq_max": max(errs) if errs else None, "sampled": len(errs),
                              "bound": 1e-12}})
    return line


# ----------------------------------------------------------------- main
DEFAULTS = {
    "caqr": {"n": 16384, "b": 128, "form": "ozaki", "seed": 1},
    "tsqr_hr": {"m": 8192, "b": 64, "seed": 0},
    "forms": {"m": 32768, "n": 16384, "b": 128, "seed": 2, "form": "ozaki"},  # --forms ozaki,fp32
    "batched": {"count": 4096, "seed": 3},
    "serve": {"count": 400, "form": "fp32", "seed": 4},
}


def main():
    args = parse()
    for k, v in DEFAULTS[args.workload].items():
        if getattr(args, k) is None:
            setattr(args, k, v)
    if args.b is None:
        args.b = 128
    if args.form is None:
        args.form = "ozaki"
    if args.impl == "reference":
        return run_reference(args)
    ctx = Ctx(args)
    fn = {"caqr": wl_caqr, "tsqr_hr": wl_tsqr_hr, "forms": wl_forms, "batched": wl_batched,
          "serve": wl_serve}[args.workload]
    line = fn(args, ctx)
    if ctx.rank == 0:
        print(json.dumps(line), flush=True)
    if ctx.dist:
        ctx.dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
