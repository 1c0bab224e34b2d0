"""Least-squares request server (continuous batching on one GPU).

`LSServer` wraps the native server of include/candmc_gb300.h
(candmc_server_*): worker threads with one CUDA stream each admit requests in
arrival order while their device-memory estimates fit in the budget, solve
them concurrently (candmc_ls_solve: CAQR in the chosen form, FP64 Q^T b and
FP64 refinement, with A, Y\\R, T and R resident across the refinement) and
copy each x back to host memory.

`poisson_trace` makes the seeded open-loop arrival trace a load test replays:
exponential inter-arrival gaps at rate `rate` (requests/s), m log-uniform in
[m_lo, m_hi], n uniform over `widths`.  `replay` submits a whole trace with
its arrival times, waits for every result and returns the per-request
timings; latency = completion - arrival, so time spent queued behind a busy
GPU or a full memory budget counts.
"""
import ctypes

import numpy as np

from . import PRECISIONS, _prec, lib
from ._abi import CandmcError, check


class LSServer:
    def __init__(self, budget_bytes=120e9, workers=8, precision="fp32", b=128, max_refine=20,
                 tol=1e-15):
        self._lib = lib()
        h = ctypes.c_void_p()
        check(self._lib.candmc_server_create(float(budget_bytes), int(workers), _prec(precision),
                                             int(b), int(max_refine), float(tol), ctypes.byref(h)),
              "candmc_server_create")
        self._h = h
        self._held = {}
        self.b = b
        self.precision = precision

    def now(self):
        """Seconds on the server clock."""
        return self._lib.candmc_server_now(self._h)

    def request_bytes(self, m, n):
        return int(self._lib.candmc_ls_request_bytes(m, n, self.b, PRECISIONS[self.precision]
                                                     if isinstance(self.precision, str)
                                                     else int(self.precision)))

    def submit(self, A, bvec, arrival=None):
        """Queue min ||A x - b||.  A: float64 host array (m x n) in column-major
        layout (a Fortran-ordered array or a column slice of one), bvec: (m,).
        arrival: earliest admission time on the server clock (None: now).
        Returns a ticket.  The arrays are held until `result` collects it."""
        A = np.asarray(A)
        if A.dtype != np.float64 or A.ndim != 2:
            raise ValueError("A must be a 2-D float64 array")
        if A.strides[0] != 8:
            A = np.asfortranarray(A)
        m, n = A.shape
        lda = A.strides[1] // 8 if n > 1 else m
        bvec = np.ascontiguousarray(np.asarray(bvec, dtype=np.float64).reshape(-1))
        if bvec.shape[0] != m:
            raise ValueError("b must have m entries")
        x = np.empty(n, dtype=np.float64)
        t = ctypes.c_int64(-1)
        st = self._lib.candmc_server_submit(self._h, A.ctypes.data, lda, m, n, bvec.ctypes.data,
                                            x.ctypes.data, -1.0 if arrival is None else float(arrival),
                                            ctypes.byref(t))
        if t.value < 0:
            check(st, "candmc_server_submit")
        self._held[t.value] = (A, bvec, x)
        return t.value

    def result(self, ticket, timeout=None):
        """(x, info) of a request; raises CandmcError if it failed, TimeoutError
        if it has not completed within `timeout` seconds."""
        info = (ctypes.c_double * 8)()
        st = self._lib.candmc_server_wait(self._h, int(ticket), -1.0 if timeout is None else float(timeout),
                                          info)
        if st == 4 and info[0] == 0 and info[3] == 0:
            raise TimeoutError(f"request {ticket} not finished")
        A, bvec, x = self._held.pop(ticket)
        d = {"status": int(info[0]), "arrival": info[1], "admit": info[2], "done": info[3],
             "refine_steps": int(info[4]), "last_correction": info[5], "bytes": int(info[6]),
             "worker": int(info[7])}
        if st != 0:
            raise CandmcError(st, f"request {ticket}")
        return x, d

    def stats(self):
        out = (ctypes.c_double * 8)()
        check(self._lib.candmc_server_stats(self._h, out), "candmc_server_stats")
        keys = ("bytes_reserved", "peak_bytes_reserved", "completed", "in_flight", "peak_in_flight",
                "pending", "budget", "workers")
        return dict(zip(keys, list(out)))

    def close(self):
        if self._h:
            self._lib.candmc_server_destroy(self._h)
            self._h = None
            self._held.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def poisson_trace(count, rate, seed=4, m_lo=512, m_hi=1048576, widths=(16, 32, 64, 128, 256)):
    """[(arrival_s, m, n)] for `count` requests of a Poisson process at `rate`/s.
    One PCG64(seed) stream draws, per request in order: the exponential gap,
    then u ~ U(ln m_lo, ln m_hi) (m = round(exp(u))), then n from `widths`."""
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    for _ in range(count):
        t += rng.exponential(1.0 / rate)
        m = int(round(np.exp(rng.uniform(np.log(m_lo), np.log(m_hi)))))
        n = int(rng.choice(widths))
        out.append((t, max(m, n), n))
    return out


def replay(server, trace, inputs, start_delay=0.05):
    """Submit every request of `trace` at its arrival time (offset by the
    server clock now + start_delay) and collect all results.
    inputs(i, m, n) -> (A, b) host arrays of request i.
    Returns (xs, infos) in trace order."""
    t0 = server.now() + start_delay
    tickets = []
    for i, (ta, m, n) in enumerate(trace):
        A, bvec = inputs(i, m, n)
        tickets.append(server.submit(A, bvec, arrival=t0 + ta))
    xs, infos = [], []
    for tk in tickets:
        x, d = server.result(tk)
        d["arrival"] -= t0
        d["admit"] -= t0
        d["done"] -= t0
        xs.append(x)
        infos.append(d)
    return xs, infos


def latency_summary(infos):
    lat = np.array([d["done"] - d["arrival"] for d in infos])
    first = min(d["arrival"] for d in infos)
    last = max(d["done"] for d in infos)
    return {"requests": len(infos), "solves_per_s": len(infos) / (last - first),
            "p50_ms": 1e3 * float(np.percentile(lat, 50)), "p99_ms": 1e3 * float(np.percentile(lat, 99)),
            "mean_queue_ms": 1e3 * float(np.mean([d["admit"] - d["arrival"] for d in infos]))}
