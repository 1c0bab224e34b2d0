"""Least-squares request server on the GPU: continuous batching, admission by
device-memory budget, arrival order, and results that do not depend on what
else is in flight.

Tolerances: x within 1e-12 relative of LAPACK's lstsq for these
well-conditioned Gaussian problems; results of a request alone and in a mix
must be bitwise equal (the kernels a request launches depend only on its own
sizes and data)."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 1e-12


@pytest.fixture(scope="module")
def cm():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import candmc_gb300 as cm
    cm.lib()
    return cm


def inputs_for(trace, seed=11):
    ss = np.random.SeedSequence(seed).spawn(len(trace))
    out = []
    for (_, m, n), s in zip(trace, ss):
        rng = np.random.default_rng(s)
        out.append((np.asfortranarray(rng.standard_normal((m, n))), rng.standard_normal(m)))
    return out


def lstsq_err(A, b, x):
    xo = np.linalg.lstsq(A, b, rcond=None)[0]
    return np.linalg.norm(x - xo) / np.linalg.norm(xo)


@pytest.mark.parametrize("form", ["fp32", "fp64"])
def test_mix_equals_alone(cm, form):
    from candmc_gb300.serve import LSServer, poisson_trace, replay
    trace = poisson_trace(20, rate=1e5, seed=4, m_lo=512, m_hi=60000, widths=(16, 64, 128, 200))
    data = inputs_for(trace)
    with LSServer(budget_bytes=40e9, workers=6, precision=form) as srv:
        xs_mix, infos = replay(srv, trace, lambda i, m, n: data[i])
        st = srv.stats()
    assert st["peak_in_flight"] > 1, st          # requests really overlapped
    assert st["bytes_reserved"] == 0 and st["completed"] == len(trace)
    with LSServer(budget_bytes=40e9, workers=1, precision=form) as srv:
        for (A, b), x_mix in zip(data, xs_mix):
            x_alone, _ = srv.result(srv.submit(A, b))
            assert np.array_equal(x_alone, x_mix)
            assert lstsq_err(A, b, x_alone) <= TOL
    for d in infos:
        assert d["status"] == 0 and d["refine_steps"] >= 1


def test_admission_respects_budget(cm):
    from candmc_gb300.serve import LSServer
    m, n = 200000, 64
    rng = np.random.default_rng(5)
    data = [(np.asfortranarray(rng.standard_normal((m, n))), rng.standard_normal(m)) for _ in range(6)]
    est = cm.lib().candmc_ls_request_bytes(m, n, 128, 2)
    budget = 2.5 * est                            # room for two at a time
    with LSServer(budget_bytes=budget, workers=6, precision="fp32") as srv:
        tickets = [srv.submit(A, b) for A, b in data]
        res = [srv.result(t) for t in tickets]
        st = srv.stats()
    assert st["peak_in_flight"] <= 2 and st["peak_bytes_reserved"] <= budget, st
    for (A, b), (x, _) in zip(data, res):
        assert lstsq_err(A, b, x) <= TOL


def test_oversized_request_rejected(cm):
    from candmc_gb300.serve import LSServer
    A = np.asfortranarray(np.random.default_rng(1).standard_normal((100000, 64)))
    b = np.ones(100000)
    with LSServer(budget_bytes=64 << 20, workers=2) as srv:
        t = srv.submit(A, b)
        with pytest.raises(cm.CandmcError) as ei:
            srv.result(t)
        assert ei.value.status == 2


def test_arrival_order_and_times(cm):
    from candmc_gb300.serve import LSServer, poisson_trace, replay
    trace = poisson_trace(30, rate=300.0, seed=7, m_lo=512, m_hi=20000, widths=(16, 32, 64))
    data = inputs_for(trace, seed=12)
    with LSServer(budget_bytes=8e9, workers=4, precision="fp32") as srv:
        xs, infos = replay(srv, trace, lambda i, m, n: data[i])
    admits = [d["admit"] for d in infos]
    assert all(a2 >= a1 for a1, a2 in zip(admits, admits[1:]))      # FIFO admission
    for d in infos:
        assert d["admit"] >= d["arrival"] - 1e-4 and d["done"] >= d["admit"]
    for (A, b), x in zip(data, xs):
        assert lstsq_err(A, b, x) <= TOL


@pytest.mark.parametrize("m,n,form", [(4096, 16, "fp32"), (300000, 128, "fp32"), (150000, 256, "fp32"),
                                      (150000, 256, "ozaki"), (70000, 256, "fp64")])
def test_request_bytes_bound_measured_use(cm, m, n, form):
    """The admission estimate covers the device pool's measured high-water of one solve."""
    from candmc_gb300.serve import LSServer
    lib = cm.lib()
    rng = np.random.default_rng(3)
    A = np.asfortranarray(rng.standard_normal((m, n)))
    b = rng.standard_normal(m)
    torch.cuda.synchronize()
    with LSServer(budget_bytes=100e9, workers=1, precision=form) as srv:
        hw = ctypes.c_uint64()
        cm.check(lib.candmc_mem_high_water(1, ctypes.byref(hw)), "high water")
        base = hw.value
        x, d = srv.result(srv.submit(A, b))
        cm.check(lib.candmc_mem_high_water(0, ctypes.byref(hw)), "high water")
    used = hw.value - base
    assert used <= d["bytes"], (used, d["bytes"])
    assert lstsq_err(A, b, x) <= TOL
