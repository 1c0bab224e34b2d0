"""Batched uneven least squares (TSQR-HR per problem, concurrent streams,
optional CUDA-graph replay) against the least-squares oracle / LAPACK.

Tolerance: x_i within 1e-12 relative of LAPACK's lstsq for these
well-conditioned Gaussian problems (the FP64-class 1e-12 bar)."""
import numpy as np
import pytest

from oracle import fixtures as fx

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


def make(problems):
    host = []
    for (m, n, rng) in problems:
        A = rng.standard_normal((m, n))
        b = rng.standard_normal((m, 1))
        host.append((A, b))
    return host


def to_dev(host):
    As = [torch.from_numpy(np.asfortranarray(A)).cuda().t().contiguous().t() for A, _ in host]
    Bs = [torch.from_numpy(np.asfortranarray(b)).cuda().t().contiguous().t() for _, b in host]
    return As, Bs


def check(host, xs):
    import candmc_gb300 as cm
    cm.batched_status()   # no device-side failure was recorded
    for (A, b), x in zip(host, xs):
        xo = np.linalg.lstsq(A, b, rcond=None)[0]
        err = np.linalg.norm(x.cpu().numpy() - xo) / np.linalg.norm(xo)
        assert err <= TOL, err


def test_batched_eager_uneven(cm):
    host = make(fx.batched_problems(48, seed=3, m_lo=128, m_hi=8192))
    As, Bs = to_dev(host)
    xs = cm.batched_ls(As, Bs, nstreams=8)
    torch.cuda.synchronize()
    check(host, xs)


def test_batched_graph_capture_and_replay(cm):
    host = make(fx.batched_problems(24, seed=5, m_lo=256, m_hi=4096))
    As, Bs = to_dev(host)
    A0 = [a.clone() for a in As]
    B0 = [b.clone() for b in Bs]
    cm.batched_ls(As, Bs, nstreams=4)      # eager run sets kernel attributes
    torch.cuda.synchronize()
    for rep in range(2):                   # capture, then replay on restored inputs
        for a, a0 in zip(As, A0):
            a.copy_(a0)
        for bb, b0 in zip(Bs, B0):
            bb.copy_(b0)
        l0 = cm.lib().candmc_launch_count()
        xs = cm.batched_ls(As, Bs, nstreams=4, use_graph=True)
        torch.cuda.synchronize()
        assert cm.lib().candmc_launch_count() - l0 >= 3 * len(host)   # replays count their kernels
        check(host, xs)


def test_batched_rejects_wide_problem(cm):
    A = torch.zeros((200, 129), dtype=torch.float64, device="cuda").t().contiguous().t()
    b = torch.zeros((200, 1), dtype=torch.float64, device="cuda")
    with pytest.raises(cm.CandmcError):
        cm.batched_ls([A], [b])


@pytest.mark.parametrize("m_lo,m_hi", [(2048, 16384), (160, 2000)])
def test_leaf_rows_tuning_keeps_results(cm, m_lo, m_hi):
    # (160, 2000): leaves of 129..224 rows, whose row slots round up to the 8-slot factor
    host = make(fx.batched_problems(12, seed=9, m_lo=m_lo, m_hi=m_hi, widths=(8, 32, 64, 128)))
    for leaf in (64, 96, 256):
        cm.set_tuning("leaf_rows", leaf)
        As, Bs = to_dev(host)
        xs = cm.batched_ls(As, Bs, nstreams=4)
        torch.cuda.synchronize()
        check(host, xs)
    cm.set_tuning("leaf_rows", 64)


@pytest.mark.parametrize("use_graph", [False, True])
def test_batched_float32_inputs(cm, use_graph):
    """The float32-input variant: A_i, b_i stored as float32, solved in FP64;
    x_i (rounded to float32) within float32 rounding of LAPACK's solution of
    the same float32 data in float64, and A_i left as it was."""
    host = make(fx.batched_problems(40, seed=7, m_lo=128, m_hi=8192))
    host32 = [(A.astype(np.float32), b.astype(np.float32)) for A, b in host]
    As = [torch.from_numpy(np.asfortranarray(A)).cuda().t().contiguous().t() for A, _ in host32]
    Bs = [torch.from_numpy(np.asfortranarray(b)).cuda().t().contiguous().t() for _, b in host32]
    A_before = [a.clone() for a in As]
    for _ in range(2):     # twice: the graph path captures, then replays
        for b, (_, bh) in zip(Bs, host32):
            b.copy_(torch.from_numpy(np.asfortranarray(bh)).cuda())
        xs = cm.batched_ls_f32(As, Bs, nstreams=8, use_graph=use_graph)
        torch.cuda.synchronize()
        cm.batched_status()
        for (A, b), x in zip(host32, xs):
            xo = np.linalg.lstsq(A.astype(np.float64), b.astype(np.float64), rcond=None)[0]
            err = np.linalg.norm(x.cpu().numpy().astype(np.float64) - xo) / np.linalg.norm(xo)
            assert err <= 2e-7, err
    for a, a0 in zip(As, A_before):
        assert torch.equal(a, a0)


@pytest.mark.parametrize("form", [0, 1])
def test_batched_panel_forms(cm, form):
    """batched_form 1 (the default): the panels' half-panel updates in emulated
    FP64 on the tensor cores for panels of at least panel_oz_min_rows rows;
    batched_form 0: on the FP64 pipe.  Same 1e-12 bar for both."""
    host = make(fx.batched_problems(24, seed=9, m_lo=2048, m_hi=65536))
    As, Bs = to_dev(host)
    try:
        cm.set_tuning("batched_form", form)
        cm.set_tuning("panel_oz_min_rows", 1024)
        xs = cm.batched_ls(As, Bs, nstreams=8)
        torch.cuda.synchronize()
    finally:
        cm.set_tuning("batched_form", 1)
        cm.set_tuning("panel_oz_min_rows", 8192)
    check(host, xs)
