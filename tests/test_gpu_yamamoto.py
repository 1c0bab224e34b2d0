"""Yamamoto's basis-kernel representation on the GPU against the oracle
(oracle/yamamoto_oracle.py, which restates alg/QR/hh_recon/yamamoto.cxx and
alg/QR/qr_2d/qr_y2d.cxx and is pinned to the Householder oracle).

The representation is defined up to the column signs of the TSQR basis: the
GPU returns Qm = Qm_ref S_ref and W = S_ref W_ref S_ref for the oracle's sign
matrix S_ref, recovered here column by column.  S*R, Y, Qm W Qm^T and every
update agree with the oracle.  Tolerances: 1e-12 relative for FP64 work
(the factorizations' own backward error bound is 1e-13 of ||A||), 1e-11 for
the emulated-FP64 update.
"""
import numpy as np
import pytest

from oracle import fixtures as fx
from oracle import yamamoto_oracle as yo

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cm():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import candmc_gb300 as cm
    cm.lib()
    return cm


def dev(x):
    return torch.from_numpy(np.asfortranarray(x)).cuda().t().contiguous().t()


def host(x):
    torch.cuda.synchronize()
    return x.cpu().numpy()


def col_signs(ours, ref):
    return np.where(np.sum(ours * ref, axis=0) >= 0, 1.0, -1.0)


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("m,b", [(64, 16), (300, 32), (500, 17), (2048, 64), (4096, 128)])
def test_yamamoto_panel(cm, m, b):
    A = fx.gaussian(m, b, 3 * m + b)
    YR, Qm_r, W_r, s_r = yo.Yamamoto(A, b)
    dA = dev(A)
    Qm, W = cm.Yamamoto(dA)
    out, Qm, W = host(dA), host(Qm), host(W)
    # S*R and Y are canonical
    assert rel(np.triu(out[:b]), np.triu(YR[:b])) <= 1e-12
    assert np.abs(np.tril(out, -1) - np.tril(YR, -1)).max() <= 1e-12
    # the pair up to the reference's signs, which are the oracle's LU signs
    d = col_signs(Qm, Qm_r)
    assert np.array_equal(d, s_r.astype(np.float64))
    assert rel(Qm * d, Qm_r) <= 1e-12
    assert rel(d[:, None] * W * d[None, :], W_r) <= 1e-12
    # the operator itself
    assert rel(Qm @ W @ Qm.T, Qm_r @ W_r @ Qm_r.T) <= 1e-12


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("ozaki", 1e-11)])
def test_upd_yamamoto_a(cm, precision, tol):
    m, b, k = 1024, 64, 300
    A = fx.gaussian(m, b, 5)
    _, Qm, W, _ = yo.Yamamoto(A, b)
    C = fx.gaussian(m, k, 6)
    ref = yo.upd_Yamamoto_A(Qm, C.copy(), W)
    dC = dev(C)
    cm.upd_Yamamoto_A(dev(Qm), dC, dev(W), precision=precision)
    assert rel(host(dC), ref) <= tol


@pytest.mark.parametrize("compute_Y", [False, True])
@pytest.mark.parametrize("precision", ["fp64", "ozaki"])
def test_qr_yamamoto_2d(cm, compute_Y, precision):
    m, k, b = 600, 400, 64
    A = fx.gaussian(m, k, 9)
    ref = A.copy()
    yo.QR_Yamamoto_2D(ref, b, compute_Y=compute_Y)
    dA = dev(A)
    cm.QR_Yamamoto_2D(dA, b, compute_Y=compute_Y, precision=precision)
    out = host(dA)
    scale = np.abs(A).max()
    assert np.abs(np.triu(out[:k]) - np.triu(ref[:k])).max() <= 1e-11 * scale
    assert np.abs(np.tril(out, -1) - np.tril(ref, -1)).max() <= 1e-11


@pytest.mark.parametrize("b,b_sub", [(128, 32), (96, 32)])
def test_qr_yamamoto_2d_2d(cm, b, b_sub):
    m, k = 700, 500
    A = fx.gaussian(m, k, 13)
    ref = A.copy()
    yo.QR_Yamamoto_2D_2D(ref, b, b_sub, compute_Y=True)
    dA = dev(A)
    cm.QR_Yamamoto_2D_2D(dA, b, b_sub, compute_Y=True)
    out = host(dA)
    scale = np.abs(A).max()
    assert np.abs(np.triu(out[:k]) - np.triu(ref[:k])).max() <= 1e-11 * scale
    assert np.abs(np.tril(out, -1) - np.tril(ref, -1)).max() <= 1e-11


def test_aggregator_matches_oracle(cm):
    m, k, b = 400, 96, 32
    A = fx.gaussian(m, k, 17)
    ragg = yo.Aggregator(m, k)
    ref = A.copy()
    yo.QR_Yamamoto_2D(ref, b, agg=ragg)
    agg = cm.Aggregator(m, k)
    dA = dev(A)
    cm.QR_Yamamoto_2D(dA, b, agg=agg)
    aQm, aT = host(agg.aQm), host(agg.aT)
    assert (agg.n, agg.shift) == (ragg.n, ragg.shift)
    d = col_signs(aQm, ragg.aQm)
    assert rel(aQm * d, ragg.aQm) <= 1e-12
    assert rel(d[:, None] * aT * d[None, :], ragg.aT) <= 1e-12
    # the aggregated operator reduces A to R
    QA = A + aQm @ (aT @ (aQm.T @ A))
    R = np.triu(host(dA)[:k])
    assert np.abs(QA[:k] - R).max() <= 1e-12 * np.abs(A).max()
    assert np.abs(QA[k:]).max() <= 1e-12 * np.abs(A).max()


def test_aggregator_too_small_is_rejected(cm):
    A = dev(fx.gaussian(200, 96, 19))
    agg = cm.Aggregator(200, 64)   # room for two 32-column panels, not three
    with pytest.raises(cm.CandmcError):
        cm.QR_Yamamoto_2D(A, 32, agg=agg)
    torch.cuda.synchronize()


def test_block_not_multiple_of_panel_is_rejected(cm):
    A = dev(fx.gaussian(200, 150, 23))
    with pytest.raises(cm.CandmcError):
        cm.QR_Yamamoto_2D_2D(A, 96, 40)
