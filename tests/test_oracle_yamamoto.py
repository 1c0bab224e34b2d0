"""The Yamamoto restatement (alg/QR/hh_recon/yamamoto.cxx, alg/QR/qr_2d/qr_y2d.cxx)
pinned to the Householder-reconstruction oracle, which the LAPACK fixtures pin:

* I + Qm W Qm^T is the Householder Q^T of the same panel, and S*R is the
  reconstruction's;
* Qm = Y W_hr S (the representation is the reconstruction's up to the signs);
* QR_Yamamoto_2D and QR_Yamamoto_2D_2D leave QR_2D's R and Y;
* the aggregator's I + aQm aT aQm^T applies the panels in order.
"""
import numpy as np
import pytest

from oracle import candmc_oracle as co
from oracle import fixtures as fx
from oracle import lapack_restated as lp
from oracle import yamamoto_oracle as yo

TOL = 1e-13


@pytest.mark.parametrize("m,b", [(64, 16), (300, 32), (257, 17)])
def test_yamamoto_panel_is_the_householder_q(m, b):
    A = fx.gaussian(m, b, m + b)
    YR, Qm, W, s = yo.Yamamoto(A, b)
    YRh, Wh = co.hh_recon_qr(A, b)
    Y = lp.unit_lower(YRh, b)
    T = co.T_from_W(Wh, Y[:b, :b])
    scale = np.abs(A).max()
    assert np.abs(Qm @ W @ Qm.T + Y @ T.T @ Y.T).max() <= TOL * 10
    assert np.abs(np.triu(YR[:b]) - np.triu(YRh[:b])).max() <= TOL * scale * 10
    assert np.abs(Qm - Y @ Wh @ np.diag(s)).max() <= TOL * 10
    # Qm's top block is Q1 - S with the sign choice of the unpivoted LU
    assert set(np.unique(s)) <= {-1, 1}
    # (I + Qm W Qm^T) A = [S R; 0]
    QA = A + Qm @ (W @ (Qm.T @ A))
    R = np.triu(YR[:b])
    assert np.abs(QA[:b] - R).max() <= TOL * scale * 10
    assert np.abs(QA[b:]).max() <= TOL * scale * 10


def test_recursive_ylu_matches_unblocked():
    rng = np.random.default_rng(4)
    Q = np.linalg.qr(rng.standard_normal((300, 150)))[0]
    A1 = Q[:150, :150].copy()
    A2 = A1.copy()
    s1 = np.zeros(150, dtype=np.int64)
    yo.signed_YLU(A1, s1)
    s2 = yo.recursive_YLU(A2)
    assert np.array_equal(s1, s2)
    assert np.abs(A1 - A2).max() <= 1e-12


@pytest.mark.parametrize("compute_Y", [False, True])
def test_qr_yamamoto_2d_leaves_qr_2d_factors(compute_Y):
    A = fx.gaussian(200, 150, 7)
    ref = A.copy()
    co.QR_2D(ref, 32)
    out = A.copy()
    yo.QR_Yamamoto_2D(out, 32, compute_Y=compute_Y)
    scale = np.abs(A).max()
    assert np.abs(np.triu(out[:150]) - np.triu(ref[:150])).max() <= 1e-12 * scale * 10
    assert np.abs(np.tril(out, -1) - np.tril(ref, -1)).max() <= 1e-12


@pytest.mark.parametrize("b,b_sub", [(64, 32), (96, 32)])
def test_qr_yamamoto_2d_2d_leaves_qr_2d_factors(b, b_sub):
    A = fx.gaussian(220, 190, 11)
    ref = A.copy()
    co.QR_2D(ref, b_sub)
    out = A.copy()
    yo.QR_Yamamoto_2D_2D(out, b, b_sub, compute_Y=True)
    scale = np.abs(A).max()
    assert np.abs(np.triu(out[:190]) - np.triu(ref[:190])).max() <= 1e-12 * scale * 10
    assert np.abs(np.tril(out, -1) - np.tril(ref, -1)).max() <= 1e-12


def test_aggregator_applies_the_panels_in_order():
    m, k, b = 160, 96, 32
    A = fx.gaussian(m, k, 21)
    agg = yo.Aggregator(m, k)
    out = A.copy()
    yo.QR_Yamamoto_2D(out, b, agg=agg)
    assert agg.n == k and agg.shift == k - b
    # block lower triangular kernel, each panel's Qm at its row offset
    assert np.abs(np.triu(agg.aT, 1)[:b, b:]).max() == 0.0
    assert np.abs(agg.aQm[:b, b:]).max() == 0.0
    QA = A + agg.aQm @ (agg.aT @ (agg.aQm.T @ A))
    R = np.triu(out[:k])
    scale = np.abs(A).max()
    assert np.abs(QA[:k] - R).max() <= 1e-12 * scale * 10
    assert np.abs(QA[k:]).max() <= 1e-12 * scale * 10


def test_upd_yamamoto_a_is_the_kernel_update():
    A = fx.gaussian(120, 24, 3)
    YR, Qm, W, s = yo.Yamamoto(A, 24)
    C = fx.gaussian(120, 40, 5)
    ref = C + Qm @ W @ Qm.T @ C
    out = yo.upd_Yamamoto_A(Qm, C.copy(), W)
    assert np.abs(out - ref).max() <= 1e-12 * np.abs(C).max()
