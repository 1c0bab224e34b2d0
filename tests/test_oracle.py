"""Pins the oracle (CPU restatement) before anything is checked against it.

Anchors: libc's srand48/drand48 (the reference fixture generator), LAPACK
itself via scipy (the library holding all of the reference's arithmetic),
the committed golden vectors, and the reference tests' own pass criteria
(test/QR/test_hh_recon.cxx:251-264, test_qr_2d.cxx:285-301,
test_bitree_tsqr.cxx:370-451, test_construct_tsqr_Q.cxx:168-191).
"""
import ctypes

import numpy as np
import pytest

from oracle import candmc_oracle as co
from oracle import fixtures as fx
from oracle import lapack_restated as lp
from oracle import reference_lapack as rl
from tests.golden.make_golden import PANELS, panel_input


def test_drand48_matches_libc():
    libc = ctypes.CDLL("libc.so.6")
    libc.drand48.restype = ctypes.c_double
    seeds = [0, 1, 99900, 99900 + 61 * 12345, 2**33 + 17, 99900 + 61 * (34 * 17 - 1)]
    want = []
    for s in seeds:
        libc.srand48(ctypes.c_long(s))
        want.append(libc.drand48())
    got = fx.drand48_first(seeds)
    assert np.array_equal(np.array(want), got)


@pytest.mark.parametrize("name,m,b,gen", PANELS)
def test_hh_recon_matches_golden(golden, name, m, b, gen):
    i = [p[0] for p in PANELS].index(name)
    A = panel_input(m, b, gen, 100 + i)
    YR, W = co.hh_recon_qr(A, b)
    scale = np.abs(golden[name + "/YR"]).max()
    assert np.abs(YR - golden[name + "/YR"]).max() <= 1e-12 * scale * max(1, b / 16)
    assert np.abs(W - golden[name + "/W"]).max() <= 1e-12 * max(1, b / 16)
    T = co.T_from_W(W, lp.unit_lower(YR, b)[:b])
    assert np.abs(T - golden[name + "/T"]).max() <= 1e-12 * max(1, b / 16)
    tau = co.tau_recon_lower(YR, b)
    assert np.abs(tau - golden[name + "/tau"]).max() <= 1e-13


@pytest.mark.parametrize("m,b,p", [(34, 17, 1), (68, 17, 2), (136, 17, 4), (168, 21, 8), (96, 32, 3), (512, 64, 4)])
def test_hh_recon_reference_criterion(m, b, p):
    """test_hh_recon: sum_j ||(A-QR)e_j||/||Ae_j|| <= 1e-9 for any process count."""
    A = fx.drand48_fixture(m, b)
    YR, W = co.hh_recon_qr(A, b, numPes=p)
    assert co.column_relative_residual(A, YR, b) <= 1e-9
    assert co.orthogonality_error(YR, b) <= 1e-6
    # canonical output: independent of the process count
    YR1, W1 = co.hh_recon_qr(A, b, numPes=1)
    assert np.abs(YR - YR1).max() <= 1e-12 * max(1, b / 8)
    assert np.abs(W - W1).max() <= 1e-12 * max(1, b / 8)


@pytest.mark.parametrize("m,b,p", [(42, 21, 1), (84, 21, 2), (168, 21, 4), (336, 21, 8)])
def test_bitree_and_construct_Q1_criteria(m, b, p):
    """test_bitree_tsqr / test_construct_tsqr_Q: ||QQ^T-I||, ||QR-A|| <= 1e-6.

    The element-wise |R| = |R_lapack| check of test_bitree_tsqr.cxx:438-451 is
    commented out in the reference; it is applied here where the fixture has
    full numerical rank (the 42 x 21 and 84 x 21 fixtures do not)."""
    A = fx.drand48_fixture(m, b)
    blocks, order = co.split_rows(A, b, p) if p > 1 else ([A.copy()], [0])
    R, taus, tree = co.bitree_tsqr(blocks, b)
    Q1 = co.join_rows(co.construct_Q1(blocks, taus, tree, b, b), order) if p > 1 else \
        co.construct_Q1(blocks, taus, tree, b, b)[0]
    assert np.linalg.norm(Q1.T @ Q1 - np.eye(b)) <= 1e-6
    assert np.linalg.norm(Q1 @ R - A) <= 1e-6
    Rl = np.triu(np.linalg.qr(A, mode="r"))
    if np.linalg.svd(A, compute_uv=False)[-1] < 1e-8:
        return
    assert np.abs(np.abs(R) - np.abs(Rl)).max() <= 1e-6 * max(1.0, np.abs(Rl).max())


def test_lapack_restatement_against_scipy():
    from scipy.linalg import lapack
    A = fx.gaussian(300, 70, 0)
    qr, tau, _, info = lapack.dgeqrf(A.copy())
    B = A.copy()
    t = lp.dgeqrf(B)
    assert np.abs(B - qr).max() < 1e-12 and np.abs(t - tau).max() < 1e-14
    Q, _, info = lapack.dorgqr(qr, tau)
    Q2 = lp.dorg2r(qr.copy(), tau)
    assert np.abs(Q - Q2).max() < 1e-13
    R1 = np.triu(fx.gaussian(24, 24, 1))
    R2 = np.triu(fx.gaussian(24, 24, 2))
    r1, r2, t, info = lapack.dtpqrt(24, 24, R1.copy(), R2.copy())
    a, bb = R1.copy(), R2.copy()
    tau2 = lp.dtpqrt_tri(a, bb)
    assert np.abs(np.triu(a) - np.triu(r1)).max() < 1e-12
    assert np.abs(np.triu(bb) - np.triu(r2)).max() < 1e-12
    assert np.abs(tau2 - np.diag(t)).max() < 1e-13


def test_upd_A_matches_dormqr(golden):
    for i, (name, m, b, gen) in enumerate(PANELS):
        YR = golden[name + "/YR"]
        C = fx.gaussian(m, 16, 200 + i)
        Y = lp.unit_lower(YR, b)
        out = co.upd_A(Y, C.copy(), W=golden[name + "/W"])
        assert np.abs(out - golden[name + "/QtC"]).max() <= 1e-12 * max(1, b / 8) * np.abs(C).max()
        out2 = co.upd_A(Y, C.copy(), W=None)
        assert np.abs(out2 - golden[name + "/QtC"]).max() <= 1e-12 * max(1, b / 8) * np.abs(C).max()


def test_QR_2D_golden_and_criterion(golden):
    A = fx.gaussian(192, 96, 7)
    A0 = A.copy()
    co.QR_2D(A, 16)
    assert np.abs(A - golden["qr2d_192x96_b16/YR"]).max() <= 1e-11
    assert co.backward_error(A0, A) <= 1e-13


@pytest.mark.parametrize("m,k,b", [(8, 4, 2), (64, 64, 16), (96, 64, 16), (40, 40, 8)])
def test_QR_2D_reference_criterion_rank_deficient_fixture(m, k, b):
    """test_qr_2d fixture (drand48 - 0.5) is numerically rank-deficient at these shapes;
    the reference's own check is backward error, which must still hold."""
    A = fx.drand48_fixture(m, k, offset=0.5)
    A0 = A.copy()
    co.QR_2D(A, b)
    assert co.column_relative_residual(A0, A, k) <= 1e-9 if m > k else True
    assert co.backward_error(A0, A) <= 1e-13


@pytest.mark.parametrize("m,n,b", [(600, 200, 64), (300, 300, 32), (1000, 130, 128)])
def test_ls_oracle_matches_lapack_lstsq(m, n, b):
    """The least-squares oracle (QR_2D on [A | B] + back substitution) against LAPACK's gelsd."""
    A = fx.gaussian(m, n, m + n)
    B = fx.gaussian(m, 3, 2)
    X = co.ls_solve(A, B, b)
    Xl = np.linalg.lstsq(A, B, rcond=None)[0]
    assert np.abs(X - Xl).max() <= 1e-12 * max(1.0, np.abs(Xl).max())


def test_invT_identities(golden):
    name, m, b = "hh_384x64", 384, 64
    YR, W, T = golden[name + "/YR"], golden[name + "/W"], golden[name + "/T"]
    Y = lp.unit_lower(YR, b)
    X1 = co.compute_invT_from_W(W, Y[:b])
    X2 = co.compute_invT_from_Y(Y)
    Xt = np.linalg.inv(T).T
    assert np.abs(X1 - Xt).max() < 1e-10
    assert np.abs(X2 - Xt).max() < 1e-10


@pytest.mark.parametrize("m,n,b", [(600, 200, 64), (2000, 256, 128), (1000, 130, 128)])
def test_reference_call_sequence_ls_matches_oracle(m, n, b):
    """The LAPACK replay of the reference's calls (hh_recon_qr + update_A on
    [A | B] + dtrsm), used as the CPU baseline of the least-squares
    workloads, agrees with the restated oracle and with LAPACK's lstsq."""
    A = fx.gaussian(m, n, 3 * m + n)
    B = fx.gaussian(m, 2, 5)
    X = rl.ls_solve_lapack(A, B, b)
    Xo = co.ls_solve(A, B, b)
    Xl = np.linalg.lstsq(A, B, rcond=None)[0]
    scale = max(1.0, np.abs(Xl).max())
    assert np.abs(X - Xo).max() <= 1e-12 * scale
    assert np.abs(X - Xl).max() <= 1e-12 * scale
