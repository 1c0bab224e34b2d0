"""Pins the oracle to the reference's own code.

Two anchors:
1. tests/golden/ref_golden.npz, written by tests/golden/make_ref_golden.py
   from the reference's QR sources compiled unmodified (oracle/build_ref.py:
   single-rank MPI, scipy's OpenBLAS).  These tests run everywhere: the
   restatement in oracle/ must reproduce every stored reference output.
2. The compiled reference itself (oracle/_ref), where it was built: the
   restatement on further shapes, and the replay in oracle/reference_lapack.py
   (the CPU baseline on hosts without the reference build) bitwise against it.

Tolerance: the outputs are the canonical Householder factor (Y, T, S*R), so
two FP64 implementations agree to a few ulps times the panel width relative
to the largest entry (TOL * max(1, b/16)); the C2-type input (singular values
down to 1e-6) is compared with a tolerance scaled by its condition number.
"""
import os

import numpy as np
import pytest

from oracle import candmc_oracle as co
from oracle import fixtures as fx
from oracle import lapack_restated as lp
from oracle import ref
from oracle import reference_lapack as rl
from oracle import yamamoto_oracle as yo
from tests.golden.make_ref_golden import C1_ROWS, CAQR, PANELS, panel_input, tree_input

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TOL = 2e-12
live = pytest.mark.skipif(not ref.available(), reason="oracle/_ref (the compiled reference) not built here")


@pytest.fixture(scope="module")
def rg():
    return np.load(os.path.join(ROOT, "tests", "golden", "ref_golden.npz"))


def close(got, want, b, scale=None, k=1.0):
    scale = np.abs(want).max() if scale is None else scale
    err = np.abs(np.asarray(got) - want).max()
    assert err <= k * TOL * max(1.0, b / 16) * max(1.0, scale), err


@pytest.mark.parametrize("name,m,b,gen,seed", PANELS)
def test_hh_recon_oracle_is_the_reference(rg, name, m, b, gen, seed):
    YR, W = co.hh_recon_qr(panel_input(m, b, gen, seed), b)
    close(YR, rg[f"hh/{name}/YR"], b)
    close(np.triu(W), np.triu(rg[f"hh/{name}/W"]), b)


def test_c1_panel_oracle_is_the_reference(rg):
    """8192 x 64, N(0,1) from seed 0 (the TSQR-HR benchmark panel)."""
    A = fx.gaussian(8192, 64, 0)
    YR, W = co.hh_recon_qr(A, 64)
    close(np.triu(YR[:64]), rg["c1/R"], 64)
    close(np.triu(W), np.triu(rg["c1/W"]), 64)
    assert np.array_equal(rg["c1/rows"], C1_ROWS)
    close(YR[C1_ROWS], rg["c1/Yrows"], 64)


@pytest.mark.parametrize("name,m,k,b,variant,b_sub,seed", CAQR)
def test_caqr_oracle_is_the_reference(rg, name, m, k, b, variant, b_sub, seed):
    A = np.asfortranarray(fx.gaussian(m, k, seed))
    co.QR_2D(A, b_sub or b)
    close(A, rg[f"qr2d/{name}/YR"], b, k=4.0)


def test_c2_type_caqr_oracle_is_the_reference(rg):
    """U diag(logspace(0,-6)) V^T, 256 x 256, b = 128, QR_2D_pipe."""
    A = np.array(rg["c2/A"], order="F")
    co.QR_2D(A, 128)
    want = rg["c2/YR"]
    # R is held element-wise; the reflectors of the trailing columns are
    # sensitive to rounding by up to kappa * u, so Y is held to that.
    close(np.triu(A), np.triu(want), 128)
    assert np.abs(np.tril(A, -1) - np.tril(want, -1)).max() <= 1e6 * 1e-15
    assert co.backward_error(rg["c2/A"], want) <= 1e-14


@pytest.mark.parametrize("b", [17, 32, 64])
def test_tree_tsqr_oracle_is_the_reference(rg, b):
    """dtpqrt on [R1; R2] (bitree_tsqr.cxx:20-34): R over V, the T blocks, and
    the strictly-lower parts of both blocks left as they were."""
    S = tree_input(b, 300 + b)
    out, T = rg[f"tree/{b}/out"], rg[f"tree/{b}/T"]
    assert np.array_equal(np.tril(out[:b], -1), np.tril(S[:b], -1))
    assert np.array_equal(np.tril(out[b:], -1), np.tril(S[b:], -1))
    R1, R2 = np.triu(S[:b]), np.triu(S[b:])
    tau = lp.dtpqrt_tri(R1, R2)
    close(np.triu(out[:b]), np.triu(R1), b)
    close(np.triu(out[b:]), np.triu(R2), b)
    close(T, lp.dtpqrt_T(R2, tau, min(b, 16)), b)


def test_single_rank_tsqr_oracle_is_the_reference(rg):
    """bitree_tsqr, construct_Q1 and apply_tsqr_QT at one rank."""
    A = fx.gaussian(256, 32, 400)
    YR = np.array(A, order="F")
    tau = lp.dgeqrf(YR)
    close(YR, rg["tsqr/YR"], 32)
    close(tau, rg["tsqr/tau"], 32)
    close(np.triu(YR[:32]), rg["tsqr/R"], 32)
    Q = np.array(YR, order="F")
    close(lp.dorg2r(Q, tau), rg["tsqr/Q1"], 32)
    B = fx.gaussian(256, 8, 401)
    close(co.apply_tsqr_QT(YR, tau, B, 32), rg["tsqr/QtB"], 32)


def test_tau_recon_oracle_is_the_reference(rg):
    YRh, _ = co.hh_recon_qr(fx.gaussian(256, 32, 406), 32)
    close(co.tau_recon("L", YRh), rg["tau/L"], 32)
    close(co.tau_recon("U", np.triu(rg["tree/32/out"][32:])), rg["tau/U"], 32)
    close(co.tau_recon("R", YRh[32:]), rg["tau/R"], 32)
    close(co.tau_recon_lower(lp.unit_lower(YRh, 32), 32, lapack_zero=True), rg["tau/L"], 32)


def test_yamamoto_oracle_is_the_reference(rg):
    A = fx.gaussian(256, 32, 402)
    YR, Qm, W, s = yo.Yamamoto(A, 32)
    close(YR, rg["yam/A"], 32)
    close(Qm, rg["yam/Qm"], 32)
    close(W, rg["yam/W"], 32, k=10.0)


def test_T_forms_oracle_are_the_reference(rg):
    YRh, Wh = co.hh_recon_qr(fx.gaussian(256, 32, 403), 32)
    Y = lp.unit_lower(YRh, 32)
    close(co.compute_invT_from_W(Wh, Y[:32]), rg["invT/fromW"], 32)
    close(np.tril(co.compute_invT_from_Y(Y)), np.tril(rg["invT/fromY"]), 32)
    close(co.compute_invT_from_Y2(Y[:, :16], Y[:, 16:]), rg["invT/fromY2"], 32)
    C = fx.gaussian(256, 48, 404)
    close(co.upd_A(Y, C.copy(), Wh), rg["upd/W"], 32)
    close(co.upd_A(Y, C.copy(), None), rg["upd/noW"], 32)


def test_yamamoto_caqr_oracle_is_the_reference(rg):
    A = np.array(fx.gaussian(192, 96, 405), order="F")
    yo.QR_Yamamoto_2D(A, 32, compute_Y=True)
    close(A, rg["yam2d/YR"], 32, k=4.0)


# ---- against the compiled reference, where it exists ----------------------
@live
def test_fixtures_are_the_reference_build(rg):
    """The committed fixtures are what the reference built here returns."""
    for name, m, b, gen, seed in PANELS[:5]:
        YR, W = ref.hh_recon_qr(panel_input(m, b, gen, seed), b)
        assert np.array_equal(YR, rg[f"hh/{name}/YR"])
    name, m, k, b, variant, b_sub, seed = CAQR[0]
    assert np.array_equal(ref.QR_2D(fx.gaussian(m, k, seed), b, variant, b_sub), rg[f"qr2d/{name}/YR"])


@live
@pytest.mark.parametrize("m,k,b", [(256, 256, 32), (768, 512, 128), (1024, 1024, 128), (1000, 600, 100)])
def test_replay_is_bitwise_the_reference(m, k, b):
    """oracle/reference_lapack.py (the CPU baseline where the reference was not
    built) is the reference's QR_2D call for call: bitwise-equal results."""
    if m % b:
        pytest.skip("the reference factors ((m/b)/p)*b rows")
    A = np.asfortranarray(fx.gaussian(m, k, m + k))
    want = ref.QR_2D(A, b)
    got = np.array(A, order="F")
    rl.QR_2D_lapack(got, b)
    assert np.array_equal(got, want)
    assert np.array_equal(ref.QR_2D(A, b, "pipe"), want)


@live
@pytest.mark.parametrize("m,b", [(300, 30), (1000, 100), (640, 128), (4096, 64), (96, 96)])
def test_reference_matches_oracle_more_shapes(m, b):
    A = fx.gaussian(m, b, 7 * m + b)
    YR, W = ref.hh_recon_qr(A, b)
    YRo, Wo = co.hh_recon_qr(A, b)
    close(YRo, YR, b)
    close(np.triu(Wo), np.triu(W), b)
    Af = np.array(A, order="F")
    Wl = rl.hh_recon_qr_lapack(rl._flat(Af), m, 0, m, b)
    assert np.array_equal(Af, YR)
    assert np.array_equal(Wl, np.triu(W))


@live
def test_reference_tree_and_nlu_match_oracle():
    for b in (5, 16, 40):
        S = tree_input(b, 900 + b)
        out, T = ref.tree_tsqr(S, b)
        R1, R2 = np.triu(S[:b]), np.triu(S[b:])
        tau = lp.dtpqrt_tri(R1, R2)
        close(np.triu(out[:b]), R1, b)
        close(np.triu(out[b:]), R2, b)
        close(T, lp.dtpqrt_T(R2, tau, min(b, 16)), b)
    # signed LU of (Q1 - S) on a Q factor's top block, b > 64 takes the recursion
    for b in (48, 100):
        Q, _ = np.linalg.qr(fx.gaussian(3 * b, b, b))
        R = np.triu(fx.gaussian(b, b, b + 1))
        A1, R1, s1 = ref.signed_NLU(Q[:b], R, recursive=(b > 64))
        A2, R2 = np.array(Q[:b]), np.array(R)
        s2 = co.recursive_NLU(A2, R2)
        assert np.array_equal(np.asarray(s1), np.asarray(s2, dtype=np.int64))
        close(A2, A1, b)
        close(R2, R1, b)


@pytest.mark.parametrize("n,b,b_sub", [(64, 16, 8), (200, 32, 16), (97, 32, 8)])
def test_full_to_band_oracle_keeps_the_spectrum(n, b, b_sub):
    """The restated full -> band reduction (alg/SE/full_to_band.cxx) is an
    orthogonal similarity onto a band of width b."""
    from oracle import se_oracle as se
    X = fx.gaussian(n, n, n)
    A = np.asfortranarray(X + X.T)
    Ar = np.array(A, order="F")
    se.sym_full2band(Ar, b, b_sub)
    B = se.band_matrix(Ar, b)
    assert np.abs(np.tril(B, -b - 1)).max() == 0.0
    ev = np.linalg.eigvalsh(A)
    assert np.abs(np.linalg.eigvalsh(B) - ev).max() <= 1e-13 * np.abs(ev).max()
