"""CPU restatement of CANDMC's Yamamoto basis-kernel representation.

TEST INFRASTRUCTURE ONLY.  Nothing in the product imports this module; the
tests use it as the reference result.

Yamamoto's representation writes the Householder Q of a TSQR panel as
    Q_HH^T = I + Qm W Qm^T,   Qm = [Q1 - S; Q2],   W = (Q1 - S)^-1 S,
where [Q1; Q2] are the first b columns of the TSQR's orthogonal factor and
S = diag(+-1) is the sign choice of the unpivoted LU of Q1 - S.  The
functions restate alg/QR/hh_recon/yamamoto.cxx and alg/QR/qr_2d/qr_y2d.cxx
on one process (a 1 x 1 grid), on top of the TSQR and explicit-Q restatements
of candmc_oracle (bitree_tsqr.cxx, construct_tsqr_Q.cxx).
"""
import numpy as np

from . import candmc_oracle as co
from . import lapack_restated as lp

BSIZE = 64      # recursion base of recursive_YLU, alg/QR/hh_recon/yamamoto.cxx:13


def signed_YLU(A, signs, off=0):
    """Sign-choice unpivoted LU of (A - S) in place (yamamoto.cxx:25-46).

    S_ii = -1 when the current pivot is positive, +1 otherwise; A becomes L\\U.
    """
    b = A.shape[0]
    for i in range(b):
        s = -1 if A[i, i] > 0 else 1
        signs[off + i] = s
        A[i, i] -= s
        A[i + 1:, i] /= A[i, i]
        A[i + 1:, i + 1:] -= np.outer(A[i + 1:, i], A[i, i + 1:])


def recursive_YLU(A, signs=None, off=0):
    """Recursive signed LU, halving until b <= BSIZE (yamamoto.cxx:57-80)."""
    b = A.shape[0]
    if signs is None:
        signs = np.zeros(b, dtype=np.int64)
    if b <= BSIZE:
        signed_YLU(A, signs, off)
        return signs
    b1 = b // 2
    recursive_YLU(A[:b1, :b1], signs, off)
    lp.dtrsm('L', 'L', 'N', 'U', 1.0, A[:b1, :b1], A[:b1, b1:])
    lp.dtrsm('R', 'U', 'N', 'N', 1.0, A[:b1, :b1], A[b1:, :b1])
    A[b1:, b1:] -= A[b1:, :b1] @ A[:b1, b1:]
    recursive_YLU(A[b1:, b1:], signs, off + b1)
    return signs


def lu_inverse(LU):
    """(L U)^-1 from the unit-lower L and upper U packed in LU: dgetri with
    identity pivots (yamamoto.cxx:150-154), restated as U^-1 (L^-1)."""
    b = LU.shape[0]
    X = np.eye(b)
    lp.dtrsm('L', 'L', 'N', 'U', 1.0, LU, X)
    lp.dtrsm('L', 'U', 'N', 'N', 1.0, LU, X)
    return X


def Yamamoto(A, b):
    """TSQR and Yamamoto's representation of an m x b panel (yamamoto.cxx:98-174).

    Returns (YR, Qm, W, signs).  YR (m x b) holds the TSQR's leaf reflectors
    below the diagonal and S*R on and above it (R copied in by copy_upper,
    :128-129, rows scaled by the signs, :160); Qm = [Q1 - S; Q2] (:157);
    W = (Q1 - S)^-1 S (:150-158).  A is not modified.
    """
    A = np.array(A, dtype=np.float64)
    m = A.shape[0]
    assert A.shape[1] == b
    blocks = [A]
    R, taus, tree = co.bitree_tsqr(blocks, b, 0)
    YR = blocks[0]
    YR[:b, :b] = np.tril(YR[:b, :b], -1) + np.triu(R)
    Qm = co.construct_Q1(blocks, taus, tree, b, b, 0)[0]
    LU = Qm[:b, :b].copy()
    signs = recursive_YLU(LU)
    W = lu_inverse(LU)
    for i in range(b):
        Qm[i, i] -= signs[i]
        W[:, i] *= signs[i]
        YR[i, i:] *= signs[i]
    return YR, Qm, W, signs


def upd_Yamamoto_A(Qm, A, W):
    """A <- A + Qm (W (Qm^T A)) = (I - Qm (-W) Qm^T) A, in place (qr_y2d.cxx:133-178)."""
    QmTA = Qm.T @ A
    QmTA2 = -(W @ QmTA)
    A -= Qm @ QmTA2
    return A


class Aggregator:
    """Aggregated representation of several panels (qr_y2d.cxx:13-66).

    aQm (lda_aQm x lda_aT) stacks the panels' Qm, each one `shift` rows lower
    than the last; aT (lda_aT x lda_aT) is block lower triangular, so that
    I + aQm aT aQm^T applies the panels in order.
    """

    def __init__(self, lda_aQm, lda_aT):
        self.lda_aQm = lda_aQm
        self.lda_aT = lda_aT
        self.aQm = np.zeros((lda_aQm, lda_aT))
        self.aT = np.zeros((lda_aT, lda_aT))
        self.n = 0
        self.shift = 0

    def reset(self):
        self.n = 0
        self.shift = 0
        self.aQm[:] = 0.0
        self.aT[:] = 0.0

    def shift_down(self, b):
        self.shift += b

    def append(self, mb, b, Qm, T):
        n, sh = self.n, self.shift
        if mb > 0:
            self.aQm[sh:sh + mb, n:n + b] = Qm[:mb, :b]
        if n == 0:
            self.aT[:b, :b] = T
        else:
            X = Qm[:mb, :b].T @ self.aQm[sh:sh + mb, :n] if mb > 0 else np.zeros((b, n))
            self.aT[n:n + b, :n] = T @ (X @ self.aT[:n, :n])
            self.aT[n:n + b, n:n + b] = T
        self.n += b


def _getrf_nopiv_check(LU):
    """dgetrf of Q1 - S (qr_y2d.cxx:222-226).  Partial pivoting keeps the
    diagonal here (|L| <= 1 for this matrix); the restatement asserts it."""
    b = LU.shape[0]
    LU = LU.copy()
    for i in range(b):
        p = i + int(np.argmax(np.abs(LU[i:, i])))
        assert abs(LU[p, i]) <= abs(LU[i, i]) * (1 + 1e-12), "pivoting would swap rows"
        LU[i + 1:, i] /= LU[i, i]
        LU[i + 1:, i + 1:] -= np.outer(LU[i + 1:, i], LU[i, i + 1:])
    return LU


def QR_Yamamoto_2D(A, b, agg=None, compute_Y=False):
    """CAQR with Yamamoto's representation on a 1 x 1 grid (qr_y2d.cxx:181-263).

    Each panel: Yamamoto on the first min(k, b) columns, the trailing update
    A += Qm W Qm^T A (update_Yamamoto_A, which also appends Qm and W to agg),
    optionally Y = Qm U^-1 written below R (compute_Y, :220-240), then the
    recursion on the trailing block (agg shifted down by b).  The last
    panel's Qm and W are appended without an update (:249-257).  A (m x k)
    is overwritten in place.
    """
    A = np.asarray(A)
    m, k = A.shape
    r0 = 0
    while True:
        mm, kk = m - r0, k - r0
        bb = min(kk, b)
        YR, Qm, W, _ = Yamamoto(A[r0:, r0:r0 + bb], bb)
        A[r0:, r0:r0 + bb] = YR
        more = kk - b > 0 and mm - b > 0
        if more:
            upd_Yamamoto_A(Qm, A[r0:, r0 + b:], W)
            if agg is not None:
                agg.append(mm, bb, Qm, W)
        if compute_Y:
            LU = _getrf_nopiv_check(Qm[:bb, :bb])
            Qm2 = Qm.copy()
            lp.dtrsm('R', 'U', 'N', 'N', 1.0, LU, Qm2)
            blk = A[r0:, r0:r0 + bb]
            blk[:bb, :] = np.triu(blk[:bb, :]) + np.tril(Qm2[:bb, :], -1)
            blk[bb:, :] = Qm2[bb:, :]
        if not more:
            if agg is not None and mm - b >= 0:
                agg.append(mm, bb, Qm, W)
            break
        if agg is not None:
            agg.shift_down(b)
        r0 += b
    return A


def QR_Yamamoto_2D_2D(A, b, b_sub, agg=None, compute_Y=False):
    """Two-level blocking (qr_y2d.cxx:265-393) on a 1 x 1 grid.

    A b-wide block is factored by QR_Yamamoto_2D with b_sub panels that
    aggregate into one representation, which then updates the columns
    beyond the block at once; the aggregator is reset and the trailing block
    recurses.
    """
    A = np.asarray(A)
    m, k = A.shape
    if k - b > 0 and m - b > 0:
        iagg = agg if agg is not None else Aggregator(m, b)
        QR_Yamamoto_2D(A[:, :min(k, b)], b_sub, iagg, compute_Y)
        upd_Yamamoto_A(iagg.aQm[:m, :b], A[:, b:], iagg.aT[:b, :b])
        iagg.reset()
        QR_Yamamoto_2D_2D(A[b:, b:], b, b_sub, iagg, compute_Y)
    else:
        QR_Yamamoto_2D(A, b_sub, agg, compute_Y)
    return A
