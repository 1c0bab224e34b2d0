"""The symmetric full -> band reduction of the reference's eigensolver,
restated on the oracle's QR pieces.

TEST INFRASTRUCTURE ONLY.  sym_full2band (alg/SE/full_to_band.cxx:27-295) on
a 1 x 1 grid: per band step, the (n - b) x b block below the diagonal block is
factored by 2D QR in panels of b_sub with its reflectors aggregated into Y
(:99, QR_2D_pipe), T^-T comes from Y^T Y (:105, compute_invT_from_Y), then
  W = Y^T A22 (:121),  Z = Y^T W^T (:160),  U = Y T^T from U invT = Y (:177),
  V' = W - Z U^T / 2 (:186),  A22 -= U V' + (U V')^T (:217-242)
and the reduction continues on A22 (:286).

The reference's own routine, compiled here on one rank, returns NaNs: it hands
its Y buffer to QR_2D_pipe as the `last_Y` argument (:99), which that routine
uses as lookahead state rather than filling with the panel's reflectors
(qr_2d.cxx:378-635), and then reads Y back (:105, :121).  This restatement
follows the algorithm the file's comments and formulas describe, with Y taken
from the factored panel.
"""
import numpy as np

from . import candmc_oracle as co
from . import lapack_restated as lp


def sym_full2band(A, b, b_sub=None):
    """A (n x n symmetric, full storage) -> in place: the lower triangle holds
    the band (diagonal blocks, R blocks below them) and the reflectors below
    the band; A's trailing blocks are updated in full."""
    b_sub = b if b_sub is None else b_sub
    n = A.shape[0]
    r0 = 0
    while n - r0 > b:
        m = n - r0 - b
        bb = min(b, m)                           # reflectors of the m x b block
        P = A[r0 + b:, r0:r0 + bb]
        co.QR_2D(P, min(b_sub, bb))              # P becomes Y\R in place
        Y = lp.unit_lower(P, bb)
        invT = co.compute_invT_from_Y(Y)         # T^-T, lower (qr_2d.cxx:22-60)
        if bb < b:                               # the block's last columns: R is trapezoidal
            co.upd_A(Y, A[r0 + b:, r0 + bb:r0 + b], None)
        U = np.linalg.solve(np.tril(invT).T, Y.T).T   # U invT = Y
        A22 = A[r0 + b:, r0 + b:]
        W = Y.T @ A22
        Z = Y.T @ W.T
        V = W - 0.5 * Z @ U.T
        X = U @ V
        A22 -= X + X.T
        r0 += b
    return A


def band_matrix(A, b):
    """The symmetric band matrix held in the lower triangle after sym_full2band:
    diagonal blocks and the upper-triangular R blocks below them."""
    n = A.shape[0]
    B = np.zeros_like(A)
    r0 = 0
    while r0 < n:
        e = min(n, r0 + b)
        D = np.tril(A[r0:e, r0:e])
        B[r0:e, r0:e] = D + np.tril(D, -1).T
        if e < n:
            e2 = min(n, e + b)
            R = np.triu(A[e:e2, r0:e])
            B[e:e2, r0:e] = R
            B[r0:e, e:e2] = R.T
        r0 = e
    return B
