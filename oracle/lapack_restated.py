"""CPU restatement of the LAPACK/BLAS routines that CANDMC's QR path calls.

TEST INFRASTRUCTURE ONLY.  This module is the arithmetic half of the oracle:
the CUDA path is checked against it, it is never part of the product path.

CANDMC does not implement this arithmetic itself.  Its QR code calls
Fortran LAPACK/BLAS ("LAPACK 3.4.0 or higher", README.md:12; the configure
probe for dtpqrt is configure:489-497) through the wrappers in
alg/shared/lapack.cxx.  The published LAPACK algorithms are restated here in
numpy, unblocked where the blocked LAPACK routine produces the same
reflectors (dgeqrf = blocked dgeqr2, dorgqr = blocked dorg2r, dtpqrt =
blocked dtpqrt2).  Column-major storage is modelled with numpy arrays indexed
[row, col]; every routine works in float64.

Reference call sites (alg/...):
  cdgeqrf   QR/tsqr/bitree_tsqr.cxx:62        -> dgeqrf
  cdtpqrt   QR/tsqr/bitree_tsqr.cxx:29        -> dtpqrt
  cdorgqr   QR/tsqr/construct_tsqr_Q.cxx:96   -> dorgqr
  cdormqr   QR/tsqr/construct_tsqr_Q.cxx:231  -> dormqr_left_notrans
  cdtprfb   QR/tsqr/construct_tsqr_Q.cxx:202  -> dtpmqrt_left_notrans
  cdtrsm    QR/hh_recon/hh_recon.cxx:30,294   -> dtrsm
  cdger     QR/hh_recon/hh_recon.cxx:64       (inlined in signed_NLU)
  cdgemm    QR/qr_2d/qr_2d.cxx:259,275        -> numpy matmul
  cdsyrk    QR/qr_2d/qr_2d.cxx:39             -> numpy matmul
"""
import math

import numpy as np


def dlarfg(alpha, x):
    """Elementary reflector H = I - tau*[1;v]*[1;v]^T with H*[alpha;x] = [beta;0].

    LAPACK dlarfg: beta = -sign(alpha)*||[alpha;x]||, tau = (beta-alpha)/beta,
    v = x/(alpha-beta).  When ||x|| == 0, tau = 0 and H = I.  (LAPACK's
    safe-minimum rescaling loop only matters for |beta| < 2^-1022 and is
    omitted.)  Returns (beta, tau, v).
    """
    x = np.asarray(x, dtype=np.float64)
    xnorm = float(np.linalg.norm(x)) if x.size else 0.0
    if xnorm == 0.0:
        return float(alpha), 0.0, x.copy()
    beta = -math.copysign(math.hypot(alpha, xnorm), alpha)
    tau = (beta - alpha) / beta
    v = x * (1.0 / (alpha - beta))
    return beta, tau, v


def dgeqr2(A):
    """Householder QR in place (LAPACK dgeqr2; dgeqrf is its blocked form).

    A (m x n) becomes Y\\R: R on and above the diagonal, the reflector tails
    below it (unit diagonal implicit).  Returns tau (min(m,n),).
    """
    m, n = A.shape
    k = min(m, n)
    tau = np.zeros(k)
    for j in range(k):
        beta, t, v = dlarfg(A[j, j], A[j + 1:, j])
        tau[j] = t
        A[j + 1:, j] = v
        A[j, j] = beta
        if j + 1 < n and t != 0.0:
            w = A[j, j + 1:] + v @ A[j + 1:, j + 1:]
            A[j, j + 1:] -= t * w
            A[j + 1:, j + 1:] -= t * np.outer(v, w)
    return tau


def dlarft(Y, tau):
    """Upper-triangular T of the compact WY form H_0 H_1 ... = I - Y T Y^T.

    LAPACK dlarft('F','C'): T[i,i] = tau_i,
    T[0:i,i] = -tau_i * T[0:i,0:i] @ (Y[:,0:i]^T Y[:,i]).
    Y is the unit-lower-trapezoidal reflector matrix (explicit ones/zeros).
    """
    k = len(tau)
    T = np.zeros((k, k))
    G = Y.T @ Y
    for i in range(k):
        T[i, i] = tau[i]
        if i:
            T[:i, i] = -tau[i] * (T[:i, :i] @ G[:i, i])
    return T


def unit_lower(YR, b):
    """Explicit unit-lower-trapezoidal Y from a Y\\R buffer (first b columns)."""
    Y = np.tril(YR[:, :b], -1)
    Y[np.arange(b), np.arange(b)] = 1.0
    return Y


def dgeqrf(A, nb=32):
    """Blocked Householder QR (LAPACK dgeqrf with block size nb).

    Same reflectors as dgeqr2; the trailing columns of each nb-wide block are
    updated by the block reflector (dlarft + dlarfb), as LAPACK does.
    """
    m, n = A.shape
    k = min(m, n)
    tau = np.zeros(k)
    for j0 in range(0, k, nb):
        j1 = min(k, j0 + nb)
        tau[j0:j1] = dgeqr2(A[j0:, j0:j1])
        if j1 < n:
            Y = unit_lower(A[j0:, j0:j1], j1 - j0)
            T = dlarft(Y, tau[j0:j1])
            C = A[j0:, j1:]
            C -= Y @ (T.T @ (Y.T @ C))
    return tau


def dorg2r(A, tau, ncols=None):
    """Explicit first ncols columns of Q = H_0 ... H_{k-1} (LAPACK dorg2r/dorgqr).

    A holds the reflectors below the diagonal of its first k = len(tau)
    columns and is overwritten with Q (m x ncols).
    """
    m = A.shape[0]
    k = len(tau)
    n = A.shape[1] if ncols is None else ncols
    Q = np.zeros((m, n))
    Q[:, :k] = A[:, :k]
    for j in range(k, n):
        Q[:, j] = 0.0
        Q[j, j] = 1.0
    for i in reversed(range(k)):
        if i + 1 < n:
            v = np.concatenate(([1.0], Q[i + 1:, i]))
            w = v @ Q[i:, i + 1:]
            Q[i:, i + 1:] -= tau[i] * np.outer(v, w)
        Q[i + 1:, i] *= -tau[i]
        Q[i, i] = 1.0 - tau[i]
        Q[:i, i] = 0.0
    A[:, :n] = Q
    return A


def dormqr_left_notrans(Yr, tau, C):
    """C <- Q C with Q = H_0 ... H_{k-1} from a Y\\R buffer (LAPACK dormqr 'L','N')."""
    k = len(tau)
    for i in reversed(range(k)):
        if tau[i] == 0.0:
            continue
        v = np.concatenate(([1.0], Yr[i + 1:, i]))
        w = v @ C[i:, :]
        C[i:, :] -= tau[i] * np.outer(v, w)
    return C


def dtpqrt_tri(R1, R2):
    """QR of two stacked upper-triangular blocks [R1; R2] (LAPACK dtpqrt, l = n).

    Restates the unblocked dtpqrt2 with a triangular ("pentagonal", l = n)
    bottom block: reflector j is [e_j; V[0:j+1, j]].  R1 becomes R, R2 becomes
    V (upper triangular).  Returns tau (n,).  dtpqrt stores the same
    reflectors plus the block-diagonal T; T is rebuilt by `dtpqrt_T` below.
    """
    n = R1.shape[1]
    tau = np.zeros(n)
    for j in range(n):
        beta, t, v = dlarfg(R1[j, j], R2[:j + 1, j])
        tau[j] = t
        R1[j, j] = beta
        R2[:j + 1, j] = v
        if j + 1 < n and t != 0.0:
            w = R1[j, j + 1:] + v @ R2[:j + 1, j + 1:]
            R1[j, j + 1:] -= t * w
            R2[:j + 1, j + 1:] -= t * np.outer(v, w)
    return tau


def dtpqrt_T(V, tau, nb):
    """The T output of dtpqrt (nb x n, ld nb) for the dtpqrt_tri reflectors:
    column c holds the upper triangle of the nb-wide diagonal block of the
    compact-WY factor of Y = [I; V] that contains c (the T of that block of
    reflectors alone); entries below each block's diagonal are zero."""
    n = V.shape[1]
    Y = np.vstack([np.eye(n), np.triu(V)])
    T = dlarft(Y, tau)
    out = np.zeros((nb, n))
    for c in range(n):
        q0 = (c // nb) * nb
        out[:c - q0 + 1, c] = T[q0:c + 1, c]
    return out


def dtpmqrt_left_notrans(V, tau, top, bottom):
    """[top; bottom] <- Q [top; bottom], Q the dtpqrt_tri factor (LAPACK dtpmqrt/dtprfb 'L','N')."""
    n = V.shape[1]
    for j in reversed(range(n)):
        if tau[j] == 0.0:
            continue
        v = V[:j + 1, j]
        w = top[j, :] + v @ bottom[:j + 1, :]
        top[j, :] -= tau[j] * w
        bottom[:j + 1, :] -= tau[j] * np.outer(v, w)
    return top, bottom


def dtrsm(side, uplo, trans, diag, alpha, A, B):
    """Triangular solve in place (BLAS dtrsm), restated by substitution.

    side 'L': B <- alpha * op(A)^-1 B;  side 'R': B <- alpha * B op(A)^-1.
    """
    n = A.shape[0]
    Ad = np.array(A[:n, :n], dtype=np.float64)
    T = np.triu(Ad) if uplo == 'U' else np.tril(Ad)
    if diag == 'U':
        T[np.arange(n), np.arange(n)] = 1.0
    if trans == 'T':
        T = T.T
    lower = (uplo == 'L') != (trans == 'T')
    if side == 'L':
        X = alpha * np.array(B, dtype=np.float64)
        rng = range(n) if lower else reversed(range(n))
        for i in rng:
            X[i, :] /= T[i, i]
            if lower:
                X[i + 1:, :] -= np.outer(T[i + 1:, i], X[i, :])
            else:
                X[:i, :] -= np.outer(T[:i, i], X[i, :])
        B[...] = X
    else:
        # X op(A) = alpha B  <=>  op(A)^T X^T = alpha B^T
        Xt = alpha * np.array(B, dtype=np.float64).T
        Tt = T.T
        lower_t = not lower
        rng = range(n) if lower_t else reversed(range(n))
        for i in rng:
            Xt[i, :] /= Tt[i, i]
            if lower_t:
                Xt[i + 1:, :] -= np.outer(Tt[i + 1:, i], Xt[i, :])
            else:
                Xt[:i, :] -= np.outer(Tt[:i, i], Xt[i, :])
        B[...] = Xt.T
    return B
