"""The reference's single-rank CAQR call sequence, executed with LAPACK/BLAS.

TEST INFRASTRUCTURE ONLY: the CPU baseline of bench.py (cpu_baseline and
`--impl reference`).  The reference itself is compiled from its own sources
where its checkout exists (oracle/build_ref.py -> oracle/_ref, x86 only: the
GPU host has neither the checkout nor a way to run an x86 build), so on the
GPU host this module stands in for it: it replays, call for call and with the
same leading dimensions and workspace sizes, what the reference's QR_2D does
on a 1 x 1 process grid, including the signed LU's dscal/dger/dtrsm/dgemm.
The LAPACK/BLAS routines are the Fortran entry points of the OpenBLAS build
bundled with scipy (LP64; `scipy_` symbol prefix), called through ctypes with
pointers into the column-major matrix, as the reference's wrappers in
alg/shared/lapack.cxx do; OpenBLAS uses every host thread.  Linked against
the same OpenBLAS, the compiled reference and this replay give bitwise-equal
results (tests/test_oracle_ref.py checks it).

  QR_2D (alg/QR/qr_2d/qr_2d.cxx:299-363), per panel:
    hh_recon_qr (alg/QR/hh_recon/hh_recon.cxx:129-321):
      bitree_tsqr with np_work == 1: copy the panel, dgeqrf   (bitree_tsqr.cxx:129-146)
      construct_Q1 with np_work == 1: copy Y, dorgqr           (construct_tsqr_Q.cxx:87-96)
      recursive_NLU on Q1's top block (dscal, dger, dtrsm, dgemm) (hh_recon.cxx:43-110,282)
      Y2 = Q2 U^-1 by dtrsm, Y and S*R back into A             (hh_recon.cxx:284-302)
      W = U S                                                  (hh_recon.cxx:304-310)
    update_A (qr_2d.cxx:124-177): pack Ybuf with a unit diagonal, then
    upd_A (qr_2d.cxx:224-282): T^-T from W by dtrsm (comp_bcast_T_from_W,
      :179-208), Z = Y^T A by dgemm (:259), Z <- (T^-T)^-1 Z by dtrsm (:271),
      A -= Y Z by dgemm (:275).
"""
import ctypes
import glob
import os

import numpy as np


_lib = None
_c_int = ctypes.c_int
_c_dbl = ctypes.c_double
_c_chr = ctypes.c_char


def _openblas():
    global _lib
    if _lib is None:
        import scipy
        d = os.path.join(os.path.dirname(scipy.__file__), "..", "scipy.libs")
        cands = sorted(glob.glob(os.path.join(d, "libscipy_openblas*.so")))
        if not cands:
            raise RuntimeError("scipy's bundled OpenBLAS was not found")
        _lib = ctypes.CDLL(cands[0])
    return _lib


def blas_threads():
    return int(_openblas().scipy_openblas_get_num_threads())


def _p(a, off=0):
    return ctypes.c_void_p(a.ctypes.data + 8 * off)


def _ref(x, t):
    return ctypes.byref(t(x))


def dgemm(ta, tb, m, n, k, alpha, A, offA, lda, B, offB, ldb, beta, C, offC, ldc):
    _openblas().scipy_dgemm_(_ref(ta.encode(), _c_chr), _ref(tb.encode(), _c_chr),
                             _ref(m, _c_int), _ref(n, _c_int), _ref(k, _c_int), _ref(alpha, _c_dbl),
                             _p(A, offA), _ref(lda, _c_int), _p(B, offB), _ref(ldb, _c_int),
                             _ref(beta, _c_dbl), _p(C, offC), _ref(ldc, _c_int))


def dtrsm(side, uplo, ta, diag, m, n, alpha, A, offA, lda, B, offB, ldb):
    _openblas().scipy_dtrsm_(_ref(side.encode(), _c_chr), _ref(uplo.encode(), _c_chr),
                             _ref(ta.encode(), _c_chr), _ref(diag.encode(), _c_chr),
                             _ref(m, _c_int), _ref(n, _c_int), _ref(alpha, _c_dbl),
                             _p(A, offA), _ref(lda, _c_int), _p(B, offB), _ref(ldb, _c_int))


def dscal(n, alpha, X, offX, incx):
    _openblas().scipy_dscal_(_ref(n, _c_int), _ref(alpha, _c_dbl), _p(X, offX), _ref(incx, _c_int))


def dger(m, n, alpha, X, offX, incx, Y, offY, incy, A, offA, lda):
    _openblas().scipy_dger_(_ref(m, _c_int), _ref(n, _c_int), _ref(alpha, _c_dbl), _p(X, offX),
                            _ref(incx, _c_int), _p(Y, offY), _ref(incy, _c_int), _p(A, offA),
                            _ref(lda, _c_int))


def dgeqrf(m, n, A, lda, tau, lwork=None):
    lwork = max(1, 64 * n) if lwork is None else max(1, lwork)
    work = np.empty(lwork)
    info = _c_int(0)
    _openblas().scipy_dgeqrf_(_ref(m, _c_int), _ref(n, _c_int), _p(A), _ref(lda, _c_int), _p(tau),
                              _p(work), _ref(lwork, _c_int), ctypes.byref(info))
    assert info.value == 0


def dorgqr(m, n, k, A, lda, tau, lwork=None):
    lwork = max(1, 64 * n) if lwork is None else max(1, lwork)
    work = np.empty(lwork)
    info = _c_int(0)
    _openblas().scipy_dorgqr_(_ref(m, _c_int), _ref(n, _c_int), _ref(k, _c_int), _p(A),
                              _ref(lda, _c_int), _p(tau), _p(work), _ref(lwork, _c_int),
                              ctypes.byref(info))
    assert info.value == 0


def _flat(A):
    """1-D view of a Fortran array's storage (for pointer arithmetic)."""
    assert A.flags.f_contiguous
    return A.reshape(-1, order="F")


def signed_NLU_lapack(A, offA, lda, R, offR, ldr, b, signs, soff):
    """signed_NLU (hh_recon.cxx:43-68) call for call: sign choice, dscal of R's
    row, column division by the pivot, dger rank-1 update.  A and R are 1-D
    views of column-major storage."""
    for i in range(b):
        d = A[offA + i * lda + i]
        s = -1 if d > 0 else 1
        signs[soff + i] = s
        A[offA + i * lda + i] = d - s
        if s == -1:
            dscal(b - i, -1.0, R, offR + i * ldr + i, ldr)
        c0 = offA + i * lda + i
        A[c0 + 1:c0 + b - i] = A[c0 + 1:c0 + b - i] / A[c0]
        if b - i - 1 > 0:
            dger(b - i - 1, b - i - 1, -1.0, A, c0 + 1, 1, A, offA + (i + 1) * lda + i, lda,
                 A, offA + (i + 1) * lda + i + 1, lda)


def recursive_NLU_lapack(A, offA, lda, R, offR, ldr, b, signs, soff=0):
    """recursive_NLU (hh_recon.cxx:80-110, BSIZE = 64) call for call."""
    if b <= 64:
        signed_NLU_lapack(A, offA, lda, R, offR, ldr, b, signs, soff)
        return
    b1 = b // 2
    b2 = b - b1
    recursive_NLU_lapack(A, offA, lda, R, offR, ldr, b1, signs, soff)
    for i in range(b1):
        if signs[soff + i] == -1:
            dscal(b2, -1.0, R, offR + b1 * ldr + i, ldr)
    dtrsm("L", "L", "N", "U", b1, b2, 1.0, A, offA, lda, A, offA + b1 * lda, lda)
    dtrsm("R", "U", "N", "N", b2, b1, 1.0, A, offA, lda, A, offA + b1, lda)
    dgemm("N", "N", b2, b2, b1, -1.0, A, offA + b1, lda, A, offA + b1 * lda, lda, 1.0, A,
          offA + b1 * (lda + 1), lda)
    recursive_NLU_lapack(A, offA + b1 * (lda + 1), lda, R, offR + b1 * (ldr + 1), ldr, b2, signs,
                         soff + b1)


def hh_recon_qr_lapack(Af, lda, off, m, b):
    """hh_recon_qr at numPes == 1 on the m x b panel at offset `off` of Af
    (hh_recon.cxx:129-321), call for call; returns W (b x b, upper)."""
    # bitree_tsqr, one process (bitree_tsqr.cxx:129-146): copy, dgeqrf with
    # lwork = m b, R = upper triangle, Y\R back into A
    buf = np.empty((m, b), order="F")
    for j in range(b):
        buf[:, j] = Af[off + j * lda: off + j * lda + m]
    tau = np.empty(b)
    dgeqrf(m, b, buf, m, tau, lwork=m * b)
    R = np.array(np.triu(buf[:b, :b]), order="F")
    # construct_Q1, one process (construct_tsqr_Q.cxx:87-96): dorgqr on a copy
    dorgqr(m, b, b, buf, m, tau, lwork=m * b)          # buf now holds Q1 (lda = m)
    q1 = _flat(buf)
    rf = _flat(R)
    signs = np.zeros(b, dtype=np.int64)
    recursive_NLU_lapack(q1, 0, m, rf, 0, b, b, signs)
    W = np.array(np.triu(buf[:b, :b]), order="F")     # copy_upper(Q1, W) (:284)
    if m > b:
        dtrsm("R", "U", "N", "N", m - b, b, 1.0, W, 0, b, buf, b, m)   # Y2 = Q2 U^-1 (:299)
    buf[:b, :b] = np.tril(buf[:b, :b], -1) + R          # copy_upper(R, A) + copy_lower(Q1, A)
    for j in range(b):
        col = buf[:, j].copy()
        Af[off + j * lda: off + j * lda + m] = col
    for i in range(b):                                  # W = U S (:304-310)
        if signs[i] == -1:
            dscal(i + 1, -1.0, W, i * b, 1)
    return W


def upd_A_lapack(Af, lda, offY, offA, m, k, b, W):
    """update_A + upd_A with W from hh_recon_qr (qr_2d.cxx:124-177, 224-282)."""
    Ybuf = np.zeros((m, b), order="F")
    for j in range(b):
        Ybuf[j + 1:, j] = Af[offY + j * lda + j + 1: offY + j * lda + m]
        Ybuf[j, j] = 1.0
    X = np.array(Ybuf[:b, :b], order="F")
    dtrsm("L", "U", "T", "N", b, b, -1.0, W, 0, b, X, 0, b)        # W^T X = -Y1
    X = np.array(np.tril(X), order="F")
    Z = np.empty((b, k), order="F")
    dgemm("T", "N", b, k, m, 1.0, Ybuf, 0, m, Af, offA, lda, 0.0, Z, 0, b)
    dtrsm("L", "L", "N", "N", b, k, 1.0, X, 0, b, Z, 0, b)
    dgemm("N", "N", m, k, b, -1.0, Ybuf, 0, m, Z, 0, b, 1.0, Af, offA, lda)


def QR_2D_lapack(A, b):
    """QR_2D on a 1 x 1 grid; A (Fortran float64, m x k, m >= k) becomes Y\\R in place."""
    m, k = A.shape
    lda = m
    Af = _flat(A)
    r0 = 0
    while True:
        mm, kk = m - r0, k - r0
        bb = min(kk, b)
        off = r0 * lda + r0
        W = hh_recon_qr_lapack(Af, lda, off, mm, bb)
        if kk - b > 0 and mm - b > 0:
            upd_A_lapack(Af, lda, off, off + b * lda, mm, kk - b, b, W)
            r0 += b
        else:
            break
    return A


def ls_solve_lapack(A, B, b):
    """Least squares by the reference's own call sequence on a 1 x 1 grid:
    hh_recon_qr on each b-column panel of A (hh_recon.cxx:129-321), update_A
    of the panel's Q^T on the rest of [A | B] (qr_2d.cxx:124-177, 224-282),
    then X = R^-1 (Q^T B)[0:n] by dtrsm.  A (m x n), B (m x r); returns X."""
    m, n = A.shape
    B = np.asarray(B, dtype=np.float64).reshape(m, -1)
    r = B.shape[1]
    Aug = np.empty((m, n + r), order="F")
    Aug[:, :n] = A
    Aug[:, n:] = B
    Af = _flat(Aug)
    lda = m
    r0 = 0
    while r0 < n:
        bb = min(b, n - r0)
        off = r0 * lda + r0
        W = hh_recon_qr_lapack(Af, lda, off, m - r0, bb)
        upd_A_lapack(Af, lda, off, off + bb * lda, m - r0, n + r - r0 - bb, bb, W)
        r0 += bb
    R = np.array(np.triu(Aug[:n, :n]), order="F")
    X = np.array(Aug[:n, n:], order="F")
    dtrsm("L", "U", "N", "N", n, r, 1.0, R, 0, n, X, 0, n)
    return X
