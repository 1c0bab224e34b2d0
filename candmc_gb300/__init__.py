"""GB300-native QR hot path of CANDMC: TSQR, Householder reconstruction, CAQR.

Python mirror of the reference's QR entry points (include/CANDMC.h ->
alg/QR/tsqr/bitree_tsqr.h, alg/QR/hh_recon/hh_recon.h, alg/QR/qr_2d/qr_2d.h,
alg/QR/qr_2d/qr_y2d.h)
on one GPU: the process grid is 1 x 1, so the MPI arguments (myRank, numPes,
root, req_id, CommData_t, pview) disappear.  Every function calls the C ABI
of libcandmc_gb300.so (include/candmc_gb300.h); there is no CPU fallback and
an unbuilt library raises.

Matrices are column-major float64, as in the reference:
  * device arrays: torch CUDA tensors with stride(0) == 1 (see `colmajor`),
    the leading dimension is stride(1); work is enqueued on the current torch
    stream (or `stream`);
  * host arrays: numpy float64 in Fortran order, updated in place (the
    reference's pointers are host memory).
Errors raise CandmcError (the reference asserts/aborts instead).
"""
import ctypes

import numpy as np

from . import _abi
from ._abi import CandmcError, check

__all__ = [
    "CandmcError", "colmajor", "empty_colmajor", "hh_recon_qr", "bitree_tsqr", "construct_Q1",
    "compute_invT_from_W", "signed_NLU", "recursive_NLU", "compute_invT_from_Y",
    "compute_invT_from_Y2", "upd_A", "update_A", "QR_2D", "QR_2D_2D", "QR_2D_pipe", "Yamamoto",
    "upd_Yamamoto_A", "Aggregator", "QR_Yamamoto_2D", "QR_Yamamoto_2D_2D", "ls_solve",
    "batched_ls", "batched_status", "set_tuning", "PRECISIONS", "lib",
]

PRECISIONS = {"fp64": 0, "ozaki": 1, "fp32": 2}


def lib():
    return _abi.load()


def _torch():
    import torch
    return torch


def colmajor(x):
    """Column-major copy of a 2-D torch tensor (stride(0) == 1)."""
    return x.t().contiguous().t()


def empty_colmajor(m, n, device="cuda", dtype=None):
    torch = _torch()
    return torch.empty((n, m), dtype=dtype or torch.float64, device=device).t()


def _is_torch(x):
    try:
        import torch
    except ImportError:
        return False
    return isinstance(x, torch.Tensor)


def _dev(x, name, rows=None):
    """(pointer, leading dimension) of a column-major CUDA float64 tensor."""
    torch = _torch()
    if not (isinstance(x, torch.Tensor) and x.is_cuda):
        raise TypeError(f"{name}: expected a CUDA tensor")
    if x.dtype not in (torch.float64, torch.int64):
        raise TypeError(f"{name}: expected float64")
    if x.dim() == 1:
        return x.data_ptr(), max(1, x.shape[0])
    if x.stride(0) != 1 and x.shape[0] > 1:
        raise ValueError(f"{name}: must be column-major (stride(0) == 1); use colmajor()")
    ld = x.stride(1) if x.shape[1] > 1 else max(1, x.shape[0])
    return x.data_ptr(), ld


def _stream(stream):
    if stream is None:
        return _torch().cuda.current_stream().cuda_stream
    return getattr(stream, "cuda_stream", stream)


def _host(x, name):
    if not isinstance(x, np.ndarray) or x.dtype != np.float64 or not x.flags.f_contiguous:
        raise TypeError(f"{name}: expected a Fortran-ordered float64 numpy array")
    if not x.flags.writeable:
        raise ValueError(f"{name}: must be writeable (updated in place)")
    return x.ctypes.data, max(1, x.shape[0])


def _prec(p):
    if isinstance(p, str):
        return PRECISIONS[p]
    return int(p)


# ------------------------------------------------------------------ panel
def hh_recon_qr(A, W=None, T=None, stream=None):
    """TSQR + Householder reconstruction (alg/QR/hh_recon/hh_recon.h:66-75).

    A (m x b) is overwritten with Y\\(S*R).  Returns (W, T): W = U*S =
    -T*Y1^T (b x b upper) and T, the compact-WY factor Q = I - Y T Y^T.
    """
    m, b = A.shape
    if isinstance(A, np.ndarray):
        pa, lda = _host(A, "A")
        W = np.zeros((b, b), order="F") if W is None else W
        T = np.zeros((b, b), order="F") if T is None else T
        check(lib().candmc_hh_recon_qr_host(pa, lda, m, b, _host(W, "W")[0], _host(T, "T")[0]),
              "hh_recon_qr")
        return W, T
    W = empty_colmajor(b, b, A.device) if W is None else W
    T = empty_colmajor(b, b, A.device) if T is None else T
    pa, lda = _dev(A, "A")
    check(lib().candmc_hh_recon_qr(pa, lda, m, b, _dev(W, "W")[0], _dev(T, "T")[0], _stream(stream)),
          "hh_recon_qr")
    return W, T


def bitree_tsqr(A, output_Y=1, stream=None):
    """Single-rank binary-tree TSQR (alg/QR/tsqr/bitree_tsqr.h:58-70): returns (R, tau);
    A becomes the LAPACK-form Y\\R when output_Y."""
    m, b = A.shape
    R = empty_colmajor(b, b, A.device)
    tau = _torch().empty(b, dtype=_torch().float64, device=A.device)
    pa, lda = _dev(A, "A")
    check(lib().candmc_bitree_tsqr(pa, lda, _dev(R, "R")[0], tau.data_ptr(), m, b, int(output_Y),
                                   _stream(stream)), "bitree_tsqr")
    return R, tau


def construct_Q1(Y, tau, k=None, stream=None):
    """First k columns of the TSQR Q (alg/QR/tsqr/bitree_tsqr.h:91-104, numPes = 1)."""
    m, b = Y.shape
    k = b if k is None else k
    Q1 = empty_colmajor(m, k, Y.device)
    py, ldy = _dev(Y, "Y")
    check(lib().candmc_construct_Q1(py, ldy, tau.data_ptr(), _dev(Q1, "Q1")[0], _dev(Q1, "Q1")[1],
                                    m, b, k, _stream(stream)), "construct_Q1")
    return Q1


def tree_tsqr(A, T=None, stream=None):
    """QR of the stacked [R1; R2] (alg/QR/tsqr/bitree_tsqr.h:16-19, dtpqrt's
    contract): A (2b x b) gets R over R1's and V over R2's upper triangle, its
    strictly-lower entries untouched.  Returns T (min(b,16) x b), dtpqrt's
    block-diagonal factor."""
    m, b = A.shape
    if m != 2 * b:
        raise ValueError("tree_tsqr: A must be 2b x b")
    pa, lda = _dev(A, "A")
    if lda != 2 * b:
        raise ValueError("tree_tsqr: the leading dimension of A must be 2b")
    nb = min(b, 16)
    T = _torch().zeros((b, nb), dtype=_torch().float64, device=A.device).t() if T is None else T
    check(lib().candmc_tree_tsqr(pa, b, _dev(T, "T")[0], _stream(stream)), "tree_tsqr")
    return T


def apply_tsqr_QT(Y, tau, B, stream=None):
    """B <- Q^T B for the single-rank TSQR factor (alg/QR/tsqr/bitree_tsqr.h:126-138)."""
    m, b = Y.shape
    py, ldy = _dev(Y, "Y")
    pb, ldb = _dev(B, "B")
    check(lib().candmc_apply_tsqr_QT(py, ldy, tau.data_ptr(), pb, ldb, m, b, B.shape[1], _stream(stream)),
          "apply_tsqr_QT")
    return B


def tau_recon(structure, Y, nrow=None, stream=None):
    """tau of the Householder vectors in Y (alg/shared/util.h:675-680):
    structure 'R', 'L' (below the diagonal) or 'U' (rows 0..i)."""
    rows, ncol = Y.shape
    nrow = rows if nrow is None else nrow
    tau = _torch().empty(ncol, dtype=_torch().float64, device=Y.device)
    py, ldy = _dev(Y, "Y")
    check(lib().candmc_tau_recon(structure.encode() if isinstance(structure, str) else structure, ncol, nrow,
                                 ldy, py, tau.data_ptr(), _stream(stream)), "tau_recon")
    return tau


def compute_invT_from_W(W, Y1, stream=None):
    """T^-T from W and Y1 (alg/QR/hh_recon/hh_recon.h:13-15): solves W^T X = -Y1."""
    b = W.shape[0]
    X = colmajor(Y1.clone())
    check(lib().candmc_compute_invT_from_W(_dev(W, "W")[0], b, _dev(X, "invT")[0], _stream(stream)),
          "compute_invT_from_W")
    return X


def _nlu(fn, A, R, stream):
    b = A.shape[0]
    signs = _torch().empty(b, dtype=_torch().int64, device=A.device)
    pa, lda = _dev(A, "A")
    pr, ldr = _dev(R, "R")
    check(fn(pa, pr, b, lda, ldr, signs.data_ptr(), _stream(stream)), "NLU")
    return signs


def signed_NLU(A, R, stream=None):
    """Sign-choice LU of (A - S) in place (alg/QR/hh_recon/hh_recon.h:27-36); returns signs."""
    return _nlu(lib().candmc_signed_NLU, A, R, stream)


def recursive_NLU(A, R, stream=None):
    """Recursive signed LU (alg/QR/hh_recon/hh_recon.h:38-49); returns signs."""
    return _nlu(lib().candmc_recursive_NLU, A, R, stream)


# ------------------------------------------------------------------ T factor
def compute_invT_from_Y(Y, T=None, stream=None):
    """T^-T = stril(Y^T Y), halved diagonal (alg/QR/qr_2d/qr_2d.h:25-31).  Writes the lower part of T."""
    mb, b = Y.shape
    T = _torch().zeros((b, b), dtype=_torch().float64, device=Y.device).t() if T is None else T
    py, ldy = _dev(Y, "Y")
    pt, ldt = _dev(T, "T")
    check(lib().candmc_compute_invT_from_Y(py, ldy, pt, ldt, mb, b, _stream(stream)), "compute_invT_from_Y")
    return T


def compute_invT_from_Y2(Y1, Y2, stream=None):
    """Y1^T Y2 (alg/QR/qr_2d/qr_2d.h:47-56)."""
    mb, b1 = Y1.shape
    b2 = Y2.shape[1]
    T = empty_colmajor(b1, b2, Y1.device)
    p1, l1 = _dev(Y1, "Y1")
    p2, l2 = _dev(Y2, "Y2")
    pt, ldt = _dev(T, "T")
    check(lib().candmc_compute_invT_from_Y2(p1, l1, p2, l2, pt, ldt, mb, b1, b2, _stream(stream)),
          "compute_invT_from_Y2")
    return T


# ------------------------------------------------------------------ CAQR
def upd_A(Y, A, W=None, W_is_T=False, precision="fp64", stream=None):
    """A <- (I - Y T Y^T)^T A (alg/QR/qr_2d/qr_2d.h:99-108); Y explicit (unit diagonal stored)."""
    mb, b = Y.shape
    kb = A.shape[1]
    py, ldy = _dev(Y, "Y")
    pa, lda = _dev(A, "A")
    pw = _dev(W, "W")[0] if W is not None else None
    check(lib().candmc_upd_A(py, ldy, pa, lda, mb, kb, b, pw, int(bool(W_is_T)), _prec(precision),
                             _stream(stream)), "upd_A")
    return A


def update_A(YR, A, b, W=None, aggreg_Y=None, W_is_T=False, precision="fp64", stream=None):
    """update_A (alg/QR/qr_2d/qr_2d.h:74-85): Y read from the Y\\R buffer YR (m x b)."""
    m, k = A.shape
    py, ldy = _dev(YR, "YR")
    pa, lda = _dev(A, "A")
    pw = _dev(W, "W")[0] if W is not None else None
    pg, ldg = _dev(aggreg_Y, "aggreg_Y") if aggreg_Y is not None else (None, 0)
    check(lib().candmc_update_A(py, ldy, pa, lda, m, k, b, pw, pg, ldg, int(bool(W_is_T)),
                                _prec(precision), _stream(stream)), "update_A")
    return A


def QR_2D(A, b, aggreg_Y=None, precision="fp64", stream=None):
    """Right-looking CAQR (alg/QR/qr_2d/qr_2d.h:124-131) on a 1 x 1 grid; A becomes Y\\R."""
    m, k = A.shape
    if isinstance(A, np.ndarray):
        pa, lda = _host(A, "A")
        check(lib().candmc_QR_2D_host(pa, lda, m, k, b, _prec(precision)), "QR_2D")
        return A
    pa, lda = _dev(A, "A")
    pg, ldg = _dev(aggreg_Y, "aggreg_Y") if aggreg_Y is not None else (None, 0)
    check(lib().candmc_QR_2D(pa, lda, m, k, b, pg, ldg, _prec(precision), _stream(stream)), "QR_2D")
    return A


def sym_full2band(A, b, b_sub=None, precision="fp64", stream=None):
    """Symmetric full -> band reduction (alg/SE/CANSE.h:17-22): A (n x n, lower
    triangle read) becomes Q^T A Q with bandwidth b in its lower triangle
    (reflectors below the band).  b_sub: the panel width of the CAQR of each
    band step (default b)."""
    n = A.shape[0]
    pa, lda = _dev(A, "A")
    check(lib().candmc_sym_full2band(pa, lda, n, b, b if b_sub is None else b_sub, _prec(precision),
                                     _stream(stream)), "sym_full2band")
    return A


def ls_solve(A, B, b=128, precision="fp64", max_refine=20, tol=1e-15, stream=None):
    """min ||A X - B||: CAQR in the given form, X0 = R^-1 Q^T B, FP64 refinement
    by corrected semi-normal equations (or of the augmented system with
    set_tuning("ls_refine", 1)).  Returns (X, stats) with stats =
    {"steps", "last_change", "first_change", "status"}."""
    import ctypes
    m, n = A.shape
    nrhs = B.shape[1]
    X = empty_colmajor(n, nrhs, A.device)
    pa, lda = _dev(A, "A")
    pb, ldb = _dev(B, "B")
    px, ldx = _dev(X, "X")
    st = (ctypes.c_double * 4)()
    check(lib().candmc_ls_solve(pa, lda, m, n, pb, ldb, nrhs, px, ldx, b, _prec(precision),
                                int(max_refine), float(tol), st, _stream(stream)), "ls_solve")
    return X, {"steps": int(st[0]), "last_change": st[1], "first_change": st[2],
               "status": int(st[3])}


def set_tuning(key, value):
    """Set a tuning knob of the library ("leaf_rows": target rows per TSQR leaf)."""
    check(lib().candmc_set_tuning(key.encode(), int(value)), "set_tuning")


def batched_ls(As, Bs, nstreams=16, use_graph=False, stream=None):
    """Solve min ||A_i x_i - b_i|| for lists of column-major CUDA tensors A_i (m_i x n_i,
    n_i <= 128) and b_i (m_i x 1).  A_i becomes Y\\R, b_i becomes Q^T b_i with
    x_i = b_i[:n_i].  Returns the list of x_i views."""
    import ctypes
    k = len(As)
    arr = lambda t, vals: (t * k)(*vals)
    ms = [a.shape[0] for a in As]
    ns = [a.shape[1] for a in As]
    pa = [_dev(a, "A")[0] for a in As]
    la = [_dev(a, "A")[1] for a in As]
    pb = [_dev(b, "B")[0] for b in Bs]
    check(lib().candmc_batched_ls(k, arr(ctypes.c_int64, ms), arr(ctypes.c_int64, ns),
                                  arr(ctypes.c_void_p, pa), arr(ctypes.c_int64, la),
                                  arr(ctypes.c_void_p, pb), int(nstreams), int(bool(use_graph)),
                                  _stream(stream)), "batched_ls")
    return [b[:n] for b, n in zip(Bs, ns)]


def batched_ls_f32(As, Bs, nstreams=16, use_graph=False, stream=None):
    """The float32-input variant of batched_ls: A_i (m_i x n_i, column-major
    float32 CUDA tensors) and b_i (m_i x 1, float32) are solved in FP64; b_i's
    first n_i entries become x_i (rounded to float32), A_i is left as it was."""
    import ctypes
    torch = _torch()
    k = len(As)
    arr = lambda t, vals: (t * k)(*vals)
    for a in As + Bs:
        if not (isinstance(a, torch.Tensor) and a.is_cuda and a.dtype == torch.float32):
            raise TypeError("batched_ls_f32: expected float32 CUDA tensors")
    ms = [a.shape[0] for a in As]
    ns = [a.shape[1] for a in As]
    la = []
    for a in As:
        if a.stride(0) != 1 and a.shape[0] > 1:
            raise ValueError("batched_ls_f32: A_i must be column-major")
        la.append(a.stride(1) if a.shape[1] > 1 else max(1, a.shape[0]))
    for b in Bs:
        if b.stride(0) != 1 and b.shape[0] > 1:
            raise ValueError("batched_ls_f32: b_i must be a contiguous column")
    check(lib().candmc_batched_ls_f32(k, arr(ctypes.c_int64, ms), arr(ctypes.c_int64, ns),
                                      arr(ctypes.c_void_p, [a.data_ptr() for a in As]), arr(ctypes.c_int64, la),
                                      arr(ctypes.c_void_p, [b.data_ptr() for b in Bs]), int(nstreams),
                                      int(bool(use_graph)), _stream(stream)), "batched_ls_f32")
    return [b[:n] for b, n in zip(Bs, ns)]


def batched_status(stream=None):
    """Wait for the stream and raise CandmcError if a batched call's kernels
    recorded a failure on this device since the last check (then cleared)."""
    import ctypes
    st = ctypes.c_int(0)
    check(lib().candmc_batched_status(_stream(stream), ctypes.byref(st)), "batched_status")
    check(st.value, "batched_ls (device status)")


def QR_2D_2D(A, b, b_sub, aggreg_Y=None, precision="fp64", stream=None):
    """Two-level blocked CAQR (alg/QR/qr_2d/qr_2d.h:176-188)."""
    m, k = A.shape
    pa, lda = _dev(A, "A")
    pg, ldg = _dev(aggreg_Y, "aggreg_Y") if aggreg_Y is not None else (None, 0)
    check(lib().candmc_QR_2D_2D(pa, lda, m, k, b, b_sub, pg, ldg, _prec(precision), _stream(stream)),
          "QR_2D_2D")
    return A


def Yamamoto(A, Qm=None, W=None, stream=None):
    """TSQR and Yamamoto's basis-kernel representation of an m x b panel
    (alg/QR/hh_recon/yamamoto.h:21-32).

    A becomes Y\\(S*R).  Returns (Qm, W) with Q^T = I + Qm W Qm^T; the pair
    equals the reference's up to the reference's own column signs (see
    candmc_Yamamoto in include/candmc_gb300.h).
    """
    m, b = A.shape
    Qm = empty_colmajor(m, b, A.device) if Qm is None else Qm
    W = empty_colmajor(b, b, A.device) if W is None else W
    pa, lda = _dev(A, "A")
    pq, ldq = _dev(Qm, "Qm")
    check(lib().candmc_Yamamoto(pa, lda, pq, ldq, m, b, _dev(W, "W")[0], _stream(stream)), "Yamamoto")
    return Qm, W


def upd_Yamamoto_A(Qm, A, W, precision="fp64", stream=None):
    """A += Qm (W (Qm^T A)) (alg/QR/qr_2d/qr_y2d.h:79-99)."""
    mb, b = Qm.shape
    kb = A.shape[1]
    pq, ldq = _dev(Qm, "Qm")
    pa, lda = _dev(A, "A")
    check(lib().candmc_upd_Yamamoto_A(pq, ldq, pa, lda, mb, kb, b, _dev(W, "W")[0], _prec(precision),
                                      _stream(stream)), "upd_Yamamoto_A")
    return A


class Aggregator:
    """The reference's aggregator (alg/QR/qr_2d/qr_y2d.h:4-44) on the device:
    aQm (lda_aQm x lda_aT) and the block-lower aT (lda_aT x lda_aT), zeroed."""

    def __init__(self, lda_aQm, lda_aT, device="cuda"):
        torch = _torch()
        self.lda_aQm, self.lda_aT = lda_aQm, lda_aT
        self.aQm = colmajor(torch.zeros(lda_aQm, lda_aT, dtype=torch.float64, device=device))
        self.aT = colmajor(torch.zeros(lda_aT, lda_aT, dtype=torch.float64, device=device))
        self.n = 0
        self.shift = 0

    def reset(self):
        self.aQm.zero_()
        self.aT.zero_()
        self.n = 0
        self.shift = 0

    def shift_down(self, b):
        self.shift += b

    def append(self, Qm, T, stream=None):
        mb, b = Qm.shape
        pq, ldq = _dev(Qm, "Qm")
        check(lib().candmc_yamamoto_append(self.aQm.data_ptr(), self.lda_aQm, self.aT.data_ptr(), self.lda_aT,
                                           self.n, self.shift, mb, b, pq, ldq, _dev(T, "T")[0],
                                           _stream(stream)), "aggregator append")
        self.n += b

    def _args(self):
        n, sh = ctypes.c_int64(self.n), ctypes.c_int64(self.shift)
        return n, sh, (self.aQm.data_ptr(), self.lda_aQm, self.aT.data_ptr(), self.lda_aT,
                       ctypes.byref(n), ctypes.byref(sh))


def QR_Yamamoto_2D(A, b, agg=None, compute_Y=False, precision="fp64", stream=None):
    """CAQR with Yamamoto's representation (alg/QR/qr_2d/qr_y2d.h:102-119)."""
    m, k = A.shape
    pa, lda = _dev(A, "A")
    if agg is None:
        rest = (None, 0, None, 0, None, None)
    else:
        n, sh, rest = agg._args()
    check(lib().candmc_QR_Yamamoto_2D(pa, lda, m, k, b, int(bool(compute_Y)), *rest, _prec(precision),
                                      _stream(stream)), "QR_Yamamoto_2D")
    if agg is not None:
        agg.n, agg.shift = n.value, sh.value
    return A


def QR_Yamamoto_2D_2D(A, b, b_sub, agg=None, compute_Y=False, precision="fp64", stream=None):
    """Two-level blocked CAQR with Yamamoto's representation (alg/QR/qr_2d/qr_y2d.h:122-139)."""
    m, k = A.shape
    pa, lda = _dev(A, "A")
    if agg is None:
        rest = (None, 0, None, 0, None, None)
    else:
        n, sh, rest = agg._args()
    check(lib().candmc_QR_Yamamoto_2D_2D(pa, lda, m, k, b, b_sub, int(bool(compute_Y)), *rest,
                                         _prec(precision), _stream(stream)), "QR_Yamamoto_2D_2D")
    if agg is not None:
        agg.n, agg.shift = n.value, sh.value
    return A


def QR_2D_pipe(A, b, precision="fp64", stream=None):
    """Lookahead CAQR (alg/QR/qr_2d/qr_2d.h:293-302): the same factorization on one GPU."""
    m, k = A.shape
    pa, lda = _dev(A, "A")
    check(lib().candmc_QR_2D_pipe(pa, lda, m, k, b, _prec(precision), _stream(stream)), "QR_2D_pipe")
    return A
