"""ctypes access to the reference's own QR functions, compiled unmodified.

TEST INFRASTRUCTURE ONLY.  oracle/build_ref.py compiles the reference's QR
sources (alg/shared, alg/QR/tsqr, alg/QR/hh_recon, alg/QR/qr_2d) with a
single-rank MPI and scipy's OpenBLAS into oracle/_ref/libcandmc_ref.so; this
module calls them on numpy arrays (column-major float64, copied in and out),
on a 1 x 1 process grid.  It exists only where the reference checkout was
present at build time: `available()` says whether it can be used.

Reference entry points wrapped (file:line of their declarations):
  tree_tsqr, local_tsqr, bitree_tsqr, construct_Q1, apply_tsqr_QT
                                      alg/QR/tsqr/bitree_tsqr.h:16-138
  tau_recon                           alg/shared/util.h:675-680
  signed_NLU, recursive_NLU, compute_invT_from_W, hh_recon_qr
                                      alg/QR/hh_recon/hh_recon.h:13-75
  Yamamoto                            alg/QR/hh_recon/yamamoto.h
  compute_invT_from_Y (x2), update_A, upd_A, QR_2D, QR_2D_2D, QR_2D_pipe
                                      alg/QR/qr_2d/qr_2d.h:25-302
  upd_Yamamoto_A, QR_Yamamoto_2D      alg/QR/qr_2d/qr_y2d.h:85-145
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_ref", "libcandmc_ref.so")
_lib = None
_P = ctypes.c_void_p
_I = ctypes.c_int64

_SIGS = {
    "ref_tree_tsqr": [_P, _P, _I, _P],
    "ref_local_tsqr": [_P, _P, _I, _I, _I, _P],
    "ref_bitree_tsqr": [_P, _I, _P, _P, _I, _I, _I, _P],
    "ref_construct_Q1": [_P, _I, _P, _P, _I, _I, _I, _I, _P],
    "ref_apply_tsqr_QT": [_P, _I, _P, _P, _I, _I, _I, _I, _P],
    "ref_tau_recon": [ctypes.c_char, _I, _I, _I, _P, _P],
    "ref_compute_invT_from_W": [_P, _I, _P],
    "ref_signed_NLU": [_P, _P, _I, _I, _I, _P],
    "ref_recursive_NLU": [_P, _P, _I, _I, _I, _P],
    "ref_hh_recon_qr": [_P, _I, _I, _I, _P],
    "ref_Yamamoto": [_P, _I, _P, _I, _I, _I, _P],
    "ref_compute_invT_from_Y": [_P, _I, _P, _I, _I, _I],
    "ref_compute_invT_from_Y2": [_P, _I, _P, _I, _P, _I, _I, _I, _I],
    "ref_update_A": [_P, _I, _P, _I, _I, _I, _I, _P, _I],
    "ref_upd_A": [_P, _I, _P, _I, _I, _I, _I, _P, _I],
    "ref_QR_2D": [_P, _I, _I, _I, _I],
    "ref_QR_2D_pipe": [_P, _I, _I, _I, _I],
    "ref_QR_2D_2D": [_P, _I, _I, _I, _I, _I],
    "ref_QR_Yamamoto_2D": [_P, _I, _I, _I, _I, _I],
    "ref_QR_Yamamoto_2D_2D": [_P, _I, _I, _I, _I, _I, _I],
    "ref_upd_Yamamoto_A": [_P, _I, _P, _I, _I, _I, _I, _P],
}


def available():
    return os.path.exists(LIB)


def lib():
    global _lib
    if _lib is None:
        if not available():
            raise RuntimeError("oracle/_ref/libcandmc_ref.so is not built (python -m oracle.build_ref)")
        _lib = ctypes.CDLL(LIB)
        for name, args in _SIGS.items():
            f = getattr(_lib, name)
            f.argtypes = args
            f.restype = None
    return _lib


def _f(a):
    return np.array(a, dtype=np.float64, order="F", copy=True)


def _p(a):
    return _P(a.ctypes.data) if a is not None else _P(0)


# ---- alg/QR/tsqr
def tree_tsqr(A, b):
    """dtpqrt of the stacked [R1; R2] (2b x b, ld 2b).  Returns (A_out, T) with
    T the min(b,16) x b block-reflector factor (bitree_tsqr.cxx:20-34)."""
    A = _f(A)
    assert A.shape == (2 * b, b)
    nb = min(b, 16)
    T = np.zeros((nb, b), order="F")
    buf = np.zeros(2 * b * b)
    lib().ref_tree_tsqr(_p(A), _p(buf), b, _p(T))
    return A, T


def bitree_tsqr(A, b, output_Y=True):
    """Single-rank bitree_tsqr: leaf dgeqrf.  Returns (A_out, R, tau)."""
    A = _f(A)
    m = A.shape[0]
    R = np.zeros((b, b), order="F")
    tau = np.zeros(b)
    lib().ref_bitree_tsqr(_p(A), m, _p(R), _p(tau), m, b, 1 if output_Y else 0, None)
    return A, R, tau


def construct_Q1(Y, tau, b, k=None):
    Y = _f(Y)
    m = Y.shape[0]
    k = b if k is None else k
    Q1 = np.zeros((m, k), order="F")
    tau = np.ascontiguousarray(tau, dtype=np.float64)
    lib().ref_construct_Q1(_p(Y), m, _p(tau), _p(Q1), m, m, b, k, None)
    return Q1


def apply_tsqr_QT(Y, tau, B, b):
    Y, B = _f(Y), _f(B)
    m, k = B.shape
    tau = np.ascontiguousarray(tau, dtype=np.float64)
    lib().ref_apply_tsqr_QT(_p(Y), Y.shape[0], _p(tau), _p(B), m, m, b, k, None)
    return B


def tau_recon(structure, Y, nrow=None):
    """util.cxx:437-466: tau from Householder vectors ('R', 'L' or 'U')."""
    Y = _f(Y)
    rows, ncol = Y.shape
    tau = np.zeros(ncol)
    lib().ref_tau_recon(structure.encode(), ncol, rows if nrow is None else nrow, rows, _p(Y), _p(tau))
    return tau


# ---- alg/QR/hh_recon
def hh_recon_qr(A, b):
    """Returns (Y\\(S R), W) for an m x b panel, m a multiple of b (the
    reference's row split, bitree_tsqr.cxx:110, drops rows otherwise)."""
    A = _f(A)
    m = A.shape[0]
    assert m % b == 0, "the reference factors ((m/b)/p)*b rows"
    W = np.zeros((b, b), order="F")
    lib().ref_hh_recon_qr(_p(A), m, m, b, _p(W))
    return A, W


def compute_invT_from_W(W, Y1):
    """T^-T from W and the unit-lower Y1 passed in invT (hh_recon.cxx:26-31)."""
    W = _f(W)
    b = W.shape[0]
    X = _f(Y1)
    lib().ref_compute_invT_from_W(_p(W), b, _p(X))
    return X


def signed_NLU(A, R, recursive=False):
    A, R = _f(A), _f(R)
    b = A.shape[0]
    signs = np.zeros(b, dtype=np.int64)
    fn = lib().ref_recursive_NLU if recursive else lib().ref_signed_NLU
    fn(_p(A), _p(R), b, b, b, signs.ctypes.data_as(_P))
    return A, R, signs


def Yamamoto(A, b):
    A = _f(A)
    m = A.shape[0]
    Qm = np.zeros((m, b), order="F")
    W = np.zeros((b, b), order="F")
    lib().ref_Yamamoto(_p(A), m, _p(Qm), m, m, b, _p(W))
    return A, Qm, W


# ---- alg/QR/qr_2d
def compute_invT_from_Y(Y, b):
    Y = _f(Y)
    T = np.zeros((b, b), order="F")
    lib().ref_compute_invT_from_Y(_p(Y), Y.shape[0], _p(T), b, Y.shape[0], b)
    return T


def compute_invT_from_Y2(Y1, Y2):
    Y1, Y2 = _f(Y1), _f(Y2)
    b1, b2 = Y1.shape[1], Y2.shape[1]
    T = np.zeros((b1, b2), order="F")
    lib().ref_compute_invT_from_Y2(_p(Y1), Y1.shape[0], _p(Y2), Y2.shape[0], _p(T), b1, Y1.shape[0], b1, b2)
    return T


def upd_A(Ybuf, A, b, W=None, W_is_T=False):
    """A <- (I - Y T Y^T)^T A with Ybuf the explicit unit-lower Y (qr_2d.cxx:224-282);
    T from W (W given) or from Y^T Y (W None)."""
    Ybuf, A = _f(Ybuf), _f(A)
    mb, kb = A.shape
    W = None if W is None else _f(W)
    lib().ref_upd_A(_p(Ybuf), Ybuf.shape[0], _p(A), mb, mb, kb, b, _p(W), 1 if W_is_T else 0)
    return A


def update_A(Y, A, b, W=None):
    """update_A with Y read from a Y\\R buffer (qr_2d.cxx:124-177)."""
    Y, A = _f(Y), _f(A)
    m, k = A.shape
    W = None if W is None else _f(W)
    lib().ref_update_A(_p(Y), Y.shape[0], _p(A), m, m, k, b, _p(W), 0)
    return A


def QR_2D(A, b, variant="plain", b_sub=None):
    """In-place CAQR on a 1 x 1 grid: variant 'plain' (QR_2D), 'pipe'
    (QR_2D_pipe) or '2d' (QR_2D_2D with inner block b_sub)."""
    A = _f(A)
    m, k = A.shape
    if variant == "plain":
        lib().ref_QR_2D(_p(A), m, m, k, b)
    elif variant == "pipe":
        lib().ref_QR_2D_pipe(_p(A), m, m, k, b)
    elif variant == "2d":
        lib().ref_QR_2D_2D(_p(A), m, m, k, b, b_sub)
    else:
        raise ValueError(variant)
    return A


def QR_Yamamoto_2D(A, b, compute_Y=True, b_sub=None):
    A = _f(A)
    m, k = A.shape
    if b_sub is None:
        lib().ref_QR_Yamamoto_2D(_p(A), m, m, k, b, 1 if compute_Y else 0)
    else:
        lib().ref_QR_Yamamoto_2D_2D(_p(A), m, m, k, b, b_sub, 1 if compute_Y else 0)
    return A


def upd_Yamamoto_A(Qm, A, b, T):
    Qm, A, T = _f(Qm), _f(A), _f(T)
    mb, kb = A.shape
    lib().ref_upd_Yamamoto_A(_p(Qm), Qm.shape[0], _p(A), mb, mb, kb, b, _p(T))
    return A


def blas_threads():
    """Threads of the OpenBLAS the reference is linked against (the same
    library scipy loads, so one setting governs both)."""
    from . import reference_lapack as rl
    return rl.blas_threads()
