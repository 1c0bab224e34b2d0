"""Generate the golden vectors in tests/golden/golden.npz.

The reference (CANDMC) keeps no stored golden data: its QR tests regenerate
inputs from srand48 and compare against LAPACK on the gathered matrix
(test/QR/test_hh_recon.cxx:126-222).  All of its QR arithmetic is LAPACK,
called in this order on one rank:
    hh_recon_qr  -> dgeqrf (bitree_tsqr.cxx:62), dorgqr (construct_tsqr_Q.cxx:96),
                    signed LU, dtrsm (hh_recon.cxx:294-299)
    upd_A        -> dgemm, dtrsm, dgemm (qr_2d.cxx:259-275)
The Householder factor that reconstruction returns is the canonical one
(unit-lower Y, T with Q = I - Y T Y^T, R with the LAPACK sign convention), so
the golden vectors are LAPACK's own outputs on the reference fixtures,
produced here with scipy's LAPACK (OpenBLAS build; LAPACK >= 3.4 API):
    YR  = dgeqrf(A)          (Y strictly below, R on/above the diagonal)
    T   = dgeqrt(A, nb=b).T  (the full b x b triangular factor)
    W   = -T * Y1^T          (hh_recon.h:58 relation)
    QtC = dormqr('L','T')    (the CAQR trailing update Q^T C)
Run:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np
from scipy.linalg import lapack

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from oracle.fixtures import drand48_fixture, gaussian  # noqa: E402

# (name, m, b, generator) -- full-rank cases only (element-wise comparable).
# Inputs are regenerated from the generator and seed (panel_input); the
# trailing-update input C of panel i is gaussian(m, 16, 200 + i).
PANELS = [
    ("hh_34x17", 34, 17, "drand48"),        # test_hh_recon default at np=1 (b=17, m=34)
    ("hh_68x17", 68, 17, "drand48"),        # np=2
    ("hh_136x17", 136, 17, "drand48"),      # np=4
    ("hh_168x21", 168, 21, "drand48"),      # test_bitree_tsqr default at np=8 (b=21, m=42*4)
    ("hh_256x32", 256, 32, "gauss"),
    ("hh_384x64", 384, 64, "gauss"),
    ("hh_160x128", 160, 128, "gauss"),
]


def panel_input(m, b, gen, seed):
    if gen == "drand48":
        return drand48_fixture(m, b)
    return gaussian(m, b, seed)


def main():
    out = {}
    for i, (name, m, b, gen) in enumerate(PANELS):
        A = panel_input(m, b, gen, 100 + i)
        qr, tau, _, info = lapack.dgeqrf(A.copy())
        assert info == 0
        v, t, info = lapack.dgeqrt(b, A.copy())
        assert info == 0
        T = np.triu(t[:b, :b])
        Y1 = np.tril(qr[:b, :b], -1) + np.eye(b)
        W = -T @ Y1.T
        out[name + "/YR"] = qr
        out[name + "/tau"] = tau
        out[name + "/T"] = T
        out[name + "/W"] = np.triu(W)
        # trailing update C <- Q^T C for a random C (the CAQR update of one panel)
        C = gaussian(m, 16, 200 + i)
        qtc, _, info = lapack.dormqr('L', 'T', qr, tau, C.copy(), lwork=max(1, 64 * 16))
        assert info == 0
        out[name + "/QtC"] = qtc
    # a full CAQR (QR_2D) case, panel width 16.  The srand48 fixture is
    # numerically rank-deficient at this shape (its seeds are an arithmetic
    # progression of the LCG), so a Gaussian input is used for element-wise data.
    A = gaussian(192, 96, 7)
    qr, tau, _, info = lapack.dgeqrf(A.copy())
    assert info == 0
    out["qr2d_192x96_b16/YR"] = qr
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **out)
    print("wrote", os.path.join(HERE, "golden.npz"), len(out), "arrays")


if __name__ == "__main__":
    main()
