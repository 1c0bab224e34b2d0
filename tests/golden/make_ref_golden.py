"""Generate tests/golden/ref_golden.npz by running the reference itself.

The reference's QR sources are compiled unmodified (oracle/build_ref.py:
single-rank MPI, scipy's OpenBLAS) and called on a 1 x 1 grid through
oracle/ref.py.  Inputs are regenerated from seeds by the tests (numpy PCG64
draws and the reference tests' srand48 fixture are bit-identical on every
platform); only the one input that goes through a LAPACK QR to be built (the
Haar-based C2-type matrix) is stored.  Outputs are what the reference
returns.

Cases (key prefix -> reference function):
  hh/<name>/{YR,W}      hh_recon_qr          alg/QR/hh_recon/hh_recon.cxx:129-321
  c1/{R,W,Yrows,rows}   hh_recon_qr on 8192 x 64 N(0,1) seed 0 (R, W and a
                        sample of Y's rows)
  qr2d/<name>/YR        QR_2D / QR_2D_pipe / QR_2D_2D   alg/QR/qr_2d/qr_2d.cxx
  c2/{A,YR}             QR_2D_pipe of a 256 x 256 U diag(logspace(0,-6)) V^T, b = 128
  tree/<b>/{in,out,T}   tree_tsqr (dtpqrt)   alg/QR/tsqr/bitree_tsqr.cxx:20-34
  tsqr/{YR,R,tau,Q1,QtB} bitree_tsqr, construct_Q1, apply_tsqr_QT (one rank)
  tau/{L,U,R}           tau_recon            alg/shared/util.cxx:437-466
  yam/{A,Qm,W}          Yamamoto             alg/QR/hh_recon/yamamoto.cxx:98-174
  invT/{fromW,fromY,fromY2}                  hh_recon.cxx:26-31, qr_2d.cxx:22-106
  upd/{W,noW}           upd_A with T from W and from Y^T Y   qr_2d.cxx:224-282
  yam2d/YR              QR_Yamamoto_2D (compute_Y)           qr_y2d.cxx:172-273

Run (where the reference checkout exists):  python tests/golden/make_ref_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from oracle import build_ref, ref  # noqa: E402
from oracle.fixtures import drand48_fixture, gaussian, svd_matrix  # noqa: E402

# hh_recon_qr panels: (name, m, b, generator, seed); m is a multiple of b
PANELS = [
    ("d34x17", 34, 17, "drand48", 0),      # test_hh_recon default (b=17, m=34 per rank)
    ("d68x17", 68, 17, "drand48", 0),
    ("d136x17", 136, 17, "drand48", 0),
    ("d168x21", 168, 21, "drand48", 0),    # test_bitree_tsqr default shape (b=21, m=42*4)
    ("g256x32", 256, 32, "gauss", 101),
    ("g384x64", 384, 64, "gauss", 102),
    ("g256x128", 256, 128, "gauss", 103),
    ("g96x3", 96, 3, "gauss", 104),
]
# CAQR cases: (name, m, k, b, variant, b_sub, seed)
CAQR = [
    ("g192_b32", 192, 192, 32, "plain", None, 105),
    ("g192_b64_2d32", 192, 192, 64, "2d", 32, 105),
    ("g256x128_b32", 256, 128, 32, "plain", None, 106),
    ("g192x128_b64_pipe", 192, 128, 64, "pipe", None, 107),
]
C1_ROWS = np.concatenate([np.arange(128), np.arange(128, 8192, 61)])


def panel_input(m, b, gen, seed):
    return drand48_fixture(m, b) if gen == "drand48" else gaussian(m, b, seed)


def tree_input(b, seed):
    """[R1; R2] with random strictly-lower parts that dtpqrt must not read."""
    R1 = gaussian(b, b, seed)
    R2 = gaussian(b, b, seed + 1)
    return np.vstack([R1, R2])


def main():
    if build_ref.build(verbose=True) is None:
        raise SystemExit("the reference checkout is needed to generate these fixtures")
    out = {}
    for name, m, b, gen, seed in PANELS:
        YR, W = ref.hh_recon_qr(panel_input(m, b, gen, seed), b)
        out[f"hh/{name}/YR"] = YR
        out[f"hh/{name}/W"] = W
    YR, W = ref.hh_recon_qr(gaussian(8192, 64, 0), 64)
    out["c1/R"] = np.triu(YR[:64])
    out["c1/W"] = W
    out["c1/rows"] = C1_ROWS
    out["c1/Yrows"] = YR[C1_ROWS]
    for name, m, k, b, variant, b_sub, seed in CAQR:
        out[f"qr2d/{name}/YR"] = ref.QR_2D(gaussian(m, k, seed), b, variant, b_sub)
    A = np.asfortranarray(svd_matrix(256, 256, 1, 1e-6))
    out["c2/A"] = A
    out["c2/YR"] = ref.QR_2D(A, 128, "pipe")
    for b in (17, 32, 64):
        S = tree_input(b, 300 + b)
        A2, T = ref.tree_tsqr(S, b)
        out[f"tree/{b}/out"] = A2
        out[f"tree/{b}/T"] = T
    A = gaussian(256, 32, 400)
    YRt, R, tau = ref.bitree_tsqr(A, 32)
    out["tsqr/YR"], out["tsqr/R"], out["tsqr/tau"] = YRt, R, tau
    out["tsqr/Q1"] = ref.construct_Q1(YRt, tau, 32)
    out["tsqr/QtB"] = ref.apply_tsqr_QT(YRt, tau, gaussian(256, 8, 401), 32)
    YRh, _ = ref.hh_recon_qr(gaussian(256, 32, 406), 32)
    out["tau/L"] = ref.tau_recon("L", YRh)
    out["tau/U"] = ref.tau_recon("U", np.triu(out["tree/32/out"][32:]))
    out["tau/R"] = ref.tau_recon("R", YRh[32:])
    A2, Qm, Wy = ref.Yamamoto(gaussian(256, 32, 402), 32)
    out["yam/A"], out["yam/Qm"], out["yam/W"] = A2, Qm, Wy
    YRh, Wh = ref.hh_recon_qr(gaussian(256, 32, 403), 32)
    Y = np.tril(YRh, -1)
    Y[np.arange(32), np.arange(32)] = 1.0
    out["invT/fromW"] = ref.compute_invT_from_W(Wh, Y[:32])
    out["invT/fromY"] = ref.compute_invT_from_Y(Y, 32)
    out["invT/fromY2"] = ref.compute_invT_from_Y2(Y[:, :16], Y[:, 16:])
    C = gaussian(256, 48, 404)
    out["upd/W"] = ref.upd_A(Y, C, 32, Wh)
    out["upd/noW"] = ref.upd_A(Y, C, 32, None)
    out["yam2d/YR"] = ref.QR_Yamamoto_2D(gaussian(192, 96, 405), 32, compute_Y=True)
    dst = os.path.join(HERE, "ref_golden.npz")
    np.savez_compressed(dst, **out)
    print(f"wrote {dst}: {len(out)} arrays, {os.path.getsize(dst) / 1e6:.2f} MB")


if __name__ == "__main__":
    main()
