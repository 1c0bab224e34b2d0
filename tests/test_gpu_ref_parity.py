"""Parity of the CUDA path with the reference's own outputs.

tests/golden/ref_golden.npz holds what the reference's QR sources, compiled
unmodified (oracle/build_ref.py), return on seeded inputs; every call below
goes through the library's C ABI on cuda:0 and is held to those outputs
element-wise.  Tolerances: the Householder factor (Y, T, S*R) is canonical,
so two FP64 implementations agree to ELEM_TOL * max(1, b/16) relative to the
largest entry; for the C2-type input (singular values down to 1e-6) R is held
to the same bound and the reflectors of the trailing columns, which move by
up to kappa * u under rounding, to kappa * 1e-15.  The emulated-FP64 (Ozaki)
form is held to the same bounds: it is meant to be FP64-accurate.

Also here, the benchmark panel (8192 x 64, N(0,1), seed 0) in full, with its
backward error and orthogonality, and an emulated-FP64 CAQR at n = 4096 on the
C2 generator against the reference's call sequence (oracle/reference_lapack.py,
bitwise the reference where both exist).
"""
import os

import numpy as np
import pytest

from oracle import candmc_oracle as co
from oracle import fixtures as fx
from oracle import lapack_restated as lp
from tests.golden.make_ref_golden import C1_ROWS, CAQR, PANELS, panel_input, tree_input

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ELEM_TOL = 2e-12
BWD_TOL = 1e-13


@pytest.fixture(scope="module")
def cm():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import candmc_gb300 as cm
    cm.lib()
    return cm


@pytest.fixture(scope="module")
def rg():
    return np.load(os.path.join(ROOT, "tests", "golden", "ref_golden.npz"))


def dev(a):
    return torch.from_numpy(np.asfortranarray(a)).cuda().t().contiguous().t()


def host(t):
    torch.cuda.synchronize()
    return np.asfortranarray(t.cpu().numpy())


def close(got, want, b, k=1.0):
    err = np.abs(np.asarray(got) - want).max()
    assert err <= k * ELEM_TOL * max(1.0, b / 16) * max(1.0, np.abs(want).max()), err


@pytest.mark.parametrize("name,m,b,gen,seed", PANELS)
def test_hh_recon_is_the_reference(cm, rg, name, m, b, gen, seed):
    dA = dev(panel_input(m, b, gen, seed))
    W, T = cm.hh_recon_qr(dA)
    close(host(dA), rg[f"hh/{name}/YR"], b)
    close(np.triu(host(W)), np.triu(rg[f"hh/{name}/W"]), b)


def test_tsqr_hr_benchmark_panel(cm, rg):
    """hh_recon_qr of the 8192 x 64 N(0,1) panel from seed 0: R, W and sampled
    Y rows against the reference, ||A - QR||/||A|| and ||I - Q^T Q|| in full."""
    A = fx.gaussian(8192, 64, 0)
    dA = dev(A)
    W, T = cm.hh_recon_qr(dA)
    YR, Th = host(dA), host(T)
    close(np.triu(YR[:64]), rg["c1/R"], 64)
    close(np.triu(host(W)), np.triu(rg["c1/W"]), 64)
    close(YR[C1_ROWS], rg["c1/Yrows"], 64)
    Y = lp.unit_lower(YR, 64)
    QR = np.vstack([np.triu(YR[:64]), np.zeros((8192 - 64, 64))])
    QR -= Y @ (Th @ (Y.T @ QR))
    assert np.linalg.norm(QR - A) / np.linalg.norm(A) <= BWD_TOL
    E = np.eye(8192, 64) - Y @ (Th @ Y[:64].T)
    assert np.linalg.norm(E.T @ E - np.eye(64)) <= 1e-13


@pytest.mark.parametrize("form", ["fp64", "ozaki"])
@pytest.mark.parametrize("name,m,k,b,variant,b_sub,seed", CAQR)
def test_caqr_is_the_reference(cm, rg, name, m, k, b, variant, b_sub, seed, form):
    if variant == "2d" and form != "fp64":
        pytest.skip("QR_2D_2D is checked in FP64")
    dA = dev(fx.gaussian(m, k, seed))
    if variant == "plain":
        cm.QR_2D(dA, b, precision=form)
    elif variant == "pipe":
        cm.QR_2D_pipe(dA, b, precision=form)
    else:
        cm.QR_2D_2D(dA, b, b_sub, precision=form)
    close(host(dA), rg[f"qr2d/{name}/YR"], b, k=4.0)


@pytest.mark.parametrize("form", ["fp64", "ozaki"])
def test_c2_type_caqr_is_the_reference(cm, rg, form):
    A = rg["c2/A"]
    dA = dev(A)
    cm.QR_2D_pipe(dA, 128, precision=form)
    YR, want = host(dA), rg["c2/YR"]
    close(np.triu(YR), np.triu(want), 128)
    assert np.abs(np.tril(YR, -1) - np.tril(want, -1)).max() <= 1e6 * 1e-15
    assert co.backward_error(A, YR) <= BWD_TOL


@pytest.mark.parametrize("b", [17, 32, 64])
def test_tree_tsqr_is_the_reference(cm, rg, b):
    """dtpqrt's contract: only the two upper triangles are read and written."""
    S = tree_input(b, 300 + b)
    dA = dev(S)
    T = cm.tree_tsqr(dA)
    out, want = host(dA), rg[f"tree/{b}/out"]
    assert np.array_equal(np.tril(out[:b], -1), np.tril(S[:b], -1))
    assert np.array_equal(np.tril(out[b:], -1), np.tril(S[b:], -1))
    close(np.triu(out[:b]), np.triu(want[:b]), b)
    close(np.triu(out[b:]), np.triu(want[b:]), b)
    close(host(T), rg[f"tree/{b}/T"], b)


def test_tree_tsqr_ignores_lower_garbage(cm):
    """Non-finite values below the diagonals are never read."""
    b = 24
    S = tree_input(b, 77)
    G = S.copy()
    G[np.tril_indices(b, -1)] = np.nan
    lo = (np.tril_indices(b, -1)[0] + b, np.tril_indices(b, -1)[1])
    G[lo] = np.inf
    d1, d2 = dev(S), dev(G)
    cm.tree_tsqr(d1)
    cm.tree_tsqr(d2)
    o1, o2 = host(d1), host(d2)
    assert np.array_equal(np.triu(o1[:b]), np.triu(o2[:b]))
    assert np.array_equal(np.triu(o1[b:]), np.triu(o2[b:]))
    assert np.all(np.isnan(o2[np.tril_indices(b, -1)])) and np.all(np.isinf(o2[lo]))


def test_single_rank_tsqr_is_the_reference(cm, rg):
    """bitree_tsqr, construct_Q1 and apply_tsqr_QT element-wise."""
    dA = dev(fx.gaussian(256, 32, 400))
    R, tau = cm.bitree_tsqr(dA)
    close(host(dA), rg["tsqr/YR"], 32)
    close(host(R), rg["tsqr/R"], 32)
    close(tau.cpu().numpy(), rg["tsqr/tau"], 32)
    close(host(cm.construct_Q1(dA, tau)), rg["tsqr/Q1"], 32)
    dB = dev(fx.gaussian(256, 8, 401))
    cm.apply_tsqr_QT(dA, tau, dB)
    close(host(dB), rg["tsqr/QtB"], 32)


def test_tau_recon_is_the_reference(cm, rg):
    """tau_recon's three structures (util.cxx:437-466)."""
    dA = dev(fx.gaussian(256, 32, 406))
    cm.hh_recon_qr(dA)
    YRh = host(dA)
    close(cm.tau_recon("L", dA).cpu().numpy(), rg["tau/L"], 32)
    close(cm.tau_recon("U", dev(np.triu(rg["tree/32/out"][32:]))).cpu().numpy(), rg["tau/U"], 32)
    close(cm.tau_recon("R", dev(YRh[32:])).cpu().numpy(), rg["tau/R"], 32)
    # an empty reflector maps to 0, as in the reference
    assert cm.tau_recon("L", dev(np.eye(4))).cpu().numpy().tolist() == [0.0, 0.0, 0.0, 0.0]


def test_yamamoto_is_the_reference(cm, rg):
    """The pair equals the reference's up to the reference's column signs d:
    Qm = Qm_ref d, W = d W_ref d, and the panel's Y\\(S R) is the same."""
    dA = dev(fx.gaussian(256, 32, 402))
    Qm, W = cm.Yamamoto(dA)
    Qm, W = host(Qm), host(W)
    d = np.where(np.sum(Qm * rg["yam/Qm"], axis=0) >= 0, 1.0, -1.0)
    close(host(dA), rg["yam/A"], 32)
    close(Qm, rg["yam/Qm"] * d[None, :], 32)
    close(W, d[:, None] * rg["yam/W"] * d[None, :], 32, k=10.0)


def test_T_forms_and_update_are_the_reference(cm, rg):
    dA = dev(fx.gaussian(256, 32, 403))
    W, _ = cm.hh_recon_qr(dA)
    Y = lp.unit_lower(host(dA), 32)
    dY = dev(Y)
    close(host(cm.compute_invT_from_W(W, dev(Y[:32]))), rg["invT/fromW"], 32)
    close(np.tril(host(cm.compute_invT_from_Y(dY))), np.tril(rg["invT/fromY"]), 32)
    close(host(cm.compute_invT_from_Y2(dev(Y[:, :16]), dev(Y[:, 16:]))), rg["invT/fromY2"], 32)
    C = fx.gaussian(256, 48, 404)
    for form in ("fp64", "ozaki"):
        close(host(cm.upd_A(dY, dev(C), W, precision=form)), rg["upd/W"], 32)
        close(host(cm.upd_A(dY, dev(C), None, precision=form)), rg["upd/noW"], 32)


def test_yamamoto_caqr_is_the_reference(cm, rg):
    dA = dev(fx.gaussian(192, 96, 405))
    cm.QR_Yamamoto_2D(dA, 32, compute_Y=True)
    close(host(dA), rg["yam2d/YR"], 32, k=4.0)


def test_ozaki_caqr_n4096_c2_input_is_the_reference():
    """Emulated-FP64 QR_2D_pipe of a 4096 x 4096 U diag(logspace(0,-6)) V^T
    (U, V Haar from seed 1), b = 128, against the reference's QR_2D call
    sequence on the same bytes: R element-wise, the trailing reflectors to
    kappa * 1e-15, and the full backward error and orthogonality."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import candmc_gb300 as cm
    from oracle import reference_lapack as rl
    n, b = 4096, 128
    A = np.asfortranarray(fx.svd_matrix(n, n, 1, 1e-6))
    want = np.array(A, order="F")
    rl.QR_2D_lapack(want, b)
    dA = dev(A)
    cm.QR_2D_pipe(dA, b, precision="ozaki")
    YR = host(dA)
    close(np.triu(YR), np.triu(want), b)
    assert np.abs(np.tril(YR, -1) - np.tril(want, -1)).max() <= 1e6 * 1e-15
    dA0 = dev(A)
    R = torch.triu(torch.from_numpy(YR).cuda())
    X = R.clone()
    YRd = dev(YR)
    for r0 in range(n - b, -1, -b):          # Q R = H_0 ... H_last R
        Y = torch.tril(YRd[r0:, r0:r0 + b], -1)
        Y[torch.arange(b), torch.arange(b)] = 1.0
        Yh = Y.cpu().numpy()
        T = torch.from_numpy(lp.dlarft(Yh, co.tau_recon_lower(Yh, b))).cuda()
        X[r0:] -= Y @ (T @ (Y.t() @ X[r0:]))
    bwd = float(torch.linalg.norm(X - dA0) / torch.linalg.norm(dA0))
    assert bwd <= BWD_TOL, bwd
