"""Parity of the CUDA path with the oracle and the golden vectors (FP64 forms).

Each test calls the library through its C ABI (candmc_gb300 -> ctypes) on
cuda:0 and compares with the oracle restatement / LAPACK golden outputs on
the same seeded inputs.  Tolerances: the Householder factor is canonical, so
Y, R, T, W agree element-wise to a few ulps times the panel width
(ELEM_TOL * max(1, b/16) relative to the largest entry); factorizations are
also held to the reference tests' criteria (test_hh_recon.cxx:251-264 and
test_qr_2d.cxx:285-301: column-relative residual <= 1e-9) and to the stated
backward-error bound of the FP64 form, ||A - QR||/||A|| <= 1e-13.
"""
import numpy as np
import pytest

from oracle import candmc_oracle as co
from oracle import fixtures as fx
from oracle import lapack_restated as lp
from tests.golden.make_golden import PANELS, panel_input

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

ELEM_TOL = 2e-12
BWD_TOL = 1e-13


@pytest.fixture(scope="module")
def cm():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import candmc_gb300 as cm
    cm.lib()
    return cm


def dev(a):
    return torch.from_numpy(np.asfortranarray(a)).cuda().t().contiguous().t() if a.ndim == 2 else \
        torch.from_numpy(a).cuda()


def host(t):
    return np.asfortranarray(t.cpu().numpy())


def tol(b, scale=1.0):
    return ELEM_TOL * max(1.0, b / 16) * max(1.0, scale)


@pytest.mark.parametrize("name,m,b,gen", PANELS)
def test_hh_recon_golden(cm, golden, name, m, b, gen):
    i = [p[0] for p in PANELS].index(name)
    A = panel_input(m, b, gen, 100 + i)
    dA = dev(A)
    W, T = cm.hh_recon_qr(dA)
    torch.cuda.synchronize()
    YR = host(dA)
    g = golden[name + "/YR"]
    assert np.abs(YR - g).max() <= tol(b, np.abs(g).max())
    assert np.abs(host(W) - golden[name + "/W"]).max() <= tol(b)
    assert np.abs(host(T) - golden[name + "/T"]).max() <= tol(b)
    assert co.column_relative_residual(A, YR, b) <= 1e-9


@pytest.mark.parametrize("m,b", [(1, 1), (5, 1), (2, 2), (3, 3), (17, 17), (34, 17), (100, 7),
                                  (64, 32), (65, 32), (1000, 33), (333, 48), (640, 64), (129, 128),
                                  (4096, 128), (8192, 64), (3000, 100), (70000, 16)])
def test_hh_recon_vs_oracle(cm, m, b):
    A = fx.gaussian(m, b, 1000 + m + b)
    YRo, Wo = co.hh_recon_qr(A, b)
    dA = dev(A)
    W, T = cm.hh_recon_qr(dA)
    torch.cuda.synchronize()
    YR = host(dA)
    D = np.abs(YR - YRo)
    if m == b:   # last reflector of a square panel: reconstruction's tau = 2 choice matches the oracle
        pass
    assert D.max() <= tol(b, np.abs(YRo).max()), D.max()
    assert np.abs(host(W) - Wo).max() <= tol(b)
    Y = lp.unit_lower(YR, b)
    To = co.T_from_W(Wo, lp.unit_lower(YRo, b)[:b])
    assert np.abs(host(T) - To).max() <= tol(b)
    assert co.orthogonality_error(YR, b) <= 1e-13 * max(1, b / 8)
    assert co.backward_error(A, YR) <= BWD_TOL


@pytest.mark.parametrize("m,b,pipe", [(300000, 32, 1), (70000, 32, 0), (40000, 24, 1)])
def test_hh_recon_many_leaves(cm, m, b, pipe):
    """Panels with hundreds to thousands of leaves: the Y formation takes each
    leaf's path product from the top-down pass over the tree nodes.  Covers the
    level-by-level tree (more than 4096 tree CTAs, or pipe_tree 0) and the
    pipelined one; same bars as test_hh_recon_vs_oracle."""
    A = fx.gaussian(m, b, 7 * m + b)
    YRo, Wo = co.hh_recon_qr(A, b)
    dA = dev(A)
    try:
        cm.set_tuning("pipe_tree", pipe)
        W, T = cm.hh_recon_qr(dA)
        torch.cuda.synchronize()
    finally:
        cm.set_tuning("pipe_tree", 1)
    YR = host(dA)
    assert np.abs(YR - YRo).max() <= tol(b, np.abs(YRo).max())
    assert np.abs(host(W) - Wo).max() <= tol(b)
    To = co.T_from_W(Wo, lp.unit_lower(YRo, b)[:b])
    assert np.abs(host(T) - To).max() <= tol(b)
    assert co.backward_error(A, YR) <= BWD_TOL


@pytest.mark.parametrize("m,b", [(34, 17), (68, 17), (136, 17), (42, 21), (8 * 21, 21)])
def test_hh_recon_reference_fixture(cm, m, b):
    """The reference test's own fixture and pass criterion (test_hh_recon.cxx)."""
    A = fx.drand48_fixture(m, b)
    dA = dev(A)
    cm.hh_recon_qr(dA)
    torch.cuda.synchronize()
    YR = host(dA)
    assert co.column_relative_residual(A, YR, b) <= 1e-9
    assert co.backward_error(A, YR) <= BWD_TOL


def test_hh_recon_host_entry(cm):
    A = fx.gaussian(500, 40, 3)
    YRo, Wo = co.hh_recon_qr(A, 40)
    Ah = np.asfortranarray(A.copy())
    W, T = cm.hh_recon_qr(Ah)
    assert np.abs(Ah - YRo).max() <= tol(40, np.abs(YRo).max())
    assert np.abs(W - Wo).max() <= tol(40)


def test_hh_recon_leading_dimension(cm):
    m, b, lda = 300, 24, 317
    A = fx.gaussian(m, b, 9)
    big = torch.zeros((b, lda), dtype=torch.float64, device="cuda").t()   # lda x b column-major
    big[:m, :] = torch.from_numpy(A).cuda()
    sub = big[:m, :]
    cm.hh_recon_qr(sub)
    torch.cuda.synchronize()
    YRo, _ = co.hh_recon_qr(A, b)
    out = host(big)
    assert np.abs(out[:m] - YRo).max() <= tol(b, np.abs(YRo).max())
    assert np.all(out[m:] == 0.0)


@pytest.mark.parametrize("m,k,b", [(192, 96, 16), (256, 256, 32), (300, 200, 64), (512, 384, 128),
                                   (1024, 1024, 128), (150, 100, 17)])
def test_QR_2D_vs_oracle(cm, golden, m, k, b):
    A = fx.gaussian(m, k, 7) if (m, k) == (192, 96) else fx.gaussian(m, k, m + k + b)
    Ao = A.copy()
    co.QR_2D(Ao, b)
    dA = dev(A)
    cm.QR_2D(dA, b)
    torch.cuda.synchronize()
    YR = host(dA)
    D = np.abs(YR - Ao)
    if m == k:
        D[-1, -1] = abs(abs(YR[-1, -1]) - abs(Ao[-1, -1]))
    assert D.max() <= 1e-11 * max(1, k / 64) * np.abs(Ao).max()
    if (m, k, b) == (192, 96, 16):
        assert np.abs(YR - golden["qr2d_192x96_b16/YR"]).max() <= 1e-11
    assert co.backward_error(A, YR) <= BWD_TOL


@pytest.mark.parametrize("m,k,b", [(8, 4, 2), (64, 64, 16), (96, 64, 16), (40, 40, 8)])
def test_QR_2D_reference_fixture(cm, m, k, b):
    """test_qr_2d's drand48-0.5 fixture (numerically rank-deficient at these shapes):
    the reference's criterion is the backward error."""
    A = fx.drand48_fixture(m, k, offset=0.5)
    dA = dev(A)
    cm.QR_2D(dA, b)
    torch.cuda.synchronize()
    assert co.backward_error(A, host(dA)) <= BWD_TOL


def test_QR_2D_host_and_pipe_and_2d2d(cm):
    A = fx.gaussian(400, 300, 11)
    Ao = A.copy()
    co.QR_2D(Ao, 32)
    Ah = np.asfortranarray(A.copy())
    cm.QR_2D(Ah, 32)
    assert np.abs(Ah - Ao).max() <= 1e-11 * np.abs(Ao).max()
    dA = dev(A)
    cm.QR_2D_pipe(dA, 32)
    torch.cuda.synchronize()
    assert np.abs(host(dA) - Ao).max() <= 1e-11 * np.abs(Ao).max()
    dA = dev(A)
    cm.QR_2D_2D(dA, 64, 32)
    torch.cuda.synchronize()
    assert np.abs(host(dA) - Ao).max() <= 1e-11 * np.abs(Ao).max()
    assert co.backward_error(A, host(dA)) <= BWD_TOL


@pytest.mark.parametrize("name,m,b,gen", PANELS)
def test_upd_A_three_T_forms(cm, golden, name, m, b, gen):
    i = [p[0] for p in PANELS].index(name)
    YR = golden[name + "/YR"]
    Wg = golden[name + "/W"]
    C = fx.gaussian(m, 16, 200 + i)
    want = golden[name + "/QtC"]
    Y = lp.unit_lower(YR, b)
    scale = np.abs(C).max()
    for W, is_T in [(Wg, False), (None, False), (co.compute_invT_from_W(Wg, Y[:b]), True)]:
        dC = dev(C)
        cm.upd_A(dev(Y), dC, None if W is None else dev(W), W_is_T=is_T)
        torch.cuda.synchronize()
        assert np.abs(host(dC) - want).max() <= 1e-11 * max(1, b / 16) * scale
    # update_A reads Y from the Y\R buffer and can aggregate Y
    dC = dev(C)
    agg = dev(np.zeros((m, b)))
    cm.update_A(dev(YR), dC, b, dev(Wg), aggreg_Y=agg)
    torch.cuda.synchronize()
    assert np.abs(host(dC) - want).max() <= 1e-11 * max(1, b / 16) * scale
    assert np.array_equal(host(agg), Y)


def test_invT_and_nlu_and_bitree(cm, golden):
    name, m, b = "hh_384x64", 384, 64
    YR, Wg, Tg = golden[name + "/YR"], golden[name + "/W"], golden[name + "/T"]
    Y = lp.unit_lower(YR, b)
    X = host(cm.compute_invT_from_W(dev(Wg), dev(Y[:b].copy())))
    assert np.abs(X - co.compute_invT_from_W(Wg, Y[:b])).max() <= 1e-11
    Xy = host(cm.compute_invT_from_Y(dev(Y)))
    assert np.abs(np.tril(Xy) - co.compute_invT_from_Y(Y)).max() <= 1e-11
    G = host(cm.compute_invT_from_Y2(dev(Y[:, :20].copy()), dev(Y[:, 20:].copy())))
    assert np.abs(G - Y[:, :20].T @ Y[:, 20:]).max() <= 1e-11
    # signed LU on a Q1_top-like block
    A = fx.gaussian(b, b, 5)
    Q, _ = np.linalg.qr(A)
    R = np.triu(fx.gaussian(b, b, 6))
    Qo, Ro = Q.copy(), R.copy()
    so = co.recursive_NLU(Qo, Ro)
    for fn in (cm.signed_NLU, cm.recursive_NLU):
        dQ, dR = dev(Q), dev(R)
        s = fn(dQ, dR).cpu().numpy()
        torch.cuda.synchronize()
        assert np.array_equal(s, so)
        assert np.abs(host(dQ) - Qo).max() <= 1e-11
        assert np.abs(host(dR) - Ro).max() <= 1e-12
    # bitree_tsqr (numPes = 1) and construct_Q1 (dorgqr)
    A = fx.gaussian(m, b, 100 + 5)
    dA = dev(A)
    R, tau = cm.bitree_tsqr(dA)
    torch.cuda.synchronize()
    assert np.abs(host(dA) - golden[name + "/YR"]).max() <= tol(b, np.abs(YR).max())
    assert np.abs(tau.cpu().numpy() - golden[name + "/tau"]).max() <= 1e-12
    assert np.abs(host(R) - np.triu(YR[:b])).max() <= tol(b, np.abs(YR).max())
    Q1 = host(cm.construct_Q1(dA, tau))
    Qo = lp.dorg2r(YR.copy(), golden[name + "/tau"])
    assert np.abs(Q1 - Qo).max() <= 1e-12 * max(1, b / 16)
    A2 = dev(A)
    R2, tau2 = cm.bitree_tsqr(A2, output_Y=0)
    torch.cuda.synchronize()
    assert np.array_equal(host(A2), A)


def test_errors_are_raised(cm):
    with pytest.raises(cm.CandmcError):
        cm.hh_recon_qr(dev(fx.gaussian(10, 20, 1)))   # m < b
    with pytest.raises(cm.CandmcError):
        cm.QR_2D(dev(fx.gaussian(10, 20, 1)), 4)        # m < k
