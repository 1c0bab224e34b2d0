"""FP32 form of the trailing update and the least-squares solver with FP64
iterative refinement.

Tolerances: refined least-squares solutions within 1e-12
relative of the FP64 oracle for well-conditioned problems; the FP32-form
factorization itself is FP32-accurate (backward error FP32_BWD_TOL).  For
ill-conditioned problems forward agreement is limited by kappa * u, so the
check there is the normal-equations residual ||A^T r|| / (||A|| ||r||).
"""
import numpy as np
import pytest

from oracle import candmc_oracle as co
from oracle import fixtures as fx

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

LS_TOL = 1e-12
FP32_BWD_TOL = 1e-5


@pytest.fixture(scope="module")
def cm():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import candmc_gb300 as cm
    cm.lib()
    return cm


def dev(a):
    return torch.from_numpy(np.asfortranarray(a)).cuda().t().contiguous().t()


def host(t):
    return np.asfortranarray(t.cpu().numpy())


@pytest.mark.parametrize("m,k,b", [(512, 384, 128), (1000, 1000, 64), (700, 300, 32)])
def test_QR_2D_fp32_form(cm, m, k, b):
    A = fx.gaussian(m, k, 11 * m + k)
    dA = dev(A)
    cm.QR_2D_pipe(dA, b, precision="fp32")
    torch.cuda.synchronize()
    YR = host(dA)
    bwd = co.backward_error(A, YR)
    assert bwd <= FP32_BWD_TOL, bwd
    Ao = A.copy()
    co.QR_2D(Ao, b)
    assert np.linalg.norm(np.triu(YR) - np.triu(Ao)) / np.linalg.norm(np.triu(Ao)) <= 1e-4


def test_upd_A_fp32_form(cm, golden):
    name, m, b = "hh_384x64", 384, 64
    from oracle import lapack_restated as lp
    YR, Wg = golden[name + "/YR"], golden[name + "/W"]
    C = fx.gaussian(m, 16, 200 + 5)
    dC = dev(C)
    cm.upd_A(dev(lp.unit_lower(YR, b)), dC, dev(Wg), precision="fp32")
    torch.cuda.synchronize()
    err = np.abs(host(dC) - golden[name + "/QtC"]).max() / np.abs(C).max()
    assert err <= 1e-5, err


@pytest.mark.parametrize("prec", ["fp64", "ozaki", "fp32"])
@pytest.mark.parametrize("m,n,nrhs,b,smin", [(2000, 500, 4, 128, None), (1536, 1024, 16, 128, 1e-3),
                                             (3000, 257, 3, 64, None)])
def test_ls_solve_refined_to_fp64(cm, prec, m, n, nrhs, b, smin):
    A = fx.gaussian(m, n, m + n) if smin is None else fx.svd_matrix(m, n, 2, smin)
    B = fx.gaussian(m, nrhs, 7)
    Xo = co.ls_solve(A, B, b)
    X, st = cm.ls_solve(dev(A), dev(B), b=b, precision=prec, max_refine=30, tol=1e-15)
    torch.cuda.synchronize()
    X = host(X)
    err = np.linalg.norm(X - Xo, axis=0) / np.linalg.norm(Xo, axis=0)
    assert err.max() <= LS_TOL, (err.max(), st)
    assert st["status"] == 0


def test_ls_solve_ill_conditioned_emulated(cm):
    """sigma from 1 to 1e-10: forward error is kappa-limited; the emulated-FP64
    solution satisfies the normal equations to FP64 level."""
    m, n = 1024, 512
    A = fx.svd_matrix(m, n, 2, 1e-10)
    B = fx.gaussian(m, 2, 9)
    X, st = cm.ls_solve(dev(A), dev(B), b=128, precision="ozaki", max_refine=0)
    torch.cuda.synchronize()
    X = host(X)
    r = B - A @ X
    nA = np.linalg.norm(A, 2)
    ne = np.linalg.norm(A.T @ r, axis=0) / (nA * np.linalg.norm(r, axis=0))
    # a backward-stable solution has ||A^T r|| <~ u ||A|| (||A|| ||x|| + ||r||)
    bound = 100 * 2.2e-16 * (nA * np.linalg.norm(X, axis=0) / np.linalg.norm(r, axis=0) + 1)
    assert (ne <= bound).all(), (ne, bound)
    Xo = co.ls_solve(A, B, 128)
    kappa = 1e10
    assert (np.linalg.norm(X - Xo, axis=0) / np.linalg.norm(Xo, axis=0)).max() <= kappa * 1e-14


@pytest.mark.parametrize("refine", [1, 0])
@pytest.mark.parametrize("prec", ["ozaki", "fp64"])
def test_ls_kappa_1e10_reaches_the_oracles_forward_error(cm, prec, refine):
    """sigma from 1 to 1e-10 (kappa = 1e10), inconsistent right-hand sides.
    No FP64 solver does better than a forward error of order kappa * u = 1e-6
    on FP64 data: LAPACK's own solution (the oracle) is that far from the exact
    one.  The refined emulated-FP64 and FP64 solutions must land at that level:
    within 10 * kappa * u of the oracle's solution, with a normal-equations
    residual ||A^T r|| / (||A|| ||r||) no larger than the oracle's."""
    m, n = 2048, 384
    A = fx.svd_matrix(m, n, 5, 1e-10)
    B = fx.gaussian(m, 2, 13)
    Xo = np.linalg.lstsq(A, B, rcond=None)[0]
    nA = np.linalg.norm(A, 2)

    def eta(X):
        r = B - A @ X
        return np.linalg.norm(A.T @ r, axis=0) / (nA * np.linalg.norm(r, axis=0))

    try:
        cm.set_tuning("ls_refine", refine)
        X, st = cm.ls_solve(dev(A), dev(B), b=128, precision=prec, max_refine=10, tol=1e-15)
        torch.cuda.synchronize()
    finally:
        cm.set_tuning("ls_refine", 0)
    X = host(X)
    assert st["status"] == 0
    err = np.linalg.norm(X - Xo, axis=0) / np.linalg.norm(Xo, axis=0)
    assert err.max() <= 10 * 1e10 * 2.2e-16, (err, st)
    assert (eta(X) <= 2 * eta(Xo)).all(), (eta(X), eta(Xo), st)


@pytest.mark.parametrize("smin", [1e-3, 1e-5])
@pytest.mark.parametrize("refine", [0, 1])
def test_ls_fp32_form_refined_at_moderate_kappa(cm, smin, refine):
    """The FP32 form's R (u_R ~ 6e-8) refined in FP64 -- corrected semi-normal
    equations or the augmented system -- reaches the FP64 oracle's solution up
    to kappa = 1e5 (contraction ~ kappa * u_R with R from A's own QR)."""
    m, n = 2000, 256
    A = fx.svd_matrix(m, n, 3, smin)
    B = fx.gaussian(m, 2, 17)
    Xo = np.linalg.lstsq(A, B, rcond=None)[0]
    try:
        cm.set_tuning("ls_refine", refine)
        X, st = cm.ls_solve(dev(A), dev(B), b=128, precision="fp32", max_refine=30, tol=1e-15)
        torch.cuda.synchronize()
    finally:
        cm.set_tuning("ls_refine", 0)
    X = host(X)
    err = np.linalg.norm(X - Xo, axis=0) / np.linalg.norm(Xo, axis=0)
    assert err.max() <= max(LS_TOL, 100 * (1 / smin) * 2.2e-16), (err, st)
