"""Emulated-FP64 form (BF16 Ozaki slices on tcgen05, FP32 accumulation).

Tolerance for the FP64 and emulated-FP64 forms (FP64-class results):
backward error ||A - QR||_F / ||A||_F <= 1e-13.  Element-wise, the emulated
trailing update agrees with the FP64 update to EMU_TOL relative to the
largest entry (a few FP64 ulps times the contraction length).
"""
import numpy as np
import pytest

from oracle import candmc_oracle as co
from oracle import fixtures as fx
from oracle import lapack_restated as lp
from tests.golden.make_golden import PANELS

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

BWD_TOL = 1e-13
EMU_TOL = 1e-13


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


@pytest.mark.parametrize("name,m,b,gen", PANELS)
def test_upd_A_ozaki_matches_lapack(cm, golden, name, m, b, gen):
    i = [p[0] for p in PANELS].index(name)
    YR, Wg = golden[name + "/YR"], golden[name + "/W"]
    C = fx.gaussian(m, 16, 200 + i)
    Y = lp.unit_lower(YR, b)
    for W in (Wg, None):
        dC = dev(C)
        cm.upd_A(dev(Y), dC, None if W is None else dev(W), precision="ozaki")
        torch.cuda.synchronize()
        err = np.abs(host(dC) - golden[name + "/QtC"]).max() / np.abs(C).max()
        assert err <= EMU_TOL * max(1, b / 16), err


def test_update_A_ozaki_wide(cm):
    """A trailing block much wider than one tile and taller than one K split."""
    m, b, n = 3000, 128, 1000
    A = fx.gaussian(m, b, 31)
    YRo, Wo = co.hh_recon_qr(A, b)
    C = fx.gaussian(m, n, 32)
    want = co.update_A(YRo, C.copy(), b, Wo)
    dC = dev(C)
    cm.update_A(dev(YRo), dC, b, dev(Wo), precision="ozaki")
    torch.cuda.synchronize()
    err = np.abs(host(dC) - want).max() / np.abs(C).max()
    assert err <= EMU_TOL * 8, err


@pytest.mark.parametrize("m,k,b", [(256, 256, 128), (512, 384, 64), (1000, 700, 128),
                                   (300, 200, 17), (640, 640, 32), (129, 100, 128)])
def test_QR_2D_ozaki(cm, m, k, b):
    A = fx.gaussian(m, k, m + 3 * k + b)
    Ao = A.copy()
    co.QR_2D(Ao, b)
    dA = dev(A)
    cm.QR_2D(dA, b, precision="ozaki")
    torch.cuda.synchronize()
    YR = host(dA)
    D = np.abs(YR - Ao)
    if m == k:
        D[-1, -1] = abs(abs(YR[-1, -1]) - abs(Ao[-1, -1]))
    assert D.max() <= 1e-10 * np.abs(Ao).max(), D.max()
    assert co.backward_error(A, YR) <= BWD_TOL


def test_QR_2D_ozaki_ill_conditioned(cm):
    """sigma from 1 to 1e-10 (the precision-forms configuration, scaled down)."""
    n = 1024
    A = fx.svd_matrix(n, n, 2, 1e-10)
    dA = dev(A)
    cm.QR_2D(dA, 128, precision="ozaki")
    torch.cuda.synchronize()
    YR = host(dA)
    assert co.backward_error(A, YR) <= BWD_TOL
    assert co.orthogonality_error(YR, 128) <= 1e-13
    # agrees with the plain FP64 form to the conditioning-independent level of R's leading part
    dB = dev(A)
    cm.QR_2D(dB, 128)
    torch.cuda.synchronize()
    R1, R2 = np.triu(YR), np.triu(host(dB))
    assert np.linalg.norm(R1 - R2) / np.linalg.norm(R2) <= 1e-12


@pytest.mark.parametrize("m,k,b,prec", [(1000, 700, 128, "ozaki"), (777, 777, 64, "ozaki"),
                                        (600, 450, 32, "fp64"), (1536, 1536, 128, "ozaki")])
def test_QR_2D_pipe_lookahead(cm, m, k, b, prec):
    """Lookahead pipeline (panel i+1 on a side stream during panel i's update)
    computes the same factorization as QR_2D."""
    A = fx.gaussian(m, k, 5 * m + k)
    Ao = A.copy()
    co.QR_2D(Ao, b)
    dA = dev(A)
    cm.QR_2D_pipe(dA, b, precision=prec)
    torch.cuda.synchronize()
    YR = host(dA)
    D = np.abs(YR - Ao)
    if m == k:
        D[-1, -1] = abs(abs(YR[-1, -1]) - abs(Ao[-1, -1]))
    assert D.max() <= 1e-10 * np.abs(Ao).max(), D.max()
    assert co.backward_error(A, YR) <= BWD_TOL


def test_QR_2D_ozaki_host_entry(cm):
    A = fx.gaussian(500, 400, 77)
    Ao = A.copy()
    co.QR_2D(Ao, 128)
    Ah = np.asfortranarray(A.copy())
    cm.QR_2D(Ah, 128, precision="ozaki")
    assert np.abs(Ah - Ao).max() <= 1e-10 * np.abs(Ao).max()
    assert co.backward_error(A, Ah) <= BWD_TOL


@pytest.mark.parametrize("m,k,b,min_rows", [(1024, 512, 128, 256), (2500, 384, 128, 1024), (640, 640, 64, 1)])
def test_panel_split_update_on_tensor_cores(cm, m, k, b, min_rows):
    """In the emulated form, a panel's own column-half update (Q1^T on the
    right half inside the recursive split) runs on the tensor cores with the
    panel in FP64 storage once the panel has min_rows rows: same factorization
    as the oracle, same backward-error bound."""
    A = fx.gaussian(m, k, 3 * m + k + min_rows)
    Ao = A.copy()
    co.QR_2D(Ao, b)
    try:
        cm.set_tuning("panel_oz_min_rows", min_rows)
        for entry in (cm.QR_2D, cm.QR_2D_pipe):
            dA = dev(A)
            entry(dA, b, precision="ozaki")
            torch.cuda.synchronize()
            YR = host(dA)
            D = np.abs(YR - Ao)
            if m == k:
                D[-1, -1] = abs(abs(YR[-1, -1]) - abs(Ao[-1, -1]))
            assert D.max() <= 1e-10 * np.abs(Ao).max(), D.max()
            assert co.backward_error(A, YR) <= BWD_TOL
    finally:
        cm.set_tuning("panel_oz_min_rows", 8192)


def test_panel_split_update_knob_rejects_negative(cm):
    with pytest.raises(Exception):
        cm.set_tuning("panel_oz_min_rows", -1)
