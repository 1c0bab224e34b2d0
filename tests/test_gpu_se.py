"""The eigensolver's symmetric full -> band reduction (alg/SE/full_to_band.cxx,
the first caller of QR_2D_pipe and compute_invT_from_Y outside the QR
directory) on the GPU, against the oracle's restatement
(oracle/se_oracle.py).

Tolerances: the band (diagonal blocks and the R blocks below them) and the
reflectors agree with the oracle element-wise to ELEM_TOL * max(1, b/16)
relative to the largest entry -- the panel factorizations are canonical
Householder factors and the two-sided updates are FP64 products; the band
matrix's eigenvalues equal A's to 1e-13 relative (an orthogonal similarity).
"""
import numpy as np
import pytest

from oracle import fixtures as fx
from oracle import se_oracle as se

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

ELEM_TOL = 2e-12


@pytest.fixture(scope="module")
def cm():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import candmc_gb300 as cm
    cm.lib()
    return cm


def sym(n, seed):
    X = fx.gaussian(n, n, seed)
    return np.asfortranarray(X + X.T)


@pytest.mark.parametrize("form", ["fp64", "ozaki"])
@pytest.mark.parametrize("n,b,b_sub", [(64, 16, 8), (200, 32, 16), (257, 32, 32), (512, 64, 32), (1000, 128, 64)])
def test_sym_full2band_matches_oracle(cm, n, b, b_sub, form):
    A = sym(n, n + b)
    want = np.array(A, order="F")
    se.sym_full2band(want, b, b_sub)
    dA = torch.from_numpy(A).cuda().t().contiguous().t()
    cm.sym_full2band(dA, b, b_sub, precision=form)
    got = np.asfortranarray(dA.cpu().numpy())
    low = np.tril(np.ones((n, n), dtype=bool))
    err = np.abs(got - want)[low].max()
    assert err <= ELEM_TOL * max(1.0, b / 16) * max(1.0, np.abs(want).max()), err
    ev = np.linalg.eigvalsh(A)
    evb = np.linalg.eigvalsh(se.band_matrix(got, b))
    assert np.abs(evb - ev).max() <= 1e-13 * np.abs(ev).max() * max(1.0, n / 256)


def test_sym_full2band_rejects_bad_blocks(cm):
    dA = torch.zeros((64, 64), dtype=torch.float64, device="cuda")
    with pytest.raises(Exception):
        cm.sym_full2band(dA, 16, 6)      # b not a multiple of b_sub
    with pytest.raises(Exception):
        cm.sym_full2band(dA, 512, 512)   # b > 256
