"""candmc_hh_recon_qr_noalloc: the TSQR-HR entry point that allocates nothing.

It serves callers that may not have a library allocate device memory while
they run (a server whose GPU memory is budgeted at start-up, a framework
whose allocator owns every device buffer); its scratch is a fixed array
inside the library.  This file is collected last so that a run stopping at
the first failure has already run every other test.

The test calls the new entry point through the C ABI twice in a row, with
different shapes (the second call must not see the first one's leftovers,
e.g. the tree arrival counters), and compares each result with the
allocating entry point candmc_hh_recon_qr on the same input, within the
tolerance of the other parity tests.  It also checks that sizes beyond the
fixed scratch are rejected.
"""
import ctypes

import numpy as np
import pytest

from oracle import fixtures as fx

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

ELEM_TOL = 2e-12


@pytest.fixture(scope="module")
def lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from candmc_gb300 import _abi, build
    build.build()
    return _abi.load()


def colmajor(a):
    return torch.from_numpy(np.asfortranarray(a)).cuda().t().contiguous().t()


def run(fn, A, b):
    m = A.shape[0]
    dA = colmajor(A)
    W = torch.zeros((b, b), dtype=torch.float64, device="cuda")
    T = torch.zeros((b, b), dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rc = fn(dA.data_ptr(), dA.stride(1), m, b, W.data_ptr(), T.data_ptr(), stream)
    torch.cuda.synchronize()
    assert rc == 0, rc
    # W and T are b x b column-major buffers with leading dimension b
    return dA.cpu().numpy(), W.cpu().numpy().T, T.cpu().numpy().T


def test_noalloc_matches_allocating_entry_point_twice(lib):
    cases = [(4096, 32, 11), (1000, 17, 12)]
    inputs = [(fx.gaussian(m, b, seed), b) for (m, b, seed) in cases]
    want = [run(lib.candmc_hh_recon_qr, A, b) for (A, b) in inputs]
    # two calls of the no-allocation entry point in a row
    got = [run(lib.candmc_hh_recon_qr_noalloc, A, b) for (A, b) in inputs]
    for (A, b), (YR_a, W_a, T_a), (YR_n, W_n, T_n) in zip(inputs, want, got):
        scale = max(1.0, np.abs(YR_a).max())
        tol = ELEM_TOL * max(1.0, b / 16)
        assert np.abs(YR_n - YR_a).max() <= tol * scale
        assert np.abs(W_n - W_a).max() <= tol
        assert np.abs(T_n - T_a).max() <= tol


def test_noalloc_rejects_sizes_beyond_its_scratch(lib):
    dA = torch.zeros((64, 9000), dtype=torch.float64, device="cuda").t()   # 9000 x 64
    W = torch.zeros((64, 64), dtype=torch.float64, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    assert lib.candmc_hh_recon_qr_noalloc(dA.data_ptr(), 9000, 9000, 33, W.data_ptr(),
                                          W.data_ptr(), s) == 1   # b > 32
    assert lib.candmc_hh_recon_qr_noalloc(dA.data_ptr(), 9000, 9000, 32, W.data_ptr(),
                                          W.data_ptr(), s) == 1   # m > 8192
    assert b"8192" in lib.candmc_last_error()
