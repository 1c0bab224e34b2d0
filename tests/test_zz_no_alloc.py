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
tolerance of the other parity tests.  The shapes include the largest case the
scratch is sized for (m = 8192, b = 32: 32 leaves and 63 tree nodes) and an
odd shape next to it.  It also checks that sizes beyond the fixed scratch are
rejected, and that a call leaves the device's memory pool untouched while the
allocating entry point (the control) does draw from it.
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
    cases = [(4096, 32, 11), (1000, 17, 12), (8192, 32, 13), (8191, 31, 14)]
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


def _pool_high_water(lib, reset):
    v = ctypes.c_uint64(0)
    assert lib.candmc_mem_high_water(1 if reset else 0, ctypes.byref(v)) == 0
    return v.value


def test_noalloc_draws_nothing_from_the_memory_pool(lib):
    m, b = 8192, 32
    A = fx.gaussian(m, b, 15)
    bufs = []
    for fn in (lib.candmc_hh_recon_qr_noalloc, lib.candmc_hh_recon_qr):
        dA = colmajor(A)
        W = torch.zeros((b, b), dtype=torch.float64, device="cuda")
        T = torch.zeros((b, b), dtype=torch.float64, device="cuda")
        bufs.append((fn, dA, W, T))
    s = torch.cuda.current_stream().cuda_stream
    fn, dA, W, T = bufs[0]
    fn(dA.data_ptr(), m, m, b, W.data_ptr(), T.data_ptr(), s)   # first call: device set-up
    torch.cuda.synchronize()
    highs = []
    for fn, dA, W, T in bufs:
        _pool_high_water(lib, True)
        before = _pool_high_water(lib, False)
        assert fn(dA.data_ptr(), m, m, b, W.data_ptr(), T.data_ptr(), s) == 0
        torch.cuda.synchronize()
        highs.append(_pool_high_water(lib, False) - before)
    assert highs[0] == 0, f"no-alloc call drew {highs[0]} bytes from the pool"
    assert highs[1] > 0, "control: the allocating entry point should draw scratch from the pool"


def test_noalloc_rejects_sizes_beyond_its_scratch(lib):
    dA = torch.zeros((64, 9000), dtype=torch.float64, device="cuda").t()   # 9000 x 64
    W = torch.zeros((64, 64), dtype=torch.float64, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    assert lib.candmc_hh_recon_qr_noalloc(dA.data_ptr(), 9000, 9000, 33, W.data_ptr(),
                                          W.data_ptr(), s) == 1   # b > 32
    assert lib.candmc_hh_recon_qr_noalloc(dA.data_ptr(), 9000, 9000, 32, W.data_ptr(),
                                          W.data_ptr(), s) == 1   # m > 8192
    assert b"8192" in lib.candmc_last_error()
