"""Host-side parts of the least-squares request server that need no GPU:
the seeded Poisson trace, the admission estimate and argument validation
of the native server API."""
import numpy as np
import pytest


def test_poisson_trace_is_seeded_and_shaped():
    from candmc_gb300.serve import poisson_trace
    a = poisson_trace(4000, rate=1000.0, seed=4)
    b = poisson_trace(4000, rate=1000.0, seed=4)
    assert a == b
    t = np.array([r[0] for r in a])
    m = np.array([r[1] for r in a])
    n = np.array([r[2] for r in a])
    gaps = np.diff(np.concatenate([[0.0], t]))
    assert np.all(gaps > 0)
    assert abs(gaps.mean() - 1e-3) < 0.1e-3            # rate 1000/s
    assert m.min() >= 512 and m.max() <= 1048576
    lm = np.log(m)
    assert abs(lm.mean() - 0.5 * (np.log(512) + np.log(1048576))) < 0.15   # log-uniform
    assert set(n.tolist()) == {16, 32, 64, 128, 256}
    assert np.all(m >= n)


@pytest.fixture(scope="module")
def lib():
    from candmc_gb300 import _abi, build
    build.build()
    return _abi.load()


def test_request_bytes_estimate(lib):
    est = lambda m, n, p=2: lib.candmc_ls_request_bytes(m, n, 128, p)
    assert est(0, 4) == 0
    for m, n in [(512, 16), (100000, 128), (1048576, 256)]:
        assert est(m, n) >= 16 * m * n                 # A and its factor at least
        assert est(2 * m, n) > est(m, n) and est(m, 2 * n) >= est(m, n)
    assert est(100000, 256, 1) > est(100000, 256, 2) > est(100000, 256, 0)


def test_server_argument_errors_without_gpu(lib):
    import ctypes
    h = ctypes.c_void_p()
    assert lib.candmc_server_create(0.0, 4, 2, 128, 10, 1e-15, ctypes.byref(h)) == 1
    assert lib.candmc_server_create(1e9, 0, 2, 128, 10, 1e-15, ctypes.byref(h)) == 1
    assert lib.candmc_server_create(1e9, 4, 9, 128, 10, 1e-15, ctypes.byref(h)) == 1
    assert lib.candmc_server_create(1e9, 4, 2, 256, 10, 1e-15, ctypes.byref(h)) == 1
    t = ctypes.c_int64()
    assert lib.candmc_server_submit(None, None, 10, 10, 4, None, None, 0.0, ctypes.byref(t)) == 1
    assert lib.candmc_server_wait(None, 0, 0.0, None) == 1
    assert lib.candmc_status_string(7) == b"request cancelled at server shutdown"
