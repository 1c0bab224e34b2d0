"""The C-ABI library builds, loads without a GPU, and exports every symbol
declared in include/candmc_gb300.h (no compute calls: those need a GPU)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def built():
    from candmc_gb300 import build
    return build.build()


def declared_symbols():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            names |= set(re.findall(r"\b(candmc_\w+)\s*\(", open(os.path.join(inc, f)).read()))
    return sorted(names)


def test_library_exports_every_declared_symbol(built):
    lib = ctypes.CDLL(built)
    names = declared_symbols()
    assert len(names) >= 18
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_the_header(built):
    from candmc_gb300 import _abi
    assert set(_abi.header_symbols()) <= set(_abi.SIGNATURES), \
        set(_abi.header_symbols()) - set(_abi.SIGNATURES)
    lib = _abi.load()
    assert lib.candmc_version() >= 100
    assert lib.candmc_status_string(0) == b"ok"
    assert lib.candmc_status_string(1) == b"invalid argument"


def test_argument_errors_without_gpu(built):
    """Argument validation happens before any device call."""
    from candmc_gb300 import _abi
    lib = _abi.load()
    assert lib.candmc_hh_recon_qr(None, 10, 10, 4, None, None, None) == 1
    assert lib.candmc_QR_2D(None, 10, 10, 10, 4, None, 0, 0, None) == 1
    assert lib.candmc_hh_recon_qr_host(None, 10, 5, 8, None, None) == 1


def test_yamamoto_argument_errors_without_gpu(built):
    """The Yamamoto entry points validate their arguments, including the
    aggregator's buffers and counters, before any device call."""
    import ctypes
    from candmc_gb300 import _abi
    lib = _abi.load()
    dummy = ctypes.c_void_p(16)   # never dereferenced: every call below fails validation first
    n, sh = ctypes.c_int64(0), ctypes.c_int64(0)
    # Yamamoto: null pointers, ldq < m
    assert lib.candmc_Yamamoto(None, 10, dummy, 10, 10, 4, dummy, None) == 1
    assert lib.candmc_Yamamoto(dummy, 10, dummy, 5, 10, 4, dummy, None) == 1
    # upd_Yamamoto_A: b above 256
    assert lib.candmc_upd_Yamamoto_A(dummy, 300, dummy, 300, 300, 10, 257, dummy, 0, None) == 1
    # aggregator append: negative counters
    assert lib.candmc_yamamoto_append(dummy, 10, dummy, 4, -1, 0, 10, 4, dummy, 10, dummy, None) == 1
    # QR_Yamamoto_2D: aQm without aT, and counters missing
    assert lib.candmc_QR_Yamamoto_2D(dummy, 10, 10, 8, 4, 0, dummy, 10, None, 8, ctypes.byref(n),
                                     ctypes.byref(sh), 0, None) == 1
    assert lib.candmc_QR_Yamamoto_2D(dummy, 10, 10, 8, 4, 0, dummy, 10, dummy, 8, None, None, 0, None) == 1
    # QR_Yamamoto_2D_2D: b not a multiple of b_sub, m < k
    assert lib.candmc_QR_Yamamoto_2D_2D(dummy, 10, 10, 8, 6, 4, 0, None, 0, None, 0, None, None, 0, None) == 1
    assert lib.candmc_QR_Yamamoto_2D_2D(dummy, 10, 6, 8, 4, 4, 0, None, 0, None, 0, None, None, 0, None) == 1


def test_batched_argument_errors_without_gpu(built):
    """The batched entry points (FP64 and float32 inputs) reject a bad
    problem before any device call: n above 128, m below n, lda below m,
    a null pointer, and a negative count."""
    import ctypes
    from candmc_gb300 import _abi
    lib = _abi.load()
    dummy = ctypes.c_void_p(16)   # never dereferenced: every call below fails validation first

    def args(m, n, lda, ptr=dummy):
        arr = lambda t, v: (t * 1)(v)
        return (arr(ctypes.c_int64, m), arr(ctypes.c_int64, n), arr(ctypes.c_void_p, ptr),
                arr(ctypes.c_int64, lda), arr(ctypes.c_void_p, dummy))

    for fn in (lib.candmc_batched_ls, lib.candmc_batched_ls_f32):
        for m, n, lda, ptr in [(200, 129, 200, dummy), (10, 20, 10, dummy), (200, 8, 100, dummy),
                               (200, 8, 200, None)]:
            pm, pn, pa, pl, pb = args(m, n, lda, ptr)
            assert fn(1, pm, pn, pa, pl, pb, 4, 0, None) == 1, (fn, m, n, lda, ptr)
        assert fn(-1, None, None, None, None, None, 4, 0, None) == 1


def test_tuning_knobs_without_gpu(built):
    """Every tuning knob the header documents is accepted in range and rejected
    out of range (host state only; the defaults are put back)."""
    import re
    from candmc_gb300 import _abi
    lib = _abi.load()
    header = open(os.path.join(ROOT, "include", "candmc_gb300.h")).read()
    cases = {   # knob: (default, a valid value, an invalid value)
        "leaf_rows": (64, 128, 16),
        "oz_reserve_sms": (32, 24, -1),
        "pipe_leaf_rows": (128, 256, 512),
        "batched_form": (1, 0, 2),
        "ls_refine": (0, 1, 3),
        "panel_oz_min_rows": (8192, 0, -5),
        "pipe_tree": (1, 0, 2),
    }
    for key, (default, ok, bad) in cases.items():
        assert re.search(r'"%s"' % key, header), key          # documented
        assert lib.candmc_set_tuning(key.encode(), ok) == 0, key
        assert lib.candmc_set_tuning(key.encode(), bad) == 1, key
        assert lib.candmc_set_tuning(key.encode(), default) == 0, key
    assert lib.candmc_set_tuning(b"no_such_knob", 1) == 1
