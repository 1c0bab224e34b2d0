"""ctypes binding of the C ABI declared in include/candmc_gb300.h.

Loading fails loudly: there is no CPU fallback for any entry point.
"""
import ctypes
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcandmc_gb300.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "candmc_gb300.h")

_i64 = ctypes.c_int64
_int = ctypes.c_int
_vp = ctypes.c_void_p
_pi64 = ctypes.POINTER(ctypes.c_int64)

# name -> argtypes (restype int unless listed in _RESTYPES)
SIGNATURES = {
    "candmc_status_string": [_int],
    "candmc_version": [],
    "candmc_last_error": [],
    "candmc_hh_recon_qr": [_vp, _i64, _i64, _i64, _vp, _vp, _vp],
    "candmc_hh_recon_qr_host": [_vp, _i64, _i64, _i64, _vp, _vp],
    "candmc_hh_recon_qr_noalloc": [_vp, _i64, _i64, _i64, _vp, _vp, _vp],
    "candmc_bitree_tsqr": [_vp, _i64, _vp, _vp, _i64, _i64, _int, _vp],
    "candmc_tree_tsqr": [_vp, _i64, _vp, _vp],
    "candmc_sym_full2band": [_vp, _i64, _i64, _i64, _i64, _int, _vp],
    "candmc_tau_recon": [ctypes.c_char, _i64, _i64, _i64, _vp, _vp, _vp],
    "candmc_construct_Q1": [_vp, _i64, _vp, _vp, _i64, _i64, _i64, _i64, _vp],
    "candmc_apply_tsqr_QT": [_vp, _i64, _vp, _vp, _i64, _i64, _i64, _i64, _vp],
    "candmc_compute_invT_from_W": [_vp, _i64, _vp, _vp],
    "candmc_signed_NLU": [_vp, _vp, _i64, _i64, _i64, _vp, _vp],
    "candmc_recursive_NLU": [_vp, _vp, _i64, _i64, _i64, _vp, _vp],
    "candmc_compute_invT_from_Y": [_vp, _i64, _vp, _i64, _i64, _i64, _vp],
    "candmc_compute_invT_from_Y2": [_vp, _i64, _vp, _i64, _vp, _i64, _i64, _i64, _i64, _vp],
    "candmc_upd_A": [_vp, _i64, _vp, _i64, _i64, _i64, _i64, _vp, _int, _int, _vp],
    "candmc_update_A": [_vp, _i64, _vp, _i64, _i64, _i64, _i64, _vp, _vp, _i64, _int, _int, _vp],
    "candmc_QR_2D": [_vp, _i64, _i64, _i64, _i64, _vp, _i64, _int, _vp],
    "candmc_QR_2D_host": [_vp, _i64, _i64, _i64, _i64, _int],
    "candmc_QR_2D_2D": [_vp, _i64, _i64, _i64, _i64, _i64, _vp, _i64, _int, _vp],
    "candmc_Yamamoto": [_vp, _i64, _vp, _i64, _i64, _i64, _vp, _vp],
    "candmc_upd_Yamamoto_A": [_vp, _i64, _vp, _i64, _i64, _i64, _i64, _vp, _int, _vp],
    "candmc_yamamoto_append": [_vp, _i64, _vp, _i64, _i64, _i64, _i64, _i64, _vp, _i64, _vp, _vp],
    "candmc_QR_Yamamoto_2D": [_vp, _i64, _i64, _i64, _i64, _int, _vp, _i64, _vp, _i64, _pi64, _pi64, _int,
                              _vp],
    "candmc_QR_Yamamoto_2D_2D": [_vp, _i64, _i64, _i64, _i64, _i64, _int, _vp, _i64, _vp, _i64, _pi64, _pi64,
                                 _int, _vp],
    "candmc_QR_2D_pipe": [_vp, _i64, _i64, _i64, _i64, _int, _vp],
    "candmc_ls_solve": [_vp, _i64, _i64, _i64, _vp, _i64, _i64, _vp, _i64, _i64, _int, _int,
                        ctypes.c_double, _vp, _vp],
    "candmc_batched_ls": [_i64, _vp, _vp, _vp, _vp, _vp, _int, _int, _vp],
    "candmc_batched_ls_f32": [_i64, _vp, _vp, _vp, _vp, _vp, _int, _int, _vp],
    "candmc_set_tuning": [ctypes.c_char_p, _i64],
    "candmc_batched_status": [_vp, _vp],
    "candmc_server_create": [ctypes.c_double, _int, _int, _i64, _int, ctypes.c_double, _vp],
    "candmc_server_submit": [_vp, _vp, _i64, _i64, _i64, _vp, _vp, ctypes.c_double, _vp],
    "candmc_server_wait": [_vp, _i64, ctypes.c_double, _vp],
    "candmc_server_now": [_vp],
    "candmc_server_stats": [_vp, _vp],
    "candmc_server_destroy": [_vp],
    "candmc_ls_request_bytes": [_i64, _i64, _i64, _int],
    "candmc_mem_high_water": [_int, _vp],
    "candmc_launch_count": [],
    "candmc_profile_begin": [ctypes.c_uint],
    "candmc_profile_end": [_int, _vp, _vp, _vp],
}
_RESTYPES = {"candmc_status_string": ctypes.c_char_p, "candmc_last_error": ctypes.c_char_p,
             "candmc_launch_count": ctypes.c_longlong, "candmc_server_now": ctypes.c_double,
             "candmc_ls_request_bytes": ctypes.c_int64}

# kernel classes of candmc_profile_begin / candmc_profile_end (CANDMC_KCLASS_*)
KCLASS = {"gemm_tn": 0, "gemm_nn": 1, "reduce": 2, "panel_leaf": 3, "panel_y": 4, "small": 5,
          "oz_slice": 6, "oz_tn": 7, "oz_nn": 8, "f32": 9, "oz_panel": 10}
NKCLASS = 16

_lib = None


def header_symbols():
    """Function names declared in include/candmc_gb300.h."""
    text = open(HEADER).read()
    return sorted(set(re.findall(r"\b(candmc_\w+)\s*\(", text)))


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            f"{LIB_PATH} is missing: build it with `python -m candmc_gb300.build` "
            "(there is no CPU fallback)")
    lib = ctypes.CDLL(LIB_PATH)
    for name, args in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = _RESTYPES.get(name, _int)
    _lib = lib
    return lib


class CandmcError(RuntimeError):
    def __init__(self, status, where):
        lib = load()
        msg = lib.candmc_status_string(status).decode()
        detail = lib.candmc_last_error().decode()
        super().__init__(f"{where}: {msg} (status {status}){': ' + detail if detail else ''}")
        self.status = status


def check(status, where):
    if status != 0:
        raise CandmcError(status, where)
