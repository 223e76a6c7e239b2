"""ctypes binding of the in-tree native library ``libchimescalc.so``.

The library is the product: every evaluation runs in its CUDA kernels.  There
is no Python or CPU fallback -- ``load()`` raises when the library has not been
built, and the library itself reports an error when no GPU is present.
"""

from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libchimescalc.so")

_lib = None

# Exported C symbols and their signatures: the reference's serial interface
# (chimescalc_serial_C.h), its per-cluster interface (chimescalc_C.h) and the
# ck_* extension (chimes_gb300.h).
D, I, LL, P, S = ctypes.c_double, ctypes.c_int, ctypes.c_longlong, ctypes.c_void_p, ctypes.c_char_p
DP, IP, LLP = ctypes.POINTER(D), ctypes.POINTER(I), ctypes.POINTER(LL)
SP = ctypes.POINTER(ctypes.c_char_p)

SIGNATURES = {
    # serial interface
    "chimes_open_instance": (P, []),
    "chimes_close_instance": (None, [P]),
    "set_chimes_serial": (None, [I]),
    "set_chimes_serial_instance": (None, [P, I]),
    "init_chimes_serial": (None, [S, IP]),
    "init_chimes_serial_instance": (None, [P, S, I]),
    "calculate_chimes": (None, [I, DP, DP, DP, SP, DP, DP, DP, DP, DP, DP, DP, DP]),
    "calculate_chimes_instance": (None, [P, I, DP, DP, DP, SP, DP, DP, DP, DP, DP, DP, DP, DP]),
    # per-cluster interface
    "get_chimes_max_2b_cutoff": (D, []),
    "get_chimes_max_3b_cutoff": (D, []),
    "get_chimes_max_4b_cutoff": (D, []),
    "get_chimes_2b_order": (I, []),
    "get_chimes_3b_order": (I, []),
    "get_chimes_4b_order": (I, []),
    "set_chimes": (None, []),
    "init_chimes": (None, [I]),
    "chimes_read_params": (None, [S]),
    "chimes_build_pair_int_trip_map": (None, []),
    "chimes_build_pair_int_quad_map": (None, []),
    "chimes_compute_2b_props": (None, [D, DP, SP, DP, DP, DP]),
    "chimes_compute_3b_props": (None, [DP, DP, SP, DP, DP, DP]),
    "chimes_compute_4b_props": (None, [DP, DP, SP, DP, DP, DP]),
    "chimes_compute_2b_props_fromf90": (None, [DP, DP, S, S, DP, DP, DP]),
    "chimes_compute_3b_props_fromf90": (None, [DP, DP, S, S, S, DP, DP, DP]),
    "chimes_compute_4b_props_fromf90": (None, [DP, DP, S, S, S, S, DP, DP, DP]),
    # extension
    "ck_set_error_mode": (I, [I]),
    "ck_last_error": (S, []),
    "ck_open": (P, []),
    "ck_close": (None, [P]),
    "ck_load_params": (I, [P, S]),
    "ck_select_params": (I, [P, I]),
    "ck_check_params": (I, [S, IP, IP, DP]),
    "ck_save_params_cache": (I, [P, I, S]),
    "ck_convert_params": (I, [S, S]),
    "ck_param_info": (I, [P, I, IP, IP, DP]),
    "ck_type_index": (I, [P, I, S]),
    "ck_tuple_table": (I, [P, I, I, IP, IP, DP]),
    "ck_tuple_factored": (I, [P, I, I, IP, IP, IP]),
    "ck_get_tuning": (I, [P, IP]),
    "ck_set_precision": (I, [P, I]),
    "ck_set_tuning": (I, [P, I, I, I]),
    "ck_set_contraction": (I, [P, I]),
    "ck_use_graph": (I, [P, I]),
    "ck_autotune_repeats": (I, [P, I]),
    "ck_autotune": (I, [P, IP]),
    "ck_calculate_batch": (I, [P, I, IP, DP, IP, DP, IP, IP, DP, DP, DP]),
    "ck_stage_batch": (I, [P, I, IP, DP, IP, DP, IP, IP]),
    "ck_launch": (I, [P]),
    "ck_collect": (I, [P, DP, DP, DP]),
    "ck_stream": (P, [P]),
    "ck_last_counts": (I, [P, LLP]),
    "ck_set_profiling": (I, [P, I]),
    "ck_fma_peak": (I, [I, DP]),
    "ck_read_stage_times": (I, [P, DP, LLP, IP]),
    "ck_last_diagnostics": (I, [P, IP]),
    "ck_export_lists": (I, [P, IP, IP, IP]),
    "ck_compute_cluster_batch": (I, [P, I, I, DP, DP, IP, DP, DP, DP, DP]),
    "ck_compute_cluster_batch_tab": (I, [P, I, I, DP, DP, IP, DP, DP, DP, DP]),
    "ck_tabulated": (I, [P, IP]),
    "ck_nl_fingerprint": (I, [P, I, LLP, DP, IP]),
    "ck_fp_histogram": (I, [P, I, LL, DP, IP, LL, DP, IP, I, I, LLP, LLP]),
    "ck_calculate_noalloc": (I, [P, I, P, P, DP, I, P, P, P, P]),
    "ck_nl_compute": (I, [P, I, DP, IP, LLP, I, IP, IP, IP, D, I, DP, DP, DP, DP, DP]),
    "ck_nl_lists": (I, [P, LLP, IP, IP]),
    "ck_server_open": (P, [I, D, LL, I]),
    "ck_server_close": (None, [P]),
    "ck_server_load_params": (I, [P, S]),
    "ck_server_submit": (LL, [P, I, I, DP, IP, DP, I]),
    "ck_server_take": (I, [P, LL, I, D, DP, DP, DP, DP]),
    "ck_server_stats": (I, [P, LLP]),
    "ck_server_worker_tuning": (I, [P, I, IP]),
    "ck_server_autotune": (I, [P, I, IP, DP, IP, DP, IP, IP, IP]),
    "ck_server_replay": (I, [P, I, IP, IP, DP, IP, DP, IP, DP, DP, DP, DP]),
}


def load() -> ctypes.CDLL:
    """Loads the native library (raises if it has not been built).  The
    environment variable CHIMES_GB300_LIB selects another build of it (the
    checked build, libchimescalc_bounds.so, for instance)."""
    global _lib
    if _lib is not None:
        return _lib
    path = os.environ.get("CHIMES_GB300_LIB") or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError("native library %s is missing: build it with "
                           "chimes_calculator_gb300.build.build() (there is no CPU fallback)" % path)
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name, None)
        if fn is None:
            continue
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def exported_symbols():
    return list(SIGNATURES)
