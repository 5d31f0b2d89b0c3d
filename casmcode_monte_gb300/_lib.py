"""ctypes binding of the C-ABI in include/montegpu.h (libmontegpu.so).

The library is built in-tree by ``casmcode_monte_gb300.build``.  There is no CPU
fallback: if the library is missing, ``lib()`` raises ``RuntimeError`` telling the user
to build it; device entry points report CUDA errors (e.g. no GPU) as ``RuntimeError``.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "lib", "libmontegpu.so")

c_int_p = C.POINTER(C.c_int)
c_long_p = C.POINTER(C.c_long)
c_ll_p = C.POINTER(C.c_longlong)
c_ull_p = C.POINTER(C.c_ulonglong)
c_double_p = C.POINTER(C.c_double)
c_float_p = C.POINTER(C.c_float)
c_int8_p = C.POINTER(C.c_int8)
c_int32_p = C.POINTER(C.c_int32)
c_uint32_p = C.POINTER(C.c_uint32)
c_uint64_p = C.POINTER(C.c_uint64)
c_size_p = C.POINTER(C.c_size_t)
vp = C.c_void_p
vpp = C.POINTER(C.c_void_p)

#: name -> (restype, argtypes) for every function declared in include/montegpu.h
SIGNATURES = {
    "mg_last_error": (C.c_char_p, []),
    "mg_version": (C.c_int, []),
    "mg_device_count": (C.c_int, [c_int_p]),
    "mg_device_sm_count": (C.c_int, [c_int_p]),
    "mg_release_cached_memory": (C.c_int, []),
    "mg_engine_create": (C.c_int, [C.c_int, vpp]),
    "mg_engine_destroy": (C.c_int, [vp]),
    "mg_engine_seed": (C.c_int, [vp, C.c_uint64]),
    "mg_engine_seed_seq": (C.c_int, [vp, c_uint64_p, C.c_size_t]),
    "mg_engine_dump": (C.c_int, [vp, C.c_char_p, C.c_size_t]),
    "mg_engine_load": (C.c_int, [vp, C.c_char_p]),
    "mg_engine_random_int": (C.c_int, [vp, C.c_uint64, c_uint64_p]),
    "mg_engine_random_real": (C.c_int, [vp, C.c_double, c_double_p]),
    "mg_ising_replay_create": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, c_double_p, c_double_p,
                                         c_double_p, c_int32_p, C.POINTER(C.c_char_p), vpp]),
    "mg_ising_replay_run": (C.c_int, [vp, C.c_int, C.c_int, c_ll_p, C.c_int, c_int_p]),
    "mg_ising_replay_get_state": (C.c_int, [vp, c_int32_p, C.POINTER(C.c_char_p), C.c_size_t,
                                            c_ull_p, c_ull_p]),
    "mg_ising_replay_last_kernel_ms": (C.c_int, [vp, c_float_p]),
    "mg_ising_replay_destroy": (C.c_int, [vp]),
    "mg_ce_model_create": (C.c_int, [C.c_int, c_double_p, C.c_int, vpp]),
    "mg_ce_model_info": (C.c_int, [vp, c_int_p, c_int_p, c_int_p]),
    "mg_ce_model_classes": (C.c_int, [vp, c_long_p, c_double_p]),
    "mg_ce_model_destroy": (C.c_int, [vp]),
    "mg_ce_batch_create": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, C.c_int, c_double_p, c_double_p,
                                     c_uint64_p, c_uint32_p, c_int8_p, C.c_int, C.c_int, vpp]),
    "mg_ce_batch_info": (C.c_int, [vp, c_int_p, c_int_p, c_int_p, c_size_p]),
    "mg_ce_batch_colors": (C.c_int, [vp, c_int32_p]),
    "mg_ce_batch_layout": (C.c_int, [vp, c_int_p]),
    "mg_ce_color_supercell": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, c_int32_p, c_int_p]),
    "mg_ce_batch_set_layout": (C.c_int, [vp, C.c_int]),
    "mg_ce_batch_autotune": (C.c_int, [vp, C.c_int, c_int_p, c_int_p, C.POINTER(C.c_float)]),
    "mg_ce_batch_run": (C.c_int, [vp, C.c_int, c_ll_p]),
    "mg_ce_batch_last_kernel_ms": (C.c_int, [vp, c_float_p]),
    "mg_ce_batch_rotation": (C.c_int, [vp, c_int_p, c_double_p]),
    "mg_ce_batch_set_rotation": (C.c_int, [vp, C.c_int]),
    "mg_ce_batch_last_launches": (C.c_int, [vp, c_int_p]),
    "mg_ce_batch_rotation_timeline": (C.c_int, [vp, c_float_p]),
    "mg_ce_canon_create": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, C.c_int, c_double_p, c_uint64_p, c_uint32_p,
                                     c_int8_p, C.c_int, vpp]),
    "mg_ce_canon_info": (C.c_int, [vp, c_int_p, c_int_p, c_int_p, c_size_p]),
    "mg_ce_canon_colors": (C.c_int, [vp, C.c_int, c_int32_p]),
    "mg_ce_canon_class_order": (C.c_int, [vp, C.c_int, c_int32_p]),
    "mg_ce_canon_run": (C.c_int, [vp, C.c_int, c_ll_p]),
    "mg_ce_canon_last_kernel_ms": (C.c_int, [vp, c_float_p]),
    "mg_ce_canon_get_occ": (C.c_int, [vp, c_int8_p]),
    "mg_ce_canon_corr": (C.c_int, [vp, c_ll_p]),
    "mg_ce_canon_destroy": (C.c_int, [vp]),
    "mg_ce_nfold_create": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, C.c_int, c_double_p, c_double_p, c_uint64_p,
                                     c_uint32_p, c_int8_p, vpp]),
    "mg_ce_nfold_run": (C.c_int, [vp, C.c_int, c_double_p]),
    "mg_ce_nfold_info": (C.c_int, [vp, c_int_p, c_int_p, c_size_p]),
    "mg_ce_nfold_last_kernel_ms": (C.c_int, [vp, c_float_p]),
    "mg_ce_nfold_get_occ": (C.c_int, [vp, c_int8_p]),
    "mg_ce_nfold_corr": (C.c_int, [vp, C.c_int, c_ll_p]),
    "mg_ce_nfold_destroy": (C.c_int, [vp]),
    "mg_ce_batch_get_occ": (C.c_int, [vp, c_int8_p]),
    "mg_ce_batch_set_occ": (C.c_int, [vp, c_int8_p]),
    "mg_ce_batch_corr": (C.c_int, [vp, c_ll_p]),
    "mg_ce_batch_delta_e": (C.c_int, [vp, c_int32_p, c_ll_p, c_int8_p, C.c_longlong, c_double_p]),
    "mg_ce_batch_destroy": (C.c_int, [vp]),
    "mg_ce_max_active_chains": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, C.c_int, c_int_p]),
    "mg_ce_pool_create": (C.c_int, [vp, C.c_longlong, C.c_int, C.c_int, vpp]),
    "mg_ce_pool_add": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, C.c_double, c_double_p, C.c_uint64, C.c_uint32,
                                 c_int8_p, c_int_p]),
    "mg_ce_pool_add_many": (C.c_int, [vp, C.c_int, c_int32_p, c_double_p, c_double_p, c_uint64_p, c_uint32_p,
                                      c_int8_p, c_int32_p]),
    "mg_ce_pool_remove": (C.c_int, [vp, C.c_int]),
    "mg_ce_pool_prepare": (C.c_int, [vp, C.c_int, C.c_int, C.c_int]),
    "mg_ce_pool_info": (C.c_int, [vp, c_ll_p, c_ll_p, c_int_p, c_int_p]),
    "mg_ce_pool_run": (C.c_int, [vp, c_int32_p, C.c_int, C.c_int, c_ll_p]),
    "mg_ce_pool_last_kernel_ms": (C.c_int, [vp, c_float_p]),
    "mg_ce_pool_last_launches": (C.c_int, [vp, c_int_p]),
    "mg_ce_pool_get_occ": (C.c_int, [vp, C.c_int, c_int8_p]),
    "mg_ce_pool_colors": (C.c_int, [vp, C.c_int, c_int32_p]),
    "mg_ce_pool_corr": (C.c_int, [vp, C.c_int, c_ll_p]),
    "mg_ce_pool_enable_series": (C.c_int, [vp, C.c_int]),
    "mg_ce_pool_series": (C.c_int, [vp, C.c_int, c_double_p, C.c_int, c_int_p]),
    "mg_ce_pool_check": (C.c_int, [vp, c_int32_p, C.c_int, C.c_double, C.c_double, c_double_p]),
    "mg_ce_pool_destroy": (C.c_int, [vp]),
    "mg_ce_replay_create": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, C.c_int, c_double_p, c_double_p, c_int8_p,
                                      C.POINTER(C.c_char_p), vpp]),
    "mg_ce_replay_run": (C.c_int, [vp, C.c_int, c_ll_p]),
    "mg_ce_replay_get_occ": (C.c_int, [vp, c_int8_p]),
    "mg_ce_replay_engine_state": (C.c_int, [vp, C.c_int, C.c_char_p, C.c_int]),
    "mg_ce_replay_candidates": (C.c_int, [vp, C.c_int, c_int32_p, c_int32_p]),
    "mg_ce_replay_counts": (C.c_int, [vp, c_ull_p, c_ull_p]),
    "mg_ce_replay_last_kernel_ms": (C.c_int, [vp, c_float_p]),
    "mg_ce_replay_destroy": (C.c_int, [vp]),
    "mg_ce_sweep_noalloc": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, C.c_int, c_double_p, c_double_p, c_uint64_p,
                                      vp, C.c_longlong, C.c_int, vp, C.c_int, vp]),
    "mg_equilibration_check": (C.c_int, [c_double_p, C.c_long, C.c_double, c_int_p, c_long_p]),
    "mg_basic_statistics": (C.c_int, [c_double_p, C.c_long, c_double_p, C.c_long, C.c_double,
                                      C.c_long, C.c_long, c_double_p, c_double_p]),
    "mg_autocorrelation_factor": (C.c_int, [c_double_p, C.c_long, C.c_double, c_double_p]),
    "mg_approx_erf_inv": (C.c_double, [C.c_double]),
}

_lock = threading.Lock()
_lib = None


def lib() -> C.CDLL:
    """Load libmontegpu.so (once); raise if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise RuntimeError(
                    f"libmontegpu.so not found at {LIB_PATH}; build it with "
                    "`python -m casmcode_monte_gb300.build` (there is no CPU fallback)"
                )
            L = C.CDLL(LIB_PATH)
            for name, (res, args) in SIGNATURES.items():
                f = getattr(L, name)
                f.restype = res
                f.argtypes = args
            _lib = L
    return _lib


def check(status: int) -> None:
    """Raise RuntimeError with the library's message on a non-zero status."""
    if status != 0:
        msg = lib().mg_last_error()
        raise RuntimeError(msg.decode() if msg else f"montegpu error {status}")


def ptr(a, ctype):
    """ctypes pointer to a contiguous numpy array."""
    return a.ctypes.data_as(C.POINTER(ctype))
