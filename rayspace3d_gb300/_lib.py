"""ctypes binding of librs.so (the C ABI declared in include/rayspace3d.h).

There is no CPU fallback: importing the binding when the library has not been
built raises, and every call that returns a non-zero rs_status raises RsError.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

LIB_PATH = _build.LIB_PATH

RS_OK = 0
RS_ERR_CUDA = 1
RS_ERR_INVALID = 2
RS_ERR_TABLE_FULL = 3
RS_ERR_OUTPUT_OVERFLOW = 4
RS_ERR_ITER_LIMIT = 5
RS_ERR_FORMAT = 6
RS_ERR_OOM = 7
RS_ERR_TARGET_OVERFLOW = 8
RS_ERR_TOO_LARGE = 9

# Every entry point of include/rayspace3d.h: name -> (restype, argtypes).
P = ctypes.c_void_p
U64 = ctypes.c_uint64
I64 = ctypes.c_int64
F = ctypes.c_float
I = ctypes.c_int
PP = ctypes.POINTER(ctypes.c_void_p)
PU64 = ctypes.POINTER(ctypes.c_uint64)

SIGNATURES = {
    "rs_version": (ctypes.c_char_p, []),
    "rs_status_string": (ctypes.c_char_p, [I]),
    "rs_bvh_build": (I, [P, U64, P, U64, P, I, PP, P]),
    "rs_bvh_build_async": (I, [P, U64, P, U64, P, I, PP, P]),
    "rs_bvh_wait": (I, [P]),
    "rs_bvh_destroy": (I, [P]),
    "rs_bvh_info": (I, [P, PU64, PU64, PU64, P, P]),
    "rs_pim": (I, [P, P, U64, F, F, F, P, P, P]),
    "rs_pim_filtered": (I, [P, P, U64, F, F, F, P, P, P]),
    "rs_pim_noalloc": (I, [P, P, U64, F, F, F, P, P, I, P]),
    "rs_compact_hits": (I, [P, U64, P, P, U64, PU64, P]),
    "rs_pairset_create": (I, [U64, I, PP, P]),
    "rs_pairset_clear": (I, [P, P]),
    "rs_pairset_destroy": (I, [P]),
    "rs_pairset_info": (I, [P, PU64, PU64, P]),
    "rs_edge_join": (I, [P, P, P, P, P, P, U64, I, P, P]),
    "rs_containment": (I, [P, P, U64, P, U64, P, I, P, P]),
    "rs_pairset_finalize": (I, [P, I, P, U64, PU64, P]),
    "rs_containment_tracked": (I, [P, P, U64, P, U64, P, I, P, I, P, P, P, U64, P]),
    "rs_pairset_set_tracking": (I, [P, I]),
    "rs_pairset_set_edge_rule": (I, [P, I, I]),
    "rs_pairset_counters": (I, [P, PU64, P]),
    "rs_estimate_grid": (I, [P, P, U64, F, F, F, ctypes.POINTER(ctypes.c_double), P, P]),
    "rs_estimate_grid_cells": (I, [P, P, U64, F, F, F, P, P]),
    "rs_estimate_pairs_from_raw": (I64, [ctypes.c_double, P, F, I]),
    "rs_kernel_pointer": (I, [P, PP]),
    "rs_hash_size_pow2": (U64, [I64]),
    "rs_hash_size_odd": (U64, [I64, F]),
    "rs_overlap_join": (I, [P, P, P, P, P, P, U64, P, P, P, P, P, P, U64, I, I, P, P]),
    "rs_overlap_join_after": (I, [P, P, P, P, P, P, U64, P, P, P, P, P, P, U64, I, I, P, P, P, P]),
    "rs_edge_index": (I, [P, P, P, U64, U64, P, ctypes.POINTER(I), P]),
    "rs_overlap_join_indexed": (I, [P, P, P, P, P, P, U64, P, P, P, P, P, P, P, U64, P, I, I, P, P, P, P]),
    "rs_overlap_join_filtered": (I, [P, U64, P, U64, P, P, P, P, P, P, U64, P, U64, P, U64, P, P, P, P, P, P, U64,
                                     I, I, I, P, P]),
    "rs_launch_count": (U64, []),
    "rs_alloc_count": (U64, []),
    "rs_profile_enable": (I, [I]),
    "rs_profile_reset": (I, []),
    "rs_profile_read": (I, [I, ctypes.POINTER(ctypes.c_double), PU64]),
    "rs_recheck_enable": (I, [I]),
    "rs_set_overlap_cull": (I, [I]),
    "rs_grid_stats": (I, [P, U64, P, U64, P, U64, I, F, P, ctypes.POINTER(F), P]),
    "rs_triangle_join": (I, [P, P, U64, P, U64, P, I, P, P]),
    "rs_extract_edges": (I, [P, U64, P, U64, P, P, P, P, P, P, U64, PU64, PU64, P]),
    "rs_mlp_create": (I, [U64, PP]),
    "rs_mlp_destroy": (I, [P]),
    "rs_mlp_num_params": (U64, []),
    "rs_mlp_get_params": (I, [P, ctypes.POINTER(F), ctypes.POINTER(F)]),
    "rs_mlp_set_params": (I, [P, ctypes.POINTER(F)]),
    "rs_mlp_features": (I, [P, P, I, P, P]),
    "rs_mlp_gemm": (I, [P, I, P, I, P, I, I, I, I, I, P]),
    "rs_mlp_set_weight_decay": (I, [P, F]),
    "rs_mlp_set_prior": (I, [P, I, F, F, F, I]),
    "rs_mlp_set_gemm": (I, [I]),
    "rs_mlp_forward": (I, [P, P, I, P, P]),
    "rs_mlp_gradients": (I, [P, P, P, I, ctypes.POINTER(F), P]),
    "rs_mlp_train_step": (I, [P, P, P, I, F, ctypes.POINTER(F), P]),
    "rs_estimate_mlp": (I, [P, P, P, I, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_double), P]),
    "rs_batch_create": (I, [PP]),
    "rs_batch_destroy": (I, [P]),
    "rs_batch_add_pim": (I, [P, P, P, U64, F, F, F, P, P, ctypes.POINTER(I)]),
    "rs_batch_add_edges": (I, [P, P, P, P, P, P, P, U64, I, P, ctypes.POINTER(I)]),
    "rs_batch_set_options": (I, [P, I, I, I]),
    "rs_batch_submit": (I, [P, P]),
    "rs_batch_wait": (I, [P, ctypes.POINTER(I)]),
    "rs_batch_autotune": (I, [P, ctypes.POINTER(I), ctypes.POINTER(I), ctypes.POINTER(I),
                              ctypes.POINTER(ctypes.c_double), P]),
    "rs_recheck_reset": (I, []),
    "rs_recheck_read": (I, [PU64, PU64]),
    "exclusive_scan_gpu": (ctypes.c_longlong, [P, P, I]),
    "merge_and_deduplicate_pairs_gpu": (ctypes.c_longlong, [P, ctypes.c_longlong, P, ctypes.c_longlong, P]),
    "compact_hash_table_pairs": (I, [P, ctypes.c_ulonglong, P, I]),
    "count_hits_gpu": (I, [P, I]),
    "compact_hits_gpu": (None, [P, P, I, ctypes.POINTER(ctypes.c_int)]),
    "rs_estimate_overlap_selectivity": (F, [P, P, I, F, F, F]),
    "rs_estimate_intersection_selectivity": (F, [P, P, I, F, F, F]),
}

_lib = None


class RsError(RuntimeError):
    def __init__(self, status: int, what: str):
        self.status = status
        super().__init__(f"{what}: rs_status {status} ({status_string(status)})")


def load(path: str = LIB_PATH):
    """Load librs.so; raises if it is missing (build it with __graft_entry__.build())."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"librs.so not found at {path}: the CUDA engine is not built "
                           "(run `python -c 'import __graft_entry__ as g; g.build()'`)")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def status_string(status: int) -> str:
    try:
        return load().rs_status_string(status).decode()
    except Exception:  # pragma: no cover - only when the library is absent
        return "?"


def check(status: int, what: str) -> None:
    if status != RS_OK:
        raise RsError(status, what)
