"""ctypes binding of libgbjoin.so (the C ABI declared in include/gbjoin.h).

The product is the shared library; this module only loads it and gives the
entry points Python signatures.  Importing it on a machine without the built
library raises -- there is no fallback implementation.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgbjoin.so")

OK, ERR_INVALID, ERR_OOM, ERR_CAPACITY, ERR_TIMEOUT, ERR_CUDA, ERR_UNSUPPORTED, \
    ERR_BUDGET, ERR_CANCELLED = range(9)
STATUS_NAMES = {0: "OK", 1: "INVALID", 2: "OOM", 3: "CAPACITY", 4: "TIMEOUT", 5: "CUDA",
                6: "UNSUPPORTED", 7: "BUDGET", 8: "CANCELLED"}

AGG_COUNT, AGG_SUM, AGG_MIN, AGG_MAX, AGG_OR, AGG_AND = range(6)
(VAL_ONE, VAL_BUILD, VAL_PROBE, VAL_PRODUCT, VAL_BUILD_ROWID, VAL_PROBE_ROWID,
 VAL_ROWID_XOR, VAL_BUILD_KEY) = range(8)
DIGIT_KEY, DIGIT_HASH = 0, 1
NOALLOC_MAX_BUILD = 1 << 20
MAX_AGGS = 8


class Agg(C.Structure):
    _fields_ = [("op", C.c_int32), ("operand", C.c_int32)]


class RadixParams(C.Structure):
    _fields_ = [("bits", C.c_int32), ("passes", C.c_int32), ("block", C.c_int32),
                ("log_parts", C.c_int32)]


class GroupbyParams(C.Structure):
    _fields_ = [("hash_bits", C.c_int32), ("strategy", C.c_int32),
                ("max_input_size", C.c_uint64), ("expected_groups", C.c_uint64)]


STAR_MAX_DIMS, STAR_MAX_ATTRS, STAR_MAX_QUERIES, STAR_MAX_GROUPS = 4, 4, 64, 4096
ATTR_I32, ATTR_I8 = 0, 1


class StarDim(C.Structure):
    _fields_ = [("n", C.c_uint64), ("key_base", C.c_int32), ("n_attrs", C.c_int32),
                ("d_attr", C.c_void_p * STAR_MAX_ATTRS), ("attr_type", C.c_int32 * STAR_MAX_ATTRS),
                ("attr_min", C.c_int32 * STAR_MAX_ATTRS), ("attr_max", C.c_int32 * STAR_MAX_ATTRS),
                ("d_keys", C.c_void_p)]


class StarFact(C.Structure):
    _fields_ = [("n", C.c_uint64), ("n_dims", C.c_int32),
                ("d_fk", C.c_void_p * STAR_MAX_DIMS), ("d_quantity", C.c_void_p),
                ("d_price", C.c_void_p)]


class StarQuery(C.Structure):
    _fields_ = [("join_mask", C.c_int32), ("pred_attr", C.c_int32 * STAR_MAX_DIMS),
                ("pred_lo", C.c_int32 * STAR_MAX_DIMS), ("pred_hi", C.c_int32 * STAR_MAX_DIMS),
                ("group_dim", C.c_int32 * 2), ("group_attr", C.c_int32 * 2)]


class StarOut(C.Structure):
    _fields_ = [("d_key_a", C.c_void_p), ("d_key_b", C.c_void_p), ("d_count", C.c_void_p),
                ("d_sum", C.c_void_p), ("d_n_groups", C.c_void_p), ("group_cap", C.c_uint64)]


SERVE_MAX_BATCH = 64


class ServeQuery(C.Structure):
    _fields_ = [("d_build_keys", C.c_void_p), ("d_build_group", C.c_void_p), ("n_build", C.c_uint64),
                ("d_probe_keys", C.c_void_p), ("d_probe_vals", C.c_void_p), ("n_probe", C.c_uint64),
                ("expected_groups", C.c_uint64), ("out_group", C.c_void_p), ("out_count", C.c_void_p),
                ("out_sum", C.c_void_p), ("out_n_groups", C.c_void_p), ("out_capacity", C.c_uint64),
                ("table_id", C.c_uint64)]


class ServerParams(C.Structure):
    _fields_ = [("hbm_budget", C.c_uint64), ("max_batch", C.c_int32), ("max_inflight", C.c_int32),
                ("use_graph", C.c_int32), ("large_slots", C.c_int32), ("small_rows", C.c_uint64)]


vp, u64, i32, i64, dbl = C.c_void_p, C.c_uint64, C.c_int32, C.c_int64, C.c_double
P = C.POINTER

# name -> (restype, argtypes); mirrors include/gbjoin.h
SIGNATURES = {
    "gbj_ctx_create": (C.c_int, [C.c_int, u64, P(vp)]),
    "gbj_ctx_destroy": (C.c_int, [vp]),
    "gbj_last_error": (C.c_char_p, [vp]),
    "gbj_ctx_device_info": (C.c_int, [vp, P(C.c_int), P(u64), P(u64)]),
    "gbj_sync": (C.c_int, [vp, vp]),
    "gbj_kernel_launches": (u64, [vp]),
    "gbj_profile_enable": (C.c_int, [vp, C.c_int]),
    "gbj_profile_kernel": (C.c_int, [vp, C.c_char_p, P(u64), P(dbl)]),
    "gbj_profile_dump": (C.c_int, [vp, C.c_char_p, u64]),
    "gbj_pool_alloc": (C.c_int, [vp, u64, P(vp)]),
    "gbj_pool_free": (C.c_int, [vp, vp]),
    "gbj_pool_stats": (C.c_int, [vp, P(u64), P(u64), P(u64)]),
    "gbj_ctx_set_pool_limit": (C.c_int, [vp, u64]),
    "gbj_join_build": (C.c_int, [vp, vp, vp, u64, i32, u64, vp, P(vp)]),
    "gbj_join_probe_agg": (C.c_int, [vp, vp, vp, vp, u64, P(Agg), i32, vp, vp]),
    "gbj_join_probe_pairs": (C.c_int, [vp, vp, vp, vp, u64, vp, vp, u64, vp, vp]),
    "gbj_join_build_i64": (C.c_int, [vp, vp, vp, u64, i32, u64, vp, P(vp)]),
    "gbj_join_probe_agg_i64": (C.c_int, [vp, vp, vp, vp, u64, P(Agg), i32, vp, vp]),
    "gbj_join_probe_pairs_i64": (C.c_int, [vp, vp, vp, vp, u64, vp, vp, u64, vp, vp]),
    "gbj_table_destroy": (C.c_int, [vp, vp]),
    "gbj_table_slots": (u64, [vp]),
    "gbj_partition": (C.c_int, [vp, vp, vp, u64, i32, i32, i32, vp, vp, vp, vp]),
    "gbj_radix_join_agg": (C.c_int, [vp, vp, vp, u64, vp, vp, u64, P(RadixParams), P(Agg), i32,
                                     vp, vp]),
    "gbj_radix_join_agg_minor": (C.c_int, [vp, vp, vp, vp, u64, vp, vp, vp, u64, P(RadixParams),
                                           P(Agg), i32, vp, vp]),
    "gbj_groupby": (C.c_int, [vp, vp, vp, u64, P(GroupbyParams), vp, vp, vp, vp, vp, u64, vp,
                              vp]),
    "gbj_groupby_i64": (C.c_int, [vp, vp, vp, u64, P(GroupbyParams), vp, vp, vp, vp, vp, u64, vp,
                                  vp]),
    "gbj_reduce": (C.c_int, [vp, vp, vp, u64, P(Agg), i32, vp, vp]),
    "gbj_gather": (C.c_int, [vp, vp, vp, u64, vp, vp]),
    "gbj_select_range": (C.c_int, [vp, vp, u64, i32, i32, vp, vp, vp]),
    "gbj_join_agg_noalloc": (C.c_int, [vp, vp, u64, vp, vp, u64, P(Agg), i32, vp, vp]),
    "gbj_star_plan_create": (C.c_int, [vp, P(StarFact), P(StarDim), P(vp)]),
    "gbj_star_run": (C.c_int, [vp, P(StarQuery), i32, P(StarOut), i32, vp]),
    "gbj_star_plan_destroy": (None, [vp]),
    "gbj_server_create": (C.c_int, [vp, P(ServerParams), P(vp)]),
    "gbj_server_submit": (C.c_int, [vp, P(ServeQuery), P(u64)]),
    "gbj_server_submit_batch": (C.c_int, [vp, P(ServeQuery), u64, P(u64)]),
    "gbj_server_wait": (C.c_int, [vp, u64, dbl, P(i32)]),
    "gbj_server_times": (C.c_int, [vp, u64, P(dbl), P(dbl), P(dbl)]),
    "gbj_server_drain": (C.c_int, [vp]),
    "gbj_server_cancel": (C.c_int, [vp, u64, P(i32)]),
    "gbj_server_pause": (C.c_int, [vp, i32]),
    "gbj_server_retries": (C.c_int, [vp, P(u64)]),
    "gbj_server_busy": (C.c_int, [vp, P(C.c_double)]),
    "gbj_server_stats": (C.c_int, [vp, P(u64), P(u64), P(u64)]),
    "gbj_server_destroy": (C.c_int, [vp]),
    "gbj_server_register_table": (C.c_int, [vp, vp, vp, u64, u64, P(u64)]),
    "gbj_server_unregister_table": (C.c_int, [vp, u64]),
    "gbj_autotune_radix_join": (C.c_int, [vp, vp, vp, u64, vp, vp, u64, P(Agg), i32, P(i32), P(dbl), vp]),
    "gbj_autotune_join": (C.c_int, [vp, vp, vp, u64, vp, vp, u64, P(Agg), i32, P(i32), P(dbl), vp]),
    "gbj_autotune_groupby": (C.c_int, [vp, vp, vp, u64, u64, P(i32), P(i32), P(dbl), vp]),
    "gbj_tune_lookup": (C.c_int, [vp, C.c_char_p, u64, u64, P(i32)]),
    "gbj_tune_clear": (C.c_int, [vp]),
    "gbj_tune_save": (C.c_int, [vp, C.c_char_p]),
    "gbj_tune_load": (C.c_int, [vp, C.c_char_p]),
    "gbj_bloom_build": (C.c_int, [vp, vp, u64, u64, vp, P(vp)]),
    "gbj_bloom_probe": (C.c_int, [vp, vp, vp, u64, vp, vp, vp]),
    "gbj_bloom_destroy": (C.c_int, [vp, vp]),
    "gbj_partition_i64": (C.c_int, [vp, vp, vp, u64, i32, i32, vp, vp, vp, vp]),
    "gbj_nest_i64": (C.c_int, [vp, vp, vp, u64, u64, vp, vp, vp, vp, vp, u64, vp, vp]),
    "gbj_radix_join_count_i64": (C.c_int, [vp, vp, u64, vp, u64, vp, vp]),
    "gbj_sort_by_key": (C.c_int, [vp, P(vp), i32, u64, i32, i32, P(vp), vp]),
    "gbj_hash_rearrange": (C.c_int, [vp, P(vp), i32, u64, i32, C.c_uint32, P(vp), vp, vp]),
    "gbj_catalog_create": (C.c_int, [vp, P(vp)]),
    "gbj_catalog_add_column": (C.c_int, [vp, C.c_char_p, C.c_char_p, vp, u64]),
    "gbj_catalog_load": (C.c_int, [vp, C.c_char_p, C.c_char_p, C.c_char_p, P(u64)]),
    "gbj_catalog_destroy": (C.c_int, [vp]),
    "gbj_plan_validate": (C.c_int, [C.c_char_p, C.c_char_p, u64]),
    "gbj_plan_execute": (C.c_int, [vp, C.c_char_p, P(vp)]),
    "gbj_result_shape": (C.c_int, [vp, P(i32), P(u64)]),
    "gbj_result_name": (C.c_char_p, [vp, i32]),
    "gbj_result_column": (C.c_int, [vp, i32, vp]),
    "gbj_result_destroy": (None, [vp]),
}

_lib = None


def load(path: str = LIB_PATH) -> C.CDLL:
    """Loads the library (once) and applies the signatures."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is not built; run `python -m proteus_gb300.build`")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name, None)
        if f is None:
            continue
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


class GbjError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


def aggs_array(aggs):
    arr = (Agg * len(aggs))()
    for i, (op, operand) in enumerate(aggs):
        arr[i].op, arr[i].operand = op, operand
    return arr
