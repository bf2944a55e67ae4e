"""ctypes wrapper of the oracle (liboracle.so) and of oracle/_ref.

TEST INFRASTRUCTURE ONLY: the oracle the CUDA path's results are compared
with, and the benchmark's CPU-baseline leg.  The product never imports this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libproteus_radix_ref.so")

vp, u64, i32, i64 = C.c_void_p, C.c_uint64, C.c_int32, C.c_int64


class ChainedTable(C.Structure):
    _fields_ = [("head", vp), ("next", vp), ("key", vp), ("payload", vp), ("n", u64),
                ("hash_bits", i32), ("key64", vp)]


_lib = None
_ref = None


def build():
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)


def build_ref(ref_root=None):
    """Compiles oracle/_ref from the reference sources (the tree named by
    `ref_root` or $PROTEUS_REF), when they are present."""
    ref_root = ref_root or os.environ.get("PROTEUS_REF")
    if not ref_root or not os.path.isdir(os.path.join(ref_root, "core", "platform")):
        return False
    subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={ref_root}"], check=True)
    return True


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        L.orc_hash_int32.restype, L.orc_hash_int32.argtypes = u64, [i32]
        L.orc_hashd.restype, L.orc_hashd.argtypes = C.c_uint32, [i32]
        L.orc_join_build.restype = C.c_int
        L.orc_join_build.argtypes = [vp, vp, u64, i32, C.POINTER(ChainedTable)]
        L.orc_join_build_mt.restype = C.c_int
        L.orc_join_build_mt.argtypes = [vp, vp, u64, i32, C.c_int, C.POINTER(ChainedTable)]
        L.orc_join_free.restype, L.orc_join_free.argtypes = None, [C.POINTER(ChainedTable)]
        L.orc_join_probe_agg.restype = C.c_int
        L.orc_join_probe_agg.argtypes = [C.POINTER(ChainedTable), vp, vp, u64, vp, vp, i32, vp,
                                         C.c_int]
        L.orc_join_probe_pairs.restype = i64
        L.orc_join_probe_pairs.argtypes = [C.POINTER(ChainedTable), vp, u64, vp, vp, u64]
        L.orc_hash_int64.restype, L.orc_hash_int64.argtypes = u64, [i64]
        L.orc_join_build_i64.restype = C.c_int
        L.orc_join_build_i64.argtypes = [vp, vp, u64, i32, C.POINTER(ChainedTable)]
        L.orc_join_probe_agg_i64.restype = C.c_int
        L.orc_join_probe_agg_i64.argtypes = [C.POINTER(ChainedTable), vp, vp, u64, vp, vp, i32, vp]
        L.orc_join_probe_pairs_i64.restype = i64
        L.orc_join_probe_pairs_i64.argtypes = [C.POINTER(ChainedTable), vp, u64, vp, vp, u64]
        L.orc_radix_cluster.restype = None
        L.orc_radix_cluster.argtypes = [vp, vp, u64, i32, i32, i32, vp, vp, vp]
        L.orc_rj_stepwise.restype, L.orc_rj_stepwise.argtypes = i64, [vp, u64, vp, u64]
        L.orc_partition_ht_counts.restype = None
        L.orc_partition_ht_counts.argtypes = [vp, u64, vp]
        L.orc_radix_join_agg.restype = C.c_int
        L.orc_radix_join_agg.argtypes = [vp, vp, u64, vp, vp, u64, i32, vp, vp, i32, vp, C.c_int]
        L.orc_radix_join_agg_minor.restype = C.c_int
        L.orc_radix_join_agg_minor.argtypes = [vp, vp, vp, u64, vp, vp, vp, u64, i32, vp, vp, i32,
                                               vp, C.c_int]
        L.orc_groupby.restype = i64
        L.orc_groupby.argtypes = [vp, vp, u64, i32, C.c_int, vp, vp, vp, vp, vp, u64]
        L.orc_reduce.restype = None
        L.orc_reduce.argtypes = [vp, vp, u64, vp, vp, i32, vp]
        L.orc_radix_cluster_i64.restype = None
        L.orc_radix_cluster_i64.argtypes = [vp, vp, u64, i32, i32, vp, vp, vp]
        L.orc_partition_ht_agg.restype = None
        L.orc_partition_ht_agg.argtypes = [vp, u64, vp, vp, vp]
        L.orc_join_count_i64.restype = i64
        L.orc_join_count_i64.argtypes = [vp, u64, vp, u64]
        L.orc_nest_i64.restype = i64
        L.orc_nest_i64.argtypes = [vp, vp, u64, vp, vp, vp, vp, vp, u64]
        L.orc_bloom_semijoin.restype = i64
        L.orc_bloom_semijoin.argtypes = [vp, u64, vp, u64, u64, vp, u64]
        L.orc_join_groupby.restype = i64
        L.orc_join_groupby.argtypes = [vp, vp, u64, vp, vp, u64, C.c_int, vp, vp, vp, vp, vp, u64]
        L.orc_star_query.restype = i64
        L.orc_star_query.argtypes = [vp, i32, vp, vp, u64, vp, vp, C.c_int, vp, vp, vp, vp, u64]
        _lib = L
    return _lib


def ref_lib():
    """The reference's own RJStepwise / partitionHT (None if not built)."""
    global _ref
    if _ref is None and os.path.exists(REF_LIB):
        R = C.CDLL(REF_LIB)
        R.ref_rj_stepwise.restype = i64
        R.ref_rj_stepwise.argtypes = [vp, C.c_uint32, vp, C.c_uint32]
        R.ref_partition_ht.restype = None
        R.ref_partition_ht.argtypes = [vp, C.c_uint32, vp, vp, vp]
        R.ref_partition_ht_agg.restype = None
        R.ref_partition_ht_agg.argtypes = [vp, C.c_uint32, vp, vp, vp]
        R.ref_rj_stepwise_agg.restype = i64
        R.ref_rj_stepwise_agg.argtypes = [vp, C.c_uint32, vp, C.c_uint32]
        R.ref_nest_counts.restype = None
        R.ref_nest_counts.argtypes = [vp, C.c_uint32, vp, C.c_uint32, vp]
        R.ref_num_radix_bits.restype = i32
        _ref = R
    return _ref


def _p(a):
    return None if a is None else a.ctypes.data_as(vp)


def _i32(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.int32)


def _aggs(aggs):
    ops = np.array([a[0] for a in aggs], dtype=np.int32)
    opd = np.array([a[1] for a in aggs], dtype=np.int32)
    return ops, opd


def join_agg(bkeys, bpay, pkeys, ppay, aggs, hash_bits=0, threads=1):
    """HashJoinChained build + probe with the fused aggregates -> int64 list."""
    L = lib()
    bkeys, bpay, pkeys, ppay = _i32(bkeys), _i32(bpay), _i32(pkeys), _i32(ppay)
    t = ChainedTable()
    if threads > 1:
        rc = L.orc_join_build_mt(_p(bkeys), _p(bpay), len(bkeys), hash_bits, threads, C.byref(t))
    else:
        rc = L.orc_join_build(_p(bkeys), _p(bpay), len(bkeys), hash_bits, C.byref(t))
    assert rc == 0
    ops, opd = _aggs(aggs)
    out = np.zeros(len(aggs), dtype=np.int64)
    rc = L.orc_join_probe_agg(C.byref(t), _p(pkeys), _p(ppay), len(pkeys), _p(ops), _p(opd),
                              len(aggs), _p(out), threads)
    L.orc_join_free(C.byref(t))
    assert rc == 0
    return [int(x) for x in out]


def join_agg_i64(bkeys, bpay, pkeys, ppay, aggs, hash_bits=0):
    """HashJoinChained over int64 keys (hashInt64 placement) -> int64 list."""
    L = lib()
    bkeys, pkeys = np.ascontiguousarray(bkeys, dtype=np.int64), np.ascontiguousarray(pkeys, dtype=np.int64)
    bpay, ppay = _i32(bpay), _i32(ppay)
    t = ChainedTable()
    assert L.orc_join_build_i64(_p(bkeys), _p(bpay), len(bkeys), hash_bits, C.byref(t)) == 0
    ops, opd = _aggs(aggs)
    out = np.zeros(len(aggs), dtype=np.int64)
    rc = L.orc_join_probe_agg_i64(C.byref(t), _p(pkeys), _p(ppay), len(pkeys), _p(ops), _p(opd),
                                  len(aggs), _p(out))
    L.orc_join_free(C.byref(t))
    assert rc == 0
    return [int(x) for x in out]


def join_pairs_i64(bkeys, pkeys, hash_bits=0):
    L = lib()
    bkeys, pkeys = np.ascontiguousarray(bkeys, dtype=np.int64), np.ascontiguousarray(pkeys, dtype=np.int64)
    t = ChainedTable()
    assert L.orc_join_build_i64(_p(bkeys), None, len(bkeys), hash_bits, C.byref(t)) == 0
    m = L.orc_join_probe_pairs_i64(C.byref(t), _p(pkeys), len(pkeys), None, None, 0)
    b = np.empty(max(m, 1), dtype=np.int32)
    p = np.empty(max(m, 1), dtype=np.int32)
    L.orc_join_probe_pairs_i64(C.byref(t), _p(pkeys), len(pkeys), _p(b), _p(p), m)
    L.orc_join_free(C.byref(t))
    return b[:m], p[:m]


def join_pairs(bkeys, pkeys, hash_bits=0):
    L = lib()
    bkeys, pkeys = _i32(bkeys), _i32(pkeys)
    t = ChainedTable()
    assert L.orc_join_build(_p(bkeys), None, len(bkeys), hash_bits, C.byref(t)) == 0
    m = L.orc_join_probe_pairs(C.byref(t), _p(pkeys), len(pkeys), None, None, 0)
    b = np.empty(max(m, 1), dtype=np.int32)
    p = np.empty(max(m, 1), dtype=np.int32)
    L.orc_join_probe_pairs(C.byref(t), _p(pkeys), len(pkeys), _p(b), _p(p), m)
    L.orc_join_free(C.byref(t))
    return b[:m], p[:m]


def radix_cluster(keys, payload, R, D, hashed):
    L = lib()
    keys, payload = _i32(keys), _i32(payload)
    n = len(keys)
    ok = np.empty(max(n, 1), dtype=np.int32)
    op = np.empty(max(n, 1), dtype=np.int32)
    off = np.empty((1 << D) + 1, dtype=np.uint64)
    L.orc_radix_cluster(_p(keys), _p(payload), n, R, D, int(hashed), _p(ok), _p(op), _p(off))
    return ok[:n], op[:n], off


def rj_stepwise(rkeys, skeys):
    L = lib()
    rkeys, skeys = _i32(rkeys), _i32(skeys)
    return int(L.orc_rj_stepwise(_p(rkeys), len(rkeys), _p(skeys), len(skeys)))


def partition_ht_counts(keys):
    L = lib()
    keys = _i32(keys)
    c = np.empty(1 << 14, dtype=np.int32)
    L.orc_partition_ht_counts(_p(keys), len(keys), _p(c))
    return c


def radix_join_agg(bkeys, bpay, pkeys, ppay, aggs, bits=0, threads=1):
    L = lib()
    bkeys, bpay, pkeys, ppay = _i32(bkeys), _i32(bpay), _i32(pkeys), _i32(ppay)
    ops, opd = _aggs(aggs)
    out = np.zeros(len(aggs), dtype=np.int64)
    rc = L.orc_radix_join_agg(_p(bkeys), _p(bpay), len(bkeys), _p(pkeys), _p(ppay), len(pkeys),
                              bits, _p(ops), _p(opd), len(aggs), _p(out), threads)
    assert rc == 0
    return [int(x) for x in out]


def radix_join_agg_minor(bkeys, bminor, bpay, pkeys, pminor, ppay, aggs, bits=0, threads=1):
    """Partitioned join whose pairs also need equal minor keys (both minor
    columns given, or both None); payloads and row ids read by row."""
    L = lib()
    bkeys, bminor, bpay = _i32(bkeys), _i32(bminor), _i32(bpay)
    pkeys, pminor, ppay = _i32(pkeys), _i32(pminor), _i32(ppay)
    ops, opd = _aggs(aggs)
    out = np.zeros(len(aggs), dtype=np.int64)
    rc = L.orc_radix_join_agg_minor(_p(bkeys), _p(bminor), _p(bpay), len(bkeys), _p(pkeys),
                                    _p(pminor), _p(ppay), len(pkeys), bits, _p(ops), _p(opd),
                                    len(aggs), _p(out), threads)
    assert rc == 0
    return [int(x) for x in out]


def groupby(keys, values, hash_bits=0, threads=1):
    """-> (keys, count, sum, min, max) sorted by key."""
    L = lib()
    keys, values = _i32(keys), _i32(values)
    n = len(keys)
    ng = L.orc_groupby(_p(keys), _p(values), n, hash_bits, threads, None, None, None, None, None, 0)
    assert ng >= 0
    k = np.empty(max(ng, 1), dtype=np.int32)
    c = np.empty(max(ng, 1), dtype=np.int64)
    s = np.empty(max(ng, 1), dtype=np.int64)
    mn = np.empty(max(ng, 1), dtype=np.int32)
    mx = np.empty(max(ng, 1), dtype=np.int32)
    ng2 = L.orc_groupby(_p(keys), _p(values), n, hash_bits, threads, _p(k), _p(c), _p(s), _p(mn),
                        _p(mx), ng)
    assert ng2 == ng
    return k[:ng], c[:ng], s[:ng], mn[:ng], mx[:ng]


def reduce(col, aggs, rows=None):
    L = lib()
    col, rows = _i32(col), _i32(rows)
    ops, opd = _aggs(aggs)
    out = np.zeros(len(aggs), dtype=np.int64)
    n = len(rows) if rows is not None else len(col)
    L.orc_reduce(_p(col), _p(rows), n, _p(ops), _p(opd), len(aggs), _p(out))
    return [int(x) for x in out]


def radix_cluster_i64(keys, payload, R, D):
    """-> (clustered keys, payloads, offsets[2^D + 1]), stable."""
    L = lib()
    keys = np.ascontiguousarray(keys, dtype=np.int64)
    pay = None if payload is None else np.ascontiguousarray(payload, dtype=np.int64)
    n = len(keys)
    ok, op = np.empty(max(n, 1), np.int64), np.empty(max(n, 1), np.int64)
    off = np.empty((1 << D) + 1, np.uint64)
    L.orc_radix_cluster_i64(_p(keys), _p(pay), n, R, D, _p(ok), _p(op), _p(off))
    return ok[:n], op[:n], off


def partition_ht_agg(keys):
    """partitionHT of the int64-key twin -> (counts[2^14], keys, row ids)."""
    L = lib()
    keys = np.ascontiguousarray(keys, dtype=np.int64)
    n = len(keys)
    c = np.empty(1 << 14, np.int32)
    ok, op = np.empty(max(n, 1), np.int64), np.empty(max(n, 1), np.int64)
    L.orc_partition_ht_agg(_p(keys), n, _p(c), _p(ok), _p(op))
    return c, ok[:n], op[:n]


def join_count_i64(r_keys, s_keys):
    """RJStepwise of the int64-key twin: matching (R, S) pairs."""
    L = lib()
    r = np.ascontiguousarray(r_keys, dtype=np.int64)
    s = np.ascontiguousarray(s_keys, dtype=np.int64)
    return int(L.orc_join_count_i64(_p(r), len(r), _p(s), len(s)))


def nest_i64(keys, vals=None):
    """RadixNest over int64 keys -> (keys, count, sum, min, max) sorted by key."""
    L = lib()
    keys = np.ascontiguousarray(keys, dtype=np.int64)
    v = None if vals is None else np.ascontiguousarray(vals, dtype=np.int64)
    n = len(keys)
    out = [np.empty(max(n, 1), np.int64) for _ in range(5)]
    ng = int(L.orc_nest_i64(_p(keys), _p(v), n, *[_p(a) for a in out], max(n, 1)))
    return tuple(a[:ng] for a in out)


def bloom_semijoin(build, probe, filter_size):
    """Positions of the probe rows the reference's bloom filter passes."""
    L = lib()
    build, probe = _i32(build), _i32(probe)
    out = np.empty(max(len(probe), 1), dtype=np.int32)
    m = L.orc_bloom_semijoin(_p(build), len(build), _p(probe), len(probe), filter_size, _p(out), len(out))
    assert m >= 0
    return out[:m]


def join_groupby(bk, bg, pk, pv, threads=1):
    """Join on build keys, group by the matched build row's group:
    -> (group, count, sum, min, max) sorted by group."""
    L = lib()
    bk, bg, pk, pv = _i32(bk), _i32(bg), _i32(pk), _i32(pv)
    ng = L.orc_join_groupby(_p(bk), _p(bg), len(bk), _p(pk), _p(pv), len(pk), threads, None, None,
                            None, None, None, 0)
    assert ng >= 0
    m = max(ng, 1)
    out = (np.empty(m, np.int32), np.empty(m, np.int64), np.empty(m, np.int64), np.empty(m, np.int32),
           np.empty(m, np.int32))
    ng2 = L.orc_join_groupby(_p(bk), _p(bg), len(bk), _p(pk), _p(pv), len(pk), threads,
                             *[_p(a) for a in out], ng)
    assert ng2 == ng
    return tuple(a[:ng] for a in out)


class StarDim(C.Structure):
    _fields_ = [("n", u64), ("key_base", i32), ("n_attrs", i32), ("attr", vp * 4),
                ("attr_type", i32 * 4), ("attr_min", i32 * 4), ("attr_max", i32 * 4), ("keys", vp)]


class StarQ(C.Structure):
    _fields_ = [("join_mask", i32), ("pred_attr", i32 * 4), ("pred_lo", i32 * 4),
                ("pred_hi", i32 * 4), ("group_dim", i32 * 2), ("group_attr", i32 * 2)]


def star_query(data, query, threads=1, rows=None):
    """One star query (a proteus_gb300.star.Query) over a StarData, on the
    fact rows [0, rows) (all when None) -> (a, b, count, sum) sorted by (a, b)."""
    L = lib()
    nd = len(data.dims)
    n = data.n_fact if rows is None else int(rows)
    fk = [np.ascontiguousarray(c[:n], dtype=np.int32) for c in data.fk]
    qty = np.ascontiguousarray(data.quantity[:n], dtype=np.int32)
    price = np.ascontiguousarray(data.price[:n], dtype=np.int32)
    fk_ptrs = (vp * 4)(*[c.ctypes.data for c in fk])
    dims = (StarDim * 4)()
    for d, dim in enumerate(data.dims):
        dims[d].n, dims[d].key_base, dims[d].n_attrs = dim.n, 1, len(dim.attrs)
        if dim.keys is not None:
            dims[d].keys = dim.keys.ctypes.data
        for a, col in enumerate(dim.attrs):
            dims[d].attr[a] = col.ctypes.data
            dims[d].attr_type[a] = 1 if col.dtype == np.int8 else 0
    q = StarQ()
    q.join_mask = query.join_mask
    for d in range(4):
        q.pred_attr[d], q.pred_lo[d], q.pred_hi[d] = query.pred_attr[d], query.pred_lo[d], query.pred_hi[d]
    for k in range(2):
        q.group_dim[k], q.group_attr[k] = query.group_dim[k], query.group_attr[k]
    cap = 4096
    a = np.empty(cap, dtype=np.int32)
    b = np.empty(cap, dtype=np.int32)
    c = np.empty(cap, dtype=np.int64)
    s = np.empty(cap, dtype=np.int64)
    ng = L.orc_star_query(fk_ptrs, nd, _p(qty), _p(price), n, dims, C.byref(q), threads, _p(a), _p(b),
                          _p(c), _p(s), cap)
    assert 0 <= ng <= cap, ng
    return a[:ng], b[:ng], c[:ng], s[:ng]


def ref_rj_stepwise(rkeys, skeys):
    R = ref_lib()
    if R is None:
        return None
    rkeys, skeys = _i32(rkeys), _i32(skeys)
    return int(R.ref_rj_stepwise(_p(rkeys), len(rkeys), _p(skeys), len(skeys)))


def ref_partition_ht_agg(keys):
    """The reference's own int64-key partitionHT (oracle/_ref)."""
    R = ref_lib()
    if R is None:
        return None
    keys = np.ascontiguousarray(keys, dtype=np.int64)
    n = len(keys)
    c = np.empty(1 << 14, dtype=np.int32)
    ok, op = np.empty(max(n, 1), np.int64), np.empty(max(n, 1), np.int64)
    R.ref_partition_ht_agg(_p(keys), n, _p(c), _p(ok), _p(op))
    return c, ok[:n], op[:n]


def ref_rj_stepwise_agg(rkeys, skeys):
    """The reference's own int64-key RJStepwise (oracle/_ref): match count."""
    R = ref_lib()
    if R is None:
        return None
    r = np.ascontiguousarray(rkeys, dtype=np.int64)
    s = np.ascontiguousarray(skeys, dtype=np.int64)
    return int(R.ref_rj_stepwise_agg(_p(r), len(r), _p(s), len(s)))


def ref_nest_counts(keys, query):
    """Group size of each query key from the reference's own partitionHT and
    bucket chains (oracle/_ref)."""
    R = ref_lib()
    if R is None:
        return None
    keys = np.ascontiguousarray(keys, dtype=np.int64)
    query = np.ascontiguousarray(query, dtype=np.int64)
    out = np.empty(max(len(query), 1), np.int64)
    R.ref_nest_counts(_p(keys), len(keys), _p(query), len(query), _p(out))
    return out[:len(query)]


def ref_partition_ht(keys):
    R = ref_lib()
    if R is None:
        return None
    keys = _i32(keys)
    n = len(keys)
    c = np.empty(1 << 14, dtype=np.int32)
    ok = np.empty(max(n, 1), dtype=np.int32)
    orows = np.empty(max(n, 1), dtype=np.int64)
    R.ref_partition_ht(_p(keys), n, _p(c), _p(ok), _p(orows))
    return c, ok[:n], orows[:n]
