"""Python wrapper over the C ABI for callers that hold torch CUDA tensors.

Device memory comes from torch tensors (the caller's) or from the library's
resident pool (scratch); kernels run on torch's current CUDA stream unless a
stream is given.  Host-side generators return numpy arrays.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi


def _ptr(t) -> int | None:
    if t is None:
        return None
    return t.data_ptr()


CUDA_STREAM_LEGACY = 1  # cudaStreamLegacy


def _cur_stream():
    """torch's current stream as a cudaStream_t for the ABI.  torch reports
    its default stream as handle 0, which the ABI reads as "the context's own
    stream"; pass cudaStreamLegacy instead so library kernels stay ordered
    with torch's copies on that stream."""
    import torch

    return torch.cuda.current_stream().cuda_stream or CUDA_STREAM_LEGACY


class Table:
    """A built join hash table (gbj_table); keeps its input tensors alive."""

    def __init__(self, ctx: "Context", handle: int, keep, i64: bool = False):
        self.ctx, self.handle, self._keep, self.i64 = ctx, handle, keep, i64

    @property
    def slots(self) -> int:
        return int(self.ctx.lib.gbj_table_slots(self.handle))

    def destroy(self):
        if self.handle:
            self.ctx.lib.gbj_table_destroy(self.ctx.handle, self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


class Context:
    """One device context with its resident pool (gbj_ctx)."""

    def __init__(self, device: int = 0, pool_bytes: int = 0):
        self.lib = abi.load()
        h = C.c_void_p()
        rc = self.lib.gbj_ctx_create(device, pool_bytes, C.byref(h))
        if rc != abi.OK:
            raise abi.GbjError(rc, "gbj_ctx_create failed")
        self.handle = h.value
        self.device = device

    # ------------------------------------------------------------ basics
    def check(self, rc: int):
        if rc != abi.OK:
            msg = self.lib.gbj_last_error(self.handle)
            raise abi.GbjError(rc, msg.decode() if msg else "")

    def sync(self, stream=None):
        self.check(self.lib.gbj_sync(self.handle, stream if stream is not None else _cur_stream()))

    def set_pool_limit(self, nbytes: int):
        """Caps the bytes the resident pool hands out (0 = no cap)."""
        self.check(self.lib.gbj_ctx_set_pool_limit(self.handle, nbytes))

    def launches(self) -> int:
        return int(self.lib.gbj_kernel_launches(self.handle))

    def device_info(self):
        sm, l2, smem = C.c_int(), C.c_uint64(), C.c_uint64()
        self.check(self.lib.gbj_ctx_device_info(self.handle, C.byref(sm), C.byref(l2), C.byref(smem)))
        return {"sm_count": sm.value, "l2_bytes": l2.value, "smem_optin": smem.value}

    def pool_stats(self):
        a, b, c = C.c_uint64(), C.c_uint64(), C.c_uint64()
        self.check(self.lib.gbj_pool_stats(self.handle, C.byref(a), C.byref(b), C.byref(c)))
        return {"capacity": a.value, "in_use": b.value, "peak": c.value}

    def profile(self, on: bool):
        self.check(self.lib.gbj_profile_enable(self.handle, 1 if on else 0))

    def profile_kernel(self, name: str):
        n, ms = C.c_uint64(), C.c_double()
        self.check(self.lib.gbj_profile_kernel(self.handle, name.encode(), C.byref(n), C.byref(ms)))
        return n.value, ms.value

    def profile_dump(self):
        buf = C.create_string_buffer(1 << 16)
        self.check(self.lib.gbj_profile_dump(self.handle, buf, len(buf)))
        out = {}
        for line in buf.value.decode().splitlines():
            name, cnt, ms = line.split()
            out[name] = (int(cnt), float(ms))
        return out

    def close(self):
        if getattr(self, "handle", None):
            self.lib.gbj_ctx_destroy(self.handle)
            self.handle = None

    def _s(self, stream):
        return stream if stream is not None else _cur_stream()

    # ------------------------------------------------------------- joins
    def join_build(self, keys, payload=None, hash_bits=0, max_build=0, stream=None) -> Table:
        """int32 keys -> gbj_join_build, int64 keys -> gbj_join_build_i64."""
        import torch

        i64 = keys.dtype == torch.int64
        fn = self.lib.gbj_join_build_i64 if i64 else self.lib.gbj_join_build
        h = C.c_void_p()
        self.check(fn(self.handle, _ptr(keys), _ptr(payload), keys.numel(), hash_bits, max_build,
                      self._s(stream), C.byref(h)))
        return Table(self, h.value, (keys, payload), i64)

    def join_probe_agg(self, table: Table, keys, payload, aggs, out=None, stream=None):
        import torch

        if out is None:
            out = torch.empty(len(aggs), dtype=torch.int64, device=keys.device)
        arr = abi.aggs_array(aggs)
        fn = self.lib.gbj_join_probe_agg_i64 if table.i64 else self.lib.gbj_join_probe_agg
        self.check(fn(self.handle, table.handle, _ptr(keys), _ptr(payload), keys.numel(), arr, len(aggs),
                      _ptr(out), self._s(stream)))
        return out

    def join_probe_pairs(self, table: Table, keys, capacity, probe_rows=None, stream=None):
        import torch

        dev = keys.device
        b = torch.empty(max(capacity, 1), dtype=torch.int32, device=dev)
        p = torch.empty(max(capacity, 1), dtype=torch.int32, device=dev)
        cnt = torch.zeros(1, dtype=torch.int64, device=dev)
        fn = self.lib.gbj_join_probe_pairs_i64 if table.i64 else self.lib.gbj_join_probe_pairs
        self.check(fn(self.handle, table.handle, _ptr(keys), _ptr(probe_rows), keys.numel(), _ptr(b),
                      _ptr(p), capacity, _ptr(cnt), self._s(stream)))
        return b, p, cnt

    def radix_join_agg(self, bkeys, bpay, pkeys, ppay, aggs, out=None, bits=0, passes=0,
                       log_parts=0, block=0, stream=None):
        import torch

        if out is None:
            out = torch.empty(len(aggs), dtype=torch.int64, device=bkeys.device)
        prm = abi.RadixParams(bits, passes, block, log_parts)
        arr = abi.aggs_array(aggs)
        self.check(self.lib.gbj_radix_join_agg(self.handle, _ptr(bkeys), _ptr(bpay), bkeys.numel(),
                                               _ptr(pkeys), _ptr(ppay), pkeys.numel(),
                                               C.byref(prm), arr, len(aggs), _ptr(out),
                                               self._s(stream)))
        return out

    def radix_join_agg_minor(self, bkeys, bminor, bpay, pkeys, pminor, ppay, aggs, out=None,
                             bits=0, passes=0, stream=None):
        """Partitioned join on (key, minor key): pairs need both equal."""
        import torch

        if out is None:
            out = torch.empty(len(aggs), dtype=torch.int64, device=bkeys.device)
        prm = abi.RadixParams(bits, passes, 0, 0)
        arr = abi.aggs_array(aggs)
        self.check(self.lib.gbj_radix_join_agg_minor(
            self.handle, _ptr(bkeys), _ptr(bminor), _ptr(bpay), bkeys.numel(), _ptr(pkeys),
            _ptr(pminor), _ptr(ppay), pkeys.numel(), C.byref(prm), arr, len(aggs), _ptr(out),
            self._s(stream)))
        return out

    def partition(self, keys, payload, bits, shift=0, digit=abi.DIGIT_HASH, stream=None):
        import torch

        dev = keys.device
        n = keys.numel()
        ok = torch.empty(max(n, 1), dtype=torch.int32, device=dev)
        op = torch.empty(max(n, 1), dtype=torch.int32, device=dev)
        off = torch.empty((1 << bits) + 1, dtype=torch.int64, device=dev)
        self.check(self.lib.gbj_partition(self.handle, _ptr(keys), _ptr(payload), n, digit, shift,
                                          bits, _ptr(ok), _ptr(op), _ptr(off), self._s(stream)))
        return ok[:n], op[:n], off

    # ---------------------------------------------------------- autotuner
    def autotune_radix_join(self, bkeys, bpay, pkeys, ppay, aggs, stream=None):
        """-> (partition bits, ms); later radix joins of this shape use it."""
        arr = abi.aggs_array(aggs)
        b, ms = C.c_int32(), C.c_double()
        self.check(self.lib.gbj_autotune_radix_join(
            self.handle, _ptr(bkeys), _ptr(bpay), bkeys.numel(), _ptr(pkeys), _ptr(ppay), pkeys.numel(),
            arr, len(aggs), C.byref(b), C.byref(ms), self._s(stream)))
        return b.value, ms.value

    def autotune_join(self, bkeys, bpay, pkeys, ppay, aggs, stream=None):
        """-> (hash_bits, ms); later builds of this size use it."""
        arr = abi.aggs_array(aggs)
        b, ms = C.c_int32(), C.c_double()
        self.check(self.lib.gbj_autotune_join(
            self.handle, _ptr(bkeys), _ptr(bpay), bkeys.numel(), _ptr(pkeys), _ptr(ppay), pkeys.numel(),
            arr, len(aggs), C.byref(b), C.byref(ms), self._s(stream)))
        return b.value, ms.value

    def autotune_groupby(self, keys, values, expected_groups, stream=None):
        """-> (strategy, bits, ms); later group-bys of this shape use it."""
        st, b, ms = C.c_int32(), C.c_int32(), C.c_double()
        self.check(self.lib.gbj_autotune_groupby(self.handle, _ptr(keys), _ptr(values), keys.numel(),
                                                 expected_groups, C.byref(st), C.byref(b), C.byref(ms),
                                                 self._s(stream)))
        return st.value, b.value, ms.value

    def tune_lookup(self, op: str, a: int, b: int) -> int:
        v = C.c_int32()
        self.check(self.lib.gbj_tune_lookup(self.handle, op.encode(), a, b, C.byref(v)))
        return v.value

    def tune_save(self, path: str):
        self.check(self.lib.gbj_tune_save(self.handle, path.encode()))

    def tune_load(self, path: str):
        self.check(self.lib.gbj_tune_load(self.handle, path.encode()))

    def tune_clear(self):
        self.check(self.lib.gbj_tune_clear(self.handle))

    # -------------------------------------------------------- bloom filter
    def bloom_build(self, keys, filter_size: int, stream=None):
        h = C.c_void_p()
        self.check(self.lib.gbj_bloom_build(self.handle, _ptr(keys), keys.numel(), filter_size,
                                            self._s(stream), C.byref(h)))
        return h.value

    def bloom_probe(self, bloom, keys, stream=None):
        """-> (passing row ids, count tensor)."""
        import torch

        n = keys.numel()
        rows = torch.empty(max(n, 1), dtype=torch.int32, device=keys.device)
        cnt = torch.zeros(1, dtype=torch.int64, device=keys.device)
        self.check(self.lib.gbj_bloom_probe(self.handle, bloom, _ptr(keys), n, _ptr(rows), _ptr(cnt),
                                            self._s(stream)))
        return rows, cnt

    def bloom_destroy(self, bloom):
        self.check(self.lib.gbj_bloom_destroy(self.handle, bloom))

    # ------------------------------------------- int64-key radix clustering
    def partition_i64(self, keys, payload, bits, shift=0, stream=None):
        """-> (clustered keys, payloads, offsets[2^bits + 1]) of int64 tuples."""
        import torch

        ok = torch.empty_like(keys)
        op = torch.empty_like(keys)
        off = torch.empty((1 << bits) + 1, dtype=torch.int64, device=keys.device)
        self.check(self.lib.gbj_partition_i64(self.handle, _ptr(keys), _ptr(payload), keys.numel(), shift, bits,
                                              _ptr(ok), _ptr(op), _ptr(off), self._s(stream)))
        return ok, op, off

    def nest_i64(self, keys, vals, out_capacity, expected_groups=0, stream=None):
        """RadixNest over int64 keys -> (keys, count, sum, min, max, n_groups) device tensors."""
        import torch

        if vals is not None and vals.numel() != keys.numel():
            raise ValueError("nest_i64: keys and values differ in length")
        cap = max(out_capacity, 1)
        outs = [torch.empty(cap, dtype=torch.int64, device=keys.device) for _ in range(5)]
        ng = torch.zeros(1, dtype=torch.int64, device=keys.device)
        self.check(self.lib.gbj_nest_i64(self.handle, _ptr(keys), _ptr(vals), keys.numel(), expected_groups,
                                         *[_ptr(o) for o in outs], out_capacity, _ptr(ng), self._s(stream)))
        return (*outs, ng)

    def radix_join_count_i64(self, r_keys, s_keys, stream=None):
        """RJStepwise of the int64 twin -> device int64[1] match count."""
        import torch

        out = torch.zeros(1, dtype=torch.int64, device=r_keys.device)
        self.check(self.lib.gbj_radix_join_count_i64(self.handle, _ptr(r_keys), r_keys.numel(), _ptr(s_keys),
                                                     s_keys.numel(), _ptr(out), self._s(stream)))
        return out

    # ----------------------------------------------------------------- sort
    def sort_by_key(self, cols, key_col: int, descending=False, stream=None):
        """-> the columns with rows ordered by cols[key_col] (stable)."""
        import torch

        n = cols[0].numel()
        outs = [torch.empty_like(c) for c in cols]
        ins = (C.c_void_p * len(cols))(*[c.data_ptr() for c in cols])
        ous = (C.c_void_p * len(cols))(*[o.data_ptr() for o in outs])
        self.check(self.lib.gbj_sort_by_key(self.handle, ins, len(cols), n, key_col, 1 if descending else 0,
                                            ous, self._s(stream)))
        return outs

    # ------------------------------------------------------ hash rearrange
    def hash_rearrange(self, cols, key_col: int, num_buckets: int, stream=None):
        """-> (bucket-major output columns, bucket offsets [num_buckets + 1])."""
        import torch

        n = cols[0].numel()
        outs = [torch.empty_like(c) for c in cols]
        off = torch.empty(num_buckets + 1, dtype=torch.int64, device=cols[0].device)
        ins = (C.c_void_p * len(cols))(*[c.data_ptr() for c in cols])
        ous = (C.c_void_p * len(cols))(*[o.data_ptr() for o in outs])
        self.check(self.lib.gbj_hash_rearrange(self.handle, ins, len(cols), n, key_col, num_buckets, ous,
                                               _ptr(off), self._s(stream)))
        return outs, off

    # ----------------------------------------------------------- group-by
    def groupby(self, keys, values, out_capacity, expected_groups=0, max_input_size=0,
                hash_bits=0, strategy=0, stream=None):
        import torch

        if keys.numel() != values.numel():
            raise ValueError("groupby: keys and values differ in length")
        dev = keys.device
        cap = max(out_capacity, 1)
        i64 = keys.dtype == torch.int64  # int64 keys: gbj_groupby_i64
        ok = torch.empty(cap, dtype=torch.int64 if i64 else torch.int32, device=dev)
        oc = torch.empty(cap, dtype=torch.int64, device=dev)
        osum = torch.empty(cap, dtype=torch.int64, device=dev)
        omin = torch.empty(cap, dtype=torch.int32, device=dev)
        omax = torch.empty(cap, dtype=torch.int32, device=dev)
        ng = torch.zeros(1, dtype=torch.int64, device=dev)
        prm = abi.GroupbyParams(hash_bits, strategy, max_input_size, expected_groups)
        fn = self.lib.gbj_groupby_i64 if i64 else self.lib.gbj_groupby
        self.check(fn(self.handle, _ptr(keys), _ptr(values), keys.numel(), C.byref(prm), _ptr(ok),
                      _ptr(oc), _ptr(osum), _ptr(omin), _ptr(omax), out_capacity, _ptr(ng),
                      self._s(stream)))
        return ok, oc, osum, omin, omax, ng

    # ------------------------------------------------------------ columns
    def reduce(self, col, aggs, rows=None, out=None, stream=None):
        import torch

        n = rows.numel() if rows is not None else col.numel()
        if out is None:
            out = torch.empty(len(aggs), dtype=torch.int64, device=col.device)
        arr = abi.aggs_array(aggs)
        self.check(self.lib.gbj_reduce(self.handle, _ptr(col), _ptr(rows), n, arr, len(aggs),
                                       _ptr(out), self._s(stream)))
        return out

    def gather(self, col, rows, stream=None):
        import torch

        out = torch.empty(max(rows.numel(), 1), dtype=torch.int32, device=col.device)
        self.check(self.lib.gbj_gather(self.handle, _ptr(col), _ptr(rows), rows.numel(), _ptr(out),
                                       self._s(stream)))
        return out[: rows.numel()]

    def select_range(self, col, lo, hi, stream=None):
        import torch

        n = col.numel()
        rows = torch.empty(max(n, 1), dtype=torch.int32, device=col.device)
        cnt = torch.zeros(1, dtype=torch.int64, device=col.device)
        self.check(self.lib.gbj_select_range(self.handle, _ptr(col), n, lo, hi, _ptr(rows), _ptr(cnt),
                                             self._s(stream)))
        return rows, cnt


# ------------------------------------------------------ host generators
# The seeded synthetic inputs live in their own library (datagen), so that a
# process can generate them without loading libgbjoin.so; re-exported here
# for callers of this module.
from datagen import gen_build_side, gen_groupby, gen_probe_uniform, gen_probe_zipf  # noqa: E402,F401
