"""Query serving: a wrapper over the gbj_server_* entry points and the
seeded served-query workload.

A served query is
    SELECT b.group, COUNT(*), SUM(p.value) FROM build b JOIN probe p
    ON b.key = p.key GROUP BY b.group
over resident device columns.  Workload shapes: build rows log-uniform in
[2^10, 2^24], probe rows log-uniform in [2^14, 2^27], match rate U[0.3, 1],
group cardinality log-uniform in [2^4, 2^16], Poisson arrivals.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np

from . import abi


@dataclass
class QueryShape:
    n_build: int
    n_probe: int
    match_rate: float
    cardinality: int
    seed: int


def gen_shapes(seed: int, n: int, log_build=(10, 24), log_probe=(14, 27), log_card=(4, 16)) -> list:
    """Seeded query shapes (draws from gbj_gen_rand: identical everywhere)."""
    import datagen

    lib = datagen.load()
    out = []
    for q in range(n):
        def u(i, q=q):
            return (int(lib.gbj_gen_rand(seed, 0x5E00 + q, i)) >> 11) * (1.0 / (1 << 53))

        nb = int(round(2.0 ** (log_build[0] + (log_build[1] - log_build[0]) * u(0))))
        npr = int(round(2.0 ** (log_probe[0] + (log_probe[1] - log_probe[0]) * u(1))))
        mr = 0.3 + 0.7 * u(2)
        card = int(round(2.0 ** (log_card[0] + (log_card[1] - log_card[0]) * u(3))))
        out.append(QueryShape(nb, npr, mr, card, seed * 1000003 + q))
    return out


def gen_query(shape: QueryShape, threads=0):
    """Host columns (build keys, build groups, probe keys, probe values)."""
    import datagen

    return datagen.gen_serve_query(shape.seed, shape.n_build, shape.n_probe, shape.match_rate,
                                   shape.cardinality, threads)


def poisson_arrivals(seed: int, n: int, rate: float) -> np.ndarray:
    """Arrival times (s) of a Poisson process of `rate` queries/s."""
    import datagen

    lib = datagen.load()
    u = np.array([(int(lib.gbj_gen_rand(seed, 0x5F00, i)) >> 11) * (1.0 / (1 << 53)) for i in range(n)])
    return np.cumsum(-np.log1p(-u) / rate)


class Output:
    """Result buffers of one query: device memory, or pinned host memory
    (device="pinned") that the kernels write directly."""

    def __init__(self, capacity: int, device="cuda"):
        import torch

        pin = device == "pinned"
        dev = "cpu" if pin else device

        def mk(n, dt):
            t = torch.zeros(n, dtype=dt, device=dev)
            return t.pin_memory() if pin else t

        self.capacity = capacity
        self.group = mk(capacity, torch.int32)
        self.count = mk(capacity, torch.int64)
        self.sum = mk(capacity, torch.int64)
        self.n = mk(1, torch.int64)

    def sorted(self):
        n = int(self.n.cpu()[0])
        n = min(n, self.capacity)
        g = self.group[:n].cpu().numpy()
        o = np.argsort(g, kind="stable")
        return g[o], self.count[:n].cpu().numpy()[o], self.sum[:n].cpu().numpy()[o]


class Server:
    """gbj_server: admission by HBM budget, continuous batching."""

    def __init__(self, ctx, hbm_budget=0, max_batch=abi.SERVE_MAX_BATCH, max_inflight=2, use_graph=True,
                 large_slots=0, small_rows=0):
        self.ctx = ctx
        prm = abi.ServerParams(hbm_budget, max_batch, max_inflight, 1 if use_graph else 0, large_slots,
                               small_rows)
        h = C.c_void_p()
        ctx.check(ctx.lib.gbj_server_create(ctx.handle, C.byref(prm), C.byref(h)))
        self.handle = h.value
        self._keep = {}

    @classmethod
    def plain(cls, ctx, hbm_budget=0):
        """One query per launch sequence, waited for before the next."""
        return cls(ctx, hbm_budget, max_batch=1, max_inflight=1, use_graph=False)

    @staticmethod
    def _query(bk, bg, pk, pv, expected_groups, out, table=0):
        """bk/bg: build columns, or None with `table` a registered table id."""
        return abi.ServeQuery(bk.data_ptr() if bk is not None else None,
                              bg.data_ptr() if bg is not None else None,
                              bk.numel() if bk is not None else 0, pk.data_ptr(), pv.data_ptr(),
                              pk.numel(), expected_groups, out.group.data_ptr(), out.count.data_ptr(),
                              out.sum.data_ptr(), out.n.data_ptr(), out.capacity, table)

    def register_table(self, bk, bg, expected_groups: int = 0) -> int:
        """Builds (bk, bg)'s join table once, resident in the pool; returns its id."""
        t = C.c_uint64()
        self.ctx.check(self.ctx.lib.gbj_server_register_table(self.handle, bk.data_ptr(), bg.data_ptr(),
                                                              bk.numel(), expected_groups, C.byref(t)))
        return t.value

    def unregister_table(self, table_id: int):
        self.ctx.check(self.ctx.lib.gbj_server_unregister_table(self.handle, table_id))

    def submit(self, bk, bg, pk, pv, expected_groups: int, out: Output, table: int = 0) -> int:
        q = self._query(bk, bg, pk, pv, expected_groups, out, table)
        t = C.c_uint64()
        self.ctx.check(self.ctx.lib.gbj_server_submit(self.handle, C.byref(q), C.byref(t)))
        self._keep[t.value] = (bk, bg, pk, pv, out)
        return t.value

    def submit_many(self, queries) -> list:
        """queries: [(bk, bg, pk, pv, expected_groups, out[, table])], queued together."""
        arr = (abi.ServeQuery * len(queries))(*[self._query(*q) for q in queries])
        tk = (C.c_uint64 * len(queries))()
        self.ctx.check(self.ctx.lib.gbj_server_submit_batch(self.handle, arr, len(queries), tk))
        for t, q in zip(tk, queries):
            self._keep[t] = q
        return list(tk)

    def wait(self, ticket: int, timeout: float = -1.0) -> int:
        st = C.c_int32()
        rc = self.ctx.lib.gbj_server_wait(self.handle, ticket, timeout, C.byref(st))
        if rc:
            raise abi.GbjError(rc, "server wait")
        self._keep.pop(ticket, None)
        return st.value

    def cancel(self, ticket: int) -> bool:
        """Cancels a still-queued query; True if it was cancelled."""
        c = C.c_int32()
        self.ctx.check(self.ctx.lib.gbj_server_cancel(self.handle, ticket, C.byref(c)))
        return bool(c.value)

    def pause(self, paused: bool = True):
        self.ctx.check(self.ctx.lib.gbj_server_pause(self.handle, int(paused)))

    def retries(self) -> int:
        r = C.c_uint64()
        self.ctx.check(self.ctx.lib.gbj_server_retries(self.handle, C.byref(r)))
        return r.value

    def times(self, ticket: int):
        a, b, c = C.c_double(), C.c_double(), C.c_double()
        self.ctx.check(self.ctx.lib.gbj_server_times(self.handle, ticket, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    def drain(self):
        self.ctx.check(self.ctx.lib.gbj_server_drain(self.handle))
        self._keep.clear()

    def busy_ms(self) -> float:
        """Summed device time of the completed batches (gbj_server_busy)."""
        ms = C.c_double()
        self.ctx.check(self.ctx.lib.gbj_server_busy(self.handle, C.byref(ms)))
        return float(ms.value)

    def stats(self):
        c, b, p = C.c_uint64(), C.c_uint64(), C.c_uint64()
        self.ctx.check(self.ctx.lib.gbj_server_stats(self.handle, C.byref(c), C.byref(b), C.byref(p)))
        return {"completed": c.value, "batches": b.value, "peak_bytes": p.value}

    def close(self):
        if self.handle:
            self.ctx.lib.gbj_server_destroy(self.handle)
            self.handle = None
            self._keep.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def latency_summary(lat_s) -> dict:
    a = np.sort(np.asarray(lat_s, dtype=np.float64)) * 1e3
    if len(a) == 0:
        return {}

    def pct(p):
        return float(a[min(len(a) - 1, int(math.ceil(p / 100.0 * len(a))) - 1)])

    return {"p50_ms": round(pct(50), 3), "p99_ms": round(pct(99), 3), "p999_ms": round(pct(99.9), 3),
            "mean_ms": round(float(a.mean()), 3), "n": int(len(a))}
