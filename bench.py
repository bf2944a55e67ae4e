"""Benchmark of the GB300 relational hot path.

Default workload: radix-partitioned hash join,
R = 2^27 unique keys, S = 2^29 keys (50% hits, hit keys Zipf theta in
{0, 0.5, 1.0}), output match count and int64 SUM(R.rowid XOR S.rowid).  One
step = the three joins (one per theta) over resident device columns.

Other workloads (same JSON contract):
  --workload plain    R = 2^20 permuted keys, S = 2^24 uniform keys,
                      COUNT and int64 SUM(R.payload * S.payload)
  --workload groupby  2^29 rows, --card C groups (--theta 0 uniform or Zipf),
                      COUNT / int64 SUM / MIN / MAX per key
  --workload star     64 star-join queries sharing one 2^28-row fact scan
  --workload serve    served stream of join + group-by queries (p50/p99)
  --workload nest     RadixNest over int64 keys: 2^27 rows, --card C keys,
                      COUNT / SUM / MIN / MAX of an int64 value

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Prints ONE JSON line (rank 0).  `value` is tuples per second over the
device-timed steps (inputs resident in HBM); `e2e` repeats the steps with
the inputs copied host->device from pinned memory and the results copied
back inside the timed region.  `--impl reference` times the CPU restatement
of the reference's algorithm (the oracle port, all host threads) on a
bounded sample of the same workload.  N > 1 runs independent replicas (one
per GPU): these joins and aggregations do not shard across GPUs here.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SEED = 20260


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="radix",
                    choices=["radix", "plain", "groupby", "star", "serve", "nest"])
    ap.add_argument("--serve-queries", type=int, default=3000, help="queries per open-loop rate")
    ap.add_argument("--log-r", type=int, default=None, help="log2 build rows (joins)")
    ap.add_argument("--log-s", type=int, default=None, help="log2 probe / input rows")
    ap.add_argument("--card", type=int, default=1 << 16, help="group-by cardinality")
    ap.add_argument("--theta", type=float, default=0.0, help="group-by Zipf exponent")
    ap.add_argument("--bits", type=int, default=0,
                    help="radix join: fixed partition bits instead of the autotuner's choice")
    ap.add_argument("--block", type=int, default=0,
                    help="radix join: fixed join kernel block size (512 or 1024) instead of the autotuner's")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-sample-log", type=int, default=26,
                    help="log2 probe / input rows per join in the CPU baseline sample")
    return ap.parse_args()


def max_over_ranks(ms: float, world: int, device: str = "cuda") -> float:
    """The slowest rank's time: every rank's timed region ends when all have
    finished (all-reduce MAX over the process group; any backend)."""
    if world > 1:
        import torch
        import torch.distributed as dist

        t = torch.tensor([ms], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    return ms


def job_value(units_per_rank_step: float, steps: int, ms: float, world: int, scale: float) -> float:
    """Whole-job throughput: the units all ranks processed / the slowest
    rank's time (replicas: every rank runs the same per-rank work)."""
    return world * units_per_rank_step * steps / (ms / 1e3) / scale


def dist_env():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)),
            int(os.environ.get("WORLD_SIZE", 1)))


# ------------------------------------------------------------- workloads
class RadixJoin:
    metric, unit = "probe Gtuples/s", "Gtuples/s"
    THETAS = (0.0, 0.5, 1.0)

    def __init__(self, args):
        self.lr = args.log_r or 27
        self.ls = args.log_s or 29
        self.nr, self.ns = 1 << self.lr, 1 << self.ls
        self.fixed_bits = args.bits
        self.fixed_block = args.block

    def describe(self):
        return {"workload": f"radix-partitioned hash join R=2^{self.lr} unique int32 keys, "
                            f"S=2^{self.ls} int32 keys (50% hits, Zipf theta 0/0.5/1.0), "
                            f"COUNT + SUM(rowid xor)",
                "n_build": self.nr, "n_probe": self.ns, "thetas": list(self.THETAS),
                "hit_rate": 0.5, "l2": "inputs larger than L2 (2 GiB probe keys per join)"}

    def generate(self):
        import datagen

        self.rk, _ = datagen.gen_build_side(SEED, self.nr, payload=False)
        self.sks = [datagen.gen_probe_zipf(SEED + i, self.ns, self.nr, th, 0.5)[0]
                    for i, th in enumerate(self.THETAS)]

    def device(self, ctx):
        import torch

        from proteus_gb300 import abi

        self.ctx = ctx
        self.aggs = [(abi.AGG_COUNT, abi.VAL_ONE), (abi.AGG_SUM, abi.VAL_ROWID_XOR)]
        self.d_r = torch.from_numpy(self.rk).cuda()
        self.d_s = [torch.from_numpy(s).cuda() for s in self.sks]
        self.outs = [torch.empty(2, dtype=torch.int64, device="cuda") for _ in self.THETAS]
        # the autotuner picks the partition bits for this shape (untimed);
        # every timed join then runs with the cached choice
        if self.fixed_bits or self.fixed_block:
            self.tuned_bits, self.tune_ms = self.fixed_bits, None
            self.block = self.fixed_block
        else:
            self.tuned_bits, self.tune_ms = ctx.autotune_radix_join(self.d_r, None, self.d_s[0], None,
                                                                    self.aggs)
            self.block = ctx.tune_lookup("radixblock", self.nr, self.ns)

    def step(self):
        for ds, o in zip(self.d_s, self.outs):
            self.ctx.radix_join_agg(self.d_r, None, ds, None, self.aggs, out=o, bits=self.fixed_bits,
                                    block=self.fixed_block)

    def results(self):
        return [o.cpu().tolist() for o in self.outs]

    def pin(self):
        import torch

        self.h_r = torch.from_numpy(self.rk).pin_memory()
        self.h_s = [torch.from_numpy(s).pin_memory() for s in self.sks]
        self.h_out = torch.empty((len(self.THETAS), 2), dtype=torch.int64).pin_memory()
        # copies run on their own stream into double-buffered device columns,
        # so the next probe side streams in while the current join computes
        self.copy_stream = torch.cuda.Stream()
        self.s_bufs = [self.d_s[0], self.d_s[1]]
        self.r_bufs = [self.d_r, torch.empty_like(self.d_r)]
        self.s_free = [torch.cuda.Event() for _ in range(2)]
        self.r_free = [torch.cuda.Event() for _ in range(2)]
        for e in self.s_free + self.r_free:
            e.record()
        self.joins, self.steps_done = 0, 0

    def e2e_step(self):
        """Every step copies R and the three S columns host -> device and the
        results back; copy i+1 overlaps join i (buffers guarded by events)."""
        import torch

        comp = torch.cuda.current_stream()
        rb = self.r_bufs[self.steps_done % 2]
        with torch.cuda.stream(self.copy_stream):
            self.copy_stream.wait_event(self.r_free[self.steps_done % 2])
            rb.copy_(self.h_r, non_blocking=True)
            r_ready = torch.cuda.Event()
            r_ready.record(self.copy_stream)
        comp.wait_event(r_ready)
        for i, (hs, o) in enumerate(zip(self.h_s, self.outs)):
            b = self.joins % 2
            with torch.cuda.stream(self.copy_stream):
                self.copy_stream.wait_event(self.s_free[b])
                self.s_bufs[b].copy_(hs, non_blocking=True)
                ready = torch.cuda.Event()
                ready.record(self.copy_stream)
            comp.wait_event(ready)
            self.ctx.radix_join_agg(rb, None, self.s_bufs[b], None, self.aggs, out=o, bits=self.fixed_bits,
                                    block=self.fixed_block)
            self.s_free[b].record(comp)
            self.h_out[i].copy_(o, non_blocking=True)
            self.joins += 1
        self.r_free[self.steps_done % 2].record(comp)
        self.steps_done += 1

    def e2e_results(self):
        return self.h_out.tolist()

    def h2d_bytes(self):
        return 4 * (self.nr + len(self.THETAS) * self.ns)

    def d2h_bytes(self):
        return 16 * len(self.THETAS)

    def units_per_step(self):
        return len(self.THETAS) * self.ns

    def kernel_bytes(self, name):
        """Algorithmic HBM bytes of all launches of `name` in one step."""
        t = len(self.THETAS) * (self.nr + self.ns)
        return {"k_pid_hist": 4 * t,            # key read
                "k_tile_pass": 28 * t,          # pass 1: key read + pair write (12 B),
                                                # pass 2: pair read + pair write (16 B)
                "k_radix_join": 8 * t}.get(name)  # partitioned pairs read once

    def extra(self, ms, steps, peak):
        comp = 4 * (self.nr + self.ns) * len(self.THETAS) * steps
        return {"job_hbm_gbs_compulsory": round(comp / (ms / 1e3) / 1e9, 1),
                "job_frac_compulsory": round(comp / (ms / 1e3) / 1e9 / peak, 4),
                "build_plus_probe_gtuples_s": round(len(self.THETAS) * (self.nr + self.ns) * steps
                                                    / (ms / 1e3) / 1e9, 3),
                "radix_bits": self.tuned_bits, "join_block": self.block,
                "radix_bits_from": "fixed" if (self.fixed_bits or self.fixed_block) else "autotuner"}

    def cpu(self, threads, sample_log):
        from oracle import oracle as O

        ns = 1 << min(sample_log, self.ls)
        aggs = [(0, 0), (1, 6)]
        t0 = time.perf_counter()
        for sk in self.sks:
            O.radix_join_agg(self.rk, None, sk[:ns], None, aggs, threads=threads)
        dt = time.perf_counter() - t0
        return len(self.THETAS) * ns, dt, (f"full R (2^{self.lr}), first {ns} rows of each S "
                                           f"(theta 0/0.5/1.0); oracle C port of the reference's "
                                           f"partitioned chained-hash join, {threads} threads")


class PlainJoin:
    metric, unit = "probe Gtuples/s", "Gtuples/s"

    def __init__(self, args):
        self.lr = args.log_r or 20
        self.ls = args.log_s or 24
        self.nr, self.ns = 1 << self.lr, 1 << self.ls

    def describe(self):
        return {"workload": f"plain hash join R=2^{self.lr} (permuted keys, payload U[0,1000)), "
                            f"S=2^{self.ls} (keys U{{1..2^{self.lr}}}), COUNT + SUM(R.p*S.p)",
                "n_build": self.nr, "n_probe": self.ns,
                "l2": "probe columns (128 MiB) larger than L2"}

    def generate(self):
        import datagen

        self.rk, self.rp = datagen.gen_build_side(SEED, self.nr)
        self.sk, self.sp = datagen.gen_probe_uniform(SEED, self.ns, self.nr)

    def device(self, ctx):
        import torch

        from proteus_gb300 import abi

        self.ctx = ctx
        self.aggs = [(abi.AGG_COUNT, abi.VAL_ONE), (abi.AGG_SUM, abi.VAL_PRODUCT)]
        self.d = [torch.from_numpy(a).cuda() for a in (self.rk, self.rp, self.sk, self.sp)]
        self.out = torch.empty(2, dtype=torch.int64, device="cuda")

    def step(self):
        t = self.ctx.join_build(self.d[0], self.d[1])
        self.ctx.join_probe_agg(t, self.d[2], self.d[3], self.aggs, out=self.out)
        t.destroy()

    def results(self):
        return self.out.cpu().tolist()

    def pin(self):
        import torch

        self.h = [torch.from_numpy(a).pin_memory() for a in (self.rk, self.rp, self.sk, self.sp)]
        self.h_out = torch.empty(2, dtype=torch.int64).pin_memory()

    def e2e_step(self):
        for h, d in zip(self.h, self.d):
            d.copy_(h, non_blocking=True)
        self.step()
        self.h_out.copy_(self.out, non_blocking=True)

    def e2e_results(self):
        return self.h_out.tolist()

    def h2d_bytes(self):
        return 8 * (self.nr + self.ns)

    def d2h_bytes(self):
        return 16

    def units_per_step(self):
        return self.ns

    def kernel_bytes(self, name):
        return {"k_jb_probe_agg": 8 * self.ns,   # probe key + payload
                "k_jb_build": 12 * self.nr}.get(name)  # key + payload read, bucket slot write

    def extra(self, ms, steps, peak):
        comp = 8 * (self.nr + self.ns) * steps
        return {"job_hbm_gbs_compulsory": round(comp / (ms / 1e3) / 1e9, 1),
                "job_frac_compulsory": round(comp / (ms / 1e3) / 1e9 / peak, 4)}

    def cpu(self, threads, sample_log):
        from oracle import oracle as O

        t0 = time.perf_counter()
        O.join_agg(self.rk, self.rp, self.sk, self.sp, [(0, 0), (1, 3)], threads=threads)
        dt = time.perf_counter() - t0
        return self.ns, dt, (f"full workload; oracle C port of HashJoinChained "
                             f"(multi-worker build, {threads} threads)")


class GroupBy:
    metric, unit = "group-by Gtuples/s", "Gtuples/s"

    def __init__(self, args):
        self.ls = args.log_s or 29
        self.n = 1 << self.ls
        self.card, self.theta = args.card, args.theta

    def describe(self):
        return {"workload": f"hash group-by 2^{self.ls} rows, {self.card} groups "
                            f"({'Zipf %.1f' % self.theta if self.theta else 'uniform'}), "
                            f"int32 value U[-2^20,2^20): COUNT, SUM int64, MIN, MAX",
                "rows": self.n, "cardinality": self.card, "theta": self.theta,
                "l2": "inputs (4 GiB) larger than L2"}

    def generate(self):
        import datagen

        self.k, self.v = datagen.gen_groupby(SEED, self.n, self.card, self.theta)

    def device(self, ctx):
        import torch

        self.ctx = ctx
        self.dk, self.dv = torch.from_numpy(self.k).cuda(), torch.from_numpy(self.v).cuda()
        self.cap = self.card + 16
        self.res = None

    def step(self):
        self.res = self.ctx.groupby(self.dk, self.dv, self.cap, expected_groups=self.card)

    def results(self):
        return int(self.res[5].cpu()[0])

    def pin(self):
        import torch

        self.hk = torch.from_numpy(self.k).pin_memory()
        self.hv = torch.from_numpy(self.v).pin_memory()
        self.h_out = [torch.empty(self.cap, dtype=t).pin_memory() for t in
                      (torch.int32, torch.int64, torch.int64, torch.int32, torch.int32)]
        self.h_n = torch.empty(1, dtype=torch.int64).pin_memory()

    def e2e_step(self):
        self.dk.copy_(self.hk, non_blocking=True)
        self.dv.copy_(self.hv, non_blocking=True)
        self.step()
        for h, d in zip(self.h_out, self.res[:5]):
            h.copy_(d, non_blocking=True)
        self.h_n.copy_(self.res[5], non_blocking=True)

    def e2e_results(self):
        return int(self.h_n[0])

    def h2d_bytes(self):
        return 8 * self.n

    def d2h_bytes(self):
        return 28 * self.cap + 8

    def units_per_step(self):
        return self.n

    def kernel_bytes(self, name):
        return {"k_groupby": 8 * self.n,       # (key, value) per row, raw or partitioned
                "k_pid_hist": 4 * self.n,      # key read
                "k_tile_pass": 16 * self.n}.get(name)  # per pass: pair read + pair write

    def extra(self, ms, steps, peak):
        comp = 8 * self.n * steps
        return {"job_hbm_gbs_compulsory": round(comp / (ms / 1e3) / 1e9, 1),
                "job_frac_compulsory": round(comp / (ms / 1e3) / 1e9 / peak, 4)}

    def cpu(self, threads, sample_log):
        from oracle import oracle as O

        n = 1 << min(sample_log + 1, self.ls)
        t0 = time.perf_counter()
        O.groupby(self.k[:n], self.v[:n], threads=threads)
        dt = time.perf_counter() - t0
        return n, dt, (f"first {n} rows; oracle C port of HashGroupByChained "
                       f"(hash-partitioned per thread), {threads} threads")


class Nest:
    """RadixNest over int64 keys (the aggregation twin): per distinct key
    COUNT, SUM, MIN, MAX of an int64 value."""
    metric, unit, dtype = "nest Gtuples/s", "Gtuples/s", "int64"

    def __init__(self, args):
        self.ls = args.log_s or 27
        self.n = 1 << self.ls
        self.card = args.card

    def describe(self):
        return {"workload": f"RadixNest int64 group-by 2^{self.ls} rows, {self.card} distinct int64 keys "
                            f"(uniform), int64 value: COUNT, SUM int64, MIN, MAX",
                "rows": self.n, "cardinality": self.card, "l2": "inputs (2 GiB) larger than L2"}

    def generate(self):
        import numpy as np

        rng = np.random.default_rng(SEED)
        base = rng.integers(np.iinfo(np.int64).min, np.iinfo(np.int64).max, self.card, dtype=np.int64)
        self.k = base[rng.integers(0, self.card, self.n)]
        self.v = rng.integers(-(1 << 40), 1 << 40, self.n, dtype=np.int64)

    def device(self, ctx):
        import torch

        self.ctx = ctx
        self.dk, self.dv = torch.from_numpy(self.k).cuda(), torch.from_numpy(self.v).cuda()
        self.cap = self.card + 16
        self.res = None

    def step(self):
        self.res = self.ctx.nest_i64(self.dk, self.dv, self.cap, expected_groups=self.card)

    def results(self):
        return int(self.res[5].cpu()[0])

    def pin(self):
        import torch

        self.hk = torch.from_numpy(self.k).pin_memory()
        self.hv = torch.from_numpy(self.v).pin_memory()
        self.h_out = [torch.empty(self.cap, dtype=torch.int64).pin_memory() for _ in range(5)]
        self.h_n = torch.empty(1, dtype=torch.int64).pin_memory()

    def e2e_step(self):
        self.dk.copy_(self.hk, non_blocking=True)
        self.dv.copy_(self.hv, non_blocking=True)
        self.step()
        for h, d in zip(self.h_out, self.res[:5]):
            h.copy_(d, non_blocking=True)
        self.h_n.copy_(self.res[5], non_blocking=True)

    def e2e_results(self):
        return int(self.h_n[0])

    def h2d_bytes(self):
        return 16 * self.n

    def d2h_bytes(self):
        return 40 * self.cap + 8

    def units_per_step(self):
        return self.n

    def kernel_bytes(self, name):
        # (int64 key, int64 value) per row: on-chip level for few groups, else the global table
        return {"k_nest_l1": 16 * self.n, "k_nest_build": 16 * self.n}.get(name)

    def extra(self, ms, steps, peak):
        comp = 16 * self.n * steps
        return {"job_hbm_gbs_compulsory": round(comp / (ms / 1e3) / 1e9, 1),
                "job_frac_compulsory": round(comp / (ms / 1e3) / 1e9 / peak, 4)}

    def cpu(self, threads, sample_log):
        from oracle import oracle as O

        n = 1 << min(sample_log - 2, self.ls)
        t0 = time.perf_counter()
        O.nest_i64(self.k[:n], self.v[:n])
        dt = time.perf_counter() - t0
        return n, dt, (f"first {n} rows; oracle C port of RadixNest over the int64 twin's partitionHT "
                       f"and bucket chains, 1 thread")


class StarBatch:
    """64 star-join query variants over a 2^28-row fact table, all in one
    graph replay sharing the fact scan (one step = one batch)."""
    metric, unit, scale = "star-join queries/s", "queries/s", 1.0

    def __init__(self, args):
        self.lf = args.log_s or 28
        self.nq = 64

    def describe(self):
        return {"workload": f"batched star join: fact 2^{self.lf} rows (4 int32 FKs into dims of "
                            f"2^21, 2557, 2^18, 2^16 rows, quantity, price), {self.nq} seeded "
                            f"query variants (3 joins, 1/5-1/50 predicates per dimension, group-by "
                            f"2 dimension attributes, SUM int64 price*quantity) in one launch "
                            f"sequence replayed from a CUDA graph",
                "fact_rows": 1 << self.lf, "queries_per_batch": self.nq,
                "l2": "fact columns (6 GiB) larger than L2"}

    def generate(self):
        from proteus_gb300 import star

        self.data = star.gen_star(SEED, n_fact=1 << self.lf)
        self.queries = star.gen_queries(SEED, self.nq, self.data.dims)

    def device(self, ctx):
        from proteus_gb300 import star

        self.ctx = ctx
        self.plan = star.StarPlan(ctx, self.data)
        self.out = self.plan.new_output(self.nq)

    def step(self):
        self.plan.run(self.queries, self.out, use_graph=True)

    def _digest(self, cnt, sm, n):
        return int(n.sum()) * 1000003 + int(cnt.sum()) * 7 + int(sm.sum() % 1000000007)

    def results(self):
        return self._digest(self.out["count"].cpu().numpy() * (self._valid_mask()),
                            self.out["sum"].cpu().numpy() * (self._valid_mask()),
                            self.out["n"].cpu().numpy())

    def _valid_mask(self):
        import numpy as np

        n = self.out["n"].cpu().numpy()
        cap = self.out["cap"]
        m = np.zeros(self.nq * cap, dtype=np.int64)
        for q in range(self.nq):
            m[q * cap:q * cap + int(n[q])] = 1
        return m

    def pin(self):
        import torch

        self.h_fk = [torch.from_numpy(c).pin_memory() for c in self.data.fk]
        self.h_qty = torch.from_numpy(self.data.quantity).pin_memory()
        self.h_price = torch.from_numpy(self.data.price).pin_memory()
        self.h_out = {k: torch.empty_like(self.out[k], device="cpu").pin_memory()
                      for k in ("a", "b", "count", "sum", "n")}

    def e2e_step(self):
        for d, h in zip(self.plan.dev_fk, self.h_fk):
            d.copy_(h, non_blocking=True)
        self.plan.dev_qty.copy_(self.h_qty, non_blocking=True)
        self.plan.dev_price.copy_(self.h_price, non_blocking=True)
        self.step()
        for k, h in self.h_out.items():
            h.copy_(self.out[k], non_blocking=True)

    def e2e_results(self):
        import numpy as np

        n = self.h_out["n"].numpy()
        cap = self.out["cap"]
        m = np.zeros(self.nq * cap, dtype=np.int64)
        for q in range(self.nq):
            m[q * cap:q * cap + int(n[q])] = 1
        return self._digest(self.h_out["count"].numpy() * m, self.h_out["sum"].numpy() * m, n)

    def h2d_bytes(self):
        return 24 * (1 << self.lf)

    def d2h_bytes(self):
        return sum(t.numel() * t.element_size() for t in self.h_out.values())

    def units_per_step(self):
        return self.nq

    def kernel_bytes(self, name):
        fact = 24 * (1 << self.lf)  # 4 FKs + quantity + price, read once per batch
        return {"star_graph": fact, "k_star_fact": fact}.get(name)

    def extra(self, ms, steps, peak):
        import torch

        # the plain form: one query per launch sequence (each scans the fact)
        outs = self.plan.new_output(1)
        for q in self.queries[:2]:
            self.plan.run([q], outs, use_graph=False)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for q in self.queries:
            self.plan.run([q], outs, use_graph=False)
        e1.record()
        torch.cuda.synchronize()
        plain_ms = e0.elapsed_time(e1)
        batched_qps = self.nq * steps / (ms / 1e3)
        plain_qps = self.nq / (plain_ms / 1e3)
        comp = 24 * (1 << self.lf) * steps
        return {"fact_gtuples_per_s": round((1 << self.lf) * steps / (ms / 1e3) / 1e9, 2),
                "job_hbm_gbs_compulsory": round(comp / (ms / 1e3) / 1e9, 1),
                "job_frac_compulsory": round(comp / (ms / 1e3) / 1e9 / peak, 4),
                "plain_one_query_per_launch_qps": round(plain_qps, 1),
                "batched_over_plain": round(batched_qps / plain_qps, 2)}

    def cpu(self, threads, sample_log):
        from oracle import oracle as O

        rows = 1 << min(sample_log + 2, self.lf)
        nq = 8
        t0 = time.perf_counter()
        for q in self.queries[:nq]:
            O.star_query(self.data, q, threads=threads, rows=rows)
        dt = time.perf_counter() - t0
        equiv = nq * rows / (1 << self.lf)  # full-size queries the sample amounts to
        return equiv, dt, (f"{nq} queries over the first {rows} fact rows (counted as {equiv:.4f} "
                           f"full-size queries); oracle C port of select -> HashJoinChained x3 -> "
                           f"HashGroupByChained, one query at a time, {threads} threads")


class Serve:
    """Served query stream: Poisson arrivals of join + group-by queries over
    64 resident query templates.  Both the plain form (one query per launch
    sequence, waited for before the next) and the batched server are swept
    over arrival rates (fractions of their own closed-loop capacity); for
    each p99 SLO the highest throughput that kept p99 within it is reported,
    and `value` is the batched server's at p99 <= 10 ms."""
    metric, unit, scale = "served queries/s at p99 <= 10 ms", "queries/s", 1.0
    custom = True

    def __init__(self, args):
        self.nt = 64
        self.ring = 256
        self.n_open = args.serve_queries

    def describe(self):
        return {"workload": "served stream of join + group-by queries (build log-uniform 2^10-2^24, "
                            "probe log-uniform 2^14-2^27, match rate U[0.3,1], groups log-uniform "
                            "2^4-2^16, COUNT + SUM int64), Poisson arrivals, tables resident in "
                            "the pool, results written to pinned host memory",
                "templates": self.nt, "queries_per_rate": self.n_open,
                "l2": "resident inputs (~9 GB) larger than L2"}

    def generate(self):
        from proteus_gb300 import serve

        self.shapes = serve.gen_shapes(SEED, self.nt)
        self.host = [serve.gen_query(sh) for sh in self.shapes]

    def device(self, ctx):
        import torch
        from proteus_gb300 import serve

        self.ctx = ctx
        self.dev = [tuple(torch.from_numpy(a).cuda() for a in h) for h in self.host]
        self.outs = [serve.Output(min(sh.cardinality, sh.n_build) + 8, device="pinned")
                     for sh in self.shapes]
        cap = max(o.capacity for o in self.outs)
        self.ring_outs = [serve.Output(cap, device="pinned") for _ in range(self.ring)]
        torch.cuda.synchronize()

    def _order(self, n, salt):
        import datagen

        return [int(datagen.load().gbj_gen_rand(SEED, 0x6000 + salt, i)) % self.nt for i in range(n)]

    def _submit(self, srv, t, out, tables):
        """Template t's query; with `tables`, against its resident build table."""
        if tables:
            _, _, pk, pv = self.dev[t]
            return srv.submit(None, None, pk, pv, self.shapes[t].cardinality, out, table=tables[t])
        return srv.submit(*self.dev[t], self.shapes[t].cardinality, out)

    def _closed(self, srv, n, salt, tables=None, busy=None):
        """Closed loop of n queries -> (queries/s, errors); `busy` (a dict)
        gets the fraction of the wall time the batches kept the GPU busy."""
        order = self._order(n, salt)
        b0 = srv.busy_ms()
        t0 = time.perf_counter()
        tickets = [self._submit(srv, t, self.ring_outs[i % self.ring], tables) for i, t in enumerate(order)]
        srv.drain()
        dt = time.perf_counter() - t0
        if busy is not None:
            busy["batch_gpu_s"] = round((srv.busy_ms() - b0) / 1e3, 4)
            busy["wall_s"] = round(dt, 4)
            busy["gpu_busy_frac"] = round((srv.busy_ms() - b0) / 1e3 / dt, 3)
        bad = sum(srv.wait(tk) != 0 for tk in tickets)
        return n / dt, bad

    # size classes of the templates by probe rows (p99 is reported per class)
    CLASSES = (("small", 1 << 20), ("medium", 1 << 24), ("large", 1 << 62))

    def _class_of(self, t):
        return next(name for name, lim in self.CLASSES if self.shapes[t].n_probe < lim)

    def _open(self, srv, rate, n, salt, tables=None):
        from proteus_gb300 import serve

        order = self._order(n, salt)
        arr = serve.poisson_arrivals(SEED + salt, n, rate)
        tickets = []
        t0 = time.perf_counter()
        for i, t in enumerate(order):
            while time.perf_counter() - t0 < arr[i]:
                pass
            tickets.append(self._submit(srv, t, self.ring_outs[i % self.ring], tables))
        srv.drain()
        lat, first, last = [], None, None
        for tk in tickets:
            a, _, c = srv.times(tk)
            lat.append(c - a)
            first = a if first is None else min(first, a)
            last = c if last is None else max(last, c)
        bad = sum(srv.wait(tk) != 0 for tk in tickets)
        # results of the last `ring` queries are intact: compare with the
        # same templates run alone
        mism = 0
        for i in range(max(0, n - self.ring), n):
            got = self.ring_outs[i % self.ring].sorted()
            exp = self.alone[order[i]]
            mism += int(len(got[0]) != len(exp[0]) or any((a != b).any() for a, b in zip(got, exp)))
        summ = serve.latency_summary(lat)
        summ.update({"rate": round(rate, 1), "throughput": round(n / (last - first), 1),
                     "errors": bad, "mismatch_vs_alone": mism})
        by = {}
        for name, _ in self.CLASSES:
            sel = [x for x, t in zip(lat, order) if self._class_of(t) == name]
            if sel:
                c = serve.latency_summary(sel)
                by[name] = {"p50_ms": c["p50_ms"], "p99_ms": c["p99_ms"], "n": c["n"]}
        summ["by_class"] = by
        return summ

    SLOS_MS = (5.0, 10.0, 20.0, 50.0)
    HEADLINE_SLO_MS = 10.0

    def _sweep(self, srv, cap, salt, tables=None):
        runs = []
        for k, frac in enumerate((0.3, 0.5, 0.7, 0.85, 0.95)):
            runs.append(self._open(srv, frac * cap, self.n_open, salt + k, tables))
        return runs

    @staticmethod
    def _best(runs, slo):
        ok = [r["throughput"] for r in runs if r["p99_ms"] <= slo and r["errors"] == 0]
        return max(ok) if ok else 0.0

    def run(self, args):
        from proteus_gb300 import serve

        ctx = self.ctx
        # each template alone (plain form): the expected result of every query
        plain = serve.Server.plain(ctx)
        self.alone = []
        for t in range(self.nt):
            o = self.outs[t]
            tk = plain.submit(*self.dev[t], self.shapes[t].cardinality, o)
            assert plain.wait(tk) == 0
            self.alone.append(o.sorted())
        self._closed(plain, 256, 1)
        plain_busy = {}
        plain_cap, bad_p = self._closed(plain, 768, 2, busy=plain_busy)
        p_runs = self._sweep(plain, plain_cap, 10)
        plain.close()

        def batched_server():
            return serve.Server(ctx, max_batch=64, max_inflight=4, use_graph=True, large_slots=2,
                                small_rows=1 << 22)

        batched = batched_server()
        self._closed(batched, 256, 4)
        bat_busy = {}
        bat_cap, bad_b = self._closed(batched, 1536, 5, busy=bat_busy)
        b_runs = self._sweep(batched, bat_cap, 20)
        st = batched.stats()
        batched.close()
        # batched, every template's build relation registered once as a
        # resident table: queries only probe and group
        resident = batched_server()
        tables = [resident.register_table(bk, bg, self.shapes[t].cardinality)
                  for t, (bk, bg, _, _) in enumerate(self.dev)]
        table_bytes = resident.stats()["peak_bytes"]
        self._closed(resident, 256, 6, tables)
        res_cap, bad_r = self._closed(resident, 1536, 7, tables)
        r_runs = self._sweep(resident, res_cap, 30, tables)
        st_r = resident.stats()
        resident.close()
        slo = {f"p99<={s:g}ms": {"plain_qps": self._best(p_runs, s), "batched_qps": self._best(b_runs, s),
                                 "batched_resident_qps": self._best(r_runs, s)}
               for s in self.SLOS_MS}
        for v in slo.values():
            v["ratio"] = round(v["batched_qps"] / v["plain_qps"], 2) if v["plain_qps"] else None
            v["resident_ratio"] = round(v["batched_resident_qps"] / v["plain_qps"], 2) if v["plain_qps"] else None
        head = slo[f"p99<={self.HEADLINE_SLO_MS:g}ms"]
        return head["batched_qps"], {
            "slo_ms": self.HEADLINE_SLO_MS,
            "plain": {"capacity_qps": round(plain_cap, 1), "closed_loop": plain_busy, "sweep": p_runs},
            "batched": {"capacity_qps": round(bat_cap, 1), "closed_loop": bat_busy, "sweep": b_runs,
                        "batches": st["batches"], "peak_pool_bytes": st["peak_bytes"]},
            "batched_resident_tables": {"capacity_qps": round(res_cap, 1), "sweep": r_runs,
                                        "batches": st_r["batches"], "table_bytes": table_bytes,
                                        "peak_pool_bytes": st_r["peak_bytes"]},
            "throughput_at_p99_slo": slo,
            "batched_over_plain_at_equal_p99": head["ratio"],
            "batched_resident_over_plain_at_equal_p99": head["resident_ratio"],
            "batched_over_plain_capacity": round(bat_cap / plain_cap, 2),
            "class_probe_rows": {name: lim for name, lim in self.CLASSES[:-1]},
            "batched_resident_over_plain_capacity": round(res_cap / plain_cap, 2),
            "closed_loop_errors": bad_p + bad_b + bad_r,
            "mismatch_vs_alone": sum(r["mismatch_vs_alone"] for r in p_runs + b_runs + r_runs),
        }

    def cpu(self, threads, sample_log):
        from oracle import oracle as O

        t0 = time.perf_counter()
        k = 0
        for t in self._order(16, 99):
            O.join_groupby(*self.host[t], threads=threads)
            k += 1
            if time.perf_counter() - t0 > 20:
                break
        dt = time.perf_counter() - t0
        return k, dt, (f"{k} queries of the template mix, one at a time; oracle C port of "
                       f"HashJoinChained -> HashGroupByChained, {threads} threads")


WORKLOADS = {"radix": RadixJoin, "plain": PlainJoin, "groupby": GroupBy, "star": StarBatch,
             "serve": Serve, "nest": Nest}


# ------------------------------------------------------------- helpers
class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index, self.samples, self.proc = index, [], None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 8:
                self.samples.append(parts)

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        sm, smax, reasons = [], None, set()
        for p in self.samples:
            try:
                sm.append(float(p[0]))
                smax = float(p[1])
            except ValueError:
                continue
            for nm, v in zip(names, p[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def hbm_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def traffic_from_profiles(workload, kernel):
    """Per-launch DRAM bytes of `kernel` from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", f"{workload}_traffic.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return d.get(kernel, {}).get("dram_bytes_per_launch")
    except (OSError, ValueError):
        return None


# ------------------------------------------------------------- arms
def run_reference(args):
    rank, _, world = dist_env()
    if rank != 0:
        return
    from oracle import oracle as O

    O.build()
    wl = WORKLOADS[args.workload](args)
    wl.generate()
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        wl.cpu(threads, args.cpu_sample_log)
    units, secs, sample = 0, 0.0, ""
    for _ in range(args.steps):
        u, dt, sample = wl.cpu(threads, args.cpu_sample_log)
        units += u
        secs += dt
    value = units / secs / getattr(wl, "scale", 1e9)
    cfg = wl.describe()  # the GPU arm's config, key for key
    cfg["parallelism"] = f"replicas x{world}"
    line = {
        "impl": "reference", "metric": wl.metric, "value": value, "unit": wl.unit,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * secs / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": getattr(wl, "dtype", "int32"), "data": "synthetic (seeded generator)",
        "config": cfg,
        "sample": sample,
        "cpu_baseline": {"value": value, "unit": wl.unit, "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": wl.unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_gpu(args):
    import torch

    rank, local_rank, world = dist_env()
    torch.cuda.set_device(local_rank)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    from proteus_gb300 import engine

    wl = WORKLOADS[args.workload](args)
    wl.generate()
    stream = torch.cuda.current_stream()
    ctx = engine.Context(local_rank, pool_bytes=24 << 30)
    wl.device(ctx)
    if getattr(wl, "custom", False):
        return run_custom(args, wl, ctx, rank, world)

    for _ in range(args.warmup):
        wl.step()
    ctx.sync()
    results = wl.results()

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    # ---- device-timed steps (inputs resident) ----
    clocks = ClockSampler(local_rank)
    barrier()
    clocks.start()
    ctx.profile(True)
    launches0 = ctx.launches()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        wl.step()
    e1.record(stream)
    barrier()
    ms = max_over_ranks(e0.elapsed_time(e1), world)
    launches = ctx.launches() - launches0
    prof = ctx.profile_dump()
    ctx.profile(False)
    clk = clocks.stop()
    ctx.sync()
    scale = getattr(wl, "scale", 1e9)
    value = job_value(wl.units_per_step(), args.steps, ms, world, scale)

    # ---- roofline of the dominant kernel ----
    peak, peak_kind = hbm_peak()
    dom_name, (dom_launches, dom_ms) = max(prof.items(), key=lambda kv: kv[1][1])
    per_step = wl.kernel_bytes(dom_name)
    roof = None
    if per_step is not None:
        achieved = per_step * args.steps / (dom_ms / 1e3) / 1e9
        roof = {"bound": "hbm", "kernel": dom_name, "achieved": round(achieved, 1),
                "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                "peak_source": peak_kind, "traffic": traffic_from_profiles(args.workload, dom_name),
                "algorithmic_bytes_per_launch": per_step * args.steps / dom_launches,
                "avg_launch_ms": dom_ms / dom_launches}
    total = sum(x[1] for x in prof.values())
    kernels = {k: {"launches": v[0], "ms_total": round(v[1], 3), "share": round(v[1] / total, 4)}
               for k, v in sorted(prof.items(), key=lambda kv: -kv[1][1])}

    # ---- end to end through the API with host buffers ----
    e2e = None
    if not args.no_e2e:
        wl.pin()
        for _ in range(max(1, args.warmup)):
            wl.e2e_step()
        barrier()
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        for _ in range(args.steps):
            wl.e2e_step()
        f1.record(stream)
        barrier()
        ems = max_over_ranks(f0.elapsed_time(f1), world)
        assert wl.e2e_results() == results, "e2e results differ from resident results"
        e2e = {"value": job_value(wl.units_per_step(), args.steps, ems, world, scale),
               "unit": wl.unit, "h2d_bytes_per_step": wl.h2d_bytes(),
               "d2h_bytes_per_step": wl.d2h_bytes(), "ms_per_step": ems / args.steps}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        u, dt, sample = wl.cpu(threads, args.cpu_sample_log)
        cpu = {"value": u / dt / scale, "unit": wl.unit, "cores": threads, "kind": "port",
               "sample": f"{sample}; {dt:.1f} s"}

    if rank == 0:
        cfg = wl.describe()
        cfg["parallelism"] = f"replicas x{world}"
        line = {
            "metric": wl.metric, "value": round(value, 3), "unit": wl.unit, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": getattr(wl, "dtype", "int32"),
            "data": "synthetic (seeded generator)", "config": cfg,
            "e2e": e2e, "roofline": roof, "cpu_baseline": cpu, "clocks": clk,
            "gpu_launches": launches, **wl.extra(ms, args.steps, peak),
            "kernels": kernels, "results": results,
        }
        print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def run_custom(args, wl, ctx, rank, world):
    """Workloads with their own measurement loop (serving): one JSON line
    with the same keys; `value` comes from the workload's run()."""
    import torch

    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    launches0 = ctx.launches()
    t0 = time.perf_counter()
    value, detail = wl.run(args)
    wall = time.perf_counter() - t0
    launches = ctx.launches() - launches0
    clk = clocks.stop()
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        u, dt, sample = wl.cpu(threads, args.cpu_sample_log)
        cpu = {"value": u / dt / wl.scale, "unit": wl.unit, "cores": threads, "kind": "port",
               "sample": f"{sample}; {dt:.1f} s"}
    if rank == 0:
        cfg = wl.describe()
        cfg["parallelism"] = f"replicas x{world}"
        line = {
            "metric": wl.metric, "value": round(world * value, 1), "unit": wl.unit, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": None,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": getattr(wl, "dtype", "int32"),
            "data": "synthetic (seeded generator)", "config": cfg,
            "e2e": {"value": round(world * value, 1), "unit": wl.unit, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": None,
                    "note": "served tables are resident by design; every query's results are "
                            "written to pinned host memory inside its measured latency"},
            "roofline": None, "cpu_baseline": cpu, "clocks": clk, "gpu_launches": launches,
            "wall_s": round(wall, 1), **detail,
        }
        print(json.dumps(line), flush=True)
    ctx.close()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
