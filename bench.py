"""Benchmark: radix-partitioned hash join, R = 2^27 unique keys, S = 2^29
keys (50% hits, hit keys Zipf theta in {0, 0.5, 1.0}), output match count and
int64 SUM(R.rowid XOR S.rowid).  One step = the three joins (one per theta)
over resident device columns.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Prints ONE JSON line (rank 0).  `value` is probe tuples per second over the
device-timed steps (inputs resident in HBM); `e2e` repeats the steps with the
probe and build key columns copied host->device from pinned memory and the
results copied back inside the timed region.  `--impl reference` times the
CPU restatement of the reference's join (the oracle port, all host threads)
on a bounded sample of the same workload.  N > 1 runs independent replicas
(one per GPU): the join does not shard across GPUs here.
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

LOG_R, LOG_S = 27, 29
THETAS = (0.0, 0.5, 1.0)
HIT_RATE = 0.5
SEED = 20260
METRIC = "probe Gtuples/s"
UNIT = "Gtuples/s"
WORKLOAD = "radix-partitioned hash join R=2^27 unique int32 keys, S=2^29 int32 keys " \
           "(50% hits, Zipf theta 0/0.5/1.0), COUNT + SUM(rowid xor)"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--log-r", type=int, default=LOG_R)
    ap.add_argument("--log-s", type=int, default=LOG_S)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-sample-log", type=int, default=26,
                    help="log2 probe rows per theta in the CPU baseline sample")
    return ap.parse_args()


def dist_env():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)),
            int(os.environ.get("WORLD_SIZE", 1)))


def gen_inputs(log_r, log_s):
    from proteus_gb300 import engine

    rk, _ = engine.gen_build_side(SEED, 1 << log_r, payload=False)
    sks = [engine.gen_probe_zipf(SEED + i, 1 << log_s, 1 << log_r, th, HIT_RATE)[0]
           for i, th in enumerate(THETAS)]
    return rk, sks


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


def kernel_bytes(name, n_r, n_s):
    """Algorithmic HBM bytes of one join's launches of `name` (all launches
    of that kernel in one join together), per the kernel's definition."""
    tuples = n_r + n_s
    return {"k_pid_hist": 4 * tuples,          # key read
            "k_tile_pass": 28 * tuples,        # pass 1: key read + pair write (12 B),
                                               # pass 2: pair read + pair write (16 B)
            "k_radix_join": 8 * tuples}.get(name)  # partitioned pairs read once


def traffic_from_profiles(kernel):
    """Per-launch DRAM bytes of `kernel` from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "radix_join_traffic.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return d.get(kernel, {}).get("dram_bytes_per_launch")
    except (OSError, ValueError):
        return None


def cpu_baseline(rk, sks, sample_log, threads):
    from oracle import oracle as O
    from proteus_gb300 import abi

    aggs = [(abi.AGG_COUNT, abi.VAL_ONE), (abi.AGG_SUM, abi.VAL_ROWID_XOR)]
    ns = 1 << sample_log
    t0 = time.perf_counter()
    tuples = 0
    for sk in sks:
        O.radix_join_agg(rk, None, sk[:ns], None, aggs, threads=threads)
        tuples += ns
    dt = time.perf_counter() - t0
    return tuples / dt / 1e9, dt


def run_reference(args):
    rank, _, world = dist_env()
    if rank != 0:
        return
    from oracle import oracle as O

    O.build()
    threads = os.cpu_count() or 1
    rk, sks = gen_inputs(args.log_r, args.log_s)
    sample = min(args.cpu_sample_log, args.log_s)
    for _ in range(args.warmup):
        cpu_baseline(rk, sks, sample, threads)
    times, vals = [], []
    for _ in range(args.steps):
        v, dt = cpu_baseline(rk, sks, sample, threads)
        vals.append(v)
        times.append(dt)
    value = (len(THETAS) << sample) * args.steps / sum(times) / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic (seeded generator)",
        "config": {"workload": WORKLOAD, "n_build": 1 << args.log_r, "n_probe": 1 << args.log_s,
                   "sample_probe_rows_per_theta": 1 << sample},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"full R (2^{args.log_r}), first 2^{sample} rows of each S "
                                   f"(theta 0/0.5/1.0); oracle C port of the reference's "
                                   f"partitioned chained-hash join, {threads} threads"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_gpu(args):
    import torch

    rank, local_rank, world = dist_env()
    torch.cuda.set_device(local_rank)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    from proteus_gb300 import abi, engine

    n_r, n_s = 1 << args.log_r, 1 << args.log_s
    rk, sks = gen_inputs(args.log_r, args.log_s)
    stream = torch.cuda.current_stream()
    d_r = torch.from_numpy(rk).cuda()
    d_s = [torch.from_numpy(s).cuda() for s in sks]
    ctx = engine.Context(local_rank, pool_bytes=24 << 30)
    aggs = [(abi.AGG_COUNT, abi.VAL_ONE), (abi.AGG_SUM, abi.VAL_ROWID_XOR)]
    outs = [torch.empty(2, dtype=torch.int64, device="cuda") for _ in THETAS]

    def step():
        for ds, o in zip(d_s, outs):
            ctx.radix_join_agg(d_r, None, ds, None, aggs, out=o)

    for _ in range(args.warmup):
        step()
    ctx.sync()
    results = [o.cpu().tolist() for o in outs]

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
        step()
    e1.record(stream)
    barrier()
    ms = e0.elapsed_time(e1)
    launches = ctx.launches() - launches0
    prof = ctx.profile_dump()
    ctx.profile(False)
    clk = clocks.stop()
    ctx.sync()
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    value = world * len(THETAS) * n_s * args.steps / (ms / 1e3) / 1e9

    # ---- roofline of the dominant kernel ----
    dom = max(prof.items(), key=lambda kv: kv[1][1])
    dom_name, (dom_launches, dom_ms) = dom
    joins = len(THETAS) * args.steps
    per_join = kernel_bytes(dom_name, n_r, n_s)
    peak, peak_kind = hbm_peak()
    roof = None
    if per_join is not None:
        achieved = per_join * joins / (dom_ms / 1e3) / 1e9
        per_launch_bytes = per_join * joins / dom_launches
        traffic = traffic_from_profiles(dom_name)
        roof = {"bound": "hbm", "kernel": dom_name, "achieved": round(achieved, 1),
                "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                "peak_source": peak_kind, "traffic": traffic,
                "algorithmic_bytes_per_launch": per_launch_bytes,
                "avg_launch_ms": dom_ms / dom_launches}
    kernels = {k: {"launches": v[0], "ms_total": round(v[1], 3),
                   "share": round(v[1] / sum(x[1] for x in prof.values()), 4)}
               for k, v in sorted(prof.items(), key=lambda kv: -kv[1][1])}
    compulsory = 4 * (n_r + n_s)  # key bytes of one join

    # ---- end to end through the API with host buffers ----
    e2e = None
    if not args.no_e2e:
        h_r = torch.from_numpy(rk).pin_memory()
        h_s = [torch.from_numpy(s).pin_memory() for s in sks]
        h_out = torch.empty((len(THETAS), 2), dtype=torch.int64).pin_memory()

        def e2e_step():
            d_r.copy_(h_r, non_blocking=True)
            for i, (hs, ds, o) in enumerate(zip(h_s, d_s, outs)):
                ds.copy_(hs, non_blocking=True)
                ctx.radix_join_agg(d_r, None, ds, None, aggs, out=o)
                h_out[i].copy_(o, non_blocking=True)

        for _ in range(max(1, args.warmup)):
            e2e_step()
        barrier()
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        for _ in range(args.steps):
            e2e_step()
        f1.record(stream)
        barrier()
        ems = f0.elapsed_time(f1)
        if world > 1:
            t = torch.tensor([ems], device="cuda")
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            ems = float(t.item())
        assert h_out.tolist() == results, "e2e results differ from resident results"
        e2e = {"value": world * len(THETAS) * n_s * args.steps / (ems / 1e3) / 1e9, "unit": UNIT,
               "h2d_bytes_per_step": 4 * (n_r + len(THETAS) * n_s),
               "d2h_bytes_per_step": 16 * len(THETAS), "ms_per_step": ems / args.steps}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        sample = min(args.cpu_sample_log, args.log_s)
        v, dt = cpu_baseline(rk, sks, sample, threads)
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"full R (2^{args.log_r}), first 2^{sample} rows of each S "
                         f"(theta 0/0.5/1.0), {dt:.1f} s; oracle C port of the reference's "
                         f"partitioned chained-hash join, {threads} threads"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic (seeded generator)",
            "config": {"workload": WORKLOAD, "n_build": n_r, "n_probe": n_s,
                       "thetas": list(THETAS), "hit_rate": HIT_RATE,
                       "parallelism": f"replicas x{world}",
                       "l2": "inputs larger than L2 (2 GiB probe keys per join)"},
            "e2e": e2e, "roofline": roof, "cpu_baseline": cpu, "clocks": clk,
            "gpu_launches": launches,
            "job_hbm_gbs_compulsory": round(compulsory * joins / (ms / 1e3) / 1e9, 1),
            "job_frac_compulsory": round(compulsory * joins / (ms / 1e3) / 1e9 / peak, 4),
            "build_plus_probe_gtuples_s": round(world * len(THETAS) * (n_r + n_s) * args.steps
                                                / (ms / 1e3) / 1e9, 3),
            "kernels": kernels, "results": results,
        }
        print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
