"""Radix clustering of int64-key tuples (the radix-aggr.cpp twins) on the
GPU: partitionHT's cluster counts equal the reference goldens and every
cluster holds exactly the oracle's tuples."""
import json
import os

import numpy as np

import pytest

import datagen
from gpu_util import dev, host
from proteus_gb300 import abi

pytestmark = pytest.mark.gpu


def _keys(lib, c):
    span = int(c["span"])
    keys = np.array([int(datagen.load().gbj_gen_rand(c["seed"], 0x6A00, i)) % span for i in range(c["n"])], dtype=np.uint64)
    return keys.view(np.int64) - (np.int64(span // 2) if span < (1 << 63) else 0)


def test_partition_ht_agg_counts(ctx, lib, oracle):
    import hashlib

    with open(os.path.join(os.path.dirname(__file__), "golden", "partition_ht_agg_cases.json")) as f:
        cases = json.load(f)["cases"]
    for c in cases:
        keys = _keys(lib, c)
        ok, orow, off = ctx.partition_i64(dev(keys), None, bits=14)
        ctx.sync()
        counts = np.diff(host(off)).astype(np.int32)
        assert hashlib.sha256(counts.tobytes()).hexdigest()[:16] == c["counts_sha"]
        ok, orow = host(ok), host(orow)
        assert (keys[orow] == ok).all()  # every tuple carries its own row id
        _, ek, er = oracle.partition_ht_agg(keys)
        offs = host(off)
        for p in np.unique(keys[:64] & ((1 << 14) - 1)):
            assert sorted(orow[offs[p]:offs[p + 1]].tolist()) == sorted(er[offs[p]:offs[p + 1]].tolist())


@pytest.mark.parametrize("shift,bits", [(0, 7), (7, 7), (20, 12), (50, 13)])
def test_partition_i64_any_digit(ctx, oracle, shift, bits):
    rng = np.random.default_rng(shift * 100 + bits)
    n = (1 << 20) + 11
    keys = rng.integers(-(1 << 62), 1 << 62, n, dtype=np.int64)
    pay = rng.integers(-(1 << 62), 1 << 62, n, dtype=np.int64)
    ok, op, off = ctx.partition_i64(dev(keys), dev(pay), bits=bits, shift=shift)
    ctx.sync()
    ek, ep, eoff = oracle.radix_cluster_i64(keys, pay, shift, bits)
    assert (host(off) == eoff.astype(np.int64)).all()
    ok, op = host(ok), host(op)
    o = host(off)
    for p in np.unique(rng.integers(0, 1 << bits, 16)):
        got = sorted(zip(ok[o[p]:o[p + 1]].tolist(), op[o[p]:o[p + 1]].tolist()))
        exp = sorted(zip(ek[o[p]:o[p + 1]].tolist(), ep[o[p]:o[p + 1]].tolist()))
        assert got == exp


def test_partition_i64_errors(ctx):
    with pytest.raises(abi.GbjError):
        ctx.partition_i64(dev(np.arange(8, dtype=np.int64)), None, bits=16)
