"""Autotuner: decisions are cached per shape, used by later calls without
explicit sizing, survive save/load, and never change results."""
import numpy as np
import pytest

from gpu_util import CONFIG1_AGGS, CONFIG2_AGGS, cpu_threads, dev, host, sort_groups
from proteus_gb300 import engine

pytestmark = pytest.mark.gpu


def test_tune_radix_join(ctx, oracle):
    ctx.tune_clear()
    bk, _ = engine.gen_build_side(31, 1 << 20, payload=False)
    pk, _ = engine.gen_probe_zipf(32, 1 << 22, 1 << 20, 0.5)
    dbk, dpk = dev(bk), dev(pk)
    assert ctx.tune_lookup("radix", 1 << 20, 1 << 22) == -1
    assert ctx.tune_lookup("radixblock", 1 << 20, 1 << 22) == -1
    bits, ms = ctx.autotune_radix_join(dbk, None, dpk, None, CONFIG2_AGGS)
    assert 1 <= bits <= 15 and ms > 0
    # the block size and, for it, the bits: both decided, both cached
    block = ctx.tune_lookup("radixblock", 1 << 20, 1 << 22)
    assert block in (512, 1024)
    assert ctx.tune_lookup("radix" if block == 1024 else "radix512", 1 << 20, 1 << 22) == bits
    out = ctx.radix_join_agg(dbk, None, dpk, None, CONFIG2_AGGS)  # uses the tuned shape and bits
    ctx.sync()
    exp = oracle.radix_join_agg(bk, None, pk, None, CONFIG2_AGGS, threads=cpu_threads())
    assert host(out).tolist() == list(exp)


def test_tune_join_and_save_load(ctx, oracle, tmp_path):
    ctx.tune_clear()
    bk, bp = engine.gen_build_side(41, 1 << 18)
    pk, pp = engine.gen_probe_uniform(42, 1 << 21, 1 << 18)
    d = [dev(x) for x in (bk, bp, pk, pp)]
    hb, ms = ctx.autotune_join(*d, CONFIG1_AGGS)
    assert 19 <= hb <= 21
    t = ctx.join_build(d[0], d[1])  # hash_bits 0: tuned size
    assert t.slots == 1 << hb
    out = ctx.join_probe_agg(t, d[2], d[3], CONFIG1_AGGS)
    ctx.sync()
    assert host(out).tolist() == list(oracle.join_agg(bk, bp, pk, pp, CONFIG1_AGGS, threads=cpu_threads()))
    path = str(tmp_path / "tune.txt")
    ctx.tune_save(path)
    ctx.tune_clear()
    assert ctx.tune_lookup("join", 1 << 18, 0) == -1
    ctx.tune_load(path)
    assert ctx.tune_lookup("join", 1 << 18, 0) == hb


@pytest.mark.parametrize("card", [1 << 10, 1 << 18])
def test_tune_groupby(ctx, oracle, card):
    ctx.tune_clear()
    k, v = engine.gen_groupby(51 + card, 1 << 22, card, 0.0)
    dk, dv = dev(k), dev(v)
    st, bits, ms = ctx.autotune_groupby(dk, dv, card)
    assert st in (1, 2) and ms > 0
    assert ctx.tune_lookup("groupby", 1 << 22, card) == (st << 8 | bits)
    res = ctx.groupby(dk, dv, card + 16, expected_groups=card)
    ctx.sync()
    got = sort_groups(*[host(x) for x in res[:5]], host(res[5])[0])
    exp = oracle.groupby(k, v, threads=cpu_threads())
    for a, b in zip(got, exp):
        assert (a == b).all()
