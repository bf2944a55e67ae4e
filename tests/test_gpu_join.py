"""Plain hash join (HashJoinChained semantics) on the GPU vs the oracle."""
import numpy as np
import pytest

from gpu_util import CONFIG1_AGGS, cpu_threads, dev, host
from proteus_gb300 import abi, engine

pytestmark = pytest.mark.gpu

ALL_AGGS = [
    (abi.AGG_COUNT, abi.VAL_ONE),
    (abi.AGG_SUM, abi.VAL_PRODUCT),
    (abi.AGG_MIN, abi.VAL_BUILD),
    (abi.AGG_MAX, abi.VAL_PROBE),
    (abi.AGG_SUM, abi.VAL_ROWID_XOR),
    (abi.AGG_MAX, abi.VAL_BUILD_ROWID),
    (abi.AGG_MIN, abi.VAL_PROBE_ROWID),
    (abi.AGG_SUM, abi.VAL_BUILD_KEY),
]


def gpu_join(ctx, rk, rp, sk, sp, aggs, hash_bits=0):
    t = ctx.join_build(dev(rk), dev(rp) if rp is not None else None, hash_bits=hash_bits)
    out = ctx.join_probe_agg(t, dev(sk), dev(sp) if sp is not None else None, aggs)
    ctx.sync()
    r = host(out).tolist()
    t.destroy()
    return r


@pytest.mark.parametrize("nr,ns,seed", [(1 << 10, 1 << 14, 1), (1 << 16, 1 << 20, 2),
                                        (1000, 77777, 3)])
def test_plain_join_small(ctx, oracle, nr, ns, seed):
    rk, rp = engine.gen_build_side(seed, nr)
    sk, sp = engine.gen_probe_uniform(seed, ns, nr)
    exp = oracle.join_agg(rk, rp, sk, sp, ALL_AGGS, threads=cpu_threads())
    assert gpu_join(ctx, rk, rp, sk, sp, ALL_AGGS) == exp


def test_plain_join_full_config(ctx, oracle):
    """R = 2^20 permuted keys, S = 2^24 uniform keys: COUNT and SUM(R.p*S.p)."""
    rk, rp = engine.gen_build_side(2024, 1 << 20)
    sk, sp = engine.gen_probe_uniform(2024, 1 << 24, 1 << 20)
    got = gpu_join(ctx, rk, rp, sk, sp, CONFIG1_AGGS)
    assert got[0] == 1 << 24  # every probe row matches exactly once
    exp = oracle.join_agg(rk, rp, sk, sp, CONFIG1_AGGS, threads=cpu_threads())
    assert got == exp


def test_duplicate_build_keys(ctx, oracle):
    rng = np.random.default_rng(5)
    rk = rng.integers(0, 300, 20000).astype(np.int32)
    rp = rng.integers(-1000, 1000, 20000).astype(np.int32)
    sk = rng.integers(-50, 400, 50000).astype(np.int32)
    sp = rng.integers(-1000, 1000, 50000).astype(np.int32)
    exp = oracle.join_agg(rk, rp, sk, sp, ALL_AGGS)
    assert gpu_join(ctx, rk, rp, sk, sp, ALL_AGGS) == exp


def test_extreme_keys(ctx, oracle):
    ext = np.array([np.iinfo(np.int32).min, np.iinfo(np.int32).max, 0, -1, 1], dtype=np.int32)
    rk = np.concatenate([ext, ext[:3], np.arange(-500, 500, dtype=np.int32)])
    rp = np.arange(len(rk), dtype=np.int32)
    sk = np.concatenate([ext, ext, np.arange(-1000, 1000, 3, dtype=np.int32)])
    sp = (np.arange(len(sk), dtype=np.int32) * 7) % 1000
    exp = oracle.join_agg(rk, rp, sk, sp, ALL_AGGS)
    assert gpu_join(ctx, rk, rp, sk, sp, ALL_AGGS) == exp


def test_empty_sides(ctx, oracle):
    rk, rp = engine.gen_build_side(1, 100)
    e = np.zeros(0, dtype=np.int32)
    ident = oracle.join_agg(e, e, rk, rp, ALL_AGGS)
    assert ident[0] == 0 and ident[2] == np.iinfo(np.int64).max
    assert gpu_join(ctx, e, e, rk, rp, ALL_AGGS) == ident
    assert gpu_join(ctx, rk, rp, e, e, ALL_AGGS) == oracle.join_agg(rk, rp, e, e, ALL_AGGS)


def test_unaligned_inputs(ctx, oracle):
    rk, rp = engine.gen_build_side(8, 5000)
    sk, sp = engine.gen_probe_uniform(8, 40001, 5000)
    import torch

    dsk = torch.cat([torch.zeros(1, dtype=torch.int32, device="cuda"), dev(sk)])[1:]
    dsp = torch.cat([torch.zeros(1, dtype=torch.int32, device="cuda"), dev(sp)])[1:]
    assert dsk.data_ptr() % 16 != 0
    t = ctx.join_build(dev(rk), dev(rp))
    out = ctx.join_probe_agg(t, dsk, dsp, ALL_AGGS)
    ctx.sync()
    assert host(out).tolist() == oracle.join_agg(rk, rp, sk, sp, ALL_AGGS)


def test_hash_bits_from_plan(ctx, oracle):
    rk, rp = engine.gen_build_side(9, 3000)
    sk, sp = engine.gen_probe_uniform(9, 9000, 3000)
    exp = oracle.join_agg(rk, rp, sk, sp, CONFIG1_AGGS, hash_bits=4)
    assert gpu_join(ctx, rk, rp, sk, sp, CONFIG1_AGGS, hash_bits=16) == exp
    t = ctx.join_build(dev(rk), dev(rp), hash_bits=16)
    assert t.slots == 1 << 16


def test_probe_pairs(ctx, oracle):
    rng = np.random.default_rng(2)
    rk = rng.integers(0, 2000, 3000).astype(np.int32)
    sk = rng.integers(0, 2500, 7000).astype(np.int32)
    eb, ep = oracle.join_pairs(rk, sk)
    t = ctx.join_build(dev(rk))
    b, p, cnt = ctx.join_probe_pairs(t, dev(sk), capacity=len(eb) + 10)
    ctx.sync()
    m = int(host(cnt)[0])
    assert m == len(eb)
    got = sorted(zip(host(b)[:m].tolist(), host(p)[:m].tolist()))
    assert got == sorted(zip(eb.tolist(), ep.tolist()))


def test_probe_pairs_capacity_error(ctx):
    rk = np.zeros(10, dtype=np.int32)
    sk = np.zeros(10, dtype=np.int32)  # 100 matches
    t = ctx.join_build(dev(rk))
    b, p, cnt = ctx.join_probe_pairs(t, dev(sk), capacity=50)
    with pytest.raises(abi.GbjError) as e:
        ctx.sync()
    assert e.value.code == abi.ERR_CAPACITY
    assert int(host(cnt)[0]) == 100
    ctx.sync()  # the error was reported once and cleared


def test_max_build_capacity(ctx):
    rk, rp = engine.gen_build_side(1, 200)
    with pytest.raises(abi.GbjError) as e:
        ctx.join_build(dev(rk), dev(rp), max_build=128)
    assert e.value.code == abi.ERR_CAPACITY


def test_invalid_aggregate(ctx):
    rk, rp = engine.gen_build_side(1, 100)
    t = ctx.join_build(dev(rk))
    with pytest.raises(abi.GbjError) as e:
        ctx.join_probe_agg(t, dev(rk), dev(rp), [(abi.AGG_SUM, abi.VAL_PRODUCT)])
    assert e.value.code == abi.ERR_INVALID
    with pytest.raises(abi.GbjError):
        ctx.join_probe_agg(t, dev(rk), dev(rp), [(9, abi.VAL_ONE)])


def test_probe_pairs_payload_table_and_int32_min(ctx, oracle):
    """Pairs from a table built with a payload (rows kept beside the
    buckets) and INT32_MIN keys on both sides (the side list)."""
    rng = np.random.default_rng(12)
    rk = rng.integers(-300, 300, 4000).astype(np.int32)
    rk[::50] = np.iinfo(np.int32).min
    rp = rng.integers(-1000, 1000, len(rk)).astype(np.int32)
    sk = rng.integers(-400, 400, 9000).astype(np.int32)
    sk[::70] = np.iinfo(np.int32).min
    eb, ep = oracle.join_pairs(rk, sk)
    t = ctx.join_build(dev(rk), dev(rp))
    b, p, cnt = ctx.join_probe_pairs(t, dev(sk), capacity=len(eb) + 10)
    ctx.sync()
    m = int(host(cnt)[0])
    assert m == len(eb)
    got = sorted(zip(host(b)[:m].tolist(), host(p)[:m].tolist()))
    assert got == sorted(zip(eb.tolist(), ep.tolist()))
    # and the aggregates over the same table
    out = ctx.join_probe_agg(t, dev(sk), dev(sk), ALL_AGGS)
    ctx.sync()
    assert host(out).tolist() == oracle.join_agg(rk, rp, sk, sk, ALL_AGGS)
