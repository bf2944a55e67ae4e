"""Plain hash join over int64 keys (HashJoinChained with an int64 key) on the
GPU vs the oracle's int64 chained join."""
import numpy as np
import pytest

from gpu_util import dev, host
from proteus_gb300 import abi

pytestmark = pytest.mark.gpu

AGGS = [
    (abi.AGG_COUNT, abi.VAL_ONE),
    (abi.AGG_SUM, abi.VAL_PRODUCT),
    (abi.AGG_MIN, abi.VAL_BUILD),
    (abi.AGG_MAX, abi.VAL_PROBE),
    (abi.AGG_SUM, abi.VAL_ROWID_XOR),
    (abi.AGG_MAX, abi.VAL_BUILD_KEY),
    (abi.AGG_MIN, abi.VAL_BUILD_KEY),
    (abi.AGG_SUM, abi.VAL_BUILD_KEY),
]


def gpu_join(ctx, rk, rp, sk, sp, aggs, hash_bits=0):
    t = ctx.join_build(dev(rk), dev(rp) if rp is not None else None, hash_bits=hash_bits)
    assert t.i64
    out = ctx.join_probe_agg(t, dev(sk), dev(sp) if sp is not None else None, aggs)
    ctx.sync()
    r = host(out).tolist()
    t.destroy()
    return r


def wide_keys(rng, n):
    """Distinct int64 keys spread over the whole range (high words differ)."""
    k = rng.choice(np.int64(1) << 62, size=n, replace=False).astype(np.int64)
    return k * rng.choice(np.array([-1, 1], dtype=np.int64), size=n) + rng.integers(-3, 3, n)


@pytest.mark.parametrize("nr,ns,seed", [(1 << 10, 1 << 14, 1), (1 << 16, 1 << 20, 2), (999, 77777, 3)])
def test_join_i64_unique(ctx, oracle, nr, ns, seed):
    rng = np.random.default_rng(seed)
    rk = np.unique(wide_keys(rng, nr))
    rng.shuffle(rk)
    rp = rng.integers(-1000, 1000, len(rk)).astype(np.int32)
    # hits, and misses that share the low 32 bits of a build key
    hit = rk[rng.integers(0, len(rk), ns)]
    miss = hit ^ (np.int64(1) << 40)
    sk = np.where(rng.random(ns) < 0.8, hit, miss).astype(np.int64)
    sp = rng.integers(-1000, 1000, ns).astype(np.int32)
    exp = oracle.join_agg_i64(rk, rp, sk, sp, AGGS)
    assert gpu_join(ctx, rk, rp, sk, sp, AGGS) == exp


def test_join_i64_duplicates_and_extremes(ctx, oracle):
    rng = np.random.default_rng(7)
    base = np.array([np.iinfo(np.int64).min, np.iinfo(np.int64).max, -1, 0, 1, 1 << 32, -(1 << 32)],
                    dtype=np.int64)
    rk = np.concatenate([np.repeat(base, 3), rng.integers(-50, 50, 20000)]).astype(np.int64)
    rng.shuffle(rk)
    rp = rng.integers(-1000, 1000, len(rk)).astype(np.int32)
    sk = np.concatenate([base, rng.integers(-60, 60, 50000), base]).astype(np.int64)
    sp = rng.integers(-1000, 1000, len(sk)).astype(np.int32)
    exp = oracle.join_agg_i64(rk, rp, sk, sp, AGGS)
    assert gpu_join(ctx, rk, rp, sk, sp, AGGS) == exp


def test_join_i64_no_payload_and_small_table(ctx, oracle):
    rng = np.random.default_rng(9)
    rk = rng.integers(-(1 << 40), 1 << 40, 5000).astype(np.int64)
    sk = np.concatenate([rk, rng.integers(-(1 << 40), 1 << 40, 5000)]).astype(np.int64)
    aggs = [(abi.AGG_COUNT, abi.VAL_ONE), (abi.AGG_SUM, abi.VAL_ROWID_XOR), (abi.AGG_MAX, abi.VAL_BUILD_ROWID)]
    exp = oracle.join_agg_i64(rk, None, sk, None, aggs)
    # hash_bits smaller than the build side: a sizing hint only, never a cap
    assert gpu_join(ctx, rk, None, sk, None, aggs, hash_bits=4) == exp


def test_join_i64_pairs(ctx, oracle):
    rng = np.random.default_rng(11)
    rk = rng.integers(-30, 30, 3000).astype(np.int64) * (1 << 35)
    sk = rng.integers(-40, 40, 7000).astype(np.int64) * (1 << 35)
    eb, ep = oracle.join_pairs_i64(rk, sk)
    t = ctx.join_build(dev(rk))
    b, p, cnt = ctx.join_probe_pairs(t, dev(sk), len(eb) + 16)
    ctx.sync()
    m = int(host(cnt)[0])
    assert m == len(eb)
    got = sorted(zip(host(b)[:m].tolist(), host(p)[:m].tolist()))
    assert got == sorted(zip(eb.tolist(), ep.tolist()))
    t.destroy()


def test_join_i64_table_kind_is_checked(ctx):
    """A probe of the other key width is refused with GBJ_ERR_INVALID."""
    import ctypes as C

    from proteus_gb300.engine import _ptr

    t64 = ctx.join_build(dev(np.arange(10, dtype=np.int64)))
    t32 = ctx.join_build(dev(np.arange(10, dtype=np.int32)))
    k32, k64 = dev(np.arange(10, dtype=np.int32)), dev(np.arange(10, dtype=np.int64))
    out = dev(np.zeros(1, dtype=np.int64))
    arr = abi.aggs_array([(abi.AGG_COUNT, abi.VAL_ONE)])
    rc = ctx.lib.gbj_join_probe_agg(ctx.handle, t64.handle, _ptr(k32), None, 10, arr, 1, _ptr(out), None)
    assert rc == abi.ERR_INVALID
    rc = ctx.lib.gbj_join_probe_agg_i64(ctx.handle, t32.handle, _ptr(k64), None, 10, arr, 1, _ptr(out), None)
    assert rc == abi.ERR_INVALID
    assert ctx.join_probe_agg(t64, k64, None, [(abi.AGG_COUNT, abi.VAL_ONE)]).cpu().tolist() == [10]
    t64.destroy()
    t32.destroy()


def test_join_i64_empty_sides(ctx, oracle):
    rng = np.random.default_rng(13)
    k = rng.integers(-(1 << 40), 1 << 40, 100).astype(np.int64)
    p = rng.integers(-9, 9, 100).astype(np.int32)
    e64, e32 = np.zeros(0, np.int64), np.zeros(0, np.int32)
    assert gpu_join(ctx, e64, e32, k, p, AGGS) == oracle.join_agg_i64(e64, e32, k, p, AGGS)
    assert gpu_join(ctx, k, p, e64, e32, AGGS) == oracle.join_agg_i64(k, p, e64, e32, AGGS)


def test_join_i64_pairs_side_list_and_duplicates(ctx, oracle):
    """Pairs with INT64_MIN keys on both sides (the side list) and duplicate
    build keys, against the oracle."""
    rng = np.random.default_rng(23)
    rk = rng.integers(-20, 20, 5000).astype(np.int64) * ((1 << 40) + 3)
    rk[::40] = np.iinfo(np.int64).min
    sk = rng.integers(-25, 25, 8000).astype(np.int64) * ((1 << 40) + 3)
    sk[::90] = np.iinfo(np.int64).min
    eb, ep = oracle.join_pairs_i64(rk, sk)
    t = ctx.join_build(dev(rk))
    b, p, cnt = ctx.join_probe_pairs(t, dev(sk), len(eb) + 16)
    ctx.sync()
    m = int(host(cnt)[0])
    assert m == len(eb)
    assert sorted(zip(host(b)[:m].tolist(), host(p)[:m].tolist())) == sorted(zip(eb.tolist(), ep.tolist()))
    t.destroy()
