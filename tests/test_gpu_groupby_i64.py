"""Hash group-by over int64 keys (HashGroupByChained with an int64 key,
int32 values) on the GPU vs the oracle's int64 grouping fold."""
import numpy as np
import pytest

from gpu_util import dev, host
from proteus_gb300 import abi

pytestmark = pytest.mark.gpu

I64, I32 = np.iinfo(np.int64), np.iinfo(np.int32)


def gpu_groupby(ctx, k, v, cap, **kw):
    res = ctx.groupby(dev(k), dev(v), cap, **kw)
    ctx.sync()
    ng = int(host(res[5])[0])
    cols = [host(t)[:ng] for t in res[:5]]
    o = np.argsort(cols[0], kind="stable")
    return tuple(c[o] for c in cols)


def check(ctx, oracle, k, v, **kw):
    # the oracle's fold over int64 keys with the int32 values widened: the
    # same groups, counts, sums and extremes
    exp = oracle.nest_i64(k, v.astype(np.int64))
    got = gpu_groupby(ctx, k, v, max(len(exp[0]), 1), **kw)
    assert got[0].dtype == np.int64 and got[3].dtype == np.int32
    assert len(got[0]) == len(exp[0])
    for name, a, b in zip(("key", "count", "sum", "min", "max"), got, exp):
        assert (a.astype(np.int64) == b).all(), name


@pytest.mark.parametrize("groups,span_bits,hinted", [(16, 60, True), (1000, 40, True), (1 << 16, 62, False),
                                                     (1 << 18, 63, True)])
def test_groupby_i64_parity(ctx, oracle, groups, span_bits, hinted):
    rng = np.random.default_rng(groups)
    base = rng.integers(-(1 << (span_bits - 1)), 1 << (span_bits - 1), groups, dtype=np.int64)
    k = base[rng.integers(0, groups, 1 << 20)]
    v = rng.integers(I32.min, I32.max, len(k), dtype=np.int64).astype(np.int32)
    check(ctx, oracle, k, v, expected_groups=groups if hinted else 0)


def test_groupby_i64_extremes_and_params(ctx, oracle):
    rng = np.random.default_rng(3)
    k = rng.integers(-3, 3, 200000).astype(np.int64) * (1 << 40)
    k[::9] = I64.min
    k[::11] = I64.max
    v = np.where(rng.random(len(k)) < 0.5, I32.max, I32.min).astype(np.int32)
    v[::5] = -1
    check(ctx, oracle, k, v, expected_groups=8)
    check(ctx, oracle, k, v, max_input_size=64)
    check(ctx, oracle, k, v, hash_bits=12, strategy=1)


def test_groupby_i64_refusals(ctx):
    k = np.arange(5000, dtype=np.int64) * 7919
    v = np.ones(5000, dtype=np.int32)
    with pytest.raises(abi.GbjError) as e:
        ctx.groupby(dev(k), dev(v), 5000, strategy=2)
    assert e.value.code == abi.ERR_UNSUPPORTED
    res = ctx.groupby(dev(k), dev(v), 100, expected_groups=5000)
    with pytest.raises(abi.GbjError) as e:
        ctx.sync()
    assert e.value.code == abi.ERR_CAPACITY
    assert int(host(res[5])[0]) == 5000


def test_groupby_i64_empty_and_tail(ctx, oracle):
    e = np.zeros(0, np.int64)
    res = ctx.groupby(dev(e), dev(np.zeros(0, np.int32)), 4)
    ctx.sync()
    assert int(host(res[5])[0]) == 0
    rng = np.random.default_rng(17)
    k = rng.integers(-5, 5, 1001).astype(np.int64) << 33  # keys equal in their low words
    v = rng.integers(-100, 100, 1001).astype(np.int32)
    check(ctx, oracle, k, v, expected_groups=10)


def test_groupby_i64_hot_key(ctx, oracle):
    """One key on most rows (more than 65535 per CTA: the on-chip level's
    flush path) with a few cold keys, hinted and unhinted."""
    rng = np.random.default_rng(29)
    k = np.where(rng.random(1 << 21) < 0.9, np.int64(-7) << 50, rng.integers(0, 64, 1 << 21)).astype(np.int64)
    v = rng.integers(I32.min, I32.max, len(k), dtype=np.int64).astype(np.int32)
    check(ctx, oracle, k, v, expected_groups=65)
    check(ctx, oracle, k, v)
