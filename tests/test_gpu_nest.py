"""RadixNest over int64 keys and the int64 RJStepwise count (the
aggregation twins of radix-aggr.cpp) on the GPU vs the oracle."""
import numpy as np
import pytest

from gpu_util import dev, host
from proteus_gb300 import abi

pytestmark = pytest.mark.gpu

I64 = np.iinfo(np.int64)


def gpu_nest(ctx, k, v, cap, **kw):
    res = ctx.nest_i64(dev(k), dev(v) if v is not None else None, cap, **kw)
    ctx.sync()
    ng = int(host(res[5])[0])
    cols = [host(t)[:ng] for t in res[:5]]
    o = np.argsort(cols[0], kind="stable")
    return tuple(c[o] for c in cols)


def check_nest(ctx, oracle, k, v, **kw):
    exp = oracle.nest_i64(k, v)
    got = gpu_nest(ctx, k, v, max(len(exp[0]), 1), **kw)
    assert len(got[0]) == len(exp[0])
    names = ("key", "count", "sum", "min", "max")
    for name, a, b in zip(names, got, exp):
        if v is None and name in ("sum", "min", "max"):
            assert (a == 0).all()
        else:
            assert (a == b).all(), name


@pytest.mark.parametrize("groups,span_bits", [(16, 60), (1000, 40), (1 << 16, 62), (1 << 18, 63)])
def test_nest_i64_parity(ctx, oracle, groups, span_bits):
    rng = np.random.default_rng(groups)
    base = rng.integers(-(1 << (span_bits - 1)), 1 << (span_bits - 1), groups, dtype=np.int64)
    k = base[rng.integers(0, groups, 1 << 20)]
    v = rng.integers(I64.min, I64.max, len(k), dtype=np.int64)
    check_nest(ctx, oracle, k, v, expected_groups=groups)
    check_nest(ctx, oracle, k, None, expected_groups=groups)


def test_nest_i64_extremes_and_empty(ctx, oracle):
    rng = np.random.default_rng(5)
    k = rng.integers(-3, 3, 100000).astype(np.int64)
    k[::9] = I64.min
    k[::11] = I64.max
    v = np.where(rng.random(len(k)) < 0.5, I64.max, I64.min).astype(np.int64)
    v[::5] = -1
    check_nest(ctx, oracle, k, v, expected_groups=8)
    check_nest(ctx, oracle, k, v)  # no size hint
    e = np.zeros(0, np.int64)
    res = ctx.nest_i64(dev(e), dev(e), 4)
    ctx.sync()
    assert int(host(res[5])[0]) == 0


def test_nest_i64_capacity_error(ctx):
    k = np.arange(5000, dtype=np.int64) * 7919
    res = ctx.nest_i64(dev(k), dev(k), 100, expected_groups=5000)
    with pytest.raises(abi.GbjError) as e:
        ctx.sync()
    assert e.value.code == abi.ERR_CAPACITY
    assert int(host(res[5])[0]) == 5000


@pytest.mark.parametrize("nr,ns,span", [(1 << 12, 1 << 14, 1 << 13), (40000, 90001, 1 << 18),
                                        (1 << 16, 1 << 16, 1 << 62), (3000, 200000, 1 << 11)])
def test_join_count_i64_parity(ctx, oracle, nr, ns, span):
    rng = np.random.default_rng(nr + ns)
    r = rng.integers(0, span, nr, dtype=np.int64) - span // 2
    s = rng.integers(0, span, ns, dtype=np.int64) - span // 2
    r[::17] = I64.min
    s[::19] = I64.min
    got = int(host(ctx.radix_join_count_i64(dev(r), dev(s)))[0])
    ctx.sync()
    assert got == oracle.join_count_i64(r, s)
    assert int(host(ctx.radix_join_count_i64(dev(r[:0]), dev(s)))[0]) == 0


def test_nest_i64_hot_groups_wrap(ctx, oracle):
    """Three keys over 2^24 rows: every CTA's on-chip slots pass the 65535-row
    bound and move to the global table; values at both int64 extremes."""
    rng = np.random.default_rng(12)
    n = (1 << 24) + 3
    k = np.array([-1, 0, 5], dtype=np.int64)[rng.integers(0, 3, n)]
    k[rng.integers(0, n, 1000)] = I64.min
    v = np.where(rng.random(n) < 0.5, I64.max, I64.min).astype(np.int64)
    v[::7] = -1
    check_nest(ctx, oracle, k, v, expected_groups=4)
