"""Hash group-by (HashGroupByChained semantics) on the GPU vs the oracle."""
import numpy as np
import pytest

from gpu_util import cpu_threads, dev, host, sort_groups
from proteus_gb300 import abi, engine

pytestmark = pytest.mark.gpu


def gpu_groupby(ctx, k, v, cap, **kw):
    res = ctx.groupby(dev(k), dev(v), cap, **kw)
    ctx.sync()
    ok, oc, osum, omin, omax, ng = [host(t) for t in res]
    return sort_groups(ok, oc, osum, omin, omax, ng[0])


def check(ctx, oracle, k, v, **kw):
    exp = oracle.groupby(k, v, threads=cpu_threads())
    got = gpu_groupby(ctx, k, v, max(len(exp[0]), 1), **kw)
    assert len(got[0]) == len(exp[0])
    for a, b in zip(got, exp):
        assert (a == b).all()


@pytest.mark.parametrize("card", [1, 16, 1000, 1 << 16])
@pytest.mark.parametrize("theta", [0.0, 1.0])
@pytest.mark.parametrize("strategy", [0, 1, 2])
def test_groupby_parity(ctx, oracle, card, theta, strategy):
    k, v = engine.gen_groupby(card * 3 + int(theta), 1 << 20, card, theta)
    check(ctx, oracle, k, v, expected_groups=card, strategy=strategy)


def test_groupby_no_hint(ctx, oracle):
    k, v = engine.gen_groupby(77, 1 << 20, 5000, 0.0)
    check(ctx, oracle, k, v)


def test_groupby_extreme_keys_and_values(ctx, oracle):
    i32 = np.iinfo(np.int32)
    k = np.array([i32.min, i32.min, i32.max, 0, -1, i32.min, 5, 5, i32.max], dtype=np.int32)
    v = np.array([i32.max, i32.min, -1, 0, 7, i32.max, i32.min, i32.max, 1], dtype=np.int32)
    k = np.tile(k, 1000)
    v = np.tile(v, 1000)
    for strategy in (1, 2):
        check(ctx, oracle, k, v, expected_groups=16, strategy=strategy)
        check(ctx, oracle, k, v, expected_groups=1 << 12, strategy=strategy)


def test_groupby_many_groups_spill(ctx, oracle):
    """More groups than the on-chip table: level-1 spills to level 2."""
    k, v = engine.gen_groupby(5, 1 << 21, 1 << 18, 0.0)
    check(ctx, oracle, k, v, expected_groups=1 << 18, strategy=1)
    check(ctx, oracle, k, v, expected_groups=1 << 18, strategy=2)


def test_groupby_capacity_error(ctx):
    k = np.arange(10000, dtype=np.int32)
    res = ctx.groupby(dev(k), dev(k), 100, expected_groups=20000)
    with pytest.raises(abi.GbjError) as e:
        ctx.sync()
    assert e.value.code == abi.ERR_CAPACITY
    assert int(host(res[5])[0]) == 10000


def test_groupby_empty(ctx):
    e = np.zeros(0, dtype=np.int32)
    res = ctx.groupby(dev(e), dev(e), 10)
    ctx.sync()
    assert int(host(res[5])[0]) == 0


@pytest.mark.parametrize("card,theta", [(1 << 4, 0.0), (1 << 10, 1.0), (1 << 16, 0.0),
                                        (1 << 20, 1.0), (1 << 24, 0.0), (1 << 24, 1.0)])
def test_groupby_full_config(ctx, oracle, card, theta):
    """2^29 rows, value U[-2^20, 2^20): full size."""
    k, v = engine.gen_groupby(900 + card.bit_length() + int(theta), 1 << 29, card, theta)
    check(ctx, oracle, k, v, expected_groups=card)


@pytest.mark.parametrize("strategy", [1, 2])
def test_groupby_hot_groups_wrap(ctx, oracle, strategy):
    """Groups far above 65535 rows per CTA with extreme values: the on-chip
    16-bit sum halves and counts are moved to level 2 before they wrap."""
    i32 = np.iinfo(np.int32)
    rng = np.random.default_rng(21)
    n = (1 << 22) + 3
    k = rng.integers(0, 3, n).astype(np.int32)
    k[rng.integers(0, n, 1000)] = i32.min
    v = np.where(rng.random(n) < 0.5, i32.max, i32.min).astype(np.int32)
    v[::7] = -1
    check(ctx, oracle, k, v, expected_groups=4, strategy=strategy)


def test_groupby_unaligned_columns(ctx, oracle):
    """Columns that do not start on a 16-byte boundary take the scalar-load form."""
    k, v = engine.gen_groupby(31, (1 << 20) + 5, 700, 0.5)
    ks, vs = slice(1, len(k) - 4), slice(3, len(v) - 2)  # equal lengths, offsets 4 and 12 bytes
    exp = oracle.groupby(k[ks], v[vs], threads=cpu_threads())
    dk, dv = dev(k), dev(v)
    assert dk[ks].numel() == dv[vs].numel() == len(k) - 5
    res = ctx.groupby(dk[ks], dv[vs], len(exp[0]), expected_groups=700, strategy=1)
    ctx.sync()
    got = sort_groups(*[host(t) for t in res[:5]], host(res[5])[0])
    for a, b in zip(got, exp):
        assert (a == b).all()


@pytest.mark.parametrize("card", [4, 12, 30, 60, 100, 300])
@pytest.mark.parametrize("theta", [0.0, 1.0])
def test_groupby_accumulator_columns(ctx, oracle, card, theta):
    """Group counts whose on-chip tables (16 x groups: 64 .. 4096 slots) take
    32, 16, 8, 4, 2 and 1 lane-indexed accumulator columns."""
    k, v = engine.gen_groupby(4000 + card + int(theta), (1 << 20) + 7, card, theta)
    check(ctx, oracle, k, v, expected_groups=card, strategy=1)
