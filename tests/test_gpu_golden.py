"""The reference's own test cases (sailors / reserves / boats / lineitem)
through the GPU path, against the reference's golden outputs."""
import numpy as np
import pytest

from gpu_util import dev, host, sort_groups
from proteus_gb300 import abi

pytestmark = pytest.mark.gpu

REDUCE3 = [(abi.AGG_MAX, abi.VAL_PROBE), (abi.AGG_SUM, abi.VAL_PROBE),
           (abi.AGG_COUNT, abi.VAL_ONE)]


def col(golden, t, c):
    return np.array(golden["reference"]["tables"][t][c], dtype=np.int32)


def case(golden, name):
    return next(c for c in golden["reference"]["cases"] if c["name"] == name)["expected"]


def join_rows(ctx, build_keys, probe_keys, hash_bits, max_build, probe_rows=None):
    t = ctx.join_build(build_keys, hash_bits=hash_bits, max_build=max_build)
    b, p, cnt = ctx.join_probe_pairs(t, probe_keys, capacity=4096, probe_rows=probe_rows)
    ctx.sync()
    m = int(host(cnt)[0])
    return b[:m], p[:m]


def test_sailors_join_left3(ctx, golden):
    exp = case(golden, "sailorsJoinLeft3")
    s_sid = dev(col(golden, "sailors", "sid"))
    r_sid, r_bid = dev(col(golden, "reserves", "sid")), dev(col(golden, "reserves", "bid"))
    b_bid = dev(col(golden, "boats", "bid"))
    rrow, srow = join_rows(ctx, r_sid, s_sid, 16, 128)     # sailors probes reserves
    bid = ctx.gather(r_bid, rrow)
    sid = ctx.gather(s_sid, srow)
    brow, prow = join_rows(ctx, b_bid, bid, 16, 128)      # then probes boats
    out = ctx.reduce(sid, REDUCE3, rows=prow)
    ctx.sync()
    assert host(out).tolist() == [exp["max_sid"], exp["sum_sid"], exp["count"]]


def test_3way_join(ctx, golden):
    exp = case(golden, "3wayJoin")
    s_sid = dev(col(golden, "sailors", "sid"))
    r_sid, r_bid = dev(col(golden, "reserves", "sid")), dev(col(golden, "reserves", "bid"))
    b_bid = dev(col(golden, "boats", "bid"))
    srow, rrow = join_rows(ctx, s_sid, r_sid, 4, 16)      # reserves probes sailors
    bid = ctx.gather(r_bid, rrow)
    sid = ctx.gather(s_sid, srow)
    brow, prow = join_rows(ctx, b_bid, bid, 4, 16)
    out = ctx.reduce(sid, REDUCE3, rows=prow)
    ctx.sync()
    assert host(out).tolist() == [exp["max_sid"], exp["sum_sid"], exp["count"]]


def test_reduce_join_radix(ctx, golden):
    exp = case(golden, "reduce-join")
    out = ctx.radix_join_agg(dev(col(golden, "sailors", "sid")), None,
                             dev(col(golden, "reserves", "sid")), None,
                             [(abi.AGG_COUNT, abi.VAL_ONE)])
    ctx.sync()
    assert host(out).tolist() == [exp["count"]]


@pytest.mark.parametrize("strategy", [1, 2])
def test_groupby_reserves(ctx, golden, strategy):
    res = ctx.groupby(dev(col(golden, "reserves", "sid")), dev(col(golden, "reserves", "bid")),
                      16, max_input_size=16, hash_bits=4, strategy=strategy)
    ctx.sync()
    k, c, s, mn, mx = sort_groups(*[host(t) for t in res[:5]], host(res[5])[0])
    assert sorted(c.tolist()) == case(golden, "nestReserves")["counts"]
    assert sorted([int(a), int(b)] for a, b in zip(c, mx)) == \
        case(golden, "multinestReserves")["count_max"]


def test_groupby_lineitem_filtered(ctx, golden):
    okey = dev(col(golden, "lineitem10", "l_orderkey"))
    rows, cnt = ctx.select_range(okey, np.iinfo(np.int32).min, 3)   # l_orderkey < 4
    ctx.sync()
    rows = rows[: int(host(cnt)[0])]
    ln = ctx.gather(dev(col(golden, "lineitem10", "l_linenumber")), rows)
    qty = ctx.gather(dev(col(golden, "lineitem10", "l_quantity")), rows)
    res = ctx.groupby(ln, qty, 16, max_input_size=16, hash_bits=4)
    ctx.sync()
    k, c, s, mn, mx = sort_groups(*[host(t) for t in res[:5]], host(res[5])[0])
    assert sorted([int(a), int(b)] for a, b in zip(c, mx)) == \
        case(golden, "nestBagTPCH")["count_max"]
