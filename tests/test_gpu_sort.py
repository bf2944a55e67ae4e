"""ORDER BY an int32 key on the GPU: the same order as a stable sort
(ties keep input order), all columns carried along."""
import numpy as np
import pytest

from gpu_util import dev, host
from proteus_gb300 import abi, engine

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,lo,hi", [(1, 0, 10), (2049, -5, 5), ((1 << 20) + 7, -(1 << 31), 1 << 31),
                                     ((1 << 22) + 1, 0, 1000)])
@pytest.mark.parametrize("desc", [False, True])
def test_sort_stable(ctx, n, lo, hi, desc):
    rng = np.random.default_rng(n + desc)
    key = rng.integers(lo, hi, n, dtype=np.int64).astype(np.int32)
    key[::13] = np.iinfo(np.int32).min
    key[::17] = np.iinfo(np.int32).max
    pay = np.arange(n, dtype=np.int32)
    other = rng.integers(-100, 100, n).astype(np.int32)
    out = ctx.sort_by_key([dev(pay), dev(key), dev(other)], key_col=1, descending=desc)
    ctx.sync()
    order = np.argsort(-key.astype(np.int64) if desc else key, kind="stable")
    assert (host(out[1]) == key[order]).all()
    assert (host(out[0]) == pay[order]).all()
    assert (host(out[2]) == other[order]).all()


def test_sort_groupby_output(ctx, oracle):
    """ORDER BY on a group-by's output gives the oracle's key order."""
    k, v = engine.gen_groupby(8, 1 << 22, 1 << 16, 0.0)
    res = ctx.groupby(dev(k), dev(v), (1 << 16) + 16, expected_groups=1 << 16)
    ctx.sync()
    n = int(host(res[5])[0])
    cnt32 = res[1][:n].to(dtype=__import__("torch").int32)
    out = ctx.sort_by_key([res[0][:n].contiguous(), cnt32.contiguous(), res[3][:n].contiguous()], 0)
    ctx.sync()
    ek, ec, _, emn, _ = oracle.groupby(k, v)
    assert (host(out[0]) == ek).all() and (host(out[1]) == ec).all() and (host(out[2]) == emn).all()


def test_sort_errors(ctx):
    with pytest.raises(abi.GbjError):
        ctx.sort_by_key([dev(np.arange(4, dtype=np.int32))], key_col=2)
