"""Bloom-filter semi-join pre-filter vs the oracle's restatement of the
reference's filter (exactly the same passing rows), and the star-join use:
filtering the fact side by a dimension's selected keys keeps every match."""
import numpy as np
import pytest

from gpu_util import dev, host
from proteus_gb300 import abi

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("filter_size", [32, 1 << 10, 1 << 20, 1 << 24])
def test_bloom_matches_oracle(ctx, oracle, filter_size):
    rng = np.random.default_rng(filter_size)
    build = rng.integers(-(1 << 31), 1 << 31, 50000, dtype=np.int64).astype(np.int32)
    probe = np.concatenate([build[:20000], rng.integers(-(1 << 31), 1 << 31, (1 << 20) - 20000,
                                                        dtype=np.int64).astype(np.int32)])
    rng.shuffle(probe)
    probe[::97] = np.iinfo(np.int32).min
    f = ctx.bloom_build(dev(build), filter_size)
    rows, cnt = ctx.bloom_probe(f, dev(probe))
    ctx.sync()
    n = int(host(cnt)[0])
    exp = oracle.bloom_semijoin(build, probe, filter_size)
    assert n == len(exp)
    assert (host(rows)[:n] == exp).all()
    # no false negatives: every probe row whose key is a build key passes
    keep = np.zeros(len(probe), bool)
    keep[host(rows)[:n]] = True
    assert keep[np.isin(probe, build)].all()
    ctx.bloom_destroy(f)


def test_bloom_edges(ctx):
    import torch

    e = torch.empty(0, dtype=torch.int32, device="cuda")
    f = ctx.bloom_build(e, 64)
    rows, cnt = ctx.bloom_probe(f, dev(np.arange(100, dtype=np.int32)))
    ctx.sync()
    assert int(host(cnt)[0]) == 0
    rows, cnt = ctx.bloom_probe(f, e)
    ctx.sync()
    assert int(host(cnt)[0]) == 0
    ctx.bloom_destroy(f)
    with pytest.raises(abi.GbjError):
        ctx.bloom_build(e, 1000)  # not a power of two
