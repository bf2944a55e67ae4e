"""Hash rearrange (HashRearrange semantics) on the GPU: every row in the
bucket the reference's hash puts it in, bucket-major, nothing lost."""
import numpy as np
import pytest

from gpu_util import dev, host
from proteus_gb300 import abi, engine

pytestmark = pytest.mark.gpu


def ref_hash(keys):
    """The expression hasher's 64-bit hash of int32 keys (wrapping uint64)."""
    h = keys.astype(np.int64).view(np.uint64)
    with np.errstate(over="ignore"):
        h = h ^ (h >> np.uint64(16))
        h = h * np.uint64(0x85EBCA6B)
        h = h ^ (h >> np.uint64(13))
        h = h * np.uint64(0xC2B2AE35)
        h = h ^ (h >> np.uint64(16))
    return h


def test_ref_hash_matches_oracle(oracle):
    ks = np.array([0, 1, -1, 7, 123456789, np.iinfo(np.int32).min, np.iinfo(np.int32).max], dtype=np.int32)
    L = oracle.lib()
    assert ref_hash(ks).tolist() == [L.orc_hash_int32(int(k)) for k in ks]


@pytest.mark.parametrize("buckets", [1, 7, 64, 1000, 32768])
def test_rearrange(ctx, buckets):
    rng = np.random.default_rng(buckets)
    n = (1 << 20) + 3
    cols = [rng.integers(-(1 << 31), 1 << 31, n, dtype=np.int64).astype(np.int32) for _ in range(3)]
    cols[1][::11] = np.iinfo(np.int32).min
    outs, off = ctx.hash_rearrange([dev(c) for c in cols], key_col=1, num_buckets=buckets)
    ctx.sync()
    off = host(off)
    outs = [host(o) for o in outs]
    b = (ref_hash(cols[1]) % np.uint64(buckets)).astype(np.int64)
    assert off[0] == 0 and off[-1] == n
    assert (np.diff(off) == np.bincount(b, minlength=buckets)).all()
    rows_in = np.stack(cols, axis=1)
    rows_out = np.stack(outs, axis=1)
    for bk in np.unique(rng.integers(0, buckets, 12)):
        got = rows_out[off[bk]:off[bk + 1]]
        exp = rows_in[b == bk]
        assert sorted(map(tuple, got)) == sorted(map(tuple, exp))
    # every row exactly once overall
    for j in range(3):
        assert np.sort(outs[j]).tolist() == np.sort(cols[j]).tolist()


def test_rearrange_edges(ctx):
    import torch

    empty = torch.empty(0, dtype=torch.int32, device="cuda")
    outs, off = ctx.hash_rearrange([empty], 0, 5)
    ctx.sync()
    assert host(off).tolist() == [0] * 6
    with pytest.raises(abi.GbjError):
        ctx.hash_rearrange([dev(np.arange(10, dtype=np.int32))], 0, 1 << 16)
    with pytest.raises(abi.GbjError):
        ctx.hash_rearrange([dev(np.arange(10, dtype=np.int32))], 1, 4)
