"""gbj_join_agg_noalloc: the join + aggregate entry point for callers that may
not allocate device memory when they call (an engine whose buffer manager
already holds its memory, a fixed admission budget, a path that cannot pay
for cudaMalloc's implicit synchronisation).  It keeps its hash table in a
fixed array inside the library, so this file checks, through the C ABI, that
it returns exactly what the allocating path (gbj_join_build +
gbj_join_probe_agg) returns, on two calls in a row that reuse that array,
and that it refuses build sides larger than the array holds.

Collected last (file name) so a failure here comes after every other test."""
import ctypes as C

import numpy as np
import pytest

from gpu_util import dev, host
from proteus_gb300 import abi, engine

pytestmark = pytest.mark.gpu

AGGS = [
    (abi.AGG_COUNT, abi.VAL_ONE),
    (abi.AGG_SUM, abi.VAL_PRODUCT),
    (abi.AGG_MIN, abi.VAL_BUILD),
    (abi.AGG_MAX, abi.VAL_PROBE),
    (abi.AGG_SUM, abi.VAL_ROWID_XOR),
    (abi.AGG_SUM, abi.VAL_BUILD_KEY),
]


def noalloc(lib, bk, bp, pk, pp, aggs):
    import torch

    out = torch.full((len(aggs),), 7, dtype=torch.int64, device="cuda")
    arr = abi.aggs_array(aggs)
    stream = torch.cuda.current_stream().cuda_stream  # 0 = legacy default stream
    rc = lib.gbj_join_agg_noalloc(bk.data_ptr(), bp.data_ptr() if bp is not None else None,
                                  bk.numel(), pk.data_ptr(),
                                  pp.data_ptr() if pp is not None else None, pk.numel(), arr,
                                  len(aggs), out.data_ptr(), stream)
    if rc != abi.OK:
        raise abi.GbjError(rc, lib.gbj_last_error(None).decode())
    return out


def allocating(ctx, bk, bp, pk, pp, aggs):
    t = ctx.join_build(bk, bp)
    out = ctx.join_probe_agg(t, pk, pp, aggs)
    ctx.sync()
    r = host(out).tolist()
    t.destroy()
    return r


def test_noalloc_matches_allocating_path_twice(lib, ctx, oracle):
    # call 1: full-size plain join (2^20 build rows, the array's maximum)
    rk, rp = engine.gen_build_side(71, abi.NOALLOC_MAX_BUILD)
    sk, sp = engine.gen_probe_uniform(71, 1 << 22, abi.NOALLOC_MAX_BUILD)
    d = [dev(x) for x in (rk, rp, sk, sp)]
    got1 = host(noalloc(lib, *d, AGGS)).tolist()
    assert got1 == allocating(ctx, *d, AGGS)
    assert got1[0] == 1 << 22
    # call 2: a smaller build side with duplicate keys reuses the array the
    # first call left filled; results must not see the old table
    rng = np.random.default_rng(5)
    rk2 = rng.integers(0, 5000, 30000).astype(np.int32)
    rp2 = rng.integers(-1000, 1000, 30000).astype(np.int32)
    sk2 = rng.integers(-100, 6000, 200001).astype(np.int32)
    sp2 = rng.integers(-1000, 1000, 200001).astype(np.int32)
    d2 = [dev(x) for x in (rk2, rp2, sk2, sp2)]
    got2 = host(noalloc(lib, *d2, AGGS)).tolist()
    assert got2 == allocating(ctx, *d2, AGGS)
    # and against the CPU oracle (the reference's chained-hash semantics), so a
    # fault shared by both GPU paths cannot pass unseen
    assert got2 == oracle.join_agg(rk2, rp2, sk2, sp2, AGGS)
    # and the first join again, after the second one
    assert host(noalloc(lib, *d, AGGS)).tolist() == got1


def test_noalloc_rejects_oversize_build(lib):
    import torch

    big = torch.zeros(abi.NOALLOC_MAX_BUILD + 1, dtype=torch.int32, device="cuda")
    with pytest.raises(abi.GbjError) as e:
        noalloc(lib, big, None, big[:10], None, [(abi.AGG_COUNT, abi.VAL_ONE)])
    assert e.value.code == abi.ERR_CAPACITY
    assert "GBJ_NOALLOC_MAX_BUILD" in str(e.value)
