"""Radix partitioning and the partitioned join on the GPU vs the oracle."""
import numpy as np
import pytest

from gpu_util import CONFIG1_AGGS, CONFIG2_AGGS, cpu_threads, dev, host
from proteus_gb300 import abi, engine

pytestmark = pytest.mark.gpu


def canonical_partitions(keys, payload, offsets):
    """Each partition's tuples sorted, so unordered partitions compare."""
    out = []
    for p in range(len(offsets) - 1):
        a, b = int(offsets[p]), int(offsets[p + 1])
        kk, pp = keys[a:b], payload[a:b]
        o = np.lexsort((pp, kk))
        out.append((kk[o], pp[o]))
    return out


@pytest.mark.parametrize("n,bits,digit,shift,with_payload", [
    (1 << 16, 1, abi.DIGIT_HASH, 0, True),
    (100003, 7, abi.DIGIT_KEY, 0, False),
    (1 << 18, 13, abi.DIGIT_HASH, 0, True),
    (1 << 18, 15, abi.DIGIT_HASH, 0, False),
    (50000, 7, abi.DIGIT_KEY, 7, True),
    (3, 4, abi.DIGIT_HASH, 0, True),
])
def test_partition_matches_radix_cluster(ctx, oracle, n, bits, digit, shift, with_payload):
    rng = np.random.default_rng(n + bits)
    keys = rng.integers(np.iinfo(np.int32).min, np.iinfo(np.int32).max, n, dtype=np.int64)
    keys = keys.astype(np.int32)
    pay = rng.integers(-10**6, 10**6, n).astype(np.int32) if with_payload else None
    ok, op, off = ctx.partition(dev(keys), dev(pay) if pay is not None else None, bits,
                                shift=shift, digit=digit)
    ctx.sync()
    ek, ep, eoff = oracle.radix_cluster(keys, pay, shift, bits, digit == abi.DIGIT_HASH)
    got_off = host(off).astype(np.uint64)
    assert (got_off == eoff).all()
    a = canonical_partitions(host(ok), host(op), got_off)
    b = canonical_partitions(ek, ep, eoff)
    for (k1, p1), (k2, p2) in zip(a, b):
        assert (k1 == k2).all() and (p1 == p2).all()


def test_partition_empty_and_invalid(ctx):
    import torch

    e = torch.zeros(0, dtype=torch.int32, device="cuda")
    ok, op, off = ctx.partition(e, e, 5)
    ctx.sync()
    assert (host(off) == 0).all()
    with pytest.raises(abi.GbjError):
        ctx.partition(dev(np.arange(10, dtype=np.int32)), None, 16)


@pytest.mark.parametrize("block", [512, 1024])
@pytest.mark.parametrize("theta", [0.0, 0.5, 1.0])
@pytest.mark.parametrize("nr,ns", [(1 << 12, 1 << 16), (1 << 18, 1 << 21)])
def test_radix_join_zipf(ctx, oracle, theta, nr, ns, block):
    rk, _ = engine.gen_build_side(31, nr, payload=False)
    sk, _ = engine.gen_probe_zipf(31, ns, nr, theta, 0.5)
    out = ctx.radix_join_agg(dev(rk), None, dev(sk), None, CONFIG2_AGGS, block=block)
    ctx.sync()
    exp = oracle.radix_join_agg(rk, None, sk, None, CONFIG2_AGGS, threads=cpu_threads())
    assert host(out).tolist() == exp
    assert exp[0] == oracle.rj_stepwise(rk, sk)


def test_radix_join_payload_aggregates(ctx, oracle):
    rk, rp = engine.gen_build_side(7, 1 << 16)
    sk, sp = engine.gen_probe_uniform(7, 1 << 20, 1 << 16)
    aggs = CONFIG1_AGGS + [(abi.AGG_MIN, abi.VAL_BUILD), (abi.AGG_MAX, abi.VAL_PROBE),
                           (abi.AGG_SUM, abi.VAL_BUILD_KEY)]
    out = ctx.radix_join_agg(dev(rk), dev(rp), dev(sk), dev(sp), aggs)
    ctx.sync()
    assert host(out).tolist() == oracle.join_agg(rk, rp, sk, sp, aggs, threads=cpu_threads())


@pytest.mark.parametrize("block", [512, 1024])
def test_radix_join_heavy_duplicates(ctx, oracle, block):
    """A build partition larger than the on-chip table is split into chunks."""
    rng = np.random.default_rng(3)
    rk = np.concatenate([np.full(30000, 77, dtype=np.int32),
                         rng.integers(0, 1 << 20, 100000).astype(np.int32)])
    sk = np.concatenate([np.full(500, 77, dtype=np.int32),
                         rng.integers(0, 1 << 20, 200000).astype(np.int32)])
    out = ctx.radix_join_agg(dev(rk), None, dev(sk), None, CONFIG2_AGGS, bits=4, block=block)
    ctx.sync()
    assert host(out).tolist() == oracle.join_agg(rk, None, sk, None, CONFIG2_AGGS)


@pytest.mark.parametrize("bits", [1, 6, 13, 15])
def test_radix_join_explicit_bits(ctx, oracle, bits):
    rk, _ = engine.gen_build_side(4, 50000, payload=False)
    sk, _ = engine.gen_probe_zipf(4, 300000, 50000, 1.0, 0.7)
    out = ctx.radix_join_agg(dev(rk), None, dev(sk), None, CONFIG2_AGGS, bits=bits)
    ctx.sync()
    assert host(out).tolist() == oracle.join_agg(rk, None, sk, None, CONFIG2_AGGS)


def test_radix_join_payload_and_rowid_on_one_side(ctx, oracle):
    """A side read both as payload and as row id runs in row mode."""
    rng = np.random.default_rng(8)
    rk = rng.integers(0, 3000, 20000).astype(np.int32)
    rp = rng.integers(-10**6, 10**6, 20000).astype(np.int32)
    sk = rng.integers(-10, 3100, 70001).astype(np.int32)
    sp = rng.integers(-10**6, 10**6, 70001).astype(np.int32)
    aggs = [(abi.AGG_SUM, abi.VAL_BUILD), (abi.AGG_SUM, abi.VAL_BUILD_ROWID),
            (abi.AGG_MAX, abi.VAL_PRODUCT), (abi.AGG_SUM, abi.VAL_ROWID_XOR),
            (abi.AGG_MIN, abi.VAL_PROBE), (abi.AGG_COUNT, abi.VAL_ONE)]
    out = ctx.radix_join_agg(dev(rk), dev(rp), dev(sk), dev(sp), aggs)
    ctx.sync()
    assert host(out).tolist() == oracle.join_agg(rk, rp, sk, sp, aggs)


@pytest.mark.parametrize("n_build,n_probe,bits", [(30000, 200003, 0), (1 << 18, 1 << 20, 12),
                                                  (5000, 40000, 3)])
def test_radix_join_minor_key(ctx, oracle, n_build, n_probe, bits):
    """Composite keys: the major key repeats, the minor key tells rows apart
    (build_k_minor / probe_k_minor)."""
    rng = np.random.default_rng(n_build + bits)
    bk = rng.integers(0, n_build // 8 + 1, n_build).astype(np.int32)
    bm = rng.integers(0, 8, n_build).astype(np.int32)
    bp = rng.integers(-1000, 1000, n_build).astype(np.int32)
    pk = rng.integers(0, n_build // 8 + 40, n_probe).astype(np.int32)
    pm = rng.integers(0, 9, n_probe).astype(np.int32)
    pp = rng.integers(-1000, 1000, n_probe).astype(np.int32)
    aggs = [(abi.AGG_COUNT, abi.VAL_ONE), (abi.AGG_SUM, abi.VAL_PRODUCT),
            (abi.AGG_SUM, abi.VAL_ROWID_XOR), (abi.AGG_MAX, abi.VAL_BUILD),
            (abi.AGG_MIN, abi.VAL_PROBE), (abi.AGG_OR, abi.VAL_BUILD_KEY),
            (abi.AGG_AND, abi.VAL_PROBE)]
    out = ctx.radix_join_agg_minor(dev(bk), dev(bm), dev(bp), dev(pk), dev(pm), dev(pp), aggs,
                                   bits=bits)
    ctx.sync()
    exp = oracle.radix_join_agg_minor(bk, bm, bp, pk, pm, pp, aggs, threads=cpu_threads())
    assert host(out).tolist() == exp
    # the minor key removes matches the major key alone would count
    major = oracle.radix_join_agg(bk, None, pk, None, aggs[:1], threads=cpu_threads())
    assert exp[0] < major[0]


def test_radix_join_minor_key_needs_both_sides(ctx):
    e = dev(np.arange(10, dtype=np.int32))
    with pytest.raises(abi.GbjError) as err:
        ctx.radix_join_agg_minor(e, e, None, e, None, None, [(abi.AGG_COUNT, abi.VAL_ONE)])
    assert err.value.code == abi.ERR_INVALID


@pytest.mark.parametrize("kw", [dict(block=256), dict(passes=3), dict(passes=1, bits=9),
                                dict(passes=2, bits=1), dict(bits=16)])
def test_radix_params_refused(ctx, kw):
    """Parameters the join cannot honour are refused, never ignored."""
    rk, _ = engine.gen_build_side(1, 1000, payload=False)
    with pytest.raises(abi.GbjError) as e:
        ctx.radix_join_agg(dev(rk), None, dev(rk), None, CONFIG2_AGGS, **kw)
    assert e.value.code == abi.ERR_UNSUPPORTED


@pytest.mark.parametrize("passes,bits,block", [(1, 0, 0), (1, 6, 1024), (2, 4, 512), (2, 0, 512),
                                               (0, 9, 1024), (0, 13, 512)])
def test_radix_params_passes_honoured(ctx, oracle, passes, bits, block):
    rk, _ = engine.gen_build_side(4, 1 << 16, payload=False)
    sk, _ = engine.gen_probe_zipf(4, 1 << 19, 1 << 16, 0.5, 0.5)
    out = ctx.radix_join_agg(dev(rk), None, dev(sk), None, CONFIG2_AGGS, bits=bits, passes=passes,
                             block=block)
    ctx.sync()
    assert host(out).tolist() == oracle.radix_join_agg(rk, None, sk, None, CONFIG2_AGGS,
                                                       threads=cpu_threads())


def test_radix_join_empty(ctx, oracle):
    rk, _ = engine.gen_build_side(1, 1000, payload=False)
    e = np.zeros(0, dtype=np.int32)
    out = ctx.radix_join_agg(dev(e), None, dev(rk), None, CONFIG2_AGGS)
    ctx.sync()
    assert host(out).tolist() == [0, 0]


@pytest.mark.parametrize("theta", [0.0, 0.5, 1.0])
def test_radix_join_full_config(ctx, oracle, theta):
    """R = 2^27 unique keys, S = 2^29 (50% hits, Zipf theta): full size."""
    nr, ns = 1 << 27, 1 << 29
    rk, _ = engine.gen_build_side(1000 + int(theta * 10), nr, payload=False)
    sk, _ = engine.gen_probe_zipf(1000 + int(theta * 10), ns, nr, theta, 0.5)
    drk, dsk = dev(rk), dev(sk)
    out = ctx.radix_join_agg(drk, None, dsk, None, CONFIG2_AGGS)
    ctx.sync()
    got = host(out).tolist()
    del drk, dsk
    exp = oracle.radix_join_agg(rk, None, sk, None, CONFIG2_AGGS, threads=cpu_threads())
    assert got == exp
    # hits are ~50% of the probe side and every hit matches exactly once
    assert abs(got[0] / ns - 0.5) < 0.001


def test_stream_ordering_with_torch(ctx, oracle):
    """Library kernels run on torch's current stream: async host->device
    copies before the call and the read-back after it need no library sync."""
    import torch

    rk, _ = engine.gen_build_side(12, 1 << 20, payload=False)
    sk, _ = engine.gen_probe_zipf(12, 1 << 23, 1 << 20, 0.5, 0.5)
    h_r, h_s = torch.from_numpy(rk).pin_memory(), torch.from_numpy(sk).pin_memory()
    d_r = torch.empty_like(h_r, device="cuda")
    d_s = torch.empty_like(h_s, device="cuda")
    exp = oracle.radix_join_agg(rk, None, sk, None, CONFIG2_AGGS, threads=cpu_threads())
    for _ in range(3):
        d_r.fill_(0)
        d_s.fill_(0)
        d_r.copy_(h_r, non_blocking=True)
        d_s.copy_(h_s, non_blocking=True)
        out = ctx.radix_join_agg(d_r, None, d_s, None, CONFIG2_AGGS)
        assert out.cpu().tolist() == exp
    with torch.cuda.stream(torch.cuda.Stream()):
        d_s.copy_(h_s, non_blocking=True)
        out = ctx.radix_join_agg(d_r, None, d_s, None, CONFIG2_AGGS)
        got = out.cpu().tolist()
    assert got == exp


def _fmix32_inv(h):
    """Inverse of murmur3's fmix32 on 32-bit values."""
    m = (1 << 32) - 1
    h ^= h >> 16
    h = (h * 0x7ED1B41D) & m
    h ^= (h >> 13) ^ (h >> 26)
    h = (h * 0xA5CB9243) & m
    h ^= h >> 16
    return h


@pytest.mark.parametrize("bits", [0, 3, 14])
def test_radix_join_extreme_keys(ctx, oracle, bits):
    """Keys at the int32 extremes, and the key whose fmix32 equals the
    on-chip table's empty marker (0x80000000), which the partitioned tuples
    carry as their hash: every one matches exactly like any other key, and
    an aggregate reading the key gets it back unhashed."""
    special = _fmix32_inv(0x80000000)
    special = special - (1 << 32) if special >= 1 << 31 else special
    rng = np.random.default_rng(bits + 5)
    extremes = np.array([np.iinfo(np.int32).min, np.iinfo(np.int32).max, -1, 0, 1, special], np.int32)
    rk = np.concatenate([extremes, extremes[[0, 5]],
                         rng.integers(-(1 << 31), 1 << 31, 40000).astype(np.int32)])
    rp = rng.integers(-1000, 1000, len(rk)).astype(np.int32)
    sk = np.concatenate([np.repeat(extremes, 3), rng.choice(rk, 100000),
                         rng.integers(-(1 << 31), 1 << 31, 20000).astype(np.int32)])
    sp = rng.integers(-1000, 1000, len(sk)).astype(np.int32)
    aggs = [(abi.AGG_COUNT, abi.VAL_ONE), (abi.AGG_SUM, abi.VAL_BUILD_KEY),
            (abi.AGG_MIN, abi.VAL_BUILD_KEY), (abi.AGG_MAX, abi.VAL_BUILD_KEY),
            (abi.AGG_SUM, abi.VAL_PRODUCT)]
    out = ctx.radix_join_agg(dev(rk), dev(rp), dev(sk), dev(sp), aggs, bits=bits)
    ctx.sync()
    assert host(out).tolist() == oracle.join_agg(rk, rp, sk, sp, aggs)
