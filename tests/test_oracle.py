"""The oracle pinned against the reference: its golden outputs and its own
RJStepwise / partitionHT compiled from source (committed counts)."""
import hashlib

import numpy as np

import pytest

import datagen
from proteus_gb300 import abi, engine

COUNT1 = (abi.AGG_COUNT, abi.VAL_ONE)


def _col(golden, table, col):
    return np.array(golden["reference"]["tables"][table][col], dtype=np.int32)


def _case(golden, name):
    return next(c for c in golden["reference"]["cases"] if c["name"] == name)


def three_way_join_oracle(O, sailors_sid, reserves_sid, reserves_bid, boats_bid):
    """probe sailors x build reserves on sid, then x build boats on bid."""
    b1, p1 = O.join_pairs(reserves_sid, sailors_sid, hash_bits=16)
    bid = reserves_bid[b1]
    sid = sailors_sid[p1]
    b2, p2 = O.join_pairs(boats_bid, bid, hash_bits=16)
    return O.reduce(sid, [(abi.AGG_MAX, abi.VAL_PROBE), (abi.AGG_SUM, abi.VAL_PROBE), COUNT1],
                    rows=p2)


def test_sailors_join_left3(oracle, golden):
    exp = _case(golden, "sailorsJoinLeft3")["expected"]
    r = three_way_join_oracle(oracle, _col(golden, "sailors", "sid"),
                              _col(golden, "reserves", "sid"), _col(golden, "reserves", "bid"),
                              _col(golden, "boats", "bid"))
    assert r == [exp["max_sid"], exp["sum_sid"], exp["count"]]


def test_3way_join_other_build_side(oracle, golden):
    # tests-output.cpp: reserves probes, sailors builds
    exp = _case(golden, "3wayJoin")["expected"]
    s_sid, r_sid = _col(golden, "sailors", "sid"), _col(golden, "reserves", "sid")
    r_bid, b_bid = _col(golden, "reserves", "bid"), _col(golden, "boats", "bid")
    b1, p1 = oracle.join_pairs(s_sid, r_sid, hash_bits=4)
    bid, sid = r_bid[p1], s_sid[b1]
    b2, p2 = oracle.join_pairs(b_bid, bid, hash_bits=4)
    got = oracle.reduce(sid, [(abi.AGG_MAX, abi.VAL_PROBE), (abi.AGG_SUM, abi.VAL_PROBE), COUNT1],
                        rows=p2)
    assert got == [exp["max_sid"], exp["sum_sid"], exp["count"]]


def test_reduce_join_radix(oracle, golden):
    exp = _case(golden, "reduce-join")["expected"]
    s_sid, r_sid = _col(golden, "sailors", "sid"), _col(golden, "reserves", "sid")
    assert oracle.rj_stepwise(s_sid, r_sid) == exp["count"]
    assert oracle.radix_join_agg(s_sid, None, r_sid, None, [COUNT1], bits=2)[0] == exp["count"]


def test_groupby_reserves(oracle, golden):
    k, c, s, mn, mx = oracle.groupby(_col(golden, "reserves", "sid"),
                                     _col(golden, "reserves", "bid"), hash_bits=4)
    assert sorted(c.tolist()) == _case(golden, "nestReserves")["expected"]["counts"]
    assert sorted([int(a), int(b)] for a, b in zip(c, mx)) == \
        _case(golden, "multinestReserves")["expected"]["count_max"]


def test_groupby_lineitem_filtered(oracle, golden):
    ok = _col(golden, "lineitem10", "l_orderkey")
    sel = np.nonzero(ok < 4)[0]
    k, c, s, mn, mx = oracle.groupby(_col(golden, "lineitem10", "l_linenumber")[sel],
                                     _col(golden, "lineitem10", "l_quantity")[sel], hash_bits=4)
    assert sorted([int(a), int(b)] for a, b in zip(c, mx)) == \
        _case(golden, "nestBagTPCH")["expected"]["count_max"]


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.int32).tobytes()).hexdigest()[:16]


def _regen(case):
    rk, _ = engine.gen_build_side(case["seed"], case["n_build"], payload=False)
    if case["kind"] == "plain":
        sk, _ = engine.gen_probe_uniform(case["seed"], case["n_probe"], case["n_build"],
                                         payload=False)
    else:
        sk, _ = engine.gen_probe_zipf(case["seed"], case["n_probe"], case["n_build"],
                                      case["theta"], 0.5)
    return rk, sk


@pytest.mark.parametrize("i", range(7))
def test_rjstepwise_golden(lib, oracle, golden, i):
    case = golden["rjstepwise"]["cases"][i]
    rk, sk = _regen(case)
    # the generator reproduces the inputs the reference was run on
    assert _sha(rk) == case["build_sha"] and _sha(sk) == case["probe_sha"]
    m = case["rjstepwise_matches"]
    assert oracle.rj_stepwise(rk, sk) == m
    assert oracle.join_agg(rk, None, sk, None, [COUNT1])[0] == m
    assert oracle.radix_join_agg(rk, None, sk, None, [COUNT1], threads=4)[0] == m
    counts = oracle.partition_ht_counts(oracle.radix_cluster(rk, None, 0, 14, 0)[0])
    assert hashlib.sha256(counts.astype(np.int32).tobytes()).hexdigest()[:16] == \
        case["partition_ht_counts_sha"]


def test_radix_cluster_equals_reference_order(oracle):
    """Two stable passes (7 + 7 bits) reproduce partitionHT's order exactly."""
    if oracle.ref_lib() is None and not oracle.build_ref():
        pytest.skip("reference tree not present (oracle/_ref cannot be built here)")
    rk, _ = engine.gen_build_side(5, 50000, payload=False)
    counts, keys, rows = oracle.ref_partition_ht(rk)
    k1, p1, _ = oracle.radix_cluster(rk, None, 0, 7, 0)
    k2, p2, _ = oracle.radix_cluster(k1, p1, 7, 7, 0)
    assert (k2 == keys).all() and (p2 == rows).all()
    assert (oracle.partition_ht_counts(k2) == counts).all()


def test_planted_mistake_is_caught(oracle, golden):
    """A wrong oracle answer must fail the golden comparison."""
    case = golden["rjstepwise"]["cases"][0]
    rk, sk = _regen(case)
    sk = sk.copy()
    sk[0] = np.int32(-7)  # a probe key that cannot match: one match fewer
    assert oracle.rj_stepwise(rk, sk) == case["rjstepwise_matches"] - 1


def test_groupby_threads_agree(oracle):
    k, v = engine.gen_groupby(3, 200000, 5000, 1.0)
    a = oracle.groupby(k, v, threads=1)
    b = oracle.groupby(k, v, threads=8)
    for x, y in zip(a, b):
        assert (x == y).all()
    assert a[1].sum() == len(k)
    assert a[2].sum() == int(v.astype(np.int64).sum())


def _agg_keys(lib, c):
    import numpy as np

    span = int(c["span"])
    keys = np.array([int(datagen.load().gbj_gen_rand(c["seed"], 0x6A00, i)) % span for i in range(c["n"])], dtype=np.uint64)
    return keys.view(np.int64) - (np.int64(span // 2) if span < (1 << 63) else 0)


def test_partition_ht_agg_matches_reference_goldens(lib, oracle):
    """The int64-key twin of partitionHT (radix-aggr.cpp): the oracle's
    restatement reproduces the reference's counts and its stable clustered
    order on every committed case."""
    import hashlib
    import json
    import os

    import numpy as np

    with open(os.path.join(os.path.dirname(__file__), "golden", "partition_ht_agg_cases.json")) as f:
        cases = json.load(f)["cases"]
    for c in cases:
        keys = _agg_keys(lib, c)
        assert hashlib.sha256(keys.tobytes()).hexdigest()[:16] == c["keys_sha"]
        counts, _, rows = oracle.partition_ht_agg(keys)
        assert hashlib.sha256(counts.astype(np.int32).tobytes()).hexdigest()[:16] == c["counts_sha"]
        assert hashlib.sha256(rows.astype(np.int64).tobytes()).hexdigest()[:16] == c["clustered_rows_sha"]
        assert int((counts > 0).sum()) == c["nonempty"]


def _i64_keys(lib, seed, n, span, salt):
    import numpy as np

    keys = np.array([int(datagen.load().gbj_gen_rand(seed, salt, i)) % span for i in range(n)], dtype=np.uint64)
    return keys.view(np.int64) - (np.int64(span // 2) if span < (1 << 63) else 0)


def test_int64_twins_match_reference_goldens(lib, oracle):
    """The int64-key twins (radix-aggr.cpp): the oracle's RJStepwise count
    and its RadixNest group sizes reproduce the reference's own results on
    every committed case."""
    import hashlib
    import json
    import os

    import numpy as np

    with open(os.path.join(os.path.dirname(__file__), "golden", "nest_i64_cases.json")) as f:
        g = json.load(f)
    for c in g["joins"]:
        span = int(c["span"])
        rk = _i64_keys(lib, c["seed"], c["nr"], span, 0x6B00)
        sk = _i64_keys(lib, c["seed"], c["ns"], span, 0x6B01)
        assert hashlib.sha256(rk.tobytes()).hexdigest()[:16] == c["r_sha"]
        assert hashlib.sha256(sk.tobytes()).hexdigest()[:16] == c["s_sha"]
        assert oracle.join_count_i64(rk, sk) == c["matches"]
    for c in g["nests"]:
        keys = _i64_keys(lib, c["seed"], c["n"], int(c["span"]), 0x6B02)
        assert hashlib.sha256(keys.tobytes()).hexdigest()[:16] == c["keys_sha"]
        k, cnt, _, _, _ = oracle.nest_i64(keys)
        assert len(k) == c["groups"] and (np.diff(k) > 0).all()
        assert hashlib.sha256(cnt.astype(np.int64).tobytes()).hexdigest()[:16] == c["counts_sha"]
        assert int(cnt.max()) == c["max_count"]


def test_nest_i64_aggregates_against_numpy(oracle):
    """SUM (int64 wrap-around), MIN, MAX of the RadixNest restatement, with
    INT64_MIN / INT64_MAX keys and values."""
    import numpy as np

    rng = np.random.default_rng(9)
    i64 = np.iinfo(np.int64)
    k = rng.integers(-40, 40, 20000).astype(np.int64) * (1 << 50)
    k[::11] = i64.min
    k[::13] = i64.max
    v = rng.integers(i64.min, i64.max, 20000, dtype=np.int64)
    v[::7] = i64.max
    gk, gc, gs, gmn, gmx = oracle.nest_i64(k, v)
    uk, inv = np.unique(k, return_inverse=True)
    s = np.zeros(len(uk), dtype=np.uint64)
    np.add.at(s, inv, v.view(np.uint64))
    mn = np.full(len(uk), i64.max)
    np.minimum.at(mn, inv, v)
    mx = np.full(len(uk), i64.min)
    np.maximum.at(mx, inv, v)
    assert (gk == uk).all() and (gc == np.bincount(inv)).all()
    assert (gs == s.view(np.int64)).all() and (gmn == mn).all() and (gmx == mx).all()
    assert oracle.nest_i64(np.zeros(0, np.int64))[0].size == 0
    assert oracle.join_count_i64(np.zeros(0, np.int64), k) == 0


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_int64_twins_equal_reference_live(oracle, seed):
    """Fresh seeded int64 inputs (duplicates, keys sharing their low cluster
    bits, negative and extreme keys): the oracle's RJStepwise count and
    RadixNest group sizes equal the reference's own, run here."""
    if oracle.ref_lib() is None and not oracle.build_ref():
        pytest.skip("reference tree not present (oracle/_ref cannot be built here)")
    rng = np.random.default_rng(seed)
    i64 = np.iinfo(np.int64)
    base = rng.integers(i64.min, i64.max, 3000, dtype=np.int64)
    base[:40] = (base[:40] >> 14) << 14  # same low 14 bits: one cluster, long chains
    base[40] = i64.max
    r = base[rng.integers(0, len(base), 20000)]
    s = np.concatenate([base[rng.integers(0, len(base), 30000)],
                        rng.integers(i64.min, i64.max, 5000, dtype=np.int64)])
    assert oracle.join_count_i64(r, s) == oracle.ref_rj_stepwise_agg(r, s)
    k, cnt, _, _, _ = oracle.nest_i64(r)
    assert (cnt == oracle.ref_nest_counts(r, k)).all()
    assert int(cnt.sum()) == len(r)


def test_logical_accumulators(oracle):
    """or / and (LogOrMonoid / LogAndMonoid): truth of the operand, 0/1 result;
    identities false / true."""
    col = np.array([0, 3, 0, -1], dtype=np.int32)
    ops = [(abi.AGG_OR, abi.VAL_PROBE), (abi.AGG_AND, abi.VAL_PROBE)]
    assert oracle.reduce(col, ops) == [1, 0]
    assert oracle.reduce(col, ops, rows=np.array([1, 3], dtype=np.int32)) == [1, 1]
    assert oracle.reduce(col, ops, rows=np.array([0, 2], dtype=np.int32)) == [0, 0]
    assert oracle.reduce(col, ops, rows=np.zeros(0, dtype=np.int32)) == [0, 1]


def test_minor_key_join_brute_force(oracle):
    """The minor-key restatement against a nested-loop join on (key, minor)."""
    rng = np.random.default_rng(3)
    bk, bm = rng.integers(0, 40, 700).astype(np.int32), rng.integers(0, 3, 700).astype(np.int32)
    pk, pm = rng.integers(0, 45, 1500).astype(np.int32), rng.integers(0, 3, 1500).astype(np.int32)
    bp, pp = rng.integers(-9, 9, 700).astype(np.int32), rng.integers(-9, 9, 1500).astype(np.int32)
    aggs = [COUNT1, (abi.AGG_SUM, abi.VAL_PRODUCT), (abi.AGG_SUM, abi.VAL_ROWID_XOR),
            (abi.AGG_MIN, abi.VAL_BUILD_ROWID), (abi.AGG_AND, abi.VAL_PROBE)]
    exp = [0, 0, 0, np.iinfo(np.int64).max, 1]
    for j in range(len(pk)):
        for i in np.nonzero((bk == pk[j]) & (bm == pm[j]))[0]:
            exp[0] += 1
            exp[1] += int(bp[i]) * int(pp[j])
            exp[2] += int(i) ^ j
            exp[3] = min(exp[3], int(i))
            exp[4] &= int(pp[j] != 0)
    for threads in (1, 3):
        assert oracle.radix_join_agg_minor(bk, bm, bp, pk, pm, pp, aggs, bits=3, threads=threads) == exp


def test_join_i64_matches_brute_force_and_int32_join(oracle):
    """The int64 chained join: brute force on wide keys, and equal to the
    int32 join when every key fits 32 bits."""
    import collections

    rng = np.random.default_rng(21)
    aggs = [(0, 0), (1, 3), (1, 6), (3, 7), (2, 4)]
    rk = rng.integers(-(1 << 62), 1 << 62, 700).astype(np.int64)
    rk[::7] = rk[3]  # duplicates
    rp = rng.integers(-1000, 1000, len(rk)).astype(np.int32)
    sk = np.concatenate([rk[rng.integers(0, len(rk), 3000)], rk[:50] ^ (1 << 33)]).astype(np.int64)
    sp = rng.integers(-1000, 1000, len(sk)).astype(np.int32)
    rows = collections.defaultdict(list)
    for i, k in enumerate(rk.tolist()):
        rows[k].append(i)
    c = s = x = 0
    mx, mn = -(1 << 63), (1 << 63) - 1
    for j, k in enumerate(sk.tolist()):
        for i in rows.get(k, []):
            c += 1
            s += int(rp[i]) * int(sp[j])
            x += i ^ j
            mx = max(mx, k)
            mn = min(mn, i)
    assert oracle.join_agg_i64(rk, rp, sk, sp, aggs) == [c, s, x, mx, mn]
    b, p = oracle.join_pairs_i64(rk, sk)
    assert len(b) == c and all(rk[bi] == sk[pi] for bi, pi in zip(b.tolist(), p.tolist()))
    k32 = rng.integers(-5000, 5000, 4000).astype(np.int32)
    q32 = rng.integers(-6000, 6000, 9000).astype(np.int32)
    p32 = rng.integers(-100, 100, 4000).astype(np.int32)
    s32 = rng.integers(-100, 100, 9000).astype(np.int32)
    assert oracle.join_agg_i64(k32.astype(np.int64), p32, q32.astype(np.int64), s32, aggs) == \
        oracle.join_agg(k32, p32, q32, s32, aggs)
    # the placement hash is murmur3's 64-bit finaliser
    assert oracle.lib().orc_hash_int64(1) == 0xB456BCFC34C2CB2C
