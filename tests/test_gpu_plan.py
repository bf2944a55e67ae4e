"""Plan façade on the GPU: the reference's golden cases as plans, and larger
plans (fused reduce over joins, materialised joins, select, group-by) against
the oracle."""
import numpy as np
import pytest

import plan_cases
from gpu_util import cpu_threads, dev
from proteus_gb300 import abi, engine
from proteus_gb300.plan import Catalog, RelBuilder, cast64, col, lit

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cat(ctx, golden):
    c = Catalog(ctx)
    t = golden["reference"]["tables"]
    for rel, name in ((plan_cases.S, "sailors"), (plan_cases.R, "reserves"), (plan_cases.B, "boats"),
                      (plan_cases.L, "lineitem10")):
        for attr, vals in t[name].items():
            c.add(rel, attr, dev(np.array(vals, dtype=np.int32)))
    yield c
    c.close()


def expected(golden, name):
    return next(c for c in golden["reference"]["cases"] if c["name"] == name)["expected"]


@pytest.mark.parametrize("name", ["sailorsJoinLeft3", "3wayJoin"])
def test_golden_join_reduce(cat, golden, name):
    out = cat.execute(plan_cases.ALL[name]())
    exp = expected(golden, name)
    assert [int(v[0]) for v in out.values()] == [exp["max_sid"], exp["sum_sid"], exp["count"]]


def test_golden_radix_join_count(cat, golden):
    out = cat.execute(plan_cases.reduce_join())
    assert int(list(out.values())[0][0]) == expected(golden, "reduce-join")["count"]


def test_golden_nest_reserves(cat, golden):
    out = cat.execute(plan_cases.nest_reserves())
    assert sorted(out["sum_0"].tolist()) == expected(golden, "nestReserves")["counts"]


@pytest.mark.parametrize("name", ["multinestReserves", "nestBagTPCH"])
def test_golden_groupby_count_max(cat, golden, name):
    out = cat.execute(plan_cases.ALL[name]())
    got = sorted(zip(out["sum_0"].tolist(), out["max_1"].tolist()))
    assert [list(x) for x in got] == expected(golden, name)["count_max"]


@pytest.fixture(scope="module")
def big(ctx):
    """Config-1 shaped relations: R 2^16 permuted keys, S 2^20 uniform keys."""
    bk, bp = engine.gen_build_side(101, 1 << 16)
    pk, pp = engine.gen_probe_uniform(102, 1 << 20, 1 << 16)
    c = Catalog(ctx)
    for a, v in (("k", bk), ("p", bp)):
        c.add("R", a, dev(v))
    for a, v in (("k", pk), ("p", pp)):
        c.add("S", a, dev(v))
    yield c, bk, bp, pk, pp
    c.close()


@pytest.mark.parametrize("kind", ["hashjoin-chained", "partitioned", "join"])
def test_fused_reduce_over_join(big, oracle, kind):
    c, bk, bp, pk, pp = big
    s, r = RelBuilder.scan("S", ["k", "p"]), RelBuilder.scan("R", ["k", "p"])
    if kind == "hashjoin-chained":
        j = s.join(r, col("R", "k"), col("S", "k"), 17, 1 << 16)
    elif kind == "partitioned":
        j = s.partitioned_join(r, col("R", "k"), col("S", "k"), 1 << 16, 1 << 20)
    else:
        j = r.radix_join(s, col("R", "k"), col("S", "k"))
    plan = j.reduce([lit(1), cast64(col("R", "p") * col("S", "p")), col("S", "p"), col("R", "p")],
                    ["sum", "sum", "max", "min"])
    out = [int(v[0]) for v in c.execute(plan).values()]
    exp = oracle.join_agg(bk, bp, pk, pp, [(abi.AGG_COUNT, abi.VAL_ONE), (abi.AGG_SUM, abi.VAL_PRODUCT),
                                           (abi.AGG_MAX, abi.VAL_PROBE), (abi.AGG_MIN, abi.VAL_BUILD)],
                          threads=cpu_threads())
    assert out == list(exp)


def test_select_join_groupby(big, oracle):
    """select on both sides, materialised join, group-by on the join output."""
    c, bk, bp, pk, pp = big
    s = RelBuilder.scan("S", ["k", "p"]).filter((col("S", "p") >= 100) & (col("S", "p") < 700))
    r = RelBuilder.scan("R", ["k", "p"]).filter(col("R", "k") <= 40000)
    j = s.join(r, col("R", "k"), col("S", "k"))
    g = j.groupby([col("R", "p")], [(lit(1), "sum"), (col("S", "p"), "sum"), (col("S", "p"), "max")],
                  10, 1 << 20)
    out = c.execute(g)
    smask = (pp >= 100) & (pp < 700)
    rmask = bk <= 40000
    bpos = np.full(1 << 17, -1, dtype=np.int64)
    bpos[bk[rmask]] = np.nonzero(rmask)[0]
    sk, sp = pk[smask], pp[smask]
    hit = bpos[sk] >= 0
    gk = bp[bpos[sk[hit]]]
    ek, ec, es, _, emx = oracle.groupby(gk, sp[hit], threads=cpu_threads())
    assert out["p"].tolist() == ek.tolist()
    assert out["sum_0"].tolist() == ec.tolist()
    assert out["sum_1"].tolist() == es.tolist()
    assert out["max_2"].tolist() == emx.tolist()


def test_unknown_relation_and_unsupported(cat):
    with pytest.raises(abi.GbjError) as e:
        cat.execute(RelBuilder.scan("nope", ["x"]).reduce([lit(1)], ["sum"]))
    assert e.value.code == abi.ERR_INVALID and "nope" in str(e.value)
    p = plan_cases.nest_reserves().node
    p["k"].append(p["k"][0])  # two keys
    with pytest.raises(abi.GbjError) as e:
        cat.execute(p)
    assert e.value.code == abi.ERR_UNSUPPORTED


def test_cpp_relbuilder_executes(golden, tmp_path):
    """The C++ builder's PreparedStatement::execute on the reference's fixtures."""
    import subprocess

    import cpp_build

    t = golden["reference"]["tables"]
    lines = []
    for rel, name in ((plan_cases.S, "sailors"), (plan_cases.R, "reserves"), (plan_cases.B, "boats"),
                      (plan_cases.L, "lineitem10")):
        for attr, vals in t[name].items():
            lines.append(" ".join([rel, attr] + [str(v) for v in vals]))
    tables = tmp_path / "tables.txt"
    tables.write_text("\n".join(lines) + "\n")
    exe = cpp_build.build_driver(tmp_path)
    out = subprocess.run([exe, "run", str(tables)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    res = {}
    for ln in out.stdout.strip().split("\n"):
        name, *cols = ln.split(" ")
        res[name] = {c.split("=")[0]: [int(x) for x in c.split("=")[1].split(",") if x] for c in cols}
    e = expected(golden, "sailorsJoinLeft3")
    r = res["sailorsJoinLeft3"]
    assert [r["max_0"][0], r["sum_1"][0], r["sum_2"][0]] == [e["max_sid"], e["sum_sid"], e["count"]]
    for name in ("multinestReserves", "nestBagTPCH"):
        got = sorted(zip(res[name]["sum_0"], res[name]["max_1"]))
        assert [list(x) for x in got] == expected(golden, name)["count_max"]


def test_sort_over_groupby_and_relation(cat, golden, big):
    # ORDER BY over a group-by (host-ordered aggregate result)
    out = cat.execute(plan_cases.multinest_reserves().sort([(col(plan_cases.R, "sid"), "DESC")]))
    assert out["sid"].tolist() == sorted(out["sid"].tolist(), reverse=True)
    # ORDER BY over a relation (device sort), two keys, stable
    c, bk, bp, pk, pp = big
    plan = (RelBuilder.scan("S", ["k", "p"]).filter(col("S", "p") < 50)
            .sort([(col("S", "p"), "ASC"), (col("S", "k"), "DESC")]))
    o = c.execute(plan)
    m = pp < 50
    exp = sorted(zip(pp[m].tolist(), (-pk[m].astype(np.int64)).tolist()))
    assert list(zip(o["S.p"].tolist(), (-o["S.k"]).tolist())) == exp


def test_project_and_rearrange(big):
    c, bk, bp, pk, pp = big
    o = c.execute(RelBuilder.scan("S", ["k", "p"]).project([col("S", "p")]))
    assert list(o) == ["S.p"] and (o["S.p"] == pp).all()
    o = c.execute(RelBuilder.scan("S", ["k", "p"]).hash_rearrange(col("S", "k"), [col("S", "k"), col("S", "p")], 64))
    assert sorted(zip(o["S.k"].tolist(), o["S.p"].tolist())) == sorted(zip(pk.tolist(), pp.tolist()))


# ------------------------------------------------ the reference's plan files
def _plans():
    import json
    import os

    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_plans.json")
    with open(path) as f:
        return {p["name"]: p for p in json.load(f)["plans"]}


@pytest.mark.parametrize("name", ["reduce-scan", "reduce-join", "reduce-select"])
def test_reference_plan_scalar(cat, name):
    """tests-plan-parsing.cpp Scan / Join / Select: the plan file verbatim."""
    p = _plans()[name]
    out = cat.execute(p["plan"])
    assert len(out) == 1
    assert [int(v) for v in list(out.values())[0]] == [p["expected"]]


def test_reference_plan_nest(cat):
    """tests-plan-parsing.cpp Nest: print -> project(_groupCount as count) -> nest."""
    p = _plans()["reduce-nest"]
    out = cat.execute(p["plan"])
    assert list(out) == ["count"]
    assert sorted(out["count"].tolist()) == sorted(r["count"] for r in p["expected"])


def test_reference_plan_multinest(cat):
    p = _plans()["reduce-multinest"]
    out = cat.execute(p["plan"])
    assert list(out) == ["outputCnt", "outputMax"]
    got = sorted(zip(out["outputCnt"].tolist(), out["outputMax"].tolist()))
    assert got == sorted((r["outputCnt"], r["outputMax"]) for r in p["expected"])


def test_reference_plan_gpu_group_by(cat, golden):
    """tests/inputs/plans/gpu-group-by.json (no golden file): SUM(sid) per rating."""
    t = golden["reference"]["tables"]["sailors"]
    exp = {}
    for sid, rating in zip(t["sid"], t["rating"]):
        exp[rating] = exp.get(rating, 0) + sid
    out = cat.execute(_plans()["gpu-group-by"]["plan"])
    assert dict(zip(out["rating"].tolist(), out["sum_0"].tolist())) == exp


def test_reference_plan_reduce_scan_gpu(cat, golden):
    t = golden["reference"]["tables"]["sailors"]["sid"]
    out = cat.execute(_plans()["reduce-scan-gpu"]["plan"])
    assert [int(v[0]) for v in out.values()] == [len(t), max(t)]


# ------------------------------------------------------------ minor keys
@pytest.fixture(scope="module")
def composite(ctx):
    """Composite-key relations: the major key repeats (about 8 rows per key),
    the minor key tells the rows of one key apart."""
    rng = np.random.default_rng(77)
    nb, npr = 40000, 300001
    rel = {"R": {"k": rng.integers(0, 5000, nb), "m": rng.integers(0, 8, nb), "p": rng.integers(-99, 99, nb)},
           "S": {"k": rng.integers(-5, 5200, npr), "m": rng.integers(0, 9, npr),
                 "p": rng.integers(-99, 99, npr)}}
    c = Catalog(ctx)
    for r, cols in rel.items():
        for a, v in cols.items():
            cols[a] = v.astype(np.int32)
            c.add(r, a, dev(cols[a]))
    yield c, rel
    c.close()


def _minor_join(rel):
    s, r = RelBuilder.scan("S", ["k", "m", "p"]), RelBuilder.scan("R", ["k", "m", "p"])
    return s.partitioned_join(r, col("R", "k"), col("S", "k"), 1 << 16, 1 << 19, col("R", "m"), col("S", "m"))


def test_plan_minor_key_fused_reduce(composite, oracle):
    c, rel = composite
    plan = _minor_join(rel).reduce([lit(1), cast64(col("R", "p") * col("S", "p")), col("S", "p"),
                                    col("R", "p")], ["sum", "sum", "max", "or"])
    out = [int(v[0]) for v in c.execute(plan).values()]
    R, S = rel["R"], rel["S"]
    aggs = [(abi.AGG_COUNT, abi.VAL_ONE), (abi.AGG_SUM, abi.VAL_PRODUCT), (abi.AGG_MAX, abi.VAL_PROBE),
            (abi.AGG_OR, abi.VAL_BUILD)]
    # the probe side (S) carries PROBE, the build side (R) BUILD
    exp = oracle.radix_join_agg_minor(R["k"], R["m"], R["p"], S["k"], S["m"], S["p"], aggs,
                                      threads=cpu_threads())
    assert out == exp
    # without the minor key the plan counts more pairs
    major = oracle.radix_join_agg(R["k"], None, S["k"], None, aggs[:1], threads=cpu_threads())[0]
    assert out[0] < major


def test_plan_minor_key_materialised(composite):
    """A group-by over the join materialises the pairs and checks the minor
    key on each (the reference checks it on each chain match)."""
    c, rel = composite
    R, S = rel["R"], rel["S"]
    plan = _minor_join(rel).groupby([col("R", "m")], [(lit(1), "sum"), (col("S", "p"), "min")], 10, 1 << 22)
    out = c.execute(plan)
    # numpy: all (r, s) with equal major and minor keys
    order = np.lexsort((R["m"], R["k"]))
    rk, rm = R["k"][order].astype(np.int64), R["m"][order].astype(np.int64)
    code_r = rk * 16 + rm
    code_s = S["k"].astype(np.int64) * 16 + S["m"]
    lo = np.searchsorted(code_r, code_s, "left")
    hi = np.searchsorted(code_r, code_s, "right")
    cnt = hi - lo
    exp_cnt, exp_min = {}, {}
    for m, c_, p in zip(S["m"], cnt, S["p"]):
        if c_:
            exp_cnt[int(m)] = exp_cnt.get(int(m), 0) + int(c_)
            exp_min[int(m)] = min(exp_min.get(int(m), 1 << 40), int(p))
    assert dict(zip(out["m"].tolist(), out["sum_0"].tolist())) == exp_cnt
    assert dict(zip(out["m"].tolist(), out["min_1"].tolist())) == exp_min


# ------------------------------------------------ logical accumulators, nest
def test_plan_logical_accumulators(big):
    c, bk, bp, pk, pp = big
    r = RelBuilder.scan("R", ["k", "p"])
    out = c.execute(r.reduce([col("R", "p"), col("R", "p"), col("R", "k") > (1 << 15), col("R", "k") > (1 << 30)],
                             ["or", "and", "or", "or"]))
    assert [int(v[0]) for v in out.values()] == [int((bp != 0).any()), int((bp != 0).all()), 1, 0]
    g = c.execute(r.groupby([col("R", "p")], [(col("R", "k"), "and"), (col("R", "k") < 100, "or"),
                                               (lit(1), "sum")], 10, 1 << 16))
    for key, a, o, n in zip(g["p"], g["and_0"], g["or_1"], g["sum_2"]):
        sel = bk[bp == key]
        assert (a, o, n) == (int((sel != 0).all()), int((sel < 100).any()), len(sel))


def test_plan_nest_matches_groupby(big):
    """nest (RadixNest, 64-bit keys) and groupby agree on the same grouping."""
    c, bk, bp, pk, pp = big
    s = RelBuilder.scan("S", ["k", "p"])
    n = c.execute(s.nest(col("S", "p"), [lit(1), col("S", "k"), col("S", "k"), col("S", "k")],
                         ["sum", "sum", "min", "max"], ["cnt", "sk", "mn", "mx"], p=col("S", "k") < 60000))
    sel = pk < 60000
    keys, inv = np.unique(pp[sel], return_inverse=True)
    assert n["p"].tolist() == keys.tolist()
    assert n["cnt"].tolist() == np.bincount(inv).tolist()
    assert n["sk"].tolist() == np.bincount(inv, weights=pk[sel].astype(np.float64)).astype(np.int64).tolist()
    assert n["mn"].tolist() == [int(pk[sel][inv == i].min()) for i in range(len(keys))]
    assert n["mx"].tolist() == [int(pk[sel][inv == i].max()) for i in range(len(keys))]
