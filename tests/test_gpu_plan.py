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
