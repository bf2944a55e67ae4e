"""Plan façade, host side: plans in the reference's format validate; plans
with unknown operators, missing fields, unsupported accumulators or bad
JSON are rejected with a message naming the problem.  No GPU."""
import json

import plan_cases
from proteus_gb300 import abi
from proteus_gb300.plan import RelBuilder, col, lit, validate


def test_golden_plans_validate(lib):
    for name, mk in plan_cases.ALL.items():
        rc, msg = validate(mk())
        assert rc == abi.OK, (name, msg)


def test_unknown_operator(lib):
    p = plan_cases.nest_reserves().node
    p["input"] = {"operator": "unnest", "input": p["input"]}
    rc, msg = validate(p)
    assert rc == abi.ERR_UNSUPPORTED and "unnest" in msg


def test_missing_field(lib):
    j = RelBuilder.scan("a", ["k"]).join(RelBuilder.scan("b", ["k"]), col("b", "k"), col("a", "k"))
    p = j.reduce([lit(1)], ["sum"]).node
    del p["input"]["build_k"]
    rc, msg = validate(p)
    assert rc == abi.ERR_INVALID and "build_k" in msg


def test_unsupported_accumulator(lib):
    p = plan_cases.nest_reserves().node
    p["e"][0]["m"] = "bagunion"
    rc, msg = validate(p)
    assert rc == abi.ERR_UNSUPPORTED and "bagunion" in msg


def test_malformed_json(lib):
    for text in ['{"operator": "scan"', '{"operator": scan}', '[1, 2', '{"operator": "scan", "plugin": {"name": "x"}} 7']:
        rc, msg = validate(text)
        assert rc == abi.ERR_INVALID, text
        assert msg.startswith("plan:")


def test_builder_emits_reference_fields(lib):
    p = json.loads(plan_cases.sailors_join_left3().json())
    assert p["operator"] == "reduce" and p["accumulator"] == ["max", "sum", "sum"]
    j = p["input"]
    assert j["operator"] == "hashjoin-chained"
    assert {"build_input", "probe_input", "build_k", "probe_k", "hash_bits", "maxBuildInputSize"} <= set(j)
    g = plan_cases.multinest_reserves().node
    assert g["operator"] == "hashgroupby-chained"
    assert {"k", "e", "hash_bits", "maxInputSize"} <= set(g) and {"e", "m", "packet", "offset"} <= set(g["e"][1])


def test_cpp_relbuilder_plans_validate(lib, tmp_path):
    """The C++ builder (include/gbj_relbuilder.hpp) emits plans the façade accepts."""
    import subprocess

    import cpp_build

    exe = cpp_build.build_driver(tmp_path)
    out = subprocess.run([exe, "validate"], capture_output=True, text=True, check=True).stdout.split("\n")
    lines = [x.split(" ", 2) for x in out if x.strip()]
    assert [x[0] for x in lines] == ["sailorsJoinLeft3", "multinestReserves", "nestBagTPCH"]
    assert all(x[1] == "0" for x in lines), lines


def test_sort_project_rearrange_validate(lib):
    from proteus_gb300.plan import RelBuilder, col, lit

    g = plan_cases.nest_reserves().sort([(col(plan_cases.R, "sid"), "DESC")])
    assert validate(g)[0] == abi.OK
    s = RelBuilder.scan("a", ["k", "v"]).project([col("a", "v")]).hash_rearrange(col("a", "v"), [col("a", "v")], 8)
    assert validate(s)[0] == abi.OK
    bad = json.loads(g.json())
    bad["e"][0]["direction"] = "UP"
    rc, msg = validate(bad)
    assert rc == abi.ERR_INVALID and "UP" in msg
