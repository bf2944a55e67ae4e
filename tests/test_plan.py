"""Plan façade, host side: plans in the reference's format validate; plans
with unknown operators, missing fields, unsupported accumulators or bad
JSON are rejected with a message naming the problem.  No GPU."""
import json

import pytest

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


def _golden_plans():
    import os

    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_plans.json")
    with open(here) as f:
        return json.load(f)["plans"]


def test_reference_plan_files_validate(lib):
    """The reference's own plan files (verbatim) pass the façade's checks."""
    for p in _golden_plans():
        rc, msg = validate(p["plan"])
        assert rc == abi.OK, (p["name"], msg)


def test_unknown_field_is_refused(lib):
    j = RelBuilder.scan("a", ["k"]).join(RelBuilder.scan("b", ["k"]), col("b", "k"), col("a", "k"))
    p = j.reduce([lit(1)], ["sum"]).node
    p["input"]["frobnicate"] = 1
    rc, msg = validate(p)
    assert rc == abi.ERR_UNSUPPORTED and "frobnicate" in msg and "hashjoin-chained" in msg
    # the minor key is a field of the partitioned join only (plan-parser.cpp:872-880)
    del p["input"]["frobnicate"]
    p["input"]["build_k_minor"] = col("b", "k").node
    p["input"]["probe_k_minor"] = col("a", "k").node
    rc, msg = validate(p)
    assert rc == abi.ERR_UNSUPPORTED and "build_k_minor" in msg


def test_minor_key_fields(lib):
    s, r = RelBuilder.scan("S", ["k", "m"]), RelBuilder.scan("R", ["k", "m"])
    ok = s.partitioned_join(r, col("R", "k"), col("S", "k"), 16, 64, col("R", "m"), col("S", "m"))
    assert validate(ok.reduce([lit(1)], ["sum"]))[0] == abi.OK
    half = s.partitioned_join(r, col("R", "k"), col("S", "k"), 16, 64, col("R", "m"))
    rc, msg = validate(half.reduce([lit(1)], ["sum"]))
    assert rc == abi.ERR_INVALID and "minor" in msg


def test_logical_accumulators_and_nest_validate(lib):
    g = RelBuilder.scan("a", ["k", "v"]).groupby([col("a", "k")], [(col("a", "v"), "or"),
                                                                   (col("a", "v"), "and")])
    assert validate(g)[0] == abi.OK
    n = RelBuilder.scan("a", ["k", "v"]).nest(col("a", "k"), [lit(1), col("a", "v")], ["sum", "max"],
                                              ["cnt", "mx"])
    assert validate(n)[0] == abi.OK
    bad = json.loads(n.json())
    bad["aggrLabels"] = ["cnt"]
    rc, msg = validate(bad)
    assert rc == abi.ERR_INVALID and "label" in msg


@pytest.mark.parametrize("op", ["split", "union-all", "unnest", "out-of-gpu-join"])
def test_operators_not_supported(lib, op):
    p = {"operator": "reduce", "e": [lit(1).node], "accumulator": ["sum"],
         "input": {"operator": op, "input": RelBuilder.scan("a", ["k"]).node}}
    rc, msg = validate(p)
    assert rc == abi.ERR_UNSUPPORTED and op in msg


def test_passthrough_operators_validate(lib):
    inner = RelBuilder.scan("a", ["k"]).node
    for op in ("block-to-tuples", "unpack", "cpu-to-gpu", "gpu-to-cpu", "mem-move-device", "router"):
        inner = {"operator": op, "input": inner}
    p = {"operator": "print", "input": {"operator": "reduce", "e": [lit(1).node], "accumulator": ["sum"],
                                        "input": inner}}
    assert validate(p)[0] == abi.OK
    inner["bogus"] = True
    assert validate(p)[0] == abi.ERR_UNSUPPORTED
