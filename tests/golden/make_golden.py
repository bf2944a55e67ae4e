"""Generates the golden fixtures under tests/golden/.

1. reference_cases.json -- the integer columns of the reference's own test
   inputs (tests/inputs/{sailors,reserves,boats}.csv,
   tests/inputs/tpch/lineitem10.csv) and the expected outputs of the
   reference tests that exercise joins, reduces and group-bys over them
   (golden files under tests/olap/outputs/).  Read from the reference tree.
2. rjstepwise_cases.json -- match counts of the reference's RJStepwise and
   cluster counts of its partitionHT (core/platform/lib/util/radix/joins/
   radix-join.cpp), compiled from source into oracle/_ref, on seeded
   synthetic inputs, plus checksums of those inputs so a test can confirm
   the generator reproduces them.

Run from the repository root:  python tests/golden/make_golden.py
(requires the reference source tree named by $PROTEUS_REF).
"""
from __future__ import annotations

import csv
import hashlib
import json
import os
import sys

import numpy as np


ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
REF = os.environ.get("PROTEUS_REF", "")
if not REF:
    raise SystemExit("set PROTEUS_REF to the reference source tree")
OUT = os.path.dirname(os.path.abspath(__file__))

import datagen  # noqa: E402  (the repository root is on sys.path now)


def read_csv(rel, delim, cols):
    rows = []
    with open(os.path.join(REF, rel)) as f:
        for r in csv.reader(f, delimiter=delim):
            if r:
                rows.append(r)
    return {name: [int(float(r[i])) for r in rows] for name, i in cols.items()}


def read_text(rel):
    with open(os.path.join(REF, rel)) as f:
        return f.read().strip()


def reference_cases():
    sailors = read_csv("tests/inputs/sailors.csv", ";", {"sid": 0, "rating": 2})
    reserves = read_csv("tests/inputs/reserves.csv", ";", {"sid": 0, "bid": 1})
    boats = read_csv("tests/inputs/boats.csv", ";", {"bid": 0})
    # l_quantity is an integral float column in this file; read as int
    lineitem = read_csv("tests/inputs/tpch/lineitem10.csv", "|",
                        {"l_orderkey": 0, "l_linenumber": 3, "l_quantity": 4})
    left3 = read_text("tests/olap/outputs/tests-sailors/sailorsJoinLeft3.csv").split(",")
    wayjoin = json.loads(read_text("tests/olap/outputs/tests-output/3wayJoin.json"))[0]
    radix_cnt = int(read_text("tests/olap/outputs/tests-plan-parsing/reduce-join-log.json"))
    nest = json.loads(read_text("tests/olap/outputs/tests-output/nestReserves.json"))
    multinest = json.loads(read_text("tests/olap/outputs/tests-output/multinestReserves.json"))
    bag = json.loads(read_text("tests/olap/outputs/tests-output/nestBagTPCH.json"))
    cases = [
        {
            "name": "sailorsJoinLeft3",
            "reference_test": "core/olap/tests/operator-tests/tests-join-sailors.cpp:127-165",
            "golden": "tests/olap/outputs/tests-sailors/sailorsJoinLeft3.csv",
            "plan": "sailors.join(reserves on sid, hash_bits 16, maxBuild 128)"
                    ".join(boats on bid).reduce(MAX sid, SUM sid, SUM 1)",
            "expected": {"max_sid": int(left3[0]), "sum_sid": int(left3[1]),
                         "count": int(left3[2])},
        },
        {
            "name": "3wayJoin",
            "reference_test": "tests/olap/tests-output.cpp:240-281",
            "golden": "tests/olap/outputs/tests-output/3wayJoin.json",
            "plan": "reserves.join(build=sailors on sid, 4, 16).join(build=boats on bid)"
                    ".reduce(MAX sid, SUM sid, SUM 1)",
            "expected": {"max_sid": wayjoin["max_sid"], "sum_sid": wayjoin["sum_sid"],
                         "count": wayjoin["cnt"]},
        },
        {
            "name": "reduce-join",
            "reference_test": "tests/olap/tests-plan-parsing.cpp:96-101",
            "golden": "tests/olap/outputs/tests-plan-parsing/reduce-join-log.json",
            "plan": "tests/inputs/plans/reduce-join.json: radix join sailors.sid = reserves.sid,"
                    " reduce SUM 1",
            "expected": {"count": radix_cnt},
        },
        {
            "name": "nestReserves",
            "reference_test": "tests/olap/tests-output.cpp:283-307",
            "golden": "tests/olap/outputs/tests-output/nestReserves.json",
            "plan": "reserves.groupby(sid; SUM 1, hash_bits 4, maxInputSize 16)",
            "expected": {"counts": sorted(r["_groupCount"] for r in nest)},
        },
        {
            "name": "multinestReserves",
            "reference_test": "tests/olap/tests-output.cpp:309-335",
            "golden": "tests/olap/outputs/tests-output/multinestReserves.json",
            "plan": "reserves.groupby(sid; SUM 1, MAX bid, hash_bits 4, maxInputSize 16)",
            "expected": {"count_max": sorted([r["_outCount"], r["_outMax"]] for r in multinest)},
        },
        {
            "name": "nestBagTPCH",
            "reference_test": "tests/olap/tests-output.cpp:208-238",
            "golden": "tests/olap/outputs/tests-output/nestBagTPCH.json",
            "plan": "lineitem.filter(l_orderkey < 4).groupby(l_linenumber; SUM 1, MAX l_quantity,"
                    " hash_bits 4, maxInputSize 16)",
            "expected": {"count_max": sorted([r["cnt"], int(r["max_qty"])] for r in bag)},
        },
    ]
    return {
        "about": "Integer columns of the reference's test inputs and the expected results of its "
                 "join / reduce / group-by tests (outputs compared unordered, as the reference "
                 "does).",
        "tables": {"sailors": sailors, "reserves": reserves, "boats": boats,
                   "lineitem10": lineitem},
        "cases": cases,
    }


def checksum(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.int32).tobytes()).hexdigest()[:16]


def rjstepwise_cases():
    from oracle import oracle as O
    from proteus_gb300 import engine as E

    O.build()
    if not O.build_ref(REF):
        raise SystemExit("reference tree not found; cannot build oracle/_ref")
    cases = []
    specs = [
        ("plain", 11, 1 << 12, 1 << 16, None),
        ("plain", 12, 1 << 16, 1 << 18, None),
        ("zipf", 13, 1 << 14, 1 << 17, 0.0),
        ("zipf", 14, 1 << 14, 1 << 17, 0.5),
        ("zipf", 15, 1 << 14, 1 << 17, 1.0),
        ("zipf", 16, 1 << 17, 1 << 19, 1.0),
        ("zipf", 17, 3001, 50000, 1.0),
    ]
    for kind, seed, nr, ns, theta in specs:
        rk, _ = E.gen_build_side(seed, nr, payload=False)
        if kind == "plain":
            sk, _ = E.gen_probe_uniform(seed, ns, nr, payload=False)
        else:
            sk, _ = E.gen_probe_zipf(seed, ns, nr, theta, 0.5)
        m = O.ref_rj_stepwise(rk, sk)
        counts, _, _ = O.ref_partition_ht(rk)
        cases.append({
            "kind": kind, "seed": seed, "n_build": nr, "n_probe": ns, "theta": theta,
            "build_sha": checksum(rk), "probe_sha": checksum(sk),
            "rjstepwise_matches": m,
            "partition_ht_counts_sha": hashlib.sha256(counts.astype(np.int32).tobytes())
            .hexdigest()[:16],
            "partition_ht_nonempty": int((counts > 0).sum()),
        })
    return {
        "about": "RJStepwise match counts and partitionHT cluster counts of the reference's "
                 "core/platform/lib/util/radix/joins/radix-join.cpp, compiled from source by "
                 "oracle/Makefile (target ref), on inputs from the seeded generators "
                 "gbj_gen_build_side / gbj_gen_probe_uniform / gbj_gen_probe_zipf.",
        "cases": cases,
    }


def partition_ht_agg_cases():
    """The reference's int64-key partitionHT (radix-aggr.cpp) on seeded keys."""
    from oracle import oracle as O
    from proteus_gb300 import abi

    O.build()
    if not O.build_ref(REF):
        raise SystemExit("reference tree not found; cannot build oracle/_ref")
    lib = abi.load()
    cases = []
    for seed, n, span in ((21, 1 << 12, 1 << 40), (22, 1 << 16, 1 << 62), (23, 50001, 1 << 20),
                          (24, 1 << 17, 1 << 63)):
        keys = np.array([int(datagen.load().gbj_gen_rand(seed, 0x6A00, i)) % span for i in range(n)], dtype=np.uint64)
        keys = keys.view(np.int64) - (np.int64(span // 2) if span < (1 << 63) else 0)
        counts, ok, orows = O.ref_partition_ht_agg(keys)
        cases.append({
            "seed": seed, "n": n, "span": str(span),
            "keys_sha": hashlib.sha256(keys.tobytes()).hexdigest()[:16],
            "counts_sha": hashlib.sha256(counts.astype(np.int32).tobytes()).hexdigest()[:16],
            "clustered_rows_sha": hashlib.sha256(orows.astype(np.int64).tobytes()).hexdigest()[:16],
            "nonempty": int((counts > 0).sum()),
        })
    return {
        "about": "partitionHT of the reference's int64-key aggregation twin "
                 "(core/platform/lib/util/radix/aggregations/radix-aggr.cpp), compiled from source by "
                 "oracle/Makefile (target ref); keys = gbj_gen_rand(seed, 0x6A00, i) mod span, shifted "
                 "to be signed; row ids in clustered order pin the stable two-pass order.",
        "cases": cases,
    }


def _i64_keys(lib, seed, n, span, salt):
    keys = np.array([int(datagen.load().gbj_gen_rand(seed, salt, i)) % span for i in range(n)], dtype=np.uint64)
    return keys.view(np.int64) - (np.int64(span // 2) if span < (1 << 63) else 0)


def nest_i64_cases():
    """The reference's int64-key RJStepwise match counts and RadixNest group
    sizes (bucket_chaining_agg_prepare / _probe over partitionHT clusters)."""
    from oracle import oracle as O
    from proteus_gb300 import abi

    O.build()
    if not O.build_ref(REF):
        raise SystemExit("reference tree not found; cannot build oracle/_ref")
    lib = abi.load()
    joins, nests = [], []
    for seed, nr, ns, span in ((31, 1 << 12, 1 << 14, 1 << 13), (32, 40000, 90001, 1 << 18),
                               (33, 1 << 16, 1 << 16, 1 << 62), (34, 3000, 200000, 1 << 11)):
        rk = _i64_keys(lib, seed, nr, span, 0x6B00)
        sk = _i64_keys(lib, seed, ns, span, 0x6B01)
        joins.append({"seed": seed, "nr": nr, "ns": ns, "span": str(span),
                      "r_sha": hashlib.sha256(rk.tobytes()).hexdigest()[:16],
                      "s_sha": hashlib.sha256(sk.tobytes()).hexdigest()[:16],
                      "matches": O.ref_rj_stepwise_agg(rk, sk)})
    for seed, n, span in ((41, 1 << 14, 1 << 10), (42, 100003, 1 << 16), (43, 1 << 16, 1 << 63),
                          (44, 50000, 1 << 40)):
        keys = _i64_keys(lib, seed, n, span, 0x6B02)
        uk = np.unique(keys)
        counts = O.ref_nest_counts(keys, uk)
        nests.append({"seed": seed, "n": n, "span": str(span),
                      "keys_sha": hashlib.sha256(keys.tobytes()).hexdigest()[:16],
                      "groups": int(len(uk)),
                      "counts_sha": hashlib.sha256(counts.astype(np.int64).tobytes()).hexdigest()[:16],
                      "max_count": int(counts.max())})
    return {
        "about": "the reference's int64-key twins (core/platform/lib/util/radix/aggregations/"
                 "radix-aggr.cpp), compiled from source by oracle/Makefile (target ref): RJStepwise match "
                 "counts, and per distinct key (ascending) the group size bucket_chaining_agg_probe finds in "
                 "its partitionHT cluster; keys = gbj_gen_rand(seed, salt, i) mod span, shifted to be signed "
                 "(salts 0x6B00 R, 0x6B01 S, 0x6B02 nest).",
        "joins": joins,
        "nests": nests,
    }


# The reference's own plan files over its CSV test inputs
# (tests/olap/tests-plan-parsing.cpp runs the first five and compares with
# tests/olap/outputs/tests-plan-parsing/*-log.json; the GPU ones have no
# golden output, their tests compare with the oracle).  Plans that read
# float columns (reduce-twofields-scan, reduce-select-gpu) are left out:
# the catalog here holds int32 columns.
PLAN_FILES = [
    ("reduce-scan", "tests/inputs/plans/reduce-scan.json",
     "tests/olap/outputs/tests-plan-parsing/reduce-scan-log.json"),
    ("reduce-join", "tests/inputs/plans/reduce-join.json",
     "tests/olap/outputs/tests-plan-parsing/reduce-join-log.json"),
    ("reduce-nest", "tests/inputs/plans/reduce-nest.json",
     "tests/olap/outputs/tests-plan-parsing/reduce-nest-log.json"),
    ("reduce-select", "tests/inputs/plans/reduce-select.json",
     "tests/olap/outputs/tests-plan-parsing/reduce-select-log.json"),
    ("reduce-multinest", "tests/inputs/plans/reduce-multinest.json",
     "tests/olap/outputs/tests-plan-parsing/reduce-multinest-log.json"),
    ("gpu-group-by", "tests/inputs/plans/gpu-group-by.json", None),
    ("reduce-scan-gpu", "tests/inputs/plans/reduce-scan-gpu.json", None),
]


def reference_plans():
    plans = []
    for name, plan, golden in PLAN_FILES:
        entry = {"name": name, "plan_file": plan, "plan": read_text(plan)}
        if golden:
            entry["golden_file"] = golden
            entry["expected"] = json.loads(read_text(golden))
        plans.append(entry)
    return {
        "about": "The reference's plan files over tests/inputs/{sailors,reserves}.csv, verbatim, with the "
                 "expected outputs of tests/olap/tests-plan-parsing.cpp where the reference has them "
                 "(compared unordered, as runAndVerify does).  Columns: reference_cases.json tables.",
        "plans": plans,
    }


GENERATORS = {
    "reference_cases": reference_cases,
    "rjstepwise_cases": rjstepwise_cases,
    "partition_ht_agg_cases": partition_ht_agg_cases,
    "nest_i64_cases": nest_i64_cases,
    "reference_plans": reference_plans,
}


def main():
    """python tests/golden/make_golden.py [name ...] (default: every fixture)."""
    names = sys.argv[1:] or list(GENERATORS)
    for name in names:
        with open(os.path.join(OUT, name + ".json"), "w") as f:
            json.dump(GENERATORS[name](), f, indent=1)
    print("wrote", ", ".join(names), "to", OUT)


if __name__ == "__main__":
    main()
