"""Plan façade: the reference's JSON plans (operator and expression names of
core/olap/lib/plan/plan-parser.cpp and expression-parser.cpp) executed on
device columns through gbj_plan_execute, plus a builder with the call shapes
of the reference's RelBuilder (core/olap/include/olap/plan/relbuilder.hpp:
scan, filter, join(build, build_k, probe_k, hash_bits, maxBuildInputSize),
groupby(k, e, hash_bits, maxInputSize), reduce(e, accumulators)).
"""
from __future__ import annotations

import ctypes as C
import json

import numpy as np

from . import abi


# ---------------------------------------------------------- expressions
class Expr:
    """An expression node in the reference's JSON form."""

    def __init__(self, node: dict):
        self.node = node

    def _bin(self, name, other):
        return Expr({"expression": name, "left": self.node, "right": lit(other).node})

    def __eq__(self, other):  # noqa: D105 - builds an eq node
        return self._bin("eq", other)

    def __lt__(self, other):
        return self._bin("lt", other)

    def __le__(self, other):
        return self._bin("le", other)

    def __gt__(self, other):
        return self._bin("gt", other)

    def __ge__(self, other):
        return self._bin("ge", other)

    def __and__(self, other):
        return self._bin("and", other)

    def __mul__(self, other):
        return self._bin("multiply", other)

    __hash__ = object.__hash__


def lit(v) -> Expr:
    if isinstance(v, Expr):
        return v
    if isinstance(v, bool):
        return Expr({"expression": "bool", "v": v})
    return Expr({"expression": "int", "v": int(v)})


def col(rel: str, attr: str) -> Expr:
    """recordProjection of attribute `attr` of relation `rel`."""
    a = {"relName": rel, "attrName": attr}
    return Expr({"expression": "recordProjection", "type": {"type": "int"},
                 "e": {"expression": "argument", "argNo": -1,
                       "type": {"type": "record", "relName": rel}, "attributes": [a]},
                 "attribute": a})


def cast64(e: Expr) -> Expr:
    return Expr({"expression": "cast", "type": {"type": "int64"}, "e": e.node})


# ------------------------------------------------------------- builder
class RelBuilder:
    """Immutable plan builder; each call returns a new builder whose root is
    the new operator (as the reference's RelBuilder does)."""

    def __init__(self, node: dict):
        self.node = node

    @staticmethod
    def scan(rel: str, attrs) -> "RelBuilder":
        return RelBuilder({"operator": "scan", "plugin": {
            "name": rel, "type": "gpu",
            "projections": [{"relName": rel, "attrName": a} for a in attrs]}})

    def filter(self, p: Expr) -> "RelBuilder":
        return RelBuilder({"operator": "select", "p": p.node, "input": self.node})

    def join(self, build: "RelBuilder", build_k: Expr, probe_k: Expr, hash_bits: int = 0,
             max_build_input_size: int = 0) -> "RelBuilder":
        """`self` is the probe side (RelBuilder::join's receiver)."""
        n = {"operator": "hashjoin-chained", "build_input": build.node, "probe_input": self.node,
             "build_k": build_k.node, "probe_k": probe_k.node}
        if hash_bits:
            n["hash_bits"] = hash_bits
        if max_build_input_size:
            n["maxBuildInputSize"] = max_build_input_size
        return RelBuilder(n)

    def partitioned_join(self, build: "RelBuilder", build_k: Expr, probe_k: Expr,
                         max_build_input_size: int = 0, max_probe_input_size: int = 0,
                         build_k_minor: Expr | None = None, probe_k_minor: Expr | None = None):
        """partitioned-hashjoin-chained; with minor keys a pair also needs
        build_k_minor == probe_k_minor."""
        n = {"operator": "partitioned-hashjoin-chained", "build_input": build.node,
             "probe_input": self.node, "build_k": build_k.node, "probe_k": probe_k.node}
        if build_k_minor is not None:
            n["build_k_minor"] = build_k_minor.node
        if probe_k_minor is not None:
            n["probe_k_minor"] = probe_k_minor.node
        if max_build_input_size:
            n["maxBuildInputSize"] = max_build_input_size
        if max_probe_input_size:
            n["maxProbeInputSize"] = max_probe_input_size
        return RelBuilder(n)

    def radix_join(self, right: "RelBuilder", left_k: Expr, right_k: Expr) -> "RelBuilder":
        """The "join" operator: self is the left (build) input."""
        return RelBuilder({"operator": "join", "p": (left_k == right_k).node,
                           "leftInput": self.node, "rightInput": right.node,
                           "leftFields": [left_k.node], "rightFields": [right_k.node]})

    def groupby(self, k, e, hash_bits: int = 10, max_input_size: int = 1 << 20) -> "RelBuilder":
        """k: [Expr]; e: [(Expr, monoid)] with monoid in sum / max / min."""
        return RelBuilder({"operator": "hashgroupby-chained", "input": self.node, "gpu": True,
                           "k": [x.node for x in k],
                           "e": [{"e": x.node, "m": m, "packet": 1, "offset": 32 * (i + 1)}
                                 for i, (x, m) in enumerate(e)],
                           "hash_bits": hash_bits, "maxInputSize": max_input_size})

    def nest(self, f: Expr, e, accumulators, labels, p: Expr | None = None) -> "RelBuilder":
        """The RadixNest operator ("nest"): group by f over the rows p keeps."""
        return RelBuilder({"operator": "nest", "input": self.node, "f": f.node, "g": f.node,
                           "p": (p if p is not None else lit(True)).node,
                           "e": [x.node for x in e], "accumulator": list(accumulators),
                           "aggrLabels": list(labels), "fields": [f.node]})

    def reduce(self, e, accumulators) -> "RelBuilder":
        return RelBuilder({"operator": "reduce", "input": self.node, "e": [x.node for x in e],
                           "accumulator": list(accumulators), "p": lit(True).node})

    def sort(self, keys) -> "RelBuilder":
        """keys: [(Expr, "ASC" | "DESC" | "NONE")]."""
        return RelBuilder({"operator": "sort", "input": self.node,
                           "e": [{"expression": x.node, "direction": d} for x, d in keys]})

    def project(self, e) -> "RelBuilder":
        return RelBuilder({"operator": "project", "input": self.node, "e": [x.node for x in e]})

    def hash_rearrange(self, key: Expr, projections, buckets: int = 2) -> "RelBuilder":
        return RelBuilder({"operator": "hash-rearrange", "input": self.node, "e": key.node,
                           "projections": [x.node for x in projections], "buckets": buckets})

    def json(self) -> str:
        return json.dumps(self.node)


# ---------------------------------------------------------- execution
def validate(plan) -> tuple[int, str]:
    """(status, message) of a host-only check of a plan."""
    lib = abi.load()
    text = plan if isinstance(plan, str) else json.dumps(plan.node if isinstance(plan, RelBuilder) else plan)
    buf = C.create_string_buffer(512)
    rc = lib.gbj_plan_validate(text.encode(), buf, len(buf))
    return rc, buf.value.decode()


class Catalog:
    """Named int32 device columns (relation, attribute) for plans."""

    def __init__(self, ctx):
        self.ctx = ctx
        h = C.c_void_p()
        ctx.check(ctx.lib.gbj_catalog_create(ctx.handle, C.byref(h)))
        self.handle = h.value
        self._keep = []

    def add(self, rel: str, attr: str, t):
        self._keep.append(t)
        self.ctx.check(self.ctx.lib.gbj_catalog_add_column(self.handle, rel.encode(), attr.encode(),
                                                           t.data_ptr(), t.numel()))

    def load(self, catalog_json: str, base_dir: str = "", relation: str | None = None) -> int:
        """Loads the int32 columns of a catalog.json in the reference's columnar
        file layout into device memory; returns the number of columns."""
        n = C.c_uint64()
        self.ctx.check(self.ctx.lib.gbj_catalog_load(self.handle, catalog_json.encode(), base_dir.encode(),
                                                     relation.encode() if relation else None, C.byref(n)))
        return n.value

    def execute(self, plan) -> dict:
        """Runs a plan (RelBuilder, dict or JSON text) -> {name: int64 numpy column}."""
        lib = self.ctx.lib
        text = plan if isinstance(plan, str) else json.dumps(
            plan.node if isinstance(plan, RelBuilder) else plan)
        r = C.c_void_p()
        self.ctx.check(lib.gbj_plan_execute(self.handle, text.encode(), C.byref(r)))
        try:
            nc, nr = C.c_int32(), C.c_uint64()
            lib.gbj_result_shape(r, C.byref(nc), C.byref(nr))
            out = {}
            for i in range(nc.value):
                a = np.empty(max(nr.value, 1), dtype=np.int64)
                lib.gbj_result_column(r, i, a.ctypes.data_as(C.c_void_p))
                out[lib.gbj_result_name(r, i).decode()] = a[:nr.value]
            return out
        finally:
            lib.gbj_result_destroy(r)

    def close(self):
        if self.handle:
            self.ctx.lib.gbj_catalog_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
