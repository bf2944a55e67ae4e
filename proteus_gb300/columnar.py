"""Writes relations in the reference's columnar file layout
(tools/prepare_data.py): one little-endian binary file per column named
"<path>.<attrName>" (int32 for int / boolean / dictionary-coded strings,
int64 for int64, float64 for float) and a catalog.json entry per relation
with the relation's path, its attributes and a "block" plugin."""
from __future__ import annotations

import json
import os

import numpy as np

_TYPES = {np.dtype(np.int32): "int", np.dtype(np.int64): "int64", np.dtype(np.float64): "float"}


def write_relation(base_dir: str, path: str, columns: dict) -> dict:
    """columns: {attrName: numpy array}; returns the catalog entry."""
    attrs = []
    n = None
    for i, (name, col) in enumerate(columns.items()):
        col = np.ascontiguousarray(col)
        if col.dtype not in _TYPES:
            raise ValueError(f"{name}: unsupported dtype {col.dtype}")
        if n is not None and len(col) != n:
            raise ValueError("columns differ in length")
        n = len(col)
        fn = os.path.join(base_dir, path + "." + name)
        os.makedirs(os.path.dirname(fn), exist_ok=True)
        col.astype(col.dtype.newbyteorder("<"), copy=False).tofile(fn)
        attrs.append({"type": {"type": _TYPES[col.dtype]}, "relName": path, "attrName": name, "attrNo": i + 1})
    return {"path": path, "type": {"type": "bag", "inner": {"type": "record", "attributes": attrs}},
            "plugin": {"type": "block", "linehint": int(n or 0)}}


def write_catalog(file: str, entries: dict):
    """entries: {relation key: catalog entry}."""
    with open(file, "w") as f:
        json.dump(entries, f, indent=4)
        f.write("\n")
