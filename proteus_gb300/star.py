"""Batched star join: the seeded star schema, the query variants and a
wrapper over the gbj_star_* entry points.

Schema (dimension row i has primary key i + 1, except the date dimension,
keyed yyyymmdd like SSB's; every column is a pure function of (seed,
column, row)):

  dim 0  customer  2^21 rows  nation int8 0..24, region int8 0..4, city int32 0..249
  dim 1  date      2557 rows  key yyyymmdd (days from 1992-01-01),
                              year int32 1992.., month int8 0..11, week int32 1..53
  dim 2  part      2^18 rows  category int8 0..24, mfgr int8 0..4, brand int32 0..999
  dim 3  supplier  2^16 rows  nation int8 0..24, region int8 0..4
  fact   2^28 rows  fk0..fk3 uniform over each dimension's keys,
                    quantity int32 1..50, price int32 900..110000

A query joins three of the four dimensions, filters each joined dimension on
one attribute with a range keeping about 1/5 to 1/50 of its rows, and groups
by one low-cardinality attribute of each of two joined dimensions (at most
25 x 25 groups), summing (int64)price * quantity.  This is the shape of the
reference's SSB star plans; the data and predicates are synthetic.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import abi

FULL_DIM_ROWS = (1 << 21, 2557, 1 << 18, 1 << 16)
FULL_FACT_ROWS = 1 << 28

# per dimension: (name, [(attr, dtype, lo, hi), ...]); date attributes are
# derived from the row number, the others are uniform draws
DIM_SPECS = (
    ("customer", [("nation", np.int8, 0, 24), ("region", np.int8, 0, 4), ("city", np.int32, 0, 249)]),
    ("date", [("year", np.int32, 1992, None), ("month", np.int8, 0, 11), ("week", np.int32, 1, 53)]),
    ("part", [("category", np.int8, 0, 24), ("mfgr", np.int8, 0, 4), ("brand", np.int32, 0, 999)]),
    ("supplier", [("nation", np.int8, 0, 24), ("region", np.int8, 0, 4)]),
)
GROUPABLE_MAX = 25  # group keys use attributes with at most this many values

_S_DIM, _S_FACT, _S_QUERY = 0x5300, 0x5400, 0x5A00


def _uniform(seed: int, stream: int, n: int, lo: int, hi: int, threads=0) -> np.ndarray:
    import datagen

    return datagen.gen_uniform_i32(seed, stream, n, lo, hi, threads)


@dataclass
class Dim:
    name: str
    n: int
    attrs: list  # numpy columns (int8 or int32)
    names: list
    lo: list
    hi: list
    keys: np.ndarray | None = None  # primary keys (int32); None: row i has key i + 1

    def key_of_rows(self, rows: np.ndarray) -> np.ndarray:
        """Primary keys of 0-based rows."""
        if self.keys is None:
            return (rows + 1).astype(np.int32)
        return self.keys[rows]


def yyyymmdd(n: int, start=(1992, 1, 1)) -> np.ndarray:
    """Keys yyyymmdd of n consecutive days from `start`."""
    import datetime

    d0 = datetime.date(*start)
    days = [d0 + datetime.timedelta(days=i) for i in range(n)]
    return np.array([d.year * 10000 + d.month * 100 + d.day for d in days], dtype=np.int32)


@dataclass
class StarData:
    dims: list
    fk: list  # int32 numpy columns, fk[d] -> dims[d]
    quantity: np.ndarray
    price: np.ndarray

    @property
    def n_fact(self) -> int:
        return int(self.quantity.shape[0])


def gen_dims(seed: int, dim_rows=FULL_DIM_ROWS) -> list:
    dims = []
    for d, ((name, spec), n) in enumerate(zip(DIM_SPECS, dim_rows)):
        cols, names, los, his = [], [], [], []
        for a, (an, dt, lo, hi) in enumerate(spec):
            r = np.arange(n, dtype=np.int64)
            if name == "date" and an == "year":
                col = (1992 + r // 365).astype(np.int32)
                lo, hi = 1992, int(col.max()) if n else 1992
            elif name == "date" and an == "month":
                col = ((r % 365) // 31).astype(np.int8)
            elif name == "date" and an == "week":
                col = ((r % 365) // 7 + 1).astype(np.int32)
            else:
                col = _uniform(seed, _S_DIM + 16 * d + a, n, lo, hi).astype(dt)
            cols.append(np.ascontiguousarray(col))
            names.append(an)
            los.append(int(lo))
            his.append(int(hi))
        dims.append(Dim(name, n, cols, names, los, his, yyyymmdd(n) if name == "date" else None))
    return dims


def gen_star(seed: int, n_fact: int = FULL_FACT_ROWS, dim_rows=FULL_DIM_ROWS, threads=0) -> StarData:
    dims = gen_dims(seed, dim_rows)
    fk = [_uniform(seed, _S_FACT + d, n_fact, 1, dims[d].n, threads) for d in range(len(dims))]
    for d, dim in enumerate(dims):
        if dim.keys is not None:  # uniform over the rows, as the keys of those rows
            fk[d] = np.ascontiguousarray(dim.keys[fk[d] - 1])
    qty = _uniform(seed, _S_FACT + 8, n_fact, 1, 50, threads)
    price = _uniform(seed, _S_FACT + 9, n_fact, 900, 110000, threads)
    return StarData(dims, fk, qty, price)


@dataclass
class Query:
    join_mask: int
    pred_attr: list = field(default_factory=lambda: [-1] * 4)
    pred_lo: list = field(default_factory=lambda: [0] * 4)
    pred_hi: list = field(default_factory=lambda: [0] * 4)
    group_dim: list = field(default_factory=lambda: [0, 0])
    group_attr: list = field(default_factory=lambda: [0, 0])

    def to_c(self) -> abi.StarQuery:
        q = abi.StarQuery()
        q.join_mask = self.join_mask
        for d in range(4):
            q.pred_attr[d], q.pred_lo[d], q.pred_hi[d] = self.pred_attr[d], self.pred_lo[d], self.pred_hi[d]
        for k in range(2):
            q.group_dim[k], q.group_attr[k] = self.group_dim[k], self.group_attr[k]
        return q


def gen_queries(seed: int, n_queries: int, dims: list) -> list:
    """Seeded query variants (draws from gbj_gen_rand, identical everywhere)."""
    import datagen

    lib = datagen.load()
    nd = len(dims)
    out = []
    for q in range(n_queries):
        def draw(i, q=q):
            return int(lib.gbj_gen_rand(seed, _S_QUERY + q, i))

        skip = draw(0) % nd
        joined = [d for d in range(nd) if d != skip] if nd > 1 else [0]
        qq = Query(join_mask=sum(1 << d for d in joined))
        for d in joined:
            dim = dims[d]
            a = draw(1 + d) % len(dim.attrs)
            span = dim.hi[a] - dim.lo[a] + 1
            sel = 0.2 * 10.0 ** (-(draw(5 + d) % 1000) / 1000.0)  # 1/5 .. 1/50
            m = max(1, min(span, int(round(sel * span))))
            start = dim.lo[a] + draw(9 + d) % (span - m + 1)
            qq.pred_attr[d], qq.pred_lo[d], qq.pred_hi[d] = a, start, start + m - 1
        ga = joined[draw(13) % len(joined)]
        rest = [d for d in joined if d != ga] or [ga]
        gb = rest[draw(14) % len(rest)]
        for k, (d, salt) in enumerate(((ga, 15), (gb, 16))):
            dim = dims[d]
            cand = [a for a in range(len(dim.attrs)) if dim.hi[a] - dim.lo[a] + 1 <= GROUPABLE_MAX]
            qq.group_dim[k] = d
            qq.group_attr[k] = cand[draw(salt) % len(cand)]
        out.append(qq)
    return out


class StarPlan:
    """gbj_star_plan over device copies of a StarData (torch tensors)."""

    def __init__(self, ctx, data: StarData, device="cuda", fact_tensors=None):
        """fact_tensors: optional device columns (fk list, quantity, price)
        to use instead of copies of data's fact columns."""
        import torch

        self.ctx = ctx
        self.dev_dims = [[torch.from_numpy(c).to(device) for c in d.attrs] for d in data.dims]
        self.dev_keys = [None if d.keys is None else torch.from_numpy(d.keys).to(device) for d in data.dims]
        if fact_tensors is None:
            self.dev_fk = [torch.from_numpy(c).to(device) for c in data.fk]
            self.dev_qty = torch.from_numpy(data.quantity).to(device)
            self.dev_price = torch.from_numpy(data.price).to(device)
        else:
            self.dev_fk, self.dev_qty, self.dev_price = list(fact_tensors[0]), fact_tensors[1], fact_tensors[2]
        torch.cuda.synchronize()
        self.dims = data.dims
        self.handle = None
        self._make()

    def _make(self):
        nd = len(self.dims)
        fact = abi.StarFact()
        fact.n = int(self.dev_qty.numel())
        fact.n_dims = nd
        for d in range(nd):
            fact.d_fk[d] = self.dev_fk[d].data_ptr()
        fact.d_quantity = self.dev_qty.data_ptr()
        fact.d_price = self.dev_price.data_ptr()
        arr = (abi.StarDim * abi.STAR_MAX_DIMS)()
        for d, dim in enumerate(self.dims):
            sd = arr[d]
            sd.n, sd.key_base, sd.n_attrs = dim.n, 1, len(dim.attrs)
            if self.dev_keys[d] is not None:
                sd.d_keys = self.dev_keys[d].data_ptr()
            for a, col in enumerate(self.dev_dims[d]):
                sd.d_attr[a] = col.data_ptr()
                sd.attr_type[a] = abi.ATTR_I8 if dim.attrs[a].dtype == np.int8 else abi.ATTR_I32
                sd.attr_min[a], sd.attr_max[a] = dim.lo[a], dim.hi[a]
        h = C.c_void_p()
        self.ctx.check(self.ctx.lib.gbj_star_plan_create(self.ctx.handle, C.byref(fact), arr, C.byref(h)))
        self.handle = h.value

    def new_output(self, n_queries: int, group_cap: int = abi.STAR_MAX_GROUPS):
        import torch

        dev = self.dev_qty.device
        n = n_queries * group_cap
        return {
            "a": torch.empty(n, dtype=torch.int32, device=dev),
            "b": torch.empty(n, dtype=torch.int32, device=dev),
            "count": torch.empty(n, dtype=torch.int64, device=dev),
            "sum": torch.empty(n, dtype=torch.int64, device=dev),
            "n": torch.zeros(n_queries, dtype=torch.int64, device=dev),
            "cap": group_cap,
        }

    def run(self, queries: list, out=None, use_graph=True, stream=None):
        from .engine import _cur_stream

        if out is None:
            out = self.new_output(len(queries))
        qa = (abi.StarQuery * len(queries))(*[q.to_c() for q in queries])
        so = abi.StarOut(out["a"].data_ptr(), out["b"].data_ptr(), out["count"].data_ptr(),
                         out["sum"].data_ptr(), out["n"].data_ptr(), out["cap"])
        s = stream if stream is not None else _cur_stream()
        self.ctx.check(self.ctx.lib.gbj_star_run(self.handle, qa, len(queries), C.byref(so),
                                                 1 if use_graph else 0, s))
        return out

    @staticmethod
    def results(out, n_queries: int):
        """Per query: (a, b, count, sum) numpy arrays."""
        n = out["n"].cpu().numpy()
        cap = out["cap"]
        cols = {k: out[k].cpu().numpy() for k in ("a", "b", "count", "sum")}
        res = []
        for q in range(n_queries):
            lo = q * cap
            res.append(tuple(cols[k][lo:lo + int(n[q])] for k in ("a", "b", "count", "sum")))
        return res

    def close(self):
        if self.handle:
            self.ctx.lib.gbj_star_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
