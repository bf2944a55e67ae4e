"""Batched star join (gbj_star_*) on the GPU vs the oracle's per-query
restatement, through the C ABI."""
import numpy as np
import pytest

from gpu_util import cpu_threads
from proteus_gb300 import abi, star

pytestmark = pytest.mark.gpu

SMALL_DIMS = (1 << 14, 2557, 1 << 12, 1 << 10)


@pytest.fixture(scope="module")
def data():
    return star.gen_star(21, n_fact=(1 << 20) + 3, dim_rows=SMALL_DIMS)


@pytest.fixture(scope="module")
def plan(ctx, data):
    p = star.StarPlan(ctx, data)
    yield p
    p.close()


@pytest.fixture(scope="module")
def expected(data, oracle):
    qs = star.gen_queries(21, 64, data.dims)
    return qs, [oracle.star_query(data, q, threads=cpu_threads()) for q in qs]


def check(got, exp):
    for i, (g, e) in enumerate(zip(got, exp)):
        assert len(g[0]) == len(e[0]), i
        for x, y in zip(g, e):
            assert (x == y).all(), i


@pytest.mark.parametrize("use_graph", [False, True])
def test_star_batch_parity(ctx, plan, expected, use_graph):
    qs, exp = expected
    out = plan.run(qs, use_graph=use_graph)
    ctx.sync()
    check(star.StarPlan.results(out, len(qs)), exp)


def test_star_graph_replays_alternate(ctx, plan, expected):
    """Four replays (two graphs alternating) with different query subsets."""
    qs, exp = expected
    subsets = [list(range(0, 64, 2)), list(range(1, 64, 3)), list(range(64)), [5]]
    outs = [plan.run([qs[i] for i in s], use_graph=True) for s in subsets]
    ctx.sync()
    for s, out in zip(subsets, outs):
        check(star.StarPlan.results(out, len(s)), [exp[i] for i in s])


def test_star_alone_equals_in_batch(ctx, plan, expected):
    qs, exp = expected
    for i in (0, 17, 63):
        out = plan.run([qs[i]], use_graph=False)
        ctx.sync()
        check(star.StarPlan.results(out, 1), [exp[i]])


def test_star_unaligned_columns_scalar_path(ctx, data, oracle):
    """Fact columns that are not 16-byte aligned take the scalar load path."""
    import torch

    fk = [torch.from_numpy(c).cuda()[1:] for c in data.fk]
    qty = torch.from_numpy(data.quantity).cuda()[1:]
    price = torch.from_numpy(data.price).cuda()[1:]
    shifted = star.StarData(data.dims, [c[1:] for c in data.fk], data.quantity[1:], data.price[1:])
    p = star.StarPlan(ctx, data, fact_tensors=(fk, qty, price))
    qs = star.gen_queries(4, 8, data.dims)
    out = p.run(qs, use_graph=False)
    ctx.sync()
    exp = [oracle.star_query(shifted, q, threads=cpu_threads()) for q in qs]
    check(star.StarPlan.results(out, len(qs)), exp)
    p.close()


def test_star_foreign_keys_outside_dimension(ctx, oracle):
    d = star.gen_star(9, n_fact=1 << 18, dim_rows=SMALL_DIMS)
    d.fk[0][::7] = 0
    d.fk[1][::11] = SMALL_DIMS[1] + 3  # not a yyyymmdd key of the date dimension
    d.fk[1][::17] = 19920100
    d.fk[2][::13] = -5
    p = star.StarPlan(ctx, d)
    qs = star.gen_queries(9, 64, d.dims)
    out = p.run(qs)
    ctx.sync()
    check(star.StarPlan.results(out, len(qs)), [oracle.star_query(d, q, threads=cpu_threads()) for q in qs])
    p.close()


def test_star_date_keys_are_yyyymmdd(data):
    """The 2,557-row date dimension is keyed yyyymmdd (1992-01-01 ..
    1998-12-31), so the batch path uses its hashed dimension table."""
    date = data.dims[1]
    assert date.n == 2557 and date.keys is not None
    assert date.keys[0] == 19920101 and date.keys[-1] == 19981231
    assert np.isin(data.fk[1], date.keys).all()


def test_star_dense_and_hashed_agree(ctx, oracle):
    """Every dimension hashed (large ones gathered from L2 through the
    table), and every dimension dense, against the oracle."""
    rng = np.random.default_rng(31)
    base = star.gen_star(13, n_fact=1 << 18, dim_rows=SMALL_DIMS)
    qs = star.gen_queries(13, 64, base.dims)
    # all dense: the date dimension with keys row + 1
    dense = star.StarData([star.Dim(d.name, d.n, d.attrs, d.names, d.lo, d.hi, None) for d in base.dims],
                          [c.copy() for c in base.fk], base.quantity, base.price)
    rows = np.searchsorted(np.sort(base.dims[1].keys), base.fk[1])
    dense.fk[1] = (np.argsort(base.dims[1].keys)[rows] + 1).astype(np.int32)
    # all hashed: scattered distinct keys for every dimension
    dims_h, fk_h = [], []
    for d, dim in enumerate(base.dims):
        keys = rng.choice(np.arange(-(1 << 30), 1 << 30, 7, dtype=np.int64), dim.n, replace=False).astype(np.int32)
        dims_h.append(star.Dim(dim.name, dim.n, dim.attrs, dim.names, dim.lo, dim.hi, keys))
        fk_h.append(keys[dense.fk[d] - 1])
    hashed = star.StarData(dims_h, fk_h, base.quantity, base.price)
    # strided keys (7 + 3 row): range-indexed, the larger dimensions through L2
    dims_s, fk_s = [], []
    for d, dim in enumerate(base.dims):
        keys = (7 + 3 * np.arange(dim.n, dtype=np.int64)).astype(np.int32)[::-1].copy()
        dims_s.append(star.Dim(dim.name, dim.n, dim.attrs, dim.names, dim.lo, dim.hi, keys))
        fk_s.append(keys[dense.fk[d] - 1])
    strided = star.StarData(dims_s, fk_s, base.quantity, base.price)
    for data in (dense, hashed, strided):
        p = star.StarPlan(ctx, data)
        out = p.run(qs)
        ctx.sync()
        check(star.StarPlan.results(out, len(qs)), [oracle.star_query(data, q, threads=cpu_threads()) for q in qs])
        p.close()


def test_star_duplicate_primary_key_refused(ctx):
    data = star.gen_star(3, n_fact=1 << 12, dim_rows=SMALL_DIMS)
    data.dims[1].keys = data.dims[1].keys.copy()
    data.dims[1].keys[100] = data.dims[1].keys[7]
    with pytest.raises(abi.GbjError) as e:
        star.StarPlan(ctx, data)
    assert e.value.code == abi.ERR_INVALID


def test_star_invalid_requests(ctx, plan, data):
    good = star.gen_queries(1, 1, data.dims)[0]
    bad = []
    q = star.gen_queries(1, 1, data.dims)[0]
    q.join_mask = 0
    bad.append(q)
    q = star.gen_queries(1, 1, data.dims)[0]
    q.join_mask = 1 << 5
    bad.append(q)
    q = star.gen_queries(1, 1, data.dims)[0]
    q.join_mask = 0b0001
    q.group_dim = [0, 2]  # dimension 2 is not joined
    bad.append(q)
    q = star.Query(join_mask=0b0101, group_dim=[0, 2], group_attr=[2, 2])  # 250 x 1000 groups
    bad.append(q)
    for q in bad:
        with pytest.raises(abi.GbjError) as e:
            plan.run([q])
        assert e.value.code == abi.ERR_INVALID
    with pytest.raises(abi.GbjError):
        plan.run([good] * 65)
    out = plan.run([good])  # the plan still works
    ctx.sync()
    assert int(out["n"][0]) > 0


def test_star_full_size(ctx, oracle):
    """2^28-row fact, full dimensions, 64 queries in one graph replay; eight
    of them checked against the oracle on the full fact table."""
    d = star.gen_star(2026, n_fact=star.FULL_FACT_ROWS)
    p = star.StarPlan(ctx, d)
    qs = star.gen_queries(2026, 64, d.dims)
    out = p.run(qs, use_graph=True)
    ctx.sync()
    got = star.StarPlan.results(out, len(qs))
    for i in range(0, 64, 8):
        check([got[i]], [oracle.star_query(d, qs[i], threads=cpu_threads())])
    p.close()
