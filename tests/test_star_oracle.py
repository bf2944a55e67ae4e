"""The star-join oracle against an independent numpy formulation of the
same query (select -> join on dense primary keys -> group by two attributes),
and properties of the seeded star workload.  CPU only."""
import numpy as np
import pytest

from proteus_gb300 import star

SMALL_DIMS = (1 << 12, 2557, 1 << 10, 1 << 8)


def numpy_star(data, q):
    n = data.n_fact
    keep = np.ones(n, dtype=bool)
    rows = {}
    for d, dim in enumerate(data.dims):
        if not (q.join_mask >> d) & 1:
            continue
        ok = np.ones(dim.n, dtype=bool)
        if q.pred_attr[d] >= 0:
            col = dim.attrs[q.pred_attr[d]].astype(np.int64)
            ok = (col >= q.pred_lo[d]) & (col <= q.pred_hi[d])
        if dim.keys is None:
            r = data.fk[d].astype(np.int64) - 1
        else:  # key -> row through the sorted keys
            order = np.argsort(dim.keys, kind="stable")
            pos = np.searchsorted(dim.keys[order], data.fk[d])
            posc = np.minimum(pos, dim.n - 1)
            r = np.where(dim.keys[order][posc] == data.fk[d], order[posc], -1).astype(np.int64)
        inr = (r >= 0) & (r < dim.n)
        keep &= inr
        rc = np.where(inr, r, 0)
        keep &= ok[rc]
        rows[d] = rc
    a = data.dims[q.group_dim[0]].attrs[q.group_attr[0]][rows[q.group_dim[0]][keep]].astype(np.int64)
    b = data.dims[q.group_dim[1]].attrs[q.group_attr[1]][rows[q.group_dim[1]][keep]].astype(np.int64)
    v = data.price[keep].astype(np.int64) * data.quantity[keep].astype(np.int64)
    key = (a << 32) | (b & 0xFFFFFFFF)
    u, inv = np.unique(key, return_inverse=True)
    cnt = np.bincount(inv, minlength=len(u)).astype(np.int64)
    s = np.zeros(len(u), dtype=np.int64)
    np.add.at(s, inv, v)
    return (u >> 32).astype(np.int32), (u & 0xFFFFFFFF).astype(np.int32), cnt, s


@pytest.fixture(scope="module")
def small():
    return star.gen_star(11, n_fact=1 << 18, dim_rows=SMALL_DIMS)


def test_oracle_matches_numpy(small, oracle):
    for q in star.gen_queries(11, 16, small.dims):
        exp = numpy_star(small, q)
        for threads in (1, 3):
            got = oracle.star_query(small, q, threads=threads)
            assert len(got[0]) == len(exp[0]) > 0
            for g, e in zip(got, exp):
                assert (g == e).all()


def test_oracle_foreign_keys_outside_dimension(oracle):
    data = star.gen_star(5, n_fact=1 << 16, dim_rows=SMALL_DIMS)
    data.fk[0][::7] = 0
    data.fk[1][::11] = 19920100  # not a date key
    data.fk[1][::13] = SMALL_DIMS[1] + 3
    q = star.Query(join_mask=0b0011, group_dim=[0, 1], group_attr=[1, 1])
    exp = numpy_star(data, q)
    got = oracle.star_query(data, q, threads=2)
    for g, e in zip(got, exp):
        assert (g == e).all()


def test_workload_shape(lib):
    data = star.gen_star(3, n_fact=1 << 16, dim_rows=SMALL_DIMS)
    for d, dim in enumerate(data.dims):
        if dim.keys is None:
            assert data.fk[d].min() >= 1 and data.fk[d].max() <= dim.n
        else:
            assert np.isin(data.fk[d], dim.keys).all() and len(np.unique(dim.keys)) == dim.n
        for col, lo, hi in zip(dim.attrs, dim.lo, dim.hi):
            assert col.min() >= lo and col.max() <= hi
    assert data.quantity.min() >= 1 and data.quantity.max() <= 50
    assert data.price.min() >= 900 and data.price.max() <= 110000
    qs = star.gen_queries(3, 64, data.dims)
    assert qs == star.gen_queries(3, 64, data.dims)  # deterministic
    for q in qs:
        assert bin(q.join_mask).count("1") == 3
        assert q.group_dim[0] != q.group_dim[1]
        groups = 1
        for k in range(2):
            dim = data.dims[q.group_dim[k]]
            groups *= dim.hi[q.group_attr[k]] - dim.lo[q.group_attr[k]] + 1
        assert groups <= 25 * 25
        for d in range(4):
            if (q.join_mask >> d) & 1:
                dim = data.dims[d]
                a = q.pred_attr[d]
                frac = (q.pred_hi[d] - q.pred_lo[d] + 1) / (dim.hi[a] - dim.lo[a] + 1)
                assert 1 / 60 <= frac <= 1 / 4 + 1e-9, (q, frac)
