"""Query serving (gbj_server_*) on the GPU: results against the oracle's
join -> group-by restatement, alone vs in a mix, plain vs batched forms,
admission by budget and error statuses."""
import numpy as np
import pytest

from gpu_util import cpu_threads, dev
from proteus_gb300 import abi, serve

pytestmark = pytest.mark.gpu

SMALL = dict(log_build=(10, 16), log_probe=(14, 19), log_card=(4, 12))


def expected(oracle, cols):
    g, c, s, _, _ = oracle.join_groupby(*cols, threads=cpu_threads())
    return g, c, s


def same(got, exp):
    assert len(got[0]) == len(exp[0])
    for a, b in zip(got, exp):
        assert (a == b).all()


@pytest.fixture(scope="module")
def workload(oracle):
    shapes = serve.gen_shapes(5, 40, **SMALL)
    host = [serve.gen_query(s) for s in shapes]
    devc = [tuple(dev(a) for a in h) for h in host]
    exp = [expected(oracle, h) for h in host]
    return shapes, devc, exp


def run_all(server, shapes, devc, order=None, together=False):
    order = list(range(len(shapes))) if order is None else order
    outs, tickets = {}, {}
    for i in order:
        cap = min(shapes[i].cardinality, shapes[i].n_build) + 8
        outs[i] = serve.Output(cap)
    if together:
        tk = server.submit_many([(*devc[i], shapes[i].cardinality, outs[i]) for i in order])
        tickets = dict(zip(order, tk))
    for i in order:
        if not together:
            tickets[i] = server.submit(*devc[i], shapes[i].cardinality, outs[i])
    status = {i: server.wait(t, timeout=120.0) for i, t in tickets.items()}
    return outs, status, tickets


@pytest.mark.parametrize("mode", ["batched_graph", "batched", "plain", "two_class"])
def test_serve_parity(ctx, workload, mode):
    shapes, devc, exp = workload
    if mode == "plain":
        srv = serve.Server.plain(ctx)
    elif mode == "two_class":
        # queries above 2^17 rows take the large-query slots
        srv = serve.Server(ctx, max_batch=16, max_inflight=4, large_slots=2, small_rows=1 << 17)
    else:
        srv = serve.Server(ctx, max_batch=16, max_inflight=3, use_graph=(mode == "batched_graph"))
    # queued together, so the request loop can batch them
    outs, status, _ = run_all(srv, shapes, devc, together=True)
    for i in outs:
        assert status[i] == abi.OK, i
        same(outs[i].sorted(), exp[i])
    st = srv.stats()
    assert st["completed"] == len(shapes)
    if mode == "plain":
        assert st["batches"] == len(shapes)
    else:
        assert st["batches"] < len(shapes)
    srv.close()


def test_serve_alone_equals_in_mix(ctx, workload):
    """Each query's result is the same run alone and inside a mix."""
    shapes, devc, exp = workload
    mix = serve.Server(ctx, max_batch=64, max_inflight=2)
    outs_mix, st_mix, _ = run_all(mix, shapes, devc, order=list(reversed(range(len(shapes)))))
    mix.close()
    alone = serve.Server(ctx, max_batch=64, max_inflight=2)
    for i in (0, 7, 21, 39):
        o, st, _ = run_all(alone, shapes, devc, order=[i])
        assert st[i] == abi.OK and st_mix[i] == abi.OK
        same(o[i].sorted(), outs_mix[i].sorted())
        same(o[i].sorted(), exp[i])
    alone.close()


def test_serve_budget_admission(ctx, workload):
    shapes, devc, exp = workload
    # budget fits about two of the largest queries at a time
    from proteus_gb300 import serve as S

    biggest = max(shapes, key=lambda s: s.n_build)
    tslots = 1 << max(10, (2 * biggest.n_build - 1).bit_length())
    budget = 2 * (tslots * 8 + (1 << 14) * 20 + 4096)
    srv = S.Server(ctx, hbm_budget=budget, max_batch=64, max_inflight=4)
    outs, status, _ = run_all(srv, shapes, devc)
    for i in outs:
        assert status[i] == abi.OK
        same(outs[i].sorted(), exp[i])
    assert 0 < srv.stats()["peak_bytes"] <= budget
    srv.close()
    # a query larger than the whole budget is refused, the others still run
    srv = S.Server(ctx, hbm_budget=budget // 8, max_batch=8, max_inflight=2)
    outs, status, _ = run_all(srv, shapes, devc, order=[shapes.index(biggest), 0])
    assert status[shapes.index(biggest)] == abi.ERR_BUDGET
    srv.close()
    # every query refused: the waiters still return
    srv = S.Server(ctx, hbm_budget=4096, max_batch=8, max_inflight=2)
    outs, status, _ = run_all(srv, shapes, devc, order=[0, 1, 2])
    assert set(status.values()) == {abi.ERR_BUDGET}
    srv.close()


def test_serve_output_capacity_status(ctx, workload):
    shapes, devc, _ = workload
    i = max(range(len(shapes)), key=lambda j: min(shapes[j].cardinality, shapes[j].n_build))
    srv = serve.Server(ctx)
    out = serve.Output(4)
    t = srv.submit(*devc[i], shapes[i].cardinality, out)
    assert srv.wait(t, timeout=120.0) == abi.ERR_CAPACITY
    srv.close()


def test_serve_duplicates_int32_min_and_empty(ctx, oracle):
    import torch

    rng = np.random.default_rng(3)
    bk = rng.integers(-50, 50, 5000).astype(np.int32)  # many duplicate keys
    bg = rng.integers(-3, 3, 5000).astype(np.int32)
    bg[::17] = np.iinfo(np.int32).min
    pk = rng.integers(-60, 60, 70000).astype(np.int32)
    pk[::5] = np.iinfo(np.int32).min
    pv = rng.integers(-1000, 1000, 70000).astype(np.int32)
    srv = serve.Server(ctx, max_batch=4)
    cases = [(bk, bg, pk, pv), (bk[:0], bg[:0], pk, pv), (bk, bg, pk[:0], pv[:0])]
    outs, tickets = [], []
    for c in cases:
        o = serve.Output(64)
        outs.append(o)
        tickets.append(srv.submit(*[dev(a) if len(a) else torch.empty(0, dtype=torch.int32, device="cuda")
                                    for a in c], 8, o))
    for c, o, t in zip(cases, outs, tickets):
        assert srv.wait(t, timeout=120.0) == abi.OK
        same(o.sorted(), expected(oracle, c))
    srv.close()


def test_serve_larger_queries(ctx, oracle):
    """A mix that includes 2^22-row builds and 2^25-row probes."""
    shapes = serve.gen_shapes(17, 6, log_build=(16, 22), log_probe=(20, 25), log_card=(4, 16))
    host = [serve.gen_query(s) for s in shapes]
    devc = [tuple(dev(a) for a in h) for h in host]
    srv = serve.Server(ctx, max_batch=8, max_inflight=2)
    outs, status, _ = run_all(srv, shapes, devc)
    for i in outs:
        assert status[i] == abi.OK
        same(outs[i].sorted(), expected(oracle, host[i]))
    srv.close()


@pytest.mark.parametrize("use_graph", [True, False])
def test_serve_resident_tables(ctx, oracle, use_graph):
    """Queries against registered (resident) build tables, mixed with queries
    that build their own, give the oracle's results; the tables survive many
    batches and several queries read one table in the same batch."""
    import torch

    rng = np.random.default_rng(11)
    builds = []
    for nb, card in [(5000, 40), (1 << 15, 3000), (300, 7)]:
        bk = rng.integers(-nb, nb, nb).astype(np.int32)  # duplicates included
        bg = rng.integers(-card, card, nb).astype(np.int32)
        bk[::97] = np.iinfo(np.int32).min
        bg[::31] = np.iinfo(np.int32).min
        builds.append((bk, bg, 2 * card + 2))
    srv = serve.Server(ctx, max_batch=16, max_inflight=3, use_graph=use_graph)
    ids = [srv.register_table(dev(bk), dev(bg), eg) for bk, bg, eg in builds]
    assert len(set(ids)) == 3 and 0 not in ids
    held = srv.stats()["peak_bytes"]
    assert held > 0
    qs, exp = [], []
    for r in range(4):  # rounds of queries, so every table serves many batches
        for j in range(12):
            b = j % 3
            bk, bg, eg = builds[b]
            npb = int(rng.integers(0, 40000))
            pk = rng.integers(-len(bk) - 5, len(bk) + 5, npb).astype(np.int32)
            pk[::13] = np.iinfo(np.int32).min
            pv = rng.integers(-1000, 1000, npb).astype(np.int32)
            resident = (j % 4) != 3
            qs.append((b, resident, dev(bk), dev(bg), dev(pk) if npb else torch.empty(0, dtype=torch.int32,
                       device="cuda"), dev(pv) if npb else torch.empty(0, dtype=torch.int32, device="cuda"), eg))
            exp.append(expected(oracle, (bk, bg, pk, pv)))
    outs = [serve.Output(q[6] + 8) for q in qs]
    batch = [((None if q[1] else q[2]), (None if q[1] else q[3]), q[4], q[5], q[6], o, ids[q[0]] if q[1] else 0)
             for q, o in zip(qs, outs)]
    tickets = srv.submit_many(batch)
    for t, o, e in zip(tickets, outs, exp):
        assert srv.wait(t, timeout=120.0) == abi.OK
        same(o.sorted(), e)
    # one by one, after all the batches above
    for i in (0, 1, 2):
        o = serve.Output(qs[i][6] + 8)
        t = srv.submit(None, None, qs[i][4], qs[i][5], qs[i][6], o, table=ids[qs[i][0]])
        assert srv.wait(t, timeout=120.0) == abi.OK
        same(o.sorted(), exp[i])
    # unknown ids are refused; an unregistered table's id is unknown
    with pytest.raises(abi.GbjError):
        srv.submit(None, None, qs[0][4], qs[0][5], qs[0][6], serve.Output(8), table=12345)
    srv.unregister_table(ids[2])
    with pytest.raises(abi.GbjError):
        srv.unregister_table(ids[2])
    with pytest.raises(abi.GbjError):
        srv.submit(None, None, qs[2][4], qs[2][5], qs[2][6], serve.Output(8), table=ids[2])
    srv.close()


def test_serve_resident_table_budget(ctx):
    bk = dev(np.arange(1 << 16, dtype=np.int32))
    srv = serve.Server(ctx, hbm_budget=1 << 16)
    with pytest.raises(abi.GbjError) as e:
        srv.register_table(bk, bk, 1 << 16)
    assert e.value.code == abi.ERR_BUDGET
    srv.close()


def test_serve_duplicate_heavy_groups(ctx, oracle):
    """Every probe row matches thousands of build rows of two groups, so a
    group slot takes far more than 65535 matches within one work item; values
    at both int32 extremes."""
    i32 = np.iinfo(np.int32)
    rng = np.random.default_rng(17)
    bk = np.full(4000, 7, dtype=np.int32)
    bg = rng.integers(0, 2, 4000).astype(np.int32)
    pk = np.full(40000, 7, dtype=np.int32)
    pk[::9] = 8  # misses
    pv = np.where(rng.random(40000) < 0.5, i32.max, i32.min).astype(np.int32)
    for srv in (serve.Server(ctx, max_batch=4), serve.Server.plain(ctx)):
        o = serve.Output(8)
        t = srv.submit(dev(bk), dev(bg), dev(pk), dev(pv), 4, o)
        assert srv.wait(t, timeout=120.0) == abi.OK
        same(o.sorted(), expected(oracle, (bk, bg, pk, pv)))
        tid = srv.register_table(dev(bk), dev(bg), 4)
        o2 = serve.Output(8)
        t = srv.submit(None, None, dev(pk), dev(pv), 4, o2, table=tid)
        assert srv.wait(t, timeout=120.0) == abi.OK
        same(o2.sorted(), expected(oracle, (bk, bg, pk, pv)))
        srv.close()


def test_serve_resident_tables_released(ctx):
    """Tables still registered when the server is destroyed go back to the
    pool; so does an unregistered one."""
    bk = dev(np.arange(1 << 16, dtype=np.int32))
    ctx.sync()
    before = ctx.pool_stats()["in_use"]
    srv = serve.Server(ctx)
    a = srv.register_table(bk, bk, 1 << 16)
    srv.register_table(bk, bk, 1 << 16)
    assert ctx.pool_stats()["in_use"] > before
    srv.unregister_table(a)
    srv.close()
    ctx.sync()
    assert ctx.pool_stats()["in_use"] == before
