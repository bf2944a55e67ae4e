"""Failure handling without a GPU fault: every failure is made on the host
(a pool cap, a paused request loop, an undersized group table, a too-small
output buffer) and must come back as a status, with the context and server
still usable afterwards."""
import pytest

from gpu_util import CONFIG2_AGGS, cpu_threads, dev, host
from proteus_gb300 import abi, engine, serve

pytestmark = pytest.mark.gpu


def test_pool_limit_gives_oom_then_recovers(ctx, oracle):
    rk, _ = engine.gen_build_side(61, 1 << 18, payload=False)
    sk, _ = engine.gen_probe_zipf(61, 1 << 20, 1 << 18, 0.5, 0.5)
    d_r, d_s = dev(rk), dev(sk)
    ctx.sync()
    ctx.set_pool_limit(1 << 20)  # far below the partition buffers' needs
    try:
        with pytest.raises(abi.GbjError) as e:
            ctx.radix_join_agg(d_r, None, d_s, None, CONFIG2_AGGS)
        assert e.value.code == abi.ERR_OOM and "limit" in str(e.value)
    finally:
        ctx.set_pool_limit(0)
    out = ctx.radix_join_agg(d_r, None, d_s, None, CONFIG2_AGGS)
    ctx.sync()
    assert host(out).tolist() == oracle.radix_join_agg(rk, None, sk, None, CONFIG2_AGGS,
                                                       threads=cpu_threads())


def _query(seed, nb, npr, card):
    sh = serve.QueryShape(nb, npr, 0.8, card, seed)
    cols = serve.gen_query(sh)
    return sh, cols, tuple(dev(a) for a in cols)


def test_server_wait_timeout_cancel_and_resume(ctx, oracle):
    srv = serve.Server(ctx, max_batch=8, max_inflight=2)
    try:
        srv.pause(True)
        qs = [_query(900 + i, 1 << 12, 1 << 15, 50) for i in range(3)]
        outs = [serve.Output(64) for _ in qs]
        tk = [srv.submit(*d, 50, o) for (_, _, d), o in zip(qs, outs)]
        # nothing runs while paused: a bounded wait gives up with TIMEOUT
        with pytest.raises(abi.GbjError) as e:
            srv.wait(tk[0], timeout=0.2)
        assert e.value.code == abi.ERR_TIMEOUT
        assert srv.cancel(tk[1])
        assert srv.wait(tk[1], timeout=1.0) == abi.ERR_CANCELLED
        assert not srv.cancel(tk[1])  # already complete
        srv.pause(False)
        for i in (0, 2):
            assert srv.wait(tk[i], timeout=60.0) == abi.OK
            eg, ec, es, _, _ = oracle.join_groupby(*qs[i][1])
            g, c, s_ = outs[i].sorted()
            assert (g == eg).all() and (c == ec).all() and (s_ == es).all()
        assert not srv.cancel(tk[0])  # launched and done: left alone
    finally:
        srv.close()


def test_server_group_overflow_is_retried(ctx, oracle):
    """expected_groups far below the build's distinct groups: the group table
    overflows, the server runs the query once more with room for every
    build row as a group, and the result is exact."""
    srv = serve.Server(ctx, max_batch=4, max_inflight=2)
    try:
        sh, cols, d = _query(931, 1 << 14, 1 << 17, 3000)
        out = serve.Output(1 << 14)
        t = srv.submit(*d, 8, out)  # 8 expected groups, about 3000 real ones
        assert srv.wait(t, timeout=60.0) == abi.OK
        assert srv.retries() == 1
        eg, ec, es, _, _ = oracle.join_groupby(*cols)
        g, c, s_ = out.sorted()
        assert (g == eg).all() and (c == ec).all() and (s_ == es).all()
        # a registered table is rebuilt the same way
        tid = srv.register_table(d[0], d[1], 4)
        assert srv.retries() == 2
        out2 = serve.Output(1 << 14)
        t2 = srv.submit(None, None, d[2], d[3], 4, out2, table=tid)
        assert srv.wait(t2, timeout=60.0) == abi.OK
        g, c, s_ = out2.sorted()
        assert (g == eg).all() and (c == ec).all() and (s_ == es).all()
        srv.unregister_table(tid)
    finally:
        srv.close()


def test_server_output_capacity_reported(ctx):
    """Too small an output buffer is the caller's limit: no retry, CAPACITY."""
    srv = serve.Server(ctx, max_batch=4, max_inflight=1)
    try:
        sh, cols, d = _query(941, 1 << 13, 1 << 15, 500)
        out = serve.Output(16)
        t = srv.submit(*d, 500, out)
        assert srv.wait(t, timeout=60.0) == abi.ERR_CAPACITY
        assert srv.retries() == 0
        # the server goes on serving
        out2 = serve.Output(1024)
        assert srv.wait(srv.submit(*d, 500, out2), timeout=60.0) == abi.OK
    finally:
        srv.close()


def test_server_pool_limit_gives_oom(ctx):
    """A query the capped pool cannot hold, with nothing in flight to free
    memory, completes with GBJ_ERR_OOM instead of waiting forever."""
    srv = serve.Server(ctx, max_batch=4, max_inflight=1)
    try:
        sh, cols, d = _query(951, 1 << 16, 1 << 16, 100)
        ctx.set_pool_limit(ctx.pool_stats()["in_use"] + (1 << 12))
        out = serve.Output(256)
        t = srv.submit(*d, 100, out)
        assert srv.wait(t, timeout=60.0) == abi.ERR_OOM
    finally:
        ctx.set_pool_limit(0)
        srv.close()
