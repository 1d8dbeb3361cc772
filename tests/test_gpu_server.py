"""GPU: the serving loop.  Requests submitted concurrently from several
client threads are batched on the fly over two lanes; every result must be
bit-identical to the same request evaluated alone.  Host-side fault
injection: a request cancelled while queued, a bounded wait that runs out.
"""
import threading

import numpy as np
import pytest

from conftest import load_case

pytestmark = pytest.mark.gpu

CASES = ["three_streams", "cut_area", "config0", "four_streams_c120"]


@pytest.fixture(scope="module")
def served(built_library):
    import milkywayathome_client_gb300 as mw
    ctx = mw.Context(0)
    wedges, keep = [], []
    for name in CASES:
        pf, sf, g = load_case(name)
        ap, sp = mw.AstronomyParameters.read(pf), mw.StarPoints.read(sf)
        keep.append((ap, sp))
        wedges.append((ctx.add_wedge(ap, sp), np.asarray(g["theta"])))
    yield ctx, wedges
    ctx.close()


def _workload(wedges, n, seed):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        w, base = wedges[rng.integers(len(wedges))]
        out.append((w, base * (1.0 + 0.002 * rng.standard_normal(base.size)), int(rng.integers(2))))
    return out


def test_served_results_equal_alone(served):
    import milkywayathome_client_gb300 as mw
    ctx, wedges = served
    work = _workload(wedges, 48, 11)
    alone = [ctx.evaluate_requests([(w, t)], p)[0] for w, t, p in work]
    with mw.Server(ctx, lanes=2, max_batch=16) as srv:
        ids = [None] * len(work)

        def client(k):
            for i in range(k, len(work), 4):
                w, t, p = work[i]
                ids[i] = srv.submit(w, t, p)

        ths = [threading.Thread(target=client, args=(k,)) for k in range(4)]
        for th in ths:
            th.start()
        for th in ths:
            th.join()
        got = [srv.wait(i, timeout=300) for i in ids]
        st = srv.stats()
    for a, b in zip(alone, got):
        assert a.likelihood == b.likelihood or (a.likelihood != a.likelihood and b.likelihood != b.likelihood)
        assert a.integrals == b.integrals
    assert st["completed"] == len(work)
    assert st["batches"] <= len(work)
    assert 0 < st["p50_latency_s"] <= st["p99_latency_s"] <= st["max_latency_s"]


def test_served_double_float_equal_alone(served):
    """The double-float form through the server: requests of all three
    forms interleaved, each batch one form, results bit-identical to the
    request evaluated alone."""
    import milkywayathome_client_gb300 as mw
    ctx, wedges = served
    rng = np.random.default_rng(29)
    work = [(w, t, int(rng.integers(3))) for w, t, _ in _workload(wedges, 24, 29)]
    assert any(p == mw.MWSEP_PLAIN_DF for _, _, p in work)
    alone = [ctx.evaluate_requests([(w, t)], p)[0] for w, t, p in work]
    with mw.Server(ctx, lanes=2, max_batch=8) as srv:
        ids = [srv.submit(w, t, p) for w, t, p in work]
        got = [srv.wait(i, timeout=300) for i in ids]
    for a, b in zip(alone, got):
        assert a.integrals == b.integrals
        assert a.likelihood == b.likelihood or (a.likelihood != a.likelihood and b.likelihood != b.likelihood)


def test_cancel_and_timeout(served):
    import milkywayathome_client_gb300 as mw
    from milkywayathome_client_gb300 import native as N
    ctx, wedges = served
    w, base = wedges[2]  # config 0: ~1.5 ms per FP64 evaluation
    with mw.Server(ctx, lanes=1, max_batch=1) as srv:
        ids = [srv.submit(w, base, mw.MWSEP_PLAIN_F64) for _ in range(40)]
        last = ids[-1]
        rc = srv.cancel(last)
        st, res = srv.try_wait(last, 60.0)
        if rc == N.MWSEP_OK:
            assert st == N.MWSEP_ERR_CANCELLED and res is None
        else:  # it had already started
            assert rc == N.MWSEP_ERR_STATE and st == N.MWSEP_OK
        # a wait that cannot be satisfied in time returns TIMEOUT and the
        # request stays pending
        fresh = srv.submit(w, base, mw.MWSEP_PLAIN_F64)
        st0, _ = srv.try_wait(fresh, 0.0)
        assert st0 in (N.MWSEP_ERR_TIMEOUT, N.MWSEP_OK)
        if st0 == N.MWSEP_ERR_TIMEOUT:
            assert srv.wait(fresh, 300).likelihood == srv.wait(ids[0], 300).likelihood
        for i in ids[1:-1]:
            srv.wait(i, 300)


def test_lane_budget_refuses_and_server_keeps_serving(served):
    """A lane whose device-memory share cannot hold even one request reports
    MWSEP_ERR_BUDGET for it (admission by HBM footprint) and stays usable."""
    import milkywayathome_client_gb300 as mw
    from milkywayathome_client_gb300 import native as N
    ctx, wedges = served
    w, base = wedges[0]
    with mw.Server(ctx, lanes=1, max_batch=8, lane_hbm_bytes=1) as srv:
        ids = [srv.submit(w, base, mw.MWSEP_MIXED_F32) for _ in range(3)]
        for i in ids:
            st, res = srv.try_wait(i, 300)
            assert st == N.MWSEP_ERR_BUDGET and res is None
        s = srv.stats()
        assert s["failed"] == 3 and s["completed"] == 0


def test_destroy_with_queued_requests_returns(served):
    """Destroying a server with work queued cancels the queue, lets the
    running batch finish, and returns."""
    import time
    import milkywayathome_client_gb300 as mw
    ctx, wedges = served
    w, base = wedges[2]
    srv = mw.Server(ctx, lanes=1, max_batch=1)
    for _ in range(50):
        srv.submit(w, base, mw.MWSEP_PLAIN_F64)
    t0 = time.perf_counter()
    srv.close()
    assert time.perf_counter() - t0 < 120
    # the context still evaluates afterwards
    r = ctx.evaluate_requests([(w, base)], mw.MWSEP_PLAIN_F64)[0]
    assert r.likelihood == r.likelihood


def test_admission_queue_bound_refuses_with_busy(served):
    """With max_queued set, a submit that finds that many requests waiting is
    refused at once with MWSEP_ERR_BUSY; accepted requests complete with the
    same bits as alone and the stats count the refusals."""
    import milkywayathome_client_gb300 as mw
    from milkywayathome_client_gb300 import native as N
    ctx, wedges = served
    w, base = wedges[2]  # config 0 in plain FP64: ~1.5 ms per evaluation
    want = ctx.evaluate_requests([(w, base)], mw.MWSEP_PLAIN_F64)[0]
    with mw.Server(ctx, lanes=1, max_batch=1, max_queued=4) as srv:
        ids, busy = [], 0
        for _ in range(60):
            try:
                ids.append(srv.submit(w, base, mw.MWSEP_PLAIN_F64))
            except mw.MwsepError as e:
                assert e.status == N.MWSEP_ERR_BUSY
                busy += 1
        for i in ids:
            assert srv.wait(i, 300).likelihood == want.likelihood
        st = srv.stats()
    assert busy > 0 and st["refused"] == busy
    assert st["completed"] == len(ids) and st["max_queue"] <= 4


def test_time_capped_batches(served):
    """target_batch_ms caps a lane's batch by predicted device time: with a
    cap far below one evaluation every batch holds one request, and results
    still equal the requests evaluated alone."""
    import milkywayathome_client_gb300 as mw
    ctx, wedges = served
    work = _workload(wedges, 24, 5)
    alone = [ctx.evaluate_requests([(w, t)], p)[0] for w, t, p in work]
    assert all(ctx.wedge_points(w) > 0 for w, _ in wedges)
    with mw.Server(ctx, lanes=1, max_batch=64, target_batch_ms=1e-6) as srv:
        ids = [srv.submit(w, t, p) for w, t, p in work]
        got = [srv.wait(i, timeout=300) for i in ids]
        st = srv.stats()
    assert st["batches"] == len(work)
    for a, b in zip(alone, got):
        assert a.integrals == b.integrals
