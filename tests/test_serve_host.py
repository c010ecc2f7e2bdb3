"""CPU tests of the serving loop's host-side logic (admission, continuous batching, cancellation, timeouts, shutdown),
run on the test executor: no CUDA call is made, meshes are not built (their size is estimated) and a batch finishes
test_ns_per_query x its queries after it starts. Failures are made on the host: requests that cannot fit, cancelled
requests, waits that run out, a server shut down with work pending."""

import time

import numpy as np
import pytest

from thea_gb300 import _native as N
from thea_gb300 import workloads as W


@pytest.fixture(scope="module")
def lib():
    from thea_gb300 import build as B
    B.build()
    return N.lib()


@pytest.fixture(scope="module")
def mesh():
    return W.noisy_icosphere(2, 7)


def server(lib, **kw):
    from thea_gb300.serve import Server
    kw.setdefault("test_executor", True)
    return Server(**kw)


def q(n, seed=0):
    return np.random.default_rng(seed).uniform(-1.5, 1.5, (n, 3)).astype(np.float32)


def test_requests_of_every_kind_complete_and_are_counted(lib, mesh):
    with server(lib, test_ns_per_query=10) as s:
        a = s.add_mesh(*mesh)
        b = s.add_mesh(*mesh)
        st = s.stats()
        assert st["resident_meshes"] == 2 and st["resident_bytes"] > 0
        ts = []
        for i in range(30):
            kind = ("closest", "ray", "knn")[i % 3]
            n = 1 + 37 * i
            d = q(n, 100 + i) if kind == "ray" else None
            ts.append(s.submit(kind, (a, b)[i % 2], q(n, i), directions=d, k=8))
        for t in ts:
            assert t.wait()
            assert t.status == N.THEA_OK and t.latency_ms >= 0
        st = s.stats()
        assert st["completed"] == 30 and st["failed"] == 0 and st["cancelled"] == 0
        assert st["queries_completed"] == sum(1 + 37 * i for i in range(30))
        assert st["batches"] >= 1 and st["p99_ms"] >= st["p50_ms"] > 0
        assert st["inflight_bytes"] == 0 and st["pending_requests"] == 0


def test_large_requests_are_cut_into_pieces_and_batches(lib, mesh):
    with server(lib, test_ns_per_query=1, max_piece_queries=1000, max_batch_queries=3000, slots=2) as s:
        m = s.add_mesh(*mesh)
        t = s.submit("closest", m, q(10500))
        assert t.wait() and t.status == N.THEA_OK
        # 11 pieces of at most 1000 queries, at most 3 per batch
        assert s.stats()["batches"] >= 4


def test_mesh_over_budget_is_refused(lib, mesh):
    with server(lib, memory_budget_bytes=4096) as s:
        with pytest.raises(N.TheaError) as e:
            s.add_mesh(*mesh)
        assert e.value.status == N.THEA_ERR_ADMISSION_REFUSED
        assert s.stats()["resident_meshes"] == 0


def test_request_that_can_never_fit_is_refused_at_submit(lib, mesh):
    V, F = mesh
    with server(lib, test_ns_per_query=1) as s:
        m = s.add_mesh(V, F)
        resident = s.stats()["resident_bytes"]
    # budget = resident + room for about 100 closest-point queries (12 B in + 8 B out each)
    with server(lib, test_ns_per_query=1, memory_budget_bytes=resident + 2000, max_piece_queries=500) as s:
        m = s.add_mesh(V, F)
        with pytest.raises(N.TheaError) as e:
            s.submit("closest", m, q(5000))
        assert e.value.status == N.THEA_ERR_ADMISSION_REFUSED
        assert s.stats()["refused"] == 1
        # a request that fits still runs
        t = s.submit("closest", m, q(50))
        assert t.wait() and t.status == N.THEA_OK


def test_memory_budget_throttles_but_everything_finishes(lib, mesh):
    V, F = mesh
    with server(lib) as s:
        resident = s.stats()["resident_bytes"] + s.add_mesh(V, F) * 0
        resident = s.stats()["resident_bytes"]
    # room for one piece of 1000 queries at a time
    budget = resident + 1000 * 20 + 100
    with server(lib, test_ns_per_query=2000, memory_budget_bytes=budget, max_piece_queries=1000, slots=3) as s:
        m = s.add_mesh(V, F)
        ts = [s.submit("closest", m, q(1000, i)) for i in range(6)]
        peak = 0
        while not all(t.wait(0) for t in ts):
            st = s.stats()
            peak = max(peak, st["inflight_bytes"])
            assert st["inflight_bytes"] + st["resident_bytes"] <= budget
            time.sleep(0.0005)
        assert all(t.status == N.THEA_OK for t in ts)
        assert 0 < peak <= 1000 * 20


def test_cancel_pending_request(lib, mesh):
    with server(lib, test_ns_per_query=20000, slots=1, max_piece_queries=1000, max_batch_queries=1000) as s:
        m = s.add_mesh(*mesh)
        busy = s.submit("closest", m, q(1000))   # about 20 ms on the only slot
        time.sleep(0.002)
        victim = s.submit("closest", m, q(5000))
        victim.cancel()
        assert victim.wait() and victim.status == N.THEA_ERR_CANCELLED
        assert busy.wait() and busy.status == N.THEA_OK
        st = s.stats()
        assert st["cancelled"] == 1 and st["completed"] == 1


def test_wait_timeout_then_completion(lib, mesh):
    with server(lib, test_ns_per_query=50000) as s:
        m = s.add_mesh(*mesh)
        t = s.submit("knn", m, q(400), k=4)      # about 20 ms
        assert t.wait(timeout_us=1000) is False
        assert t.status is None
        assert t.wait() and t.status == N.THEA_OK


def test_smallest_remaining_request_goes_first(lib, mesh):
    with server(lib, test_ns_per_query=10000, slots=1, max_piece_queries=500, max_batch_queries=500,
                max_wait_ms=10000) as s:
        m = s.add_mesh(*mesh)
        first = s.submit("closest", m, q(500))    # occupies the slot for about 5 ms
        time.sleep(0.001)
        big = s.submit("closest", m, q(5000))
        small = s.submit("closest", m, q(10))
        for t in (first, big, small):
            assert t.wait() and t.status == N.THEA_OK
        assert small.latency_ms < big.latency_ms


def test_removed_mesh_takes_no_new_requests_and_is_released_after_its_requests(lib, mesh):
    with server(lib, test_ns_per_query=20000) as s:
        m = s.add_mesh(*mesh)
        keep = s.add_mesh(*mesh)
        before = s.stats()["resident_bytes"]
        t = s.submit("ray", m, q(500), directions=q(500, 1))
        s.remove_mesh(m)
        with pytest.raises(N.TheaError) as e:
            s.submit("closest", m, q(5))
        assert e.value.status == N.THEA_ERR_INVALID_ARGUMENT
        assert t.wait() and t.status == N.THEA_OK
        st = s.stats()
        assert st["resident_meshes"] == 1 and st["resident_bytes"] == before // 2
        assert s.submit("closest", keep, q(5)).wait()


def test_invalid_requests_are_rejected(lib, mesh):
    with server(lib) as s:
        m = s.add_mesh(*mesh)
        for kw in (dict(kind="closest", mesh=m + 5, queries=q(4)), dict(kind="knn", mesh=m, queries=q(4), k=0),
                   dict(kind="knn", mesh=m, queries=q(4), k=33), dict(kind="closest", mesh=m, queries=q(0)),
                   dict(kind="ray", mesh=m, queries=q(4))):
            with pytest.raises(N.TheaError) as e:
                s.submit(**kw)
            assert e.value.status == N.THEA_ERR_INVALID_ARGUMENT


def test_shutdown_with_pending_work_returns(lib, mesh):
    s = server(lib, test_ns_per_query=1000, slots=1, max_piece_queries=1000, max_batch_queries=1000)
    m = s.add_mesh(*mesh)
    keep = [s.submit("closest", m, q(1000, i)) for i in range(50)]  # about 50 ms of queued work
    t0 = time.perf_counter()
    s.close()
    assert time.perf_counter() - t0 < 5.0
    del keep
