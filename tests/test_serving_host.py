"""Host logic of the request loop (no GPU): admission into batches and the
latency percentiles."""
import collections
import threading

import pytest


def _fake_server(max_rows, pitch, kmax, hit_budget):
    from siml_gb300.serving import LingoServer, ServerConfig
    srv = object.__new__(LingoServer)
    srv.cfg = ServerConfig(max_rows=max_rows, width=64, kmax=kmax, pitch=pitch, hit_budget=hit_budget)
    srv.queue = collections.deque()
    srv.cv = threading.Condition()
    srv.stop_flag = False
    return srv


def _req(i, rows, kind="topk", k=8):
    from siml_gb300.serving import Request
    return Request(i, [b"CCCCO"] * rows, kind=kind, k=k)


def test_admission_by_rows_and_memory():
    srv = _fake_server(max_rows=16, pitch=16, kmax=8, hit_budget=10 * 16 * 8 + 40)
    for i, (rows, kind) in enumerate([(5, "topk"), (6, "threshold"), (4, "threshold"), (3, "topk"), (10, "topk")]):
        srv.queue.append(_req(i, rows, kind))
    b1 = srv._take_batch()
    # rows 5 + 6 = 11 fit; the 4-row threshold request needs 4 x (16 x 8 + 4) bytes more than the budget left
    assert [r.rid for r in b1] == [0, 1]
    b2 = srv._take_batch()
    assert [r.rid for r in b2] == [2, 3]          # 10 more rows would pass 16
    b3 = srv._take_batch()
    assert [r.rid for r in b3] == [4]
    srv.stop_flag = True
    assert srv._take_batch() is None


def test_first_request_always_admitted():
    srv = _fake_server(max_rows=8, pitch=64, kmax=8, hit_budget=16)
    srv.queue.append(_req(0, 8, "threshold"))
    assert [r.rid for r in srv._take_batch()] == [0]


def test_percentiles():
    from siml_gb300.serving import percentiles
    v = list(range(1, 101))
    p = percentiles(v)
    assert p == {"p50": 50.0, "p95": 95.0, "p99": 99.0}
    assert percentiles([])["p99"] is None


def test_request_validation():
    from siml_gb300.serving import Request
    with pytest.raises(ValueError):
        Request(0, [b"CC"], kind="nearest")
    r = Request(1, ["CCO", b"CCN"], kind="threshold")
    assert r.rows == 2 and r.smiles == [b"CCO", b"CCN"]


def test_batches_grow_under_a_backlog():
    from siml_gb300.serving import ServerConfig
    srv = _fake_server(max_rows=16, pitch=16, kmax=8, hit_budget=1 << 20)
    srv.cfg = ServerConfig(max_rows=16, soft_rows=8, backlog_rows=20, width=64, kmax=8, pitch=16,
                           hit_budget=1 << 20)
    for i in range(3):
        srv.queue.append(_req(i, 5))
    assert [r.rid for r in srv._take_batch()] == [0]        # 15 queued rows: soft limit 8
    for i in range(3, 8):
        srv.queue.append(_req(i, 5))
    assert [r.rid for r in srv._take_batch()] == [1, 2, 3]  # 35 queued rows > 20: up to 16


def test_cancel_before_admission():
    """A cancelled request leaves the queue at once with a RequestCancelled
    error; one already taken into a batch cannot be cancelled."""
    from siml_gb300.serving import RequestCancelled
    srv = _fake_server(max_rows=8, pitch=16, kmax=8, hit_budget=1 << 20)
    reqs = [_req(i, 3) for i in range(4)]
    srv.queue.extend(reqs)
    b1 = srv._take_batch()
    assert [r.rid for r in b1] == [0, 1]
    assert not srv.cancel(reqs[0])                 # already in a batch
    assert srv.cancel(reqs[2])
    assert reqs[2].done.is_set() and isinstance(reqs[2].error, RequestCancelled)
    assert not srv.cancel(reqs[2])                 # no longer queued
    assert [r.rid for r in srv._take_batch()] == [3]
