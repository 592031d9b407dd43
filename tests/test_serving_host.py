"""Host logic of the request loop (no GPU): admission into batches and the
latency percentiles."""
import collections
import threading

import pytest


def _fake_server(max_rows, pitch, kmax, hit_budget, free=1 << 40):
    """A server with no engine: the device's free memory is the reading of
    a probe the test controls (a one-element list)."""
    from siml_gb300.serving import LingoServer, ServerConfig
    srv = object.__new__(LingoServer)
    srv.free = [free]
    srv.cfg = ServerConfig(max_rows=max_rows, width=64, kmax=kmax, pitch=pitch, hit_budget=hit_budget,
                           mem_reserve=0, mem_probe=lambda: srv.free[0], mem_poll_s=0.001)
    srv.queue = collections.deque()
    srv.cv = threading.Condition()
    srv.stop_flag = False
    srv.deferrals = 0
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


def test_request_beyond_the_hit_budget_is_refused_at_submit():
    srv = _fake_server(max_rows=8, pitch=64, kmax=8, hit_budget=16)
    srv._compile = lambda req: None
    with pytest.raises(ValueError, match="hit memory"):
        srv.submit(_req(0, 8, "threshold"))
    assert not srv.queue


def test_admit_takes_the_oldest_requests_that_fit():
    from siml_gb300.serving import ServerConfig, admit
    cfg = ServerConfig(max_rows=16, width=64, kmax=8, pitch=16, hit_budget=1 << 20)
    q = [_req(0, 4, "threshold"), _req(1, 4), _req(2, 10), _req(3, 1)]
    need_thr = 4 * (16 * 8 + 4)
    assert [r.rid for r in admit(q, cfg, 1 << 20, 16)] == [0, 1]          # 10 more rows would pass 16
    assert [r.rid for r in admit(q, cfg, need_thr + 4 * 8 * 8, 64)] == [0, 1]   # memory for two requests only
    assert admit(q, cfg, need_thr - 1, 64) == []                            # not even the oldest: wait


def test_low_free_memory_defers_the_batch_until_memory_frees():
    """Another tenant holds the device memory: the oldest request's hit
    buffers do not fit, so no batch forms and nothing fails; the requests
    stay queued and form a batch once the free-memory reading rises."""
    srv = _fake_server(max_rows=16, pitch=16, kmax=8, hit_budget=1 << 20, free=100)
    reqs = [_req(0, 4, "threshold"), _req(1, 3)]
    srv.queue.extend(reqs)
    got = []
    th = threading.Thread(target=lambda: got.append(srv._take_batch()))
    th.start()
    th.join(0.2)
    assert th.is_alive() and not got                      # deferred, still waiting
    assert srv.deferrals > 10 and len(srv.queue) == 2
    assert all(r.error is None and not r.done.is_set() for r in reqs)
    srv.free[0] = 1 << 30                                  # the other tenant frees its memory
    th.join(5)
    assert not th.is_alive() and [r.rid for r in got[0]] == [0, 1]


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
                           hit_budget=1 << 20, mem_reserve=0, mem_probe=lambda: 1 << 40)
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


def test_start_freezes_the_heap_unless_told_not_to():
    """A server moves the objects alive at start into the collector's
    permanent generation (a full collection while serving then scans only
    newer objects); gc_freeze=False leaves the collector alone."""
    import gc
    srv = _fake_server(max_rows=8, pitch=64, kmax=8, hit_budget=1 << 20)
    srv.icv = threading.Condition()
    srv.threads = []
    srv._batcher = srv._completer = lambda: None
    keep = [[i] for i in range(2000)]
    try:
        gc.unfreeze()
        srv.start()
        srv.stop()
        assert gc.get_freeze_count() >= len(keep)
        gc.unfreeze()
        srv.cfg.gc_freeze = False
        srv.start()
        srv.stop()
        assert gc.get_freeze_count() == 0
    finally:
        gc.unfreeze()
