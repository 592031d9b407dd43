"""The request loop against the oracle: every request's answer equals the
reference rule on the same molecules, and is the same whether the request
is served alone or batched with others arriving at the same time."""
import threading
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _db(n=6000):
    from siml_gb300 import synthetic as S
    return S.smiles_set(S.SEED_SERVING, S.UNIFORM_20_90, n)


def _requests(rng, nreq, first, kinds=("topk", "threshold"), max_q=40, k=10):
    from siml_gb300 import synthetic as S
    from siml_gb300.serving import Request
    out, pos = [], first
    for i in range(nreq):
        q = int(rng.integers(1, max_q + 1))
        smi = S.smiles_list(S.SEED_SERVING, S.UNIFORM_20_90, q, first=pos)
        pos += q
        out.append(Request(i, smi, kind=kinds[i % len(kinds)], k=k, lo=0.75))
    return out


def _oracle_answer(oracle, db, req, lo=0.75):
    qs = oracle.compile_strings(req.smiles)
    if req.kind == "topk":
        oi, os_ = oracle.topk_block(qs, db, 0, req.rows, req.k)
        return [(oi[r], os_[r]) for r in range(req.rows)]
    nq = db[0].shape[0]
    oi, osm, oc = oracle.neighbors_block(qs, db, 0, req.rows, lo, 1.1, nq)
    return [(oi[r, :oc[r]], osm[r, :oc[r]]) for r in range(req.rows)]


def _same(a, b):
    return len(a) == len(b) and all(np.array_equal(x[0], y[0]) and
                                    np.array_equal(np.asarray(x[1]).view(np.uint32), np.asarray(y[1]).view(np.uint32))
                                    for x, y in zip(a, b))


def _server(db, **kw):
    from siml_gb300 import GPULingo
    from siml_gb300.serving import LingoServer, ServerConfig
    gl = GPULingo(0)
    gl.set_qsmiles(*db)
    return LingoServer(gl, ServerConfig(**kw))


def test_serving_mix_equals_alone_and_oracle(native, oracle):
    from siml_gb300.serving import Request, serve_unbatched
    base = _db()
    # 50 more copies of molecule 100: its threshold row has more hits than the
    # batch pitch, and its top-k ties at 1.0 resolve to the lowest indices
    index = np.arange(6000)
    index[2000:2050] = 100
    db = tuple(np.ascontiguousarray(a[index]) for a in base)
    from siml_gb300 import synthetic as S
    dup = S.smiles_list(S.SEED_SERVING, S.UNIFORM_20_90, 30, first=90)
    srv = _server(db, max_rows=64, width=128, kmax=16, pitch=32)
    rng = np.random.default_rng(5)
    reqs = _requests(rng, 40, first=6000)
    reqs.append(Request(999, dup, kind="threshold"))
    reqs.append(Request(998, dup[:7], kind="topk", k=16))
    srv.start()

    def feed():
        for r in reqs:
            r.arrival = time.perf_counter()
            srv.submit(r)
            time.sleep(float(rng.exponential(0.0005)))

    th = threading.Thread(target=feed)
    th.start()
    th.join()
    for r in reqs:
        assert r.done.wait(120), r.rid
    srv.stop()
    assert srv.batches < len(reqs)             # requests were batched together
    assert max(srv.batch_rows) <= 64
    for r in reqs:
        assert r.error is None, r.error
        assert _same(r.result, _oracle_answer(oracle, db, r)), r.rid
    # alone: the same requests one at a time through the per-request path
    for r in reqs[:12] + reqs[-2:]:
        a = Request(r.rid, r.smiles, kind=r.kind, k=r.k)
        serve_unbatched(srv, a)
        assert _same(a.result, r.result), r.rid
    assert any(len(x[0]) > 32 for x in reqs[-2].result)   # a row re-run past the batch pitch


def test_serving_admission_limits(native):
    from siml_gb300.serving import Request
    db = _db(3000)
    srv = _server(db, max_rows=16, width=128, kmax=8, pitch=16, hit_budget=16 * 8 * 8)
    from siml_gb300 import synthetic as S
    smi = S.smiles_list(S.SEED_SERVING, S.UNIFORM_20_90, 17, first=3000)
    with pytest.raises(ValueError):
        srv.submit(Request(0, smi, kind="topk", k=8))        # more rows than a batch
    with pytest.raises(ValueError):
        srv.submit(Request(1, smi[:3], kind="topk", k=9))    # k above kmax
    wide = bytes(np.random.default_rng(4).choice(np.frombuffer(b"CNOSPFcnosp()=#[]", np.uint8), 400))
    with pytest.raises(ValueError):
        srv.submit(Request(2, [smi[0], wide], kind="topk", k=8))   # more unique LINGOs than the rows hold
    reqs = [Request(i, smi[i:i + 5], kind="topk", k=8) for i in range(6)]
    srv.start()
    for r in reqs:
        srv.submit(r)
    for r in reqs:
        assert r.done.wait(60)
    srv.stop()
    # three 5-row requests fit a 16-row batch; the memory budget (16 rows x 8 hits) admits three too
    assert max(srv.batch_rows) <= 15
    assert all(r.error is None for r in reqs)


def test_serving_defers_batches_while_device_memory_is_held(native, oracle):
    """Admission by free device memory: while the free-memory reading is
    below the oldest request's hit buffers (as when another tenant holds the
    GPU's memory) no batch forms and no request fails; once the reading
    rises the queued requests are served, each with the answer it gets
    alone and the oracle's."""
    from siml_gb300.serving import serve_unbatched, Request
    db = _db()
    state = {"probes": 0}

    def probe():
        state["probes"] += 1
        # 64 bytes (below one query row's hit buffers), then plenty
        return 64 if state["probes"] < 40 else 1 << 34

    srv = _server(db, max_rows=256, width=128, kmax=16, pitch=256, lo=0.75, mem_reserve=0, mem_probe=probe,
                  mem_poll_s=0.002)
    rng = np.random.default_rng(11)
    reqs = _requests(rng, 12, 6000, max_q=60)
    for r in reqs:
        srv.submit(r)
    t0 = time.perf_counter()
    srv.start()
    for r in reqs:
        assert r.done.wait(120), r.rid
    srv.stop()
    assert srv.deferrals >= 30 and state["probes"] >= 40
    assert min(r.t_admit for r in reqs) - t0 > 0.05   # nothing admitted while memory was short
    for r in reqs:
        assert r.error is None, r.error
        a = Request(r.rid, r.smiles, kind=r.kind, k=r.k, lo=r.lo)
        serve_unbatched(srv, a)
        assert _same(a.result, r.result), r.rid
    for r in reqs[:3]:
        assert _same(r.result, _oracle_answer(oracle, db, r)), r.rid
