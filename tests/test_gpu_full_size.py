"""Full-size checks on the 1,000,000-molecule database of the row-block and
fused-search workloads (lognormal lengths, median 45 chars), on the
2,000,000-molecule database of the ragged batched jobs and on the
10,000,000-molecule serving database.

The oracle computes a few complete rows bit for bit. Over the whole
1,024 x 1,000,000 block the tests check properties that hold at any size:
- a molecule's similarity with itself is 1;
- the block is symmetric where the ref rows are database molecules;
- getNeighbors, top-k and both histograms, each computed by its own fused
  kernel, are derived exactly from the rows block, with the rules the
  reference states: the fp32 magnitude bound, then lo <= t < hi, indices
  ascending (pysiml/kernels.py:437-448); bins (unsigned)(t*100) capped at 100
  (pysiml/kernels.py:660-661); top-k ties to the lower index; 1000 bins of
  min((unsigned)(t*1000), 999)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROWS = 1024
DB_N = 1_000_000


@pytest.fixture(scope="module")
def full(native):
    torch = pytest.importorskip("torch")
    from siml_gb300 import GPULingo, synthetic as S
    db = S.smiles_set(S.SEED_DB_1M, S.LOGNORMAL_45, DB_N)
    ref = tuple(a[:ROWS] for a in db)   # database molecules 0..1023 as the ref rows
    gl = GPULingo(0)
    gl.set_qsmiles(*db)
    gl.set_refsmiles(*ref)
    block = gl.getMultipleRowsDevice(0, ROWS)
    torch.cuda.synchronize()
    yield gl, db, ref, block
    del block
    torch.cuda.empty_cache()


def test_rows_block_full_size(full, oracle):
    import torch
    gl, db, ref, block = full
    assert block.shape == (ROWS, DB_N)
    # self-similarity and symmetry over the ref molecules' own columns
    assert bool((torch.diagonal(block[:, :ROWS]) == 1.0).all())
    sq = block[:, :ROWS].view(torch.int32)
    assert torch.equal(sq, sq.t())
    # complete rows against the oracle, bit for bit (rows in different 32-row groups)
    rows = [0, 7, 31, 32, 511, 1023]
    sub = tuple(a[rows] for a in ref)
    want = oracle.tanimoto_block(sub, db, 0, len(rows))
    got = block[rows].cpu().numpy()
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


@pytest.mark.parametrize("lo", [0.2, 0.7])
def test_neighbors_full_size_equal_the_rows_block(full, lo):
    import torch
    gl, db, ref, block = full
    dev = block.device
    amag = torch.from_numpy(ref[3].astype(np.int32)).to(dev)
    bmag = torch.from_numpy(db[3].astype(np.int32)).to(dev)
    # the kernel compares with the fp32 bounds (0.7f < 0.7)
    lo32 = torch.tensor(lo, dtype=torch.float32, device=dev)
    hi32 = torch.tensor(1.1, dtype=torch.float32, device=dev)
    counts, cols, vals = [], [], []
    for r0 in range(0, ROWS, 128):
        b = block[r0:r0 + 128]
        a = amag[r0:r0 + 128, None]
        bound = torch.minimum(a, bmag[None, :]).float() / torch.maximum(a, bmag[None, :]).float()
        m = (bound >= lo32) & (b >= lo32) & (b < hi32)
        counts.append(m.sum(1, dtype=torch.int32))
        nz = m.nonzero()
        cols.append(nz[:, 1].to(torch.int32))
        vals.append(b[nz[:, 0], nz[:, 1]])
        del bound, m
    want_cnt = torch.cat(counts)
    want_cols = torch.cat(cols)
    want_vals = torch.cat(vals)
    assert int(want_cnt.min()) >= 1   # every ref molecule finds itself
    pitch = 16 * ((int(want_cnt.max()) + 15) // 16)
    idx = torch.empty((ROWS, pitch), dtype=torch.int32, device=dev)
    sims = torch.empty((ROWS, pitch), dtype=torch.float32, device=dev)
    cnt = torch.empty(ROWS, dtype=torch.int32, device=dev)
    gl.neighborsDevice(0, ROWS, lo, 1.1, pitch, idx, sims, cnt)
    torch.cuda.synchronize()
    assert torch.equal(cnt, want_cnt)
    listed = torch.arange(pitch, device=dev)[None, :] < cnt[:, None]
    assert torch.equal(idx[listed], want_cols)   # row-major: ascending indices per row
    assert torch.equal(sims[listed].view(torch.int32), want_vals.view(torch.int32))


def test_topk_full_size_equals_the_rows_block(full):
    import torch
    gl, db, ref, block = full
    k = 100
    dev = block.device
    idx = torch.empty((ROWS, k), dtype=torch.int32, device=dev)
    sims = torch.empty((ROWS, k), dtype=torch.float32, device=dev)
    gl.topKDevice(0, ROWS, k, idx, sims)
    torch.cuda.synchronize()
    for r0 in range(0, ROWS, 128):
        # a stable descending sort keeps the lower index first among equal similarities
        v, i = torch.sort(block[r0:r0 + 128], dim=1, descending=True, stable=True)
        assert torch.equal(idx[r0:r0 + 128], i[:, :k].to(torch.int32))
        assert torch.equal(sims[r0:r0 + 128].view(torch.int32), v[:, :k].contiguous().view(torch.int32))
        del v, i


def test_histograms_full_size_equal_the_rows_block(full):
    import torch
    gl, db, ref, block = full
    dev = block.device
    h1000 = torch.zeros(1000, dtype=torch.int64, device=dev)
    h101 = torch.zeros((ROWS, 101), dtype=torch.int64, device=dev)
    for r0 in range(0, ROWS, 128):
        b = block[r0:r0 + 128]
        h1000 += torch.bincount((b * 1000.0).to(torch.int32).clamp(max=999).view(-1), minlength=1000)
        bins = (b * 100.0).to(torch.int64).clamp(max=100) + 101 * torch.arange(b.shape[0], device=dev)[:, None]
        h101[r0:r0 + 128] = torch.bincount(bins.view(-1), minlength=101 * b.shape[0]).view(-1, 101)
        del bins
    got1000 = gl.getSimilarityHistogram(0, ROWS)
    assert int(got1000.sum()) == ROWS * DB_N
    assert np.array_equal(got1000.astype(np.int64), h1000.cpu().numpy())
    got101 = gl.getMultipleHistogrammedRows(0, ROWS)
    assert np.array_equal(np.asarray(got101)[:, :101].astype(np.int64), h101.cpu().numpy())


RAGGED_DB_N = 2_000_000


@pytest.fixture(scope="module")
def ragged(native):
    torch = pytest.importorskip("torch")
    from siml_gb300 import GPULingo, synthetic as S
    db = S.smiles_set(S.SEED_RAGGED, S.BIMODAL_35_110, RAGGED_DB_N)
    gl = GPULingo(0)
    gl.set_qsmiles(*db)
    gl.set_refsmiles(*db)
    jobs = S.ragged_jobs(S.SEED_RAGGED, RAGGED_DB_N, 512)
    yield gl, db, jobs
    torch.cuda.empty_cache()


def test_ragged_jobs_full_size(ragged, oracle):
    """512 jobs of the ragged workload on its full 2M-molecule bimodal
    database (rows log-uniform 1-2,048, columns log-uniform 1,000-200,000,
    T >= 0.6, pitch 128): one batched run (autotuned tile), its CUDA-graph
    replay and the plain one-call-per-job path give identical results, and
    the two smallest jobs equal the oracle."""
    import torch
    from siml_gb300 import _native as N
    gl, db, jobs = ragged
    lo, maxn = 0.6, 128
    plan = gl.planNeighborBatch(jobs, lo, 1.1, maxn)
    idx, sims, cnt = plan.buffers(with_sims=True)
    plan.run(idx, sims, cnt)
    # the same plan captured in a CUDA graph and replayed into other buffers
    g_idx, g_sims, g_cnt = plan.buffers(with_sims=True)
    cap = torch.cuda.Stream()
    cap.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(cap):
        plan.run(g_idx, g_sims, g_cnt, stream=cap)
    torch.cuda.current_stream().wait_stream(cap)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        plan.run(g_idx, g_sims, g_cnt, stream=torch.cuda.current_stream())
    g_idx.fill_(-1)
    g_sims.fill_(-1.0)
    g_cnt.fill_(-1)
    graph.replay()
    # plain path: one range search per job
    p_idx, p_sims, p_cnt = plan.buffers(with_sims=True)
    J = plan.jobs.tolist()
    for rb, re, cb, ce, o in J:
        if re > rb:
            gl.neighborsRangeDevice(rb, re, cb, ce, lo, 1.1, plan.pitch, p_idx[o:o + re - rb],
                                    p_sims[o:o + re - rb], p_cnt[o:o + re - rb])
    torch.cuda.synchronize()
    N.check(N.lib().siml_async_status(gl._h), "siml_async_status")
    n = plan.rows_out
    listed = torch.arange(plan.pitch, device=cnt.device)[None, :] < torch.clamp(cnt[:n], max=plan.pitch)[:, None]
    for oi, os_, oc in ((g_idx, g_sims, g_cnt), (p_idx, p_sims, p_cnt)):
        assert torch.equal(oc[:n], cnt[:n])
        assert torch.equal(oi[:n][listed], idx[:n][listed])
        assert torch.equal(os_[:n][listed].view(torch.int32), sims[:n][listed].view(torch.int32))
    res = plan.split(idx, sims, cnt)
    pairs = (jobs[:, 1] - jobs[:, 0]) * (jobs[:, 3] - jobs[:, 2])
    for i in [int(x) for x in np.argsort(pairs, kind="stable")[:2]]:
        rb, re, cb, ce = (int(v) for v in jobs[i])
        m, s, c = res[i]
        om, os_, oc = oracle.neighbors_range_block(db, db, rb, re, cb, ce, lo, 1.1, maxn)
        assert np.array_equal(c, oc)
        for r in range(re - rb):
            k = min(int(c[r]), plan.pitch)
            assert np.array_equal(m[r, :k], om[r, :k])
            assert np.array_equal(s[r, :k].view(np.uint32), os_[r, :k].view(np.uint32))


SERVING_DB_N = 10_000_000


def test_serving_full_size(native, oracle):
    """The serving workload's 10M-molecule database made resident from the
    GPU compiler: requests of 1-512 query SMILES (log-uniform), half top-50
    and half T >= 0.75, are queued together for the server; each answer
    equals the same request served alone, and the two smallest equal the
    oracle."""
    import torch
    from siml_gb300 import GPULingo, synthetic as S
    from siml_gb300.compiler import compile_buffer, compile_buffer_gpu
    from siml_gb300.serving import LingoServer, Request, ServerConfig, serve_unbatched
    buf, off = S.smiles_buffer(S.SEED_SERVING, S.UNIFORM_20_90, SERVING_DB_N)
    db = compile_buffer(buf, off)
    db_dev = compile_buffer_gpu(buf, off)
    del buf, off
    # the GPU compiler's arrays equal the host compiler's, molecule for molecule
    for a, b in zip(db, db_dev):
        assert tuple(b.shape) == a.shape
        for i0 in range(0, SERVING_DB_N, 1_000_000):
            assert torch.equal(torch.from_numpy(np.ascontiguousarray(a[i0:i0 + 1_000_000])).to(b.device),
                               b[i0:i0 + 1_000_000]), i0
    gl = GPULingo(0)
    gl.set_qsmiles(*db_dev)
    del db_dev
    srv = LingoServer(gl, ServerConfig(max_rows=512, width=128, kmax=64, pitch=256, lo=0.75))
    rng = np.random.default_rng(20260005)
    reqs, pos = [], SERVING_DB_N
    for i in range(16):
        q = int(np.floor(np.exp(rng.uniform(0.0, np.log(513.0)))))
        smi = S.smiles_list(S.SEED_SERVING, S.UNIFORM_20_90, q, first=pos)
        pos += q
        reqs.append(Request(i, smi, kind="topk" if i % 2 == 0 else "threshold", k=50, lo=0.75))
    for r in reqs:   # all queued before the loop starts: batches take as many as fit
        srv.submit(r)
    srv.start()
    for r in reqs:
        assert r.done.wait(300), r.rid
    srv.stop()
    assert srv.batches < len(reqs)
    for r in reqs:
        assert r.error is None, r.error
        a = Request(r.rid, r.smiles, kind=r.kind, k=r.k, lo=r.lo)
        serve_unbatched(srv, a)
        assert len(a.result) == len(r.result) == r.rows
        for x, y in zip(a.result, r.result):
            assert np.array_equal(x[0], y[0]) and np.array_equal(np.asarray(x[1]).view(np.uint32),
                                                                 np.asarray(y[1]).view(np.uint32)), r.rid
    for r in sorted(reqs, key=lambda q: q.rows)[:2]:
        qs = oracle.compile_strings(r.smiles)
        if r.kind == "topk":
            oi, os_ = oracle.topk_block(qs, db, 0, r.rows, r.k)
            want = [(oi[q], os_[q]) for q in range(r.rows)]
        else:
            oi, osm, oc = oracle.neighbors_block(qs, db, 0, r.rows, 0.75, 1.1, 4096)
            assert int(oc.max()) <= 4096
            want = [(oi[q, :oc[q]], osm[q, :oc[q]]) for q in range(r.rows)]
        for x, y in zip(r.result, want):
            assert np.array_equal(x[0], y[0]) and np.array_equal(np.asarray(x[1]).view(np.uint32),
                                                                 np.asarray(y[1]).view(np.uint32)), r.rid
    del srv, gl
    torch.cuda.empty_cache()
