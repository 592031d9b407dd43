"""Database slabs on the GPU: one engine per slab (as one GPU per slab would
hold it), each searching all rows against its own slab; the host merges of
siml_gb300.replicas then give exactly what one engine over the whole
database gives.  On one GPU the engines share the device; with several
GPUs each would run on its own."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _engine(ref, qry):
    from siml_gb300 import GPULingo
    gl = GPULingo(0)
    gl.set_refsmiles(*ref)
    gl.set_qsmiles(*qry)
    return gl


@pytest.mark.parametrize("nshards,lo,pitch", [(2, 0.3, 16), (3, 0.1, 64), (4, 0.6, 16)])
def test_slab_engines_merge_to_one_search(native, set4096, nshards, lo, pitch):
    from siml_gb300 import replicas
    qry = set4096
    ref = tuple(np.ascontiguousarray(a[:96]) for a in qry)
    n = qry[0].shape[0]
    bounds = replicas.shard_bounds(n, nshards)
    full = _engine(ref, qry)
    slabs = [_engine(ref, tuple(np.ascontiguousarray(a[b:e]) for a in qry)) for b, e in bounds]
    # getNeighbors with similarities: each slab with one wave of extra room
    parts = []
    for (b, e), gl in zip(bounds, slabs):
        m, s, c = gl.getNeighborsWithSimilarities(0, 96, lo, 1.1, pitch + 128)
        parts.append((np.where(m >= 0, m + b, m), s, c))
    mi, ms, mc = replicas.merge_neighbors(parts, bounds, pitch)
    wi, ws, wc = full.getNeighborsWithSimilarities(0, 96, lo, 1.1, pitch)
    assert np.array_equal(mc, wc)
    for r in range(96):
        k = min(int(wc[r]), pitch)
        assert np.array_equal(mi[r, :k], wi[r, :k]), r
        assert np.array_equal(ms[r, :k].view(np.uint32), np.asarray(ws)[r, :k].view(np.uint32)), r
    # top-k
    tparts = []
    for (b, e), gl in zip(bounds, slabs):
        ti, ts = gl.getTopK(0, 96, 12)
        tparts.append((np.where(ti >= 0, ti + b, ti), ts))
    ti, ts = replicas.merge_topk(tparts, 12)
    wi, ws = full.getTopK(0, 96, 12)
    assert np.array_equal(ti, wi) and np.array_equal(ts.view(np.uint32), np.asarray(ws).view(np.uint32))
    # full-matrix rows and histograms
    assert np.array_equal(replicas.merge_rows([gl.getMultipleRows(0, 96) for gl in slabs]),
                          full.getMultipleRows(0, 96))
    assert np.array_equal(replicas.merge_hist([np.asarray(gl.getMultipleHistogrammedRows(0, 96)) for gl in slabs]),
                          np.asarray(full.getMultipleHistogrammedRows(0, 96)))
