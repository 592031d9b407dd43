"""Vocabularies too large for the shared-memory table: the pairs are split
by database frequency into common ones (direct table) and rare ones (a
per-group hash of the ref rows' rare pairs, with each database molecule's
rare entries in a side list).  Every call must still give exactly what the
reference gives (the oracle restates pysiml/_CPULingo.c:53-71 and the GPU
kernels' rules), and ref sets whose rows hold too many rare entries must
fall back to the per-pair merge with the same results."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

WIDE = np.frombuffer(b"CcNnOoSsPpFIBrlK()[]=#@+-H/\\%.0123456789abdefghijkmqtuvwxyzAEGJLMQRTUVWXYZ", np.uint8)


def _strings(rng, n, lo, hi):
    lens = rng.integers(lo, hi, n)
    return [bytes(rng.choice(WIDE, size=int(k)).astype(np.uint8)) for k in lens]


def _sets(ref_strings, db_strings):
    from siml_gb300 import compiler as PC
    pack = lambda ss: (b"".join(ss), np.concatenate([[0], np.cumsum([len(s) for s in ss])]).astype(np.int64))
    db = PC.compile_buffer(*pack(db_strings))
    ref = PC.compile_buffer(*pack(ref_strings))
    w = max(db[0].shape[1], ref[0].shape[1])
    pad = lambda a: np.pad(a, ((0, 0), (0, w - a.shape[1])))
    return (pad(ref[0]), pad(ref[1]), ref[2], ref[3]), (pad(db[0]), pad(db[1]), db[2], db[3])


def _mixed(rng, n_db, n_ref, short=True):
    """A database of common-alphabet molecules (frequent pairs) and wide-
    alphabet ones (rare pairs); refs drawn from it plus new strings.  Short:
    refs cut to 40 bytes (at most ~40 rare entries a row); long: the wide
    molecules run 150-260 bytes and some refs are whole wide molecules, so
    rows hold well over 96 rare entries."""
    from siml_gb300 import synthetic as S
    common = S.smiles_list(S.SEED_ALLPAIRS, S.UNIFORM_20_90, n_db // 2, first=50_000)
    wide = _strings(rng, n_db - n_db // 2, 20, 60) if short else _strings(rng, n_db - n_db // 2, 150, 260)
    db = [s for pair in zip(common, wide) for s in pair]
    pick = rng.choice(len(db), n_ref - 8, replace=False)
    if short:
        ref = [db[i][:40] for i in pick] + _strings(rng, 8, 10, 40)
    else:
        ref = [db[i] for i in pick] + [wide[i] for i in range(8)]
    return _sets(ref, db)


def _engine(ref, qry):
    from siml_gb300 import GPULingo
    gl = GPULingo(0)
    gl.set_refsmiles(*ref)
    gl.set_qsmiles(*qry)
    return gl


def test_split_vocabulary_rows_neighbors_hist_topk(native, oracle):
    rng = np.random.default_rng(31)
    ref, qry = _mixed(rng, 30_000, 72)
    gl = _engine(ref, qry)
    st = gl.vocabStats()
    assert st["ncommon"] < st["nvid"] and st["nrare"] > 0 and 0 < st["row_max_rare"] <= 96, st
    n = ref[0].shape[0]
    got = gl.getMultipleRows(0, n)
    assert np.array_equal(got.view(np.uint32), oracle.tanimoto_block(ref, qry, 0, n).view(np.uint32))
    for lo, maxn in [(0.3, 64), (0.05, 16)]:
        m, c = gl.getNeighbors(0, n, lo, 1.1, maxn)
        oi, osm, oc = oracle.neighbors_block(ref, qry, 0, n, lo, 1.1, maxn)
        assert np.array_equal(c, oc)
        for r in range(n):
            k = min(int(c[r]), m.shape[1])
            assert np.array_equal(m[r, :k], oi[r, :k]), r
    h = gl.getMultipleHistogrammedRows(0, n)
    assert np.array_equal(np.asarray(h)[:, :101], oracle.hist101_block(ref, qry, 0, n))
    idx, sims = gl.getTopK(0, n, 20)
    oi, os_ = oracle.topk_block(ref, qry, 0, n, 20)
    assert np.array_equal(idx, oi) and np.array_equal(np.asarray(sims).view(np.uint32), os_.view(np.uint32))


@pytest.mark.parametrize("rows", [64, 32])
def test_split_vocabulary_rows_each_rare_path(native, oracle, rows):
    """The full matrix on a split vocabulary through each way of counting
    the rare pairs (a second pass over the pairs that share one, or the
    kernel's hash), for 64-row and 32-row groups: equal to the oracle, and
    a launch of the scheduled kernel took the path asked for whenever its
    table leaves rare pairs (rare_path -1: the call ran on another kernel,
    as the 64-row hash does for rows with more than 24 rare entries)."""
    from siml_gb300 import GPULingo, _native as N
    rng = np.random.default_rng(37)
    ref, qry = _mixed(rng, 30_000, 72)
    want = oracle.tanimoto_block(ref, qry, 0, ref[0].shape[0])
    seen = set()
    for fix in (1, 0):
        gl = GPULingo(0)
        N.check(N.lib().siml_set_tuning(gl._h, N.SIML_TUNE_SCHED_ROWS, rows), "sched rows")
        N.check(N.lib().siml_set_tuning(gl._h, N.SIML_TUNE_RARE_FIXUP, fix), "rare fixup")
        gl.set_refsmiles(*ref)
        gl.set_qsmiles(*qry)
        got = gl.getMultipleRows(0, ref[0].shape[0])
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (rows, fix)
        rv = gl.rowsVocab()
        if rv["rare_path"] >= 0:
            split = rv["table_pairs"] < gl.vocabStats()["nvid"]
            assert (rv["rare_path"] == 0) == (not split), rv
            if split and not fix:
                assert rv["rare_path"] == 1, rv
        seen.add(rv["rare_path"])
    if rows == 32:
        assert 1 in seen and 2 in seen, seen   # both ways ran


def test_split_vocabulary_batched_jobs(native, oracle):
    rng = np.random.default_rng(32)
    ref, qry = _mixed(rng, 20_000, 64)
    gl = _engine(ref, qry)
    assert gl.vocabStats()["ncommon"] < gl.vocabStats()["nvid"]
    jobs = [(0, 40, 0, 20_000), (10, 64, 5_000, 12_000), (3, 4, 19_000, 20_000), (30, 31, 0, 1)]
    plan = gl.planNeighborBatch(jobs, 0.2, 1.1, 32, tile_chunks=8)
    idx, sims, cnt = plan.buffers(with_sims=True)
    plan.run(idx, sims, cnt)
    for job, (m, s, c) in zip(jobs, plan.split(idx, sims, cnt)):
        oi, osm, oc = oracle.neighbors_range_block(ref, qry, job[0], job[1], job[2], job[3], 0.2, 1.1, 32)
        assert np.array_equal(c, oc), job
        for r in range(job[1] - job[0]):
            k = min(int(c[r]), m.shape[1])
            assert np.array_equal(m[r, :k], oi[r, :k]), (job, r)
            assert np.array_equal(s[r, :k].view(np.uint32), osm[r, :k].view(np.uint32)), (job, r)


def test_split_vocabulary_rows_with_many_rare_pairs_use_the_merge(native, oracle):
    rng = np.random.default_rng(33)
    ref, qry = _mixed(rng, 12_000, 40, short=False)
    gl = _engine(ref, qry)
    st = gl.vocabStats()
    assert st["ncommon"] < st["nvid"] and st["row_max_rare"] > 96, st
    n = ref[0].shape[0]
    got = gl.getMultipleRows(0, n)
    assert np.array_equal(got.view(np.uint32), oracle.tanimoto_block(ref, qry, 0, n).view(np.uint32))
    m, c = gl.getNeighbors(0, n, 0.2, 1.1, 32)
    oi, osm, oc = oracle.neighbors_block(ref, qry, 0, n, 0.2, 1.1, 32)
    assert np.array_equal(c, oc)
