"""GPU per-row top-k against the oracle: the k best similarities of each
row, best first, ties to the lower index, -1 padding past the query set."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _engine(ref, qry):
    from siml_gb300 import GPULingo
    gl = GPULingo(0)
    gl.set_refsmiles(*ref)
    gl.set_qsmiles(*qry)
    return gl


def _check(gl, oracle, ref, qry, rb, rl, k):
    idx, sims = gl.getTopK(rb, rl, k)
    oi, os_ = oracle.topk_block(ref, qry, rb, rl, k)
    assert np.array_equal(idx, oi), k
    assert np.array_equal(sims.view(np.uint32), os_.view(np.uint32)), k


@pytest.mark.parametrize("k", [1, 5, 50, 100, 256])
def test_topk_synthetic(native, oracle, set4096, k):
    gl = _engine(set4096, set4096)
    _check(gl, oracle, set4096, set4096, 0, 96, k)
    _check(gl, oracle, set4096, set4096, 1000, 1031, k)


def test_topk_golden_ties_and_padding(native, oracle, golden):
    """The golden set has repeated and empty molecules (ties, zeros)."""
    q = (golden["lingos"], golden["counts"], golden["lengths"], golden["mags"])
    gl = _engine(q, q)
    n = q[0].shape[0]
    for k in (3, 40, 128):
        _check(gl, oracle, q, q, 0, n, k)
    small = tuple(a[:20] for a in q)
    g2 = _engine(q, small)
    _check(g2, oracle, q, small, 0, 50, 32)   # k > 20 queries: padded


def test_topk_fallback_large_k(native, oracle, set4096):
    gl = _engine(set4096, set4096)
    _check(gl, oracle, set4096, set4096, 0, 8, 600)


def _dup_db(s, index):
    index = np.asarray(index, dtype=np.int64)
    return tuple(np.ascontiguousarray(a[index]) for a in s)


def test_topk_refinement_and_rowscan_paths(native, oracle, set4096):
    """Duplicated molecules make the sample bound admit more candidates than
    a row's candidate segments hold (8,192 per row): one row needs a second
    collection pass (its bound is raised from the kept candidates), another
    overflows twice and is scanned exactly.  Both must still equal the
    oracle, ties to the lower index."""
    R = 0
    t0 = oracle.tanimoto_block(set4096, set4096, R, R + 1)[0]
    order = np.argsort(-t0, kind="stable")
    cands = [int(i) for i in order if i != R and 0.05 < t0[i] < 0.95]
    A, B, C = cands[0], cands[len(cands) // 3], cands[2 * len(cands) // 3]
    assert t0[A] > t0[B] > t0[C]
    rest = [i for i in range(1, 4096) if i not in (A, B, C)]
    # C first (the sample sees only C), then B, three A, 9,000 copies of R, the rest
    index = [C] * 6000 + [B] * 6000 + [A] * 3 + [R] * 9000 + rest
    db = _dup_db(set4096, index)
    ref = _dup_db(set4096, [R, A, B, C, 17, 18])
    gl = _engine(ref, db)
    for k in (5, 64, 100):
        _check(gl, oracle, ref, db, 0, ref[0].shape[0], k)
    # without the R copies row R's second pass fits
    index2 = [C] * 6000 + [B] * 6000 + [A] * 3 + rest
    db2 = _dup_db(set4096, index2)
    g2 = _engine(ref, db2)
    for k in (1, 5, 8):
        _check(g2, oracle, ref, db2, 0, ref[0].shape[0], k)


def test_topk_multiple_row_blocks(native, oracle, set4096):
    """More rows than one threshold-and-collect pass handles at once."""
    big = _dup_db(set4096, np.arange(9000) % 4096)
    gl = _engine(big, set4096)
    idx, sims = gl.getTopK(0, 9000, 7)
    oi, os_ = oracle.topk_block(big, set4096, 8000, 9000, 7)
    assert np.array_equal(idx[8000:], oi)
    assert np.array_equal(sims[8000:].view(np.uint32), os_.view(np.uint32))
    assert np.array_equal(idx[:4096], idx[4096:8192])
