"""GPU parity of getNeighbors (pysiml/GPULingo.py:467-534, kernel
pysiml/kernels.py:393-475) against the oracle's CPU restatement: identical
counts (including wave-granular overflow counts), indices in ascending order
and, for the similarity variant, bit-identical fp32 similarities."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _engine(ref, qry):
    from siml_gb300 import GPULingo
    gl = GPULingo(0)
    gl.set_refsmiles(*ref)
    gl.set_qsmiles(*qry)
    return gl


def _check(gl, oracle, ref, qry, rowbase, rowlimit, lo, hi=1.1, maxneighbors=None):
    idx, sims, cnt = gl.getNeighborsWithSimilarities(rowbase, rowlimit, lo, hi, maxneighbors)
    oidx, osims, ocnt = oracle.neighbors_block(ref, qry, rowbase, rowlimit, lo, hi, maxneighbors)
    assert np.array_equal(cnt, ocnt), (lo, hi, maxneighbors)
    pitch = oidx.shape[1]
    for r in range(rowlimit - rowbase):
        k = min(int(cnt[r]), pitch)
        assert np.array_equal(idx[r, :k], oidx[r, :k]), (r, lo, hi, maxneighbors)
        assert np.array_equal(sims[r, :k].view(np.uint32), osims[r, :k].view(np.uint32)), r
    # the reference-shaped call returns the same indices and counts
    m2, c2 = gl.getNeighbors(rowbase, rowlimit, lo, hi, maxneighbors)
    assert np.array_equal(c2, cnt) and m2.shape == idx.shape
    for r in range(rowlimit - rowbase):
        k = min(int(cnt[r]), pitch)
        assert np.array_equal(m2[r, :k], idx[r, :k])
    return cnt


def _golden_sets(golden):
    q = (golden["lingos"], golden["counts"], golden["lengths"], golden["mags"])
    return q, q


@pytest.mark.parametrize("lo,hi", [(0.7, 1.1), (0.3, 1.1), (0.05, 1.1), (0.2, 0.5), (0.0, 1.1), (0.9, 1.0)])
def test_neighbors_golden(native, oracle, golden, lo, hi):
    ref, qry = _golden_sets(golden)
    gl = _engine(ref, qry)
    n = ref[0].shape[0]
    _check(gl, oracle, ref, qry, 0, n, lo, hi)


@pytest.mark.parametrize("maxneighbors", [1, 10, 16, 100, 300])
def test_neighbors_overflow_semantics(native, oracle, golden, maxneighbors):
    """Counts grow by whole waves of 128 columns once a row overflows its
    pitch 16*ceil(maxneighbors/16)."""
    ref, qry = _golden_sets(golden)
    gl = _engine(ref, qry)
    n = ref[0].shape[0]
    cnt = _check(gl, oracle, ref, qry, 0, n, 0.02, 1.1, maxneighbors)
    pitch = 16 * ((maxneighbors + 15) // 16)
    if maxneighbors < 100:
        assert np.any(cnt > pitch)


def test_neighbors_synthetic_self(native, oracle, set4096):
    """A database searched with its own molecules: every molecule with LINGOs
    finds itself at 1.0, in 16-row and odd-sized blocks."""
    gl = _engine(set4096, set4096)
    for rb, rl in [(0, 32), (100, 117), (4000, 4096), (0, 1024)]:
        cnt = _check(gl, oracle, set4096, set4096, rb, rl, 0.7)
        assert np.all(cnt >= 1)
    _check(gl, oracle, set4096, set4096, 0, 256, 0.12, 1.1, 64)
    _check(gl, oracle, set4096, set4096, 0, 64, 0.0, 0.05, 32)


def test_neighbors_edge_values(native, oracle, golden):
    ref, qry = _golden_sets(golden)
    gl = _engine(ref, qry)
    n = ref[0].shape[0]
    idx, cnt = gl.getNeighbors(0, n, float("nan"))
    assert np.all(cnt == 0)
    m, c = gl.getNeighbors(5, 5, 0.5)
    assert m.shape == (0, 0) and c.shape == (0,)
    _check(gl, oracle, ref, qry, 0, n, -1.0, 0.5, 40)
    _check(gl, oracle, ref, qry, 3, 40, 0.4, 0.4)


def test_neighbors_merge_path(native, oracle):
    """Large vocabulary: no table fits, every row takes the ordered scan."""
    rng = np.random.default_rng(5)

    def rs(n, w):
        L = np.zeros((n, w), np.int32)
        C = np.zeros((n, w), np.int32)
        ln = np.zeros(n, np.int32)
        for i in range(n):
            codes = np.unique(rng.integers(0, 10 ** 9, size=int(rng.integers(1, w + 1))).astype(np.int32))
            L[i, :len(codes)] = codes
            C[i, :len(codes)] = rng.integers(1, 3, size=len(codes))
            ln[i] = len(codes)
        return L, C, ln, C.sum(1).astype(np.int32)
    qry = rs(2500, 64)
    ref = tuple(a[:50].copy() for a in qry)
    gl = _engine(ref, qry)
    _check(gl, oracle, ref, qry, 0, 50, 0.3)
    _check(gl, oracle, ref, qry, 0, 50, 0.0, 1.1, 5)


@pytest.mark.parametrize("window", [64, 256, 2048, 8192])
def test_neighbors_mixed_lengths_sort_windows(native, oracle, window):
    """A bimodal database (short and long molecules): threshold searches skip
    whole chunks whose magnitudes cannot reach the bound, for every sort
    window; results equal the oracle."""
    from siml_gb300 import synthetic as S
    db = S.smiles_set(S.SEED_RAGGED, S.BIMODAL_35_110, 12000)
    q = tuple(a[:300] for a in db)
    gl = _engine(q, db)
    from siml_gb300 import _native as N
    N.check(N.lib().siml_set_tuning(gl._h, N.SIML_TUNE_SORT_WINDOW, window))
    for lo, maxn in ((0.6, 64), (0.3, 200), (0.9, 16)):
        _check(gl, oracle, q, db, 0, 300, lo, 1.1, maxn)
    idx, cnt = gl.getNeighbors(0, 300, 0.6, 1.1, 64)
    assert np.all(cnt >= 1)   # every row finds itself


def test_evaluated_pairs_counter(native, oracle):
    """Threshold searches on a mixed-length database skip chunks: the
    evaluated pairs are fewer than the logical pairs, and a bound of 0 skips
    nothing."""
    from siml_gb300 import synthetic as S
    db = S.smiles_set(S.SEED_RAGGED, S.BIMODAL_35_110, 20000)
    q = tuple(a[:256] for a in db)
    gl = _engine(q, db)
    gl.evaluatedPairs(reset=True)
    gl.getNeighbors(0, 256, 0.8, 1.1, 64)
    hi = gl.evaluatedPairs(reset=True)
    gl.getNeighbors(0, 256, 0.0, 0.01, 64)
    lo = gl.evaluatedPairs(reset=True)
    assert 0 < hi < lo
    assert lo >= 256 * 20000
    assert gl.evaluatedPairs() == 0
