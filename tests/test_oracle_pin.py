"""Pins the oracle (oracle/) to the reference: against the golden fixtures
made by the reference's own compiled code (tests/golden/make_golden.py), and,
where the reference build exists (oracle/_ref), against it directly."""
import numpy as np
import pytest

from siml_gb300 import synthetic as S


def test_oracle_compiler_matches_golden(oracle, golden):
    L, C, ln, mg = oracle.compile_strings(golden["strings"])
    assert np.array_equal(L, golden["lingos"])
    assert np.array_equal(C, golden["counts"])
    assert np.array_equal(ln, golden["lengths"])
    assert np.array_equal(mg, golden["mags"])


def test_oracle_tanimoto_matches_golden(oracle, golden):
    rows = golden["rows"]
    q = (golden["lingos"], golden["counts"], golden["lengths"], golden["mags"])
    ref = tuple(a[rows] for a in q)
    T = oracle.tanimoto_block(ref, q, 0, len(rows), nthreads=1)
    assert np.array_equal(T, golden["tanimoto"])
    TP = oracle.tanimoto_block(ref, q, 0, len(rows), nthreads=4)
    assert np.array_equal(TP, golden["tanimoto"])


def test_oracle_rowhistogram_matches_golden(oracle, golden):
    assert np.array_equal(oracle.rowHistogram101(golden["tanimoto"]), golden["hist101"])


def test_oracle_invariants(oracle, golden):
    """Self-similarity diagonal is exactly 1 where a molecule has LINGOs, and
    the compiler's magnitude equals the count sum for ASCII strings."""
    q = (golden["lingos"], golden["counts"], golden["lengths"], golden["mags"])
    n = len(golden["strings"])
    T = oracle.tanimoto_block(q, q, 0, n)
    d = np.diag(T)
    assert np.all(d[golden["mags"] > 0] == 1.0)
    assert np.all(d[golden["mags"] == 0] == 0.0)
    ascii_rows = [i for i, s in enumerate(golden["strings"]) if all(b < 0x80 for b in s)]
    assert np.array_equal(golden["counts"][ascii_rows].sum(1), golden["mags"][ascii_rows])


def _ref_or_skip(oracle, name):
    m = oracle.reference_module(name)
    if m is None:
        pytest.skip("reference build (oracle/_ref) not present")
    return m


@pytest.mark.parametrize("dist,seed", [(S.UNIFORM_20_90, S.SEED_ALLPAIRS), (S.LOGNORMAL_45, S.SEED_DB_1M),
                                       (S.BIMODAL_35_110, S.SEED_RAGGED)])
def test_oracle_matches_reference_build(oracle, native, dist, seed):
    cc = _ref_or_skip(oracle, "_ccompiler")
    cp = _ref_or_skip(oracle, "_CPULingo")
    strs = S.smiles_list(seed, dist, 700, first=5000)
    L, C, ln, mg = oracle.compile_strings(strs)
    L2, C2, ln2, mg2 = cc.SMILEStoMatrices([s + b"\n" for s in strs])
    assert np.array_equal(L, L2) and np.array_equal(C, C2)
    assert np.array_equal(ln, ln2[:, 0]) and np.array_equal(mg, mg2[:, 0])
    q = (L, C, ln, mg)
    T = oracle.tanimoto_block(q, q, 100, 300)
    T2 = cp.getTanimotoBlockParallel(L[100:300], C[100:300], mg[100:300].reshape(-1, 1), ln[100:300].reshape(-1, 1),
                                     L, C, mg.reshape(-1, 1), ln.reshape(-1, 1), 4)
    assert np.array_equal(T, T2)


def test_oracle_matches_reference_on_demo_file(oracle):
    """The reference's example data file, read in place (never copied)."""
    import os
    if not oracle.REFERENCE_ROOT:
        pytest.skip("reference project not present")
    path = os.path.join(oracle.REFERENCE_ROOT, "examples", "demo4096.smi")
    if not os.path.exists(path):
        pytest.skip("reference example data not present")
    cc = _ref_or_skip(oracle, "_ccompiler")
    cp = _ref_or_skip(oracle, "_CPULingo")
    with open(path, "rb") as f:
        lines = f.readlines()
    L, C, ln, mg, _ = oracle.cSMILEStoMatrices(lines)
    L2, C2, ln2, mg2 = cc.SMILEStoMatrices(lines)
    assert np.array_equal(L, L2) and np.array_equal(C, C2) and np.array_equal(ln, ln2) and np.array_equal(mg, mg2)
    q = (L, C, ln, mg)
    T = oracle.tanimoto_block(q, q, 0, 256)
    T2 = cp.getTanimotoBlockParallel(L[:256], C[:256], mg[:256], ln[:256], L, C, mg, ln, 4)
    assert np.array_equal(T, T2)


def test_neighbors_oracle_consistent_with_matrix(oracle, golden):
    """getNeighbors' CPU form agrees with thresholding the Tanimoto matrix
    (no overflow) and reports wave-granular counts on overflow."""
    q = (golden["lingos"], golden["counts"], golden["lengths"], golden["mags"])
    n = len(golden["strings"])
    T = oracle.tanimoto_block(q, q, 0, n)
    idx, sims, cnt = oracle.neighbors_block(q, q, 0, n, 0.05, 1.1, maxneighbors=n)
    for r in range(n):
        ma = golden["mags"][r]
        mb = golden["mags"]
        bound = np.minimum(ma, mb).astype(np.float32) / np.maximum(ma, mb).astype(np.float32)
        want = np.nonzero((bound >= np.float32(0.05)) & (T[r] >= np.float32(0.05)) & (T[r] < np.float32(1.1)))[0]
        assert cnt[r] == len(want)
        assert np.array_equal(idx[r, :cnt[r]], want)
        assert np.array_equal(sims[r, :cnt[r]], T[r, want])
    # overflow: pitch 16, counts grow by whole waves of 128 columns
    idx, sims, cnt = oracle.neighbors_block(q, q, 0, n, 0.0, 1.1, maxneighbors=10)
    for r in range(n):
        ma = golden["mags"][r]
        mb = golden["mags"]
        bound = np.minimum(ma, mb).astype(np.float32) / np.maximum(ma, mb).astype(np.float32)
        hits = np.nonzero((bound >= 0) & (T[r] >= 0) & (T[r] < np.float32(1.1)))[0]
        if len(hits) > 16:
            wave = hits[16] // 128
            assert cnt[r] == np.count_nonzero(hits < (wave + 1) * 128)
            assert np.array_equal(idx[r, :16], hits[:16])
        else:
            assert cnt[r] == len(hits)


def test_topk_and_hist1000_oracle(oracle, golden):
    q = (golden["lingos"], golden["counts"], golden["lengths"], golden["mags"])
    n = len(golden["strings"])
    T = oracle.tanimoto_block(q, q, 0, 40)
    idx, sims = oracle.topk_block(q, q, 0, 40, 25)
    for r in range(40):
        order = np.lexsort((np.arange(n), -T[r].astype(np.float64)))[:25]
        assert np.array_equal(idx[r], order)
        assert np.array_equal(sims[r], T[r, order])
    h = oracle.hist1000_block(q, q, 0, 40)
    s = T * np.float32(1000.0)
    b = np.minimum(s.astype(np.uint32), 999)
    assert np.array_equal(h, np.bincount(b.ravel(), minlength=1000).astype(np.uint64))
