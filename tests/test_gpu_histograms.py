"""GPU parity of the histogram paths against the oracle: per-row 101-bin
histograms (getMultipleHistogrammedRows, pysiml/kernels.py:606-666), the
1000-bin histogram of a row block, and rowHistogram101
(pysiml/_cpuutil.cpp:52-126) against the golden fixture made by the
reference's own code."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _engine(ref, qry):
    from siml_gb300 import GPULingo
    gl = GPULingo(0)
    gl.set_refsmiles(*ref)
    gl.set_qsmiles(*qry)
    return gl


def test_hist101_golden(native, oracle, golden):
    q = (golden["lingos"], golden["counts"], golden["lengths"], golden["mags"])
    gl = _engine(q, q)
    n = q[0].shape[0]
    got = gl.getMultipleHistogrammedRows(0, n)
    assert got.shape == (n, 101) and got.dtype == np.int32
    assert np.array_equal(got, oracle.hist101_block(q, q, 0, n))
    assert np.all(got.sum(1) == n)


def test_hist101_synthetic_blocks(native, oracle, set4096):
    gl = _engine(set4096, set4096)
    for rb, rl in [(0, 32), (50, 133), (3000, 4096)]:
        assert np.array_equal(gl.getMultipleHistogrammedRows(rb, rl), oracle.hist101_block(set4096, set4096, rb, rl))
    gl.getMultipleHistogrammedRows_async(0, 7)
    assert gl.retrieveAsyncResult().shape == (7, 101)


def test_global_histogram(native, oracle, set4096, golden):
    gl = _engine(set4096, set4096)
    h = gl.getSimilarityHistogram(0, 1000)
    assert h.dtype == np.uint64 and int(h.sum()) == 1000 * 4096
    assert np.array_equal(h, oracle.hist1000_block(set4096, set4096, 0, 1000))
    # accumulates across calls
    gl.getSimilarityHistogram(1000, 2000, out=h)
    want = oracle.hist1000_block(set4096, set4096, 0, 2000)
    assert np.array_equal(h, want)
    q = (golden["lingos"], golden["counts"], golden["lengths"], golden["mags"])
    g2 = _engine(q, q)
    assert np.array_equal(g2.getSimilarityHistogram(0, q[0].shape[0]), oracle.hist1000_block(q, q, 0, q[0].shape[0]))


def test_global_histogram_device_out(native, oracle, set4096):
    torch = pytest.importorskip("torch")
    gl = _engine(set4096, set4096)
    out = torch.zeros(1000, dtype=torch.int64, device="cuda")
    gl.getSimilarityHistogram(0, 512, out=out)
    assert np.array_equal(out.cpu().numpy().astype(np.uint64), oracle.hist1000_block(set4096, set4096, 0, 512))


def test_row_histogram101_utility(native, golden):
    from siml_gb300.utilities import rowHistogram101
    T = golden["tanimoto"]
    assert np.array_equal(rowHistogram101(T), golden["hist101"])
    rng = np.random.default_rng(3)
    X = rng.uniform(-0.2, 1.3, size=(37, 1001)).astype(np.float32)
    X[0, :5] = [0.0, 0.01, 0.99999994, 1.0, np.nan]
    from oracle import cpulingo as O
    assert np.array_equal(rowHistogram101(X), O.rowHistogram101(X))
    D = X.astype(np.float64)
    s = D * 100.0
    want = np.where(~(s >= 0), 0, np.minimum(np.where(s >= 0, s, 0).astype(np.uint64), 100))
    want = np.stack([np.bincount(r, minlength=101) for r in want]).astype(np.uint32)
    assert np.array_equal(rowHistogram101(D), want)
    with pytest.raises(ValueError):
        rowHistogram101(np.zeros((3, 3), np.int32))


def test_shared_engine_users_from_two_threads(native):
    """rowHistogram101 and the GPU compiler share one engine per device; two
    host threads using them at once get the single-thread results."""
    import threading
    import torch
    from siml_gb300 import synthetic as S, utilities as U
    from siml_gb300.compiler import compile_buffer, compile_buffer_gpu
    rng = np.random.default_rng(11)
    mats = [torch.from_numpy(rng.random((300, 2000), dtype=np.float32)).cuda() for _ in range(2)]
    want_h = [U.rowHistogram101(m.cpu().numpy()) for m in mats]
    buf, off = S.smiles_buffer(S.SEED_ALLPAIRS, S.UNIFORM_20_90, 3000)
    want_c = compile_buffer(buf, off)
    errors = []

    def work(i):
        try:
            s = torch.cuda.Stream()
            with torch.cuda.stream(s):
                for _ in range(10):
                    h = U.rowHistogram101(mats[i])
                    c = compile_buffer_gpu(buf, off)
                    s.synchronize()
                    assert np.array_equal(h.cpu().numpy().astype(np.uint32), want_h[i])
                    assert all(np.array_equal(a.cpu().numpy(), b) for a, b in zip(c, want_c))
        except Exception as e:  # reported in the main thread
            errors.append(e)

    ts = [threading.Thread(target=work, args=(i,)) for i in range(2)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert not errors, errors
