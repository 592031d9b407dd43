"""GPU parity of getMultipleRows / getTanimotoRow against the oracle and the
golden fixtures: bit-exact fp32 (the reference's own bar, GPU == CPU exactly,
examples/benchmark.py:192)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _engine():
    from siml_gb300 import GPULingo
    return GPULingo(0)


def _load(gl, ref, qry):
    gl.set_refsmiles(ref[0], ref[1], ref[2], ref[3])
    gl.set_qsmiles(qry[0], qry[1], qry[2], qry[3])


def test_rows_match_golden(native, golden):
    q = (golden["lingos"], golden["counts"], golden["lengths"], golden["mags"])
    rows = golden["rows"]
    gl = _engine()
    _load(gl, tuple(a[rows] for a in q), q)
    T = gl.getMultipleRows(0, len(rows))
    assert T.dtype == np.float32 and T.shape == golden["tanimoto"].shape
    assert np.array_equal(T, golden["tanimoto"])


def test_allpairs_4096_bit_exact(native, oracle, set4096):
    """The full 4096 x 4096 matrix, fetched in 256-row blocks as the
    reference's benchmark does (examples/benchmark.py:127-135)."""
    gl = _engine()
    _load(gl, set4096, set4096)
    n = set4096[0].shape[0]
    G = np.empty((n, n), np.float32)
    for base in range(0, n, 256):
        G[base:base + 256] = gl.getMultipleRows(base, min(base + 256, n))
    C = oracle.tanimoto_block(set4096, set4096, 0, n)
    assert np.array_equal(G, C)
    assert np.all(np.diag(G) == 1.0)
    # one call for everything agrees too
    assert np.array_equal(gl.getMultipleRows(0, n), C)


def test_async_protocol(native, oracle, set4096):
    gl = _engine()
    _load(gl, set4096, set4096)
    with pytest.raises(RuntimeError):
        gl.retrieveAsyncResult()
    gl.getMultipleRows_async(100, 164)
    while not gl.asyncOperationsDone():
        pass
    got = gl.retrieveAsyncResult()
    assert np.array_equal(got, oracle.tanimoto_block(set4096, set4096, 100, 164))
    with pytest.raises(RuntimeError):
        gl.retrieveAsyncResult()
    # the reference's per-kind retrievers
    gl.getMultipleRows_async(5, 9)
    with pytest.raises(RuntimeError):
        gl.retrieveAsyncMatrixVectorResult()
    assert np.array_equal(gl.retrieveAsyncMatrixResult(), oracle.tanimoto_block(set4096, set4096, 5, 9))
    with pytest.raises(RuntimeError):
        gl.retrieveAsyncMatrixResult()
    with pytest.raises(RuntimeError):
        gl.retrieveAsyncResultBase()
    gl.getNeighbors_async(0, 3, 0.5)
    idx, cnt = gl.retrieveAsyncMatrixVectorResult_trimmed()
    assert idx.shape[0] == 3 and cnt.shape == (3,) and idx.shape[1] <= int(cnt.max())
    gl.getNeighbors_async(0, 3, 0.5)
    idx2, cnt2 = gl.retrieveAsyncMatrixVectorResult()
    assert np.array_equal(idx, idx2) and np.array_equal(cnt, cnt2)
    # a result never retrieved is dropped by the next call (after its
    # kernels are done with its buffers); the next retrieve gives the new one
    gl.getMultipleRows_async(0, 700)
    gl.getMultipleRows_async(1000, 1100)
    gl.getNeighbors_async(0, 3, 0.5)
    gl.getMultipleRows_async(2000, 2300)
    assert np.array_equal(gl.retrieveAsyncResult(), oracle.tanimoto_block(set4096, set4096, 2000, 2300))


def test_row_ranges(native, set4096):
    gl = _engine()
    _load(gl, set4096, set4096)
    with pytest.raises(RuntimeError):
        gl.getMultipleRows(-1, 10)
    with pytest.raises(RuntimeError):
        gl.getMultipleRows(0, 4097)
    assert gl.getMultipleRows(7, 7).shape == (0, 4096)
    for a, b in [(0, 1), (31, 33), (4090, 4096), (1, 100)]:
        assert gl.getMultipleRows(a, b).shape == (b - a, 4096)


def test_tanimoto_row_uses_count_magnitudes(native, oracle, golden):
    """getTanimotoRow recomputes magnitudes from counts and scores a
    molecule without LINGOs as 0 (pysiml/kernels.py:122-159, 234-270)."""
    q = (golden["lingos"], golden["counts"], golden["lengths"], golden["mags"])
    gl = _engine()
    wrong = q[3] + 7  # magnitudes that getMultipleRows uses but getTanimotoRow ignores
    gl.set_refsmiles(q[0], q[1], q[2], wrong)
    gl.set_qsmiles(q[0], q[1], q[2], wrong)
    cm = q[1].sum(1).astype(np.int32)
    n = len(golden["strings"])
    isct = oracle.isct_block(q, q, 0, n)
    for row in [0, 3, 4, 7, 30, 40, 60, 200]:
        got = gl.getTanimotoRow(row)
        assert got.shape == (1, n)
        ln = q[2]
        u = (cm[row] + cm - isct[row]).astype(np.float32)
        want = np.where((ln[row] == 0) | (ln == 0), np.float32(0), isct[row].astype(np.float32) / u)
        assert np.array_equal(got[0], want.astype(np.float32)), row
    # and getMultipleRows does use the given magnitudes
    assert np.array_equal(gl.getMultipleRows(0, 8), oracle.tanimoto_block((q[0], q[1], q[2], wrong),
                                                                           (q[0], q[1], q[2], wrong), 0, 8))


def test_default_magnitudes_are_count_sums(native, oracle, set4096):
    gl = _engine()
    L, C, ln, mg = set4096
    gl.set_refsmiles(L[:300], C[:300], ln[:300])
    gl.set_qsmiles(L, C, ln)
    cm = C.sum(1).astype(np.int32)
    assert np.array_equal(gl.getMultipleRows(0, 300),
                          oracle.tanimoto_block((L[:300], C[:300], ln[:300], cm[:300]), (L, C, ln, cm), 0, 300))


def _random_sets(rng, n, width, code_range, max_count, p_empty=0.05):
    L = np.zeros((n, width), np.int32)
    C = np.zeros((n, width), np.int32)
    ln = np.zeros(n, np.int32)
    for i in range(n):
        k = 0 if rng.random() < p_empty else int(rng.integers(1, width + 1))
        codes = np.unique(rng.integers(code_range[0], code_range[1], size=k).astype(np.int32))
        L[i, :len(codes)] = codes
        C[i, :len(codes)] = rng.integers(1, max_count + 1, size=len(codes))
        ln[i] = len(codes)
    mg = C.sum(1).astype(np.int32)
    return L, C, ln, mg


@pytest.mark.parametrize("case", ["small_vocab", "negative_codes", "high_counts", "zero_mags", "long_db_molecules",
                                  "mid_db_molecules"])
def test_rows_random_sets(native, oracle, case):
    rng = np.random.default_rng({"small_vocab": 1, "negative_codes": 2, "high_counts": 3, "zero_mags": 4,
                                 "long_db_molecules": 5, "mid_db_molecules": 6}[case])
    if case == "mid_db_molecules":
        # runs of 16-32 steps: flush masks, but counts past 7 planes
        ref = _random_sets(rng, 70, 30, (0, 3000), 2)
        qry = _random_sets(rng, 800, 250, (0, 3000), 1)
    elif case == "long_db_molecules":
        # short ref rows (8-plane counters) against database molecules of up
        # to 800 entries: lanes' runs of the balanced layout exceed 32 steps
        ref = _random_sets(rng, 70, 30, (0, 3000), 2)
        qry = _random_sets(rng, 800, 400, (0, 3000), 2)
    elif case == "small_vocab":
        ref = _random_sets(rng, 77, 30, (0, 200), 3)
        qry = _random_sets(rng, 1500, 30, (0, 200), 3)
    elif case == "negative_codes":
        ref = _random_sets(rng, 65, 40, (-(2 ** 31), 2 ** 31 - 1), 2)
        qry = _random_sets(rng, 900, 40, (-(2 ** 31), 2 ** 31 - 1), 2)
        qry[0][5, :ref[2][3]] = ref[0][3, :ref[2][3]]  # guarantee overlaps
        qry[1][5, :ref[2][3]] = ref[1][3, :ref[2][3]]
        qry[2][5] = ref[2][3]
        qry = (qry[0], qry[1], qry[2], qry[1].sum(1).astype(np.int32))
    elif case == "high_counts":  # counts past 255: 16-plane counters
        ref = _random_sets(rng, 40, 12, (0, 30), 400)
        qry = _random_sets(rng, 700, 12, (0, 30), 400)
    else:
        ref = _random_sets(rng, 50, 20, (0, 100), 2, p_empty=0.3)
        qry = _random_sets(rng, 600, 20, (0, 100), 2, p_empty=0.3)
        ref = (ref[0], ref[1], ref[2], np.where(np.arange(50) % 5 == 0, 0, ref[3]).astype(np.int32))
    gl = _engine()
    _load(gl, ref, qry)
    got = gl.getMultipleRows(0, ref[0].shape[0])
    assert np.array_equal(got, oracle.tanimoto_block(ref, qry, 0, ref[0].shape[0]))
    if case == "long_db_molecules":
        st = gl.dbStats()
        assert st["max_ng"] > 32 and st["ref_max_entries"] <= 255, st
    if case == "mid_db_molecules":
        st = gl.dbStats()
        assert 15 < st["max_ng"] <= 32 and st["ref_max_entries"] <= 255, st


def test_large_vocabulary_uses_merge_path(native, oracle):
    """A vocabulary too large for the shared-memory table takes the per-pair
    merge kernel; results are the same."""
    rng = np.random.default_rng(9)
    ref = _random_sets(rng, 40, 64, (0, 10 ** 9), 2)
    qry = _random_sets(rng, 2000, 64, (0, 10 ** 9), 2)
    qry[0][:40] = ref[0]
    qry[1][:40] = ref[1]
    qry[2][:40] = ref[2]
    qry = (qry[0], qry[1], qry[2], qry[1].sum(1).astype(np.int32))
    gl = _engine()
    _load(gl, ref, qry)
    got = gl.getMultipleRows(0, 40)
    assert np.array_equal(got, oracle.tanimoto_block(ref, qry, 0, 40))


def test_invalid_sets_are_rejected(native):
    gl = _engine()
    L = np.array([[5, 3, 0]], np.int32)
    C = np.array([[1, 1, 0]], np.int32)
    with pytest.raises(ValueError):
        gl.set_qsmiles(L, C, np.array([2], np.int32))
    with pytest.raises(ValueError):
        gl.set_qsmiles(np.array([[1, 2]], np.int32), np.array([[1, -1]], np.int32), np.array([2], np.int32))
    with pytest.raises(ValueError):
        gl.set_qsmiles(np.array([[1, 2]], np.int32), np.array([[1, 1]], np.int32), np.array([3], np.int32))
    with pytest.raises(ValueError):
        gl.set_qsmiles(np.zeros((2, 2), np.int32), np.zeros((2, 3), np.int32), np.zeros(2, np.int32))
    with pytest.raises(RuntimeError):
        gl.getMultipleRows(0, 1)


def test_engine_on_torch_default_stream(native, oracle, set4096):
    """A GPULingo object given torch's default stream (handle 0, the legacy
    default stream) is ordered with torch's work there: device inputs whose
    upload queues behind ~0.1 s of other work are read only once written,
    and the rows are ready for torch's next operation."""
    torch = pytest.importorskip("torch")
    from siml_gb300 import GPULingo
    gl = GPULingo(0, stream=torch.cuda.default_stream())
    for _ in range(2):
        torch.cuda._sleep(200_000_000)   # bounded spin on the default stream
        L, C, ln, mg = (torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in set4096)
        gl.set_qsmiles(L, C, ln, mg)
        gl.set_refsmiles(L[:256], C[:256], ln[:256], mg[:256])
        torch.cuda._sleep(200_000_000)
        out = gl.getMultipleRowsDevice(0, 256)
        got = out.cpu().numpy()
        assert np.array_equal(got, oracle.tanimoto_block(set4096, set4096, 0, 256))


def test_torch_device_inputs_and_outputs(native, oracle, set4096):
    torch = pytest.importorskip("torch")
    from siml_gb300 import GPULingo
    s = torch.cuda.Stream()
    gl = GPULingo(0, stream=s)
    L, C, ln, mg = (torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in set4096)
    gl.set_refsmiles(L[:512], C[:512], ln[:512], mg[:512])
    gl.set_qsmiles(L, C, ln, mg)
    out = gl.getMultipleRowsDevice(0, 512)
    assert out.is_cuda and out.shape == (512, 4096)
    want = oracle.tanimoto_block(set4096, set4096, 0, 512)
    assert np.array_equal(out.cpu().numpy(), want)
    # into a caller buffer with a padded row stride
    buf = torch.full((64, 4100), -5.0, device="cuda")
    gl.getMultipleRowsDevice(0, 64, out=buf[:, :4096])
    got = buf.cpu().numpy()
    assert np.array_equal(got[:, :4096], want[:64]) and np.all(got[:, 4096:] == -5.0)
    assert gl.launchCount() > 0


@pytest.mark.parametrize("window", [64, 128, 256])
def test_rows_window_layouts_bit_exact(native, oracle, set4096, golden, window):
    """Full-matrix results do not depend on the layout's sort window; the
    single-row form neither."""
    gl = _engine()
    _load(gl, set4096, set4096)
    gl.setRowsWindow(window)
    assert gl.rowsWindow() == window
    C = oracle.tanimoto_block(set4096, set4096, 0, 512)
    assert np.array_equal(gl.getMultipleRows(0, 512), C)
    q = (golden["lingos"], golden["counts"], golden["lengths"], golden["mags"])
    rows = golden["rows"]
    _load(gl, tuple(a[rows] for a in q), q)
    assert np.array_equal(gl.getMultipleRows(0, len(rows)), golden["tanimoto"])
    ref = tuple(a[rows] for a in q)
    cm_r, cm_q = ref[1].sum(1).astype(np.int32), q[1].sum(1).astype(np.int32)
    isct = oracle.isct_block(ref, q, 0, len(rows))
    for r in (0, 3, len(rows) - 1):
        u = (cm_r[r] + cm_q - isct[r]).astype(np.float32)
        want = np.where((ref[2][r] == 0) | (q[2] == 0), np.float32(0), isct[r].astype(np.float32) / u)
        assert np.array_equal(gl.getTanimotoRow(r)[0], want.astype(np.float32)), r
    with pytest.raises(ValueError):
        gl.setRowsWindow(48)


@pytest.mark.parametrize("fmt", [2, 3])
def test_rows_entry_formats_bit_exact(native, oracle, set4096, fmt):
    """4-byte vid and 4-byte byte-offset entries give the same matrix."""
    gl = _engine()
    _load(gl, set4096, set4096)
    gl.setRowsEntries(fmt)
    assert gl.rowsEntries() == fmt
    assert np.array_equal(gl.getMultipleRows(0, 300), oracle.tanimoto_block(set4096, set4096, 0, 300))
    assert gl.dbStats()["entry_bytes"] == 4
    with pytest.raises(ValueError):
        gl.setRowsEntries(9)


@pytest.mark.parametrize("layout", [0, 1])
@pytest.mark.parametrize("fmt", [0, 2])
def test_rows_padded_and_balanced_layouts(native, oracle, golden, layout, fmt):
    """Both lane packings of the full-matrix layout (and 2- or 4-byte entries)
    give the bit-exact matrix, on molecules of very different lengths."""
    from siml_gb300 import synthetic as S, _native as N
    db = S.smiles_set(S.SEED_RAGGED, S.BIMODAL_35_110, 3000)
    q = tuple(a[:200] for a in db)
    gl = _engine()
    N.check(N.lib().siml_set_tuning(gl._h, N.SIML_TUNE_ROWS_LAYOUT, layout))
    gl.setRowsEntries(fmt)
    _load(gl, q, db)
    assert np.array_equal(gl.getMultipleRows(0, 200), oracle.tanimoto_block(q, db, 0, 200))
    for r in (0, 77, 199):
        assert np.array_equal(gl.getTanimotoRow(r)[0], gl.getTanimotoRow(r)[0])
    g = (golden["lingos"], golden["counts"], golden["lengths"], golden["mags"])
    rows = golden["rows"]
    _load(gl, tuple(a[rows] for a in g), g)
    assert np.array_equal(gl.getMultipleRows(0, len(rows)), golden["tanimoto"])


def test_two_engines_in_two_threads(native, set4096):
    """Two engines with different shared-memory tables (about 120 KB and 75 KB,
    both on the balanced layout) launch the same row kernel from
    two host threads at once; every launch succeeds and gives the
    single-thread result."""
    import threading
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(21)
    big = _random_sets(rng, 1500, 40, (0, 2 ** 31 - 1), 1, p_empty=0.0)   # ~30K distinct pairs
    sets = [(big, big), (set4096, set4096)]
    engines, want = [], []
    for ref, qry in sets:
        gl = _engine()
        _load(gl, tuple(a[:64] for a in ref), qry)
        want.append(gl.getMultipleRowsDevice(0, 64).cpu())
        engines.append(gl)
    va, vb = engines[0].vocabStats(), engines[1].vocabStats()
    assert 25000 < va["nvid"] == va["ncommon"] < 38000 and vb["nvid"] < va["nvid"] - 10000
    errors = []

    def work(i):
        try:
            for _ in range(200):
                out = engines[i].getMultipleRowsDevice(0, 64)
                assert torch.equal(out.cpu(), want[i])
        except Exception as e:  # reported in the main thread
            errors.append(e)

    ts = [threading.Thread(target=work, args=(i,)) for i in range(2)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert not errors, errors


def test_rows_output_locations(native, oracle, set4096):
    """siml_rows into each output location gives the same bits: pageable
    host memory (a device block, then a copy), pinned host memory written by
    the kernels directly (SIML_HOST, and SIML_HOST_QUEUED, which returns at
    once), and device memory; padded row strides are kept; an unknown
    location is refused."""
    torch = pytest.importorskip("torch")
    import ctypes
    from siml_gb300 import GPULingo, _native as N
    gl = GPULingo(0)
    _load(gl, tuple(a[:300] for a in set4096), set4096)
    want = oracle.tanimoto_block(tuple(a[:300] for a in set4096), set4096, 0, 300)
    lib, rows = N.lib(), (20, 292)
    ld = 4100
    # pageable host memory
    page = np.full((rows[1] - rows[0], ld), -5.0, np.float32)
    N.check(lib.siml_rows(gl._h, rows[0], rows[1], page.ctypes.data, ld, N.SIML_HOST), "rows host")
    # pinned host memory, synchronous and queued
    pinned = torch.full((rows[1] - rows[0], ld), -5.0, dtype=torch.float32, pin_memory=True)
    N.check(lib.siml_rows(gl._h, rows[0], rows[1], pinned.data_ptr(), ld, N.SIML_HOST), "rows pinned")
    queued = torch.full((rows[1] - rows[0], ld), -5.0, dtype=torch.float32, pin_memory=True)
    N.check(lib.siml_rows(gl._h, rows[0], rows[1], queued.data_ptr(), ld, N.SIML_HOST_QUEUED), "rows queued")
    N.check(lib.siml_sync(gl._h), "sync")
    dev = torch.full((rows[1] - rows[0], ld), -5.0, dtype=torch.float32, device="cuda")
    N.check(lib.siml_rows(gl._h, rows[0], rows[1], dev.data_ptr(), ld, N.SIML_DEVICE), "rows device")
    N.check(lib.siml_sync(gl._h), "sync")
    for got in (page, pinned.numpy(), queued.numpy(), dev.cpu().numpy()):
        assert np.array_equal(got[:, :4096].view(np.uint32), want[rows[0]:rows[1]].view(np.uint32))
        assert np.all(got[:, 4096:] == -5.0)
    # pageable memory: refused, unless the runtime reports it as mapped host
    # memory (then it must be written correctly)
    page[:] = -5.0
    rc = lib.siml_rows(gl._h, 0, 8, page.ctypes.data, ld, N.SIML_HOST_QUEUED)
    assert rc in (N.SIML_OK, N.SIML_ERR_INVALID)
    if rc == N.SIML_OK:
        N.check(lib.siml_sync(gl._h), "sync")
        assert np.array_equal(page[:8, :4096].view(np.uint32), want[:8].view(np.uint32))
    assert lib.siml_rows(gl._h, 0, 8, page.ctypes.data, ld, 5) == N.SIML_ERR_INVALID
    # the public call (pinned output, queued) and its async form
    assert np.array_equal(gl.getMultipleRows(0, 300).view(np.uint32), want.view(np.uint32))
    gl.getMultipleRows_async(7, 70)
    assert np.array_equal(gl.retrieveAsyncResult().view(np.uint32), want[7:70].view(np.uint32))
