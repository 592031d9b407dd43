"""The scheduled full-matrix kernel (k_rows_sched, the default path of
getMultipleRows), with 64-row groups (the default) and 32-row groups:
bit-exact against the oracle at window edges (database sizes around the
window and not multiples of 4), row counts that are not multiples of the
group, molecules long enough that chunks are split across warps, magnitudes
outside the fast division's range, empty molecules, a vocabulary larger than
the 64-row table (numbered by frequency, its rarest pairs through the hash),
and the fallbacks when the output cannot take 16-byte stores."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(params=[64, 32], ids=["rows64", "rows32"])
def rows(request):
    return request.param


def _engine(rows=64):
    from siml_gb300 import GPULingo, _native as N
    gl = GPULingo(0)
    N.check(N.lib().siml_set_tuning(gl._h, N.SIML_TUNE_SCHED_ROWS, rows))
    return gl


def _load(gl, ref, qry):
    gl.set_refsmiles(*ref)
    gl.set_qsmiles(*qry)


def _bimodal(n, first=0):
    from siml_gb300 import synthetic as S
    return S.smiles_set(S.SEED_RAGGED, S.BIMODAL_35_110, n, first=first)


@pytest.mark.parametrize("groups", [2, 4])
@pytest.mark.parametrize("nq", [1, 33, 255, 257, 511, 512, 513, 1025, 2049, 4099, 6150])
def test_sched_window_edges(native, oracle, nq, groups, rows):
    from siml_gb300 import _native as N
    db = _bimodal(nq)
    ref = _bimodal(77, first=100_000)
    gl = _engine(rows)
    N.check(N.lib().siml_set_tuning(gl._h, N.SIML_TUNE_SCHED_GROUPS, groups))
    _load(gl, ref, db)
    info = gl.rowsInfo()
    win = (2048 if rows == 32 else 1024) // groups
    assert info["scheduled"] == 1 and info["windows"] == (nq + win - 1) // win
    want = oracle.tanimoto_block(ref, db, 0, 77)
    for r0, r1 in [(0, 77), (0, 1), (5, 36), (40, 73)]:
        got = gl.getMultipleRows(r0, r1)
        assert np.array_equal(got.view(np.uint32), want[r0:r1].view(np.uint32)), (r0, r1)


def test_sched_splits_long_chunks(native, oracle, rows):
    """A bimodal database (30% of molecules around 110 characters): windows
    hold chunks several times longer than the mean share of a warp, so they
    are split into items whose counts add in shared memory."""
    db = _bimodal(20_000)
    ref = _bimodal(64, first=50_000)
    gl = _engine(rows)
    _load(gl, ref, db)
    info = gl.rowsInfo()
    nchunks = (20_000 + 31) // 32
    assert info["scheduled"] == 1 and info["items"] > nchunks   # some chunks were split
    got = gl.getMultipleRows(0, 64)
    assert np.array_equal(got.view(np.uint32), oracle.tanimoto_block(ref, db, 0, 64).view(np.uint32))


def test_sched_magnitudes_outside_the_fast_range(native, oracle, rows):
    """User magnitudes of zero, below the count sum or above 32,768, on rows
    and on columns, take the IEEE division; the rest of each 4-column group
    with them."""
    db = tuple(np.array(a) for a in _bimodal(3000))
    ref = tuple(np.array(a) for a in _bimodal(40, first=9000))
    rng = np.random.default_rng(7)
    qm = db[3].copy()
    pick = rng.choice(3000, 60, replace=False)
    qm[pick[:20]] = 0
    qm[pick[20:40]] = np.maximum(qm[pick[20:40]] - 3, 0)
    qm[pick[40:]] = 40000 + pick[40:]
    rm = ref[3].copy()
    rm[[3, 17]] = [0, 50000]
    db2 = (db[0], db[1], db[2], qm)
    ref2 = (ref[0], ref[1], ref[2], rm)
    gl = _engine(rows)
    _load(gl, ref2, db2)
    assert gl.rowsInfo()["scheduled"] == 1
    assert np.array_equal(gl.getMultipleRows(0, 40).view(np.uint32),
                          oracle.tanimoto_block(ref2, db2, 0, 40).view(np.uint32))
    # rows that are all in the fast range, against the same columns
    ok = [r for r in range(40) if r not in (3, 17)]
    ref3 = tuple(a[ok] for a in ref2)
    _load(gl, ref3, db2)
    assert np.array_equal(gl.getMultipleRows(0, len(ok)).view(np.uint32),
                          oracle.tanimoto_block(ref3, db2, 0, len(ok)).view(np.uint32))


def test_sched_empty_molecules(native, oracle, rows):
    from siml_gb300.compiler import cSMILEStoMatrices
    from siml_gb300 import synthetic as S
    smi = S.smiles_list(S.SEED_ALLPAIRS, S.UNIFORM_20_90, 2500)
    smi[::97] = [b"C"] * len(smi[::97])      # no LINGOs at all
    smi[5::131] = [b"CCC"] * len(smi[5::131])
    L, C, ln, mg, _ = cSMILEStoMatrices(smi)
    db = (L, C, ln.reshape(-1), mg.reshape(-1))
    ref = tuple(a[:50] for a in db)
    gl = _engine(rows)
    _load(gl, ref, db)
    assert gl.rowsInfo()["scheduled"] == 1
    assert np.array_equal(gl.getMultipleRows(0, 50).view(np.uint32),
                          oracle.tanimoto_block(ref, db, 0, 50).view(np.uint32))


def test_sched_output_strides_and_fallbacks(native, oracle, rows):
    """A row stride that is a multiple of 4 takes the scheduled kernel with
    padding left untouched; a stride that is not, or an output not on a
    16-byte boundary, takes the natural-order kernel; all agree."""
    torch = pytest.importorskip("torch")
    db = _bimodal(5000)
    ref = _bimodal(45, first=70_000)
    want = oracle.tanimoto_block(ref, db, 0, 45)
    gl = _engine(rows)
    _load(gl, ref, db)
    for ld, off in [(5004, 0), (5001, 0), (5004, 1)]:
        buf = torch.full((45 * ld + 8,), -3.0, dtype=torch.float32, device="cuda")
        out = buf[off:off + 45 * ld].view(45, ld)[:, :5000]
        gl.getMultipleRowsDevice(0, 45, out=out)
        got = out.cpu().numpy()
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (ld, off)
        pad = buf[off:off + 45 * ld].view(45, ld)[:, 5000:]
        assert bool((pad == -3.0).all()), (ld, off)


def test_sched_equals_balanced_layout(native, set4096, rows):
    from siml_gb300 import _native as N
    gl = _engine(rows)
    _load(gl, tuple(a[:300] for a in set4096), set4096)
    a = gl.getMultipleRowsDevice(0, 300).cpu()
    N.check(N.lib().siml_set_tuning(gl._h, N.SIML_TUNE_ROWS_LAYOUT, N.SIML_ROWS_BALANCED))
    assert gl.rowsInfo()["scheduled"] == 0
    b = gl.getMultipleRowsDevice(0, 300).cpu()
    N.check(N.lib().siml_set_tuning(gl._h, N.SIML_TUNE_ROWS_LAYOUT, N.SIML_ROWS_SCHEDULED))
    c = gl.getMultipleRowsDevice(0, 300).cpu()
    import torch
    assert torch.equal(a.view(torch.int32), b.view(torch.int32)) and torch.equal(a.view(torch.int32),
                                                                                 c.view(torch.int32))


def test_sched_vocabulary_larger_than_the_64_row_table(native, oracle):
    """200,000 lognormal molecules hold more pairs than the 64-row table
    (about 16.9K): the vocabulary is numbered by frequency, the kernel keeps
    the most frequent pairs and looks the rest up in its 64-bit-mask hash.
    Equal to the oracle and to 32-row groups, which hold the whole table."""
    from siml_gb300 import synthetic as S
    db = S.smiles_set(S.SEED_DB_1M, S.LOGNORMAL_45, 200_000)
    ref = S.smiles_set(S.SEED_DB_1M, S.LOGNORMAL_45, 130, first=1_000_000)
    from siml_gb300 import _native as N
    want = oracle.tanimoto_block(ref, db, 0, 130)
    for r, fix in ((64, 1), (64, 0), (32, 1)):
        gl = _engine(r)
        # 1: rare pairs skipped by the table pass and recomputed after it;
        # 0: counted through the kernel's hash
        N.check(N.lib().siml_set_tuning(gl._h, N.SIML_TUNE_RARE_FIXUP, fix))
        _load(gl, ref, db)
        assert gl.vocabStats()["nvid"] > 20_000
        assert gl.rowsInfo()["scheduled"] == 1
        got = gl.getMultipleRows(0, 130)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (r, fix)
        rv = gl.rowsVocab()
        split = rv["table_pairs"] < gl.vocabStats()["nvid"]
        assert split == (r == 64) and (rv["nrare"] > 0) == split, (r, rv)
        # the path the launch took: 2 second pass, 1 hash, 0 nothing rare
        assert rv["rare_path"] == ((2 if fix else 1) if split else 0), (r, fix, rv)
        # a row range that does not start at 0, into a strided device output
        torch = pytest.importorskip("torch")
        buf = torch.full((64, 200_008), -5.0, dtype=torch.float32, device="cuda")
        out = buf[:, :200_000]
        gl.getMultipleRowsDevice(37, 101, out=out)
        assert np.array_equal(out.cpu().numpy().view(np.uint32), want[37:101].view(np.uint32)), (r, fix)
        assert bool((buf[:, 200_000:] == -5.0).all())
