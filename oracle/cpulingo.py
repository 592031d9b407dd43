"""ORACLE — test infrastructure only.

Python side of the CPU oracle: a Python-3 restatement of the reference's
``pysiml.CPULingo`` (pysiml/CPULingo.py:43-197) and ``pysiml.compiler`` /
``pysiml.utilities`` entry points over ``oracle/liblingo_oracle.so`` (the C
restatement in oracle/lingo_oracle.c), plus CPU forms of the GPU-only
getNeighbors / histogram semantics and the project's top-k and 1000-bin
histogram.  Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU
baseline leg use this module; the product package never imports it.

``reference_module(name)`` imports the reference's own compiled extension
modules from oracle/_ref (built by ``make -C oracle ref`` where the reference
sources are present); it returns None where they are not built.
"""
from __future__ import annotations

import ctypes
import importlib
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liblingo_oracle.so")
REF_DIR = os.path.join(HERE, "_ref")


def _reference_root():
    """Root of the reference project (read in place, never copied): the
    SIML_REFERENCE_ROOT environment variable, else the root the reference
    build in oracle/_ref was made from (oracle/_ref/SOURCE), else None."""
    env = os.environ.get("SIML_REFERENCE_ROOT")
    if env:
        return env
    try:
        with open(os.path.join(REF_DIR, "SOURCE")) as fh:
            return fh.read().strip() or None
    except OSError:
        return None


REFERENCE_ROOT = _reference_root()

_lib = None


def build(force: bool = False) -> str:
    if force or not os.path.exists(LIB_PATH) or \
            os.path.getmtime(LIB_PATH) < os.path.getmtime(os.path.join(HERE, "lingo_oracle.c")):
        subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    return LIB_PATH


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        P, I64, I32, F32 = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_float
        sig = {
            "oracle_tanimoto_block": (I32, [P, P, P, P, I64, I64, P, P, P, P, I64, I64, P, I64, I32]),
            "oracle_isct_block": (I32, [P, P, P, I64, I64, P, P, P, I64, I64, P, I64, I32]),
            "oracle_neighbors_block": (I32, [P, P, P, P, I64, I64, P, P, P, P, I64, I64, F32, F32, I64,
                                             P, P, P, I32]),
            "oracle_row_histogram101": (I32, [P, I64, I64, I64, P]),
            "oracle_hist101_block": (I32, [P, P, P, P, I64, I64, P, P, P, P, I64, I64, P, I32]),
            "oracle_hist1000_block": (I32, [P, P, P, P, I64, I64, P, P, P, P, I64, I64, P, I32]),
            "oracle_topk_block": (I32, [P, P, P, P, I64, I64, P, P, P, P, I64, I64, I64, P, P, I32]),
            "oracle_compile_one": (I32, [ctypes.c_char_p, I64, P, P, P]),
            "oracle_compile_batch": (I64, [ctypes.c_char_p, P, I64, P, P, P, P, I64]),
            "oracle_tanimoto_pair": (F32, [P, P, P, P, I32, I32, I32, I32]),
            "oracle_synth_lengths": (I32, [ctypes.c_uint64, I32, I64, I64, P]),
            "oracle_synth_smiles": (I32, [ctypes.c_uint64, I32, I64, I64, P, I64, P]),
            "oracle_scan_block": (I32, [P, P, P, P, I64, I64, P, P, P, P, I64, I64, P, I64, F32, F32, I64,
                                        P, P, P, I64, P, P, P, P, I32]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def reference_module(name: str):
    """The reference's own compiled module (`_CPULingo`, `_ccompiler`,
    `_cpuutil`) from oracle/_ref, or None when it was not built here."""
    path = os.path.join(REF_DIR, name + ".so")
    if not os.path.exists(path):
        return None
    if REF_DIR not in sys.path:
        sys.path.insert(0, REF_DIR)
    try:
        return importlib.import_module(name)
    except ImportError:
        return None


def _c(a, dtype=np.int32):
    return np.ascontiguousarray(a, dtype=dtype)


def _set(L, C, lengths, mags):
    L = _c(L)
    C = _c(C)
    lengths = _c(np.asarray(lengths).reshape(-1))
    mags = _c(np.asarray(mags).reshape(-1))
    return L, C, lengths, mags


# --------------------------------------------------------------- compiler ----
def _pack(strings):
    strings = [s.encode("utf-8") if isinstance(s, str) else bytes(s) for s in strings]
    off = np.zeros(len(strings) + 1, dtype=np.int64)
    if strings:
        np.cumsum([len(s) for s in strings], out=off[1:])
    return b"".join(strings) or b"\0", off


def compile_strings(strings):
    """(lingos [n,w], counts [n,w], lengths [n], mags [n]) per the reference C
    compiler's rules (pysiml/_ccompiler.cpp:178-381)."""
    buf, off = _pack(strings)
    n = len(off) - 1
    L = lib()
    w = int(L.oracle_compile_batch(buf, off.ctypes.data, n, None, None, None, None, 0))
    lingos = np.zeros((n, w), np.int32)
    counts = np.zeros((n, w), np.int32)
    lengths = np.zeros(n, np.int32)
    mags = np.zeros(n, np.int32)
    if n and w:
        rc = L.oracle_compile_batch(buf, off.ctypes.data, n, lingos.ctypes.data, counts.ctypes.data,
                                    lengths.ctypes.data, mags.ctypes.data, w)
        assert rc >= 0
    elif n:
        for s in range(n):
            c = np.zeros(8, np.int32)
            k = np.zeros(8, np.int32)
            m = ctypes.c_int32(0)
            lengths[s] = 0
            L.oracle_compile_one(buf[off[s]:off[s + 1]] or b"\0", int(off[s + 1] - off[s]), c.ctypes.data,
                                 k.ctypes.data, ctypes.addressof(m))
            mags[s] = m.value
    return lingos, counts, lengths, mags


def synth_buffer(seed, model, n, first=0):
    """(bytes, offsets[n+1]) of molecules [first, first+n) of the seeded
    synthetic workload (model 0 uniform 20-90, 1 lognormal 45, 2 bimodal
    35/110), from the oracle's own copy of the generator."""
    L = lib()
    lens = np.empty(max(n, 1), np.int32)
    assert L.oracle_synth_lengths(int(seed), int(model), int(first), int(n), lens.ctypes.data) == 0
    total = int(lens[:n].sum(dtype=np.int64))
    buf = np.empty(max(total, 1), np.uint8)
    off = np.empty(n + 1, np.int64)
    assert L.oracle_synth_smiles(int(seed), int(model), int(first), int(n), buf.ctypes.data, buf.shape[0],
                                 off.ctypes.data) == 0
    return buf[:total].tobytes(), off


def compile_buffer(buf, off):
    """compile_strings over a concatenated buffer and its offsets[n+1]."""
    off = np.ascontiguousarray(off, dtype=np.int64)
    n = len(off) - 1
    L = lib()
    data = buf if len(buf) else b"\0"
    w = int(L.oracle_compile_batch(data, off.ctypes.data, n, None, None, None, None, 0))
    lingos = np.zeros((n, max(w, 1)), np.int32)
    counts = np.zeros((n, max(w, 1)), np.int32)
    lengths = np.zeros(n, np.int32)
    mags = np.zeros(n, np.int32)
    if n and w:
        assert L.oracle_compile_batch(data, off.ctypes.data, n, lingos.ctypes.data, counts.ctypes.data,
                                      lengths.ctypes.data, mags.ctypes.data, w) >= 0
        return lingos, counts, lengths, mags
    return compile_strings([buf[off[i]:off[i + 1]] for i in range(n)])


def synth_set(seed, model, n, first=0):
    """Compiled synthetic set (lingos, counts, lengths, mags), oracle-side."""
    return compile_buffer(*synth_buffer(seed, model, n, first))


def cSMILEStoMatrices(smileslist):
    """pysiml/compiler.py:53-82 over the oracle compiler."""
    items = list(smileslist)
    L, C, ln, mg = compile_strings(items)

    def name(s):
        f = s.split()
        return f[1] if len(f) > 1 else (b"" if isinstance(s, bytes) else "")
    return L, C, ln.reshape(-1, 1), mg.reshape(-1, 1), [name(s) for s in items]


def SMILEStoMatrices_python(smileslist):
    """Pure-Python-loop restatement of pysiml/compiler.py:98-194 (the Python
    compiler variant): first field, digits 1-9 -> '0', every 4-byte window
    (little-endian int32), sorted unique with counts; mags = count sums."""
    rows = []
    names = []
    for line in smileslist:
        b = line.encode("utf-8") if isinstance(line, str) else bytes(line)
        fields = b.split()
        smi = fields[0] if fields else b""
        smi = bytes(b"0"[0] if 0x31 <= ch <= 0x39 else ch for ch in smi)
        bag = {}
        for p in range(len(smi) - 3):
            v = smi[p] | (smi[p + 1] << 8) | (smi[p + 2] << 16) | (smi[p + 3] << 24)
            if v >= 1 << 31:
                v -= 1 << 32
            bag[v] = bag.get(v, 0) + 1
        rows.append(sorted(bag.items()))
        names.append(fields[1].decode("utf-8", "replace") if len(fields) > 1 else "")
    w = max([len(r) for r in rows] + [0])
    L = np.zeros((len(rows), w), np.int32)
    C = np.zeros_like(L)
    ln = np.zeros((len(rows), 1), np.int32)
    for i, r in enumerate(rows):
        ln[i] = len(r)
        for j, (k, c) in enumerate(r):
            L[i, j] = k
            C[i, j] = c
    return L, C, ln, C.sum(1).astype(np.int32), names


# ------------------------------------------------------------- similarity ----
class CPULingo:
    """pysiml/CPULingo.py:43-197 restated for Python 3 over the oracle."""

    def __init__(self):
        self.rlingos = self.rcounts = self.rlengths = self.rmags = None
        self.qlingos = self.qcounts = self.qlengths = self.qmags = None
        self.lastasyncresult = None

    def supportsParallel(self):
        return True

    def set_refsmiles(self, refsmilesmat, refcountsmat, reflengths, refmags=None):
        self.rlingos, self.rcounts = _c(refsmilesmat), _c(refcountsmat)
        self.rlengths = _c(np.asarray(reflengths).reshape(-1))
        # quirk kept: the default magnitude is the sum of the length vector
        # along axis 1 (pysiml/CPULingo.py:82), i.e. the unique-LINGO count
        self.rmags = _c(np.asarray(refmags).reshape(-1)) if refmags is not None else \
            _c(np.asarray(reflengths).reshape(len(self.rlengths), -1).sum(1))

    def set_qsmiles(self, qsmilesmat, qcountsmat, querylengths, querymags=None):
        self.qlingos, self.qcounts = _c(qsmilesmat), _c(qcountsmat)
        self.qlengths = _c(np.asarray(querylengths).reshape(-1))
        self.qmags = _c(np.asarray(querymags).reshape(-1)) if querymags is not None else \
            _c(np.asarray(querylengths).reshape(len(self.qlengths), -1).sum(1))

    def _check(self):
        if any(x is None for x in (self.rlingos, self.qlingos)):
            raise ValueError("CPULingo object not fully initialized")

    def getMultipleRows_async(self, rowbase, rowlimit, nprocs=1):
        self._check()
        self.lastasyncresult = tanimoto_block((self.rlingos, self.rcounts, self.rlengths, self.rmags),
                                              (self.qlingos, self.qcounts, self.qlengths, self.qmags),
                                              rowbase, rowlimit, nthreads=max(1, nprocs))

    def getMultipleRows(self, rowbase, rowlimit, nprocs=1):
        self.getMultipleRows_async(rowbase, rowlimit, nprocs)
        return self.retrieveAsyncResult()

    def getTanimotoRow_async(self, row):
        self.getMultipleRows_async(row, row + 1)

    def getTanimotoRow(self, row):
        self.getTanimotoRow_async(row)
        return self.retrieveAsyncResult()

    def retrieveAsyncResult(self):
        return self.lastasyncresult

    def asyncOperationsDone(self):
        return True


def _args(ref, qry, rowbase, rowlimit):
    rl, rc, rlen, rmag = _set(*ref)
    ql, qc, qlen, qmag = _set(*qry)
    rows = rowlimit - rowbase
    rw = rl.shape[1] if rl.ndim == 2 else 0
    qw = ql.shape[1] if ql.ndim == 2 else 0
    base = rowbase * max(rw, 0)
    rlp = rl.ctypes.data + 4 * base
    rcp = rc.ctypes.data + 4 * base
    return (rlp, rcp, rlen.ctypes.data + 4 * rowbase, rmag.ctypes.data + 4 * rowbase, rows, max(rw, 1),
            ql.ctypes.data, qc.ctypes.data, qlen.ctypes.data, qmag.ctypes.data, ql.shape[0], max(qw, 1)), \
        (rl, rc, rlen, rmag, ql, qc, qlen, qmag)


def tanimoto_block(ref, qry, rowbase, rowlimit, nthreads=0):
    """float32 [rows, nq] — getTanimotoBlock[Parallel] (pysiml/_CPULingo.c:83-465)."""
    a, keep = _args(ref, qry, rowbase, rowlimit)
    out = np.empty((a[4], a[10]), np.float32)
    lib().oracle_tanimoto_block(*a, out.ctypes.data, max(a[10], 1), int(nthreads))
    return out


def isct_block(ref, qry, rowbase, rowlimit, nthreads=0):
    a, keep = _args(ref, qry, rowbase, rowlimit)
    out = np.empty((a[4], a[10]), np.int32)
    lib().oracle_isct_block(a[0], a[1], a[2], a[4], a[5], a[6], a[7], a[8], a[10], a[11], out.ctypes.data,
                            max(a[10], 1), int(nthreads))
    return out


def pitch_of(maxneighbors):
    """Row pitch of getNeighbors' output, 16*ceil(maxneighbors/16) (pysiml/GPULingo.py:491)."""
    return 16 * ((int(maxneighbors) + 15) // 16)


def neighbors_block(ref, qry, rowbase, rowlimit, lo, hi=1.1, maxneighbors=None, nthreads=0):
    """getNeighbors semantics (pysiml/kernels.py:393-475): (idx [rows, pitch],
    sims [rows, pitch], counts [rows]); entries past a row's count are -1/NaN."""
    a, keep = _args(ref, qry, rowbase, rowlimit)
    if maxneighbors is None:
        maxneighbors = a[10]
    pitch = pitch_of(maxneighbors)
    idx = np.full((a[4], pitch), -1, np.int32)
    sims = np.full((a[4], pitch), np.nan, np.float32)
    counts = np.zeros(a[4], np.int32)
    lib().oracle_neighbors_block(*a, np.float32(lo), np.float32(hi), pitch, idx.ctypes.data, sims.ctypes.data,
                                 counts.ctypes.data, int(nthreads))
    return idx, sims, counts


def neighbors_range_block(ref, qry, rowbase, rowlimit, col_begin, col_end, lo, hi=1.1, maxneighbors=None,
                          nthreads=0):
    """getNeighbors against query columns [col_begin, col_end) only: the
    reference's search run on that slice of the query set (so overflow waves
    start at col_begin), indices shifted back to absolute query indices."""
    sl = tuple(None if x is None else np.asarray(x)[col_begin:col_end] for x in qry)
    if maxneighbors is None:
        maxneighbors = np.asarray(qry[0]).shape[0]
    idx, sims, counts = neighbors_block(ref, sl, rowbase, rowlimit, lo, hi, maxneighbors, nthreads)
    idx = np.where(idx >= 0, idx + np.int32(col_begin), idx).astype(np.int32)
    return idx, sims, counts


def hist101_block(ref, qry, rowbase, rowlimit, nthreads=0):
    """int32 [rows, 101] — getMultipleHistogrammedRows (pysiml/kernels.py:606-666)."""
    a, keep = _args(ref, qry, rowbase, rowlimit)
    out = np.zeros((a[4], 101), np.int32)
    lib().oracle_hist101_block(*a, out.ctypes.data, int(nthreads))
    return out


def hist1000_block(ref, qry, rowbase, rowlimit, nthreads=0):
    """uint64 [1000], bin = min((unsigned)(t*1000.0f), 999)."""
    a, keep = _args(ref, qry, rowbase, rowlimit)
    out = np.zeros(1000, np.uint64)
    lib().oracle_hist1000_block(*a, out.ctypes.data, int(nthreads))
    return out


def topk_block(ref, qry, rowbase, rowlimit, k, nthreads=0):
    """(idx [rows, k], sims [rows, k]) — k best per row, ties to lower index."""
    a, keep = _args(ref, qry, rowbase, rowlimit)
    idx = np.empty((a[4], k), np.int32)
    sims = np.empty((a[4], k), np.float32)
    rc = lib().oracle_topk_block(*a, int(k), idx.ctypes.data, sims.ctypes.data, int(nthreads))
    assert rc == 0
    return idx, sims


def scan_block(ref, qry, rowbase, rowlimit, rows=True, lo=None, hi=1.1, maxneighbors=None, k=0,
               hist101=False, hist1000=None, nthreads=0):
    """Every product of a row block from one merge per pair (oracle_scan_block):
    a dict with 'rows' (fp32 [rows, nq]), 'nbr' (idx, sims, counts as
    neighbors_block, when lo is given), 'topk' (idx, sims as topk_block, when
    k > 0), 'hist101' (int32 [rows, 101]); hist1000, a uint64 [1000] array, is
    accumulated into when given."""
    a, keep = _args(ref, qry, rowbase, rowlimit)
    nr, nq = a[4], a[10]
    res = {}
    out = np.empty((nr, nq), np.float32) if rows else None
    nb = None
    if lo is not None:
        pitch = pitch_of(nq if maxneighbors is None else maxneighbors)
        nb = (np.full((nr, pitch), -1, np.int32), np.full((nr, pitch), np.nan, np.float32), np.zeros(nr, np.int32))
    else:
        pitch = 0
    tk = (np.empty((nr, k), np.int32), np.empty((nr, k), np.float32)) if k > 0 else None
    h101 = np.zeros((nr, 101), np.int32) if hist101 else None
    if hist1000 is not None:
        assert hist1000.dtype == np.uint64 and hist1000.shape == (1000,) and hist1000.flags.c_contiguous
    ptr = lambda x: None if x is None else x.ctypes.data
    rc = lib().oracle_scan_block(*a, ptr(out), max(nq, 1), np.float32(lo if lo is not None else 0.0),
                                 np.float32(hi), pitch, ptr(nb[0] if nb else None), ptr(nb[1] if nb else None),
                                 ptr(nb[2] if nb else None), int(k), ptr(tk[0] if tk else None),
                                 ptr(tk[1] if tk else None), ptr(h101), ptr(hist1000), int(nthreads))
    assert rc == 0
    if out is not None:
        res["rows"] = out
    if nb is not None:
        res["nbr"] = nb
    if tk is not None:
        res["topk"] = tk
    if h101 is not None:
        res["hist101"] = h101
    return res


def rowHistogram101(M):
    """uint32 [rows, 101] — pysiml/utilities.py:44-55 (float32 input)."""
    M = np.ascontiguousarray(M, dtype=np.float32)
    out = np.zeros((M.shape[0], 101), np.uint32)
    lib().oracle_row_histogram101(M.ctypes.data, M.shape[0], M.shape[1], M.shape[1], out.ctypes.data)
    return out
