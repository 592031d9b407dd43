"""Drop-in for pySIML's ``pysiml.GPULingo.GPULingo`` (pysiml/GPULingo.py:158-648).

Same constructor, method names, positional signatures, return shapes and
async protocol as the reference; the work runs in the sm_103a kernels of
``libsiml_gb300.so`` through its C ABI (include/siml_gb300.h).

Differences a caller may notice (all listed in the repository's design notes):

* The reference's texture-size limits (ref set <= 32768 rows, query set <=
  65536 molecules, <= 32768 padded LINGO columns, GPULingo.py:206-207,
  269-270) do not apply.
* Input codes of each molecule must be strictly increasing and counts
  non-negative (what the SMILES compiler produces); the reference's merge
  silently computes something else for unsorted input, this raises
  ``ValueError``.
* ``getNeighbors`` returns at most ``pitch`` columns even when a row
  overflowed (the reference copies ``max(count)`` columns and reads past its
  buffer in that case, GPULingo.py:597-613).
* ``retrieveAsyncResult`` without a pending call raises ``RuntimeError``
  (the reference raises an undefined name, GPULingo.py:623-640).

Inputs may be numpy arrays or torch tensors (CPU or CUDA).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native as N

try:  # torch provides device buffers and stream interop; it is optional
    import torch
except Exception:  # pragma: no cover - torch is present wherever tests run
    torch = None


def _prep_matrix(a, what):
    if torch is not None and isinstance(a, torch.Tensor):
        if a.dim() != 2:
            raise ValueError("%s did not have dimension 2" % what)
        return a.to(torch.int32).contiguous()
    a = np.ascontiguousarray(np.asarray(a), dtype=np.int32)
    if a.ndim != 2:
        raise ValueError("%s did not have dimension 2" % what)
    return a


def _prep_vector(a, n, what):
    if a is None:
        return None
    if torch is not None and isinstance(a, torch.Tensor):
        if not (a.dim() == 1 or (a.dim() == 2 and a.shape[1] == 1)):
            raise ValueError("%s was not 1-D" % what)
        a = a.reshape(-1).to(torch.int32).contiguous()
    else:
        a = np.asarray(a)
        if not (a.ndim == 1 or (a.ndim == 2 and a.shape[1] == 1)):
            raise ValueError("%s was not 1-D" % what)
        a = np.ascontiguousarray(a.reshape(-1), dtype=np.int32)
    if a.shape[0] != n:
        raise ValueError("%s length did not equal number of rows of its Lingo matrix" % what)
    return a


def _where(*arrays):
    for a in arrays:
        if a is not None and torch is not None and isinstance(a, torch.Tensor) and a.is_cuda:
            return N.SIML_DEVICE
    return N.SIML_HOST


class GPULingo:
    """LINGO similarities on CUDA device *deviceID* (pysiml/GPULingo.py:158-173)."""

    def __init__(self, deviceID=0, stream=None):
        self.deviceID = deviceID
        self.nref = 0
        self.nquery = 0
        self.rlengths = None
        self.rshape = None
        self.qshape = None
        self.last_async_width = None
        self._pending = None
        self._h = ctypes.c_void_p()
        L = N.lib()
        N.check(L.siml_create(int(deviceID), ctypes.byref(self._h)), "siml_create")
        # With torch present the engine runs on a torch stream so that device
        # buffers from torch's caching allocator are ordered correctly.
        if stream is None and torch is not None:
            stream = torch.cuda.Stream(device=torch.device("cuda", deviceID))
        self._stream = stream
        if stream is not None:
            N.check(L.siml_set_stream(self._h, N.stream_arg(stream)), "siml_set_stream")

    @property
    def stream(self):
        """The torch stream the engine's kernels run on (None without torch)."""
        return self._stream

    def _enter(self):
        """Orders the engine's stream after work queued on torch's current stream."""
        if self._stream is not None:
            self._stream.wait_stream(torch.cuda.current_stream(self._device()))

    def _leave(self, *tensors):
        """Keeps tensors written by the engine alive for its stream and orders
        torch's current stream after the engine's work."""
        if self._stream is not None:
            for t in tensors:
                if t is not None and isinstance(t, torch.Tensor) and t.is_cuda:
                    t.record_stream(self._stream)
            torch.cuda.current_stream(self._device()).wait_stream(self._stream)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                N.lib().siml_destroy(h)
            except Exception:
                pass
            self._h = None

    # ------------------------------------------------------------------ sets
    def _set(self, fn, mat, cnt, lengths, mags, tag):
        L = N.lib()
        mat = _prep_matrix(mat, "%s Lingo matrix" % tag)
        cnt = _prep_matrix(cnt, "%s Lingo count matrix" % tag)
        if tuple(mat.shape) != tuple(cnt.shape):
            raise ValueError("%s Lingo and Lingo count matrix did not have identical shapes" % tag)
        n, w = int(mat.shape[0]), int(mat.shape[1])
        lengths = _prep_vector(lengths, n, "%s length vector" % tag)
        mags = _prep_vector(mags, n, "%s magnitude vector" % tag)
        where = _where(mat, cnt, lengths, mags)
        self._enter()
        N.check(fn(self._h, N.ptr(mat), N.ptr(cnt), N.ptr(lengths), N.ptr(mags), n, w, w, where), tag)
        return n, w, lengths

    def set_refsmiles(self, refsmilesmat, refcountsmat, reflengths, refmags=None):
        """Sets the reference SMILES set (pysiml/GPULingo.py:187-242).  Magnitudes
        default to the per-row count sums when *refmags* is None."""
        n, w, lengths = self._set(N.lib().siml_set_ref, refsmilesmat, refcountsmat, reflengths, refmags,
                                  "Reference")
        self.nref = n
        self.rshape = (n, w)
        self.rlengths = lengths

    def set_qsmiles(self, qsmilesmat, qcountsmat, querylengths, querymags=None):
        """Sets the query SMILES set — the resident database (pysiml/GPULingo.py:246-313)."""
        n, w, _ = self._set(N.lib().siml_set_query, qsmilesmat, qcountsmat, querylengths, querymags, "Query")
        self.nquery = n
        self.qshape = (n, w)

    # --------------------------------------------------------------- helpers
    def _device(self):
        return torch.device("cuda", self.deviceID)

    def _check_rows(self, rowbase, rowlimit):
        if self.qshape is None or self.rshape is None:
            raise RuntimeError("GPULingo object not fully initialized (call set_refsmiles and set_qsmiles)")
        if rowbase < 0 or rowlimit > self.nref:
            raise RuntimeError("row range [%d, %d) outside the reference set of %d rows" % (rowbase, rowlimit, self.nref))
        if rowlimit < rowbase:
            raise ValueError("negative dimensions are not allowed")

    # ------------------------------------------------------------ row blocks
    def getTanimotoRow(self, rowidx):
        """Single Tanimoto row (pysiml/GPULingo.py:316-326)."""
        self.getTanimotoRow_async(rowidx)
        return self.retrieveAsyncResult()

    def getTanimotoRow_async(self, rowidx):
        """Queues one row; magnitudes are recomputed from the counts as the
        reference's single-row kernel does (pysiml/kernels.py:234-270)."""
        self._check_rows(rowidx, rowidx + 1)
        nq = self.nquery
        if torch is not None:
            out = torch.empty((1, max(nq, 1)), dtype=torch.float32, device=self._device())
            self._enter()
            N.check(N.lib().siml_row_single(self._h, int(rowidx), out.data_ptr(), N.SIML_DEVICE), "getTanimotoRow")
        else:
            out = np.empty((1, max(nq, 1)), dtype=np.float32)
            N.check(N.lib().siml_row_single(self._h, int(rowidx), out.ctypes.data, N.SIML_HOST), "getTanimotoRow")
        self.last_async_width = nq
        self._set_pending(("matrix", out, nq))

    def getMultipleRows(self, rowbase, rowlimit):
        """Tanimoto rows [rowbase, rowlimit) x all queries (pysiml/GPULingo.py:354-363)."""
        self.getMultipleRows_async(rowbase, rowlimit)
        return self.retrieveAsyncResult()

    def getMultipleRows_async(self, rowbase, rowlimit):
        """Queues the row block (pysiml/GPULingo.py:366-404)."""
        self._check_rows(rowbase, rowlimit)
        rows, nq = rowlimit - rowbase, self.nquery
        if torch is not None:
            # the kernels write the block straight into pinned host memory
            # (reused by torch's host allocator) over the host link, queued on
            # the engine's stream: no device block and no separate copy
            host = torch.empty((rows, max(nq, 1)), dtype=torch.float32, pin_memory=True)
            self._enter()
            try:
                N.check(N.lib().siml_rows(self._h, int(rowbase), int(rowlimit), host.data_ptr(), max(nq, 1),
                                          N.SIML_HOST_QUEUED), "getMultipleRows")
            except Exception:
                N.lib().siml_sync(self._h)   # kernels queued before the failure may still write `host`
                raise
            self.last_async_width = nq
            self._set_pending(("matrix", host, nq))
            return
        else:
            out = np.empty((rows, max(nq, 1)), dtype=np.float32)
            N.check(N.lib().siml_rows(self._h, int(rowbase), int(rowlimit), out.ctypes.data, max(nq, 1),
                                      N.SIML_HOST), "getMultipleRows")
        self.last_async_width = nq
        self._set_pending(("matrix", out, nq))

    def getMultipleRowsDevice(self, rowbase, rowlimit, out=None):
        """Row block left in device memory as a CUDA float32 tensor [rows, nquery]
        (or written into *out*, any row stride).  Ordered after the engine's
        stream on torch's current stream."""
        self._check_rows(rowbase, rowlimit)
        rows, nq = rowlimit - rowbase, self.nquery
        if out is None:
            out = torch.empty((rows, max(nq, 1)), dtype=torch.float32, device=self._device())
        if out.dtype != torch.float32 or not out.is_cuda or out.stride(1) != 1:
            raise ValueError("out must be a CUDA float32 tensor with unit column stride")
        self._enter()
        N.check(N.lib().siml_rows(self._h, int(rowbase), int(rowlimit), out.data_ptr(), out.stride(0),
                                  N.SIML_DEVICE), "getMultipleRowsDevice")
        self._leave(out)
        return out

    # ------------------------------------------------------------ histograms
    def getMultipleHistogrammedRows(self, rowbase, rowlimit):
        """Per-row 101-bin histograms of rows [rowbase, rowlimit), bins
        (unsigned)(T*100) (pysiml/GPULingo.py:407-417); int32 [rows, 101]."""
        self.getMultipleHistogrammedRows_async(rowbase, rowlimit)
        return self.retrieveAsyncResult()

    def getMultipleHistogrammedRows_async(self, rowbase, rowlimit):
        """Queues the histograms (pysiml/GPULingo.py:420-463)."""
        self._check_rows(rowbase, rowlimit)
        rows = rowlimit - rowbase
        L = N.lib()
        if torch is not None:
            out = torch.empty((rows, 112), dtype=torch.int32, device=self._device())
            self._enter()
            if rows:
                N.check(L.siml_hist101(self._h, int(rowbase), int(rowlimit), out.data_ptr(), 112, N.SIML_DEVICE),
                        "getMultipleHistogrammedRows")
        else:
            out = np.zeros((rows, 112), dtype=np.int32)
            if rows:
                N.check(L.siml_hist101(self._h, int(rowbase), int(rowlimit), out.ctypes.data, 112, N.SIML_HOST),
                        "getMultipleHistogrammedRows")
        self.last_async_width = 101
        self._set_pending(("matrix", out, 101))

    def getSimilarityHistogram(self, rowbase, rowlimit, out=None):
        """One 1000-bin histogram of every similarity of rows [rowbase,
        rowlimit) x all queries, bin min((unsigned)(T*1000), 999); uint64
        [1000].  Accumulates into *out* when given (numpy or CUDA tensor)."""
        self._check_rows(rowbase, rowlimit)
        L = N.lib()
        if torch is not None and isinstance(out, torch.Tensor) and out.is_cuda:
            if out.dtype != torch.int64 or out.numel() != 1000:
                raise ValueError("out must be a CUDA int64 tensor of 1000 elements")
            self._enter()
            N.check(L.siml_hist_global(self._h, int(rowbase), int(rowlimit), out.data_ptr(), N.SIML_DEVICE),
                    "getSimilarityHistogram")
            self._leave(out)
            return out
        host = np.zeros(1000, dtype=np.uint64) if out is None else out
        if host.dtype != np.uint64 or host.shape != (1000,) or not host.flags.c_contiguous:
            raise ValueError("out must be a contiguous uint64 array of 1000 elements")
        self._enter()
        N.check(L.siml_hist_global(self._h, int(rowbase), int(rowlimit), host.ctypes.data, N.SIML_HOST),
                "getSimilarityHistogram")
        return host

    # ----------------------------------------------------------------- top-k
    def getTopK(self, rowbase, rowlimit, k):
        """The k most similar queries of each ref row in [rowbase, rowlimit):
        (indices int32 [rows, k], similarities float32 [rows, k]), best first,
        ties to the lower query index; rows with fewer than k queries are
        padded with -1 / -1.0."""
        self._check_rows(rowbase, rowlimit)
        rows = rowlimit - rowbase
        k = int(k)
        if k < 1:
            raise ValueError("k must be >= 1")
        L = N.lib()
        if torch is not None:
            idx = torch.empty((rows, k), dtype=torch.int32, device=self._device())
            sims = torch.empty((rows, k), dtype=torch.float32, device=self._device())
            self._enter()
            if rows:
                N.check(L.siml_topk(self._h, int(rowbase), int(rowlimit), k, idx.data_ptr(), sims.data_ptr(),
                                    N.SIML_DEVICE), "getTopK")
            N.check(L.siml_sync(self._h), "siml_sync")
            return idx.cpu().numpy(), sims.cpu().numpy()
        idx = np.empty((rows, k), dtype=np.int32)
        sims = np.empty((rows, k), dtype=np.float32)
        if rows:
            N.check(L.siml_topk(self._h, int(rowbase), int(rowlimit), k, idx.ctypes.data, sims.ctypes.data,
                                N.SIML_HOST), "getTopK")
        return idx, sims

    def topKDevice(self, rowbase, rowlimit, k, idx, sims):
        """Top-k into caller CUDA tensors idx int32 [rows, k], sims float32 [rows, k]."""
        self._check_rows(rowbase, rowlimit)
        self._enter()
        N.check(N.lib().siml_topk(self._h, int(rowbase), int(rowlimit), int(k), idx.data_ptr(), sims.data_ptr(),
                                  N.SIML_DEVICE), "topKDevice")
        self._leave(idx, sims)

    # ------------------------------------------------------------- neighbors
    def getNeighbors(self, rowbase, rowlimit, lowerbound, upperbound=1.1, maxneighbors=None):
        """Query indices with lowerbound <= T < upperbound per ref row
        (pysiml/GPULingo.py:516-534).  Returns (matrix [rows, max count], counts
        [rows]); entries of row i beyond counts[i] are undefined, and a count
        above the pitch 16*ceil(maxneighbors/16) marks an overflowed row."""
        self.getNeighbors_async(rowbase, rowlimit, lowerbound, upperbound, maxneighbors)
        return self.retrieveAsyncResult()

    def getNeighbors_async(self, rowbase, rowlimit, lowerbound, upperbound=1.1, maxneighbors=None):
        """Queues a neighbour search (pysiml/GPULingo.py:467-513)."""
        self._queue_neighbors(rowbase, rowlimit, lowerbound, upperbound, maxneighbors, False)

    def getNeighborsWithSimilarities(self, rowbase, rowlimit, lowerbound, upperbound=1.1, maxneighbors=None):
        """As getNeighbors, plus the fp32 similarity of each listed neighbour:
        returns (indices, similarities, counts)."""
        self._queue_neighbors(rowbase, rowlimit, lowerbound, upperbound, maxneighbors, True)
        return self.retrieveAsyncResult()

    def neighborsDevice(self, rowbase, rowlimit, lowerbound, upperbound, pitch, idx, sims, counts):
        """Neighbour search into caller-provided CUDA tensors: idx int32
        [rows, pitch], sims float32 [rows, pitch] or None, counts int32 [rows]."""
        self._check_rows(rowbase, rowlimit)
        self._enter()
        N.check(N.lib().siml_neighbors(self._h, int(rowbase), int(rowlimit), ctypes.c_float(lowerbound),
                                       ctypes.c_float(upperbound), int(pitch), idx.data_ptr(), N.ptr(sims),
                                       counts.data_ptr(), N.SIML_DEVICE), "neighborsDevice")
        self._leave(idx, sims, counts)

    def neighborsRangeDevice(self, rowbase, rowlimit, colbegin, colend, lowerbound, upperbound, pitch, idx, sims,
                             counts):
        """neighborsDevice restricted to query columns [colbegin, colend):
        absolute indices, overflow counted in waves of 128 from colbegin."""
        self._check_rows(rowbase, rowlimit)
        self._enter()
        N.check(N.lib().siml_neighbors_range(self._h, int(rowbase), int(rowlimit), int(colbegin), int(colend),
                                             ctypes.c_float(lowerbound), ctypes.c_float(upperbound), int(pitch),
                                             idx.data_ptr(), N.ptr(sims), counts.data_ptr(), N.SIML_DEVICE),
                "neighborsRangeDevice")
        self._leave(idx, sims, counts)

    def getNeighborsRange(self, rowbase, rowlimit, colbegin, colend, lowerbound, upperbound=1.1,
                          maxneighbors=None):
        """getNeighbors over query columns [colbegin, colend) only."""
        self._queue_neighbors(rowbase, rowlimit, lowerbound, upperbound, maxneighbors, False, (colbegin, colend))
        return self.retrieveAsyncResult()

    def planNeighborBatch(self, jobs, lowerbound, upperbound=1.1, maxneighbors=None, tile_chunks=0, rows_cap=32,
                          merge_rows=0):
        """A reusable plan (siml_gb300.batch.NeighborBatch) of ragged jobs
        (row_begin, row_end, col_begin, col_end[, out_row]).  tile_chunks <= 0
        tunes the plan's shape (or reuses one tuned for the same kind of
        plan); otherwise tile_chunks, rows_cap and merge_rows are used."""
        from .batch import NeighborBatch
        return NeighborBatch(self, jobs, lowerbound, upperbound, maxneighbors, tile_chunks, rows_cap, merge_rows)

    def getNeighborsBatch(self, jobs, lowerbound, upperbound=1.1, maxneighbors=None, with_sims=False):
        """Runs ragged jobs in one batch; returns one getNeighbors-style
        result per job."""
        plan = self.planNeighborBatch(jobs, lowerbound, upperbound, maxneighbors)
        idx, sims, cnt = plan.buffers(with_sims)
        plan.run(idx, sims, cnt)
        return plan.split(idx, sims, cnt)

    def _queue_neighbors(self, rowbase, rowlimit, lowerbound, upperbound, maxneighbors, with_sims, cols=None):
        self._check_rows(rowbase, rowlimit)
        if maxneighbors is None:
            maxneighbors = self.nquery
        pitch = 16 * ((int(maxneighbors) + 15) // 16)
        rows = rowlimit - rowbase
        L = N.lib()
        if cols is None:
            fn = L.siml_neighbors
            args = (self._h, int(rowbase), int(rowlimit), ctypes.c_float(lowerbound), ctypes.c_float(upperbound),
                    pitch)
        else:
            fn = L.siml_neighbors_range
            args = (self._h, int(rowbase), int(rowlimit), int(cols[0]), int(cols[1]), ctypes.c_float(lowerbound),
                    ctypes.c_float(upperbound), pitch)
        if torch is not None:
            dev = self._device()
            idx = torch.empty((rows, max(pitch, 1)), dtype=torch.int32, device=dev)
            sims = torch.empty((rows, max(pitch, 1)), dtype=torch.float32, device=dev) if with_sims else None
            cnt = torch.empty(max(rows, 1), dtype=torch.int32, device=dev)
            self._enter()
            N.check(fn(*args, idx.data_ptr(), N.ptr(sims), cnt.data_ptr(), N.SIML_DEVICE), "getNeighbors")
        else:
            idx = np.empty((rows, max(pitch, 1)), dtype=np.int32)
            sims = np.empty((rows, max(pitch, 1)), dtype=np.float32) if with_sims else None
            cnt = np.empty(max(rows, 1), dtype=np.int32)
            N.check(fn(*args, idx.ctypes.data, N.ptr(sims), cnt.ctypes.data, N.SIML_HOST), "getNeighbors")
        self.last_async_width = maxneighbors
        self._set_pending(("neighbors", idx, sims, cnt, pitch, rows))

    # ----------------------------------------------------------- async glue
    def _set_pending(self, pending):
        """Makes *pending* the one outstanding result (pysiml/GPULingo.py:350,
        400, 460, 512).  A result never retrieved is dropped, as the reference
        drops it, but only once the engine's stream has finished writing its
        buffers: torch's allocators know nothing of the engine's kernels and
        would otherwise hand those buffers out again while a kernel writes."""
        if self._pending is not None:
            N.check(N.lib().siml_sync(self._h), "siml_sync")
        self._pending = pending

    def retrieveAsyncResult(self):
        """Result of the last async call (pysiml/GPULingo.py:538-640)."""
        if self._pending is None:
            raise RuntimeError("Error: tried to call retrieveAsyncResult without a pending asynchronous result")
        kind, *payload = self._pending
        self._pending = None
        N.check(N.lib().siml_sync(self._h), "siml_sync")
        if kind == "matrix":
            out, width = payload[0], payload[1]
            if torch is not None and isinstance(out, torch.Tensor):
                host = (out.cpu() if out.is_cuda else out).numpy()
            else:
                host = out
            return host[:, :width]
        if kind == "neighbors":
            idx, sims, cnt, pitch, rows = payload
            host = lambda a: a.cpu().numpy() if torch is not None and isinstance(a, torch.Tensor) else a
            counts = host(cnt)[:rows].copy()
            ncols = int(min(counts.max(), pitch)) if rows else 0
            mat = host(idx[:, :ncols]) if rows else np.empty((0, 0), np.int32)
            if sims is None:
                return np.ascontiguousarray(mat), counts
            return np.ascontiguousarray(mat), np.ascontiguousarray(host(sims[:, :ncols]) if rows else
                                                                   np.empty((0, 0), np.float32)), counts
        if kind == "ready":
            return payload[0]
        raise RuntimeError("unknown pending result")

    # The reference rebinds retrieveAsyncResult to one of these per call
    # kind; they are public names there, so they are kept for callers that
    # use them directly.
    def retrieveAsyncMatrixResult(self):
        """Matrix result of a pending getTanimotoRow_async, getMultipleRows_async
        or getMultipleHistogrammedRows_async (pysiml/GPULingo.py:536-555)."""
        self._expect_pending("matrix")
        return self.retrieveAsyncResult()

    def retrieveAsyncMatrixVectorResult(self):
        """(indices, counts) of a pending getNeighbors_async
        (pysiml/GPULingo.py:558-583).  Here both forms return the columns up to
        the largest count, as retrieveAsyncResult does."""
        self._expect_pending("neighbors")
        return self.retrieveAsyncResult()

    def retrieveAsyncMatrixVectorResult_trimmed(self):
        """(indices, counts) of a pending getNeighbors_async, trimmed to the
        largest count (pysiml/GPULingo.py:585-622)."""
        self._expect_pending("neighbors")
        return self.retrieveAsyncResult()

    def retrieveAsyncResultBase(self):
        """What retrieveAsyncResult is reset to after a retrieval
        (pysiml/GPULingo.py:624-628): always an error."""
        raise RuntimeError("Error: tried to call retrieveAsyncResult without a pending asynchronous result")

    def _expect_pending(self, kind):
        if self._pending is None:
            self.retrieveAsyncResultBase()
        if self._pending[0] != kind:
            raise RuntimeError("the pending asynchronous result is a %s result, not a %s result"
                               % (self._pending[0], kind))

    def asyncOperationsDone(self):
        """True once all queued work of this object has finished (pysiml/GPULingo.py:642-647)."""
        done = ctypes.c_int(0)
        N.check(N.lib().siml_query_done(self._h, ctypes.byref(done)), "asyncOperationsDone")
        return bool(done.value)

    # -------------------------------------------------------------- extras
    def dbStats(self):
        """Layout statistics of the resident database (dict)."""
        a = (ctypes.c_int64 * 8)()
        N.check(N.lib().siml_db_stats(self._h, a), "siml_db_stats")
        keys = ["nvid", "entry_bytes", "ngroups_total", "nchunks", "max_ng", "n", "ref_max_entries", "qry_max_entries"]
        return dict(zip(keys, [int(x) for x in a]))

    def memInfo(self):
        """(free, total) device memory of this object's GPU in bytes."""
        f, t = ctypes.c_int64(0), ctypes.c_int64(0)
        N.check(N.lib().siml_mem_info(self._h, ctypes.byref(f), ctypes.byref(t)), "siml_mem_info")
        return int(f.value), int(t.value)

    def rowsInfo(self):
        """The full-matrix path of the current sets (dict): scheduled (1 when
        getMultipleRows runs on the scheduled layout), its work items,
        windows and the most steps of one item."""
        a = (ctypes.c_int64 * 4)()
        N.check(N.lib().siml_rows_info(self._h, a), "siml_rows_info")
        return dict(zip(["scheduled", "items", "windows", "max_item_steps"], [int(x) for x in a]))

    def rowsVocab(self):
        """Vocabulary split of the scheduled full-matrix layout (dict): pairs
        in its shared-memory table, rare database entries, most rare entries
        in one ref row, and how the last getMultipleRows launch counted the
        rare pairs (rare_path: 0 none, 1 hash in the table pass, 2 second
        pass, -1 before a launch)."""
        a = (ctypes.c_int64 * 4)()
        N.check(N.lib().siml_rows_vocab(self._h, a), "siml_rows_vocab")
        return dict(zip(["table_pairs", "nrare", "row_max_rare", "rare_path"], [int(x) for x in a]))

    def vocabStats(self):
        """Vocabulary split of the resident database (dict): pairs, common
        pairs (shared-memory table), rare database entries, most rare entries
        in one ref row."""
        a = (ctypes.c_int64 * 4)()
        N.check(N.lib().siml_vocab_stats(self._h, a), "siml_vocab_stats")
        return dict(zip(["nvid", "ncommon", "nrare", "row_max_rare"], [int(x) for x in a]))

    def setRowsWindow(self, window):
        """Sort window (32 = natural order, 64, 128 or 256) of the layout the
        full-matrix calls stream; see SIML_TUNE_ROWS_WINDOW."""
        N.check(N.lib().siml_set_tuning(self._h, N.SIML_TUNE_ROWS_WINDOW, int(window)), "setRowsWindow")

    def setRowsEntries(self, fmt):
        """Entry format of the full-matrix layout (SIML_ENTRIES_AUTO, _U16,
        _U32 or _OFFSETS); see SIML_TUNE_ROWS_ENTRIES."""
        N.check(N.lib().siml_set_tuning(self._h, N.SIML_TUNE_ROWS_ENTRIES, int(fmt)), "setRowsEntries")

    def rowsEntries(self):
        v = ctypes.c_int64()
        N.check(N.lib().siml_get_tuning(self._h, N.SIML_TUNE_ROWS_ENTRIES, ctypes.byref(v)), "rowsEntries")
        return int(v.value)

    def rowsWindow(self):
        v = ctypes.c_int64()
        N.check(N.lib().siml_get_tuning(self._h, N.SIML_TUNE_ROWS_WINDOW, ctypes.byref(v)), "rowsWindow")
        return int(v.value)

    def evaluatedPairs(self, reset=False):
        """Pairs the threshold kernels evaluated since the last reset (chunks
        skipped by the magnitude bound excluded)."""
        v = ctypes.c_uint64()
        N.check(N.lib().siml_eval_pairs(self._h, ctypes.byref(v), 1 if reset else 0), "siml_eval_pairs")
        return int(v.value)

    def launchCount(self):
        """Kernel launches issued by this object so far."""
        return int(N.lib().siml_launch_count(self._h))

    def lastKernelMs(self):
        """Device time of the dominant kernel of the last call (CUDA events)."""
        return float(N.lib().siml_last_kernel_ms(self._h))

