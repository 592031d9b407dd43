"""Batched ragged neighbour jobs (include/siml_gb300.h, siml_batch_*).

A job is ``(row_begin, row_end, col_begin, col_end)``: ref rows against a
range of the resident query set, searched with getNeighbors' rule
(pysiml/kernels.py:393-475).  The reference runs one ``getNeighbors`` call
per job (pysiml/GPULingo.py:467-513); a :class:`NeighborBatch` plans all jobs
once and runs them as one persistent launch, which can be captured in a CUDA
graph and replayed.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native as N

try:
    import torch
except Exception:  # pragma: no cover
    torch = None


def job_array(jobs):
    """int64 [njobs, 5] {row_begin, row_end, col_begin, col_end, out_row}.
    Jobs given with four fields get consecutive output rows."""
    rows = []
    nxt = 0
    for j in jobs:
        j = [int(x) for x in j]
        if len(j) == 4:
            j = j + [nxt]
        elif len(j) != 5:
            raise ValueError("a job is (row_begin, row_end, col_begin, col_end[, out_row])")
        nxt = max(nxt, j[4] + max(0, j[1] - j[0]))
        rows.append(j)
    return np.ascontiguousarray(np.array(rows, dtype=np.int64).reshape(-1, 5))


class NeighborBatch:
    """A plan of neighbour jobs on one GPULingo object.

    ``pitch`` is 16*ceil(maxneighbors/16) as getNeighbors computes it.  The
    plan stays valid until the object's ref or query set is replaced."""

    def __init__(self, gl, jobs, lowerbound, upperbound=1.1, maxneighbors=None, tile_chunks=0, rows_cap=32,
                 merge_rows=0):
        """tile_chunks <= 0: the plan's shape (tile, row cap, merge cut-off)
        is tuned, or taken from an earlier plan of the same kind; otherwise
        the given shape is used as is."""
        self._gl = gl
        self._b = ctypes.c_void_p()
        self.jobs = job_array(jobs)
        if maxneighbors is None:
            maxneighbors = gl.nquery
        self.maxneighbors = int(maxneighbors)
        self.pitch = 16 * ((self.maxneighbors + 15) // 16)
        self.lowerbound = float(lowerbound)
        self.upperbound = float(upperbound)
        gl._check_rows(0, 0)
        N.check(N.lib().siml_batch_create_shaped(gl._h, self.jobs.shape[0], self.jobs.ctypes.data,
                                                 ctypes.c_float(lowerbound), ctypes.c_float(upperbound), self.pitch,
                                                 int(tile_chunks), int(rows_cap), int(merge_rows),
                                                 ctypes.byref(self._b)), "siml_batch_create")
        r, n, t, sb, ub = (ctypes.c_int64() for _ in range(5))
        N.check(N.lib().siml_batch_info(self._b, ctypes.byref(r), ctypes.byref(n), ctypes.byref(t),
                                        ctypes.byref(sb), ctypes.byref(ub)), "siml_batch_info")
        self.rows_out, self.nitems, self.tile_chunks = int(r.value), int(n.value), int(t.value)
        sh = (ctypes.c_int64 * 4)()
        N.check(N.lib().siml_batch_shape(self._b, sh), "siml_batch_shape")
        self.rows_cap, self.merge_rows, self.shape_from_cache = int(sh[1]), int(sh[2]), bool(sh[3])
        self.stream_bytes = int(sb.value)   # database bytes one run streams (every work item)
        self.unique_bytes = int(ub.value)   # every job's database range once
        self.pairs = int(sum(max(0, j[1] - j[0]) * max(0, j[3] - j[2]) for j in self.jobs.tolist()))

    def __del__(self):
        b = getattr(self, "_b", None)
        if b is not None and b.value:
            try:
                N.lib().siml_batch_destroy(b)
            except Exception:
                pass
            self._b = None

    def buffers(self, with_sims=False):
        """Fresh device outputs (idx [rows_out, pitch], sims or None, counts [rows_out])."""
        dev = self._gl._device()
        idx = torch.empty((max(self.rows_out, 1), max(self.pitch, 1)), dtype=torch.int32, device=dev)
        sims = torch.empty_like(idx, dtype=torch.float32) if with_sims else None
        cnt = torch.empty(max(self.rows_out, 1), dtype=torch.int32, device=dev)
        return idx, sims, cnt

    def run(self, idx, sims, counts, stream=None):
        """Queues the batch.  With ``stream`` (a torch stream, e.g. the one a
        CUDA graph is being captured on) the work goes on it directly;
        otherwise on the object's stream, ordered after torch's current stream."""
        L = N.lib()
        if stream is not None:
            N.check(L.siml_batch_run(self._b, idx.data_ptr(), N.ptr(sims), counts.data_ptr(),
                                     N.stream_arg(stream)), "siml_batch_run")
            return
        gl = self._gl
        gl._enter()
        N.check(L.siml_batch_run(self._b, idx.data_ptr(), N.ptr(sims), counts.data_ptr(), None), "siml_batch_run")
        gl._leave(idx, sims, counts)

    def split(self, idx, sims, counts):
        """Per-job host results in getNeighbors' form: a list of
        (matrix [rows, min(max count, pitch)], counts [rows]) — with the
        similarities as a middle element when ``sims`` is given."""
        torch.cuda.current_stream(self._gl._device()).synchronize()
        # a work item outside the plan's extents is skipped by the kernel and
        # reported here
        N.check(N.lib().siml_async_status(self._gl._h), "siml_batch_run")
        hi = idx.cpu().numpy()
        hs = sims.cpu().numpy() if sims is not None else None
        hc = counts.cpu().numpy()
        out = []
        for rb, re, cb, ce, o in self.jobs.tolist():
            rows = max(0, re - rb)
            c = hc[o:o + rows].copy()
            w = int(min(c.max(), self.pitch)) if rows else 0
            m = np.ascontiguousarray(hi[o:o + rows, :w])
            if hs is None:
                out.append((m, c))
            else:
                out.append((m, np.ascontiguousarray(hs[o:o + rows, :w]), c))
        return out
