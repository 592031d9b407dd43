"""Request loop over a resident database: continuous batching of similarity
queries on one GPU.

A request carries SMILES strings and asks either for the top-k most similar
database molecules of each string (ties to the lower index) or for every
database molecule with Tanimoto >= a threshold (getNeighbors' rule,
pysiml/kernels.py:393-475).  The reference answers one call at a time
(pysiml/GPULingo.py:467-534); here a batcher thread admits queued requests
into the next batch while earlier batches run:

* admission: a request joins the forming batch while the batch's query rows
  fit one slot region of the ref buffer and its hit buffers fit the device
  memory that is free right now (cudaMemGetInfo plus what torch's cache holds
  unused, less a reserve, capped by the configured budget).  FIFO: the first
  request that does not fit waits for the next batch, and when not even the
  oldest request fits the free memory (another tenant holds it) the batch is
  deferred, not failed, until memory frees up;
* hit buffers are allocated per batch on the engine's stream and released
  once the batch's results are handed out;
* two slot regions alternate, so the next batch is compiled, written and
  queued on the stream while the previous one computes and its results come
  back; a region is reused only after its results have been handed out;
* results are exact and independent of the batch a request lands in (the
  kernels are deterministic and every ordering is total), which the tests
  check alone against in a mix.

The per-request path (`serve_unbatched`) runs the same steps one request at a
time, as a caller of the reference's API would.
"""
from __future__ import annotations

import collections
import ctypes
import gc
import math
import threading
import time

import numpy as np

from . import _native as N

try:
    import torch
except Exception:  # pragma: no cover
    torch = None

TOPK = "topk"
THRESHOLD = "threshold"


class RequestCancelled(RuntimeError):
    """The error of a request withdrawn by LingoServer.cancel before it
    joined a batch."""


class Request:
    """One request: `smiles` (a list of bytes) and the kind of answer.

    After completion `result` holds, per query string, either (indices,
    similarities) of its top-k, or (indices, similarities) of every hit in
    ascending index order; `t_done - arrival` is the latency in seconds."""

    __slots__ = ("rid", "smiles", "kind", "k", "lo", "arrival", "t_admit", "t_done", "result", "error", "done",
                 "rows", "compiled")

    def __init__(self, rid, smiles, kind=TOPK, k=50, lo=0.75, arrival=None):
        if kind not in (TOPK, THRESHOLD):
            raise ValueError("kind must be 'topk' or 'threshold'")
        self.rid = rid
        self.smiles = [s.encode() if isinstance(s, str) else bytes(s) for s in smiles]
        self.kind = kind
        self.k = int(k)
        self.lo = float(lo)
        self.arrival = time.perf_counter() if arrival is None else arrival
        self.t_admit = None
        self.t_done = None
        self.result = None
        self.error = None
        self.done = threading.Event()
        self.rows = len(self.smiles)
        self.compiled = None   # (lingos, counts, lengths, mags) once compiled

    def latency(self):
        return None if self.t_done is None else self.t_done - self.arrival


def compile_into(smiles, L, C, ln, mg, width):
    """Compiles SMILES into the first len(smiles) rows of preallocated
    [*, width] arrays in one pass (ValueError when a molecule has more unique
    LINGOs than width)."""
    n = len(smiles)
    off = np.zeros(n + 1, dtype=np.int64)
    np.cumsum([len(s) for s in smiles], out=off[1:])
    buf = b"".join(smiles) or b"\0"
    lib = N.lib()
    rc = lib.siml_compile_smiles(buf, off.ctypes.data, n, L.ctypes.data, C.ctypes.data, ln.ctypes.data,
                                 mg.ctypes.data, width)
    if rc != N.SIML_OK:
        msg = N.last_error()
        w = lib.siml_compile_width(buf, off.ctypes.data, n)
        if w > width:
            raise ValueError("a query molecule has %d unique LINGOs, more than the server's width %d" % (w, width))
        raise ValueError(msg or "siml_compile_smiles failed")


class _Region:
    """One slot region: ref rows [base, base + max_rows), its pinned host
    staging and result buffers, and the device hit buffers of the batch it
    holds (allocated when the batch is admitted)."""

    def __init__(self, base, cfg, dev):
        self.base = base
        pin = lambda shape, dt: torch.empty(shape, dtype=dt).pin_memory()
        R, W = cfg.max_rows, cfg.width
        self.hL, self.hC = pin((R, W), torch.int32), pin((R, W), torch.int32)
        self.hlen, self.hmag = pin((R,), torch.int32), pin((R,), torch.int32)
        self.k_idx = self.k_sims = self.n_idx = self.n_sims = self.n_cnt = None
        self.o_kidx, self.o_ksims = pin((R, cfg.kmax), torch.int32), pin((R, cfg.kmax), torch.float32)
        self.o_nidx, self.o_nsims = pin((R, cfg.pitch), torch.int32), pin((R, cfg.pitch), torch.float32)
        self.o_ncnt = pin((R,), torch.int32)
        self.free = threading.Event()
        self.free.set()


class ServerConfig:
    """max_rows: query rows a batch may hold (one slot region); soft_rows: the
    batch size while the queue is short (smaller batches, shorter waits);
    backlog_rows: queued rows past which batches grow to max_rows for
    throughput; width: LINGO columns per query row; kmax: largest k a top-k
    request may ask; pitch: hits per row a threshold batch keeps before an
    overflowing row is re-run alone; hit_budget: device bytes of hit buffers
    one batch may claim; mem_reserve: device bytes left free for others when
    admitting; mem_probe: callable returning the device bytes free for hit
    buffers (default: cudaMemGetInfo plus torch's unused cache); mem_poll_s:
    how often a deferred batch probes the memory again; gc_freeze: at start,
    move every object alive into the collector's permanent generation
    (gc.freeze), so that a full collection while serving scans only objects
    made since.  A full collection holds the interpreter lock, which the
    batcher and completer threads need: over a process with a large heap
    (torch and its modules, earlier results) one took 35-80 ms and every
    request queued behind it."""

    def __init__(self, max_rows=1024, width=256, kmax=64, pitch=256, hit_budget=None, lo=0.75, soft_rows=None,
                 backlog_rows=None, mem_reserve=256 << 20, mem_probe=None, mem_poll_s=0.002, gc_freeze=True):
        self.max_rows = int(max_rows)
        self.soft_rows = int(soft_rows) if soft_rows else self.max_rows
        self.backlog_rows = int(backlog_rows) if backlog_rows else 8 * self.max_rows
        self.width = int(width)
        self.kmax = int(kmax)
        self.pitch = int(pitch)
        self.lo = float(lo)
        self.hit_budget = int(hit_budget) if hit_budget else self.max_rows * max(self.pitch * 8 + 4, self.kmax * 8)
        self.mem_reserve = int(mem_reserve)
        self.mem_probe = mem_probe
        self.mem_poll_s = float(mem_poll_s)
        self.gc_freeze = bool(gc_freeze)


def _hit_bytes(req, cfg):
    """Device bytes of a request's hit buffers: index, similarity (and count)
    per threshold row at the batch pitch; the top-k lists at the batch's k,
    bounded by kmax."""
    return req.rows * (cfg.pitch * 8 + 4 if req.kind == THRESHOLD else cfg.kmax * 8)


def admit(queue, cfg, avail_bytes, row_limit):
    """The requests at the head of `queue` (oldest first) that form the next
    batch: they are taken while their query rows fit row_limit and their hit
    buffers fit min(cfg.hit_budget, avail_bytes).  An empty list means the
    oldest request does not fit the free memory and the batch waits."""
    budget = min(cfg.hit_budget, avail_bytes)
    batch, rows, hits = [], 0, 0
    for r in queue:
        need = _hit_bytes(r, cfg)
        if hits + need > budget:
            break
        if batch and rows + r.rows > row_limit:
            break
        batch.append(r)
        rows += r.rows
        hits += need
    return batch


class LingoServer:
    """Continuous-batching request loop on a GPULingo object whose query set
    (the database) is already set.  The object's ref set becomes the server's
    slot buffer."""

    def __init__(self, gl, cfg=None):
        if torch is None:
            raise RuntimeError("the request loop needs torch for pinned buffers and streams")
        self.gl = gl
        self.cfg = cfg or ServerConfig()
        self.dev = gl._device()
        R, W = self.cfg.max_rows, self.cfg.width
        zeros = np.zeros((2 * R, W), dtype=np.int32)
        gl.set_refsmiles(zeros, zeros, np.zeros(2 * R, dtype=np.int32))
        N.check(N.lib().siml_set_tuning(gl._h, N.SIML_TUNE_ROW_STRIDE, 4 * W), "siml_set_tuning")
        self.regions = [_Region(0, self.cfg, self.dev), _Region(R, self.cfg, self.dev)]
        self.queue = collections.deque()
        self.cv = threading.Condition()
        self.inflight = collections.deque()
        self.icv = threading.Condition()
        self.stop_flag = False
        self.batcher_done = False
        self.elock = threading.Lock()   # one host thread at a time on the engine handle
        self.batches = 0
        self.deferrals = 0      # batch formations put off for lack of free device memory
        self.pairs = 0
        self.batch_rows = []
        self.gpu_ms = 0.0       # device time of the batches (write, search, copy back)
        self.launch_s = 0.0     # host time compiling, writing and queueing batches
        self.deliver_s = 0.0    # host time handing results to requests
        self.threads = []

    # ------------------------------------------------------------- control
    def start(self):
        if self.cfg.gc_freeze:
            gc.freeze()
        self.stop_flag = False
        self.batcher_done = False
        self.threads = [threading.Thread(target=self._batcher, daemon=True),
                        threading.Thread(target=self._completer, daemon=True)]
        for t in self.threads:
            t.start()
        return self

    def stop(self):
        """Serves what is queued, then ends both threads."""
        with self.cv:
            self.stop_flag = True
            self.cv.notify_all()
        if self.threads:
            self.threads[0].join()
        with self.icv:
            self.batcher_done = True
            self.icv.notify_all()
        if self.threads:
            self.threads[1].join()
        self.threads = []

    def submit(self, req):
        if req.rows > self.cfg.max_rows:
            raise ValueError("request of %d queries exceeds the batch size %d" % (req.rows, self.cfg.max_rows))
        if _hit_bytes(req, self.cfg) > self.cfg.hit_budget:
            raise ValueError("request of %d queries needs more hit memory than the batch budget" % req.rows)
        if req.kind == TOPK and not 1 <= req.k <= self.cfg.kmax:
            raise ValueError("k must be in [1, %d]" % self.cfg.kmax)
        if req.kind == THRESHOLD and req.lo != self.cfg.lo:
            raise ValueError("threshold requests use the server's bound %g" % self.cfg.lo)
        # compiled in the caller's thread: a malformed request is refused here
        # and never reaches a batch, and the batcher only copies rows
        self._compile(req)
        with self.cv:
            self.queue.append(req)
            self.cv.notify()
        return req

    def cancel(self, req):
        """Withdraws a request that is still queued: it completes at once with
        a RequestCancelled error and never joins a batch.  Returns False when
        it has already joined one (its answer still arrives) or is not queued
        here."""
        with self.cv:
            try:
                self.queue.remove(req)
            except ValueError:
                return False
        req.compiled = None
        req.error = RequestCancelled("request %r was cancelled before it joined a batch" % (req.rid,))
        req.t_done = time.perf_counter()
        req.done.set()
        return True

    def _compile(self, req):
        if req.compiled is None:
            W = self.cfg.width
            arrays = (np.empty((req.rows, W), np.int32), np.empty((req.rows, W), np.int32),
                      np.empty(req.rows, np.int32), np.empty(req.rows, np.int32))
            compile_into(req.smiles, *arrays, W)
            req.compiled = arrays

    # ------------------------------------------------------------- batcher
    def free_device_bytes(self):
        """Device bytes hit buffers may take now: the probe's reading (by
        default cudaMemGetInfo's free bytes plus what torch's cache holds
        unused) less the reserve."""
        cfg = self.cfg
        if cfg.mem_probe is not None:
            free = int(cfg.mem_probe())
        else:
            free, _ = self.gl.memInfo()
            free += torch.cuda.memory_reserved(self.dev) - torch.cuda.memory_allocated(self.dev)
        return free - cfg.mem_reserve

    def _take_batch(self):
        cfg = self.cfg
        with self.cv:
            while True:
                while not self.queue and not self.stop_flag:
                    self.cv.wait()
                if self.stop_flag and not self.queue:
                    return None
                queued = sum(r.rows for r in self.queue)
                limit = cfg.max_rows if queued > cfg.backlog_rows else cfg.soft_rows
                batch = admit(self.queue, cfg, self.free_device_bytes(), limit)
                if batch:
                    for _ in batch:
                        self.queue.popleft()
                    return batch
                # the oldest request's hit buffers do not fit the free device
                # memory: the batch waits for memory, the requests stay queued
                self.deferrals += 1
                self.cv.wait(timeout=cfg.mem_poll_s)

    def _batcher(self):
        seq = 0
        while True:
            region = self.regions[seq % 2]
            region.free.wait()
            batch = self._take_batch()
            if batch is None:
                return
            region.free.clear()
            try:
                t = time.perf_counter()
                item = self._launch(batch, region)
                self.launch_s += time.perf_counter() - t
            except Exception as e:  # report the failure on every request of the batch
                for r in batch:
                    r.error = e
                    r.t_done = time.perf_counter()
                    r.done.set()
                region.free.set()
                continue
            with self.icv:
                self.inflight.append(item)
                self.icv.notify()
            seq += 1

    def _launch(self, batch, region):
        gl, cfg = self.gl, self.cfg
        now = time.perf_counter()
        thr = [r for r in batch if r.kind == THRESHOLD]
        tk = [r for r in batch if r.kind == TOPK]
        nt = sum(r.rows for r in thr)
        nk = sum(r.rows for r in tk)
        kmax = max([r.k for r in tk], default=1)
        L, C = region.hL.numpy(), region.hC.numpy()
        ln, mg = region.hlen.numpy(), region.hmag.numpy()
        row = 0
        for r in thr + tk:
            r.t_admit = now
            self._compile(r)
            cL, cC, cln, cmg = r.compiled
            L[row:row + r.rows] = cL
            C[row:row + r.rows] = cC
            ln[row:row + r.rows] = cln
            mg[row:row + r.rows] = cmg
            r.compiled = None
            row += r.rows
        with self.elock:
            # the batch's hit buffers, on the engine's stream (released after
            # delivery); admitted against the free memory just read
            with torch.cuda.stream(gl.stream):
                if nt:
                    region.n_idx = torch.empty((nt, cfg.pitch), dtype=torch.int32, device=self.dev)
                    region.n_sims = torch.empty((nt, cfg.pitch), dtype=torch.float32, device=self.dev)
                    region.n_cnt = torch.empty((nt,), dtype=torch.int32, device=self.dev)
                if nk:
                    region.k_idx = torch.empty((nk, kmax), dtype=torch.int32, device=self.dev)
                    region.k_sims = torch.empty((nk, kmax), dtype=torch.float32, device=self.dev)
            return self._queue(batch, thr, tk, nt, nk, kmax, region)

    def _queue(self, batch, thr, tk, nt, nk, kmax, region):
        gl, cfg = self.gl, self.cfg
        L, C = region.hL.numpy(), region.hC.numpy()
        ln, mg = region.hlen.numpy(), region.hmag.numpy()
        lib = N.lib()
        n = nt + nk
        N.check(lib.siml_write_ref_rows(gl._h, region.base, L.ctypes.data, C.ctypes.data, ln.ctypes.data,
                                        mg.ctypes.data, n, cfg.width, cfg.width), "siml_write_ref_rows")
        st = gl.stream
        b = region.base
        ev0 = torch.cuda.Event(enable_timing=True)
        ev0.record(st)
        if nt:
            N.check(lib.siml_neighbors(gl._h, b, b + nt, ctypes.c_float(cfg.lo), ctypes.c_float(1.1), cfg.pitch,
                                       region.n_idx.data_ptr(), region.n_sims.data_ptr(), region.n_cnt.data_ptr(),
                                       N.SIML_DEVICE), "siml_neighbors")
        if nk:
            N.check(lib.siml_topk(gl._h, b + nt, b + nt + nk, kmax, region.k_idx.data_ptr(), region.k_sims.data_ptr(),
                                  N.SIML_DEVICE), "siml_topk")
        with torch.cuda.stream(st):
            if nt:
                region.o_ncnt[:nt].copy_(region.n_cnt[:nt], non_blocking=True)
                region.o_nidx[:nt].copy_(region.n_idx[:nt], non_blocking=True)
                region.o_nsims[:nt].copy_(region.n_sims[:nt], non_blocking=True)
            if nk:
                m = nk * kmax
                region.o_kidx.view(-1)[:m].copy_(region.k_idx.view(-1), non_blocking=True)
                region.o_ksims.view(-1)[:m].copy_(region.k_sims.view(-1), non_blocking=True)
            ev = torch.cuda.Event(enable_timing=True)
            ev.record(st)
        self.batches += 1
        self.pairs += n * gl.nquery
        self.batch_rows.append(n)
        return (batch, thr, tk, nt, nk, kmax, region, (ev0, ev))

    # ----------------------------------------------------------- completer
    def _completer(self):
        while True:
            with self.icv:
                while not self.inflight and not self.batcher_done:
                    self.icv.wait()
                if not self.inflight:
                    return
                item = self.inflight.popleft()
            batch, thr, tk, nt, nk, kmax, region, (ev0, ev) = item
            try:
                ev.synchronize()
                with self.elock:   # a bounded top-k wait that expired in this batch
                    N.check(N.lib().siml_async_status(self.gl._h), "siml_async_status")
                self.gpu_ms += ev0.elapsed_time(ev)
                t = time.perf_counter()
                self._deliver(thr, tk, nt, nk, kmax, region)
                self.deliver_s += time.perf_counter() - t
            except Exception as e:
                for r in batch:
                    r.error = e
            t = time.perf_counter()
            region.k_idx = region.k_sims = region.n_idx = region.n_sims = region.n_cnt = None
            region.free.set()
            for r in batch:
                r.t_done = t
                r.done.set()

    def _deliver(self, thr, tk, nt, nk, kmax, region):
        cfg = self.cfg
        cnt = region.o_ncnt.numpy()
        nidx, nsims = region.o_nidx.numpy(), region.o_nsims.numpy()
        # one block copy per request out of the region's pinned buffers (they
        # are reused by a later batch); rows are views into it
        row = 0
        for r in thr:
            c = cnt[row:row + r.rows]
            w = int(min(int(c.max()), cfg.pitch)) if r.rows else 0
            bi, bs = nidx[row:row + r.rows, :w].copy(), nsims[row:row + r.rows, :w].copy()
            res = []
            for q in range(r.rows):
                cq = int(c[q])
                res.append(self._rerun_row(region.base + row + q, cq) if cq > cfg.pitch else (bi[q, :cq], bs[q, :cq]))
            r.result = res
            row += r.rows
        kid = region.o_kidx.numpy().reshape(-1)[:nk * kmax].reshape(nk, kmax) if nk else None
        ksm = region.o_ksims.numpy().reshape(-1)[:nk * kmax].reshape(nk, kmax) if nk else None
        row = 0
        for r in tk:
            bi, bs = kid[row:row + r.rows, :r.k].copy(), ksm[row:row + r.rows, :r.k].copy()
            r.result = list(zip(bi, bs))
            row += r.rows

    def _rerun_row(self, ref_row, count):
        """A threshold row with more hits than the batch pitch, searched
        again alone with room for all of them (the region is still held)."""
        pitch = 16 * ((count + 15) // 16)
        idx = np.empty((1, pitch), dtype=np.int32)
        sims = np.empty((1, pitch), dtype=np.float32)
        cnt = np.empty(1, dtype=np.int32)
        with self.elock:
            N.check(N.lib().siml_neighbors(self.gl._h, ref_row, ref_row + 1, ctypes.c_float(self.cfg.lo),
                                           ctypes.c_float(1.1), pitch, idx.ctypes.data, sims.ctypes.data,
                                           cnt.ctypes.data, N.SIML_HOST), "siml_neighbors")
        c = int(cnt[0])
        return idx[0, :c].copy(), sims[0, :c].copy()


def serve_unbatched(server, req):
    """The per-request path: one request written, searched and read back on
    its own, synchronously (uses the server's first region; do not mix with
    a running batch loop)."""
    region = server.regions[0]
    req.t_admit = time.perf_counter()
    thr = [req] if req.kind == THRESHOLD else []
    tk = [req] if req.kind == TOPK else []
    batch = server._launch([req], region)
    _, _, _, nt, nk, kmax, _, (_, ev) = batch
    ev.synchronize()
    N.check(N.lib().siml_async_status(server.gl._h), "siml_async_status")
    server._deliver(thr, tk, nt, nk, kmax, region)
    region.k_idx = region.k_sims = region.n_idx = region.n_sims = region.n_cnt = None
    req.t_done = time.perf_counter()
    req.done.set()
    return req


def percentiles(values, ps=(50, 95, 99)):
    if not values:
        return {("p%d" % p): None for p in ps}
    v = np.sort(np.asarray(values, dtype=np.float64))
    out = {}
    for p in ps:
        i = min(len(v) - 1, max(0, int(math.ceil(p / 100.0 * len(v))) - 1))
        out["p%d" % p] = float(v[i])
    return out
