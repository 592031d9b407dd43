"""The multi-GPU path on CPU: two gloo ranks run the bench's replica split
(round-robin row blocks, max-over-ranks timing) over the oracle.  Together
they cover every block once, and the union equals one process's answer."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from oracle import cpulingo as O
    from siml_gb300 import replicas
    import torch.distributed as dist
    assert replicas.init("gloo")
    r, w, _ = replicas.env()
    assert (r, w) == (rank, world)
    q = O.compile_strings([b"CCCCCCOCC(=O)N" + bytes([65 + i % 20]) * (i % 7) for i in range(64)])
    rows_per_block, nblocks, steps = 8, 8, 4
    got = {}
    replicas.barrier()
    for k in range(steps):
        b = replicas.block_of(k, w, r, nblocks)
        got[b] = O.tanimoto_block(q, q, b * rows_per_block, (b + 1) * rows_per_block)
    mx = replicas.max_over_ranks(float(10 + rank))
    objs = [None] * w
    dist.all_gather_object(objs, got)
    if rank == 0:
        merged = {}
        for d in objs:
            for b, m in d.items():
                assert b not in merged, "block %d computed twice" % b
                merged[b] = m
        full = O.tanimoto_block(q, q, 0, 64)
        assert sorted(merged) == list(range(nblocks))
        for b, m in merged.items():
            assert np.array_equal(m, full[b * rows_per_block:(b + 1) * rows_per_block])
        assert mx == 10.0 + world - 1
        assert replicas.jobs_of(10, w, 0) == [0, 2, 4, 6, 8] and replicas.jobs_of(10, w, 1) == [1, 3, 5, 7, 9]
        open(os.path.join(out_dir, "ok"), "w").write("ok")
    replicas.barrier()
    replicas.finish()


def test_two_gloo_ranks_cover_every_block_once(oracle, tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.spawn(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    assert (tmp_path / "ok").exists()


def test_single_rank_needs_no_group():
    from siml_gb300 import replicas
    assert replicas.init("gloo") is False or replicas.env()[1] > 1
    assert replicas.max_over_ranks(3.5) == 3.5
    assert replicas.block_of(5, 1, 0, 4) == 1


def _slab(qry, b, e):
    return tuple(np.ascontiguousarray(np.asarray(a)[b:e]) for a in qry)


@pytest.mark.parametrize("seed,nshards,lo,pitch", [(1, 2, 0.3, 16), (2, 3, 0.15, 32), (3, 5, 0.5, 16),
                                                   (4, 4, 0.0, 48), (5, 2, 0.9, 16)])
def test_shard_merges_equal_one_search(oracle, seed, nshards, lo, pitch):
    """Database slabs searched apart and merged on the host give exactly the
    one-search answer: getNeighbors with the overflow waves, top-k with its
    tie rule, histograms and full-matrix rows."""
    from siml_gb300 import replicas
    rng = np.random.default_rng(seed)
    alpha = np.frombuffer(b"CCCCccNO()=1", np.uint8)
    strs = [bytes(rng.choice(alpha, size=int(rng.integers(6, 40))).astype(np.uint8)) for _ in range(1500)]
    qry = oracle.compile_strings(strs)
    ref = _slab(qry, 0, 24)
    n = qry[0].shape[0]
    bounds = replicas.shard_bounds(n, nshards)
    assert bounds[0][0] == 0 and bounds[-1][1] == n and all(b % 128 == 0 or b == e for b, e in bounds)
    rows = ref[0].shape[0]
    parts = [oracle.neighbors_range_block(ref, qry, 0, rows, b, e, lo, 1.1, pitch + 128) for b, e in bounds]
    mi, ms, mc = replicas.merge_neighbors(parts, bounds, pitch)
    oi, osm, oc = oracle.neighbors_block(ref, qry, 0, rows, lo, 1.1, pitch)
    assert np.array_equal(mc, oc)
    for r in range(rows):
        k = min(int(oc[r]), pitch)
        assert np.array_equal(mi[r, :k], oi[r, :k]), r
        assert np.array_equal(ms[r, :k].view(np.uint32), osm[r, :k].view(np.uint32)), r
    k = 10
    tparts = []
    for b, e in bounds:
        ti, ts = oracle.topk_block(ref, _slab(qry, b, e), 0, rows, k)
        tparts.append((np.where(ti >= 0, ti + b, ti), ts))
    ti, ts = replicas.merge_topk(tparts, k)
    wi, ws = oracle.topk_block(ref, qry, 0, rows, k)
    assert np.array_equal(ti, wi) and np.array_equal(ts.view(np.uint32), ws.view(np.uint32))
    hparts = [oracle.hist101_block(ref, _slab(qry, b, e), 0, rows) for b, e in bounds]
    assert np.array_equal(replicas.merge_hist(hparts), oracle.hist101_block(ref, qry, 0, rows))
    rparts = [oracle.tanimoto_block(ref, _slab(qry, b, e), 0, rows) for b, e in bounds]
    assert np.array_equal(replicas.merge_rows(rparts), oracle.tanimoto_block(ref, qry, 0, rows))


def _shard_rank_main(rank, world, port, out_dir):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from oracle import cpulingo as O
    from siml_gb300 import replicas
    import torch.distributed as dist
    assert replicas.init("gloo")
    r, w, _ = replicas.env()
    qry = O.compile_strings([b"CCCCCCOCC(=O)N" + bytes([65 + i % 20]) * (i % 7) + b"CC(O)" * (i % 3)
                             for i in range(700)])
    ref = tuple(np.ascontiguousarray(np.asarray(a)[:16]) for a in qry)
    bounds = replicas.shard_bounds(qry[0].shape[0], w)
    b, e = bounds[r]
    pitch = 32
    mine = O.neighbors_range_block(ref, qry, 0, 16, b, e, 0.4, 1.1, pitch + 128)
    objs = [None] * w
    dist.all_gather_object(objs, mine)
    if rank == 0:
        mi, ms, mc = replicas.merge_neighbors(objs, bounds, pitch)
        oi, osm, oc = O.neighbors_block(ref, qry, 0, 16, 0.4, 1.1, pitch)
        assert np.array_equal(mc, oc)
        for row in range(16):
            k = min(int(oc[row]), pitch)
            assert np.array_equal(mi[row, :k], oi[row, :k])
        open(os.path.join(out_dir, "ok"), "w").write("ok")
    replicas.barrier()
    replicas.finish()


def test_two_gloo_ranks_search_database_slabs(oracle, tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.spawn(_shard_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    assert (tmp_path / "ok").exists()
