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
