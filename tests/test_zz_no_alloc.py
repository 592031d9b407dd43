"""siml_topk_noalloc, the top-k entry point for callers that cannot allocate
device memory on the request path (it takes all scratch from the library's
static 16 MiB device array), checked through the C ABI against siml_topk and
the oracle on two calls in a row.  Collected last on purpose: it only adds to
what the other tests cover."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _tensors(rows, k):
    torch = pytest.importorskip("torch")
    return (torch.empty((rows, k), dtype=torch.int32, device="cuda"),
            torch.empty((rows, k), dtype=torch.float32, device="cuda"))


def _engine(db):
    from siml_gb300 import GPULingo
    gl = GPULingo(0)
    gl.set_refsmiles(*db)
    gl.set_qsmiles(*db)
    return gl


def test_topk_noalloc_needs_the_sorted_layout(native):
    """On a fresh engine, and after calls that build only the full-matrix
    layout (dbStats, getMultipleRows), the call refuses with SIML_ERR_STATE
    and writes nothing."""
    import torch
    from siml_gb300 import _native as N
    from siml_gb300 import synthetic as S
    db = S.smiles_set(S.SEED_ALLPAIRS, S.UNIFORM_20_90, 4096)
    gl = _engine(db)
    L = N.lib()
    i0, s0 = _tensors(8, 10)
    i0.fill_(-7)
    torch.cuda.synchronize()
    assert L.siml_topk_noalloc(gl._h, 0, 8, 10, i0.data_ptr(), s0.data_ptr()) == N.SIML_ERR_STATE, N.last_error()
    gl.dbStats()
    gl.getMultipleRows(0, 8)
    assert L.siml_topk_noalloc(gl._h, 0, 8, 10, i0.data_ptr(), s0.data_ptr()) == N.SIML_ERR_STATE, N.last_error()
    assert "window-sorted" in N.last_error()
    assert bool((i0 == -7).all())


def test_topk_noalloc_matches_topk_and_the_oracle(native, oracle):
    import torch
    from siml_gb300 import _native as N
    from siml_gb300 import synthetic as S
    db = S.smiles_set(S.SEED_ALLPAIRS, S.UNIFORM_20_90, 4096)
    gl = _engine(db)
    L = N.lib()
    h = gl._h
    gl.vocabStats()   # builds the window-sorted layout
    # heap path (k <= 256) and the per-row scan (k > 256, no scratch)
    for rb, rl, k in [(0, 96, 50), (1000, 1077, 100), (300, 340, 300)]:
        want_i, want_s = _tensors(rl - rb, k)
        N.check(L.siml_topk(h, rb, rl, k, want_i.data_ptr(), want_s.data_ptr(), N.SIML_DEVICE))
        N.check(L.siml_sync(h))
        oi, os_ = oracle.topk_block(db, db, rb, rl, k)
        for _ in range(2):  # two calls in a row share the static scratch
            got_i, got_s = _tensors(rl - rb, k)
            got_i.fill_(-7)
            got_s.fill_(-7.0)
            torch.cuda.synchronize()
            N.check(L.siml_topk_noalloc(h, rb, rl, k, got_i.data_ptr(), got_s.data_ptr()))
            assert torch.equal(got_i, want_i)
            assert torch.equal(got_s.view(torch.int32), want_s.view(torch.int32))
            assert np.array_equal(got_i.cpu().numpy(), oi)
            assert np.array_equal(got_s.cpu().numpy().view(np.uint32), os_.view(np.uint32))


def test_topk_noalloc_refuses_oversized_requests(native):
    from siml_gb300 import _native as N
    from siml_gb300 import synthetic as S
    db = S.smiles_set(S.SEED_ALLPAIRS, S.UNIFORM_20_90, 4096)
    ref = tuple(np.concatenate([a, a, a]) for a in db)   # 12,288 rows
    from siml_gb300 import GPULingo
    gl = GPULingo(0)
    gl.set_refsmiles(*ref)
    gl.set_qsmiles(*db)
    gl.vocabStats()
    # 12,288 rows x k 256 x 8 bytes of partial heaps alone exceed 16 MiB
    i0, s0 = _tensors(12288, 256)
    rc = N.lib().siml_topk_noalloc(gl._h, 0, 12288, 256, i0.data_ptr(), s0.data_ptr())
    assert rc == N.SIML_ERR_INVALID
    assert "static scratch" in N.last_error()
