"""Failure handling on the GPU without a GPU fault: device allocations refused
on the host (siml_debug_fail_alloc, the out-of-memory a full GPU would
report) at every allocation of set-up, layout build and a first call.  Each
refusal surfaces as SimlError(SIML_ERR_NOMEM); the same engine then
completes the work, bit-exact against the oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_refused_allocations_leave_the_engine_usable(native, oracle, set4096):
    from siml_gb300 import GPULingo, _native as N
    ref = tuple(a[:96] for a in set4096)
    want = oracle.tanimoto_block(ref, set4096, 0, 96)
    L = N.lib()
    failed_at = []
    try:
        for nth in range(1, 40):
            gl = GPULingo(0)
            N.check(L.siml_debug_fail_alloc(nth))
            try:
                gl.set_qsmiles(*set4096)
                gl.set_refsmiles(*ref)
                got = gl.getMultipleRows(0, 96)
                ti, ts = gl.getTopK(0, 96, 5)
            except N.SimlError as e:
                assert e.code == N.SIML_ERR_NOMEM and "siml_debug_fail_alloc" in str(e)
                failed_at.append(nth)
            N.check(L.siml_debug_fail_alloc(0))
            # the same engine, set up again where the refusal interrupted it
            gl.set_qsmiles(*set4096)
            gl.set_refsmiles(*ref)
            assert np.array_equal(gl.getMultipleRows(0, 96), want), nth
            ti, ts = gl.getTopK(0, 96, 5)
            oi, os_ = oracle.topk_block(ref, set4096, 0, 96, 5)
            assert np.array_equal(ti, oi) and np.array_equal(ts.view(np.uint32), os_.view(np.uint32)), nth
    finally:
        L.siml_debug_fail_alloc(0)
    assert len(failed_at) >= 10   # set-up, vocabulary, row lists and both layouts


def test_damaged_row_lists_are_reported_not_used(native, oracle, set4096):
    """A ref row's entry list damaged after it was built (a vid outside the
    database vocabulary, written with siml_debug_set_row_vid) is never used
    as a table index: the kernels skip the entry and the call reports
    SIML_ERR_STATE; a batch plan refuses the row when it is made, and a plan
    made before the damage reports it from the run's synchronization.  The
    same engine then gives the oracle's results once the ref set is loaded
    again.  Nothing faults on the GPU."""
    torch = pytest.importorskip("torch")
    from siml_gb300 import GPULingo, _native as N
    ref = tuple(a[:64] for a in set4096)
    want = oracle.tanimoto_block(ref, set4096, 0, 64)
    L = N.lib()
    gl = GPULingo(0)
    gl.set_qsmiles(*set4096)
    gl.set_refsmiles(*ref)
    assert np.array_equal(gl.getMultipleRows(0, 64), want)
    nvid = gl.vocabStats()["nvid"]
    assert gl.vocabStats()["ncommon"] == nvid   # no rare-vid hash: the entry cannot be held
    plan = gl.planNeighborBatch([(0, 10, 0, 4096)], 0.3, 1.1, 64)
    N.check(L.siml_debug_set_row_vid(gl._h, 5, 0, nvid + 7))
    # a host-result call and a queued call each report it
    # (SIML_ERR_STATE surfaces as the reference's RuntimeError)
    with pytest.raises(RuntimeError, match="rare-vid hash"):
        gl.getMultipleRows(0, 64)
    with pytest.raises(RuntimeError, match="rare-vid hash"):
        gl.getNeighborsWithSimilarities(0, 64, 0.3, 1.1, 64)
    # batches: refused at plan creation; a plan made before reports at sync
    with pytest.raises(RuntimeError, match="vocabulary"):
        gl.planNeighborBatch([(0, 10, 0, 4096)], 0.3, 1.1, 64)
    idx, sims, cnt = plan.buffers(with_sims=True)
    plan.run(idx, sims, cnt)
    torch.cuda.synchronize()
    assert L.siml_sync(gl._h) == N.SIML_ERR_STATE
    assert L.siml_sync(gl._h) == N.SIML_OK   # reported once
    # loading the ref set again rebuilds the lists
    gl.set_refsmiles(*ref)
    assert np.array_equal(gl.getMultipleRows(0, 64), want)
    gi, gs, gc = gl.getNeighborsWithSimilarities(0, 64, 0.3, 1.1, 64)
    oi, os_, oc = oracle.neighbors_block(ref, set4096, 0, 64, 0.3, 1.1, 64)
    assert np.array_equal(gc, oc)
