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
