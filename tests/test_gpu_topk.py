"""GPU per-row top-k against the oracle: the k best similarities of each
row, best first, ties to the lower index, -1 padding past the query set."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _engine(ref, qry):
    from siml_gb300 import GPULingo
    gl = GPULingo(0)
    gl.set_refsmiles(*ref)
    gl.set_qsmiles(*qry)
    return gl


def _check(gl, oracle, ref, qry, rb, rl, k):
    idx, sims = gl.getTopK(rb, rl, k)
    oi, os_ = oracle.topk_block(ref, qry, rb, rl, k)
    assert np.array_equal(idx, oi), k
    assert np.array_equal(sims.view(np.uint32), os_.view(np.uint32)), k


@pytest.mark.parametrize("k", [1, 5, 50, 100, 256])
def test_topk_synthetic(native, oracle, set4096, k):
    gl = _engine(set4096, set4096)
    _check(gl, oracle, set4096, set4096, 0, 96, k)
    _check(gl, oracle, set4096, set4096, 1000, 1031, k)


def test_topk_golden_ties_and_padding(native, oracle, golden):
    """The golden set has repeated and empty molecules (ties, zeros)."""
    q = (golden["lingos"], golden["counts"], golden["lengths"], golden["mags"])
    gl = _engine(q, q)
    n = q[0].shape[0]
    for k in (3, 40, 128):
        _check(gl, oracle, q, q, 0, n, k)
    small = tuple(a[:20] for a in q)
    g2 = _engine(q, small)
    _check(g2, oracle, q, small, 0, 50, 32)   # k > 20 queries: padded


def test_topk_fallback_large_k(native, oracle, set4096):
    gl = _engine(set4096, set4096)
    _check(gl, oracle, set4096, set4096, 0, 8, 600)
