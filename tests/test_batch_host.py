"""Host-side logic of the batched neighbour path (no GPU): job lists and the
oracle's column-range restatement."""
import numpy as np
import pytest


def test_job_array_assigns_consecutive_rows():
    from siml_gb300.batch import job_array
    a = job_array([(0, 4, 0, 10), (10, 10, 3, 7), (7, 9, 1, 2)])
    assert a.dtype == np.int64 and a.shape == (3, 5)
    assert a[:, 4].tolist() == [0, 4, 4]
    b = job_array([(0, 4, 0, 10, 20), (5, 6, 0, 1)])
    assert b[:, 4].tolist() == [20, 24]
    assert job_array([]).shape == (0, 5)
    with pytest.raises(ValueError):
        job_array([(1, 2, 3)])


def test_oracle_range_equals_full_search_on_whole_range(oracle, set4096):
    """The column-range restatement over [0, n) is getNeighbors itself, and a
    range's counts equal a search of that slice of the query set."""
    full = oracle.neighbors_block(set4096, set4096, 0, 64, 0.06, 1.1, 48)
    rng = oracle.neighbors_range_block(set4096, set4096, 0, 64, 0, 4096, 0.06, 1.1, 48)
    for a, b in zip(full, rng):
        assert np.array_equal(a, b, equal_nan=True)
    idx, sims, cnt = oracle.neighbors_range_block(set4096, set4096, 0, 64, 1000, 3000, 0.06, 1.1, 48)
    for r in range(64):
        k = min(int(cnt[r]), 48)
        assert np.all((idx[r, :k] >= 1000) & (idx[r, :k] < 3000))
        assert np.all(np.diff(idx[r, :k]) > 0)
