"""Host-side rules of the GPULingo wrapper (no GPU): the one outstanding
async result (pysiml/GPULingo.py:350, 400, 460, 512, 553) and when the
engine's stream is waited for before a result's buffers are released."""
import ctypes

import pytest

HANDLE = ctypes.c_void_p(0)


class _FakeLib:
    def __init__(self, rc=0):
        self.calls = []
        self.rc = rc

    def siml_sync(self, h):
        self.calls.append(("sync", h))
        return self.rc

    def siml_last_error(self):
        return b"a bounded device wait gave up"


def _wrapper(monkeypatch, lib):
    import importlib
    G = importlib.import_module("siml_gb300.GPULingo")
    from siml_gb300 import _native as N
    monkeypatch.setattr(N, "lib", lambda: lib)
    gl = object.__new__(G.GPULingo)
    gl._h = HANDLE   # a null handle: the destructor has nothing to destroy
    gl._pending = None
    return gl


def test_replacing_a_pending_result_waits_for_the_stream(monkeypatch):
    lib = _FakeLib()
    gl = _wrapper(monkeypatch, lib)
    gl._set_pending(("matrix", "first", 4))
    assert lib.calls == []                      # nothing outstanding: no wait
    gl._set_pending(("matrix", "second", 4))
    assert lib.calls == [("sync", HANDLE)]    # the dropped result's writes finished first
    assert gl._pending == ("matrix", "second", 4)


def test_retrieve_waits_and_clears(monkeypatch):
    import numpy as np
    lib = _FakeLib()
    gl = _wrapper(monkeypatch, lib)
    with pytest.raises(RuntimeError):
        gl.retrieveAsyncResult()
    gl._set_pending(("matrix", np.arange(12, dtype=np.float32).reshape(2, 6), 4))
    got = gl.retrieveAsyncResult()
    assert lib.calls == [("sync", HANDLE)] and got.shape == (2, 4) and gl._pending is None
    with pytest.raises(RuntimeError):
        gl.retrieveAsyncResult()


def test_a_dropped_results_error_is_reported(monkeypatch):
    from siml_gb300 import _native as N
    lib = _FakeLib(rc=N.SIML_ERR_TIMEOUT)
    gl = _wrapper(monkeypatch, lib)
    gl._set_pending(("matrix", "first", 4))
    with pytest.raises(N.SimlError):
        gl._set_pending(("matrix", "second", 4))
