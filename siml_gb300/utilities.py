"""Drop-in for pySIML's ``pysiml.utilities`` (pysiml/utilities.py).

``rowHistogram101`` runs on the GPU (the reference's is a C loop,
pysiml/_cpuutil.cpp:52-126): a uint32 [rows, 101] histogram of each row of a
float32 or float64 matrix, bins (-inf, 0.01), [0.01, 0.02), ..., [0.99, 1.0),
[1.0, inf).  numpy input gives numpy output; a CUDA tensor gives a CUDA tensor.
"""
from __future__ import annotations

import ctypes
import threading

import numpy as np

from . import _native as N

try:
    import torch
except Exception:  # pragma: no cover
    torch = None

_engines = {}
_lock = threading.Lock()


class _Shared:
    """The module's engine handle for one device, with the lock that its users
    (rowHistogram101 and the GPU compiler) hold while they set its stream and
    run: an engine handle serves one host thread at a time."""

    def __init__(self, h):
        self.h = h
        self.lock = threading.Lock()


def _shared(device: int) -> _Shared:
    with _lock:
        e = _engines.get(device)
        if e is None:
            h = ctypes.c_void_p()
            N.check(N.lib().siml_create(int(device), ctypes.byref(h)), "siml_create")
            e = _engines[device] = _Shared(h)
        return e


def rowHistogram101(datamatrix, device: int = 0):
    L = N.lib()
    if torch is not None and isinstance(datamatrix, torch.Tensor) and datamatrix.is_cuda:
        if datamatrix.dim() != 2:
            raise ValueError("Data given to rowHistogram101 was not of dimension 2")
        if datamatrix.dtype not in (torch.float32, torch.float64):
            raise ValueError("Data given to rowHistogram101 was not of float (float32) or double (float64) type")
        d = datamatrix if datamatrix.stride(1) == 1 else datamatrix.contiguous()
        out = torch.empty((d.shape[0], 101), dtype=torch.int32, device=d.device)
        e = _shared(d.device.index)
        with e.lock:
            N.check(L.siml_set_stream(e.h, N.stream_arg(torch.cuda.current_stream(d.device))), "siml_set_stream")
            fn = L.siml_row_histogram101_f64 if d.dtype == torch.float64 else L.siml_row_histogram101
            N.check(fn(e.h, d.data_ptr(), d.shape[0], d.shape[1], d.stride(0), out.data_ptr(), N.SIML_DEVICE),
                    "rowHistogram101")
        return out
    a = np.asarray(datamatrix)
    if a.dtype not in (np.float32, np.float64):
        raise ValueError("Data given to rowHistogram101 was not of float (float32) or double (float64) type")
    if a.ndim != 2:
        raise ValueError("Data given to rowHistogram101 was not of dimension 2")
    a = np.ascontiguousarray(a)
    out = np.zeros((a.shape[0], 101), dtype=np.uint32)
    e = _shared(device)
    with e.lock:
        N.check(L.siml_set_stream(e.h, None), "siml_set_stream")
        fn = L.siml_row_histogram101_f64 if a.dtype == np.float64 else L.siml_row_histogram101
        N.check(fn(e.h, a.ctypes.data, a.shape[0], a.shape[1], a.shape[1], out.ctypes.data, N.SIML_HOST),
                "rowHistogram101")
    return out
