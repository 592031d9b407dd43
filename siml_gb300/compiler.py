"""Drop-in for pySIML's ``pysiml.compiler`` (pysiml/compiler.py).

``cSMILEStoMatrices`` runs the native multithreaded compiler
(siml_gb300/csrc/lingo_compiler.cpp), which produces exactly the reference C
compiler's output (pysiml/_ccompiler.cpp).  ``compile_buffer_gpu`` produces
the same arrays on the GPU (siml_gb300/csrc/compile_gpu.cu, sharing the
rules of siml_gb300/csrc/lingo_compile_core.h).  ``SMILEStoMatrices``,
``SMILEStoMultiset`` and ``preprocessNumbers`` restate the reference's pure
Python variants (pysiml/compiler.py:98-194) for Python 3.

Strings may be ``str`` (encoded as UTF-8) or ``bytes``; a file object works
as an iterable of lines.
"""
from __future__ import annotations


import numpy as np

from . import _native as N


def _to_bytes_list(smileslist):
    out = []
    for s in smileslist:
        out.append(s.encode("utf-8") if isinstance(s, str) else bytes(s))
    return out


def _pack(strings):
    offsets = np.zeros(len(strings) + 1, dtype=np.int64)
    if strings:
        np.cumsum([len(s) for s in strings], out=offsets[1:])
    return b"".join(strings), offsets


def compile_buffer(buf: bytes, offsets: np.ndarray):
    """Compiles concatenated SMILES (string i at buf[offsets[i]:offsets[i+1]])
    into (lingos [n, w], counts [n, w], lengths [n], mags [n]) int32 arrays."""
    L = N.lib()
    offsets = np.ascontiguousarray(offsets, dtype=np.int64)
    n = offsets.shape[0] - 1
    cbuf = buf if buf else b"\0"
    # one pass: each string compiled once into staging sized like the text
    # (a string has at most as many unique windows as bytes), then scattered
    total = int(offsets[-1]) if n > 0 else 0
    stage_codes = np.empty(max(total, 1), dtype=np.int32)
    stage_counts = np.empty(max(total, 1), dtype=np.int32)
    lengths = np.empty(n, dtype=np.int32)
    mags = np.empty(n, dtype=np.int32)
    w = L.siml_compile_stage(cbuf, offsets.ctypes.data, n, stage_codes.ctypes.data, stage_counts.ctypes.data,
                             lengths.ctypes.data, mags.ctypes.data)
    if w < 0:
        N.check(int(-w), "siml_compile_stage")
    lingos = np.empty((n, w), dtype=np.int32)
    counts = np.empty((n, w), dtype=np.int32)
    N.check(L.siml_compile_scatter(offsets.ctypes.data, n, stage_codes.ctypes.data, stage_counts.ctypes.data,
                                   lengths.ctypes.data, lingos.ctypes.data, counts.ctypes.data, w),
            "siml_compile_scatter")
    return lingos, counts, lengths, mags


def compile_buffer_gpu(buf, offsets, device: int = 0):
    """compile_buffer on the GPU: the same four arrays, as int32 CUDA tensors
    on cuda:device (queued on torch's current stream).  buf is bytes or a
    uint8 CUDA tensor holding offsets[-1] bytes; offsets an int64 array or
    tensor of n+1 entries.  The result can go straight to set_qsmiles /
    set_refsmiles without a host round trip."""
    import torch
    from .utilities import _shared
    dev = torch.device("cuda", device)
    off_h = offsets.cpu().numpy() if isinstance(offsets, torch.Tensor) else np.asarray(offsets)
    off_h = np.ascontiguousarray(off_h, dtype=np.int64).reshape(-1)
    n = off_h.shape[0] - 1
    if n < 0:
        raise ValueError("offsets needs at least one entry")
    total = int(off_h[-1]) if n >= 0 else 0
    if isinstance(buf, torch.Tensor):
        if not buf.is_cuda or buf.dtype != torch.uint8:
            raise ValueError("a tensor buffer must be a uint8 CUDA tensor")
        text = buf.contiguous()
        if text.numel() < total:
            raise ValueError("buffer holds %d bytes, offsets need %d" % (text.numel(), total))
    else:
        raw = memoryview(buf).cast("B")
        if raw.nbytes < total:
            raise ValueError("buffer holds %d bytes, offsets need %d" % (raw.nbytes, total))
        if total == 0:
            text = torch.zeros(1, dtype=torch.uint8, device=dev)
        else:
            import warnings
            with warnings.catch_warnings():   # read-only host bytes, only ever read
                warnings.simplefilter("ignore")
                host = torch.from_numpy(np.frombuffer(raw[:total], dtype=np.uint8))
            text = host.to(dev)
    off_d = torch.from_numpy(off_h).to(dev)
    L = N.lib()
    e = _shared(device)
    with e.lock:
        h = e.h
        N.check(L.siml_set_stream(h, N.stream_arg(torch.cuda.current_stream(dev))), "siml_set_stream")
        # one pass: every string compiled once into staging (its stretch of
        # the byte range holds its unique codes), then scattered into rows
        stage_codes = torch.empty(max(total, 1), dtype=torch.int32, device=dev)
        stage_counts = torch.empty(max(total, 1), dtype=torch.int32, device=dev)
        lengths = torch.empty(max(n, 1), dtype=torch.int32, device=dev)[:n]
        mags = torch.empty(max(n, 1), dtype=torch.int32, device=dev)[:n]
        w = L.siml_compile_stage_gpu(h, text.data_ptr(), off_d.data_ptr(), n, stage_codes.data_ptr(),
                                     stage_counts.data_ptr(), lengths.data_ptr(), mags.data_ptr())
        if w < 0:
            N.check(int(-w), "siml_compile_stage_gpu")
        lingos = torch.empty((n, w), dtype=torch.int32, device=dev)
        counts = torch.empty((n, w), dtype=torch.int32, device=dev)
        if w > 0 and n > 0:
            N.check(L.siml_compile_scatter_gpu(h, off_d.data_ptr(), n, stage_codes.data_ptr(), stage_counts.data_ptr(),
                                               lengths.data_ptr(), lingos.data_ptr(), counts.data_ptr(), w),
                    "siml_compile_scatter_gpu")
        del stage_codes, stage_counts   # the scatter has returned: its reads are done
    return lingos, counts, lengths, mags


def _getSMILESname(smi):
    fields = smi.split()
    if len(fields) > 1:
        return fields[1]
    return b"" if isinstance(smi, bytes) else ""


def cSMILEStoMatrices(smileslist):
    """SMILES strings -> (Lingo matrix, count matrix, length vector [N,1],
    magnitude vector [N,1], names), as pysiml/compiler.py:53-82."""
    items = list(smileslist)
    strings = _to_bytes_list(items)
    buf, offsets = _pack(strings)
    lingos, counts, lengths, mags = compile_buffer(buf, offsets)
    names = [_getSMILESname(s) for s in items]
    return lingos, counts, lengths.reshape(-1, 1), mags.reshape(-1, 1), names


_DIGITS = bytes.maketrans(b"123456789", b"000000000")


def preprocessNumbers(smi, xtable=None):
    """Maps digits 1-9 to '0' (pysiml/compiler.py:135-149)."""
    if isinstance(smi, str):
        return smi.translate(str.maketrans("123456789", "000000000"))
    return bytes(smi).translate(_DIGITS)


def SMILEStoMultiset(smiles):
    """Sorted unique 4-byte windows and counts of one string, no preprocessing
    (pysiml/compiler.py:98-133); returns two int32 [k, 1] arrays."""
    b = smiles.encode("utf-8") if isinstance(smiles, str) else bytes(smiles)
    a = np.frombuffer(b, dtype=np.uint8).astype(np.uint32)
    if a.shape[0] < 4:
        codes = np.zeros(0, dtype=np.int32)
    else:
        codes = (a[:-3] | (a[1:-2] << 8) | (a[2:-1] << 16) | (a[3:] << 24)).view(np.int32)
    u, c = np.unique(codes, return_counts=True)
    return u.astype(np.int32).reshape(-1, 1), c.astype(np.int32).reshape(-1, 1)


def SMILEStoMatrices(smileslist):
    """Pure-Python-variant compiler (pysiml/compiler.py:151-194): first
    whitespace field of each line, digits 1-9 -> '0', all 4-byte windows.
    Magnitudes are the count sums (shape [N])."""
    lingos, counts, names = [], [], []
    maxw = 0
    for line in smileslist:
        fields = line.split()
        smi = preprocessNumbers(fields[0]) if fields else (b"" if isinstance(line, bytes) else "")
        l, c = SMILEStoMultiset(smi)
        lingos.append(l)
        counts.append(c)
        names.append(fields[1] if len(fields) > 1 else (b"" if isinstance(line, bytes) else ""))
        maxw = max(maxw, l.shape[0])
    n = len(lingos)
    lm = np.zeros((n, maxw), dtype=np.int32)
    cm = np.zeros_like(lm)
    ln = np.empty((n, 1), dtype=np.int32)
    for i in range(n):
        k = lingos[i].shape[0]
        ln[i] = k
        lm[i, :k] = lingos[i][:, 0]
        cm[i, :k] = counts[i][:, 0]
    return lm, cm, ln, np.int32(cm.sum(1)), names
