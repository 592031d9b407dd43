"""On-disk SMILES sets, so a large database is compiled once and loads in
seconds.

A set is a directory of four .npy files, the zero-padded arrays the compiler
produces (pysiml/_ccompiler.cpp:354-357): lingos and counts [n, width] int32,
lengths and mags [n] int32, plus `set.json` with the sizes.  `load_set`
memory-maps them, so the arrays stream straight into `set_qsmiles`.
`compile_file` compiles a .smi file (one SMILES per line; text after the
first space is a name) into such a directory chunk by chunk, with the
multithreaded native compiler.
"""
from __future__ import annotations

import json
import os

import numpy as np

from . import _native as N
from .compiler import compile_buffer

_NAMES = ("lingos", "counts", "lengths", "mags")
FORMAT = "siml-set-1"


def save_set(path, lingos, counts, lengths, mags):
    """Writes a compiled set to directory `path` (created if needed)."""
    os.makedirs(path, exist_ok=True)
    arrays = (np.ascontiguousarray(lingos, np.int32), np.ascontiguousarray(counts, np.int32),
              np.ascontiguousarray(np.asarray(lengths).reshape(-1), np.int32),
              np.ascontiguousarray(np.asarray(mags).reshape(-1), np.int32))
    n = arrays[0].shape[0]
    if arrays[1].shape != arrays[0].shape or arrays[2].shape[0] != n or arrays[3].shape[0] != n:
        raise ValueError("inconsistent set shapes")
    for name, a in zip(_NAMES, arrays):
        np.save(os.path.join(path, name + ".npy"), a)
    with open(os.path.join(path, "set.json"), "w") as f:
        json.dump({"format": FORMAT, "n": int(n), "width": int(arrays[0].shape[1])}, f)


def load_set(path, mmap=True):
    """(lingos, counts, lengths, mags) of a saved set, memory-mapped by default."""
    with open(os.path.join(path, "set.json")) as f:
        meta = json.load(f)
    if meta.get("format") != FORMAT:
        raise ValueError("%s: not a %s directory" % (path, FORMAT))
    mode = "r" if mmap else None
    arrays = tuple(np.load(os.path.join(path, name + ".npy"), mmap_mode=mode) for name in _NAMES)
    if arrays[0].shape != (meta["n"], meta["width"]):
        raise ValueError("%s: array shapes do not match set.json" % path)
    return arrays


def _lines(path):
    with open(path, "rb") as f:
        for line in f:
            line = line.strip()
            if line:
                yield line.split(None, 1)[0]


def _pack(strings):
    off = np.zeros(len(strings) + 1, dtype=np.int64)
    if strings:
        np.cumsum([len(s) for s in strings], out=off[1:])
    return b"".join(strings), off


def compile_file(smi_path, out_dir, chunk=1 << 20):
    """Compiles a .smi file into a saved set; returns the molecule count.
    Two passes: the widest molecule fixes the width, then each chunk is
    compiled straight into the memory-mapped output."""
    lib = N.lib()
    width, n, chunks = 0, 0, []
    batch = []
    for s in _lines(smi_path):
        batch.append(s)
        if len(batch) == chunk:
            chunks.append(len(batch))
            buf, off = _pack(batch)
            w = lib.siml_compile_width(buf or b"\0", off.ctypes.data, len(batch))
            if w < 0:
                N.check(int(-w), "siml_compile_width")
            width, n, batch = max(width, int(w)), n + len(batch), []
    if batch:
        buf, off = _pack(batch)
        w = lib.siml_compile_width(buf or b"\0", off.ctypes.data, len(batch))
        if w < 0:
            N.check(int(-w), "siml_compile_width")
        width, n = max(width, int(w)), n + len(batch)
    width = max(width, 1)
    os.makedirs(out_dir, exist_ok=True)
    mm = {name: np.lib.format.open_memmap(os.path.join(out_dir, name + ".npy"), mode="w+", dtype=np.int32,
                                          shape=(n, width) if name in ("lingos", "counts") else (n,))
          for name in _NAMES}
    row, batch = 0, []

    def flush(b, row):
        buf, off = _pack(b)
        L, C, ln, mg = compile_buffer(buf, off)
        k = len(b)
        mm["lingos"][row:row + k, :L.shape[1]] = L
        mm["lingos"][row:row + k, L.shape[1]:] = 0
        mm["counts"][row:row + k, :C.shape[1]] = C
        mm["counts"][row:row + k, C.shape[1]:] = 0
        mm["lengths"][row:row + k] = ln
        mm["mags"][row:row + k] = mg
        return row + k

    for s in _lines(smi_path):
        batch.append(s)
        if len(batch) == chunk:
            row, batch = flush(batch, row), []
    if batch:
        row = flush(batch, row)
    for a in mm.values():
        a.flush()
    with open(os.path.join(out_dir, "set.json"), "w") as f:
        json.dump({"format": FORMAT, "n": int(n), "width": int(width)}, f)
    return n
