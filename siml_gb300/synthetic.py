"""Seeded synthetic SMILES-like workloads (native generator, csrc/synth.cpp).

Molecule i of a set depends only on (seed, length model, i), so any slice of a
set can be regenerated and x86 and Arm hosts produce identical bytes.
"""
from __future__ import annotations

import numpy as np

from . import _native as N
from .compiler import compile_buffer

UNIFORM_20_90 = N.SYNTH_UNIFORM_20_90
LOGNORMAL_45 = N.SYNTH_LOGNORMAL_45
BIMODAL_35_110 = N.SYNTH_BIMODAL_35_110
CHEM_45 = N.SYNTH_CHEM_45           # lognormal 45 with bracket atoms, charges, %nn ring labels

# Seeds of the benchmark workloads.  Query sets are later index ranges of the
# same generator as their database.
SEED_ALLPAIRS = 20260001   # 4,096 strings, uniform 20-90 chars, both sets
SEED_DB_1M = 20260002      # 1M database (lognormal median 45) + its query rows
SEED_RAGGED = 20260004     # 2M bimodal database of the ragged-job workload
SEED_SERVING = 20260005    # 10M serving database (uniform 20-90) + requests
SEED_CHEM = 20260006       # chemistry-like 1M database (bracket atoms, charges)


def smiles_buffer(seed: int, dist: int, n: int, first: int = 0):
    """(bytes, offsets[n+1]) of molecules [first, first+n)."""
    L = N.lib()
    lens = np.empty(n, dtype=np.int32)
    N.check(L.siml_synth_lengths(seed, dist, first, n, lens.ctypes.data), "siml_synth_lengths")
    total = int(lens.sum(dtype=np.int64))
    buf = np.empty(max(total, 1), dtype=np.uint8)
    offsets = np.empty(n + 1, dtype=np.int64)
    N.check(L.siml_synth_smiles(seed, dist, first, n, buf.ctypes.data, buf.shape[0], offsets.ctypes.data),
            "siml_synth_smiles")
    return buf[:total].tobytes(), offsets


def smiles_list(seed: int, dist: int, n: int, first: int = 0):
    buf, off = smiles_buffer(seed, dist, n, first)
    return [buf[off[i]:off[i + 1]] for i in range(n)]


def smiles_set(seed: int, dist: int, n: int, first: int = 0):
    """Compiled set: (lingos [n,w], counts [n,w], lengths [n], mags [n])."""
    buf, off = smiles_buffer(seed, dist, n, first)
    return compile_buffer(buf, off)


def ragged_jobs(seed: int, n_db: int, njobs: int, rows_max: int = 2048, cols_min: int = 1000,
                cols_max: int = 200_000):
    """Neighbour jobs over one n_db-molecule set used as both sides: int64
    [njobs, 4] {row_begin, row_end, col_begin, col_end}.  Row counts are
    log-uniform in [1, rows_max], column counts log-uniform in [cols_min,
    cols_max]; both ranges start uniformly at random."""
    rng = np.random.default_rng(seed)
    nr = np.floor(np.exp(rng.uniform(0.0, np.log(rows_max + 1), njobs))).astype(np.int64).clip(1, rows_max)
    nc = np.floor(np.exp(rng.uniform(np.log(cols_min), np.log(cols_max + 1), njobs))).astype(np.int64)
    nc = nc.clip(cols_min, min(cols_max, n_db))
    nr = nr.clip(1, n_db)
    rb = np.floor(rng.random(njobs) * (n_db - nr + 1)).astype(np.int64)
    cb = np.floor(rng.random(njobs) * (n_db - nc + 1)).astype(np.int64)
    return np.ascontiguousarray(np.stack([rb, rb + nr, cb, cb + nc], 1))
