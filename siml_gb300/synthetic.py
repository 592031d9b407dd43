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

# Seeds of the benchmark workloads.  Query sets are later index ranges of the
# same generator as their database.
SEED_ALLPAIRS = 20260001   # 4,096 strings, uniform 20-90 chars, both sets
SEED_DB_1M = 20260002      # 1M database (lognormal median 45) + its query rows
SEED_RAGGED = 20260004     # 2M bimodal database of the ragged-job workload
SEED_SERVING = 20260005    # 10M serving database (uniform 20-90) + requests


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
