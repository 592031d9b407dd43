"""Generates tests/golden/golden.npz from the reference's own compiled C code.

Run in a container where the reference sources are present:

    make -C oracle ref && python tests/golden/make_golden.py

It compiles SMILES with the reference's ``_ccompiler.SMILEStoMatrices``
(pysiml/_ccompiler.cpp), computes Tanimoto blocks with
``_CPULingo.getTanimotoBlock`` / ``getTanimotoBlockParallel``
(pysiml/_CPULingo.c) and row histograms with ``_cpuutil.rowHistogram101``
(pysiml/_cpuutil.cpp), and stores inputs and outputs.  Inputs are the seeded
synthetic strings of siml_gb300.synthetic plus hand-made edge cases.

Every string is passed to the reference with a trailing newline.  The
reference compiler sizes its scratch buffer from the raw string length and,
for a string of length 4k with no terminator, reads three bytes past the part
it zeroed (pysiml/_ccompiler.cpp:298-313 vs :139-148), picking up leftovers of
earlier strings; a newline ends the string without changing its LINGOs (the
edge cases below never end inside a '+', '-', 'H', '[' digit run, where a
newline would be copied).
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from oracle import cpulingo as O  # noqa: E402
from siml_gb300 import synthetic as S  # noqa: E402

EDGE_STRINGS = [
    b"", b"C", b"CC", b"CCC", b"CCCC", b"CCCCC", b"CCCCCC",
    b"c1ccccc1", b"c1ccccc1 benzene", b"CC(=O)O acetic acid", b"CC(=O)O\tacetic",
    b" CCCC", b"CCO\r\n", b"CCN\nCCC",
    b"C[C@H]1CC1O", b"[NH3+]CCC(=O)[O-]", b"[2H]C([2H])([2H])O", b"CC%12CCC%12C", b"C%1CC",
    b"C1CC2CC1CC2", b"OC1=CC=CC=C1OH2x", b"H2O2x", b"CCH3C", b"N#N", b"Cl/C=C/Cl",
    b"C" * 40, b"C" * 300, b"c1ccc(cc1)c1ccccc1" * 3, b"CCOCCOCCOCCOCCOCCOCCOCCOCC",
    b"CC\xc3\xa9CCCCCCCCCC", b"\xc3\xa9CCCCCCCCCCCC", b"CCCC\xe2\x82\xacNCCCCCCCC",
    b"OCC\xc2\xb0C(C)CCCCCCCCO",
]


def _ref(name):
    m = O.reference_module(name)
    if m is None:
        raise SystemExit("reference module %s not built: run `make -C oracle ref` first" % name)
    return m


def pack(strings):
    off = np.zeros(len(strings) + 1, np.int64)
    np.cumsum([len(s) for s in strings], out=off[1:])
    return np.frombuffer(b"".join(strings) or b"\0", np.uint8)[:off[-1]].copy(), off


def main():
    cc, cp, cu = _ref("_ccompiler"), _ref("_CPULingo"), _ref("_cpuutil")
    synth = (S.smiles_list(S.SEED_ALLPAIRS, S.UNIFORM_20_90, 200)
             + S.smiles_list(S.SEED_DB_1M, S.LOGNORMAL_45, 200)
             + S.smiles_list(S.SEED_RAGGED, S.BIMODAL_35_110, 100))
    strings = EDGE_STRINGS + synth
    L, C, ln, mg = cc.SMILEStoMatrices([s + b"\n" for s in strings])
    ln = ln[:, 0].copy()
    mg = mg[:, 0].copy()
    # Tanimoto block: rows = 64 synthetic + all edge cases, columns = everything
    nedge = len(EDGE_STRINGS)
    rows = list(range(nedge)) + list(range(nedge, nedge + 64))
    RL, RC = L[rows].copy(), C[rows].copy()
    Rln, Rmg = ln[rows].copy(), mg[rows].copy()
    T = cp.getTanimotoBlock(RL, RC, Rmg.reshape(-1, 1), Rln.reshape(-1, 1), L, C, mg.reshape(-1, 1), ln.reshape(-1, 1))
    TP = cp.getTanimotoBlockParallel(RL, RC, Rmg.reshape(-1, 1), Rln.reshape(-1, 1), L, C, mg.reshape(-1, 1),
                                     ln.reshape(-1, 1), 4)
    assert np.array_equal(T, TP), "reference serial and parallel blocks differ"
    H = cu.rowHistogram101(T)
    buf, off = pack(strings)
    out = os.path.join(HERE, "golden.npz")
    np.savez_compressed(out, smiles_buf=buf, smiles_off=off, lingos=L, counts=C, lengths=ln, mags=mg,
                        rows=np.asarray(rows, np.int64), tanimoto=T, hist101=H,
                        n_edge=np.int64(nedge))
    print("wrote", out, os.path.getsize(out), "bytes;", len(strings), "strings, block", T.shape)


if __name__ == "__main__":
    main()
