"""SMILES -> LINGO compiler of the product (siml_gb300.compiler, native
lingo_compiler.cpp) against the oracle and the golden fixtures."""
import numpy as np
import pytest

from siml_gb300 import compiler as PC
from siml_gb300 import synthetic as S


def _cmp(a, b):
    La, Ca, la, ma = a
    Lb, Cb, lb, mb = b
    assert np.array_equal(np.asarray(la).reshape(-1), np.asarray(lb).reshape(-1))
    assert np.array_equal(np.asarray(ma).reshape(-1), np.asarray(mb).reshape(-1))
    w = max(La.shape[1], Lb.shape[1])
    pad = lambda M: np.pad(M, ((0, 0), (0, w - M.shape[1])))
    assert np.array_equal(pad(La), pad(Lb))
    assert np.array_equal(pad(Ca), pad(Cb))


def test_compiler_matches_golden(native, golden):
    buf = b"".join(golden["strings"])
    off = golden["smiles_off"]
    L, C, ln, mg = PC.compile_buffer(buf, off)
    assert L.shape == golden["lingos"].shape
    _cmp((L, C, ln, mg), (golden["lingos"], golden["counts"], golden["lengths"], golden["mags"]))


def test_cSMILEStoMatrices_api(native, oracle):
    smi = ["c1ccccc1 benzene", b"CCO ethanol\n", "CC(=O)O", "C"]
    L, C, ln, mg, names = PC.cSMILEStoMatrices(smi)
    assert ln.shape == (4, 1) and mg.shape == (4, 1) and L.dtype == np.int32
    assert names == ["benzene", b"ethanol", "", ""]
    _cmp((L, C, ln, mg), oracle.cSMILEStoMatrices(smi)[:4])
    assert mg[3, 0] == 0 and ln[3, 0] == 0


ALPHABET = list(b"CcNnOoSFlBr()=#123456789%+-H[]@/\\ ") + [0x0A, 0x0D, 0x09, 0x00, 0x80, 0xC3, 0xA9, 0xFF, 0xE2]


@pytest.mark.parametrize("seed", range(4))
def test_compiler_fuzz_against_oracle(native, oracle, seed):
    """Random byte strings over SMILES characters, digits, '%', '+-H[',
    terminators, NUL and bytes >= 0x80 (the reference's sign-extending shift)."""
    rng = np.random.default_rng(1000 + seed)
    strs = []
    for _ in range(3000):
        n = int(rng.integers(0, 40))
        w = rng.random(len(ALPHABET))
        w[-9:] *= 0.05 if seed % 2 == 0 else 0.6
        p = w / w.sum()
        strs.append(bytes(rng.choice(ALPHABET, size=n, p=p).astype(np.uint8)))
    buf = b"".join(strs)
    off = np.zeros(len(strs) + 1, np.int64)
    np.cumsum([len(s) for s in strs], out=off[1:])
    got = PC.compile_buffer(buf, off)
    want = oracle.compile_strings(strs)
    _cmp(got, want)


def test_compiler_synthetic_sets(native, oracle):
    for seed, dist in [(S.SEED_ALLPAIRS, S.UNIFORM_20_90), (S.SEED_DB_1M, S.LOGNORMAL_45),
                       (S.SEED_RAGGED, S.BIMODAL_35_110)]:
        strs = S.smiles_list(seed, dist, 2000, first=123)
        _cmp(S.smiles_set(seed, dist, 2000, first=123), oracle.compile_strings(strs))


def test_python_variant_compiler(native, oracle):
    smi = ["c1ccccc1 benzene", "CC(=O)O", "C", "[NH3+]CC12", "c1ccc2c(c1)cccc2 naphthalene"]
    L, C, ln, mg, names = PC.SMILEStoMatrices(smi)
    L2, C2, ln2, mg2, names2 = oracle.SMILEStoMatrices_python(smi)
    assert np.array_equal(L, L2) and np.array_equal(C, C2) and np.array_equal(ln, ln2)
    assert np.array_equal(mg, mg2) and mg.shape == (5,)
    assert names == names2
    assert PC.preprocessNumbers("C1CC2N3") == "C0CC0N0"


def test_synthetic_generator_is_deterministic(native):
    a = S.smiles_list(S.SEED_DB_1M, S.LOGNORMAL_45, 50, first=1000)
    b = S.smiles_list(S.SEED_DB_1M, S.LOGNORMAL_45, 10, first=1020)
    assert a[20:30] == b
    # fixed bytes: the same strings are produced on every host
    import hashlib
    h = hashlib.sha256(b"|".join(S.smiles_list(S.SEED_ALLPAIRS, S.UNIFORM_20_90, 64))).hexdigest()
    assert h == SYNTH_SHA256_64


# sha256 of the first 64 strings of the 4,096-string set joined by "|" (pinned on x86;
# the GPU hosts are Arm and must produce the same bytes)
SYNTH_SHA256_64 = "c795cb381d2b390216d0a9e0db24c6a813d8aba11f2bc650651bf9366db59a30"


def test_oracle_generator_equals_the_product_generator(native, oracle):
    """The oracle's copy of the workload generator (used by the CPU reference
    arm, which loads no product code) gives the product's bytes for every
    length model, and the oracle compiler its arrays."""
    from oracle import workloads as W
    assert (W.UNIFORM_20_90, W.LOGNORMAL_45, W.BIMODAL_35_110, W.CHEM_45) == \
        (S.UNIFORM_20_90, S.LOGNORMAL_45, S.BIMODAL_35_110, S.CHEM_45)
    assert (W.SEED_ALLPAIRS, W.SEED_DB_1M, W.SEED_RAGGED, W.SEED_SERVING, W.SEED_CHEM) == \
        (S.SEED_ALLPAIRS, S.SEED_DB_1M, S.SEED_RAGGED, S.SEED_SERVING, S.SEED_CHEM)
    for seed, model in ((S.SEED_ALLPAIRS, S.UNIFORM_20_90), (S.SEED_DB_1M, S.LOGNORMAL_45),
                        (S.SEED_RAGGED, S.BIMODAL_35_110), (S.SEED_CHEM, S.CHEM_45)):
        a = S.smiles_buffer(seed, model, 3000, first=999_000)
        b = oracle.synth_buffer(seed, model, 3000, first=999_000)
        assert a[0] == b[0] and np.array_equal(a[1], b[1])
        want = S.smiles_set(seed, model, 3000, first=999_000)
        got = oracle.synth_set(seed, model, 3000, first=999_000)
        assert all(np.array_equal(x, y) for x, y in zip(got, want))


def test_host_compiler_two_pass_entries_and_scatter_width(native):
    """The two-pass C entries (width, then fill) give what the one-pass
    staging path of compile_buffer gives, and the scatter refuses a width
    below the widest string."""
    from siml_gb300 import _native as N, synthetic as S
    from siml_gb300.compiler import compile_buffer
    buf, off = S.smiles_buffer(S.SEED_RAGGED, S.BIMODAL_35_110, 3000)
    one = compile_buffer(buf, off)
    L = N.lib()
    n = len(off) - 1
    w = L.siml_compile_width(buf, off.ctypes.data, n)
    assert w == one[0].shape[1]
    two = [np.empty((n, w), np.int32), np.empty((n, w), np.int32), np.empty(n, np.int32), np.empty(n, np.int32)]
    N.check(L.siml_compile_smiles(buf, off.ctypes.data, n, *(a.ctypes.data for a in two), w))
    for a, b in zip(one, two):
        assert np.array_equal(a, b)
    sc, sn = np.empty(int(off[-1]), np.int32), np.empty(int(off[-1]), np.int32)
    ln, mg = np.empty(n, np.int32), np.empty(n, np.int32)
    assert L.siml_compile_stage(buf, off.ctypes.data, n, sc.ctypes.data, sn.ctypes.data, ln.ctypes.data,
                                mg.ctypes.data) == w
    narrow = [np.empty((n, w - 1), np.int32) for _ in range(2)]
    assert L.siml_compile_scatter(off.ctypes.data, n, sc.ctypes.data, sn.ctypes.data, ln.ctypes.data,
                                  narrow[0].ctypes.data, narrow[1].ctypes.data, w - 1) == N.SIML_ERR_INVALID
