"""On-disk SMILES sets (no GPU): save/load round trip and streaming
compilation of a .smi file, equal to the in-memory compiler."""
import numpy as np


def test_save_load_round_trip(native, tmp_path, set4096):
    from siml_gb300 import store
    store.save_set(str(tmp_path / "s"), *set4096)
    got = store.load_set(str(tmp_path / "s"))
    for a, b in zip(got, set4096):
        assert np.array_equal(np.asarray(a), np.asarray(b).reshape(np.asarray(a).shape))
    assert isinstance(got[0], np.memmap)


def test_compile_file_matches_compiler(native, tmp_path):
    from siml_gb300 import store, synthetic as S
    from siml_gb300.compiler import cSMILEStoMatrices
    smi = S.smiles_list(S.SEED_ALLPAIRS, S.UNIFORM_20_90, 2500)
    path = tmp_path / "x.smi"
    with open(path, "wb") as f:
        for i, s in enumerate(smi):
            f.write(s + b" mol%d\n" % i)
        f.write(b"\n")   # a blank line is skipped
    n = store.compile_file(str(path), str(tmp_path / "set"), chunk=700)
    assert n == 2500
    L, C, ln, mg = store.load_set(str(tmp_path / "set"))
    RL, RC, Rln, Rmg, names = cSMILEStoMatrices(smi)
    w = RL.shape[1]
    assert L.shape[1] >= w and not np.any(np.asarray(L)[:, w:]) and not np.any(np.asarray(C)[:, w:])
    assert np.array_equal(np.asarray(L)[:, :w], RL) and np.array_equal(np.asarray(C)[:, :w], RC)
    assert np.array_equal(ln, Rln.reshape(-1)) and np.array_equal(mg, Rmg.reshape(-1))
