"""Shared fixtures.  Tests marked ``gpu`` need a CUDA GPU (GB300); everything
else runs on the CPU.  The oracle (oracle/) only computes the expected results."""
import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a)")


@pytest.fixture(scope="session")
def native():
    from siml_gb300 import build, _native
    build.build()
    return _native.lib()


@pytest.fixture(scope="session")
def oracle():
    from oracle import cpulingo
    cpulingo.build()
    return cpulingo


@pytest.fixture(scope="session")
def golden():
    g = np.load(os.path.join(REPO, "tests", "golden", "golden.npz"))
    d = {k: g[k] for k in g.files}
    buf = d["smiles_buf"].tobytes()
    off = d["smiles_off"]
    d["strings"] = [buf[off[i]:off[i + 1]] for i in range(len(off) - 1)]
    return d


@pytest.fixture(scope="session")
def set4096(native):
    from siml_gb300 import synthetic as S
    return S.smiles_set(S.SEED_ALLPAIRS, S.UNIFORM_20_90, 4096)
