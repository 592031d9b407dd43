"""The C-ABI library: loads, exports every entry point include/siml_gb300.h
declares, and reports errors through status codes (no GPU needed)."""
import os
import re

import pytest

from tests.conftest import REPO


def header_symbols():
    text = open(os.path.join(REPO, "include", "siml_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(siml_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported(native):
    syms = header_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(native, s), s


def test_version_and_error_reporting(native):
    from siml_gb300 import _native as N
    assert b"sm_103a" in native.siml_version()
    # bad arguments: status + message, no crash
    rc = native.siml_compile_smiles(b"abc", None, 1, None, None, None, None, 4)
    assert rc == N.SIML_ERR_INVALID
    assert "bad arguments" in N.last_error()
    with pytest.raises(ValueError):
        N.check(rc)


def test_async_error_words_decode_on_the_host(native):
    """How siml_sync reports the error bits the kernels set: bit 1 (a top-k
    lock wait ran out) as SIML_ERR_TIMEOUT, bit 2 (a batch work item outside
    its plan) and bit 3 (a ref-row vid the shared table cannot hold) as
    SIML_ERR_STATE, each with its own message; the lowest bit decides."""
    from siml_gb300 import _native as N
    assert native.siml_debug_async_status(0) == N.SIML_OK
    assert native.siml_debug_async_status(1) == N.SIML_ERR_TIMEOUT
    assert "lock wait" in N.last_error()
    assert native.siml_debug_async_status(2) == N.SIML_ERR_STATE
    assert "work item" in N.last_error()
    assert native.siml_debug_async_status(4) == N.SIML_ERR_STATE
    assert "rare-vid hash" in N.last_error()
    assert native.siml_debug_async_status(6) == N.SIML_ERR_STATE
    assert "work item" in N.last_error()
    assert native.siml_debug_async_status(7) == N.SIML_ERR_TIMEOUT


def test_null_handle_is_rejected(native):
    from siml_gb300 import _native as N
    assert native.siml_sync(None) == N.SIML_ERR_INVALID
    assert native.siml_rows(None, 0, 1, None, 1, 0) == N.SIML_ERR_INVALID
    assert native.siml_launch_count(None) == -1


def test_gpulingo_fails_loudly_without_gpu(native):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from siml_gb300 import GPULingo, _native as N
    with pytest.raises((N.SimlError, ValueError)):
        GPULingo(0)


def test_sliced_counter_host_unit(tmp_path):
    """The bit-sliced counter and plane transpose of the kernels
    (siml_gb300/csrc/lingo_core.cuh) checked against scalar sums on the host."""
    import subprocess
    exe = str(tmp_path / "sct")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(REPO, "siml_gb300", "csrc"),
                    "-I", os.path.join(REPO, "include"),
                    os.path.join(REPO, "tests", "native", "sliced_counter_test.cpp"), "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr


def test_stream_argument_maps_torch_default_stream_to_legacy():
    """siml_set_stream(NULL) selects the engine's own (non-blocking) stream,
    so torch's default stream (handle 0) is passed as cudaStreamLegacy."""
    from siml_gb300 import _native as N

    class _S:
        def __init__(self, h):
            self.cuda_stream = h

    assert N.stream_arg(_S(0)).value == N.CUDA_STREAM_LEGACY == 1
    assert N.stream_arg(_S(0x7F001234)).value == 0x7F001234


def test_header_is_plain_c_and_links(native, tmp_path):
    """include/siml_gb300.h compiles as strict C99 and a C caller links
    against the library, as a cgo or C binding would."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "caller.c"
    src.write_text('#include "siml_gb300.h"\n'
                   'int main(void) {\n'
                   '    siml_engine* h = 0;\n'
                   '    int rc = siml_create(0, &h);\n'
                   '    if (rc == SIML_OK) siml_destroy(h);\n'
                   '    return siml_last_error() == 0;\n'
                   '}\n')
    lib_dir = os.path.join(REPO, "siml_gb300")
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", str(src), "-o",
                        str(tmp_path / "caller"), "-I", os.path.join(REPO, "include"), "-L", lib_dir,
                        "-lsiml_gb300", "-Wl,-rpath," + lib_dir], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_header_constants_match_the_python_binding():
    """Every #define of the C header has the same value on the Python side:
    status codes, pointer locations and tuning keys in _native, the synthetic
    generator's models in synthetic."""
    import os
    import re
    from siml_gb300 import _native as N
    from siml_gb300 import synthetic as S
    path = os.path.join(os.path.dirname(__file__), "..", "include", "siml_gb300.h")
    defs = re.findall(r"^#define (SIML_[A-Z0-9_]+)\s+(-?\w+)", open(path).read(), re.M)
    assert len(defs) > 20
    for name, value in defs:
        if name.startswith("SIML_SYNTH_"):
            assert getattr(S, name[len("SIML_SYNTH_"):]) == int(value, 0), name
        else:
            assert getattr(N, name) == int(value, 0), name
