"""The GPU SMILES -> LINGO compiler (siml_gb300.compiler.compile_buffer_gpu,
csrc/compile_gpu.cu) against the golden fixtures made with the reference's
own compiler (pysiml/_ccompiler.cpp:276-381) and against the host compiler,
which the oracle pins: same widths, codes, counts, lengths and magnitudes,
byte for byte, including strings past the 1,024-byte shared-memory path."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cpu(strs):
    from siml_gb300 import compiler as PC
    buf = b"".join(strs)
    off = np.zeros(len(strs) + 1, np.int64)
    np.cumsum([len(s) for s in strs], out=off[1:])
    return PC.compile_buffer(buf, off), buf, off


def _gpu(buf, off):
    from siml_gb300 import compiler as PC
    return tuple(t.cpu().numpy() for t in PC.compile_buffer_gpu(buf, off))


def _same(a, b):
    for x, y in zip(a, b):
        assert x.shape == y.shape
        assert np.array_equal(x, y)


def test_gpu_compiler_matches_golden(native, golden):
    buf = b"".join(golden["strings"])
    got = _gpu(buf, golden["smiles_off"])
    _same(got, (golden["lingos"], golden["counts"], golden["lengths"], golden["mags"]))


ALPHABET = list(b"CcNnOoSFlBr()=#123456789%+-H[]@/\\ ") + [0x0A, 0x0D, 0x09, 0x00, 0x80, 0xC3, 0xA9, 0xFF, 0xE2]


@pytest.mark.parametrize("seed", range(4))
def test_gpu_compiler_fuzz(native, seed):
    """Random byte strings over SMILES characters, digits, '%', '+-H[',
    terminators, NUL and bytes >= 0x80 (the reference's sign-extending shift)."""
    rng = np.random.default_rng(2000 + seed)
    strs = []
    for _ in range(3000):
        n = int(rng.integers(0, 60))
        w = rng.random(len(ALPHABET))
        w[-9:] *= 0.05 if seed % 2 == 0 else 0.6
        strs.append(bytes(rng.choice(ALPHABET, size=n, p=w / w.sum()).astype(np.uint8)))
    want, buf, off = _cpu(strs)
    _same(_gpu(buf, off), want)


def test_gpu_compiler_long_strings(native):
    """Strings around and far past the shared-memory limit, ASCII and with
    high bytes, mixed with short ones."""
    rng = np.random.default_rng(77)
    strs = []
    for n in [1020, 1023, 1024, 1025, 1028, 2047, 2048, 2049, 5000, 12000]:
        for hi in (False, True):
            pool = list(b"CcNnOo()=#12345%+-H[") + ([0xC3, 0xA9, 0xFF] if hi else [])
            strs.append(bytes(rng.choice(pool, size=n).astype(np.uint8)))
            strs.append(b"CCO")
    strs.append(b"C" * 3000)        # one unique code, count 2997
    strs.append(b"c1ccccc1" * 400)  # few unique codes, long runs
    want, buf, off = _cpu(strs)
    _same(_gpu(buf, off), want)


def test_gpu_compiler_degenerate_inputs(native):
    want, buf, off = _cpu([b"", b"C", b"CC", b"CCC", b" CCCC", b"\nCCCC"])
    got = _gpu(buf, off)
    assert got[0].shape == (6, 0)
    _same(got, want)
    got = _gpu(b"", np.zeros(1, np.int64))
    assert got[0].shape == (0, 0) and got[2].shape == (0,)
    from siml_gb300 import compiler as PC
    with pytest.raises(ValueError):
        PC.compile_buffer_gpu(b"CCCC", np.array([0, 3, 2], np.int64))   # decreasing offsets
    with pytest.raises(ValueError):
        PC.compile_buffer_gpu(b"CC", np.array([0, 4], np.int64))        # buffer too short


def test_gpu_compiled_set_gives_the_same_rows(native):
    """A database compiled on the GPU and set from device tensors gives the
    same Tanimoto rows as the host-compiled set."""
    import torch
    from siml_gb300 import GPULingo
    from siml_gb300 import synthetic as S
    from siml_gb300 import compiler as PC
    buf, off = S.smiles_buffer(S.SEED_DB_1M, S.LOGNORMAL_45, 20000)
    cpu = PC.compile_buffer(buf, off)
    gpu = PC.compile_buffer_gpu(buf, off)
    _same(tuple(t.cpu().numpy() for t in gpu), cpu)
    q = S.smiles_set(S.SEED_DB_1M, S.LOGNORMAL_45, 64, first=20000)
    a, b = GPULingo(0), GPULingo(0)
    a.set_refsmiles(*q)
    b.set_refsmiles(*q)
    a.set_qsmiles(*cpu)
    b.set_qsmiles(*gpu)
    torch.cuda.synchronize()
    assert np.array_equal(a.getMultipleRows(0, 64).view(np.uint32), b.getMultipleRows(0, 64).view(np.uint32))


def test_gpu_compiler_is_ordered_after_torch_default_stream(native):
    """The compiler runs on torch's current stream.  With torch's default
    stream (handle 0, the legacy default stream) busy for ~0.1 s when the
    call is made, the byte upload and the output arrays' zero fill queue
    behind that work; the compile must wait for them rather than run on a
    stream of its own."""
    import torch
    from siml_gb300 import synthetic as S
    buf, off = S.smiles_buffer(S.SEED_SERVING, S.UNIFORM_20_90, 50000)
    want, _, _ = _cpu([buf[off[i]:off[i + 1]] for i in range(len(off) - 1)])
    assert torch.cuda.current_stream().cuda_stream == 0
    for _ in range(2):
        torch.cuda._sleep(200_000_000)   # bounded spin on the default stream
        got = _gpu(buf, off)
        _same(got, want)


def test_gpu_compiler_two_pass_entries_and_scatter_width(native):
    """The two-pass C entries (width, then fill) give what the one-pass
    staging path of compile_buffer_gpu gives, and the scatter refuses a
    width below the widest string."""
    import torch
    from siml_gb300 import _native as N, synthetic as S
    from siml_gb300.compiler import compile_buffer_gpu
    buf, off = S.smiles_buffer(S.SEED_RAGGED, S.BIMODAL_35_110, 5000)
    one = compile_buffer_gpu(buf, off)
    dev = one[0].device
    text = torch.from_numpy(np.frombuffer(buf, dtype=np.uint8).copy()).to(dev)
    off_d = torch.from_numpy(off).to(dev)
    L = N.lib()
    from siml_gb300.utilities import _shared
    e = _shared(0)
    with e.lock:
        h = e.h
        N.check(L.siml_set_stream(h, N.stream_arg(torch.cuda.current_stream())), "siml_set_stream")
        w = L.siml_compile_width_gpu(h, text.data_ptr(), off_d.data_ptr(), len(off) - 1)
        assert w == one[0].shape[1]
        n = len(off) - 1
        got = [torch.zeros((n, w), dtype=torch.int32, device=dev) for _ in range(2)]
        got += [torch.zeros(n, dtype=torch.int32, device=dev) for _ in range(2)]
        N.check(L.siml_compile_smiles_gpu(h, text.data_ptr(), off_d.data_ptr(), n, *(t.data_ptr() for t in got), w))
        # the scatter with a width one short of the widest string
        sc = torch.empty(int(off[-1]), dtype=torch.int32, device=dev)
        sn = torch.empty_like(sc)
        ln = torch.empty(n, dtype=torch.int32, device=dev)
        mg = torch.empty(n, dtype=torch.int32, device=dev)
        assert L.siml_compile_stage_gpu(h, text.data_ptr(), off_d.data_ptr(), n, sc.data_ptr(), sn.data_ptr(),
                                        ln.data_ptr(), mg.data_ptr()) == w
        narrow = torch.empty((n, w - 1), dtype=torch.int32, device=dev)
        rc = L.siml_compile_scatter_gpu(h, off_d.data_ptr(), n, sc.data_ptr(), sn.data_ptr(), ln.data_ptr(),
                                        narrow.data_ptr(), narrow.clone().data_ptr(), w - 1)
        assert rc == N.SIML_ERR_INVALID
    for a, b in zip(got, one):
        assert torch.equal(a, b)
