"""The allocation-free pairwise entry point gives the same scores as the regular one.

Some callers of this library cannot call ``cudaMalloc`` / ``cudaFree``: a host application whose own allocator
already holds the device memory, or a latency-bound loop that cannot afford the device-wide synchronisation of
``cudaFree``. ``szs_gb300_score_pairwise_noalloc_u64tape`` serves them from a fixed device array inside the library.
These tests call it through the C-ABI on device-resident tapes and compare it, score for score, with
``szs_*_pairwise_u64tape`` on two calls in a row (the array keeps the previous call's contents), then check that it
refuses what its fixed scratch cannot hold. The file name makes pytest collect it after every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DNA = np.frombuffer(b"ACGT", dtype=np.uint8)
PROTEIN = np.frombuffer(b"ARNDCQEGHILKMFPSTWYV", dtype=np.uint8)


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    import stringzillas_gb300 as szs
    from stringzillas_gb300 import _native
    if "cuda" not in szs.__capabilities__ or not torch.cuda.is_available():
        pytest.fail("no CUDA device visible: GPU tests must run on a GPU")
    return torch, szs, _native


def device_tape(torch, native, strings):
    data = np.frombuffer(b"".join(strings), dtype=np.uint8) if strings else np.zeros(0, dtype=np.uint8)
    offsets = np.zeros(len(strings) + 1, dtype=np.int64)
    offsets[1:] = np.cumsum([len(s) for s in strings])
    d = torch.from_numpy(data.copy()).cuda() if data.size else torch.zeros(1, dtype=torch.uint8, device="cuda")
    o = torch.from_numpy(offsets).cuda()
    return native.U64Tape(d.data_ptr(), o.data_ptr(), len(strings)), (d, o)


def strings_of(rng, count, lengths, alphabet):
    return [bytes(rng.choice(alphabet, size=int(rng.integers(*lengths)))) for _ in range(count)]


def workload(rng, alphabet, count):
    """Short pairs, multi-strip pairs below the 2,048-byte row limit, and one-strip pairs with a long partner."""
    first = strings_of(rng, count, (0, 200), alphabet) + strings_of(rng, count, (257, 2047), alphabet) + \
        strings_of(rng, count, (1, 256), alphabet)
    second = strings_of(rng, count, (0, 200), alphabet) + strings_of(rng, count, (257, 2047), alphabet) + \
        strings_of(rng, count, (2048, 6000), alphabet)
    return first, second


def engines(szs):
    rng = np.random.default_rng(2)
    b2c = np.zeros(256, dtype=np.uint8)
    b2c[PROTEIN] = np.arange(1, 21, dtype=np.uint8)
    table = np.zeros((32, 32), dtype=np.int8)
    table[1:21, 1:21] = rng.integers(-4, 8, size=(20, 20))
    dna_b2c = np.zeros(256, dtype=np.uint8)
    dna_b2c[DNA] = [1, 2, 3, 4]
    dna = np.zeros((32, 32), dtype=np.int8)
    dna[1:5, 1:5] = -3
    np.fill_diagonal(dna[1:5, 1:5], 2)
    return [
        ("nw-affine", szs.NeedlemanWunschScores(b2c, table, open=-11, extend=-1), PROTEIN),
        ("sw-linear", szs.SmithWatermanScores(dna_b2c, dna, open=-4, extend=-4), DNA),
        ("lev-affine", szs.LevenshteinDistances(0, 4, 5, 2), DNA),
        ("lev-unit", szs.LevenshteinDistances(), DNA),
        ("nw-linear", szs.NeedlemanWunschScores(b2c, table, open=-5, extend=-5), PROTEIN),
        ("sw-affine", szs.SmithWatermanScores(dna_b2c, dna, open=-5, extend=-2), DNA),
    ]


ENGINE_NAMES = ["nw-affine", "sw-linear", "lev-affine", "lev-unit", "nw-linear", "sw-affine"]


def regular(env, engine, a, b, count):
    torch, szs, native = env
    out = torch.empty(count, dtype=torch.int64, device="cuda")
    err = ctypes.c_char_p()
    status = getattr(native.lib, f"szs_{engine._algo}_pairwise_u64tape")(
        engine.handle, szs._scope_handle(None), ctypes.byref(a), ctypes.byref(b), ctypes.c_void_p(out.data_ptr()),
        ctypes.byref(err))
    assert status == 0, err.value
    return out.cpu().numpy()


def allocation_free(env, engine, a, b, out):
    torch, szs, native = env
    err = ctypes.c_char_p()
    status = native.lib.szs_gb300_score_pairwise_noalloc_u64tape(
        engine.handle, szs._scope_handle(None), ctypes.byref(a), ctypes.byref(b), ctypes.c_void_p(out), ctypes.byref(err))
    return status, err.value


@pytest.mark.parametrize("index", range(len(ENGINE_NAMES)), ids=ENGINE_NAMES)
def test_matches_regular_entry_point_twice(env, index):
    """Every kernel instance (kind x linear / affine), with empty sides on either string, on two calls in a row."""
    torch, szs, native = env
    name, engine, alphabet = engines(szs)[index]
    rng = np.random.default_rng(100 + index)
    for call, count in enumerate((40, 23)):  # two calls in a row, different shapes
        first, second = workload(rng, alphabet, count)
        first += [b"", b"", bytes(rng.choice(alphabet, size=300))]
        second += [bytes(rng.choice(alphabet, size=7)), b"", b""]
        a, keep_a = device_tape(torch, native, first)
        b, keep_b = device_tape(torch, native, second)
        want = regular(env, engine, a, b, len(first))
        out = torch.full((len(first),), -777, dtype=torch.int64, device="cuda")
        status, message = allocation_free(env, engine, a, b, out.data_ptr())
        assert status == 0, f"{name} call {call}: {message}"
        got = out.cpu().numpy()
        bad = np.flatnonzero(got != want)
        assert bad.size == 0, f"{name} call {call}: {bad.size} differ, first {bad[:5]}: {got[bad[:5]]} vs {want[bad[:5]]}"


def test_rejects_what_the_fixed_scratch_cannot_hold(env):
    torch, szs, native = env
    _, engine, alphabet = engines(szs)[0]
    rng = np.random.default_rng(9)
    first = [bytes(rng.choice(alphabet, size=300)), bytes(rng.choice(alphabet, size=50))]
    second = [bytes(rng.choice(alphabet, size=3000)), bytes(rng.choice(alphabet, size=60))]
    a, keep_a = device_tape(torch, native, first)
    b, keep_b = device_tape(torch, native, second)
    out = torch.zeros(2, dtype=torch.int64, device="cuda")
    out.fill_(-777)
    status, message = allocation_free(env, engine, a, b, out.data_ptr())
    assert status == native.OVERFLOW_RISK and b"2,048" in message
    # The rejected pair's slot reads 0, the pair that fits is still scored, and the next call starts from a cleared
    # error word.
    assert int(out[0]) == 0
    assert int(out[1]) == int(regular(env, engine, a, b, 2)[1])
    first, second = first[1:], second[1:]
    a, keep_a = device_tape(torch, native, first)
    b, keep_b = device_tape(torch, native, second)
    status, message = allocation_free(env, engine, a, b, out.data_ptr())
    assert status == 0, message


def test_rejects_host_memory(env):
    torch, szs, native = env
    _, engine, _ = engines(szs)[3]
    data = np.frombuffer(b"ACGTACGT", dtype=np.uint8)
    offsets = np.array([0, 4, 8], dtype=np.uint64)
    a = native.U64Tape(data.ctypes.data, offsets.ctypes.data, 2)
    out = np.zeros(2, dtype=np.int64)
    status, _ = allocation_free(env, engine, a, a, out.ctypes.data)
    assert status == native.DEVICE_MEMORY_MISMATCH


def test_keeps_the_callers_current_device(env):
    torch, szs, native = env
    _, engine, alphabet = engines(szs)[3]
    a, keep = device_tape(torch, native, [b"ACGT", b"GATTACA"])
    out = torch.zeros(2, dtype=torch.int64, device="cuda")
    before = torch.cuda.current_device()
    status, message = allocation_free(env, engine, a, a, out.data_ptr())
    assert status == 0, message
    assert torch.cuda.current_device() == before
    assert out.cpu().tolist() == [0, 0]


def test_rejects_another_gpus_memory(env):
    """Tapes on GPU 1 with a scope on GPU 0 would be read without a peer mapping: refused before any launch."""
    torch, szs, native = env
    if torch.cuda.device_count() < 2:
        pytest.skip("needs two visible GPUs")
    _, engine, _ = engines(szs)[3]
    data = torch.frombuffer(bytearray(b"ACGTACGT"), dtype=torch.uint8).to("cuda:1")
    offsets = torch.tensor([0, 4, 8], dtype=torch.int64, device="cuda:1")
    a = native.U64Tape(data.data_ptr(), offsets.data_ptr(), 2)
    out = torch.zeros(2, dtype=torch.int64, device="cuda:1")
    status, _ = allocation_free(env, engine, a, a, out.data_ptr())
    assert status == native.DEVICE_MEMORY_MISMATCH
