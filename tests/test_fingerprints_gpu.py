"""Min-Hash fingerprints on the GPU against the reference library's own outputs (golden fixtures) and the oracle's
integer restatement (c/stringzillas/fingerprints.cuh:27-222, include/stringzillas/fingerprints/serial.hpp)."""
import ctypes
import os

import numpy as np
import pytest

from oracle import oracle
from stringzillas_gb300 import workloads as w

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "golden.npz")


@pytest.fixture(scope="module")
def szs():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    import stringzillas_gb300
    return stringzillas_gb300


def _golden_cases():
    with np.load(GOLDEN) as data:
        return {str(name): {k.split("__", 1)[1]: data[k] for k in data.files if k.startswith(f"fp_{name}__")}
                for name in data["__fingerprints__"]}


GOLDEN_CASES = _golden_cases()


def _strs(szs, data, offsets):
    return szs.Strs.from_buffers(np.ascontiguousarray(data, dtype=np.uint8),
                                 np.ascontiguousarray(offsets, dtype=np.uint64))


@pytest.mark.parametrize("name", sorted(GOLDEN_CASES))
def test_golden_fingerprints_match_reference(szs, name):
    case = GOLDEN_CASES[name]
    dimensions, seed = (int(x) for x in case["params"])
    widths = case["widths"].astype(np.uint64) if len(case["widths"]) else None
    engine = szs.Fingerprints(ndim=dimensions, window_widths=widths, seed=seed)
    hashes, counts = engine(_strs(szs, case["data"], case["offsets"]))
    np.testing.assert_array_equal(hashes, case["hashes"])
    np.testing.assert_array_equal(counts, case["counts"])


def _random_texts(rng, count, low, high, alphabet):
    alphabet = np.frombuffer(alphabet, dtype=np.uint8)
    lengths = rng.integers(low, high + 1, size=count)
    offsets = np.zeros(count + 1, dtype=np.uint64)
    offsets[1:] = np.cumsum(lengths)
    return rng.choice(alphabet, size=int(offsets[-1])).astype(np.uint8), offsets


@pytest.mark.parametrize("dimensions,widths,seed", [
    (1, [3], 0),
    (31, [1, 2, 200], 5),
    (33, None, 17),
    (100, [4, 9], 2**63 + 11),
    (512, None, 42),             # sliced: 8 widths x 64
    (256, [5, 31], 7),           # sliced: 2 widths x 128
    (192, [5, 31], 7),           # not sliced: 192 / 2 = 96 is no multiple of 64
])
def test_random_texts_match_oracle(szs, dimensions, widths, seed):
    rng = np.random.default_rng(dimensions + seed % 1000)
    data, offsets = _random_texts(rng, 300, 0, 400, b"ACGTacgt\x00\xff NXYZ")
    engine = szs.Fingerprints(dimensions, None if widths is None else np.array(widths, dtype=np.uint64), seed=seed)
    hashes, counts = engine(_strs(szs, data, offsets))
    want_h, want_c = oracle.fingerprints(dimensions, (data, offsets), widths, seed)
    np.testing.assert_array_equal(hashes, want_h)
    np.testing.assert_array_equal(counts, want_c)


def test_u32_and_u64_tapes_and_device_outputs_agree(szs):
    import torch
    rng = np.random.default_rng(3)
    data, offsets = _random_texts(rng, 500, 0, 200, b"abcdefghij")
    engine = szs.Fingerprints(64, seed=9)
    base_h, base_c = engine(_strs(szs, data, offsets))
    narrow = szs.Strs.from_buffers(data, offsets.astype(np.uint32))
    h32, c32 = engine(narrow)
    np.testing.assert_array_equal(h32, base_h)
    np.testing.assert_array_equal(c32, base_c)
    # Device-resident texts and outputs, rows padded to a wider stride.
    device_texts = szs.to_device(_strs(szs, data, offsets))
    out_h = torch.zeros((500, 80), dtype=torch.int32, device="cuda")
    out_c = torch.zeros((500, 80), dtype=torch.int32, device="cuda")
    engine(device_texts, out=(out_h, out_c))
    np.testing.assert_array_equal(out_h[:, :64].cpu().numpy().view(np.uint32), base_h)
    np.testing.assert_array_equal(out_c[:, :64].cpu().numpy().view(np.uint32), base_c)
    assert int(out_h[:, 64:].abs().sum()) == 0 and int(out_c[:, 64:].abs().sum()) == 0
    # Host outputs with padded rows.
    wide_h = np.zeros((500, 70), dtype=np.uint32)
    wide_c = np.zeros((500, 70), dtype=np.uint32)
    engine(_strs(szs, data, offsets), out=(wide_h, wide_c))
    np.testing.assert_array_equal(wide_h[:, :64], base_h)
    np.testing.assert_array_equal(wide_c[:, :64], base_c)


def test_edge_texts(szs):
    texts = [b"", b"a", b"ab", b"abc", b"\x00" * 40, b"\xff" * 40, bytes(range(256)), b"x" * 5000]
    offsets = np.zeros(len(texts) + 1, dtype=np.uint64)
    offsets[1:] = np.cumsum([len(t) for t in texts])
    data = np.frombuffer(b"".join(texts), dtype=np.uint8).copy()
    engine = szs.Fingerprints(40, np.array([1, 2, 3, 4, 31], dtype=np.uint64), seed=1)
    hashes, counts = engine(_strs(szs, data, offsets))
    want_h, want_c = oracle.fingerprints(40, (data, offsets), [1, 2, 3, 4, 31], 1)
    np.testing.assert_array_equal(hashes, want_h)
    np.testing.assert_array_equal(counts, want_c)
    assert (hashes[0] == 0xFFFFFFFF).all() and (counts[0] == 0).all()
    # A run of one byte has a single window value: every window is the minimum.
    run = counts[7].reshape(-1)
    widths = np.array([1, 2, 3, 4, 31] * 8)
    np.testing.assert_array_equal(run, 5000 - widths + 1)
    empty_h, empty_c = engine([])
    assert empty_h.shape == (0, 40) and empty_c.shape == (0, 40)


def test_utf8_entry_points_forward_to_bytes(szs):
    from stringzillas_gb300 import _native
    lib = _native.lib
    rng = np.random.default_rng(4)
    data, offsets = _random_texts(rng, 50, 0, 100, "αβγabc".encode())
    err = ctypes.c_char_p()
    handles = []
    outputs = []
    for init, call, free in ((lib.szs_fingerprints_init, lib.szs_fingerprints_u64tape, lib.szs_fingerprints_free),
                             (lib.szs_fingerprints_utf8_init, lib.szs_fingerprints_utf8_u64tape,
                              lib.szs_fingerprints_utf8_free)):
        handle = ctypes.c_void_p()
        assert init(96, 256, None, 0, 3, None, 0, ctypes.byref(handle), ctypes.byref(err)) == _native.SUCCESS
        tape = _native.U64Tape(data.ctypes.data, offsets.ctypes.data, len(offsets) - 1)
        h = np.zeros((50, 96), np.uint32)
        c = np.zeros((50, 96), np.uint32)
        assert call(handle, None, ctypes.byref(tape), h.ctypes.data, 384, c.ctypes.data, 384,
                    ctypes.byref(err)) == _native.SUCCESS
        outputs.append((h, c))
        handles.append((handle, free))
    np.testing.assert_array_equal(outputs[0][0], outputs[1][0])
    np.testing.assert_array_equal(outputs[0][1], outputs[1][1])
    for handle, free in handles:
        free(handle)


def test_large_corpus_sampled_rows(szs):
    """A full-size corpus (reads of the 2 KiB class); a seeded sample of rows checked against the oracle."""
    (data, offsets), _ = w.levenshtein_reads(20000, 1500, 2500, 0.0, 0.0, seed=12)
    engine = szs.Fingerprints(128, seed=0)
    hashes, counts = engine(_strs(szs, data, offsets))
    rng = np.random.default_rng(0)
    picks = np.sort(rng.choice(len(offsets) - 1, size=40, replace=False))
    sub_offsets = np.concatenate([[0], np.cumsum(offsets[picks + 1] - offsets[picks])]).astype(np.uint64)
    sub_data = np.concatenate([data[offsets[i]:offsets[i + 1]] for i in picks])
    want_h, want_c = oracle.fingerprints(128, (sub_data, sub_offsets), None, 0)
    np.testing.assert_array_equal(hashes[picks], want_h)
    np.testing.assert_array_equal(counts[picks], want_c)
    assert (counts >= 1).all()


@pytest.mark.parametrize("ndim", [1, 7, 64, 1024])
def test_reference_test_shapes(szs, ndim):
    """The reference's own checks (test/fingerprints.py): shapes and dtypes, identical texts agree, different texts
    differ, degenerate texts are deterministic; values from the oracle."""
    engine = szs.Fingerprints(ndim=ndim)
    hashes, counts = engine(szs.Strs([]))
    assert hashes.shape == (0, ndim) and counts.shape == (0, ndim)
    assert hashes.dtype == np.uint32 and counts.dtype == np.uint32
    texts = ["hello", "world", "hello", "a", "a" * 40, "b", "", "a" * 5]
    hashes, counts = engine(szs.Strs(texts))
    assert hashes.shape == (len(texts), ndim)
    np.testing.assert_array_equal(hashes[0], hashes[2])
    np.testing.assert_array_equal(counts[0], counts[2])
    assert ndim < 7 or not np.array_equal(hashes[0], hashes[1])
    data = np.frombuffer("".join(texts).encode(), dtype=np.uint8).copy()
    offsets = np.concatenate([[0], np.cumsum([len(t) for t in texts])]).astype(np.uint64)
    want_h, want_c = oracle.fingerprints(ndim, (data, offsets))
    np.testing.assert_array_equal(hashes, want_h)
    np.testing.assert_array_equal(counts, want_c)
    again_h, again_c = engine(szs.Strs(texts))
    np.testing.assert_array_equal(again_h, hashes)
    np.testing.assert_array_equal(again_c, counts)
