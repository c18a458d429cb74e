"""The three scorer ABI forms of the reference, called directly through ctypes, against the oracle.

The reference declares each scorer three times (include/stringzillas/stringzillas.h:184-218 for Levenshtein,
:325-359 Needleman-Wunsch, :395-429 Smith-Waterman): over ``sz_sequence_t`` (strings reached through ``get_start`` /
``get_length`` callbacks), over Arrow-like tapes with 32-bit offsets and over tapes with 64-bit offsets. Each form
fills a ``queries x candidates`` matrix with a row stride in elements, or the symmetric matrix when ``candidates`` is
NULL. These tests call every form of every scorer in cross, symmetric and strided layouts, with host and
device-resident tapes, plus the pairwise extension over 32-bit tapes, and compare with the oracle bit for bit.
"""
import ctypes
import zlib

import numpy as np
import pytest

from conftest import tape
from oracle import oracle

pytestmark = pytest.mark.gpu

DNA = np.frombuffer(b"ACGT", dtype=np.uint8)
PROTEIN = np.frombuffer(b"ARNDCQEGHILKMFPSTWYV", dtype=np.uint8)


@pytest.fixture(scope="module")
def env():
    import stringzillas_gb300 as szs
    from stringzillas_gb300 import _native
    if "cuda" not in szs.__capabilities__:
        pytest.fail("no CUDA device visible: GPU tests must run on a GPU")
    return szs, _native


def tables(rng, family):
    b2c = np.zeros(256, dtype=np.uint8)
    table = np.zeros((32, 32), dtype=np.int8)
    if family == "nw":
        b2c[PROTEIN] = np.arange(1, 21, dtype=np.uint8)
        table[1:21, 1:21] = rng.integers(-4, 8, size=(20, 20))  # asymmetric on purpose
    else:
        b2c[DNA] = [1, 2, 3, 4]
        table[1:5, 1:5] = -3
        np.fill_diagonal(table[1:5, 1:5], 2)
    return b2c, table


ENGINES = [("lev-unit", "lev", (0, 1, 1, 1)), ("lev-affine", "lev", (0, 4, 5, 2)),
           ("nw-affine", "nw", (-11, -1)), ("nw-linear", "nw", (-4, -4)),
           ("sw-affine", "sw", (-5, -2)), ("sw-linear", "sw", (-3, -3))]


def make(szs, rng, family, costs):
    if family == "lev":
        return szs.LevenshteinDistances(*costs), oracle.levenshtein_costs(*costs), DNA
    b2c, table = tables(rng, family)
    kind = oracle.NEEDLEMAN_WUNSCH if family == "nw" else oracle.SMITH_WATERMAN
    cls = szs.NeedlemanWunschScores if family == "nw" else szs.SmithWatermanScores
    return (cls(b2c, table, open=costs[0], extend=costs[1]), oracle.alignment_costs(kind, b2c, table, *costs),
            PROTEIN if family == "nw" else DNA)


def corpus(rng, count, alphabet):
    """Empty, one-character, short and multi-strip strings, plus a pair long enough for a band."""
    lengths = [0, 1, 2] + [int(x) for x in rng.integers(0, 400, size=count - 4)] + [2600]
    return [bytes(rng.choice(alphabet, size=n)) for n in lengths]


class SequenceOf:
    """An ``sz_sequence_t`` over a list of bytes: the callbacks hand out pointers into one host buffer."""

    def __init__(self, native, strings):
        self.data, self.offsets = tape(strings)
        self.data = np.ascontiguousarray(self.data) if self.data.size else np.zeros(1, dtype=np.uint8)
        base = self.data.ctypes.data
        offsets = self.offsets
        self._start = native.SequenceStart(lambda handle, i: base + int(offsets[i]))
        self._length = native.SequenceLength(lambda handle, i: int(offsets[i + 1] - offsets[i]))
        self.struct = native.Sequence(None, len(strings), self._start, self._length)


def host_u32(native, strings):
    data, offsets = tape(strings)
    data = data.copy() if data.size else np.zeros(1, dtype=np.uint8)
    offsets = offsets.astype(np.uint32)
    return native.U32Tape(data.ctypes.data, offsets.ctypes.data, len(strings)), (data, offsets)


def device_u32(native, strings):
    import torch
    data, offsets = tape(strings)
    d = torch.from_numpy(data.copy()).cuda() if data.size else torch.zeros(1, dtype=torch.uint8, device="cuda")
    o = torch.from_numpy(offsets.astype(np.int32)).cuda()
    return native.U32Tape(d.data_ptr(), o.data_ptr(), len(strings)), (d, o)


def call_matrix(szs, native, engine, suffix, queries, candidates, rows, cols, stride):
    """Calls ``szs_<algo><suffix>`` into a host matrix of ``rows x stride`` pre-filled with a sentinel; returns the
    whole matrix (the padding columns must stay untouched)."""
    out = np.full((rows, stride), -777, dtype=np.int64)
    err = ctypes.c_char_p()
    fn = getattr(native.lib, f"szs_{engine._algo}{suffix}")
    status = fn(engine.handle, szs._scope_handle(None), ctypes.byref(queries),
                None if candidates is None else ctypes.byref(candidates), ctypes.c_void_p(out.ctypes.data), stride,
                ctypes.byref(err))
    assert status == 0, err.value
    return out


@pytest.mark.parametrize("name,family,costs", ENGINES, ids=[e[0] for e in ENGINES])
def test_sequence_callback_form(env, port, name, family, costs):
    """``szs_<algo>(engine, device, sz_sequence_t const *, sz_sequence_t const *, results, stride, error)``."""
    szs, native = env
    rng = np.random.default_rng(zlib.crc32(repr(("seq", name)).encode()))
    engine, oracle_costs, alphabet = make(szs, rng, family, costs)
    queries, candidates = corpus(rng, 11, alphabet), corpus(rng, 14, alphabet)
    q, c = SequenceOf(native, queries), SequenceOf(native, candidates)
    want = port.cross(oracle_costs, tape(queries), tape(candidates))
    for stride in (len(candidates), len(candidates) + 5):
        got = call_matrix(szs, native, engine, "", q.struct, c.struct, len(queries), len(candidates), stride)
        np.testing.assert_array_equal(got[:, :len(candidates)], want)
        assert (got[:, len(candidates):] == -777).all()
    want_sym = port.cross(oracle_costs, tape(queries))
    got = call_matrix(szs, native, engine, "", q.struct, None, len(queries), len(queries), len(queries) + 3)
    np.testing.assert_array_equal(got[:, :len(queries)], want_sym)
    assert (got[:, len(queries):] == -777).all()


@pytest.mark.parametrize("resident", ["host", "device"])
@pytest.mark.parametrize("name,family,costs", ENGINES, ids=[e[0] for e in ENGINES])
def test_u32tape_form(env, port, name, family, costs, resident):
    """``szs_<algo>_u32tape`` cross (unit and wider stride) and symmetric, host and device-resident tapes."""
    szs, native = env
    rng = np.random.default_rng(zlib.crc32(repr(("u32", name, resident)).encode()))
    engine, oracle_costs, alphabet = make(szs, rng, family, costs)
    queries, candidates = corpus(rng, 13, alphabet), corpus(rng, 9, alphabet)
    make_tape = host_u32 if resident == "host" else device_u32
    (q, keep_q), (c, keep_c) = make_tape(native, queries), make_tape(native, candidates)
    want = port.cross(oracle_costs, tape(queries), tape(candidates))
    for stride in (len(candidates), len(candidates) + 7):
        got = call_matrix(szs, native, engine, "_u32tape", q, c, len(queries), len(candidates), stride)
        np.testing.assert_array_equal(got[:, :len(candidates)], want)
        assert (got[:, len(candidates):] == -777).all()
    got = call_matrix(szs, native, engine, "_u32tape", q, None, len(queries), len(queries), len(queries))
    np.testing.assert_array_equal(got, port.cross(oracle_costs, tape(queries)))


@pytest.mark.parametrize("name,family,costs", ENGINES, ids=[e[0] for e in ENGINES])
def test_u32tape_sliced_offsets(env, port, name, family, costs):
    """32-bit tapes whose first offset is not zero (a slice of a larger tape), host-resident."""
    szs, native = env
    rng = np.random.default_rng(zlib.crc32(repr(("slice", name)).encode()))
    engine, oracle_costs, alphabet = make(szs, rng, family, costs)
    strings = corpus(rng, 20, alphabet)
    data, offsets = tape(strings)
    offsets = offsets.astype(np.uint32)
    lo, hi = 5, 17
    sub = native.U32Tape(data.ctypes.data, offsets[lo:].ctypes.data, hi - lo)
    got = call_matrix(szs, native, engine, "_u32tape", sub, None, hi - lo, hi - lo, hi - lo)
    np.testing.assert_array_equal(got, port.cross(oracle_costs, tape(strings[lo:hi])))


@pytest.mark.parametrize("name,family,costs", ENGINES, ids=[e[0] for e in ENGINES])
def test_pairwise_u32tape(env, port, name, family, costs):
    """The pairwise extension over 32-bit tapes, host and device-resident."""
    szs, native = env
    rng = np.random.default_rng(zlib.crc32(repr(("pw32", name)).encode()))
    engine, oracle_costs, alphabet = make(szs, rng, family, costs)
    first, second = corpus(rng, 60, alphabet), corpus(rng, 60, alphabet)
    want = port.pairs(oracle_costs, tape(first), tape(second))
    for make_tape in (host_u32, device_u32):
        (a, keep_a), (b, keep_b) = make_tape(native, first), make_tape(native, second)
        out = np.full(len(first), -777, dtype=np.int64)
        err = ctypes.c_char_p()
        status = getattr(native.lib, f"szs_{engine._algo}_pairwise_u32tape")(
            engine.handle, szs._scope_handle(None), ctypes.byref(a), ctypes.byref(b),
            ctypes.c_void_p(out.ctypes.data), ctypes.byref(err))
        assert status == 0, err.value
        np.testing.assert_array_equal(out, want)


def test_arrow_tapes_used_in_place(env, port):
    """Arrow string arrays (32-bit offsets) and large-string arrays (64-bit) reach the engine without copies or
    widening, sliced or whole; where pyarrow is absent, numpy buffers laid out the same way stand in for them."""
    szs, native = env
    rng = np.random.default_rng(31)
    strings = [bytes(rng.choice(DNA, size=int(n))) for n in rng.integers(0, 300, size=120)]
    others = [bytes(rng.choice(DNA, size=int(n))) for n in rng.integers(0, 300, size=120)]
    try:
        import pyarrow as pa
        a32 = szs.Strs(pa.array(strings, type=pa.binary()))
        b32 = szs.Strs(pa.array(others, type=pa.binary()))
        a64 = szs.Strs(pa.array(strings, type=pa.large_binary()))
        sliced = szs.Strs(pa.array(strings, type=pa.binary()).slice(7, 50))
    except ImportError:
        def tape32(items):
            data, offsets = tape(items)
            return szs.Strs.from_buffers(data.copy(), offsets.astype(np.uint32))
        a32, b32 = tape32(strings), tape32(others)
        a64 = szs.Strs.from_buffers(*tape(strings))
        sliced = tape32(strings)[7:57]
    assert a32.tape()[1] == 32 and a64.tape()[1] == 64
    engine = szs.LevenshteinDistances(0, 2, 3, 1)
    costs = oracle.levenshtein_costs(0, 2, 3, 1)
    want = port.pairs(costs, tape(strings), tape(others))
    np.testing.assert_array_equal(engine.pairwise(a32, b32).astype(np.int64), want)
    np.testing.assert_array_equal(engine.pairwise(a64, b32).astype(np.int64), want)  # mixed widths
    np.testing.assert_array_equal(engine(sliced).astype(np.int64), port.cross(costs, tape(strings[7:57])))
    np.testing.assert_array_equal(engine(a32[:20], b32[5:30]).astype(np.int64),
                                  port.cross(costs, tape(strings[:20]), tape(others[5:30])))
