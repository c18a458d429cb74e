"""GPU parity: every route of the engine against the oracle, bit for bit, through the C-ABI."""
import numpy as np
import pytest

from conftest import tape
from oracle import oracle

pytestmark = pytest.mark.gpu

DNA = np.frombuffer(b"ACGT", dtype=np.uint8)
PROTEIN = np.frombuffer(b"ARNDCQEGHILKMFPSTWYV", dtype=np.uint8)


@pytest.fixture(scope="module")
def szs():
    import stringzillas_gb300
    if "cuda" not in stringzillas_gb300.__capabilities__:
        pytest.fail("no CUDA device visible: GPU tests must run on a GPU")
    return stringzillas_gb300


def zlib_seed(*parts):
    import zlib
    return zlib.crc32(repr(parts).encode())


def random_strings(rng, count, low, high, alphabet):
    return [bytes(rng.choice(alphabet, size=int(rng.integers(low, high + 1)))) for _ in range(count)]


def dna_tables():
    b2c = np.zeros(256, dtype=np.uint8)
    b2c[DNA] = [1, 2, 3, 4]
    table = np.zeros((32, 32), dtype=np.int8)
    table[1:5, 1:5] = -3
    np.fill_diagonal(table[1:5, 1:5], 2)
    return b2c, table


def protein_tables(rng, symmetric=True):
    b2c = np.zeros(256, dtype=np.uint8)
    b2c[PROTEIN] = np.arange(1, 21, dtype=np.uint8)
    table = np.zeros((32, 32), dtype=np.int8)
    core = rng.integers(-4, 4, size=(20, 20))
    if symmetric:
        core = np.triu(core) + np.triu(core, 1).T
        np.fill_diagonal(core, rng.integers(4, 12, size=20))
    table[1:21, 1:21] = core
    return b2c, table


ENGINES = [
    ("lev-unit", "lev", (0, 1, 1, 1)),
    ("lev-linear", "lev", (0, 3, 2, 2)),
    ("lev-affine", "lev", (0, 4, 5, 2)),
    ("lev-match-cost", "lev", (1, 3, 4, 1)),
    ("nw-linear", "nw", (-5, -5)),
    ("nw-affine", "nw", (-11, -1)),
    ("sw-linear", "sw", (-5, -5)),
    ("sw-affine", "sw", (-5, -2)),
    ("nw-positive-gaps", "nw", (3, 1)),
]


def make_engine(szs, family, costs, b2c, table):
    if family == "lev":
        return szs.LevenshteinDistances(*costs), oracle.levenshtein_costs(*costs)
    kind = oracle.NEEDLEMAN_WUNSCH if family == "nw" else oracle.SMITH_WATERMAN
    cls = szs.NeedlemanWunschScores if family == "nw" else szs.SmithWatermanScores
    return cls(b2c, table, open=costs[0], extend=costs[1]), oracle.alignment_costs(kind, b2c, table, *costs)


@pytest.mark.parametrize("family,costs", [("lev", (0, 2, 3, 1)), ("lev", (0, 3, 2, 2)), ("nw", (-11, -1)),
                                          ("nw", (-4, -4)), ("sw", (-5, -2)), ("sw", (-3, -3))])
def test_forced_64bit_cells(szs, port, family, costs):
    """The 64-bit wavefront is the route the reach bound takes for spans near 2^31 / magnitude (pairs of millions of
    characters); the tuning forces it onto ordinary pairs: every cost family, empty sides, multi-strip and long pairs
    (no band: 64-bit pairs stay on the wavefront), cross products, both schedules, all equal to the oracle."""
    rng = np.random.default_rng(zlib_seed(f"{family}{costs}"))
    alphabet = PROTEIN if family == "nw" else DNA
    b2c, table = protein_tables(rng) if family == "nw" else dna_tables()
    lengths = [(int(rng.integers(0, 300)), int(rng.integers(0, 300))) for _ in range(150)]
    lengths += [(0, 40), (40, 0), (1, 1), (700, 1900), (1500, 3100)]
    first = [bytes(rng.choice(alphabet, size=n)) for n, _ in lengths]
    second = [bytes(rng.choice(alphabet, size=m)) for _, m in lengths]
    engine, oracle_costs = make_engine(szs, family, costs, b2c, table)
    want = port.pairs(oracle_costs, tape(first), tape(second))
    engine.set_tuning({"cell_bits": [64] * 16})
    for schedule in ("batched", "plain"):
        engine.set_schedule(schedule)
        np.testing.assert_array_equal(engine.pairwise(szs.Strs(first), szs.Strs(second)).astype(np.int64), want)
    engine.set_schedule("batched")
    queries, candidates = first[:31], second[:29]
    np.testing.assert_array_equal(engine(szs.Strs(queries), szs.Strs(candidates)).astype(np.int64),
                                  port.cross(oracle_costs, tape(queries), tape(candidates)))
    engine.set_tuning(None)


@pytest.mark.parametrize("name,family,costs", ENGINES, ids=[e[0] for e in ENGINES])
@pytest.mark.parametrize("lengths", [(0, 6), (1, 40), (50, 600), (900, 2100)], ids=["tiny", "short", "strips", "long"])
def test_pairwise_matches_oracle(szs, port, name, family, costs, lengths):
    rng = np.random.default_rng(abs(hash((name, lengths))) % 2**32)
    alphabet = DNA if family != "nw" or name == "nw-positive-gaps" else PROTEIN
    b2c, table = dna_tables() if alphabet is DNA else protein_tables(rng)
    count = 200 if lengths[1] <= 600 else 24
    first = random_strings(rng, count, *lengths, alphabet)
    second = random_strings(rng, count, *lengths, alphabet)
    engine, oracle_costs = make_engine(szs, family, costs, b2c, table)
    got = engine.pairwise(szs.Strs(first), szs.Strs(second)).astype(np.int64)
    want = port.pairs(oracle_costs, tape(first), tape(second))
    bad = np.flatnonzero(got != want)
    assert bad.size == 0, f"{name}: {bad.size} mismatches, first {bad[:5]}: got {got[bad[:5]]} want {want[bad[:5]]}"
    if lengths[1] > 1024:  # few pairs: the longer ones took the bands; the wavefront routes must agree
        engine.set_tuning({"band_min_rows_few": 1 << 20})
        np.testing.assert_array_equal(engine.pairwise(szs.Strs(first), szs.Strs(second)).astype(np.int64), want)


@pytest.mark.parametrize("family,costs", [("nw", (-3, -1)), ("sw", (-3, -1)), ("nw", (-2, -2)), ("sw", (-4, -4))])
def test_asymmetric_table_orientation(szs, port, family, costs):
    """Cost lookups must stay cost(first[i], second[j]) whichever string the kernel lays along its rows."""
    rng = np.random.default_rng(11)
    b2c, table = protein_tables(rng, symmetric=False)
    first = random_strings(rng, 150, 1, 400, PROTEIN)
    second = random_strings(rng, 150, 1, 400, PROTEIN)
    second[:20] = [bytes(rng.choice(PROTEIN, size=len(f))) for f in first[:20]]  # equal lengths too
    engine, oracle_costs = make_engine(szs, family, costs, b2c, table)
    got = engine.pairwise(szs.Strs(first), szs.Strs(second)).astype(np.int64)
    want = port.pairs(oracle_costs, tape(first), tape(second))
    np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("name,family,costs", ENGINES[:1] + ENGINES[2:3] + ENGINES[5:6] + ENGINES[7:8],
                         ids=["lev-unit", "lev-affine", "nw-affine", "sw-affine"])
def test_cross_and_symmetric_matrices(szs, port, name, family, costs):
    rng = np.random.default_rng(5)
    alphabet = DNA if family != "nw" else PROTEIN
    b2c, table = dna_tables() if alphabet is DNA else protein_tables(rng)
    queries = random_strings(rng, 9, 0, 300, alphabet)
    candidates = random_strings(rng, 13, 0, 300, alphabet)
    engine, oracle_costs = make_engine(szs, family, costs, b2c, table)
    got = engine(szs.Strs(queries), szs.Strs(candidates)).astype(np.int64)
    want = port.cross(oracle_costs, tape(queries), tape(candidates))
    np.testing.assert_array_equal(got, want)
    got_sym = engine(szs.Strs(queries)).astype(np.int64)
    want_sym = port.cross(oracle_costs, tape(queries))
    np.testing.assert_array_equal(got_sym, want_sym)
    # out= with a wider row stride keeps the padding untouched
    out = np.full((9, 20), 7, dtype=engine._dtype)
    returned = engine(szs.Strs(queries), szs.Strs(candidates), out=out)
    assert returned is out
    np.testing.assert_array_equal(out[:, :13].astype(np.int64), want)
    assert (out[:, 13:] == 7).all()


@pytest.mark.parametrize("name,family,costs", ENGINES[:1] + ENGINES[5:6] + ENGINES[7:8],
                         ids=["lev-unit", "nw-affine", "sw-affine"])
def test_cross_and_symmetric_with_long_strings(szs, port, name, family, costs):
    """Cross-product and symmetric calls whose few long pairs take the grouped band, mixed with empty and short
    strings on the warp routes."""
    rng = np.random.default_rng(8)
    alphabet = DNA if family != "nw" else PROTEIN
    b2c, table = dna_tables() if alphabet is DNA else protein_tables(rng)
    queries = [bytes(rng.choice(alphabet, size=n)) for n in (3000, 0, 40, 2200)]
    candidates = [bytes(rng.choice(alphabet, size=n)) for n in (2600, 1, 3500)]
    candidates[2] = queries[0][:2000] + candidates[2][2000:]  # related: a large local score
    engine, oracle_costs = make_engine(szs, family, costs, b2c, table)
    got = engine(szs.Strs(queries), szs.Strs(candidates)).astype(np.int64)
    np.testing.assert_array_equal(got, port.cross(oracle_costs, tape(queries), tape(candidates)))
    got_sym = engine(szs.Strs(queries)).astype(np.int64)
    np.testing.assert_array_equal(got_sym, port.cross(oracle_costs, tape(queries)))


@pytest.mark.parametrize("symbols", [4, 8, 30, 256])
def test_warp_myers_long_patterns(szs, port, symbols):
    """Unit-cost Levenshtein with shorter sides 513..8,192 takes the warp-per-pair bit-parallel route (W words per
    lane, the carry and the shifted-out deltas passed down the lanes); longer ones take the bands. Code planes
    follow the batch alphabet (2, 3, 5 or 8)."""
    rng = np.random.default_rng(symbols + 100)
    alphabet = np.arange(256, dtype=np.uint8)[:symbols] if symbols < 256 else np.arange(256, dtype=np.uint8)
    lengths = [(512, 600), (513, 513), (514, 2000), (1023, 1100), (1024, 1024), (1025, 1030), (2048, 5000),
               (3000, 3000), (4096, 4200), (4097, 4100)]
    if symbols == 4:
        lengths += [(3500, 16390), (700, 40000), (8192, 8200), (8193, 8193)]
    first = [bytes(rng.choice(alphabet, size=n)) for n, _ in lengths]
    second = [bytes(rng.choice(alphabet, size=m)) for _, m in lengths]
    # Related pairs (small distances) and one swapped orientation (the longer string first).
    second[3] = first[3][:900] + second[3][900:]
    second[6] = first[6] + second[6][2048:]
    first[4], second[4] = second[4], first[4]
    engine = szs.LevenshteinDistances()
    want = port.pairs(oracle.levenshtein_costs(), tape(first), tape(second))
    for schedule in ("batched", "plain"):
        engine.set_schedule(schedule)
        got = engine.pairwise(szs.Strs(first), szs.Strs(second)).astype(np.int64)
        np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("schedule", ["batched", "plain"])
@pytest.mark.parametrize("symbols", [1, 2, 4, 7, 256], ids=["1sym", "2sym", "4sym", "7sym", "256sym"])
def test_myers_every_word_count(szs, port, symbols, schedule):
    """Unit-cost Levenshtein takes the bit-parallel routes: one thread per pair for shorter sides up to 512 (the
    shared-table kernel over at most four symbol codes, code planes above), one warp per pair up to 8,192. Every word
    count, texts shorter and longer than the pattern, empty partners; the plain form runs each route with the word
    count of the batch's longest pattern, checked here on a batch whose patterns are all short as well."""
    rng = np.random.default_rng(3 + symbols)
    alphabet = np.frombuffer(b"ACGTNRYK", dtype=np.uint8)[:symbols] if symbols < 256 else \
        np.arange(256, dtype=np.uint8)
    first, second = [], []
    for n in list(range(1, 70)) + list(range(90, 530, 7)) + [600, 1100, 2100]:
        first.append(bytes(rng.choice(alphabet, size=n)))
        second.append(bytes(rng.choice(alphabet, size=int(rng.integers(max(0, n - 60), n + 400)))))
    first[5], second[5] = second[5], first[5]  # the pattern on the second side
    first += [b"", bytes(rng.choice(alphabet, size=40))]
    second += [bytes(rng.choice(alphabet, size=40)), b""]
    engine = szs.LevenshteinDistances()
    engine.set_schedule(schedule)
    got = engine.pairwise(szs.Strs(first), szs.Strs(second)).astype(np.int64)
    want = port.pairs(oracle.levenshtein_costs(), tape(first), tape(second))
    np.testing.assert_array_equal(got, want)
    short_first = [bytes(rng.choice(alphabet, size=int(rng.integers(1, 70)))) for _ in range(300)]
    short_second = [bytes(rng.choice(alphabet, size=int(rng.integers(1, 300)))) for _ in range(300)]
    got = engine.pairwise(szs.Strs(short_first), szs.Strs(short_second)).astype(np.int64)
    np.testing.assert_array_equal(got, port.pairs(oracle.levenshtein_costs(), tape(short_first), tape(short_second)))


@pytest.mark.parametrize("schedule", ["batched", "plain"])
def test_schedules_agree(szs, port, schedule):
    rng = np.random.default_rng(21)
    b2c, table = protein_tables(rng)
    first = random_strings(rng, 300, 0, 700, PROTEIN)
    second = random_strings(rng, 300, 0, 700, PROTEIN)
    for family, costs in (("nw", (-11, -1)), ("sw", (-5, -2)), ("lev", (0, 1, 1, 1))):
        engine, oracle_costs = make_engine(szs, family, costs, b2c, table)
        engine.set_schedule(schedule)
        got = engine.pairwise(szs.Strs(first), szs.Strs(second)).astype(np.int64)
        np.testing.assert_array_equal(got, port.pairs(oracle_costs, tape(first), tape(second)))


def test_device_resident_and_sliced_inputs(szs, port):
    rng = np.random.default_rng(8)
    strings = random_strings(rng, 40, 0, 200, DNA)
    engine = szs.LevenshteinDistances(0, 2, 3, 1)
    host = szs.Strs(strings)
    sliced = host[5:25]  # first offset is not zero
    want = port.cross(oracle.levenshtein_costs(0, 2, 3, 1), tape(strings[5:25]), tape(strings[:10]))
    np.testing.assert_array_equal(engine(sliced, host[:10]).astype(np.int64), want)
    device = szs.to_device(szs.Strs(strings))
    np.testing.assert_array_equal(engine(device[5:25], device[:10]).astype(np.int64), want)


def test_reference_known_answers(szs):
    """Hand-checked cases of the reference's own tests (test/similarities.py:124-143, :170-197)."""
    unit = szs.LevenshteinDistances()

    def d(engine, a, b):
        return int(engine(szs.Strs([a]), szs.Strs([b]))[0, 0])

    assert d(unit, "hello", "hello") == 0
    assert d(unit, "hello", "hell") == 1
    assert d(unit, "", "") == 0
    assert d(unit, "", "abc") == 3
    assert d(unit, "abc", "") == 3
    assert d(unit, "abc", "ac") == 1
    assert d(unit, "abc", "a_bc") == 1
    assert d(unit, "abc", "adc") == 1
    assert d(unit, "ggbuzgjux{}l", "gbuzgjux{}l") == 1
    assert d(unit, "abcdefgABCDEFG", "ABCDEFGabcdefg") == 14
    mismatch, opening, extension = 4, 3, 2
    custom = szs.LevenshteinDistances(open=opening, extend=extension, mismatch=mismatch)
    assert d(custom, "hello", "hello") == 0
    assert d(custom, "hello", "hell") == opening
    assert d(custom, "", "") == 0
    assert d(custom, "", "abc") == opening + 2 * extension
    assert d(custom, "abc", "") == opening + 2 * extension
    assert d(custom, "abc", "ac") == opening
    assert d(custom, "abc", "a_bc") == opening
    assert d(custom, "abc", "adc") == mismatch
    assert d(custom, "ggbuzgjux{}l", "gbuzgjux{}l") == opening
    assert d(custom, "abcdefgABCDEFG", "ABCDEFGabcdefg") == min(14 * mismatch, 2 * opening + 12 * extension)


def test_insertion_ladder(szs):
    """Each random insertion raises the distance by exactly one (test/similarities.py:105-122)."""
    rng = np.random.default_rng(42)
    engine = szs.LevenshteinDistances()
    a = bytes(rng.choice(np.frombuffer(b"abcdefghijklmnopqrstuvwxyz", np.uint8), size=20))
    b = a
    for i in range(150):
        pos = int(rng.integers(0, len(b)))
        b = b[:pos] + bytes([int(rng.integers(97, 123))]) + b[pos:]
        assert int(engine(szs.Strs([a]), szs.Strs([b]))[0, 0]) == i + 1


def test_needleman_wunsch_is_negative_levenshtein(szs, port):
    """NW with a -1/0 class table and -1 gaps equals minus the unit edit distance (test/similarities.py:290-319)."""
    rng = np.random.default_rng(4)
    b2c = (np.arange(256) % 32).astype(np.uint8)
    table = np.full((32, 32), -1, dtype=np.int8)
    np.fill_diagonal(table, 0)
    letters = np.frombuffer(b"abcdefghijklmnopqrstuvwxyz", np.uint8)
    first = random_strings(rng, 300, 10, 400, letters)
    second = random_strings(rng, 300, 10, 400, letters)
    nw = szs.NeedlemanWunschScores(b2c, table, open=-1, extend=-1)
    lev = szs.LevenshteinDistances()
    np.testing.assert_array_equal(nw.pairwise(szs.Strs(first), szs.Strs(second)),
                                  -lev.pairwise(szs.Strs(first), szs.Strs(second)).astype(np.int64))


@pytest.mark.parametrize("symbols", [4, 32, 33, 256])
def test_levenshtein_dp_over_alphabets(szs, port, symbols):
    """Non-unit Levenshtein takes the 16x2 route over the batch alphabet: with a profile when it has at most 32
    symbols, comparing codes otherwise."""
    rng = np.random.default_rng(symbols)
    alphabet = np.arange(256, dtype=np.uint8)[:symbols] if symbols < 256 else np.arange(256, dtype=np.uint8)
    first = random_strings(rng, 101, 0, 700, alphabet)
    second = random_strings(rng, 101, 0, 700, alphabet)
    for costs in ((0, 2, 3, 1), (1, 3, 2, 2)):
        engine = szs.LevenshteinDistances(*costs)
        got = engine.pairwise(szs.Strs(first), szs.Strs(second)).astype(np.int64)
        np.testing.assert_array_equal(got, port.pairs(oracle.levenshtein_costs(*costs), tape(first), tape(second)))


TEXT = np.frombuffer(bytes(range(32, 127)), dtype=np.uint8)


@pytest.mark.parametrize("rows", [4, 8, 12, 16])
@pytest.mark.parametrize("costs", [(0, 2, 3, 1), (0, 3, 2, 2), (1, 3, 4, 1), (0, 127, 100, 100), (3, 1, 5, 5),
                                   (4, 4, 1, 6), (0, 5, 3, 1), (1, 9, 4, 2)])
def test_levenshtein_compare_mode(szs, port, rows, costs):
    """Levenshtein over more than 32 byte values on the 16x2 route takes each cell's cost from comparing the two
    pairs' codes: every rows-per-lane instance, linear and affine gaps, both forms (one multiply-add when match and
    mismatch minus the affine shift have one sign, a mask and a select when they straddle zero: the last two cost
    sets), costs near the byte limit (short pairs) and a match dearer than a mismatch, partners of uneven shapes in
    one warp, codes 0 and 255 side by side, both schedules."""
    rng = np.random.default_rng(rows * 1000 + sum(map(abs, costs)))
    extremes = np.array([0, 1, 127, 128, 254, 255], dtype=np.uint8)
    first, second = [], []
    for k in range(61):  # odd: one warp scores a single pair
        alphabet = TEXT if k % 3 else np.arange(256, dtype=np.uint8)
        first.append(bytes(rng.choice(alphabet, size=int(rng.integers(0, 700)))))
        second.append(bytes(rng.choice(alphabet, size=int(rng.integers(0, 700)))))
    first += [bytes(rng.choice(extremes, size=300)), b"", bytes(rng.choice(TEXT, size=1)), bytes(rng.choice(TEXT, size=650))]
    second += [bytes(rng.choice(extremes, size=310)), bytes(rng.choice(TEXT, size=500)), bytes(rng.choice(TEXT, size=640)),
               bytes(rng.choice(TEXT, size=3))]
    second[5] = first[5][:200] + second[5][200:]  # a long shared stretch
    engine = szs.LevenshteinDistances(*costs)
    engine.set_tuning({"packed_rows": [rows] * 16, "band_min_rows": 4096, "band_min_rows_packed": 4096,
                       "band_min_rows_few": 4096, "band_min_rows_compare": 4096})
    want = port.pairs(oracle.levenshtein_costs(*costs), tape(first), tape(second))
    for schedule in ("batched", "plain"):
        engine.set_schedule(schedule)
        got = engine.pairwise(szs.Strs(first), szs.Strs(second)).astype(np.int64)
        np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("family,costs", [("nw", (-11, -1)), ("sw", (-5, -2)), ("nw", (-4, -4)), ("sw", (-3, -3))])
def test_packed_couples_with_uneven_partners(szs, port, family, costs):
    """Two pairs share a warp on the 16x2 route: odd counts, and partners of very different shapes."""
    rng = np.random.default_rng(77)
    b2c, table = protein_tables(rng)
    first, second = [], []
    for _ in range(37):  # odd
        n = int(rng.integers(1, 900))
        m = int(rng.integers(1, 900))
        first.append(bytes(rng.choice(PROTEIN, size=n)))
        second.append(bytes(rng.choice(PROTEIN, size=m)))
    first += [bytes(rng.choice(PROTEIN, size=1))] * 3 + [bytes(rng.choice(PROTEIN, size=800))]
    second += [bytes(rng.choice(PROTEIN, size=800))] * 3 + [bytes(rng.choice(PROTEIN, size=2))]
    engine, oracle_costs = make_engine(szs, family, costs, b2c, table)
    engine.set_tuning({"band_min_rows_few": 1 << 20})  # keep the longer pairs on the 16x2 wavefront
    for schedule in ("batched", "plain"):
        engine.set_schedule(schedule)
        got = engine.pairwise(szs.Strs(first), szs.Strs(second)).astype(np.int64)
        np.testing.assert_array_equal(got, port.pairs(oracle_costs, tape(first), tape(second)))


@pytest.mark.parametrize("family,costs", [("sw", (-5, -2)), ("nw", (-11, -1)), ("lev", (0, 1, 1, 1)), ("lev", (0, 3, 2, 2)),
                                          ("sw", (-4, -4)), ("nw", (-3, -3))])
def test_band_route_long_pairs(szs, port, family, costs):
    """Shorter sides above 1,024 go to the band kernel (one CTA of warps per pair, strips in a ring)."""
    rng = np.random.default_rng(123)
    alphabet = PROTEIN if family == "nw" else DNA
    b2c, table = (protein_tables(rng) if family == "nw" else dna_tables())
    lengths = [(1025, 1025), (1100, 9000), (2600, 3100), (4100, 2050), (1500, 1500), (5000, 5003)]
    first = [bytes(rng.choice(alphabet, size=n)) for n, _ in lengths]
    second = [bytes(rng.choice(alphabet, size=m)) for _, m in lengths]
    # A related pair, so local scores are large.
    second[2] = first[2][100:2900] + bytes(rng.choice(alphabet, size=300))
    engine, oracle_costs = make_engine(szs, family, costs, b2c, table)
    want = port.pairs(oracle_costs, tape(first), tape(second))
    # Six long pairs leave most CTA slots free: the batched form gives each pair a group of CTAs; the plain form
    # keeps one CTA per pair.
    for schedule in ("batched", "plain"):
        engine.set_schedule(schedule)
        got = engine.pairwise(szs.Strs(first), szs.Strs(second)).astype(np.int64)
        np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("family,costs", [("sw", (-5, -2)), ("nw", (-11, -1)), ("lev", (0, 1, 1, 1)),
                                          ("lev", (0, 2, 3, 1)), ("sw", (-3, -3))])
def test_grouped_band_few_long_pairs(szs, port, family, costs):
    """One or a few long pairs: each gets a group of CTAs (one cooperative launch) whose warps share the strip ring
    through global memory. Pairs with fewer strips than the group has warps leave warps idle."""
    rng = np.random.default_rng(31)
    alphabet = PROTEIN if family == "nw" else DNA
    b2c, table = (protein_tables(rng) if family == "nw" else dna_tables())
    engine, oracle_costs = make_engine(szs, family, costs, b2c, table)
    for lengths in ([(6000, 7000)], [(5001, 7001)], [(1100, 20000)], [(3000, 3000), (2500, 9000), (1200, 1301)],
                    [(1030, 1030)] * 2 + [(4000, 4100)]):
        first = [bytes(rng.choice(alphabet, size=n)) for n, _ in lengths]
        second = [bytes(rng.choice(alphabet, size=m)) for _, m in lengths]
        second[0] = first[0][: lengths[0][0] // 2] + second[0][lengths[0][0] // 2:]  # related: large local scores
        got = engine.pairwise(szs.Strs(first), szs.Strs(second)).astype(np.int64)
        np.testing.assert_array_equal(got, port.pairs(oracle_costs, tape(first), tape(second)))


@pytest.mark.parametrize("family,costs", [("nw", (-11, -1)), ("lev", (0, 2, 3, 3))])
def test_grouped_band_more_strips_than_32_ctas_hold(szs, port, family, costs):
    """One pair of 36,000 x 36,500 on 32-bit cells: 282 strips of 128 rows, so its group takes 36 CTAs (more than a
    32-CTA group's 256 warps) and every strip has its own warp."""
    rng = np.random.default_rng(53)
    alphabet = PROTEIN if family == "nw" else DNA
    b2c, table = (protein_tables(rng) if family == "nw" else dna_tables())
    engine, oracle_costs = make_engine(szs, family, costs, b2c, table)
    first = [bytes(rng.choice(alphabet, size=36000))]
    second = [first[0][:18000] + bytes(rng.choice(alphabet, size=18500))]
    got = engine.pairwise(szs.Strs(first), szs.Strs(second)).astype(np.int64)
    np.testing.assert_array_equal(got, port.pairs(oracle_costs, tape(first), tape(second)))


@pytest.mark.parametrize("family,costs", [("lev", (0, 2, 3, 1)), ("lev", (0, 2, 3, 3)), ("nw", (-11, -1)),
                                          ("nw", (-4, -4)), ("sw", (-5, -2)), ("sw", (-3, -3))])
def test_grouped_band_two_columns_per_step(szs, port, family, costs):
    """Groups of CTAs on 4-row strips score two columns per lane-step: odd and even column counts (the last step's
    second column past the end), the corner in either column, related pairs (large local scores), both orientations,
    one pair alone and three at once. 32-bit cells are forced so that local scores take the 32-bit band too."""
    rng = np.random.default_rng(zlib_seed(f"two-columns{family}{costs}"))
    alphabet = PROTEIN if family == "nw" else DNA
    b2c, table = protein_tables(rng) if family == "nw" else dna_tables()
    engine, oracle_costs = make_engine(szs, family, costs, b2c, table)
    engine.set_tuning({"cell_bits": [32] * 16})
    for lengths in ([(5001, 6001)], [(6003, 4097)], [(3001, 3003), (2999, 7002), (4000, 4001)], [(7000, 7000)]):
        first = [bytes(rng.choice(alphabet, size=n)) for n, _ in lengths]
        second = [bytes(rng.choice(alphabet, size=m)) for _, m in lengths]
        half = min(lengths[0]) // 2
        second[0] = first[0][:half] + second[0][half:]
        got = engine.pairwise(szs.Strs(first), szs.Strs(second)).astype(np.int64)
        np.testing.assert_array_equal(got, port.pairs(oracle_costs, tape(first), tape(second)))
    engine.set_tuning(None)


@pytest.mark.parametrize("case", ["dense-nw-affine", "dense-sw-linear", "utf8-wide"])
def test_grouped_band_two_columns_dense_and_wide(szs, port, case):
    """The two-column sweep over a dense 256 x 256 table (every byte value) and over 16-bit codes (UTF-8 with more
    than 256 code points), one long pair with an odd number of columns, against the oracle."""
    rng = np.random.default_rng(zlib_seed(case))
    if case.startswith("dense"):
        family, costs = ("nw", (-11, -1)) if case == "dense-nw-affine" else ("sw", (-3, -3))
        cls = szs.NeedlemanWunschScores if family == "nw" else szs.SmithWatermanScores
        kind = oracle.NEEDLEMAN_WUNSCH if family == "nw" else oracle.SMITH_WATERMAN
        table = rng.integers(-9, 10, size=(256, 256)).astype(np.int8)
        engine = cls.dense(table, open=costs[0], extend=costs[1])
        want_costs = oracle.dense_costs(kind, table, *costs)
        everything = np.arange(256, dtype=np.uint8)
        first, second = [bytes(rng.choice(everything, size=2601))], [bytes(rng.choice(everything, size=3001))]
    else:
        letters = [chr(c) for c in range(0x4E00, 0x4E00 + 3000)]
        first = ["".join(rng.choice(letters, size=4001))]
        second = [first[0][:2000] + "".join(rng.choice(letters, size=3001))]
        engine = szs.LevenshteinDistancesUTF8(0, 2, 3, 1)
        want_costs = oracle.levenshtein_utf8_costs(0, 2, 3, 1)
        engine.set_tuning({"cell_bits": [32] * 16})
    got = engine.pairwise(szs.Strs(first), szs.Strs(second)).astype(np.int64)
    np.testing.assert_array_equal(got, port.pairs(want_costs, tape(first), tape(second)))


@pytest.mark.parametrize("family,costs", [("sw", (-5, -2)), ("nw", (-11, -1)), ("lev", (0, 2, 3, 1))])
def test_grouped_band_beside_small_launches(szs, port, family, costs):
    """A cooperative grouped-band launch queued behind small launches that take a few CTA slots first (grids that
    do not fill the device go first): the group still meets, every score equals the oracle, no wait gives up."""
    rng = np.random.default_rng(47)
    alphabet = PROTEIN if family == "nw" else DNA
    b2c, table = (protein_tables(rng) if family == "nw" else dna_tables())
    lengths = [(6000, 6500), (5000, 9000)] + [(int(rng.integers(20, 300)), int(rng.integers(20, 300)))
                                              for _ in range(50)]
    first = [bytes(rng.choice(alphabet, size=n)) for n, _ in lengths]
    second = [bytes(rng.choice(alphabet, size=m)) for _, m in lengths]
    second[0] = first[0][:3000] + second[0][3000:]
    engine, oracle_costs = make_engine(szs, family, costs, b2c, table)
    want = port.pairs(oracle_costs, tape(first), tape(second))
    for _ in range(3):
        got = engine.pairwise(szs.Strs(first), szs.Strs(second)).astype(np.int64)
        np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("family,costs,extreme", [
    ("nw", (-30, -2), 120),    # 120 - (-30) leaves a signed byte: the affine pairs leave the 16x2 route
    ("sw", (-30, -2), 110),
    ("nw", (-30, -2), 90),     # 90 + 30 still fits: the 16x2 route keeps them
    ("sw", (-40, -40), 127),   # linear gaps take costs as they are
    ("nw", (20, 1), -110),     # positive open: -110 - 20 leaves a signed byte
])
def test_profile_byte_range(szs, port, family, costs, extreme):
    """The 16x2 route stores `cost - open` (affine) or `cost` (linear) in int8 profiles; tables outside that range
    are scored by the 32-bit route. Either way the scores equal the oracle's."""
    rng = np.random.default_rng(abs(extreme) + (0 if family == "nw" else 1000))
    b2c, table = protein_tables(rng)
    table[3, 3] = extreme
    table[5, 7] = -extreme // 2
    first = random_strings(rng, 96, 1, 400, PROTEIN)
    second = random_strings(rng, 96, 1, 400, PROTEIN)
    engine, oracle_costs = make_engine(szs, family, costs, b2c, table)
    got = engine.pairwise(szs.Strs(first), szs.Strs(second)).astype(np.int64)
    np.testing.assert_array_equal(got, port.pairs(oracle_costs, tape(first), tape(second)))


@pytest.mark.parametrize("costs", [(0, 127, 100, 100), (0, 120, 127, 1), (5, 100, 120, 127), (0, 127, 0, 127)])
def test_levenshtein_large_costs(szs, port, costs):
    """Levenshtein costs near the top of their signed-byte range on short strings, where the length bound alone
    allows 16-bit cells: profile entries `cost - open` stay inside a signed byte for non-negative costs."""
    rng = np.random.default_rng(sum(costs))
    first = random_strings(rng, 64, 0, 60, DNA)
    second = random_strings(rng, 64, 0, 60, DNA)
    engine = szs.LevenshteinDistances(*costs)
    got = engine.pairwise(szs.Strs(first), szs.Strs(second)).astype(np.int64)
    np.testing.assert_array_equal(got, port.pairs(oracle.levenshtein_costs(*costs), tape(first), tape(second)))


@pytest.mark.parametrize("family,costs", [("lev", (0, 1, 1, 1)), ("lev", (0, 2, 3, 1)), ("nw", (-11, -1)), ("sw", (-5, -2))])
def test_graph_replay_reads_fresh_inputs(szs, port, family, costs):
    """Device-resident calls are captured as CUDA graphs and replayed; a replay must score the bytes currently in
    the buffers, and a new alphabet or a new shape must not replay a stale graph."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(31)
    b2c, table = dna_tables()
    engine, oracle_costs = make_engine(szs, family, costs, b2c, table)
    lengths_a = rng.integers(0, 700, size=300)
    lengths_b = rng.integers(0, 700, size=300)
    lengths_a[:3] = [1500, 2100, 40]  # a band pair and a 32-bit pair among the packed ones
    lengths_b[:3] = [1400, 2200, 3000]
    offsets_a = np.concatenate([[0], np.cumsum(lengths_a)]).astype(np.int64)
    offsets_b = np.concatenate([[0], np.cumsum(lengths_b)]).astype(np.int64)
    data_a = torch.empty(int(offsets_a[-1]), dtype=torch.uint8, device="cuda")
    data_b = torch.empty(int(offsets_b[-1]), dtype=torch.uint8, device="cuda")
    first = szs.Strs.from_buffers(data_a, torch.from_numpy(offsets_a).cuda())
    second = szs.Strs.from_buffers(data_b, torch.from_numpy(offsets_b).cuda())
    out = torch.empty(300, dtype=torch.int64, device="cuda")
    before = engine.stats()["graph_replays"]
    for round_, alphabet in enumerate([b"ACGT", b"ACGT", b"ACGT", b"AC", b"ACGT"]):
        letters = np.frombuffer(alphabet, dtype=np.uint8)
        host_a = rng.choice(letters, size=int(offsets_a[-1])).astype(np.uint8)
        host_b = rng.choice(letters, size=int(offsets_b[-1])).astype(np.uint8)
        shared = min(len(host_a), len(host_b)) // 3
        host_b[:shared] = host_a[:shared]  # related stretches: larger local scores
        data_a.copy_(torch.from_numpy(host_a))
        data_b.copy_(torch.from_numpy(host_b))
        engine.pairwise(first, second, out=out)
        want = port.pairs(oracle_costs, (host_a, offsets_a), (host_b, offsets_b))
        np.testing.assert_array_equal(out.cpu().numpy(), want, err_msg=f"round {round_}")
    assert engine.stats()["graph_replays"] - before >= 2


@pytest.mark.parametrize("tuning", [
    {"packed_rows": [4] * 16, "packed_warps": [1, 2, 8, 3]},
    {"packed_rows": [16] * 16, "band_min_rows": 300, "packed_warps": [8, 8, 8, 8], "band_min_rows_packed": 300},
    {"cell_bits": [32] * 16, "band_min_rows": 4096},
    {"packed_rows": [12] * 8 + [8] * 8, "cell_bits": [0, 0, 0, 0, 0, 32, 0, 32] + [0] * 8},
], ids=["rows4", "rows16-lowband", "wide-only", "mixed"])
@pytest.mark.parametrize("family,costs", [("nw", (-11, -1)), ("sw", (-5, -5)), ("lev", (0, 2, 3, 1))])
def test_any_tuning_keeps_scores(szs, port, tuning, family, costs):
    """Tunings only move pairs between routes and launch shapes: every tuning gives the oracle's scores."""
    rng = np.random.default_rng(17)
    alphabet = PROTEIN if family == "nw" else DNA
    b2c, table = protein_tables(rng) if family == "nw" else dna_tables()
    lengths = [(int(rng.integers(0, 1500)), int(rng.integers(0, 1500))) for _ in range(120)]
    lengths += [(3000, 2500), (600, 4000), (5, 5000)]
    first = [bytes(rng.choice(alphabet, size=n)) for n, _ in lengths]
    second = [bytes(rng.choice(alphabet, size=m)) for _, m in lengths]
    engine, oracle_costs = make_engine(szs, family, costs, b2c, table)
    engine.set_tuning(tuning)
    got = engine.pairwise(szs.Strs(first), szs.Strs(second)).astype(np.int64)
    np.testing.assert_array_equal(got, port.pairs(oracle_costs, tape(first), tape(second)))


@pytest.mark.parametrize("family,costs", [("lev", (0, 1, 1, 1)), ("sw", (-5, -2)), ("lev", (0, 2, 3, 1))],
                         ids=["lev-unit", "sw", "lev-affine"])
def test_pipelined_pinned_host_call(szs, port, family, costs):
    """Pairwise calls on large pinned host tapes are cut into chunks whose copies overlap the previous chunk's
    scoring (planned ahead from a sample of the first chunk for unit costs, from the offsets alone for alignment
    engines, after each chunk's bytes for the other Levenshtein costs); the chunked call must equal the oracle and
    the device-resident call."""
    torch = pytest.importorskip("torch")
    from stringzillas_gb300 import workloads as w
    unit = costs == (0, 1, 1, 1)
    count = 420_000 if unit else 700_000
    (fd, fo), (sd, so) = w.levenshtein_reads(count, 100, 300, 0.05, 0.02, seed=3) if unit else \
        w.levenshtein_reads(count, 60, 100, 0.10, 0.02, seed=4)
    assert fd.nbytes + sd.nbytes > 2 * (48 << 20), "the call must span several chunks"
    b2c, table = dna_tables()
    engine, oracle_costs = make_engine(szs, family, costs, b2c, table)
    pinned = [torch.from_numpy(x).pin_memory() for x in (fd, fo.astype(np.uint64).view(np.int64),
                                                          sd, so.astype(np.uint64).view(np.int64))]
    first = szs.Strs.from_buffers(pinned[0], pinned[1])
    second = szs.Strs.from_buffers(pinned[2], pinned[3])
    want = port.pairs(oracle_costs, (fd, fo), (sd, so))
    for chunk_kb in (0, 4096):  # the default chunks, then about forty smaller ones
        engine.set_tuning({"pipeline_chunk_kb": chunk_kb})
        out = torch.full((count,), -7, dtype=torch.int64).pin_memory()
        engine.pairwise(first, second, out=out)
        stats = engine.stats()
        assert stats["last_pairs"] == count and stats["last_cells"] == w.cells((fd, fo), (sd, so))
        np.testing.assert_array_equal(out.numpy(), want)
    device = szs.to_device(szs.Strs.from_buffers(fd, fo.astype(np.uint64)))
    device_b = szs.to_device(szs.Strs.from_buffers(sd, so.astype(np.uint64)))
    np.testing.assert_array_equal(engine.pairwise(device, device_b).astype(np.int64), want)


def test_pipelined_chunks_planned_from_a_sample(szs, port):
    """Pipelined unit-cost calls plan every chunk before its bytes land, from the alphabet of the first chunk's bytes:
    later chunks with a fifth symbol in a shorter or a longer string, or with a pair too long for the thread route,
    are scored again exactly and equal the oracle."""
    torch = pytest.importorskip("torch")
    from stringzillas_gb300 import workloads as w
    count = 200_000
    (fd, fo), (sd, so) = w.levenshtein_reads(count, 100, 300, 0.05, 0.02, seed=8)
    first = [bytes(fd[fo[i]:fo[i + 1]]) for i in range(count)]
    second = [bytes(sd[so[i]:so[i + 1]]) for i in range(count)]
    first[150_000] = first[150_000][:40] + b"N" + first[150_000][41:]
    second[180_000] = second[180_000][:90] + b"NN" + second[180_000][92:]
    rng = np.random.default_rng(8)
    first[190_000] = bytes(rng.choice(DNA, size=1500))
    second[190_000] = bytes(rng.choice(DNA, size=1700))
    (fd, fo), (sd, so) = tape(first), tape(second)
    engine = szs.LevenshteinDistances()
    pinned = [torch.from_numpy(np.array(x)).pin_memory() for x in (fd, fo.astype(np.uint64).view(np.int64),
                                                                    sd, so.astype(np.uint64).view(np.int64))]
    a = szs.Strs.from_buffers(pinned[0], pinned[1])
    b = szs.Strs.from_buffers(pinned[2], pinned[3])
    want = port.pairs(oracle.levenshtein_costs(), (fd, fo), (sd, so))
    for chunk_kb in (4096, 16384):  # about twenty chunks (more than the contexts in flight), then five
        engine.set_tuning({"pipeline_chunk_kb": chunk_kb})
        for _ in range(2):  # the second call replays the captured graphs
            out = torch.full((count,), -7, dtype=torch.int64).pin_memory()
            engine.pairwise(a, b, out=out)
            np.testing.assert_array_equal(out.numpy(), want)


@pytest.mark.parametrize("family,costs", [("lev", (0, 1, 1, 1)), ("lev", (0, 2, 3, 1)), ("lev", (0, 3, 2, 2)),
                                          ("nw", (-11, -1)), ("nw", (-4, -4)), ("sw", (-5, -2)), ("sw", (-3, -3))])
def test_band16_route(szs, port, family, costs):
    """Long pairs that fit 16-bit cells take the 16-bit band (two row strips per warp, 512-row super-strips):
    shapes around the super-strip size, a high half that is all filler, and local scores near their bound."""
    rng = np.random.default_rng(91)
    alphabet = PROTEIN if family == "nw" else DNA
    b2c, table = (protein_tables(rng) if family == "nw" else dna_tables())
    if family == "nw":  # the reach bound (n + m + 4) * 11 < 32767 keeps these on 16-bit cells
        lengths = [(601, 601), (700, 1400), (1023, 1024), (1025, 1300), (1400, 1500), (512 * 2 + 3, 1200)]
    else:
        lengths = [(601, 601), (700, 2400), (1024, 1024), (1025, 3000), (1536, 1600), (2049, 2100), (3000, 9000),
                   (520, 6000)]
    first = [bytes(rng.choice(alphabet, size=n)) for n, _ in lengths]
    second = [bytes(rng.choice(alphabet, size=m)) for _, m in lengths]
    second[1] = first[1][:600] + second[1][600:]         # a long related stretch: large local scores
    second[4] = first[4][100:1500] + second[4][1400:]
    engine, oracle_costs = make_engine(szs, family, costs, b2c, table)
    engine.set_tuning({"band_min_rows_packed": 600})
    got = engine.pairwise(szs.Strs(first), szs.Strs(second)).astype(np.int64)
    np.testing.assert_array_equal(got, port.pairs(oracle_costs, tape(first), tape(second)))
    # The plain form keeps the same route, in input order.
    engine.set_schedule("plain")
    got = engine.pairwise(szs.Strs(first), szs.Strs(second)).astype(np.int64)
    np.testing.assert_array_equal(got, port.pairs(oracle_costs, tape(first), tape(second)))


@pytest.mark.parametrize("costs", [(0, 2, 3, 1), (0, 3, 2, 2), (1, 3, 4, 1), (3, 1, 5, 5), (0, 5, 3, 1)])
def test_band16_compare_mode(szs, port, costs):
    """Long Levenshtein pairs over more than 32 byte values take the 16-bit band in compare mode, one CTA per pair
    and (few pairs) grouped CTAs: shapes around the super-strip size, a long shared stretch, codes 0 and 255."""
    rng = np.random.default_rng(sum(costs) + 5)
    lengths = [(601, 601), (700, 1400), (1023, 1024), (1025, 1300), (1400, 1500), (512 * 2 + 3, 1200), (2049, 2100)]
    first = [bytes(rng.choice(TEXT, size=n)) for n, _ in lengths]
    second = [bytes(rng.choice(TEXT, size=m)) for _, m in lengths]
    second[1] = first[1][:600] + second[1][600:]
    first[3] = bytes(rng.choice(np.array([0, 255, 65], dtype=np.uint8), size=1025))
    second[3] = bytes(rng.choice(np.array([0, 255, 66], dtype=np.uint8), size=1300))
    engine = szs.LevenshteinDistances(*costs)
    engine.set_tuning({"band_min_rows_packed": 600, "band_min_rows_compare": 600})
    want = port.pairs(oracle.levenshtein_costs(*costs), tape(first), tape(second))
    for schedule in ("batched", "plain"):
        engine.set_schedule(schedule)
        np.testing.assert_array_equal(engine.pairwise(szs.Strs(first), szs.Strs(second)).astype(np.int64), want)
    engine.set_schedule("batched")
    few = [1, 6]  # two long pairs: grouped CTAs
    sub_first, sub_second = [first[i] for i in few], [second[i] for i in few]
    np.testing.assert_array_equal(engine.pairwise(szs.Strs(sub_first), szs.Strs(sub_second)).astype(np.int64),
                                  want[few])


def test_band16_local_scores_past_the_16bit_limit(szs, port):
    """Local scores run on 16-bit cells beyond their proven bound; a pair whose maximum reaches 32767 minus the
    largest gain is scored again on 32-bit cells inside the same CTA. Identical long strings score 2 per base."""
    rng = np.random.default_rng(5)
    b2c, table = dna_tables()  # match +2, mismatch -3
    engine, oracle_costs = make_engine(szs, "sw", (-5, -2), b2c, table)
    base = rng.choice(DNA, size=17_500)
    first, second = [], []
    for n, m, related in ((17_000, 17_000, True),    # 34,000: past the limit, rescored
                          (16_383, 16_383, True),    # 32,766: at the limit (32,765), rescored
                          (16_382, 16_382, True),    # 32,764: just below, exact on 16-bit cells
                          (17_000, 17_400, False),   # unrelated: small score, never rescored
                          (2_000, 3_000, True)):     # short: provably within the bound
        a = bytes(base[:n])
        b = bytes(base[:m]) if related else bytes(rng.choice(DNA, size=m))
        first.append(a)
        second.append(b)
    got = engine.pairwise(szs.Strs(first), szs.Strs(second)).astype(np.int64)
    want = port.pairs(oracle_costs, tape(first), tape(second))
    np.testing.assert_array_equal(got, want)
    assert want[0] == 34_000 and want[1] == 32_766 and want[2] == 32_764


@pytest.mark.parametrize("family,costs", [("nw", (-11, -1)), ("nw", (-4, -4)), ("sw", (-5, -2)), ("sw", (-3, -3))])
def test_dense_tables(szs, port, family, costs):
    """Dense 256 x 256 tables: a dense expansion of a class fold scores like the class engine (which the reference
    pins), and an arbitrary asymmetric dense table matches the oracle's dense restatement on every route."""
    rng = np.random.default_rng(23)
    b2c, table = protein_tables(rng, symmetric=False)
    expanded = table[b2c[:, None], b2c[None, :]]  # [first byte][second byte]
    cls = szs.NeedlemanWunschScores if family == "nw" else szs.SmithWatermanScores
    kind = oracle.NEEDLEMAN_WUNSCH if family == "nw" else oracle.SMITH_WATERMAN
    lengths = [(int(rng.integers(0, 900)), int(rng.integers(0, 900))) for _ in range(150)]
    lengths += [(1100, 1350), (1400, 1200), (3000, 200)]  # band routes and long single strips
    first = [bytes(rng.choice(PROTEIN, size=n)) for n, _ in lengths]
    second = [bytes(rng.choice(PROTEIN, size=m)) for _, m in lengths]
    dense_engine = cls.dense(np.ascontiguousarray(expanded), open=costs[0], extend=costs[1])
    class_engine = cls(b2c, table, open=costs[0], extend=costs[1])
    got = dense_engine.pairwise(szs.Strs(first), szs.Strs(second)).astype(np.int64)
    np.testing.assert_array_equal(got, class_engine.pairwise(szs.Strs(first), szs.Strs(second)))
    # An arbitrary table over 24 bytes (not expressible as a 32-class fold of these letters' classes).
    letters = np.frombuffer(b"ARNDCQEGHILKMFPSTWYVBZX*", dtype=np.uint8)
    arbitrary = np.zeros((256, 256), dtype=np.int8)
    arbitrary[np.ix_(letters, letters)] = rng.integers(-6, 9, size=(24, 24))
    first = [bytes(rng.choice(letters, size=n)) for n, _ in lengths]
    second = [bytes(rng.choice(letters, size=m)) for _, m in lengths]
    engine = cls.dense(arbitrary, open=costs[0], extend=costs[1])
    got = engine.pairwise(szs.Strs(first), szs.Strs(second)).astype(np.int64)
    want = port.pairs(oracle.dense_costs(kind, arbitrary, *costs), tape(first), tape(second))
    np.testing.assert_array_equal(got, want)
    # A cross product and the symmetric form go through the same per-call table.
    cross = engine(szs.Strs(first[:20]), szs.Strs(second[:15]))
    for q in range(20):
        np.testing.assert_array_equal(cross[q], port.pairs(oracle.dense_costs(kind, arbitrary, *costs),
                                                           tape([first[q]] * 15), tape(second[:15])))


@pytest.mark.parametrize("family,costs", [("nw", (-11, -1)), ("nw", (-4, -4)), ("sw", (-5, -2)), ("sw", (-3, -3))])
def test_dense_tables_over_every_byte(szs, port, family, costs):
    """Dense tables over more than 32 distinct bytes: the 32-bit routes read the whole 256 x 256 table from shared
    memory (warp wavefront, band, grouped band), both orientations of a pair, against the oracle."""
    rng = np.random.default_rng(29)
    cls = szs.NeedlemanWunschScores if family == "nw" else szs.SmithWatermanScores
    kind = oracle.NEEDLEMAN_WUNSCH if family == "nw" else oracle.SMITH_WATERMAN
    table = rng.integers(-9, 10, size=(256, 256)).astype(np.int8)  # asymmetric
    engine = cls.dense(table, open=costs[0], extend=costs[1])
    want_costs = oracle.dense_costs(kind, table, *costs)
    everything = np.arange(256, dtype=np.uint8)
    for lengths in ([(int(rng.integers(0, 700)), int(rng.integers(0, 700))) for _ in range(120)] + [(1500, 1200)],
                    [(2600, 3000)], [(40, 33), (33, 40)]):
        first = [bytes(rng.choice(everything, size=n)) for n, _ in lengths]
        second = [bytes(rng.choice(everything, size=m)) for _, m in lengths]
        got = engine.pairwise(szs.Strs(first), szs.Strs(second)).astype(np.int64)
        np.testing.assert_array_equal(got, port.pairs(want_costs, tape(first), tape(second)))
    # Forty distinct bytes, a cross product (queries shorter and longer than candidates: both orientations).
    forty = np.arange(40, 80, dtype=np.uint8)
    queries = [bytes(rng.choice(forty, size=n)) for n in (5, 300, 80)]
    candidates = [bytes(rng.choice(forty, size=n)) for n in (120, 7, 300, 0)]
    got = engine(szs.Strs(queries), szs.Strs(candidates)).astype(np.int64)
    np.testing.assert_array_equal(got, port.cross(want_costs, tape(queries), tape(candidates)))


def _golden_cases():
    import os
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "golden.npz")
    with np.load(path) as data:
        return {str(name): {k.split("__", 1)[1]: data[k] for k in data.files if k.startswith(f"{name}__")}
                for name in data["__names__"]}


GOLDEN = _golden_cases()


@pytest.mark.parametrize("name", sorted(GOLDEN))
def test_engine_matches_reference_outputs(szs, name):
    """Every golden case (outputs of the reference library compiled from its sources) through the engine."""
    case = GOLDEN[name]
    kind = int(case["kind"][0])
    match, mismatch, open_, extend = (int(x) for x in case["costs"])
    if kind == oracle.LEVENSHTEIN:
        cls = szs.LevenshteinDistancesUTF8 if int(case["utf8"][0]) else szs.LevenshteinDistances
        engine = cls(match, mismatch, open_, extend)
    else:
        cls = szs.NeedlemanWunschScores if kind == oracle.NEEDLEMAN_WUNSCH else szs.SmithWatermanScores
        engine = cls(case["b2c"], np.ascontiguousarray(case["table"]), open=open_, extend=extend)
    q = szs.Strs.from_buffers(case["q_data"], case["q_offsets"])
    c = szs.Strs.from_buffers(case["c_data"], case["c_offsets"])
    mode = int(case["mode"][0])
    if mode == 0:
        got = engine.pairwise(q, c)
    elif mode == 1:
        got = engine(q, c)
    else:
        got = engine(q)
    np.testing.assert_array_equal(np.asarray(got).astype(np.int64), case["expected"])


@pytest.mark.parametrize("costs", [(0, 1, 1, 1), (0, 3, 2, 2), (0, 4, 5, 2), (1, 3, 4, 1)])
def test_utf8_levenshtein_routes(szs, port, costs):
    """Code-point distances across the routes: short and long pairs, up to 256 distinct code points (one-byte
    codes)."""
    rng = np.random.default_rng(sum(costs) + 1)
    letters = [chr(c) for c in range(0x3041, 0x3041 + 80)] + [chr(c) for c in range(0x1F600, 0x1F600 + 60)] + \
        list("abcdefghij") + [chr(c) for c in range(0x400, 0x400 + 100)]
    assert len(letters) == 250
    lengths = [(int(rng.integers(0, 300)), int(rng.integers(0, 300))) for _ in range(200)]
    lengths += [(700, 900), (1500, 1600), (3000, 2600)]
    first = ["".join(rng.choice(letters, size=n)) for n, _ in lengths]
    second = ["".join(rng.choice(letters, size=m)) for _, m in lengths]
    second[-1] = first[-1][:2000] + second[-1][2000:]  # related: small distance on a band pair
    engine = szs.LevenshteinDistancesUTF8(*costs)
    got = engine.pairwise(szs.Strs(first), szs.Strs(second)).astype(np.int64)
    want = port.pairs(oracle.levenshtein_utf8_costs(*costs), tape(first), tape(second))
    np.testing.assert_array_equal(got, want)
    cross = engine(szs.Strs(first[:12]), szs.Strs(second[:9]))
    np.testing.assert_array_equal(cross.astype(np.int64), port.cross(oracle.levenshtein_utf8_costs(*costs),
                                                                     tape(first[:12]), tape(second[:9])))


@pytest.mark.parametrize("costs", [(0, 1, 1, 1), (0, 2, 3, 1), (1, 3, 2, 2), (0, 5, 3, 1)])
def test_utf8_levenshtein_over_many_code_points(szs, port, costs):
    """More than 256 distinct code points: 16-bit codes on every route (thread and warp bit-parallel kernels with 16
    code planes, the 16x2 wavefront and 16-bit band in compare mode, both cost forms, the 32-bit wavefront and band
    where the bound needs them), short and long pairs, both orientations and a cross product."""
    rng = np.random.default_rng(sum(costs) + 7)
    letters = [chr(c) for c in range(0x4E00, 0x4E00 + 3000)] + list("abcdefghij")
    lengths = [(int(rng.integers(0, 300)), int(rng.integers(0, 300))) for _ in range(150)]
    lengths += [(255, 400), (256, 256), (257, 300), (700, 900), (1500, 1600), (3000, 2600), (9000, 9100)]
    first = ["".join(rng.choice(letters, size=n)) for n, _ in lengths]
    second = ["".join(rng.choice(letters, size=m)) for _, m in lengths]
    second[-2] = first[-2][:2000] + second[-2][2000:]  # related: small distances on long pairs
    second[-1] = first[-1][:8000] + second[-1][8000:]
    first[-4], second[-4] = second[-4], first[-4]
    engine = szs.LevenshteinDistancesUTF8(*costs)
    want = port.pairs(oracle.levenshtein_utf8_costs(*costs), tape(first), tape(second))
    for schedule in ("batched", "plain"):
        engine.set_schedule(schedule)
        got = engine.pairwise(szs.Strs(first), szs.Strs(second)).astype(np.int64)
        np.testing.assert_array_equal(got, want)
    engine.set_schedule("batched")
    cross = engine(szs.Strs(first[:12]), szs.Strs(second[:9]))
    np.testing.assert_array_equal(cross.astype(np.int64), port.cross(oracle.levenshtein_utf8_costs(*costs),
                                                                     tape(first[:12]), tape(second[:9])))


@pytest.mark.parametrize("rows", [4, 8, 12, 16])
@pytest.mark.parametrize("costs", [(0, 2, 3, 1), (0, 3, 2, 2), (3, 1, 5, 5), (0, 5, 3, 1)])
def test_utf8_compare_mode_over_16bit_codes(szs, port, rows, costs):
    """16-bit codes on the 16x2 routes: every rows-per-lane instance of the wavefront and the 16-bit band (tuned down
    to 600 rows), codes that differ only in their high byte, uneven partners, odd counts."""
    rng = np.random.default_rng(rows * 100 + sum(costs))
    # 300 distinct code points: the codes above 255 share their low byte with codes below it.
    letters = [chr(c) for c in range(0x3041, 0x3041 + 86)] + [chr(c) for c in range(0xAC00, 0xAC00 + 214)]
    lengths = [(int(rng.integers(0, 500)), int(rng.integers(0, 500))) for _ in range(41)]
    lengths += [(601, 700), (1025, 1300), (700, 1400), (2049, 2100)]
    first = ["".join(rng.choice(letters, size=n)) for n, _ in lengths]
    second = ["".join(rng.choice(letters, size=m)) for _, m in lengths]
    second[-3] = first[-3][:500] + second[-3][500:]
    engine = szs.LevenshteinDistancesUTF8(*costs)
    engine.set_tuning({"packed_rows": [rows] * 16, "band_min_rows": 600, "band_min_rows_packed": 600,
                       "band_min_rows_few": 600, "band_min_rows_compare": 600})
    want = port.pairs(oracle.levenshtein_utf8_costs(*costs), tape(first), tape(second))
    for schedule in ("batched", "plain"):
        engine.set_schedule(schedule)
        np.testing.assert_array_equal(engine.pairwise(szs.Strs(first), szs.Strs(second)).astype(np.int64), want)


@pytest.mark.parametrize("schedule", ["batched", "plain"], ids=["grouped-band", "one-cta-band"])
@pytest.mark.parametrize("family", ["nw", "sw"], ids=["band32-nw", "band16-sw"])
def test_bounded_wait_gives_up_and_next_call_is_exact(szs, port, family, schedule):
    """The band kernels' waits are bounded. With the bound tuned down to one poll (about 100 ns), the strips below
    the first cannot find the strip above ready (it needs dozens of column steps first), so the waits give up: the
    call returns an error status instead of hanging, and nothing faults. The next call at the built-in bound is
    bit-exact. Few long pairs in the batched form take the cooperative grouped band (its barrier is bounded the same
    way); the plain form gives each pair one CTA. Protein NW at -11/-1 needs 32-bit cells, DNA SW 16-bit ones."""
    rng = np.random.default_rng(77 if family == "nw" else 78)
    if family == "nw":
        b2c, table = protein_tables(rng)
        first = random_strings(rng, 3, 5000, 6000, PROTEIN)
        second = random_strings(rng, 3, 5000, 6000, PROTEIN)
        engine, oracle_costs = make_engine(szs, "nw", (-11, -1), b2c, table)
    else:
        b2c, table = dna_tables()
        first = random_strings(rng, 3, 5000, 6000, DNA)
        second = random_strings(rng, 3, 5000, 6000, DNA)
        engine, oracle_costs = make_engine(szs, "sw", (-5, -2), b2c, table)
    engine.set_schedule(schedule)
    a, b = szs.Strs(first), szs.Strs(second)
    engine.set_tuning({"band_wait_polls": 1})
    with pytest.raises(RuntimeError, match="bounded wait"):
        engine.pairwise(a, b)
    engine.set_tuning(None)
    got = engine.pairwise(a, b).astype(np.int64)
    np.testing.assert_array_equal(got, port.pairs(oracle_costs, tape(first), tape(second)))


@pytest.mark.parametrize("where", ["pattern", "text", "both", "none"])
def test_sampled_alphabet_guess_is_verified(szs, port, where):
    """Unit-cost Levenshtein guesses the batch alphabet from the first MiB of each tape and the shared-table kernel
    checks every byte against the guess; a byte the sample missed makes the engine score the call again with the
    exact alphabet. Batches of more than 1 MiB per tape whose last pairs hold a fifth symbol in the shorter string,
    the longer one, or both, all equal the oracle, as does a device-resident tape whose bytes after its last string
    lie outside the alphabet."""
    rng = np.random.default_rng(101)
    count = 9000
    first = random_strings(rng, count, 100, 200, DNA)
    second = random_strings(rng, count, 150, 300, DNA)  # second strings are the longer ones (texts)
    if where in ("pattern", "both"):
        first[-3] = first[-3][:50] + b"N" + first[-3][51:]
    if where in ("text", "both"):
        second[-2] = second[-2][:70] + b"NN" + second[-2][72:]
    engine = szs.LevenshteinDistances()
    want = port.pairs(oracle.levenshtein_costs(), tape(first), tape(second))
    for schedule in ("batched", "plain"):
        engine.set_schedule(schedule)
        got = engine.pairwise(szs.Strs(first), szs.Strs(second)).astype(np.int64)
        np.testing.assert_array_equal(got, want)
    engine.set_schedule("batched")
    # Device-resident tapes with bytes outside the alphabet right after the last string.
    import torch
    data_a, offsets_a = tape(first)
    data_b, offsets_b = tape(second)
    padded_a = np.concatenate([data_a, np.frombuffer(b"ZZZZZZZZZZZZZZZZ", dtype=np.uint8)])
    padded_b = np.concatenate([data_b, np.frombuffer(b"\x00" * 16, dtype=np.uint8)])
    a = szs.Strs.from_buffers(torch.from_numpy(padded_a).cuda(), torch.from_numpy(offsets_a.astype(np.int64)).cuda())
    b = szs.Strs.from_buffers(torch.from_numpy(padded_b).cuda(), torch.from_numpy(offsets_b.astype(np.int64)).cuda())
    np.testing.assert_array_equal(engine.pairwise(a, b).astype(np.int64), want)
    np.testing.assert_array_equal(engine.pairwise(b, a).astype(np.int64), want)


def test_sampled_alphabet_with_other_routes(szs, port):
    """A guessed DNA alphabet with a long pair on the warp-per-pair route, and a cross product over a five-symbol
    batch: both fall back to the exact alphabet before scoring."""
    rng = np.random.default_rng(102)
    first = random_strings(rng, 7000, 100, 200, DNA) + [bytes(rng.choice(DNA, size=3000))]
    second = random_strings(rng, 7000, 100, 300, DNA) + [bytes(rng.choice(DNA, size=3200))]
    engine = szs.LevenshteinDistances()
    got = engine.pairwise(szs.Strs(first), szs.Strs(second)).astype(np.int64)
    np.testing.assert_array_equal(got, port.pairs(oracle.levenshtein_costs(), tape(first), tape(second)))
    five = np.frombuffer(b"ACGTN", dtype=np.uint8)
    queries = random_strings(rng, 40, 0, 300, five)
    candidates = random_strings(rng, 30, 0, 300, DNA)
    got = engine(szs.Strs(queries), szs.Strs(candidates)).astype(np.int64)
    np.testing.assert_array_equal(got, port.cross(oracle.levenshtein_costs(), tape(queries), tape(candidates)))


@pytest.mark.parametrize("name,family,costs", ENGINES, ids=[e[0] for e in ENGINES])
def test_short_pairs_every_segment_shape(szs, port, name, family, costs):
    """Shorter sides up to 128 take the segmented short-pair kernel (segments of 16 to 128 rows, two pairs per
    segment; 8 rows per lane for protein profiles, 16 for DNA, 12 for the 24-, 48- and 96-row shapes): every shape and
    both sides of each shape's limit, partners from 1 to 600 characters, odd counts that leave segments and halves
    empty, both schedules, and the short threshold tuned down."""
    rng = np.random.default_rng(zlib_seed(name))
    alphabet = DNA if family != "nw" or name == "nw-positive-gaps" else PROTEIN
    b2c, table = dna_tables() if alphabet is DNA else protein_tables(rng, symmetric=False)
    lengths = [(int(rng.integers(1, 129)), int(rng.integers(1, 300))) for _ in range(333)]
    lengths += [(n, m) for n in (1, 2, 15, 16, 17, 23, 24, 25, 31, 32, 33, 47, 48, 49, 63, 64, 65, 95, 96, 97, 127, 128)
                for m in (1, 3, 64, 65, 600)]
    first = [bytes(rng.choice(alphabet, size=n)) for n, _ in lengths]
    second = [bytes(rng.choice(alphabet, size=m)) for _, m in lengths]
    for k in range(0, len(first), 7):
        first[k], second[k] = second[k], first[k]  # the short string on the second side
    engine, oracle_costs = make_engine(szs, family, costs, b2c, table)
    want = port.pairs(oracle_costs, tape(first), tape(second))
    for schedule in ("batched", "plain"):
        engine.set_schedule(schedule)
        got = engine.pairwise(szs.Strs(first), szs.Strs(second)).astype(np.int64)
        bad = np.flatnonzero(got != want)
        assert bad.size == 0, f"{name} {schedule}: {bad.size} mismatches, first {bad[:5]}: {got[bad[:5]]} vs {want[bad[:5]]}"
    engine.set_schedule("batched")
    for short_rows in (16, 24, 32, 48, 64, 96):
        engine.set_tuning({"short_max_rows": short_rows})
        np.testing.assert_array_equal(engine.pairwise(szs.Strs(first), szs.Strs(second)).astype(np.int64), want)
    engine.set_tuning(None)
    queries, candidates = first[:23], second[:17]
    np.testing.assert_array_equal(engine(szs.Strs(queries), szs.Strs(candidates)).astype(np.int64),
                                  port.cross(oracle_costs, tape(queries), tape(candidates)))


@pytest.mark.parametrize("costs", [(0, 2, 3, 1), (0, 3, 2, 2), (3, 1, 5, 5), (0, 5, 3, 1)])
def test_short_pairs_compare_mode(szs, port, costs):
    """Levenshtein over more than 32 byte values on the short-pair kernel compares codes: both cost forms, codes 0 and
    255 side by side."""
    rng = np.random.default_rng(sum(costs) + 500)
    letters = np.arange(256, dtype=np.uint8)
    lengths = [(int(rng.integers(1, 129)), int(rng.integers(1, 200))) for _ in range(301)]
    first = [bytes(rng.choice(letters, size=n)) for n, _ in lengths]
    second = [bytes(rng.choice(letters, size=m)) for _, m in lengths]
    first[0], second[0] = b"\x00\xff" * 20, b"\xff\x00" * 30
    engine = szs.LevenshteinDistances(*costs)
    want = port.pairs(oracle.levenshtein_costs(*costs), tape(first), tape(second))
    for schedule in ("batched", "plain"):
        engine.set_schedule(schedule)
        np.testing.assert_array_equal(engine.pairwise(szs.Strs(first), szs.Strs(second)).astype(np.int64), want)


@pytest.mark.parametrize("longest", [64, 65], ids=["all-short", "one-long"])
def test_tiny_token_cross_product_in_place(szs, port, longest):
    """Unit-cost cross products of tokens of at most 64 bytes into device-resident matrices are scored by one
    thread per cell without planning; a token of 65 bytes makes the call take the general path. Empty tokens,
    one- and two-word patterns, 32- and 64-bit offsets, and a row stride wider than the candidates."""
    import torch
    rng = np.random.default_rng(longest)
    letters = np.arange(256, dtype=np.uint8)
    queries = [bytes(rng.choice(letters, size=int(n))) for n in rng.integers(0, 41, size=150)]
    candidates = [bytes(rng.choice(letters[:6], size=int(n))) for n in rng.integers(0, 41, size=90)]
    queries[3], queries[4], candidates[5] = b"", bytes(rng.choice(letters, size=64)), bytes(rng.choice(letters, size=longest))
    queries[7] = candidates[8] = bytes(rng.choice(letters[:6], size=33))
    want = port.cross(oracle.levenshtein_costs(), tape(queries), tape(candidates))
    engine = szs.LevenshteinDistances()
    for bits in (32, 64):
        def device(items):
            data, offsets = tape(items)
            return szs.Strs.from_buffers(torch.from_numpy(data.copy()).cuda(),
                                         torch.from_numpy(offsets.astype(np.int32 if bits == 32 else np.int64)).cuda())
        out = torch.full((len(queries), len(candidates) + 3), -1, dtype=torch.int64, device="cuda")
        engine(device(queries), device(candidates), out=out)
        got = out.cpu().numpy()
        np.testing.assert_array_equal(got[:, :len(candidates)], want)
        assert (got[:, len(candidates):] == -1).all()


@pytest.mark.parametrize("schedule", ["batched", "plain"])
def test_long_unit_levenshtein_chain(szs, port, schedule):
    """Unit-cost pairs whose shorter side passes 8,192 characters take a chain of warps (1,024 rows each, bits handed
    from warp to warp through global memory): lengths just past the limit, across warp and CTA boundaries, a 50,000
    character mutant pair, a pair with the pattern on the second side, and one pair per chain launch."""
    from stringzillas_gb300 import workloads as w
    rng = np.random.default_rng(123)
    first, second = [], []
    for n in (8193, 9216, 10000, 20480 + 7):
        first.append(bytes(rng.choice(DNA, size=n)))
        second.append(bytes(rng.choice(DNA, size=n + int(rng.integers(-100, 3000)))))
    a = DNA[rng.integers(0, 4, size=50000)]
    b, _ = w._mutate(rng, a, np.array([0, 50000]), DNA, 0.03, 0.01)
    first.append(bytes(b)), second.append(bytes(a))  # the shorter string on either side
    first.append(bytes(rng.choice(DNA, size=40))), second.append(bytes(rng.choice(DNA, size=9000)))
    engine = szs.LevenshteinDistances()
    engine.set_schedule(schedule)
    got = engine.pairwise(szs.Strs(first), szs.Strs(second)).astype(np.int64)
    np.testing.assert_array_equal(got, port.pairs(oracle.levenshtein_costs(), tape(first), tape(second)))


def test_long_unit_levenshtein_chain_wait_gives_up(szs, port):
    """The chain's waits are bounded like the bands': tuned down to one poll they give up, the call reports an error,
    and the next call at the built-in bound is exact."""
    rng = np.random.default_rng(124)
    first = [bytes(rng.choice(DNA, size=30000))]
    second = [bytes(rng.choice(DNA, size=30500))]
    engine = szs.LevenshteinDistances()
    engine.set_tuning({"band_wait_polls": 1})
    with pytest.raises(RuntimeError, match="bounded wait"):
        engine.pairwise(szs.Strs(first), szs.Strs(second))
    engine.set_tuning(None)
    np.testing.assert_array_equal(engine.pairwise(szs.Strs(first), szs.Strs(second)).astype(np.int64),
                                  port.pairs(oracle.levenshtein_costs(), tape(first), tape(second)))


def test_long_unit_levenshtein_chain_waves(szs, port):
    """Many long unit-cost pairs at once: chains side by side in waves of cooperative launches (several waves here),
    each pair's result equal to the oracle's."""
    rng = np.random.default_rng(125)
    count = 1500
    lengths = rng.integers(8193, 9000, size=count)
    first = [bytes(rng.choice(DNA, size=int(n))) for n in lengths]
    second = [bytes(rng.choice(DNA, size=int(n) + int(rng.integers(0, 200)))) for n in lengths]
    got = szs.LevenshteinDistances().pairwise(szs.Strs(first), szs.Strs(second)).astype(np.int64)
    np.testing.assert_array_equal(got, port.pairs(oracle.levenshtein_costs(), tape(first), tape(second)))
