"""The oracle (C restatement) against the reference's own outputs, and its internal consistency. CPU only."""
import os

import numpy as np
import pytest

from conftest import tape
from oracle import oracle

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "golden.npz")


def golden_cases():
    with np.load(GOLDEN) as data:
        names = list(data["__names__"])
        cases = {}
        for name in names:
            cases[name] = {field: data[f"{name}__{field}"] for field in
                           ("kind", "costs", "b2c", "table", "mode", "q_data", "q_offsets", "c_data", "c_offsets",
                            "expected", "utf8")}
    return cases


CASES = golden_cases()


def costs_of(case):
    kind = int(case["kind"][0])
    match, mismatch, open_, extend = (int(x) for x in case["costs"])
    if kind == oracle.LEVENSHTEIN:
        if int(case["utf8"][0]):
            return oracle.levenshtein_utf8_costs(match, mismatch, open_, extend)
        return oracle.levenshtein_costs(match, mismatch, open_, extend)
    return oracle.alignment_costs(kind, case["b2c"], case["table"], open_, extend)


@pytest.mark.parametrize("name", sorted(CASES))
def test_port_matches_reference_outputs(port, name):
    case = CASES[name]
    costs = costs_of(case)
    mode = int(case["mode"][0])
    q = (case["q_data"], case["q_offsets"])
    c = (case["c_data"], case["c_offsets"])
    if mode == 0:
        got = port.pairs(costs, q, c, threads=2)
    elif mode == 1:
        got = port.cross(costs, q, c, threads=2)
    else:
        got = port.cross(costs, q, None, threads=2)
    np.testing.assert_array_equal(got, case["expected"])


def test_golden_covers_the_reference_known_answers():
    """Spot values the reference's tests assert by hand (test/similarities.py:134-143, :188-197)."""
    unit = CASES["kat_unit"]["expected"]
    assert list(unit) == [0, 1, 0, 3, 3, 1, 1, 1, 1, 14]
    custom = CASES["kat_custom_gaps"]["expected"]
    mismatch, opening, extension = 4, 3, 2
    assert list(custom) == [0, opening, 0, opening + 2 * extension, opening + 2 * extension, opening, opening,
                            mismatch, opening, min(14 * mismatch, 2 * opening + 12 * extension)]


def test_golden_covers_the_reference_utf8_known_answers():
    """The UTF-8 pairs the reference's tests assert by hand (test/similarities.py:159-166): code points, not bytes."""
    assert list(CASES["utf8_kat_unit"]["expected"]) == [1, 3, 1, 1, 2, 1, 2, 2, 2]


def test_bit_parallel_equals_dynamic_programming(port):
    """Unit Levenshtein goes through the bit-parallel method; NW with a -1/0 table and -1 gaps (a DP) is its
    negation."""
    rng = np.random.default_rng(0)
    alphabet = np.frombuffer(b"ACGTacgtNx", np.uint8)
    first = [bytes(rng.choice(alphabet, size=int(rng.integers(0, 700)))) for _ in range(150)]
    second = [bytes(rng.choice(alphabet, size=int(rng.integers(0, 700)))) for _ in range(150)]
    b2c = np.arange(256, dtype=np.uint8) % 32
    b2c[np.frombuffer(b"ACGTacgtNx", np.uint8)] = np.arange(1, 11)
    table = np.full((32, 32), -1, dtype=np.int8)
    np.fill_diagonal(table, 0)
    lev = port.pairs(oracle.levenshtein_costs(), tape(first), tape(second))
    nw = port.pairs(oracle.alignment_costs(oracle.NEEDLEMAN_WUNSCH, b2c, table, -1, -1), tape(first), tape(second))
    np.testing.assert_array_equal(lev, -nw)


def test_threads_do_not_change_results(port):
    rng = np.random.default_rng(1)
    first = [bytes(rng.choice(np.frombuffer(b"ACGT", np.uint8), size=int(rng.integers(0, 300)))) for _ in range(300)]
    second = [bytes(rng.choice(np.frombuffer(b"ACGT", np.uint8), size=int(rng.integers(0, 300)))) for _ in range(300)]
    costs = oracle.levenshtein_costs(0, 4, 5, 2)
    np.testing.assert_array_equal(port.pairs(costs, tape(first), tape(second), threads=1),
                                  port.pairs(costs, tape(first), tape(second), threads=8))


@pytest.mark.skipif(not oracle.reference_available(), reason="reference library not built in this tree")
def test_port_matches_reference_library_on_random_inputs(port):
    """Where the reference tree is present, compare directly over all cost modes and an asymmetric table."""
    ref = oracle.Reference()
    rng = np.random.default_rng(3)
    b2c = np.zeros(256, np.uint8)
    b2c[np.frombuffer(b"ACGT", np.uint8)] = [1, 2, 3, 4]
    table = rng.integers(-5, 6, size=(32, 32)).astype(np.int8)
    modes = [oracle.levenshtein_costs(), oracle.levenshtein_costs(0, 3, 2, 2), oracle.levenshtein_costs(1, 2, 6, 1),
             oracle.alignment_costs(oracle.NEEDLEMAN_WUNSCH, b2c, table, -3, -1),
             oracle.alignment_costs(oracle.SMITH_WATERMAN, b2c, table, -3, -1),
             oracle.alignment_costs(oracle.NEEDLEMAN_WUNSCH, b2c, table, -2, -2),
             oracle.alignment_costs(oracle.SMITH_WATERMAN, b2c, table, 2, 1)]
    for costs in modes:
        q = [bytes(rng.choice(np.frombuffer(b"ACGTN", np.uint8), size=int(rng.integers(0, 90)))) for _ in range(7)]
        c = [bytes(rng.choice(np.frombuffer(b"ACGT", np.uint8), size=int(rng.integers(0, 90)))) for _ in range(6)]
        np.testing.assert_array_equal(port.cross(costs, tape(q), tape(c)), ref.cross(costs, tape(q), tape(c)))
        np.testing.assert_array_equal(port.cross(costs, tape(q)), ref.cross(costs, tape(q)))


def _fingerprint_cases():
    with np.load(GOLDEN) as data:
        return {str(name): {k.split("__", 1)[1]: data[k] for k in data.files if k.startswith(f"fp_{name}__")}
                for name in data["__fingerprints__"]}


FINGERPRINTS = _fingerprint_cases()


@pytest.mark.parametrize("name", sorted(FINGERPRINTS))
def test_fingerprints_match_reference_outputs(name):
    """The oracle's integer restatement of the Min-Hash engine against the reference library's own outputs."""
    case = FINGERPRINTS[name]
    dimensions, seed = (int(x) for x in case["params"])
    widths = [int(w) for w in case["widths"]] or None
    hashes, counts = oracle.fingerprints(dimensions, (case["data"], case["offsets"]), widths, seed)
    np.testing.assert_array_equal(hashes, case["hashes"])
    np.testing.assert_array_equal(counts, case["counts"])
