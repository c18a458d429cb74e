"""The benchmark configurations at their full sizes: exact parity where the oracle is fast enough (the bit-parallel
Levenshtein batch), sampled parity plus size-independent properties elsewhere (swap symmetry under symmetric
tables, self-alignment scores, bounds, batched == plain)."""
import numpy as np
import pytest

from oracle import oracle
from stringzillas_gb300 import workloads as w

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def szs():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    import stringzillas_gb300
    return stringzillas_gb300


@pytest.fixture(scope="module")
def port():
    return oracle.Port()


def _strs(szs, tape):
    return szs.to_device(szs.Strs.from_buffers(tape[0], tape[1].astype(np.uint64)))


def _subset(tape, picks):
    data, offsets = tape
    lengths = (offsets[picks + 1] - offsets[picks]).astype(np.int64)
    sub_offsets = np.concatenate([[0], np.cumsum(lengths)]).astype(np.uint64)
    sub_data = np.concatenate([data[offsets[i]:offsets[i + 1]] for i in picks]) if len(picks) else data[:0]
    return sub_data, sub_offsets


def test_batched_levenshtein_full_size(szs, port):
    """1,048,576 DNA pairs, lengths U[100, 300]: every distance equals the oracle's (bit-parallel on all host
    cores), swapping the sides changes nothing, and every distance respects |n - m| <= d <= max(n, m)."""
    first, second = w.levenshtein_reads(1 << 20, 100, 300, 0.03, 0.01, seed=42)
    engine = szs.LevenshteinDistances()
    a, b = _strs(szs, first), _strs(szs, second)
    got = engine.pairwise(a, b).astype(np.int64)
    np.testing.assert_array_equal(got, port.pairs(oracle.levenshtein_costs(), first, second))
    np.testing.assert_array_equal(engine.pairwise(b, a).astype(np.int64), got)
    n, m = np.diff(first[1]).astype(np.int64), np.diff(second[1]).astype(np.int64)
    assert (got >= np.abs(n - m)).all() and (got <= np.maximum(n, m)).all()
    assert (engine.pairwise(a, a) == 0).all()


def test_protein_needleman_wunsch_full_size(szs, port):
    """262,144 protein pairs (lengths lognormal(350, 0.6) in [50, 2000], affine -11/-1): a seeded sample equals the
    oracle, the symmetric table makes scores swap-invariant over all pairs, and the plain form agrees."""
    first, second = w.protein_pairs(262144, seed=42)
    b2c, table = w.protein_table(seed=42)
    engine = szs.NeedlemanWunschScores(b2c, table, open=-11, extend=-1)
    a, b = _strs(szs, first), _strs(szs, second)
    got = engine.pairwise(a, b).astype(np.int64)
    picks = np.sort(np.random.default_rng(0).choice(len(got), size=4096, replace=False))
    want = port.pairs(oracle.alignment_costs(oracle.NEEDLEMAN_WUNSCH, b2c, table, -11, -1),
                      _subset(first, picks), _subset(second, picks))
    np.testing.assert_array_equal(got[picks], want)
    np.testing.assert_array_equal(engine.pairwise(b, a).astype(np.int64), got)
    engine.set_schedule("plain")
    np.testing.assert_array_equal(engine.pairwise(a, b).astype(np.int64), got)


def test_long_dna_smith_waterman_full_size(szs, port):
    """8,192 long DNA pairs (lengths log-uniform [1,000, 30,000], planted shared segments, +2/-3, -5/-2): the 48
    smallest pairs and 16 of the largest (8 with both sides of 25k-30k characters, 8 more from the top decile by
    cells, which holds half of the batch's cells) equal the oracle on all host cores, scores are swap-invariant and within [0, 2 min(n, m)], and each
    string aligned with itself scores 2 per base."""
    first, second = w.local_dna_pairs(8192, seed=42)
    b2c, table = w.dna_table(2, -3)
    engine = szs.SmithWatermanScores(b2c, table, open=-5, extend=-2)
    a, b = _strs(szs, first), _strs(szs, second)
    got = engine.pairwise(a, b).astype(np.int64)
    n, m = np.diff(first[1]).astype(np.int64), np.diff(second[1]).astype(np.int64)
    assert (got >= 0).all() and (got <= 2 * np.minimum(n, m)).all()
    smallest = np.sort(np.argsort(n * m)[:48])
    want = port.pairs(oracle.alignment_costs(oracle.SMITH_WATERMAN, b2c, table, -5, -2),
                      _subset(first, smallest), _subset(second, smallest))
    np.testing.assert_array_equal(got[smallest], want)
    cells, shorter = n * m, np.minimum(n, m)
    pick = np.random.default_rng(2)
    longest = pick.choice(np.flatnonzero(shorter >= 25000), size=8, replace=False)
    top_decile = np.setdiff1d(np.flatnonzero(cells >= np.percentile(cells, 90)), longest)
    largest = np.sort(np.concatenate([longest, pick.choice(top_decile, size=8, replace=False)]))
    want = port.pairs(oracle.alignment_costs(oracle.SMITH_WATERMAN, b2c, table, -5, -2),
                      _subset(first, largest), _subset(second, largest))
    np.testing.assert_array_equal(got[largest], want)
    np.testing.assert_array_equal(engine.pairwise(b, a).astype(np.int64), got)
    picks = np.sort(np.random.default_rng(1).choice(8192, size=256, replace=False))
    sub = _strs(szs, _subset(first, picks))
    np.testing.assert_array_equal(engine.pairwise(sub, sub).astype(np.int64), 2 * n[picks])
