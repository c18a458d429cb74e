"""The seeded workload generators produce the configured shapes, deterministically."""
import numpy as np

from stringzillas_gb300 import workloads as w


def test_levenshtein_reads_shape_and_mutation_rates():
    (a, ao), (b, bo) = w.levenshtein_reads(4096, 100, 300, 0.03, 0.01, seed=5)
    lengths = np.diff(ao)
    assert lengths.min() >= 100 and lengths.max() <= 300
    assert set(np.unique(a)) <= set(b"ACGT") and set(np.unique(b)) <= set(b"ACGT")
    delta = np.diff(bo) - lengths
    assert abs(delta.mean()) < 0.2  # insertions and deletions balance
    (a2, _), (b2, _) = w.levenshtein_reads(4096, 100, 300, 0.03, 0.01, seed=5)
    assert np.array_equal(a, a2) and np.array_equal(b, b2)


def test_text_pairs_use_the_printable_bytes():
    (a, ao), (b, bo) = w.text_pairs(4096, 100, 300, 0.05, 0.02, seed=5)
    lengths = np.diff(ao)
    assert lengths.min() >= 100 and lengths.max() <= 300
    assert set(np.unique(a)) == set(range(32, 127)) and set(np.unique(b)) <= set(range(32, 127))
    (a2, _), (b2, _) = w.text_pairs(4096, 100, 300, 0.05, 0.02, seed=5)
    assert np.array_equal(a, a2) and np.array_equal(b, b2)


def test_cjk_pairs_are_utf8_of_the_ideographs():
    (a, ao), (b, bo) = w.cjk_pairs(512, 100, 300, 0.05, 0.02, seed=3)
    lengths = np.diff(ao) // 3
    assert lengths.min() >= 100 and lengths.max() <= 300 and (np.diff(ao) % 3 == 0).all()
    text = a[ao[0]:ao[1]].tobytes().decode("utf-8")
    assert len(text) == lengths[0] and all(0x4E00 <= ord(c) < 0x4E00 + 3000 for c in text)
    assert len(b[bo[0]:bo[1]].tobytes().decode("utf-8")) > 0


def test_protein_pairs_lengths_and_identity():
    (a, ao), (b, bo) = w.protein_pairs(2000, seed=1)
    lengths = np.diff(ao)
    assert lengths.min() >= 50 and lengths.max() <= 2000
    assert 250 < np.median(lengths) < 450
    b2c, table = w.protein_table(seed=1)
    core = table[1:21, 1:21]
    assert np.array_equal(core, core.T)
    assert core.diagonal().min() >= 4 and core.diagonal().max() <= 11
    off = core[~np.eye(20, dtype=bool)]
    assert off.min() >= -4 and off.max() <= 3
    assert (b2c != 0).sum() == 20


def test_local_dna_pairs_share_a_segment():
    (a, ao), (b, bo) = w.local_dna_pairs(8, low=1000, high=4000, seed=3)
    lengths = np.diff(ao)
    assert lengths.min() >= 1000 and lengths.max() <= 4000
    assert w.cells((a, ao), (b, bo)) == int(np.dot(np.diff(ao), np.diff(bo)))
