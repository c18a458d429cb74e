"""Seeded synthetic workloads with the shapes of the engine's benchmark configurations.

No public dataset is named for these workloads; every input is generated here from a ``numpy`` PCG64 seed.
Each generator returns tapes as ``(data: uint8[], offsets: int64[count + 1])`` pairs.

* ``levenshtein_reads``: DNA pairs, first string length uniform in [low, high], second derived from the first by
  per-base substitutions and single-character insertions/deletions (configs "plain Levenshtein" 1,024 pairs
  U[64,256] 5%/2%, and "batched Levenshtein" 1,048,576 pairs U[100,300] 3%/1%).
* ``short_pairs``: DNA or protein pairs with first lengths uniform in [low, high] (16-128 by default) and a mutant
  partner, for the short-pair kernel.
* ``protein_pairs``: 20 amino acids at background frequencies, length log-normal (median 350, sigma 0.6) clipped to
  [50, 2000], partner = a mutant with the requested identity (substitutions plus a small indel rate).
* ``protein_table``: symmetric int8 20x20 scores, diagonal U{4..11}, off-diagonal U{-4..3}, folded into the
  reference's 256-byte class map + 32x32 table (letters -> classes 1..20, everything else -> class 0).
* ``local_dna_pairs``: DNA strings with log-uniform lengths in [1,000, 30,000], each pair sharing one planted
  segment of U{500..5000} bp at random offsets with 10% divergence, random flanks.
* ``dna_table``: match +2 / mismatch -3 over A, C, G, T (classes 1..4), class 0 for other bytes.
* ``serving_requests``: the serving stream's requests: 1-4,096 pairs each (log-uniform), kinds Levenshtein /
  Needleman-Wunsch / Smith-Waterman in ratio 2:1:1, pair lengths log-uniform in [16, 16,384]; Levenshtein pairs are
  DNA reads with 5% substitutions + 2% indels, alignment pairs are proteins with a 70%-identity partner.
"""
from __future__ import annotations

import numpy as np

DNA = np.frombuffer(b"ACGT", dtype=np.uint8)
AMINO_ACIDS = np.frombuffer(b"ARNDCQEGHILKMFPSTWYV", dtype=np.uint8)
PRINTABLE = np.arange(32, 127, dtype=np.uint8)  # the 95 printable ASCII bytes
AMINO_FREQUENCIES = np.array([.074, .052, .045, .054, .025, .034, .054, .074, .026, .068,
                              .099, .058, .025, .047, .039, .057, .051, .013, .032, .073])


def _offsets(lengths) -> np.ndarray:
    offsets = np.zeros(len(lengths) + 1, dtype=np.int64)
    np.cumsum(lengths, out=offsets[1:])
    return offsets


def _letters(rng, alphabet, size, probabilities=None):
    """`size` letters drawn from `alphabet` (uniform, or by `probabilities` at 1/65536 resolution)."""
    if probabilities is None:
        index_type = np.uint8 if len(alphabet) <= 256 else np.int64
        return alphabet[rng.integers(0, len(alphabet), size=size, dtype=index_type)]
    edges = np.cumsum(probabilities / np.sum(probabilities)) * 65536.0
    lut = alphabet[np.minimum(np.searchsorted(edges, np.arange(65536) + 0.5), len(alphabet) - 1)]
    return lut[rng.integers(0, 65536, size=size, dtype=np.uint16)]


def _chance(rng, size, rate):
    """Boolean mask with each entry set with probability `rate` (32-bit threshold)."""
    return rng.integers(0, 1 << 32, size=size, dtype=np.uint64) < np.uint64(int(rate * (1 << 32)))


def _mutate(rng, data, offsets, alphabet, substitution_rate, indel_rate, probabilities=None):
    """Per-base substitutions (always to a different letter) then single-character insertions and deletions.
    Returns the mutated tape; pair i of the result derives from pair i of the input."""
    letters = np.sort(alphabet)
    data = data.copy()
    substitute = np.flatnonzero(_chance(rng, data.shape[0], substitution_rate))
    if substitute.size:
        codes = np.searchsorted(letters, data[substitute])
        shift = rng.integers(1, len(letters), size=codes.shape[0])
        data[substitute] = letters[(codes + shift) % len(letters)]
    delete = _chance(rng, data.shape[0], indel_rate / 2)
    insert = _chance(rng, data.shape[0], indel_rate / 2) & ~delete
    copies = 1 - delete.astype(np.int64) + insert.astype(np.int64)
    mutated = np.repeat(data, copies)
    inserted_at = np.cumsum(copies)[insert] - 1
    mutated[inserted_at] = _letters(rng, alphabet, inserted_at.shape[0], probabilities)
    per_base = np.zeros(data.shape[0] + 1, dtype=np.int64)
    np.cumsum(copies, out=per_base[1:])
    return mutated, per_base[offsets]


def levenshtein_reads(count, low, high, substitution_rate, indel_rate, seed=42):
    """DNA pairs for the Levenshtein configurations."""
    rng = np.random.Generator(np.random.PCG64(seed))
    lengths = rng.integers(low, high + 1, size=count)
    offsets = _offsets(lengths)
    first = _letters(rng, DNA, int(offsets[-1]))
    second, second_offsets = _mutate(rng, first, offsets, DNA, substitution_rate, indel_rate)
    return (first, offsets), (second, second_offsets)


def text_pairs(count, low, high, substitution_rate, indel_rate, seed=42):
    """Printable-text pairs (95 byte values, uniform) for Levenshtein with non-unit costs."""
    rng = np.random.Generator(np.random.PCG64(seed))
    lengths = rng.integers(low, high + 1, size=count)
    offsets = _offsets(lengths)
    first = _letters(rng, PRINTABLE, int(offsets[-1]))
    second, second_offsets = _mutate(rng, first, offsets, PRINTABLE, substitution_rate, indel_rate)
    return (first, offsets), (second, second_offsets)


def byte_pairs(count, low, high, substitution_rate, indel_rate, seed=42):
    """Pairs over all 256 byte values (uniform), for dense 256 x 256 substitution tables."""
    rng = np.random.Generator(np.random.PCG64(seed))
    lengths = rng.integers(low, high + 1, size=count)
    offsets = _offsets(lengths)
    every = np.arange(256, dtype=np.uint8)
    first = _letters(rng, every, int(offsets[-1]))
    second, second_offsets = _mutate(rng, first, offsets, every, substitution_rate, indel_rate)
    return (first, offsets), (second, second_offsets)


def dense_table(seed=42):
    """A seeded asymmetric 256 x 256 int8 table: diagonal 4..11, elsewhere -9..3."""
    rng = np.random.Generator(np.random.PCG64(seed))
    table = rng.integers(-9, 4, size=(256, 256)).astype(np.int8)
    np.fill_diagonal(table, rng.integers(4, 12, size=256).astype(np.int8))
    return table


CJK_FIRST, CJK_COUNT = 0x4E00, 3000  # the first 3,000 CJK unified ideographs: three UTF-8 bytes each


def cjk_pairs(count, low, high, substitution_rate, indel_rate, seed=42):
    """UTF-8 pairs of CJK text (3,000 code points, uniform) for UTF-8 Levenshtein over 16-bit codes: lengths in code
    points; the returned tapes hold UTF-8 bytes, three per code point."""
    rng = np.random.Generator(np.random.PCG64(seed))
    lengths = rng.integers(low, high + 1, size=count)
    offsets = _offsets(lengths)
    alphabet = np.arange(CJK_COUNT, dtype=np.int64)
    first = _letters(rng, alphabet, int(offsets[-1]))
    second, second_offsets = _mutate(rng, first, offsets, alphabet, substitution_rate, indel_rate)

    def encode(indices):
        points = indices + CJK_FIRST
        out = np.empty((points.shape[0], 3), dtype=np.uint8)
        out[:, 0] = 0xE0 | (points >> 12)
        out[:, 1] = 0x80 | ((points >> 6) & 0x3F)
        out[:, 2] = 0x80 | (points & 0x3F)
        return out.reshape(-1)

    return (encode(first), offsets * 3), (encode(second), second_offsets * 3)


def short_pairs(count, low=16, high=128, alphabet="dna", substitution_rate=0.10, indel_rate=0.02, seed=42):
    """Short pairs, first length uniform in [low, high], partner a mutant of it: DNA (uniform letters) or protein
    (background frequencies)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    lengths = rng.integers(low, high + 1, size=count)
    offsets = _offsets(lengths)
    if alphabet == "protein":
        p = AMINO_FREQUENCIES / AMINO_FREQUENCIES.sum()
        first = _letters(rng, AMINO_ACIDS, int(offsets[-1]), p)
        second, second_offsets = _mutate(rng, first, offsets, AMINO_ACIDS, substitution_rate, indel_rate,
                                         probabilities=p)
    else:
        first = _letters(rng, DNA, int(offsets[-1]))
        second, second_offsets = _mutate(rng, first, offsets, DNA, substitution_rate, indel_rate)
    return (first, offsets), (second, second_offsets)


def protein_pairs(count, median=350.0, sigma=0.6, low=50, high=2000, identity=0.70, indel_rate=0.02, seed=42):
    """Protein pairs for the Needleman-Wunsch configuration."""
    rng = np.random.Generator(np.random.PCG64(seed))
    lengths = np.clip(np.rint(rng.lognormal(np.log(median), sigma, size=count)), low, high).astype(np.int64)
    offsets = _offsets(lengths)
    p = AMINO_FREQUENCIES / AMINO_FREQUENCIES.sum()
    first = _letters(rng, AMINO_ACIDS, int(offsets[-1]), p)
    second, second_offsets = _mutate(rng, first, offsets, AMINO_ACIDS, 1.0 - identity, indel_rate, probabilities=p)
    return (first, offsets), (second, second_offsets)


def protein_table(seed=42):
    """(byte_to_class[256] uint8, class_costs[32, 32] int8) of a seeded symmetric 20x20 score matrix."""
    rng = np.random.Generator(np.random.PCG64(seed))
    core = rng.integers(-4, 4, size=(20, 20))
    core = np.triu(core, 1)
    core = core + core.T
    np.fill_diagonal(core, rng.integers(4, 12, size=20))
    byte_to_class = np.zeros(256, dtype=np.uint8)
    byte_to_class[AMINO_ACIDS] = np.arange(1, 21, dtype=np.uint8)
    table = np.zeros((32, 32), dtype=np.int8)
    table[1:21, 1:21] = core
    return byte_to_class, table


def dna_table(match=2, mismatch=-3):
    byte_to_class = np.zeros(256, dtype=np.uint8)
    byte_to_class[DNA] = np.arange(1, 5, dtype=np.uint8)
    table = np.zeros((32, 32), dtype=np.int8)
    table[1:5, 1:5] = mismatch
    np.fill_diagonal(table[1:5, 1:5], match)
    return byte_to_class, table


def local_dna_pairs(count, low=1000, high=30000, segment_low=500, segment_high=5000, divergence=0.10, seed=42):
    """Long DNA pairs sharing one planted, diverged segment, for the Smith-Waterman configuration."""
    rng = np.random.Generator(np.random.PCG64(seed))
    log_low, log_high = np.log(low), np.log(high)
    first_lengths = np.exp(rng.uniform(log_low, log_high, size=count)).astype(np.int64)
    second_lengths = np.exp(rng.uniform(log_low, log_high, size=count)).astype(np.int64)
    first_offsets, second_offsets = _offsets(first_lengths), _offsets(second_lengths)
    first = _letters(rng, DNA, int(first_offsets[-1]))
    second = _letters(rng, DNA, int(second_offsets[-1]))
    segment_lengths = np.minimum(rng.integers(segment_low, segment_high + 1, size=count),
                                 np.minimum(first_lengths, second_lengths))
    for i in range(count):
        length = int(segment_lengths[i])
        a_at = int(first_offsets[i] + rng.integers(0, first_lengths[i] - length + 1))
        b_at = int(second_offsets[i] + rng.integers(0, second_lengths[i] - length + 1))
        segment = first[a_at:a_at + length].copy()
        diverge = rng.random(length) < divergence
        segment[diverge] = _letters(rng, DNA, int(diverge.sum()))
        second[b_at:b_at + length] = segment
    return (first, first_offsets), (second, second_offsets)


def cells(first, second) -> int:
    """Sum over pairs of len(first_i) * len(second_i): the cell count GCUPS divides by."""
    return int(np.dot(np.diff(first[1]).astype(np.int64), np.diff(second[1]).astype(np.int64)))


def serving_requests(count, min_pairs=1, max_pairs=4096, min_length=16, max_length=16384, seed=42,
                     kinds=("lev", "lev", "nw", "sw")):
    """`count` requests of the serving stream: dicts with ``kind`` ("lev", "nw" or "sw"), ``first`` and ``second``
    tapes, ``pairs`` and ``cells``. Kinds are drawn uniformly from `kinds` (2:1:1 by default); each pair's first
    length is log-uniform and its partner is a mutant of it."""
    rng = np.random.Generator(np.random.PCG64(seed))
    kinds = rng.choice(np.array(list(kinds)), size=count)
    pair_counts = np.exp(rng.uniform(np.log(min_pairs), np.log(max_pairs + 1), size=count)).astype(np.int64)
    pair_counts = np.clip(pair_counts, min_pairs, max_pairs)
    requests = []
    p = AMINO_FREQUENCIES / AMINO_FREQUENCIES.sum()
    for kind, pairs in zip(kinds, pair_counts):
        lengths = np.exp(rng.uniform(np.log(min_length), np.log(max_length + 1), size=int(pairs))).astype(np.int64)
        lengths = np.clip(lengths, min_length, max_length)
        offsets = _offsets(lengths)
        if kind == "lev":
            first = _letters(rng, DNA, int(offsets[-1]))
            second, second_offsets = _mutate(rng, first, offsets, DNA, 0.05, 0.02)
        else:
            first = _letters(rng, AMINO_ACIDS, int(offsets[-1]), p)
            second, second_offsets = _mutate(rng, first, offsets, AMINO_ACIDS, 0.30, 0.02, probabilities=p)
        requests.append({"kind": str(kind), "first": (first, offsets), "second": (second, second_offsets),
                         "pairs": int(pairs), "cells": cells((first, offsets), (second, second_offsets))})
    return requests
