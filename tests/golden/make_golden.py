"""Generates ``tests/golden/golden.npz``: inputs and the reference's own outputs for them.

Run in a tree where the reference sources are present (it builds ``oracle/_ref/libszs_ref.so`` from them with
``oracle/Makefile`` and reads the reference's BLOSUM62 / NUC.4.4 class folds by compiling a 20-line program against
its headers). The fixture then travels with the repository, so tests on machines without the reference still pin
the oracle and the engine to numbers the reference produced.

Cases:
* ``kat_*``: the hand-checked pairs of the reference's tests (test/similarities.py:124-143, :170-197);
* ``degenerate_*``: the degenerate corpora of test/similarities.py:472-508 under the cost modes of :75-94, as cross
  products and symmetric self-similarity matrices;
* ``random_*``: the batch shapes of test/szs_helpers.py:18-25 (unit Levenshtein, pairwise);
* ``nw_minus_lev``: the NW == -Levenshtein identity setup of test/similarities.py:290-319;
* ``asym_*``: an asymmetric class table, to pin which string indexes the rows of the table;
* ``blosum62_*`` / ``nuc44_*``: the reference's built-in tables (serial.hpp:191-256);
* ``config1``: the whole CPU-runnable benchmark configuration (1,024 DNA pairs);
* ``c3_sample`` / ``c4_sample``: seeded samples of the NW protein and SW long-DNA configurations;
* ``utf8_*``: UTF-8 Levenshtein (code points), known answers, degenerate corpus and random multi-script pairs;
* ``fp_*``: Min-Hash fingerprints in both dimension layouts of the reference's engine.
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
REFERENCE = os.environ.get("SZS_REFERENCE_TREE", "/root/reference")

from oracle import oracle  # noqa: E402
from stringzillas_gb300 import workloads  # noqa: E402

TABLES_PROGRAM = r"""
#include <cstdio>
#include "stringzillas/similarities/serial.hpp"
namespace szs = ashvardanian::stringzillas;
static void dump(char const *name, szs::error_costs_32x32_t const &t) {
    std::printf("%s", name);
    for (int i = 0; i < 256; ++i) std::printf(" %d", (int)t.byte_to_class[i]);
    for (int i = 0; i < 32; ++i)
        for (int j = 0; j < 32; ++j) std::printf(" %d", (int)t.class_substitution_costs[i][j]);
    std::printf("\n");
}
int main() {
    dump("blosum62", szs::error_costs_32x32_t::blosum62());
    dump("nuc44", szs::error_costs_32x32_t::nuc44());
}
"""


def reference_tables():
    with tempfile.TemporaryDirectory() as tmp:
        source = os.path.join(tmp, "tables.cpp")
        binary = os.path.join(tmp, "tables")
        with open(source, "w") as f:
            f.write(TABLES_PROGRAM)
        subprocess.run(["g++", "-std=c++20", "-O1", "-w", f"-I{REFERENCE}/include", f"-I{REFERENCE}/forkunion/include",
                        "-DSZ_USE_CUDA=0", "-DSZ_DYNAMIC_DISPATCH=0", "-DFU_WITH_TOPOLOGY=0", source, "-o", binary],
                       check=True)
        out = subprocess.run([binary], check=True, capture_output=True, text=True).stdout
    tables = {}
    for line in out.strip().splitlines():
        name, *values = line.split()
        values = np.array([int(v) for v in values])
        tables[name] = (values[:256].astype(np.uint8), values[256:].astype(np.int8).reshape(32, 32))
    return tables


def tape(strings):
    strings = [s if isinstance(s, bytes) else s.encode() for s in strings]
    data = np.frombuffer(b"".join(strings), dtype=np.uint8) if strings else np.zeros(0, dtype=np.uint8)
    offsets = np.zeros(len(strings) + 1, dtype=np.uint64)
    offsets[1:] = np.cumsum([len(s) for s in strings])
    return data.copy(), offsets


MODES = {"pairwise": 0, "cross": 1, "symmetric": 2}


class Fixture:
    def __init__(self):
        self.ref = oracle.Reference()
        self.arrays = {}
        self.names = []
        self.fingerprint_names = []

    def add(self, name, costs, mode, queries, candidates=None):
        q = tape(queries)
        c = tape(candidates) if candidates is not None else (np.zeros(0, np.uint8), np.zeros(1, np.uint64))
        if mode == "pairwise":
            expected = self.ref.pairs(costs, q, c)
        elif mode == "cross":
            expected = self.ref.cross(costs, q, c)
        else:
            expected = self.ref.cross(costs, q)
        prefix = f"{name}__"
        self.arrays[prefix + "kind"] = np.array([costs.kind])
        self.arrays[prefix + "costs"] = np.array([costs.match, costs.mismatch, costs.open, costs.extend], np.int8)
        self.arrays[prefix + "utf8"] = np.array([costs.utf8])
        self.arrays[prefix + "b2c"] = np.frombuffer(bytes(costs.byte_to_class), np.uint8).copy()
        self.arrays[prefix + "table"] = np.frombuffer(bytes(costs.class_costs), np.int8).reshape(32, 32).copy()
        self.arrays[prefix + "mode"] = np.array([MODES[mode]])
        self.arrays[prefix + "q_data"], self.arrays[prefix + "q_offsets"] = q
        self.arrays[prefix + "c_data"], self.arrays[prefix + "c_offsets"] = c
        self.arrays[prefix + "expected"] = np.asarray(expected, dtype=np.int64)
        self.names.append(name)

    def add_fingerprints(self, name, dimensions, widths, seed, texts):
        """Min-Hash fingerprints: stored under `fp_<name>__*`, listed in `__fingerprints__`."""
        t = tape(texts)
        hashes, counts = self.ref.fingerprints(dimensions, t, widths, seed)
        prefix = f"fp_{name}__"
        self.arrays[prefix + "params"] = np.array([dimensions, seed], dtype=np.uint64)
        self.arrays[prefix + "widths"] = np.array(widths if widths else [], dtype=np.uint64)
        self.arrays[prefix + "data"], self.arrays[prefix + "offsets"] = t
        self.arrays[prefix + "hashes"], self.arrays[prefix + "counts"] = hashes, counts
        self.fingerprint_names.append(name)

    def save(self, path):
        self.arrays["__names__"] = np.array(self.names)
        self.arrays["__fingerprints__"] = np.array(self.fingerprint_names)
        np.savez_compressed(path, **self.arrays)


def random_strings(rng, count, low, high, alphabet):
    alphabet = np.frombuffer(alphabet, dtype=np.uint8)
    return [bytes(rng.choice(alphabet, size=int(rng.integers(low, high + 1)))) for _ in range(count)]


def main():
    subprocess.run(["make", "-s", "-j8", "-C", os.path.join(REPO, "oracle"), "ref", f"REF={REFERENCE}"], check=True)
    tables = reference_tables()
    fx = Fixture()
    lev = oracle.levenshtein_costs

    kat_first = ["hello", "hello", "", "", "abc", "abc", "abc", "abc", "ggbuzgjux{}l", "abcdefgABCDEFG"]
    kat_second = ["hello", "hell", "", "abc", "", "ac", "a_bc", "adc", "gbuzgjux{}l", "ABCDEFGabcdefg"]
    fx.add("kat_unit", lev(), "pairwise", kat_first, kat_second)
    fx.add("kat_custom_gaps", lev(0, 4, 3, 2), "pairwise", kat_first, kat_second)

    degenerate = ["", "a", "b", "aaaaaaaaaa", "abcdefghijklmnopqrstuvwxyz", "zyxwvutsrqponmlkjihgfedcba",
                  "1234567890" * 5, "a" * 1200 + "b" * 50]
    for mode_name, costs in (("unit", lev()), ("linear", lev(0, 3, 2, 2)), ("affine", lev(0, 4, 5, 2))):
        fx.add(f"degenerate_bytes_{mode_name}", costs, "cross", degenerate, degenerate)
        fx.add(f"degenerate_bytes_{mode_name}_self", costs, "symmetric", degenerate)

    protein_alphabet = "ARNDCQEGHILKMFPSTWYV"
    degenerate_protein = ["", "A", "W", "AAAAAAAAAA", protein_alphabet, protein_alphabet[::-1], "WWWWWWWWWW",
                          "ARNDCQEGHI" * 60]
    b2c, table = tables["blosum62"]
    for kind, kind_name in ((oracle.NEEDLEMAN_WUNSCH, "nw"), (oracle.SMITH_WATERMAN, "sw")):
        for gaps_name, gaps in (("linear", (-5, -5)), ("affine", (-11, -1))):
            costs = oracle.alignment_costs(kind, b2c, table, *gaps)
            fx.add(f"blosum62_{kind_name}_{gaps_name}", costs, "cross", degenerate_protein, degenerate_protein)
            fx.add(f"blosum62_{kind_name}_{gaps_name}_self", costs, "symmetric", degenerate_protein)

    rng = np.random.default_rng(2024)
    letters = b"abcdefghijklmnopqrstuvwxyz"
    for shape_name, (count, low, high) in (("one_large", (1, 50, 1024)), ("few_big", (7, 30, 128)),
                                           ("many_small", (1000, 10, 30))):
        first = random_strings(rng, count, low, high, letters)
        second = random_strings(rng, count, low, high, letters)
        fx.add(f"random_{shape_name}", lev(), "pairwise", first, second)

    b2c_mod = (np.arange(256) % 32).astype(np.uint8)
    minus_one = np.full((32, 32), -1, dtype=np.int8)
    np.fill_diagonal(minus_one, 0)
    first = random_strings(rng, 60, 10, 300, letters)
    second = random_strings(rng, 60, 10, 300, letters)
    fx.add("nw_minus_lev", oracle.alignment_costs(oracle.NEEDLEMAN_WUNSCH, b2c_mod, minus_one, -1, -1), "pairwise",
           first, second)

    asym_b2c = np.zeros(256, dtype=np.uint8)
    asym_b2c[np.frombuffer(protein_alphabet.encode(), np.uint8)] = np.arange(1, 21, dtype=np.uint8)
    asym = np.zeros((32, 32), dtype=np.int8)
    asym[1:21, 1:21] = rng.integers(-6, 7, size=(20, 20))
    queries = random_strings(rng, 12, 1, 400, protein_alphabet.encode())
    candidates = random_strings(rng, 9, 1, 400, protein_alphabet.encode()) + [bytes(reversed(q)) for q in queries[:3]]
    for kind, kind_name in ((oracle.NEEDLEMAN_WUNSCH, "nw"), (oracle.SMITH_WATERMAN, "sw")):
        for gaps_name, gaps in (("linear", (-3, -3)), ("affine", (-4, -1))):
            fx.add(f"asym_{kind_name}_{gaps_name}", oracle.alignment_costs(kind, asym_b2c, asym, *gaps), "cross",
                   queries, candidates)

    n_b2c, n_table = tables["nuc44"]
    first = random_strings(rng, 40, 1, 700, b"ACGTN")
    second = random_strings(rng, 40, 1, 700, b"ACGT")
    fx.add("nuc44_sw_affine", oracle.alignment_costs(oracle.SMITH_WATERMAN, n_b2c, n_table, -5, -2), "pairwise",
           first, second)
    fx.add("nuc44_nw_linear", oracle.alignment_costs(oracle.NEEDLEMAN_WUNSCH, n_b2c, n_table, -4, -4), "pairwise",
           first, second)

    def tape_strings(t, limit=None):
        data, offsets = t
        count = len(offsets) - 1 if limit is None else min(limit, len(offsets) - 1)
        return [bytes(data[offsets[i]:offsets[i + 1]]) for i in range(count)]

    first, second = workloads.levenshtein_reads(1024, 64, 256, 0.05, 0.02, seed=42)
    fx.add("config1", lev(), "pairwise", tape_strings(first), tape_strings(second))

    first, second = workloads.protein_pairs(300, seed=42)
    p_b2c, p_table = workloads.protein_table(seed=42)
    fx.add("c3_sample", oracle.alignment_costs(oracle.NEEDLEMAN_WUNSCH, p_b2c, p_table, -11, -1), "pairwise",
           tape_strings(first, 120), tape_strings(second, 120))

    first, second = workloads.local_dna_pairs(12, low=1000, high=3500, segment_high=1500, seed=42)
    d_b2c, d_table = workloads.dna_table(2, -3)
    fx.add("c4_sample", oracle.alignment_costs(oracle.SMITH_WATERMAN, d_b2c, d_table, -5, -2), "pairwise",
           tape_strings(first), tape_strings(second))

    # UTF-8 Levenshtein: the reference tests' known answers (test/similarities.py:151-166), its degenerate UTF-8
    # corpus (:473, :484-493) under the three cost modes, and random multi-script pairs, some of whose strings end
    # in the middle of a sequence (the decoder then reads on into the next string of the tape).
    utf8 = oracle.levenshtein_utf8_costs
    kat_a = ["hello", "\U0002070e \U00020731 \U00020779 \U00020c53", "\U0001f496", "αβγδ",
             "école", "façade", "Schön", "München", "こんにちは世界"]
    kat_b = ["hell", "\U0002070e\U00020731\U00020779\U00020c53", "\U0001f497", "αγδ",
             "école", "facade", "Schön", "Muenchen", "こんばんは世界"]
    fx.add("utf8_kat_unit", utf8(), "pairwise", kat_a, kat_b)
    fx.add("utf8_kat_custom_gaps", utf8(0, 4, 3, 3), "pairwise", kat_a, kat_b)
    degenerate_utf8 = ["", "x", "é", "\U0001f680", "あ" * 10, "abcXYZ123",
                       "こんにちは世界" * 5, "あ" * 600 + "い" * 20]
    for mode_name, costs in (("unit", utf8()), ("linear", utf8(0, 3, 2, 2)), ("affine", utf8(0, 4, 5, 2))):
        fx.add(f"utf8_degenerate_{mode_name}", costs, "cross", degenerate_utf8, degenerate_utf8)
        fx.add(f"utf8_degenerate_{mode_name}_self", costs, "symmetric", degenerate_utf8)
    letters = list("abcdefghéüñαβжאあい世界\U0001f680\U0001f496")

    def utf8_strings(count, low, high):
        return ["".join(rng.choice(letters, size=int(rng.integers(low, high + 1)))).encode() for _ in range(count)]

    first, second = utf8_strings(80, 0, 120), utf8_strings(80, 0, 120)
    for i in range(0, 79, 9):  # cut inside a multi-byte sequence (never the tape's last string)
        if len(first[i]) > 1 and first[i][-1] >= 0x80:
            first[i] = first[i][:-1]
        if len(second[i]) > 1 and second[i][-1] >= 0x80:
            second[i] = second[i][:-1]
    fx.add("utf8_random_unit", utf8(), "pairwise", first, second)
    fx.add("utf8_random_affine", utf8(0, 2, 3, 1), "pairwise", first, second)
    fx.add("utf8_random_cross", utf8(0, 3, 2, 2), "cross", first[:25], second[:30])

    # Min-Hash fingerprints (include/stringzillas/fingerprints/serial.hpp) in both dimension layouts: 64-dimension
    # slices per width (1,024 dims over the default widths; 128 over two) and widths interleaved per dimension.
    printable = [bytes(rng.integers(32, 127, size=int(rng.integers(0, 400))).astype(np.uint8)) for _ in range(60)]
    printable += [b"", b"a", b"ab", b"abc", b"x" * 31, b"y" * 32, "こんにちは世界".encode() * 3]
    dna_texts = random_strings(rng, 30, 0, 2000, b"ACGT")
    fx.add_fingerprints("default_1024", 1024, None, 0, printable)
    fx.add_fingerprints("sliced_128", 128, [4, 8], 42, printable)
    fx.add_fingerprints("interleaved_100", 100, [3, 5, 7], 0, printable)
    fx.add_fingerprints("interleaved_dna", 96, [2, 3, 31], 123456789, dna_texts)

    path = os.path.join(HERE, "golden.npz")
    fx.save(path)
    print(f"wrote {path}: {len(fx.names)} cases, {os.path.getsize(path) / 1024:.0f} KiB")


if __name__ == "__main__":
    main()
