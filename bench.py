#!/usr/bin/env python3
"""Benchmark of the GB300 batched scoring engine.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload c2|c1|c3|c4]

One step = one pass of the engine over one whole batch: every pair of the workload scored through the C-ABI
(`szs_*_pairwise_u64tape`). The headline workload is the batched-Levenshtein configuration: 1,048,576 DNA pairs,
lengths U[100,300], partner = 3% substitutions + 1% indels, unit costs. Inputs are seeded synthetic data.

* `value`: GCUPS (sum of len(a)*len(b) over pairs / seconds) with inputs resident in HBM, timed with CUDA events on the
  stream the engine runs on (a scope bound to torch's current stream), K steps between barriers.
* `e2e`: the same through the same C-ABI call with pinned HOST tapes and a host result array: the engine's H2D copy
  of the inputs and D2H copy of the results are inside the timed region.
* `plain`: the same device-resident measurement with the engine's plain schedule (one launch of one kernel shape
  over the pairs in input order).
* `roofline`: the scoring kernels' algorithmic HBM bytes per step over their event-timed duration, against the
  measured copy bandwidth; `roofline_int`: their algorithmic integer operations against the integer issue rate
  measured live by `szs_gb300_measure_integer_peaks` (the bound that actually applies to this path).
* `cpu_baseline`: the oracle's C restatement (bit-parallel for unit costs) on all host cores.

`--impl reference` times that CPU implementation alone and prints its line (rank 0 only under torchrun).
Multi-GPU (torchrun): every rank scores its own batch (seed + rank), no data-path collective; the time is the
maximum over ranks and `value` aggregates all ranks' cells (weak scaling).
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "GCUPS batched Levenshtein/NW/SW, 1 GB300, vs plain launch; serving p50/p99 ms"

# Algorithmic integer operations per DP cell of each route, counted from the kernels' recurrences:
#  - bit-parallel (unit Levenshtein): per 32-cell word and column, B code-plane LOP3s + 11 ops of the Myers step
#    (Xv, Eq&Pv, 2-op carried add, Xh, Ph, Mh, two funnel shifts, Pv, Mv); DNA needs B = 2 -> 13 / 32 per cell.
#  - wavefront, 32-bit cells: linear 4 = opt(up, left) + (diag + s) + fused add-opt + cost unpack;
#    affine 7 = E (add + fused add-opt) + F (add + fused add-opt) + (diag + s) + 3-way opt + cost unpack.
#  - 16x2 packed cells (the NW / SW configurations run there: warp route and 16-bit band): per register of two
#    cells, affine 5 DPX (E, diag + s against E, F, max, + open) + 1 byte permute of the two pairs' costs, plus the
#    running maximum for local scores -> 3.0 (global) / 3.5 (local) per cell.
#  - 16x2 compare mode (Levenshtein over more than 32 byte values): per register of two cells, affine 5 DPX + 1 DPX
#    add-min (0 where the codes are equal, else 1) + 1 multiply-add giving both pairs' costs -> 3.5 per cell.
#  - bit-parallel over at most four symbols (the shared-table kernel, DNA): the match masks come from shared memory,
#    so per word and column only the 10 ops of the Myers step remain -> 10 / 32 per cell.
OPS_PER_CELL = {"myers_dna": 13.0 / 32.0, "myers_dna_table": 10.0 / 32.0, "dp_linear": 4.0, "dp_affine": 7.0,
                "packed_affine": 3.0, "packed_affine_local": 3.5, "packed_compare_affine": 3.5}

WORKLOADS = {
    "c1": "plain Levenshtein: 1,024 DNA pairs, len U[64,256], partner 5% subs + 2% indels, unit costs",
    "c2": "batched Levenshtein: 1,048,576 DNA pairs, len U[100,300], partner 3% subs + 1% indels, unit costs",
    "c3": "Needleman-Wunsch affine protein: 262,144 pairs, len lognormal(350, 0.6) in [50,2000], 70% identity, "
          "seeded symmetric int8 table (diag 4..11, off -4..3), open -11 extend -1",
    "c4": "Smith-Waterman affine DNA: 8,192 pairs, len log-uniform [1,000, 30,000], planted 500-5,000 bp shared "
          "segment with 10% divergence, match +2 mismatch -3 open -5 extend -2",
    # Profiling cases for the 32-bit routes (not bench lines of the default run).
    "p_band32": "profiling case, Needleman-Wunsch affine protein long pairs: 1,024 pairs, len lognormal(4000, 0.3) in "
                "[2500, 8000], 70% identity, open -11 extend -1 (the reach bound exceeds int16: 32-bit band)",
    "p_dp32": "profiling case, Needleman-Wunsch affine protein with a wide table: 65,536 pairs, len lognormal(350, 0.6) "
              "in [50, 2000], diagonal 100..120, open -30 extend -2 (costs outside the int8 profile: 32-bit wavefront)",
    "text": "Levenshtein on printable text: 262,144 pairs, len U[100,300], 95 byte values, partner 5% subs + 2% indels, "
            "match 0 mismatch 2 open 3 extend 1 (16x2 wavefront in compare mode)",
    "p_cjk": "profiling case, UTF-8 Levenshtein on CJK text: 65,536 pairs, len U[100,300] code points of 3,000 "
             "ideographs (three UTF-8 bytes each), partner 5% subs + 2% indels, match 0 mismatch 2 open 3 extend 1 "
             "(16-bit codes; 16x2 wavefront in compare mode)",
    "p_long_lev": "profiling case, unit-cost Levenshtein on long DNA reads: 16,384 pairs, len U[1,000, 4,000], partner 3% "
                  "subs + 1% indels (warp-per-pair bit-parallel kernel)",
    "p_dense": "profiling case, Needleman-Wunsch affine over a dense 256 x 256 table: 131,072 pairs, len U[100,300] over all "
               "256 byte values, partner 10% subs + 2% indels, seeded table (diagonal 4..11, elsewhere -9..3), open -11 "
               "extend -1 (32-bit wavefront reading the whole table from shared memory)",
    "short_nw": "short pairs, Needleman-Wunsch affine protein: 1,048,576 pairs, len U[16, 128], 70% identity, the protein "
                "configuration's table, open -11 extend -1 (segmented short-pair kernel)",
    "short_sw": "short pairs, Smith-Waterman affine DNA: 1,048,576 pairs, len U[16, 128], partner 10% subs + 2% indels, "
                "match +2 mismatch -3 open -5 extend -2 (segmented short-pair kernel)",
    "short_lev": "short pairs, Levenshtein with costs (0, 2, 3, 1) on DNA: 1,048,576 pairs, len U[16, 128], partner 5% "
                 "subs + 2% indels (segmented short-pair kernel)",
}


# DRAM bytes per step of the dominant kernels, from one ncu capture of the same command
# (profiles/myers_table_c2_dram_traffic.txt: dram__bytes_read.sum + dram__bytes_write.sum over one step's launches).
DRAM_TRAFFIC_PER_STEP = {"c2": 702.2e6 + 1.1e6}

# What ncu shows about the dominant kernel's integer pipe, beside the algorithmic fraction above
# (profiles/myers_table_c2_batched_levenshtein.txt).
PIPE_EVIDENCE = {"c2": "ncu, shared-table bit-parallel kernel (W = 8 and 7): ALU pipe 84 % busy, 12.4 ALU instructions "
                       "executed per pattern word and text column against the step's 10 (byte extraction, table "
                       "address, alphabet check, pattern setup)"}


def parse_args():
    parser = argparse.ArgumentParser()
    parser.add_argument("--gpus", type=int, default=1)
    parser.add_argument("--steps", type=int, default=10)
    parser.add_argument("--warmup", type=int, default=3)
    parser.add_argument("--impl", choices=["ours", "reference"], default="ours")
    parser.add_argument("--workload", choices=sorted(WORKLOADS), default="c2")
    parser.add_argument("--no-extra", action="store_true", help="skip the other workloads' lines")
    parser.add_argument("--cpu-seconds", type=float, default=12.0, help="CPU-baseline sample budget")
    parser.add_argument("--fingerprints-only", action="store_true",
                        help="run only the Min-Hash leg and print its JSON object")
    parser.add_argument("--fp-documents", type=int, default=16384, help="documents of the Min-Hash leg")
    parser.add_argument("--cross-only", action="store_true", help="run only the all-pairs leg and print its object")
    parser.add_argument("--serving-only", action="store_true", help="run only the serving leg and print its object")
    parser.add_argument("--long-only", action="store_true", help="run only the long-pair leg and print its object")
    return parser.parse_args()


def _workloads_module():
    """The seeded generators, loaded from their file alone: importing the package would load the engine's library,
    which the CPU arm (``--impl reference``) must not map."""
    import importlib.util
    name = "szs_bench_workloads"
    if name not in sys.modules:
        spec = importlib.util.spec_from_file_location(name, os.path.join(HERE, "stringzillas_gb300", "workloads.py"))
        module = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(module)
        sys.modules[name] = module
    return sys.modules[name]


def make_workload(name, seed):
    w = _workloads_module()
    if name == "c1":
        first, second = w.levenshtein_reads(1024, 64, 256, 0.05, 0.02, seed=seed)
        return first, second, ("lev", None)
    if name == "c2":
        first, second = w.levenshtein_reads(1 << 20, 100, 300, 0.03, 0.01, seed=seed)
        return first, second, ("lev", None)
    if name == "c3":
        first, second = w.protein_pairs(262144, seed=seed)
        return first, second, ("nw", w.protein_table(seed=seed))
    if name == "p_band32":
        first, second = w.protein_pairs(1024, median=4000.0, sigma=0.3, low=2500, high=8000, seed=seed)
        return first, second, ("nw32", (*w.protein_table(seed=seed), -11, -1))
    if name == "p_cjk":
        first, second = w.cjk_pairs(65536, 100, 300, 0.05, 0.02, seed=seed)
        return first, second, ("levu", (0, 2, 3, 1))
    if name == "p_long_lev":
        first, second = w.levenshtein_reads(16384, 1000, 4000, 0.03, 0.01, seed=seed)
        return first, second, ("lev", None)
    if name == "text":
        first, second = w.text_pairs(262144, 100, 300, 0.05, 0.02, seed=seed)
        return first, second, ("levc", (0, 2, 3, 1))
    if name == "short_nw":
        first, second = w.short_pairs(1 << 20, 16, 128, "protein", 0.28, 0.02, seed=seed)
        return first, second, ("nw", w.protein_table(seed=seed))
    if name == "short_sw":
        first, second = w.short_pairs(1 << 20, 16, 128, "dna", 0.10, 0.02, seed=seed)
        return first, second, ("sw", w.dna_table(2, -3))
    if name == "short_lev":
        first, second = w.short_pairs(1 << 20, 16, 128, "dna", 0.05, 0.02, seed=seed)
        return first, second, ("levp", (0, 2, 3, 1))
    if name == "p_dense":
        first, second = w.byte_pairs(131072, 100, 300, 0.10, 0.02, seed=seed)
        return first, second, ("nwd", (w.dense_table(seed=seed), -11, -1))
    if name == "p_dp32":
        first, second = w.protein_pairs(65536, seed=seed)
        byte_to_class, table = w.protein_table(seed=seed)
        table = table.copy()
        diagonal = np.arange(1, 21)
        table[diagonal, diagonal] = 100 + np.arange(20)
        return first, second, ("nw32", (byte_to_class, table, -30, -2))
    first, second = w.local_dna_pairs(8192, seed=seed)
    return first, second, ("sw", w.dna_table(2, -3))


def make_engine(kind_and_tables):
    """The workload's engine with the committed autotuned table installed (if the package has one)."""
    import stringzillas_gb300 as szs
    from stringzillas_gb300 import autotune
    kind, tables = kind_and_tables
    if kind == "lev":
        engine = szs.LevenshteinDistances()
    elif kind in ("levc", "levp"):  # Levenshtein with the given (match, mismatch, open, extend)
        engine = szs.LevenshteinDistances(*tables)
    elif kind == "levu":  # UTF-8 Levenshtein with the given (match, mismatch, open, extend)
        engine = szs.LevenshteinDistancesUTF8(*tables)
    elif kind == "nw":
        engine = szs.NeedlemanWunschScores(*tables, open=-11, extend=-1)
    elif kind == "nw32":  # profiling cases of the 32-bit routes: (byte_to_class, table, open, extend)
        engine = szs.NeedlemanWunschScores(*tables[:2], open=tables[2], extend=tables[3])
    elif kind == "nwd":  # a dense 256 x 256 table: (table, open, extend)
        engine = szs.NeedlemanWunschScores.dense(tables[0], open=tables[1], extend=tables[2])
    else:
        engine = szs.SmithWatermanScores(*tables, open=-5, extend=-2)
    autotune.apply(engine)
    return engine


TUNING_TABLE = os.path.join("stringzillas_gb300", "tuning", "gb300.json")


def tuning_source():
    # Read from the file path (not through the package) so both arms print the same key without loading the engine.
    return "autotuned table " + TUNING_TABLE if os.path.exists(os.path.join(HERE, TUNING_TABLE)) else "built-in"


def workload_config(name, first, second, world):
    """The ``config`` object both arms print for a workload."""
    cells = int(np.dot(np.diff(first[1]).astype(np.int64), np.diff(second[1]).astype(np.int64)))
    return {"workload": WORKLOADS[name], "pairs": len(first[1]) - 1, "cells_per_step": cells,
            "input_bytes_per_step": int(first[0].shape[0] + second[0].shape[0]), "tuning": tuning_source(),
            "l2": "inputs larger than L2 (129 MB), no flush between steps",
            "parallelism": f"pairs: each of {world} ranks scores its own batch, no collective"}


def oracle_costs(kind_and_tables):
    from oracle import oracle
    kind, tables = kind_and_tables
    if kind == "lev":
        return oracle.levenshtein_costs()
    if kind in ("levc", "levp"):
        return oracle.levenshtein_costs(*tables)
    if kind == "levu":
        return oracle.levenshtein_utf8_costs(*tables)
    if kind == "nw":
        return oracle.alignment_costs(oracle.NEEDLEMAN_WUNSCH, *tables, -11, -1)
    if kind == "nw32":
        return oracle.alignment_costs(oracle.NEEDLEMAN_WUNSCH, *tables)
    if kind == "nwd":
        return oracle.dense_costs(oracle.NEEDLEMAN_WUNSCH, *tables)
    return oracle.alignment_costs(oracle.SMITH_WATERMAN, *tables, -5, -2)


def ops_per_cell(kind_and_tables):
    kind = kind_and_tables[0]
    if kind == "lev":
        return OPS_PER_CELL["myers_dna_table"]
    if kind in ("nw32", "nwd"):
        return OPS_PER_CELL["dp_affine"]
    if kind in ("levc", "levu"):
        return OPS_PER_CELL["packed_compare_affine"]
    if kind == "levp":
        return OPS_PER_CELL["packed_affine"]
    return OPS_PER_CELL["packed_affine_local"] if kind == "sw" else OPS_PER_CELL["packed_affine"]


class Clocks:
    """Samples SM clocks and throttle reasons with nvidia-smi while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.device_index = device_index
        self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.process = None

    def __enter__(self):
        try:
            self.process = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "100",
                 "-i", str(self.device_index)], stdout=self.file, stderr=subprocess.DEVNULL)
        except OSError:
            self.process = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.process:
            self.process.terminate()
            try:
                self.process.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.process.kill()
        self.file.flush()

    def summary(self):
        self.file.seek(0)
        rows = [line.strip().split(", ") for line in self.file.read().splitlines() if line.strip()]
        os.unlink(self.file.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(r[1]) for r in rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        sm_max = [float(r[2]) for r in rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for r in rows:
            for name, flag in zip(names, r[5:9]):
                if flag.strip().lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(sm_max) if sm_max else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def measured_peaks():
    try:
        with open(os.path.join(HERE, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
        return float(peaks["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def integer_peaks(device):
    from stringzillas_gb300._native import lib
    rates = (ctypes.c_double * 5)()
    err = ctypes.c_char_p()
    status = lib.szs_gb300_measure_integer_peaks(device, rates, 5, ctypes.byref(err))
    if status != 0:
        return None
    return {"lop3": rates[0], "iadd3": rates[1], "dpx_viaddmax_s32": rates[2], "dpx_vimax3_s32": rates[3],
            "dpx_viaddmax_s16x2": rates[4]}


class DeviceBatch:
    """A workload's tapes in HBM plus the C-ABI structs that point at them."""

    def __init__(self, first, second, torch):
        from stringzillas_gb300 import _native
        self.tensors = []
        self.tapes = []
        for data, offsets in (first, second):
            d = torch.from_numpy(data).cuda()
            o = torch.from_numpy(offsets.astype(np.int64)).cuda()
            self.tensors += [d, o]
            self.tapes.append(_native.U64Tape(d.data_ptr(), o.data_ptr(), len(offsets) - 1))
        self.count = len(first[1]) - 1
        self.out = torch.empty(self.count, dtype=torch.int64, device="cuda")


class HostBatch:
    """The same tapes in pinned host memory, with a pinned host result array."""

    def __init__(self, first, second, torch):
        from stringzillas_gb300 import _native
        self.tensors = []
        self.tapes = []
        self.bytes_in = 0
        for data, offsets in (first, second):
            d = torch.from_numpy(data).pin_memory()
            o = torch.from_numpy(offsets.astype(np.int64)).pin_memory()
            self.tensors += [d, o]
            self.bytes_in += d.numel() + o.numel() * 8
            self.tapes.append(_native.U64Tape(d.data_ptr(), o.data_ptr(), len(offsets) - 1))
        self.count = len(first[1]) - 1
        self.out = torch.empty(self.count, dtype=torch.int64).pin_memory()
        self.bytes_out = self.count * 8


def call_pairwise(engine, scope, batch):
    from stringzillas_gb300._native import lib
    err = ctypes.c_char_p()
    # The Levenshtein pairwise entry point serves the UTF-8 engines too (no separate _utf8 pairwise symbol).
    algo = "levenshtein_distances" if engine._algo.startswith("levenshtein_distances") else engine._algo
    fn = getattr(lib, f"szs_{algo}_pairwise_u64tape")
    status = fn(engine.handle, scope.handle, ctypes.byref(batch.tapes[0]), ctypes.byref(batch.tapes[1]),
                ctypes.c_void_p(batch.out.data_ptr()), ctypes.byref(err))
    if status != 0:
        raise RuntimeError(f"engine call failed ({status}): {err.value}")
    return engine.stats()


def timed_steps(engine, scope, batch, steps, warmup, torch, barrier):
    for _ in range(warmup):
        call_pairwise(engine, scope, batch)
    stream = torch.cuda.current_stream()
    begin, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    barrier()
    begin.record(stream)
    compute_ms, launches, cells = 0.0, 0, 0
    for _ in range(steps):
        stats = call_pairwise(engine, scope, batch)
        compute_ms += stats["last_compute_ms"]
        launches += stats["last_launches"]
        cells += stats["last_cells"]
    end.record(stream)
    torch.cuda.synchronize()
    barrier()
    return begin.elapsed_time(end), compute_ms, launches, cells


def cpu_baseline(first, second, kind_and_tables, seconds_budget):
    """The oracle's C restatement on all host cores over a bounded prefix of the same pairs."""
    from oracle import oracle
    port = oracle.Port()
    costs = oracle_costs(kind_and_tables)
    threads = os.cpu_count() or 1
    count = len(first[1]) - 1

    def sample(k):
        a = (first[0], first[1][:k + 1])
        b = (second[0], second[1][:k + 1])
        t0 = time.perf_counter()
        port.pairs(costs, a, b, threads)
        elapsed = time.perf_counter() - t0
        cells = int(np.dot(np.diff(a[1]).astype(np.int64), np.diff(b[1]).astype(np.int64)))
        return elapsed, cells

    k = max(1, count // 256)
    elapsed, cells = sample(k)
    if elapsed < seconds_budget / 4 and k < count:
        k = min(count, max(k + 1, int(k * seconds_budget / max(elapsed, 1e-3))))
        elapsed, cells = sample(k)
    return {"value": cells / elapsed / 1e9, "unit": "GCUPS", "cores": threads, "kind": "port",
            "sample": f"first {k} of {count} pairs ({cells:.3e} cells, {elapsed:.2f} s), oracle C restatement"}


SERVING_RATES = (120.0, 400.0)  # offered loads, requests per second (Poisson arrivals)
SERVING_AGING_MS = 50     # size-aware admission: a request waiting this long goes first
SERVING_REQUESTS = 240    # requests per run, drawn from a pool of 48 distinct ones
NW_SW_BURST = 64          # requests of the NW / SW-only burst, drawn from a pool of 32


def serving_engines(szs):
    from stringzillas_gb300 import workloads as w
    protein = w.protein_table(seed=42)
    from stringzillas_gb300 import autotune
    engines = {"lev": szs.LevenshteinDistances(),
               "nw": szs.NeedlemanWunschScores(*protein, open=-11, extend=-1),
               "sw": szs.SmithWatermanScores(*protein, open=-11, extend=-1)}
    for engine in engines.values():
        autotune.apply(engine)
    return engines


def serve_stream(szs, server, engines, pool, order, arrivals):
    """Submits pool[order[i]] at host time arrivals[i] (seconds from start); returns per-request infos and the
    wall time from the first submission to the last result."""
    import threading
    strs = [(szs.Strs.from_buffers(*r["first"]), szs.Strs.from_buffers(*r["second"])) for r in pool]
    tickets = [None] * len(order)
    ready = threading.Semaphore(0)

    def submitter(start):
        for i, (k, at) in enumerate(zip(order, arrivals)):
            delay = start + at - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
            tickets[i] = server.submit(engines[pool[k]["kind"]], *strs[k])
            ready.release()

    start = time.perf_counter()
    thread = threading.Thread(target=submitter, args=(start,))
    thread.start()
    infos = []
    for i in range(len(order)):
        ready.acquire()
        tickets[i].result()
        infos.append(tickets[i].info)
    wall = time.perf_counter() - start
    thread.join()
    return infos, wall


def serving_leg(szs):
    """C5: Poisson arrivals at a fixed offered load, and a saturating burst, against the serving loop (merged
    batches, 4 lanes) and the per-request plain form (one lane, one request per batch, plain schedule)."""
    from stringzillas_gb300 import workloads as w
    pool = w.serving_requests(48, seed=42)
    engines = serving_engines(szs)
    rng = np.random.Generator(np.random.PCG64(7))
    order = rng.integers(0, len(pool), size=SERVING_REQUESTS)
    gaps = rng.exponential(1.0, size=SERVING_REQUESTS)  # one seeded arrival pattern, scaled to each load
    cells = int(sum(pool[k]["cells"] for k in order))
    forms = {"serving": dict(lanes=4, arena_bytes=4 << 30),
             "serving_size_aware": dict(lanes=4, arena_bytes=4 << 30, aging_ms=SERVING_AGING_MS),
             "per_request_plain": dict(lanes=1, max_batch_requests=1, schedule="plain", arena_bytes=4 << 30)}
    # The same four lanes without batching: one request per batch, plain schedule (isolates what batching buys).
    same_lanes = {"per_request_plain_4_lanes": dict(lanes=4, max_batch_requests=1, schedule="plain",
                                                    arena_bytes=4 << 30)}
    out = {"offered_requests_per_s": list(SERVING_RATES), "requests": SERVING_REQUESTS, "cells": cells,
           "offered_gcups": [cells / (np.cumsum(gaps / rate))[-1] / 1e9 for rate in SERVING_RATES],
           "mix": "Levenshtein:NW:SW 2:1:1, 1-4,096 pairs per request, pair lengths log-uniform [16, 16,384]",
           "admission": f"serving: oldest waiting request first; serving_size_aware: smallest first, aging bound "
                        f"{SERVING_AGING_MS} ms"}
    for name, config in forms.items():
        row = {}
        with szs.Server(**config) as server:
            serve_stream(szs, server, engines, pool, order[:8], np.zeros(8))  # warm-up: builds lane buffers
            rates = SERVING_RATES if name != "per_request_plain" else SERVING_RATES[:1]
            for rate in rates:
                arrivals = np.cumsum(gaps / rate)
                infos, wall = serve_stream(szs, server, engines, pool, order, arrivals)
                latencies = np.array([i["done_ms"] for i in infos])
                queued = np.array([i["admitted_ms"] for i in infos])
                row[f"{rate:g}_per_s"] = {
                    "p50_ms": float(np.percentile(latencies, 50)), "p99_ms": float(np.percentile(latencies, 99)),
                    "mean_ms": float(latencies.mean()), "queue_p50_ms": float(np.percentile(queued, 50)),
                    "queue_p99_ms": float(np.percentile(queued, 99)),
                    "achieved_gcups_at_offered_load": cells / wall / 1e9}
            burst_infos, burst_wall = serve_stream(szs, server, engines, pool, order, np.zeros(len(order)))
            stats = server.stats()
        row.update({"saturated_gcups": cells / burst_wall / 1e9,
                    "saturated_p99_ms": float(np.percentile([i["done_ms"] for i in burst_infos], 99)),
                    "batches": stats["batches"], "peak_inflight_batches": stats["peak_inflight"],
                    "arena_peak_bytes": stats["arena_peak_bytes"], "kernel_launches": stats["kernel_launches"]})
        out[name] = row
    out["saturated_serving_over_plain"] = (out["serving"]["saturated_gcups"] /
                                           out["per_request_plain"]["saturated_gcups"])
    # The latency floor: each distinct request of the pool served alone on an idle server (one lane, one request
    # per batch, batched schedule), admission to delivery, weighted by how often the stream draws it.
    alone = np.zeros(len(pool))
    with szs.Server(lanes=1, max_batch_requests=1, arena_bytes=4 << 30) as server:
        strs = [(szs.Strs.from_buffers(*r["first"]), szs.Strs.from_buffers(*r["second"])) for r in pool]
        server.submit(engines[pool[0]["kind"]], *strs[0]).result()  # warm-up
        for k, request in enumerate(pool):
            ticket = server.submit(engines[request["kind"]], *strs[k])
            ticket.result()
            alone[k] = ticket.info["done_ms"] - ticket.info["admitted_ms"]
    drawn = alone[order]
    out["service_alone"] = {"p50_ms": float(np.percentile(drawn, 50)), "p99_ms": float(np.percentile(drawn, 99)),
                            "max_ms": float(drawn.max()),
                            "note": "each request scored alone on an idle server: the floor under its latency"}
    # Mixed-length NW / SW only: a saturating burst of alignment requests, both forms.
    nw_sw = w.serving_requests(32, seed=43, kinds=("nw", "sw"))
    burst = rng.integers(0, len(nw_sw), size=NW_SW_BURST)
    burst_cells = int(sum(nw_sw[k]["cells"] for k in burst))
    mix = {"requests": NW_SW_BURST, "cells": burst_cells,
           "mix": "NW:SW 1:1 (affine protein), 1-4,096 pairs per request, pair lengths log-uniform [16, 16,384]"}
    for name, config in {**forms, **same_lanes}.items():
        with szs.Server(**config) as server:
            serve_stream(szs, server, engines, nw_sw, burst[:4], np.zeros(4))
            infos, wall = serve_stream(szs, server, engines, nw_sw, burst, np.zeros(len(burst)))
        mix[name] = {"saturated_gcups": burst_cells / wall / 1e9,
                     "p99_ms": float(np.percentile([i["done_ms"] for i in infos], 99))}
    mix["serving_over_plain"] = mix["serving"]["saturated_gcups"] / mix["per_request_plain"]["saturated_gcups"]
    mix["serving_over_plain_same_lanes"] = (mix["serving"]["saturated_gcups"] /
                                            mix["per_request_plain_4_lanes"]["saturated_gcups"])
    out["nw_sw_burst"] = mix
    return out


# The reference's published all-pairs figures on an H100 (include/stringzillas/similarities/README.md:13-26):
# balanced tiles of equal-length `acgt` sequences, unit cost scheme, GCUPS.
REFERENCE_H100_CROSS_GCUPS = {100: {"levenshtein": 1499.8, "needleman_wunsch": 187.3, "smith_waterman": 164.8},
                              1000: {"levenshtein": 5910.8, "needleman_wunsch": 711.3, "smith_waterman": 615.8}}


def cross_product_leg(szs, torch, scope, steps=10, warmup=3):
    """All-pairs tiles at the reference's published methodology: a balanced square of 256 pairs per SM (q197 x c198
    on 152 SMs) of equal-length `acgt` sequences at 100 and 1,000 bytes, unit costs (Levenshtein 0/1/1; NW and SW
    match 0, mismatch -1, gap -1), device-resident tapes and result matrix, CUDA events over `steps` calls. Plus a
    tiny-token cross product (2,048 x 2,048 printable tokens of 4-16 bytes) on the one-thread-per-cell path."""
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    pairs = 256 * sms
    rows = int(np.sqrt(pairs))
    cols = (pairs + rows - 1) // rows
    stream = torch.cuda.current_stream()
    letters = np.frombuffer(b"acgt", dtype=np.uint8)
    b2c = np.zeros(256, dtype=np.uint8)
    b2c[letters] = [1, 2, 3, 4]
    table = np.zeros((32, 32), dtype=np.int8)
    table[1:5, 1:5] = -1
    np.fill_diagonal(table[1:5, 1:5], 0)
    engines = {"levenshtein": szs.LevenshteinDistances(),
               "needleman_wunsch": szs.NeedlemanWunschScores(b2c, table, open=-1, extend=-1),
               "smith_waterman": szs.SmithWatermanScores(b2c, table, open=-1, extend=-1)}

    def device_strs(data, count, length):
        offsets = np.arange(count + 1, dtype=np.int64) * length
        return szs.Strs.from_buffers(torch.from_numpy(data).cuda(), torch.from_numpy(offsets).cuda())

    def timed(engine, queries, candidates, out):
        for _ in range(warmup):
            engine(queries, candidates, device=scope, out=out)
        begin, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        begin.record(stream)
        for _ in range(steps):
            engine(queries, candidates, device=scope, out=out)
        end.record(stream)
        torch.cuda.synchronize()
        return begin.elapsed_time(end) / steps

    out = {"method": f"balanced all-pairs tile q{rows} x c{cols} (256 pairs per SM x {sms} SMs), equal-length acgt "
                     "sequences, unit costs, device-resident inputs and results, one call per step",
           "tile": [rows, cols]}
    rng = np.random.Generator(np.random.PCG64(11))
    for length in (100, 1000):
        queries = device_strs(letters[rng.integers(0, 4, size=rows * length)], rows, length)
        candidates = device_strs(letters[rng.integers(0, 4, size=cols * length)], cols, length)
        result = torch.empty((rows, cols), dtype=torch.int64, device="cuda")
        cells = rows * cols * length * length
        row = {}
        for name, engine in engines.items():
            ms = timed(engine, queries, candidates, result)
            row[name] = {"GCUPS": cells / (ms * 1e-3) / 1e9, "ms_per_call": ms,
                         "reference_h100_GCUPS": REFERENCE_H100_CROSS_GCUPS[length][name]}
        out[f"{length}_bytes"] = row
    # Tiny tokens: the one-thread-per-cell path.
    count = 2048
    lengths = rng.integers(4, 17, size=2 * count)
    data = rng.integers(32, 127, size=int(lengths.sum()), dtype=np.uint8)
    offsets = np.zeros(2 * count + 1, dtype=np.int64)
    np.cumsum(lengths, out=offsets[1:])
    queries = szs.Strs.from_buffers(torch.from_numpy(data[:offsets[count]].copy()).cuda(),
                                    torch.from_numpy(offsets[:count + 1].copy()).cuda())
    candidates = szs.Strs.from_buffers(torch.from_numpy(data[offsets[count]:].copy()).cuda(),
                                       torch.from_numpy((offsets[count:] - offsets[count]).copy()).cuda())
    result = torch.empty((count, count), dtype=torch.int64, device="cuda")
    ms = timed(engines["levenshtein"], queries, candidates, result)
    cells = int(lengths[:count].sum()) * int(lengths[count:].sum())
    out["tiny_tokens"] = {"workload": "unit-cost Levenshtein, 2,048 x 2,048 printable tokens of 4-16 bytes",
                          "GCUPS": cells / (ms * 1e-3) / 1e9, "ms_per_call": ms,
                          "cells_per_second": count * count / (ms * 1e-3)}
    return out


def long_pairs_leg(szs, torch, scope, steps=3, warmup=1):
    """Single very long pairs, one call each, device-resident: unit-cost Levenshtein at 50,000, 100,000 and 200,000
    characters a side and linear-gap Levenshtein (0, 2, 3, 3) at 50,000 and 100,000 (a 3% substitution + 1% indel
    mutant), Smith-Waterman affine DNA (+2/-3, -5/-2) and
    Needleman-Wunsch affine protein (-11/-1) at 30,000 with a planted shared segment. GCUPS from CUDA events."""
    from stringzillas_gb300 import workloads as w
    stream = torch.cuda.current_stream()
    rng = np.random.Generator(np.random.PCG64(5))
    dna = np.frombuffer(b"ACGT", dtype=np.uint8)
    protein = np.frombuffer(b"ARNDCQEGHILKMFPSTWYV", dtype=np.uint8)

    def pair(alphabet, length, mutate=True):
        a = alphabet[rng.integers(0, len(alphabet), size=length)]
        if mutate:
            b, _ = w._mutate(rng, a, np.array([0, length]), alphabet, 0.03, 0.01)
        else:
            b = alphabet[rng.integers(0, len(alphabet), size=length)]
            b[length // 3:length // 3 + 5000] = a[length // 2:length // 2 + 5000]
        return a, b

    def device(strings):
        data = np.concatenate(strings)
        offsets = np.zeros(len(strings) + 1, dtype=np.int64)
        np.cumsum([len(x) for x in strings], out=offsets[1:])
        return szs.Strs.from_buffers(torch.from_numpy(data).cuda(), torch.from_numpy(offsets).cuda())

    protein_b2c, protein_table = w.protein_table(seed=42)
    cases = [("levenshtein_50k", szs.LevenshteinDistances(), pair(dna, 50000)),
             ("levenshtein_100k", szs.LevenshteinDistances(), pair(dna, 100000)),
             ("levenshtein_200k", szs.LevenshteinDistances(), pair(dna, 200000)),
             ("levenshtein_linear_50k", szs.LevenshteinDistances(0, 2, 3, 3), pair(dna, 50000)),
             ("levenshtein_linear_100k", szs.LevenshteinDistances(0, 2, 3, 3), pair(dna, 100000)),
             ("smith_waterman_30k", szs.SmithWatermanScores(*w.dna_table(2, -3), open=-5, extend=-2),
              pair(dna, 30000, mutate=False)),
             ("needleman_wunsch_30k", szs.NeedlemanWunschScores(protein_b2c, protein_table, open=-11, extend=-1),
              pair(protein, 30000, mutate=False))]
    out = {}
    for name, engine, (a, b) in cases:
        first, second = device([a]), device([b])
        result = torch.empty(1, dtype=torch.int64, device="cuda")
        for _ in range(warmup):
            engine.pairwise(first, second, device=scope, out=result)
        begin, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        begin.record(stream)
        for _ in range(steps):
            engine.pairwise(first, second, device=scope, out=result)
        end.record(stream)
        torch.cuda.synchronize()
        ms = begin.elapsed_time(end) / steps
        out[name] = {"GCUPS": len(a) * len(b) / (ms * 1e-3) / 1e9, "ms_per_call": ms, "lengths": [len(a), len(b)]}
    return out


FINGERPRINT_WORKLOAD = ("Min-Hash fingerprints: 16,384 documents, len U[1,000, 3,000] printable bytes, 1,024 dimensions, "
                        "default widths {3,4,5,7,9,11,15,31} (64-dimension slices), seed 0")
# Integer operations per byte and dimension, counted from the rolling step: x = state*a + D*out + (D + 1 + in) (two
# 32x64-bit products as multiply-adds and two 64-bit adds: 6), the reduction to [0, 2m) (shift, multiply-high,
# shift, 32x64-bit product, 64-bit subtract: 7) and the high-word test against the running minimum (3). The
# executed count (ncu, profiles/fingerprints_minhash_1024d.txt) is 28.8 instructions per byte-dimension.
FINGERPRINT_OPS_PER_BYTE_DIM = 16.0
FINGERPRINT_EXECUTED_INST_PER_BYTE_DIM = 28.8


def fingerprint_texts(count=16384, low=1000, high=3000, seed=7):
    rng = np.random.Generator(np.random.PCG64(seed))
    lengths = rng.integers(low, high + 1, size=count)
    offsets = np.zeros(count + 1, dtype=np.uint64)
    np.cumsum(lengths, out=offsets[1:])
    data = rng.integers(32, 127, size=int(offsets[-1]), dtype=np.uint8)
    return data, offsets


def fingerprints_leg(szs, torch, scope, peaks, steps=3, warmup=3, cpu_seconds=10.0, documents=16384):
    """Min-Hash leg: device-resident texts and outputs timed with CUDA events; e2e from pinned host tapes into
    pinned host outputs; the oracle's C restatement on one core over a sample of the documents."""
    dims = 1024
    data, offsets = fingerprint_texts(documents)
    count = len(offsets) - 1
    engine = szs.Fingerprints(dims)
    stream = torch.cuda.current_stream()

    def timed(texts, out, k):
        for _ in range(warmup):
            engine(texts, device=scope, out=out)
        begin, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        begin.record(stream)
        for _ in range(k):
            engine(texts, device=scope, out=out)
        end.record(stream)
        torch.cuda.synchronize()
        return begin.elapsed_time(end) / k

    d_texts = szs.Strs.from_buffers(torch.from_numpy(data).cuda(), torch.from_numpy(offsets.astype(np.int64)).cuda())
    d_out = (torch.empty((count, dims), dtype=torch.int32, device="cuda"),
             torch.empty((count, dims), dtype=torch.int32, device="cuda"))
    device_ms = timed(d_texts, d_out, steps)
    h_texts = szs.Strs.from_buffers(torch.from_numpy(data).pin_memory(),
                                    torch.from_numpy(offsets.astype(np.int64)).pin_memory())
    h_out = (torch.empty((count, dims), dtype=torch.int32).pin_memory(),
             torch.empty((count, dims), dtype=torch.int32).pin_memory())
    e2e_ms = timed(h_texts, h_out, steps)
    # Parity of the timed outputs on a sample of documents.
    from oracle import oracle
    picks = np.arange(0, count, 997)
    sub_offsets = np.concatenate([[0], np.cumsum(offsets[picks + 1] - offsets[picks])]).astype(np.uint64)
    sub_data = np.concatenate([data[offsets[i]:offsets[i + 1]] for i in picks])
    want_h, want_c = oracle.fingerprints(dims, (sub_data, sub_offsets))
    got_h = h_out[0].numpy().view(np.uint32)[picks]
    got_c = h_out[1].numpy().view(np.uint32)[picks]
    exact = bool(np.array_equal(got_h, want_h) and np.array_equal(got_c, want_c))
    # CPU: the oracle on one core, documents until the time budget is spent.
    done_bytes, begin = 0, time.perf_counter()
    for i in range(count):
        a, b = int(offsets[i]), int(offsets[i + 1])
        oracle.fingerprints(dims, (data[a:b], np.array([0, b - a], dtype=np.uint64)))
        done_bytes += b - a
        if time.perf_counter() - begin > cpu_seconds:
            break
    cpu_s = time.perf_counter() - begin
    byte_dims = float(offsets[-1]) * dims
    int_peak = None if not peaks else peaks["lop3"]
    ops = byte_dims * FINGERPRINT_OPS_PER_BYTE_DIM
    return {
        "workload": FINGERPRINT_WORKLOAD.replace("16,384", f"{count:,}"), "unit": "G byte-dimensions/s",
        "value": byte_dims / (device_ms * 1e-3) / 1e9, "ms_per_step": device_ms,
        "documents_per_s": count / (device_ms * 1e-3), "text_gbs": float(offsets[-1]) / (device_ms * 1e-3) / 1e9,
        "e2e": {"value": byte_dims / (e2e_ms * 1e-3) / 1e9, "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": int(data.nbytes + offsets.nbytes), "d2h_bytes_per_step": 2 * count * dims * 4},
        "roofline_int": {"bound": "int_pipe", "achieved": ops / (device_ms * 1e-3) / 1e12,
                         "peak": None if int_peak is None else int_peak / 1e12, "unit": "Tops/s",
                         "frac": None if int_peak is None else ops / (device_ms * 1e-3) / int_peak,
                         "ops_per_byte_dimension": FINGERPRINT_OPS_PER_BYTE_DIM,
                         "executed_instructions_per_byte_dimension": FINGERPRINT_EXECUTED_INST_PER_BYTE_DIM,
                         "note": "bound by the integer multiply-add pipe (68.9% busy in ncu), not by memory"},
        "cpu_baseline": {"value": done_bytes * dims / cpu_s / 1e9, "unit": "G byte-dimensions/s", "cores": 1,
                         "kind": "port", "sample": f"{done_bytes} bytes of the documents, oracle C restatement"},
        "sample_parity_exact": exact,
        "gpu_launches_per_step": 1,
    }


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    first, second, kind_and_tables = make_workload(args.workload, 42)
    values = []
    baseline = None
    for step in range(args.warmup + args.steps):
        baseline = cpu_baseline(first, second, kind_and_tables, args.cpu_seconds / max(1, args.warmup + args.steps))
        if step >= args.warmup:
            values.append(baseline["value"])
    value = statistics.median(values)
    config = workload_config(args.workload, first, second, int(os.environ.get("WORLD_SIZE", "1")))
    cells = config["cells_per_step"]
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "GCUPS", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": cells / (value * 1e9) * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64 bit-vectors / int64",
        "data": "synthetic (seeded numpy PCG64)", "config": config,
        "cpu_baseline": dict(baseline, value=value),
        "e2e": {"value": value, "unit": "GCUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))

    def barrier():
        if dist is not None:
            dist.barrier()

    import stringzillas_gb300 as szs
    first, second, kind_and_tables = make_workload(args.workload, 42 + rank)
    engine = make_engine(kind_and_tables)
    scope = szs.DeviceScope(gpu_device=local_rank, stream=torch.cuda.current_stream())
    device_batch = DeviceBatch(first, second, torch)
    pairs = device_batch.count
    input_bytes = int(first[0].shape[0] + second[0].shape[0])

    peaks = integer_peaks(local_rank)
    with Clocks(local_rank) as clocks:
        elapsed_ms, compute_ms, launches, cells_total = timed_steps(engine, scope, device_batch, args.steps,
                                                                    args.warmup, torch, barrier)
    clock_summary = clocks.summary()

    slowest_ms = elapsed_ms
    all_cells = cells_total
    if dist is not None:
        t = torch.tensor([elapsed_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        slowest_ms = float(t.item())
        c = torch.tensor([float(cells_total)], device="cuda", dtype=torch.float64)
        dist.all_reduce(c, op=dist.ReduceOp.SUM)
        all_cells = float(c.item())
    value = all_cells / (slowest_ms * 1e-3) / 1e9
    cells_per_step = cells_total / args.steps

    # The plain one-launch-per-batch form of the same kernels.
    engine.set_schedule("plain")
    plain_steps = max(1, min(args.steps, 5))
    plain_ms, plain_compute_ms, _, plain_cells = timed_steps(engine, scope, device_batch, plain_steps, 1, torch,
                                                             barrier)
    engine.set_schedule("batched")

    # End to end through the same C-ABI with host buffers: copies in the timed region.
    del device_batch
    host_batch = HostBatch(first, second, torch)
    # Two warm-up calls: the first builds the pipelined path's chunk contexts and captures their graphs.
    e2e_steps = max(1, min(args.steps, 5))
    e2e_ms, _, _, e2e_cells = timed_steps(engine, scope, host_batch, e2e_steps, 2, torch, barrier)

    line = None
    if rank == 0:
        hbm_peak, peak_source = measured_peaks()
        step_compute_s = compute_ms / args.steps * 1e-3
        algorithmic_bytes = input_bytes + 8 * pairs
        achieved_gbs = algorithmic_bytes / step_compute_s / 1e9
        int_ops = cells_per_step * ops_per_cell(kind_and_tables)
        int_peak = None
        if peaks:
            int_peak = {"lev": peaks["lop3"], "nw32": peaks["dpx_viaddmax_s32"], "nwd": peaks["dpx_viaddmax_s32"]}.get(
                kind_and_tables[0], peaks["dpx_viaddmax_s16x2"])
        line = {
            "metric": METRIC, "value": value, "unit": "GCUPS", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": slowest_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": {"lev": "u32", "levc": "int16x2", "levu": "int16x2",
                                                     "levp": "int16x2"}.get(kind_and_tables[0], "int32"),
            "data": "synthetic (seeded numpy PCG64)",
            "config": workload_config(args.workload, first, second, world),
            "roofline": {"bound": "hbm", "achieved": achieved_gbs, "peak": hbm_peak, "unit": "GB/s",
                         "frac": achieved_gbs / hbm_peak, "traffic": DRAM_TRAFFIC_PER_STEP.get(args.workload),
                         "traffic_unit": "bytes per step (all scoring launches of one step)",
                         "note": f"peak of {peak_source}; the path is integer-issue bound, see roofline_int"},
            "roofline_int": {"bound": "int_pipe", "achieved": int_ops / step_compute_s / 1e12,
                             "peak": None if int_peak is None else int_peak / 1e12, "unit": "Tops/s",
                             "frac": None if int_peak is None else int_ops / step_compute_s / int_peak,
                             "ops_per_cell": ops_per_cell(kind_and_tables), "measured_peaks_tops":
                                 None if peaks is None else {k: v / 1e12 for k, v in peaks.items()},
                             "pipe_evidence": PIPE_EVIDENCE.get(args.workload)},
            "plain": {"value": plain_cells / (plain_ms * 1e-3) / 1e9, "unit": "GCUPS",
                      "ms_per_step": plain_ms / plain_steps, "compute_ms_per_step": plain_compute_ms / plain_steps},
            "batched_over_plain": value / (plain_cells / (plain_ms * 1e-3) / 1e9 * world),
            "e2e": {"value": e2e_cells / (e2e_ms * 1e-3) / 1e9, "unit": "GCUPS", "ms_per_step": e2e_ms / e2e_steps,
                    "h2d_bytes_per_step": host_batch.bytes_in, "d2h_bytes_per_step": host_batch.bytes_out},
            "clocks": clock_summary,
            "gpu_launches": launches,
            "compute_ms_per_step": compute_ms / args.steps,
        }
    del host_batch

    if rank == 0 and world == 1 and not args.no_extra:
        line["cpu_baseline"] = cpu_baseline(first, second, kind_and_tables, args.cpu_seconds)
        extra = {}
        for name in ("c3", "c4", "text", "short_nw", "short_sw", "short_lev"):
            if name == args.workload:
                continue
            f, s, kt = make_workload(name, 42)
            eng = make_engine(kt)
            batch = DeviceBatch(f, s, torch)
            row = {"workload": WORKLOADS[name]}
            for schedule in ("batched", "plain"):
                eng.set_schedule(schedule)
                ms, cms, _, cells = timed_steps(eng, scope, batch, 2, 1, torch, barrier)
                row[schedule] = {"GCUPS": cells / (ms * 1e-3) / 1e9, "ms_per_step": ms / 2,
                                 "compute_ms_per_step": cms / 2}
            row["batched_over_plain"] = row["batched"]["GCUPS"] / row["plain"]["GCUPS"]
            if peaks:
                ops = ops_per_cell(kt)
                achieved = (row["batched"]["GCUPS"] * 1e9 * row["batched"]["ms_per_step"] /
                            row["batched"]["compute_ms_per_step"] * ops)
                row["roofline_int"] = {"ops_per_cell": ops, "achieved_tops": achieved / 1e12,
                                       "peak_tops": peaks["dpx_viaddmax_s16x2"] / 1e12,
                                       "frac": achieved / peaks["dpx_viaddmax_s16x2"],
                                       "note": "over the scoring kernels' event-timed duration"}
            row["cpu_baseline"] = cpu_baseline(f, s, kt, 3.0)
            extra[name] = row
            del batch
        line["extra"] = extra
        line["cross_product"] = cross_product_leg(szs, torch, scope)
        line["long_pairs"] = long_pairs_leg(szs, torch, scope)
        line["serving"] = serving_leg(szs)
        line["fingerprints"] = fingerprints_leg(szs, torch, scope, peaks)
    elif rank == 0:
        line["cpu_baseline"] = None
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def run_fingerprints_only(args):
    import torch
    import stringzillas_gb300 as szs
    torch.cuda.set_device(0)
    scope = szs.DeviceScope(gpu_device=0, stream=torch.cuda.current_stream())
    leg = fingerprints_leg(szs, torch, scope, integer_peaks(0), steps=args.steps, warmup=args.warmup,
                           cpu_seconds=args.cpu_seconds, documents=args.fp_documents)
    print(json.dumps(leg), flush=True)


def run_cross_only(args):
    import torch
    import stringzillas_gb300 as szs
    torch.cuda.set_device(0)
    scope = szs.DeviceScope(gpu_device=0, stream=torch.cuda.current_stream())
    print(json.dumps(cross_product_leg(szs, torch, scope, steps=args.steps, warmup=args.warmup)), flush=True)


def main():
    args = parse_args()
    if args.long_only:
        import torch
        import stringzillas_gb300 as szs
        torch.cuda.set_device(0)
        scope = szs.DeviceScope(gpu_device=0, stream=torch.cuda.current_stream())
        print(json.dumps(long_pairs_leg(szs, torch, scope)), flush=True)
    elif args.serving_only:
        import stringzillas_gb300 as szs
        print(json.dumps(serving_leg(szs)), flush=True)
    elif args.cross_only:
        run_cross_only(args)
    elif args.fingerprints_only:
        run_fingerprints_only(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
