"""Autotuner for the engine's per-length-bin choices (``szs_gb300_tuning_t``).

For every engine family (kind x linear/affine gaps) and every length class k (pairs whose shorter side n has
floor(log2 n) == k) it times, on synthetic pairs of that class, each candidate of

* cell width: 16x2 packed cells (where the length bound allows them) or 32-bit cells,
* tile shape: rows per lane R in {4, 8, 12, 16} of the packed wavefront (a warp's strip is 32 R rows), one R for
  the whole class or R chosen per pair by the planner's step-cost model,
* pairs per block: warps per CTA in {2, 4, 8} of the packed launches (each warp scores two pairs at once),

and keeps the fastest by the scoring kernels' CUDA-event time (``last_compute_ms``). The step-cost model's four
costs (one lane step with R rows per lane) are fitted from the fixed-R timings: each timing divided by the lane
steps its batch needs with that R (strips x (m + 31) summed over the pairs). Then it picks the band threshold
(shorter sides above it go to the one-CTA-per-pair band kernel) on a batch of long pairs. The result is a
JSON file that ``apply`` installs on an engine. The reference fixes its tier thresholds at compile time; this module
has no counterpart there.

    python -m stringzillas_gb300.autotune --out stringzillas_gb300/tuning/gb300.json
"""
from __future__ import annotations

import argparse
import json
import os
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_TABLE = os.path.join(HERE, "tuning", "gb300.json")
CLASSES = range(3, 11)        # shorter sides 8 .. 2047 (longer pairs take the band by default)
ROWS = (4, 8, 12, 16)
WARPS = (2, 4, 8)
BAND_THRESHOLDS = (512, 1024, 2048, 4096)
PACKED_BAND_THRESHOLDS = (1024, 2048, 4096, 8192)


def family_of(engine) -> str:
    """"lev-unit", "lev-linear", "lev-affine", "nw-linear", ... for an engine object of this package."""
    from . import LevenshteinDistances, NeedlemanWunschScores
    costs = engine.description
    if isinstance(engine, LevenshteinDistances):
        match, mismatch, open_, extend = (int(x) for x in costs.split(","))
        if (match, mismatch, open_, extend) == (0, 1, 1, 1):
            return "lev-unit"
        return "lev-linear" if open_ == extend else "lev-affine"
    fields = dict(part.split("=") for part in costs.split(","))
    kind = "nw" if isinstance(engine, NeedlemanWunschScores) else "sw"
    return f"{kind}-{'linear' if fields['open'] == fields['extend'] else 'affine'}"


def _engines(szs):
    from . import workloads as w
    protein = w.protein_table(seed=42)
    return {
        "lev-unit": lambda: szs.LevenshteinDistances(),
        "lev-linear": lambda: szs.LevenshteinDistances(0, 2, 3, 3),
        "lev-affine": lambda: szs.LevenshteinDistances(0, 2, 3, 1),
        "nw-linear": lambda: szs.NeedlemanWunschScores(*protein, open=-4, extend=-4),
        "nw-affine": lambda: szs.NeedlemanWunschScores(*protein, open=-11, extend=-1),
        "sw-linear": lambda: szs.SmithWatermanScores(*protein, open=-4, extend=-4),
        "sw-affine": lambda: szs.SmithWatermanScores(*protein, open=-11, extend=-1),
    }


def _batch(szs, rng, low, high, target_cells, alphabet, sides=None):
    """Device-resident pairs with both lengths uniform in [low, high), about `target_cells` cells; with `sides`
    (a list) the pairs' (shorter, longer) sides are appended to it."""
    mean = (low + high) / 2
    # Enough pairs for several waves of warps on every SM, so a class is not measured on a half-empty GPU.
    count = int(max(1 << 15, min(1 << 20, target_cells / (mean * mean))))
    la = rng.integers(low, high, size=count)
    lb = rng.integers(low, high, size=count)
    tapes = []
    for lengths in (la, lb):
        offsets = np.zeros(count + 1, dtype=np.uint64)
        np.cumsum(lengths, out=offsets[1:])
        data = rng.choice(alphabet, size=int(offsets[-1])).astype(np.uint8)
        tapes.append(szs.to_device(szs.Strs.from_buffers(data, offsets)))
    if sides is not None:
        sides.append((np.minimum(la, lb), np.maximum(la, lb)))
    return tapes[0], tapes[1], int(np.dot(la, lb))


def lane_steps(n, m, rows):
    """Lane steps of the 16x2 route for pairs of shorter sides n and longer sides m with `rows` rows per lane."""
    strips = (n + 32 * rows - 1) // (32 * rows)
    return float(np.sum(strips * (m + 31)))


def fit_step_costs(classes):
    """Relative cost of one lane step per rows choice (R = 4 -> 100) from fixed-R timings: for each class, time / lane
    steps; the median over the classes."""
    ratios = []
    for timings, (n, m) in classes:
        per_step = [timings[f"16x2 R={rows}"] / lane_steps(n, m, rows) for rows in ROWS]
        ratios.append([p / per_step[0] for p in per_step])
    if not ratios:
        return [0, 0, 0, 0]
    return [int(round(100 * float(np.median([r[i] for r in ratios])))) for i in range(len(ROWS))]


def _time(engine, first, second, out, repeats=3):
    engine.pairwise(first, second, out=out)  # warm-up (captures the call's graphs)
    best = float("inf")
    for _ in range(repeats):
        engine.pairwise(first, second, out=out)
        best = min(best, engine.stats()["last_compute_ms"])
    return best


def tune_family(szs, make_engine, family, rng, target_cells=4e9, log=print):
    from . import workloads as w
    alphabet = w.DNA if family.startswith("lev") else w.AMINO_ACIDS
    engine = make_engine()
    # While the warp routes are measured, keep every measured class off the band.
    table = {"packed_rows": [0] * 16, "cell_bits": [0] * 16, "band_min_rows": 1 << (max(CLASSES) + 1),
             "packed_warps": [0] * 4, "band_min_rows_packed": 1 << (max(CLASSES) + 1)}
    measurements = {}
    rows_votes = {}
    batches, fits = {}, []
    for k in CLASSES:
        if family == "lev-unit" and k < 9:
            continue  # the bit-parallel route takes these
        lengths = []
        first, second, cells = _batch(szs, rng, 1 << k, 1 << (k + 1), target_cells, alphabet, lengths)
        out = np.empty(len(first), dtype=engine._dtype)
        timings = {}
        base = dict(table)
        engine.set_tuning(dict(base, cell_bits=[32 if c == k else 0 for c in range(16)]))
        timings["32-bit"] = _time(engine, first, second, out)
        for rows in ROWS:
            engine.set_tuning(dict(base, packed_rows=[rows if c == k else 0 for c in range(16)]))
            timings[f"16x2 R={rows}"] = _time(engine, first, second, out)
        best = min(timings, key=timings.get)
        if best == "32-bit":
            table["cell_bits"][k] = 32
        else:
            rows = int(best.split("=")[1])
            table["packed_rows"][k] = rows
            if 6 <= k <= 9:  # classes with several strips and many waves of warps fit the step costs
                fits.append((timings, lengths[0]))
            batches[k] = (first, second, cells, out, timings)
        measurements[f"class {k} (n in [{1 << k}, {1 << (k + 1)}))"] = {
            "cells": cells, "GCUPS": {name: cells / (ms * 1e6) for name, ms in timings.items()}, "best": best}
        log(f"  {family:10s} class {k:2d}: best {best:12s} "
            + " ".join(f"{n}={cells / (ms * 1e6):7.0f}" for n, ms in timings.items()))
    # Rows per lane chosen per pair by the step-cost model, against the class's best fixed choice.
    table["packed_step_cost"] = fit_step_costs(fits)
    measurements["packed_step_cost"] = table["packed_step_cost"]
    for k, (first, second, cells, out, timings) in sorted(batches.items()):
        trial = dict(table, packed_rows=[0 if c == k else r for c, r in enumerate(table["packed_rows"])])
        engine.set_tuning(trial)
        model_ms = _time(engine, first, second, out)
        best_ms = min(timings.values())
        key = f"class {k} (n in [{1 << k}, {1 << (k + 1)}))"
        measurements[key]["GCUPS"]["16x2 per-pair model"] = cells / (model_ms * 1e6)
        if model_ms < best_ms:
            table["packed_rows"][k] = 0
            measurements[key]["best"] = "16x2 per-pair model"
        log(f"  {family:10s} class {k:2d}: per-pair model {cells / (model_ms * 1e6):7.0f} "
            f"(best fixed {cells / (best_ms * 1e6):7.0f})")
    del batches
    # The rows choices that classes use, for the warps-per-CTA pass (the model's pairs count for every choice).
    for k in CLASSES:
        rows = table["packed_rows"][k]
        if rows:
            rows_votes.setdefault(rows, []).append(k)
    # Pairs per block: warps per CTA for each rows choice, on the classes that chose it.
    engine.set_tuning(table)
    for rows, classes in sorted(rows_votes.items()):
        low, high = 1 << min(classes), 1 << (max(classes) + 1)
        first, second, cells = _batch(szs, rng, low, high, target_cells, alphabet)
        out = np.empty(len(first), dtype=engine._dtype)
        timings = {}
        for warps in WARPS:
            trial = dict(table, packed_warps=list(table["packed_warps"]))
            trial["packed_warps"][rows // 4 - 1] = warps
            engine.set_tuning(trial)
            timings[warps] = _time(engine, first, second, out)
        best = min(timings, key=timings.get)
        table["packed_warps"][rows // 4 - 1] = best
        measurements[f"warps per CTA, R={rows}"] = {str(w_): cells / (ms * 1e6) for w_, ms in timings.items()}
        log(f"  {family:10s} R={rows:2d}: warps per CTA {best} "
            + " ".join(f"{w_}={cells / (ms * 1e6):7.0f}" for w_, ms in timings.items()))
    # Band thresholds on 512 long pairs (shorter sides log-uniform in [256, 8192]; `band_min_rows_few`, which would
    # lower every threshold for a batch this small, is switched off while measuring): first for pairs on 32-bit cells
    # (16-bit cells switched off), then for pairs that fit 16-bit cells. A batch this size is a fraction of a wave, as
    # the merged batches of a serving stream often are; thresholds measured on a full wave (8,192 pairs) raised the
    # protein batch by 1.5 % but lowered the mixed-length NW/SW burst by 12 %.
    count = 512
    lengths = [np.exp(rng.uniform(np.log(256), np.log(8192), size=count)).astype(np.int64) for _ in range(2)]
    tapes = []
    for lens in lengths:
        offsets = np.zeros(count + 1, dtype=np.uint64)
        np.cumsum(lens, out=offsets[1:])
        tapes.append(szs.to_device(szs.Strs.from_buffers(
            rng.choice(alphabet, size=int(offsets[-1])).astype(np.uint8), offsets)))
    cells = int(np.dot(lengths[0], lengths[1]))
    out = np.empty(count, dtype=engine._dtype)
    for field, thresholds, trial_base in (
            ("band_min_rows", BAND_THRESHOLDS, dict(table, cell_bits=[32] * 16)),
            ("band_min_rows_packed", PACKED_BAND_THRESHOLDS, dict(table))):
        timings = {}
        for threshold in thresholds:
            engine.set_tuning(dict(trial_base, band_min_rows_few=1 << 30, **{field: threshold}))
            timings[threshold] = _time(engine, tapes[0], tapes[1], out, repeats=2)
        best = min(timings, key=timings.get)
        table[field] = best
        measurements[field] = {str(t): cells / (ms * 1e6) for t, ms in timings.items()}
        log(f"  {family:10s} {field} {best} " + " ".join(f"{t}={cells / (ms * 1e6):7.0f}"
                                                        for t, ms in timings.items()))
    return table, measurements


def autotune(families=None, seed=7, target_cells=4e9, log=print) -> dict:
    import stringzillas_gb300 as szs
    from . import _native
    rng = np.random.default_rng(seed)
    makers = _engines(szs)
    families = list(makers) if families is None else list(families)
    started = time.time()
    result = {"device": _device_name(), "generated_by": "python -m stringzillas_gb300.autotune",
              "metric": "GCUPS of the scoring kernels (CUDA events), synthetic pairs per length class",
              "library": os.path.basename(_native.LIBRARY_PATH), "families": {}}
    for family in families:
        table, measurements = tune_family(szs, makers[family], family, rng, target_cells, log)
        result["families"][family] = {"tuning": table, "measurements": measurements}
    result["seconds"] = time.time() - started
    return result


def _device_name() -> str:
    try:
        import torch
        return torch.cuda.get_device_name(0)
    except Exception:  # torch absent or no device: the name is informational only
        return "unknown"


def load(path: str = DEFAULT_TABLE) -> dict | None:
    """The tuning file, or None if it does not exist."""
    if not os.path.exists(path):
        return None
    with open(path) as f:
        return json.load(f)


def apply(engine, table: dict | None = None) -> bool:
    """Installs the tuned choices for `engine`'s family from `table` (default: the committed GB300 file).
    Returns False (and leaves the engine's built-in choices) when the table has no entry for the family."""
    table = load() if table is None else table
    if not table:
        return False
    entry = table.get("families", {}).get(family_of(engine))
    if not entry:
        return False
    engine.set_tuning(entry["tuning"])
    return True


def main():
    parser = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    parser.add_argument("--out", default=DEFAULT_TABLE)
    parser.add_argument("--families", nargs="*", default=None)
    parser.add_argument("--cells", type=float, default=4e9, help="cells per measured batch")
    args = parser.parse_args()
    result = autotune(args.families, target_cells=args.cells)
    os.makedirs(os.path.dirname(os.path.abspath(args.out)), exist_ok=True)
    with open(args.out, "w") as f:
        json.dump(result, f, indent=1)
    print(f"wrote {args.out} in {result['seconds']:.1f} s")


if __name__ == "__main__":
    main()
