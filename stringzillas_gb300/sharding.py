"""Pair sharding across GPUs (one process per GPU): pairs are independent, so a batch splits with no exchange.

``partition`` assigns pairs to ranks by longest-processing-time order on their cell counts (n * m), so every rank
gets about the same work however uneven the lengths; ``score_sharded`` scores a rank's share with its local engine
and, when asked, gathers all ranks' results back into input order with one ``all_gather`` of (index, score)
tensors. The scoring itself never communicates; the gather is the only collective and happens after the scores are
final. The reference has no multi-GPU path for this workload (one device per scope).
"""
from __future__ import annotations

import heapq

import numpy as np


def partition(first_lengths, second_lengths, world_size: int) -> list:
    """Pair indices of each rank (ascending), balancing the sum of n * m per rank (LPT greedy)."""
    first_lengths = np.asarray(first_lengths, dtype=np.int64)
    second_lengths = np.asarray(second_lengths, dtype=np.int64)
    if first_lengths.shape != second_lengths.shape:
        raise ValueError("pairwise inputs must have the same length")
    if world_size < 1:
        raise ValueError("world_size must be positive")
    cells = first_lengths * second_lengths + 1  # +1: even empty pairs cost a task
    order = np.argsort(-cells, kind="stable")
    heap = [(0, rank) for rank in range(world_size)]
    owner = np.empty(len(cells), dtype=np.int64)
    for index in order:
        load, rank = heapq.heappop(heap)
        owner[index] = rank
        heapq.heappush(heap, (load + int(cells[index]), rank))
    return [np.flatnonzero(owner == rank) for rank in range(world_size)]


def _subset(tape, indices):
    """(data, offsets) of the strings at `indices` of a (data, offsets) tape, copied contiguously."""
    data, offsets = tape
    offsets = np.asarray(offsets, dtype=np.int64)
    starts, ends = offsets[indices], offsets[indices + 1]
    lengths = ends - starts
    out_offsets = np.zeros(len(indices) + 1, dtype=np.int64)
    np.cumsum(lengths, out=out_offsets[1:])
    if len(indices) == 0 or out_offsets[-1] == 0:
        return np.zeros(0, dtype=np.uint8), out_offsets
    gather = np.repeat(starts - out_offsets[:-1], lengths) + np.arange(out_offsets[-1])
    return np.asarray(data, dtype=np.uint8)[gather], out_offsets


def score_sharded(score, first, second, rank: int, world_size: int, group=None, gather: bool = True):
    """Scores this rank's share of the pairs with `score(first_tape, second_tape) -> int64 array` and, if `gather`,
    returns every pair's score in input order on every rank (else this rank's indices and scores).

    `first` and `second` are (data uint8[], offsets int64[count + 1]) tapes, identical on every rank.
    """
    import torch
    import torch.distributed as dist
    offsets_a = np.asarray(first[1], dtype=np.int64)
    offsets_b = np.asarray(second[1], dtype=np.int64)
    shares = partition(np.diff(offsets_a), np.diff(offsets_b), world_size)
    mine = shares[rank]
    scores = np.asarray(score(_subset(first, mine), _subset(second, mine)), dtype=np.int64)
    if not gather:
        return mine, scores
    count = len(offsets_a) - 1
    # Ranks hold different numbers of pairs: pad to the largest share, then keep the valid prefix of each.
    longest = max(len(share) for share in shares)
    packed = torch.full((2, longest), -1, dtype=torch.int64)
    packed[0, :len(mine)] = torch.from_numpy(mine)
    packed[1, :len(mine)] = torch.from_numpy(scores)
    gathered = [torch.empty_like(packed) for _ in range(world_size)]
    dist.all_gather(gathered, packed, group=group)
    out = np.empty(count, dtype=np.int64)
    for share, block in zip(shares, gathered):
        out[block[0, :len(share)].numpy()] = block[1, :len(share)].numpy()
    return out
