"""Multi-GPU pair sharding on CPU: the LPT partition and a world-size-2 gloo run of the gather path, with the oracle
standing in for each rank's GPU engine (no GPU in these tests)."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from stringzillas_gb300 import sharding, workloads as w


def test_partition_covers_every_pair_once_and_balances_cells():
    rng = np.random.default_rng(1)
    a = np.exp(rng.uniform(0, np.log(20000), size=5000)).astype(np.int64)
    b = np.exp(rng.uniform(0, np.log(20000), size=5000)).astype(np.int64)
    for world in (1, 2, 3, 8):
        shares = sharding.partition(a, b, world)
        joined = np.sort(np.concatenate(shares))
        np.testing.assert_array_equal(joined, np.arange(len(a)))
        loads = [int(np.sum(a[s] * b[s] + 1)) for s in shares]
        # LPT: no rank carries more than the mean plus the largest single pair.
        assert max(loads) <= sum(loads) / world + int(np.max(a * b + 1))
    with pytest.raises(ValueError):
        sharding.partition(a, b[:-1], 2)


def test_subset_copies_the_selected_strings():
    (data, offsets), _ = w.levenshtein_reads(50, 0, 20, 0.1, 0.1, seed=5)
    picks = np.array([3, 0, 49, 7, 7])
    sub_data, sub_offsets = sharding._subset((data, offsets), picks)
    for k, i in enumerate(picks):
        assert bytes(sub_data[sub_offsets[k]:sub_offsets[k + 1]]) == bytes(data[offsets[i]:offsets[i + 1]])


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, first, second, results):
    import torch.distributed as dist
    from oracle import oracle
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    port_engine = oracle.Port()
    costs = oracle.levenshtein_costs()
    out = sharding.score_sharded(lambda a, b: port_engine.pairs(costs, a, b), first, second, rank, world)
    results[rank] = out.tolist()
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_gloo_gather_matches_single_rank(port):
    first, second = w.levenshtein_reads(300, 0, 120, 0.05, 0.02, seed=11)
    want = port.pairs(__import__("oracle.oracle", fromlist=["x"]).levenshtein_costs(), first, second)
    manager = mp.get_context("spawn").Manager()
    results = manager.dict()
    mp.start_processes(_rank_main, args=(2, _free_port(), first, second, results), nprocs=2, join=True,
                       start_method="spawn")
    for rank in range(2):
        np.testing.assert_array_equal(np.array(results[rank], dtype=np.int64), want)
