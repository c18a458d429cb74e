"""Serving loop on the GPU: a mixed stream of Levenshtein / Needleman-Wunsch / Smith-Waterman requests, submitted
while earlier ones are still on the device, must give every request exactly the scores it gets alone."""
import threading
import time

import numpy as np
import pytest

from conftest import tape
from oracle import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def szs():
    import stringzillas_gb300
    if "cuda" not in stringzillas_gb300.__capabilities__:
        pytest.fail("no CUDA device visible: GPU tests must run on a GPU")
    return stringzillas_gb300


@pytest.fixture(scope="module")
def engines(szs):
    from stringzillas_gb300 import workloads as w
    protein_b2c, protein_table = w.protein_table(7)
    dna_b2c, dna_table = w.dna_table(2, -3)
    return {
        "lev": (szs.LevenshteinDistances(), oracle.levenshtein_costs()),
        "lev-affine": (szs.LevenshteinDistances(0, 2, 3, 1), oracle.levenshtein_costs(0, 2, 3, 1)),
        "nw": (szs.NeedlemanWunschScores(protein_b2c, protein_table, -11, -1),
               oracle.alignment_costs(oracle.NEEDLEMAN_WUNSCH, protein_b2c, protein_table, -11, -1)),
        "sw": (szs.SmithWatermanScores(dna_b2c, dna_table, -5, -2),
               oracle.alignment_costs(oracle.SMITH_WATERMAN, dna_b2c, dna_table, -5, -2)),
    }


def _requests(rng, count, max_pairs, max_length):
    alphabets = {"lev": b"ACGT", "lev-affine": b"ACGT", "nw": b"ARNDCQEGHILKMFPSTWYV", "sw": b"ACGT"}
    kinds = list(alphabets)
    out = []
    for _ in range(count):
        kind = kinds[int(rng.integers(0, len(kinds)))]
        alphabet = np.frombuffer(alphabets[kind], dtype=np.uint8)
        pairs = int(np.exp(rng.uniform(0, np.log(max_pairs + 1))))
        first, second = [], []
        for _ in range(pairs):
            n = int(np.exp(rng.uniform(0, np.log(max_length + 1)))) - 1
            m = max(0, n + int(rng.integers(-5, 6)))
            a = rng.choice(alphabet, size=n)
            b = rng.choice(alphabet, size=m)
            keep = min(n, m) // 2
            b[:keep] = a[:keep]  # related prefix: large local scores, short edit distances
            first.append(bytes(a))
            second.append(bytes(b))
        out.append((kind, first, second))
    return out


@pytest.mark.parametrize("aging_ms", [0, 40], ids=["arrival-order", "size-aware"])
def test_mixed_stream_equals_alone(szs, engines, port, aging_ms):
    """Both admission orders: arrival order, and smallest request first with a 40 ms aging bound."""
    rng = np.random.default_rng(2024)
    requests = _requests(rng, 60, 48, 700)
    # A few long pairs ride along (band and 32-bit routes inside merged batches).
    long_a = bytes(rng.choice(np.frombuffer(b"ACGT", dtype=np.uint8), size=2600))
    requests.append(("sw", [long_a, long_a[:1500]], [long_a[300:2900], long_a[::-1][:1400]]))
    requests.append(("lev", [long_a[:1200]], [long_a[50:1300]]))
    with szs.Server(lanes=3, arena_bytes=64 << 20, aging_ms=aging_ms) as server:
        tickets = [None] * len(requests)

        def submitter():
            for i, (kind, first, second) in enumerate(requests):
                tickets[i] = server.submit(engines[kind][0], szs.Strs(first), szs.Strs(second))
                if i % 7 == 0:
                    time.sleep(0.002)

        thread = threading.Thread(target=submitter)
        thread.start()
        thread.join()
        served = [ticket.result().copy() for ticket in tickets]
        infos = [ticket.info for ticket in tickets]
        stats = server.stats()
    assert stats["completed"] == len(requests)
    assert stats["batches"] <= len(requests)
    assert stats["cells"] == sum(info["cells"] for info in infos)
    for (kind, first, second), got, info in zip(requests, served, infos):
        engine, costs = engines[kind]
        alone = engine.pairwise(szs.Strs(first), szs.Strs(second))
        np.testing.assert_array_equal(got, alone)
        assert info["status"] == 0 and info["done_ms"] >= info["admitted_ms"] >= 0
        if sum(len(a) * len(b) for a, b in zip(first, second)) < 2_000_000:
            np.testing.assert_array_equal(got.astype(np.int64), port.pairs(costs, tape(first), tape(second)))


def test_batches_merge_under_load(szs, engines):
    """Requests queued while the only lane is busy are merged into one batch of the same engine."""
    rng = np.random.default_rng(5)
    engine = engines["nw"][0]
    alphabet = np.frombuffer(b"ARNDCQEGHILKMFPSTWYV", dtype=np.uint8)
    big = [bytes(rng.choice(alphabet, size=1800)) for _ in range(400)]
    small = [[bytes(rng.choice(alphabet, size=int(rng.integers(1, 200)))) for _ in range(5)] for _ in range(12)]
    with szs.Server(lanes=1) as server:
        first = server.submit(engine, szs.Strs(big), szs.Strs(big[::-1]))
        rest = [server.submit(engine, szs.Strs(s), szs.Strs(s[::-1])) for s in small]
        first.result()
        results = [t.result() for t in rest]
        batches = {t.info["batch"] for t in rest}
    assert len(batches) < len(rest), "requests that waited together should share batches"
    for s, got in zip(small, results):
        np.testing.assert_array_equal(got, engine.pairwise(szs.Strs(s), szs.Strs(s[::-1])))


def test_arena_budget(szs, engines):
    """A tiny arena admits one small batch at a time; a request larger than the arena fails alone."""
    rng = np.random.default_rng(11)
    engine = engines["lev"][0]
    alphabet = np.frombuffer(b"ACGT", dtype=np.uint8)
    small = [[bytes(rng.choice(alphabet, size=int(rng.integers(0, 300)))) for _ in range(8)] for _ in range(10)]
    huge = [bytes(rng.choice(alphabet, size=40_000))]
    with szs.Server(lanes=2, arena_bytes=64 << 10) as server:
        tickets = [server.submit(engine, szs.Strs(s), szs.Strs(s[::-1])) for s in small[:5]]
        too_big = server.submit(engine, szs.Strs(huge), szs.Strs(huge))
        tickets += [server.submit(engine, szs.Strs(s), szs.Strs(s[::-1])) for s in small[5:]]
        results = [t.result() for t in tickets]
        with pytest.raises(MemoryError):
            too_big.result()
        stats = server.stats()
    assert stats["arena_peak_bytes"] <= 64 << 10
    for s, got in zip(small, results):
        np.testing.assert_array_equal(got, engine.pairwise(szs.Strs(s), szs.Strs(s[::-1])))


def test_per_request_plain_form(szs, engines):
    """One lane, one request per batch, plain schedule: the comparison form of the serving benchmark."""
    rng = np.random.default_rng(3)
    requests = _requests(rng, 12, 20, 400)
    with szs.Server(lanes=1, max_batch_requests=1, schedule="plain") as server:
        tickets = [server.submit(engines[k][0], szs.Strs(a), szs.Strs(b)) for k, a, b in requests]
        results = [t.result() for t in tickets]
        assert all(t.info["batch_requests"] == 1 for t in tickets)
    for (kind, first, second), got in zip(requests, results):
        np.testing.assert_array_equal(got, engines[kind][0].pairwise(szs.Strs(first), szs.Strs(second)))


def test_device_resident_request(szs, engines):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(9)
    engine = engines["sw"][0]
    alphabet = np.frombuffer(b"ACGT", dtype=np.uint8)
    first = [bytes(rng.choice(alphabet, size=int(rng.integers(0, 500)))) for _ in range(40)]
    second = [bytes(rng.choice(alphabet, size=int(rng.integers(0, 500)))) for _ in range(40)]
    host_a, host_b = szs.Strs(first), szs.Strs(second)
    dev_a = szs.Strs.from_buffers(torch.from_numpy(host_a._data.copy()).cuda(),
                                  torch.from_numpy(host_a._offsets.astype(np.int64)).cuda())
    dev_b = szs.Strs.from_buffers(torch.from_numpy(host_b._data.copy()).cuda(),
                                  torch.from_numpy(host_b._offsets.astype(np.int64)).cuda())
    out = torch.zeros(40, dtype=torch.int64, device="cuda")
    with szs.Server(lanes=2) as server:
        ticket = server.submit(engine, dev_a, dev_b, out=out)
        ticket.result()
    np.testing.assert_array_equal(out.cpu().numpy(), engine.pairwise(host_a, host_b))


def test_merged_batch_of_pageable_pinned_device_and_managed_inputs(szs, engines, port):
    """One merged batch whose requests hold their strings in pageable host memory, page-locked host memory (copied
    into the arena straight from the caller's buffers), device memory and managed memory, on either side and mixed
    within a request, slices with non-zero first offsets among them: every request equals the oracle."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(31)
    engine, costs = engines["lev-affine"]
    alphabet = np.frombuffer(b"ACGT", dtype=np.uint8)

    def strings(count):
        return [bytes(rng.choice(alphabet, size=int(rng.integers(0, 300)))) for _ in range(count)]

    def placed(items, where):
        host = szs.Strs(items)
        data, offsets = host._data.copy(), host._offsets.astype(np.int64)
        if where == "pageable":
            return host
        if where == "pinned":
            return szs.Strs.from_buffers(torch.from_numpy(data).pin_memory(), torch.from_numpy(offsets).pin_memory())
        if where == "device":
            return szs.Strs.from_buffers(torch.from_numpy(data).cuda(), torch.from_numpy(offsets).cuda())
        return szs.to_device(host)  # managed

    places = ["pageable", "pinned", "device", "managed"]
    requests = []
    for k in range(12):
        count = int(rng.integers(1, 60))
        first, second = strings(count + 3), strings(count + 3)
        a, b = placed(first, places[k % 4]), placed(second, places[(k // 4 + k) % 4])
        requests.append((a[3:], b[3:], first[3:], second[3:]))  # slices: offsets start past zero
    with szs.Server(lanes=1, max_batch_requests=16) as server:
        blocker = server.submit(engines["nw"][0], szs.Strs(strings(200)), szs.Strs(strings(200)))
        tickets = [server.submit(engine, a, b) for a, b, _, _ in requests]  # merged while the blocker runs
        blocker.result()
        for ticket, (_, _, first, second) in zip(tickets, requests):
            np.testing.assert_array_equal(ticket.result(), port.pairs(costs, tape(first), tape(second)))
    assert max(t.info["batch_requests"] for t in tickets) > 1


def test_size_aware_admission_order(szs, engines):
    """With one lane busy, a small request submitted after a large one of another engine runs first under
    size-aware admission, and after it in arrival order; results are the same either way."""
    rng = np.random.default_rng(17)
    dna = np.frombuffer(b"ACGT", dtype=np.uint8)
    protein = np.frombuffer(b"ARNDCQEGHILKMFPSTWYV", dtype=np.uint8)
    blocker = [bytes(rng.choice(protein, size=4000)) for _ in range(1500)]  # ~10 ms on the device
    large = [bytes(rng.choice(protein, size=1500)) for _ in range(200)]
    small = [bytes(rng.choice(dna, size=50)) for _ in range(4)]
    order = {}
    for aging_ms in (0, 10_000):
        with szs.Server(lanes=1, aging_ms=aging_ms) as server:
            first = server.submit(engines["nw"][0], szs.Strs(blocker), szs.Strs(blocker[::-1]))
            time.sleep(0.001)
            big = server.submit(engines["sw"][0], szs.Strs(large), szs.Strs(large[::-1]))
            tiny = server.submit(engines["lev"][0], szs.Strs(small), szs.Strs(small[::-1]))
            first.result(), big.result(), tiny.result()
            order[aging_ms] = (big.info["batch"], tiny.info["batch"])
            np.testing.assert_array_equal(tiny.result(), engines["lev"][0].pairwise(szs.Strs(small), szs.Strs(small[::-1])))
    assert order[0][0] < order[0][1], "arrival order: the earlier large request runs first"
    assert order[10_000][1] < order[10_000][0], "size-aware: the small request passes the large one"
