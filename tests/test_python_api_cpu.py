"""Host-side behaviour of the Python callables (argument validation, containers); no GPU needed."""
import numpy as np
import pytest

import stringzillas_gb300 as szs


def test_device_scope_validation():
    with pytest.raises(ValueError):
        szs.DeviceScope(cpu_cores=4, gpu_device=0)
    with pytest.raises(TypeError):
        szs.DeviceScope(cpu_cores="invalid")
    with pytest.raises(TypeError):
        szs.DeviceScope(gpu_device="invalid")
    assert repr(szs.DeviceScope(cpu_cores=2)) == "DeviceScope(CPUs:2)"
    assert repr(szs.DeviceScope(cpu_cores=1)) == "DeviceScope(default)"
    if "cuda" not in szs.__capabilities__:
        with pytest.raises(RuntimeError):
            szs.DeviceScope(gpu_device=0)


def test_cpu_scope_rejects_the_gpu_engine():
    engine = szs.LevenshteinDistances()
    with pytest.raises(RuntimeError):
        engine(szs.Strs(["hello", "world"]), szs.Strs(["hallo", "word"]), device=szs.DeviceScope(cpu_cores=2))


def test_levenshtein_constructor_validation():
    with pytest.raises(ValueError):
        szs.LevenshteinDistances(mismatch=300)
    with pytest.raises(TypeError):
        szs.LevenshteinDistances(capabilities="cuda")
    assert "LevenshteinDistances" in repr(szs.LevenshteinDistances(0, 2, 3, 1))


def test_alignment_constructor_validation():
    b2c = np.zeros(256, np.uint8)
    table = np.zeros((32, 32), np.int8)
    with pytest.raises(TypeError):
        szs.NeedlemanWunschScores()
    with pytest.raises(TypeError):
        szs.NeedlemanWunschScores(list(b2c), table)
    with pytest.raises(ValueError):
        szs.NeedlemanWunschScores(np.zeros(255, np.uint8), table)
    with pytest.raises(TypeError):
        szs.SmithWatermanScores(b2c.astype(np.int8), table)
    with pytest.raises(ValueError):
        szs.SmithWatermanScores(b2c, np.zeros((16, 16), np.int8))
    with pytest.raises(TypeError):
        szs.SmithWatermanScores(b2c, table.astype(np.int16))
    with pytest.raises(ValueError):
        szs.SmithWatermanScores(b2c, np.asfortranarray(np.arange(1024, dtype=np.int8).reshape(32, 32)))
    with pytest.raises(ValueError):
        szs.NeedlemanWunschScores(b2c, table, open=-200)


def test_strs_container():
    s = szs.Strs(["hello", "", "world", "café"])
    assert len(s) == 4
    assert list(s) == ["hello", "", "world", "café"]
    view = s[1:3]
    assert len(view) == 2 and list(view) == ["", "world"]
    assert s[-1] == "café"
    b = szs.Strs([b"\x00\xff", b"x"])
    assert list(b) == [b"\x00\xff", b"x"]
    with pytest.raises(TypeError):
        szs.Strs([1, 2])
    tape, bits = s[2:4].tape()
    assert bits == 64 and tape.count == 2


def test_strs_from_pyarrow():
    pa = pytest.importorskip("pyarrow")
    arrow = pa.array(["hello", "", "world", "a"])
    s = szs.Strs(arrow)
    assert list(s) == ["hello", "", "world", "a"]
    assert list(szs.Strs(arrow.slice(1, 2))) == ["", "world"]
    # Zero copy: the tape points into Arrow's own buffers, 32-bit offsets stay 32-bit, 64-bit ones stay 64-bit.
    tape, bits = s.tape()
    _, offsets_buffer, data_buffer = arrow.buffers()
    assert bits == 32 and tape.offsets == offsets_buffer.address and tape.data == data_buffer.address
    sliced, bits = szs.Strs(arrow.slice(1, 2)).tape()
    assert bits == 32 and sliced.offsets == offsets_buffer.address + 4 and sliced.count == 2
    large = pa.array(["xy", "z"], type=pa.large_string())
    tape, bits = szs.Strs(large).tape()
    assert bits == 64 and tape.offsets == large.buffers()[1].address


def test_calls_validate_before_running():
    engine = szs.LevenshteinDistances()
    with pytest.raises(TypeError):
        engine("not strs")
    with pytest.raises(TypeError):
        engine(szs.Strs(["a"]), device="gpu")
    with pytest.raises(ValueError):
        engine(szs.Strs(["a", "b"]), szs.Strs(["c"]), out=np.zeros((1, 1), np.uint64))
    with pytest.raises(TypeError):
        engine(szs.Strs(["a"]), szs.Strs(["c"]), out=np.zeros((1, 1), np.int64))
    with pytest.raises(ValueError):
        engine.pairwise(szs.Strs(["a", "b"]), szs.Strs(["c"]))
    # Empty inputs return empty matrices without touching a device.
    assert engine(szs.Strs([]), szs.Strs([])).shape == (0, 0)
    assert engine(szs.Strs(["a"]), szs.Strs([])).shape == (1, 0)


def test_server_validation_without_a_gpu():
    """The serving loop needs a GPU; the ABI structs match the header's layout."""
    from stringzillas_gb300 import _native
    import ctypes
    assert ctypes.sizeof(_native.ServerConfig) == 8 * 8
    assert ctypes.sizeof(_native.RequestInfo) == 7 * 8
    assert ctypes.sizeof(_native.ServerStats) == 10 * 8
    if "cuda" in szs.__capabilities__:
        pytest.skip("a GPU is visible")
    with pytest.raises(RuntimeError):
        szs.Server()
    # Submissions to an invalid handle fail cleanly instead of crashing.
    handle = ctypes.c_void_p()
    err = ctypes.c_char_p()
    ticket = ctypes.c_uint64()
    status = _native.lib.szs_gb300_server_submit(handle, None, None, None, None, ctypes.byref(ticket),
                                                 ctypes.byref(err))
    assert status != 0 and err.value
    assert _native.lib.szs_gb300_server_wait(handle, 1, None, ctypes.byref(err)) != 0


def test_serving_workload_shape():
    from stringzillas_gb300 import workloads as w
    requests = w.serving_requests(40, seed=3, max_pairs=64, max_length=300)
    kinds = [r["kind"] for r in requests]
    assert set(kinds) <= {"lev", "nw", "sw"} and kinds.count("lev") > 5
    for r in requests:
        assert 1 <= r["pairs"] <= 64
        assert len(r["first"][1]) == r["pairs"] + 1 == len(r["second"][1])
        lengths = np.diff(r["first"][1])
        assert lengths.min() >= 16 and lengths.max() <= 300
        assert r["cells"] == int(np.dot(lengths, np.diff(r["second"][1])))


def test_tuning_round_trip_and_validation():
    from stringzillas_gb300 import autotune, workloads as w
    engine = szs.NeedlemanWunschScores(*w.protein_table(), open=-11, extend=-1)
    assert engine.get_tuning() == {"packed_rows": [0] * 16, "cell_bits": [0] * 16, "band_min_rows": 0,
                                   "packed_warps": [0] * 4, "band_min_rows_packed": 0, "pipeline_chunk_kb": 0,
                                   "packed_step_cost": [0] * 4, "band_min_rows_few": 0, "band_min_rows_compare": 0,
                                   "band_wait_polls": 0, "short_max_rows": 0}
    tuning = {"packed_rows": [0, 0, 0, 4, 4, 8, 8, 12, 16, 16, 16, 0, 0, 0, 0, 0], "cell_bits": [32] + [0] * 15,
              "band_min_rows": 2048, "packed_warps": [2, 4, 8, 4], "band_min_rows_packed": 3000,
              "pipeline_chunk_kb": 8192, "packed_step_cost": [100, 170, 240, 320], "band_min_rows_few": 700,
              "band_min_rows_compare": 1500, "band_wait_polls": 1000, "short_max_rows": 32}
    engine.set_tuning(tuning)
    assert engine.get_tuning() == tuning
    for bad in ({"packed_rows": [3] * 16}, {"cell_bits": [16] * 16}, {"cell_bits": [48] * 16},
                {"packed_warps": [9, 0, 0, 0]}, {"packed_rows": [4] * 15}, {"bogus": 1}):
        with pytest.raises(ValueError):
            engine.set_tuning(bad)
    assert engine.get_tuning() == tuning  # rejected tunings leave the installed one
    engine.set_tuning(None)
    assert engine.get_tuning()["band_min_rows"] == 0
    # Families and applying a table.
    assert autotune.family_of(engine) == "nw-affine"
    assert autotune.family_of(szs.LevenshteinDistances()) == "lev-unit"
    assert autotune.family_of(szs.LevenshteinDistances(0, 2, 3, 3)) == "lev-linear"
    assert autotune.family_of(szs.SmithWatermanScores(*w.dna_table(), open=-5, extend=-5)) == "sw-linear"
    table = {"families": {"nw-affine": {"tuning": tuning}}}
    assert autotune.apply(engine, table) and engine.get_tuning() == tuning
    assert not autotune.apply(szs.LevenshteinDistances(), table)


def test_dense_table_constructor_validation():
    table = np.zeros((256, 256), dtype=np.int8)
    engine = szs.NeedlemanWunschScores.dense(table, open=-4, extend=-1)
    assert isinstance(engine, szs.NeedlemanWunschScores)
    assert isinstance(szs.SmithWatermanScores.dense(table), szs.SmithWatermanScores)
    with pytest.raises(ValueError):
        szs.NeedlemanWunschScores.dense(np.zeros((32, 32), dtype=np.int8))
    with pytest.raises(TypeError):
        szs.NeedlemanWunschScores.dense(np.zeros((256, 256), dtype=np.int16))
    with pytest.raises(TypeError):
        szs.NeedlemanWunschScores.dense([[0] * 256] * 256)


def test_step_cost_fit_recovers_planted_costs():
    """The autotuner's step-cost fit: timings made from planted per-step costs give those costs back."""
    from stringzillas_gb300 import autotune
    rng = np.random.default_rng(2)
    planted = [100, 170, 250, 340]
    classes = []
    for k in (6, 7, 8, 9):
        la, lb = rng.integers(1 << k, 1 << (k + 1), size=(2, 5000))
        n, m = np.minimum(la, lb), np.maximum(la, lb)
        timings = {f"16x2 R={rows}": cost * autotune.lane_steps(n, m, rows) * 1e-9
                   for rows, cost in zip(autotune.ROWS, planted)}
        classes.append((timings, (n, m)))
    assert autotune.fit_step_costs(classes) == planted
    assert autotune.fit_step_costs([]) == [0, 0, 0, 0]
