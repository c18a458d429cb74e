"""The C-ABI library loads and exports every declared entry point; host-side validation works without a GPU."""
import ctypes
import os
import re

import numpy as np
import pytest

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "stringzillas_gb300.h")


@pytest.fixture(scope="module")
def native():
    from stringzillas_gb300 import _native
    return _native


def declared_functions():
    with open(HEADER) as f:
        text = f.read()
    return sorted(set(re.findall(r"SZS_GB300_API\s+[\w\s\*]+?\b(\w+)\s*\(", text)))


def test_every_declared_symbol_is_exported(native):
    names = declared_functions()
    assert len(names) >= 40
    missing = [name for name in names if not hasattr(native.lib, name)]
    assert not missing, f"not exported: {missing}"


def test_reference_entry_points_are_all_declared():
    """Every scoring, scope, runtime and stub symbol of the reference's header has a declaration here
    (include/stringzillas/stringzillas.h:33-551)."""
    names = set(declared_functions())
    expected = {"szs_version_major", "szs_version_minor", "szs_version_patch", "szs_capabilities",
                "szs_capabilities_comptime", "szs_capabilities_runtime", "sz_memory_allocator_init_unified",
                "szs_device_scope_init_default", "szs_device_scope_init_cpu_cores", "szs_device_scope_init_gpu_device",
                "szs_device_scope_get_cpu_cores", "szs_device_scope_get_gpu_device",
                "szs_device_scope_get_capabilities", "szs_device_scope_free", "szs_unified_alloc", "szs_unified_free",
                "szs_fingerprints_init", "szs_fingerprints_sequence", "szs_fingerprints_u32tape",
                "szs_fingerprints_u64tape", "szs_fingerprints_free", "szs_fingerprints_utf8_init",
                "szs_fingerprints_utf8_sequence", "szs_fingerprints_utf8_u32tape", "szs_fingerprints_utf8_u64tape",
                "szs_fingerprints_utf8_free"}
    for algo in ("levenshtein_distances", "levenshtein_distances_utf8", "needleman_wunsch_scores",
                 "smith_waterman_scores"):
        expected |= {f"szs_{algo}_init", f"szs_{algo}", f"szs_{algo}_u32tape", f"szs_{algo}_u64tape",
                     f"szs_{algo}_free"}
    assert expected <= names, sorted(expected - names)


def test_versions(native):
    assert (native.lib.szs_version_major(), native.lib.szs_version_minor(), native.lib.szs_version_patch()) == (5, 3, 2)
    assert native.lib.szs_capabilities_comptime() & native.CAP_CUDA


def make_engine(native, kind, **kw):
    handle = ctypes.c_void_p()
    err = ctypes.c_char_p()
    if kind == "lev":
        status = native.lib.szs_levenshtein_distances_init(kw.get("match", 0), kw.get("mismatch", 1),
                                                           kw.get("open", 1), kw.get("extend", 1), None, 0,
                                                           ctypes.byref(handle), ctypes.byref(err))
    else:
        b2c = np.zeros(256, np.uint8)
        table = np.zeros((32, 32), np.int8)
        status = getattr(native.lib, f"szs_{kind}_init")(b2c.ctypes.data, table.ctypes.data, -2, -1, None, 0,
                                                         ctypes.byref(handle), ctypes.byref(err))
    return status, handle, err


@pytest.mark.parametrize("kind", ["lev", "needleman_wunsch_scores", "smith_waterman_scores"])
def test_engine_lifecycle_without_gpu(native, kind):
    status, handle, err = make_engine(native, kind)
    assert status == 0 and handle.value
    algo = "levenshtein_distances" if kind == "lev" else kind
    getattr(native.lib, f"szs_{algo}_free")(handle)


def test_engine_must_be_null_on_entry(native):
    handle = ctypes.c_void_p(1234)
    err = ctypes.c_char_p()
    status = native.lib.szs_levenshtein_distances_init(0, 1, 1, 1, None, 0, ctypes.byref(handle), ctypes.byref(err))
    assert status != 0 and err.value


def test_negative_levenshtein_costs_are_rejected(native):
    status, _, err = make_engine(native, "lev", match=-1)
    assert status == native.OVERFLOW_RISK and b"non-negative" in err.value


def test_cpu_scope_is_rejected_before_any_device_work(native):
    status, engine, _ = make_engine(native, "lev")
    scope = ctypes.c_void_p()
    err = ctypes.c_char_p()
    assert native.lib.szs_device_scope_init_cpu_cores(4, ctypes.byref(scope), ctypes.byref(err)) == 0
    cores = ctypes.c_size_t()
    assert native.lib.szs_device_scope_get_cpu_cores(scope, ctypes.byref(cores), ctypes.byref(err)) == 0
    assert cores.value == 4
    data = np.frombuffer(b"abcabd", np.uint8)
    offsets = np.array([0, 3, 6], np.uint64)
    tape = native.U64Tape(data.ctypes.data, offsets.ctypes.data, 2)
    out = np.zeros((2, 2), np.uint64)
    status = native.lib.szs_levenshtein_distances_u64tape(engine, scope, ctypes.byref(tape), ctypes.byref(tape),
                                                          out.ctypes.data, 2, ctypes.byref(err))
    assert status == native.DEVICE_CODE_MISMATCH
    native.lib.szs_device_scope_free(scope)
    native.lib.szs_levenshtein_distances_free(engine)


def test_pairwise_count_mismatch_and_small_stride(native):
    _, engine, _ = make_engine(native, "lev")
    err = ctypes.c_char_p()
    data = np.frombuffer(b"abcabd", np.uint8)
    two = np.array([0, 3, 6], np.uint64)
    one = np.array([0, 3], np.uint64)
    a = native.U64Tape(data.ctypes.data, two.ctypes.data, 2)
    b = native.U64Tape(data.ctypes.data, one.ctypes.data, 1)
    out = np.zeros(4, np.int64)
    assert native.lib.szs_levenshtein_distances_pairwise_u64tape(engine, None, ctypes.byref(a), ctypes.byref(b),
                                                                 out.ctypes.data, ctypes.byref(err)) == \
        native.UNEXPECTED_DIMENSIONS
    assert native.lib.szs_levenshtein_distances_u64tape(engine, None, ctypes.byref(a), ctypes.byref(a),
                                                        out.ctypes.data, 1, ctypes.byref(err)) == \
        native.UNEXPECTED_DIMENSIONS
    native.lib.szs_levenshtein_distances_free(engine)


def test_fingerprints_engine_validates_its_arguments(native):
    """Creation is host-only; calls need a GPU (c/stringzillas/fingerprints.cuh:27-141)."""
    err = ctypes.c_char_p()
    widths = (ctypes.c_size_t * 2)(5, 0)
    handle = ctypes.c_void_p()
    assert native.lib.szs_fingerprints_init(64, 256, widths, 2, 42, None, 0, ctypes.byref(handle),
                                            ctypes.byref(err)) == native.UNEXPECTED_DIMENSIONS
    assert not handle.value
    assert native.lib.szs_fingerprints_init(0, 256, None, 0, 42, None, 0, ctypes.byref(handle),
                                            ctypes.byref(err)) == native.UNEXPECTED_DIMENSIONS
    for init in (native.lib.szs_fingerprints_init, native.lib.szs_fingerprints_utf8_init):
        handle = ctypes.c_void_p()
        assert init(100, 256, None, 0, 7, None, 0, ctypes.byref(handle), ctypes.byref(err)) == native.SUCCESS
        assert handle.value
        # A second init into a live handle is refused.
        assert init(100, 256, None, 0, 7, None, 0, ctypes.byref(handle), ctypes.byref(err)) == native.UNKNOWN
        data = np.frombuffer(b"hello world", dtype=np.uint8).copy()
        offsets = np.array([0, 5, 11], dtype=np.uint64)
        tape = native.U64Tape(data.ctypes.data, offsets.ctypes.data, 2)
        hashes = np.zeros((2, 100), np.uint32)
        counts = np.zeros((2, 100), np.uint32)
        # Strides are bytes and must cover a row.
        assert native.lib.szs_fingerprints_u64tape(handle, None, ctypes.byref(tape), hashes.ctypes.data, 100,
                                                   counts.ctypes.data, 400, ctypes.byref(err)) == \
            native.UNEXPECTED_DIMENSIONS
        status = native.lib.szs_fingerprints_u64tape(handle, None, ctypes.byref(tape), hashes.ctypes.data, 400,
                                                     counts.ctypes.data, 400, ctypes.byref(err))
        assert status == native.MISSING_GPU  # no GPU in the CPU suite
        native.lib.szs_fingerprints_free(handle)
    # Freeing a scoring engine through the fingerprint entry point is ignored (handles are tagged).
    native.lib.szs_fingerprints_free(None)


def test_utf8_and_byte_engines_do_not_mix(native):
    """UTF-8 engines are their own handle type, as in the reference: byte entry points refuse them and back."""
    err = ctypes.c_char_p()
    utf8, byte = ctypes.c_void_p(), ctypes.c_void_p()
    assert native.lib.szs_levenshtein_distances_utf8_init(0, 1, 1, 1, None, 0, ctypes.byref(utf8),
                                                          ctypes.byref(err)) == native.SUCCESS
    assert native.lib.szs_levenshtein_distances_init(0, 1, 1, 1, None, 0, ctypes.byref(byte),
                                                     ctypes.byref(err)) == native.SUCCESS
    data = np.frombuffer("αβγ".encode(), dtype=np.uint8).copy()
    offsets = np.array([0, len(data)], dtype=np.uint64)
    tape = native.U64Tape(data.ctypes.data, offsets.ctypes.data, 1)
    out = np.zeros(1, dtype=np.uint64)
    assert native.lib.szs_levenshtein_distances_u64tape(utf8, None, ctypes.byref(tape), ctypes.byref(tape),
                                                        out.ctypes.data, 1, ctypes.byref(err)) == native.UNKNOWN
    assert native.lib.szs_levenshtein_distances_utf8_u64tape(byte, None, ctypes.byref(tape), ctypes.byref(tape),
                                                             out.ctypes.data, 1, ctypes.byref(err)) == native.UNKNOWN
    native.lib.szs_levenshtein_distances_utf8_free(utf8)
    native.lib.szs_levenshtein_distances_free(byte)
