"""Loads ``libszs_gb300.so`` and declares the C-ABI prototypes (include/stringzillas_gb300.h).

The library is the product: there is no CPU fallback. If it cannot be loaded (not built, no CUDA runtime), importing
the package raises, so nothing silently runs elsewhere.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

c_size_t = ctypes.c_size_t
c_void_p = ctypes.c_void_p
c_int = ctypes.c_int
c_int8 = ctypes.c_int8
c_char_p = ctypes.c_char_p
c_status = ctypes.c_int


class U32Tape(ctypes.Structure):
    """``sz_sequence_u32tape_t``"""
    _fields_ = [("data", c_void_p), ("offsets", c_void_p), ("count", c_size_t)]


class U64Tape(ctypes.Structure):
    """``sz_sequence_u64tape_t``"""
    _fields_ = [("data", c_void_p), ("offsets", c_void_p), ("count", c_size_t)]


# ``sz_sequence_member_start_t`` / ``sz_sequence_member_length_t``: (handle, index) -> start pointer / length.
SequenceStart = ctypes.CFUNCTYPE(c_void_p, c_void_p, c_size_t)
SequenceLength = ctypes.CFUNCTYPE(c_size_t, c_void_p, c_size_t)


class Sequence(ctypes.Structure):
    """``sz_sequence_t``: strings reached through two callbacks."""
    _fields_ = [("handle", c_void_p), ("count", c_size_t), ("get_start", SequenceStart),
                ("get_length", SequenceLength)]


class Stats(ctypes.Structure):
    """``szs_gb300_stats_t``"""
    _fields_ = [
        ("last_call_ms", ctypes.c_double),
        ("last_compute_ms", ctypes.c_double),
        ("last_cells", ctypes.c_uint64),
        ("last_pairs", ctypes.c_uint64),
        ("last_launches", ctypes.c_uint64),
        ("graph_replays", ctypes.c_uint64),
        ("kernel_launches", ctypes.c_uint64),
    ]


def _load() -> ctypes.CDLL:
    # Rebuilds only when the sources changed since the last build (content digest), so a stale library with
    # missing entry points is never loaded.
    path = _build.build() if _build.nvcc_available() else _build.LIBRARY
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing and nvcc is unavailable to build it")
    return ctypes.CDLL(path)


lib = _load()
LIBRARY_PATH = _build.LIBRARY

_err = ctypes.POINTER(c_char_p)

for _name in ("szs_version_major", "szs_version_minor", "szs_version_patch"):
    getattr(lib, _name).restype = c_int
    getattr(lib, _name).argtypes = []
for _name in ("szs_capabilities", "szs_capabilities_comptime", "szs_capabilities_runtime"):
    getattr(lib, _name).restype = ctypes.c_uint32
    getattr(lib, _name).argtypes = []

lib.szs_device_scope_init_default.restype = c_status
lib.szs_device_scope_init_default.argtypes = [ctypes.POINTER(c_void_p), _err]
lib.szs_device_scope_init_cpu_cores.restype = c_status
lib.szs_device_scope_init_cpu_cores.argtypes = [c_size_t, ctypes.POINTER(c_void_p), _err]
lib.szs_device_scope_init_gpu_device.restype = c_status
lib.szs_device_scope_init_gpu_device.argtypes = [c_size_t, ctypes.POINTER(c_void_p), _err]
lib.szs_device_scope_get_cpu_cores.restype = c_status
lib.szs_device_scope_get_cpu_cores.argtypes = [c_void_p, ctypes.POINTER(c_size_t), _err]
lib.szs_device_scope_get_gpu_device.restype = c_status
lib.szs_device_scope_get_gpu_device.argtypes = [c_void_p, ctypes.POINTER(c_size_t), _err]
lib.szs_device_scope_get_capabilities.restype = c_status
lib.szs_device_scope_get_capabilities.argtypes = [c_void_p, ctypes.POINTER(ctypes.c_uint32), _err]
lib.szs_gb300_device_scope_init_stream.restype = c_status
lib.szs_gb300_device_scope_init_stream.argtypes = [c_size_t, c_void_p, ctypes.POINTER(c_void_p), _err]
lib.szs_device_scope_free.restype = None
lib.szs_device_scope_free.argtypes = [c_void_p]

lib.szs_unified_alloc.restype = c_void_p
lib.szs_unified_alloc.argtypes = [c_size_t]
lib.szs_unified_free.restype = None
lib.szs_unified_free.argtypes = [c_void_p, c_size_t]

lib.szs_levenshtein_distances_init.restype = c_status
lib.szs_levenshtein_distances_init.argtypes = [c_int8, c_int8, c_int8, c_int8, c_void_p, ctypes.c_uint32,
                                               ctypes.POINTER(c_void_p), _err]
lib.szs_levenshtein_distances_utf8_init.restype = c_status
lib.szs_levenshtein_distances_utf8_init.argtypes = [c_int8, c_int8, c_int8, c_int8, c_void_p, ctypes.c_uint32,
                                                    ctypes.POINTER(c_void_p), _err]
for _algo in ("needleman_wunsch_scores", "smith_waterman_scores"):
    fn = getattr(lib, f"szs_{_algo}_init")
    fn.restype = c_status
    fn.argtypes = [c_void_p, c_void_p, c_int8, c_int8, c_void_p, ctypes.c_uint32, ctypes.POINTER(c_void_p), _err]
for _algo in ("levenshtein_distances", "levenshtein_distances_utf8", "needleman_wunsch_scores",
              "smith_waterman_scores"):
    for _suffix in ("_u32tape", "_u64tape", ""):
        fn = getattr(lib, f"szs_{_algo}{_suffix}")
        fn.restype = c_status
        fn.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_size_t, _err]
    fn = getattr(lib, f"szs_{_algo}_free")
    fn.restype = None
    fn.argtypes = [c_void_p]
for _algo in ("levenshtein_distances", "needleman_wunsch_scores", "smith_waterman_scores"):
    for _suffix in ("_pairwise_u32tape", "_pairwise_u64tape"):
        fn = getattr(lib, f"szs_{_algo}{_suffix}")
        fn.restype = c_status
        fn.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, _err]
    fn = getattr(lib, f"szs_{_algo}_free")
    fn.restype = None
    fn.argtypes = [c_void_p]

for _algo in ("fingerprints", "fingerprints_utf8"):
    fn = getattr(lib, f"szs_{_algo}_init")
    fn.restype = c_status
    fn.argtypes = [c_size_t, c_size_t, c_void_p, c_size_t, ctypes.c_uint64, c_void_p, ctypes.c_uint32,
                   ctypes.POINTER(c_void_p), _err]
    for _suffix in ("_sequence", "_u32tape", "_u64tape"):
        fn = getattr(lib, f"szs_{_algo}{_suffix}")
        fn.restype = c_status
        fn.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p, c_size_t, c_void_p, c_size_t, _err]
    fn = getattr(lib, f"szs_{_algo}_free")
    fn.restype = None
    fn.argtypes = [c_void_p]

for _algo in ("needleman_wunsch_scores", "smith_waterman_scores"):
    fn = getattr(lib, f"szs_gb300_{_algo}_init_dense")
    fn.restype = c_status
    fn.argtypes = [c_void_p, c_int8, c_int8, c_void_p, ctypes.c_uint32, ctypes.POINTER(c_void_p), _err]

lib.szs_gb300_score_pairwise_noalloc_u64tape.restype = c_status
lib.szs_gb300_score_pairwise_noalloc_u64tape.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, _err]
lib.szs_gb300_engine_set_schedule.restype = c_status
lib.szs_gb300_engine_set_schedule.argtypes = [c_void_p, c_int, _err]
lib.szs_gb300_measure_integer_peaks.restype = c_status
lib.szs_gb300_measure_integer_peaks.argtypes = [c_size_t, ctypes.POINTER(ctypes.c_double), c_size_t, _err]
lib.szs_gb300_engine_get_stats.restype = c_status
lib.szs_gb300_engine_get_stats.argtypes = [c_void_p, ctypes.POINTER(Stats), _err]


class Tuning(ctypes.Structure):
    """``szs_gb300_tuning_t``"""
    _fields_ = [
        ("packed_rows", ctypes.c_uint8 * 16),
        ("cell_bits", ctypes.c_uint8 * 16),
        ("band_min_rows", ctypes.c_uint32),
        ("packed_warps", ctypes.c_uint32 * 4),
        ("band_min_rows_packed", ctypes.c_uint32),
        ("pipeline_chunk_kb", ctypes.c_uint32),
        ("packed_step_cost", ctypes.c_uint16 * 4),
        ("band_min_rows_few", ctypes.c_uint32),
        ("band_min_rows_compare", ctypes.c_uint32),
        ("band_wait_polls", ctypes.c_uint32),
        ("short_max_rows", ctypes.c_uint32),
    ]


lib.szs_gb300_engine_set_tuning.restype = c_status
lib.szs_gb300_engine_set_tuning.argtypes = [c_void_p, ctypes.POINTER(Tuning), _err]
lib.szs_gb300_engine_get_tuning.restype = c_status
lib.szs_gb300_engine_get_tuning.argtypes = [c_void_p, ctypes.POINTER(Tuning), _err]


class ServerConfig(ctypes.Structure):
    """``szs_gb300_server_config_t``"""
    _fields_ = [
        ("gpu_device", c_size_t),
        ("arena_bytes", c_size_t),
        ("lanes", c_size_t),
        ("max_batch_pairs", c_size_t),
        ("max_batch_requests", c_size_t),
        ("schedule", c_int),
        ("max_batch_cells", c_size_t),
        ("aging_ms", c_size_t),
    ]


class RequestInfo(ctypes.Structure):
    """``szs_gb300_request_info_t``"""
    _fields_ = [
        ("status", c_status),
        ("admitted_ms", ctypes.c_double),
        ("done_ms", ctypes.c_double),
        ("batch", ctypes.c_uint64),
        ("batch_requests", ctypes.c_uint64),
        ("batch_pairs", ctypes.c_uint64),
        ("cells", ctypes.c_uint64),
    ]


class ServerStats(ctypes.Structure):
    """``szs_gb300_server_stats_t``"""
    _fields_ = [
        ("requests", ctypes.c_uint64),
        ("completed", ctypes.c_uint64),
        ("batches", ctypes.c_uint64),
        ("pairs", ctypes.c_uint64),
        ("cells", ctypes.c_uint64),
        ("arena_bytes", ctypes.c_uint64),
        ("arena_peak_bytes", ctypes.c_uint64),
        ("peak_inflight", ctypes.c_uint64),
        ("kernel_launches", ctypes.c_uint64),
        ("device_ms", ctypes.c_double),
    ]


lib.szs_gb300_server_init.restype = c_status
lib.szs_gb300_server_init.argtypes = [ctypes.POINTER(ServerConfig), ctypes.POINTER(c_void_p), _err]
lib.szs_gb300_server_submit.restype = c_status
lib.szs_gb300_server_submit.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                        ctypes.POINTER(ctypes.c_uint64), _err]
lib.szs_gb300_server_wait.restype = c_status
lib.szs_gb300_server_wait.argtypes = [c_void_p, ctypes.c_uint64, ctypes.POINTER(RequestInfo), _err]
lib.szs_gb300_server_get_stats.restype = c_status
lib.szs_gb300_server_get_stats.argtypes = [c_void_p, ctypes.POINTER(ServerStats), _err]
lib.szs_gb300_server_free.restype = None
lib.szs_gb300_server_free.argtypes = [c_void_p]

# Status codes (include/stringzillas_gb300.h; values of the reference's types.h:699-721).
SUCCESS = 0
BAD_ALLOC = -10
INVALID_UTF8 = -12
OVERFLOW_RISK = -14
UNEXPECTED_DIMENSIONS = -15
MISSING_GPU = -16
DEVICE_CODE_MISMATCH = -17
DEVICE_MEMORY_MISMATCH = -18
UNKNOWN = -1

CAP_CUDA, CAP_KEPLER, CAP_HOPPER = 1 << 21, 1 << 22, 1 << 23
CAP_SERIAL, CAP_PARALLEL = 1, 1 << 2


def raise_for(status: int, message, context: str) -> None:
    """Maps a status onto the exception type the reference's binding raises
    (python/stringzillas/stringzillas.c:21-32)."""
    if status == SUCCESS:
        return
    detail = message.decode() if isinstance(message, bytes) else (message or "Unknown error")
    text = f"{context}: {detail}"
    if status == BAD_ALLOC:
        raise MemoryError(text)
    if status in (INVALID_UTF8, UNEXPECTED_DIMENSIONS):
        raise ValueError(text)
    if status == OVERFLOW_RISK:
        raise OverflowError(text)
    raise RuntimeError(text)
