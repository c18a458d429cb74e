"""Python access to the parity oracle. TEST INFRASTRUCTURE ONLY.

Two CPU implementations of the StringZillas scoring path are reachable from here:

* ``Port``: the C restatement in ``oracle/szs_oracle.c`` (always buildable, on x86 and Arm);
* ``Reference``: the reference's own ``szs_*`` serial library compiled from the reference sources into
  ``oracle/_ref/libszs_ref.so`` by ``oracle/Makefile`` (only where the reference tree is present).

Only tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` import this module. Inputs are
Arrow-like tapes: a ``uint8`` data array plus ``uint64`` offsets with ``count + 1`` entries.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_PATH = os.path.join(HERE, "_build", "liboracle_port.so")
REF_PATH = os.path.join(HERE, "_ref", "libszs_ref.so")

LEVENSHTEIN, NEEDLEMAN_WUNSCH, SMITH_WATERMAN = 0, 1, 2
CAP_SERIAL = 1
CAP_ANY = 0x7FFFFFFF


class Costs(ctypes.Structure):
    """Mirror of ``oracle_costs_t``."""

    _fields_ = [
        ("kind", ctypes.c_int),
        ("match", ctypes.c_int8),
        ("mismatch", ctypes.c_int8),
        ("open", ctypes.c_int8),
        ("extend", ctypes.c_int8),
        ("byte_to_class", ctypes.c_uint8 * 256),
        ("class_costs", ctypes.c_int8 * 1024),
        ("dense_costs", ctypes.c_void_p),
        ("utf8", ctypes.c_int),
    ]


def levenshtein_costs(match=0, mismatch=1, open=1, extend=1) -> Costs:
    c = Costs()
    c.kind, c.match, c.mismatch, c.open, c.extend = LEVENSHTEIN, match, mismatch, open, extend
    return c


def levenshtein_utf8_costs(match=0, mismatch=1, open=1, extend=1) -> Costs:
    """Levenshtein over UTF-8 code points (the batch drivers decode both strings first)."""
    c = levenshtein_costs(match, mismatch, open, extend)
    c.utf8 = 1
    return c


def alignment_costs(kind, byte_to_class, class_costs, open, extend) -> Costs:
    c = Costs()
    c.kind, c.open, c.extend = kind, open, extend
    b2c = np.ascontiguousarray(byte_to_class, dtype=np.uint8).reshape(256)
    table = np.ascontiguousarray(class_costs, dtype=np.int8).reshape(1024)
    ctypes.memmove(c.byte_to_class, b2c.ctypes.data, 256)
    ctypes.memmove(c.class_costs, table.ctypes.data, 1024)
    return c


def dense_costs(kind, table, open, extend) -> Costs:
    """Costs over a dense 256 x 256 table [first byte][second byte] (the engine's dense-table extension). The
    returned object keeps the table alive."""
    c = Costs()
    c.kind, c.open, c.extend = kind, open, extend
    c._dense = np.ascontiguousarray(table, dtype=np.int8).reshape(65536)
    c.dense_costs = c._dense.ctypes.data
    return c


def build_port(force: bool = False) -> str:
    """Compiles the C restatement with the committed Makefile (plain gcc, no ISA flags)."""
    if force or not os.path.exists(PORT_PATH):
        subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    return PORT_PATH


def _ptr(array):
    return ctypes.c_void_p(array.ctypes.data) if array is not None else ctypes.c_void_p(0)


class Port:
    """The C restatement."""

    def __init__(self, path: str | None = None):
        self.lib = ctypes.CDLL(path or build_port())
        self.lib.oracle_score_pair.restype = ctypes.c_int64
        self.lib.oracle_score_pair.argtypes = [
            ctypes.POINTER(Costs), ctypes.c_char_p, ctypes.c_size_t, ctypes.c_char_p, ctypes.c_size_t]
        self.lib.oracle_score_pairs_u64tape.restype = ctypes.c_int
        self.lib.oracle_score_pairs_u64tape.argtypes = [ctypes.POINTER(Costs)] + [ctypes.c_void_p] * 4 + [
            ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t]
        self.lib.oracle_score_cross_u64tape.restype = ctypes.c_int
        self.lib.oracle_score_cross_u64tape.argtypes = [
            ctypes.POINTER(Costs), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p,
            ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t]

    def pair(self, costs: Costs, a: bytes, b: bytes) -> int:
        return int(self.lib.oracle_score_pair(ctypes.byref(costs), a, len(a), b, len(b)))

    def pairs(self, costs: Costs, first, second, threads: int = 0) -> np.ndarray:
        (fd, fo), (sd, so) = first, second
        fo = np.ascontiguousarray(fo, dtype=np.uint64)
        so = np.ascontiguousarray(so, dtype=np.uint64)
        count = len(fo) - 1
        out = np.zeros(count, dtype=np.int64)
        if count:
            rc = self.lib.oracle_score_pairs_u64tape(
                ctypes.byref(costs), _ptr(fd), _ptr(fo), _ptr(sd), _ptr(so), count, _ptr(out), threads)
            if rc:
                raise MemoryError("oracle scratch allocation failed")
        return out

    def cross(self, costs: Costs, queries, candidates=None, threads: int = 0) -> np.ndarray:
        qd, qo = queries
        qo = np.ascontiguousarray(qo, dtype=np.uint64)
        nq = len(qo) - 1
        if candidates is None:
            cd, co, nc = None, None, nq
        else:
            cd, co = candidates
            co = np.ascontiguousarray(co, dtype=np.uint64)
            nc = len(co) - 1
        out = np.zeros((nq, nc), dtype=np.int64)
        if nq and nc:
            rc = self.lib.oracle_score_cross_u64tape(
                ctypes.byref(costs), _ptr(qd), _ptr(qo), nq, _ptr(cd) if cd is not None else None,
                _ptr(co) if co is not None else None, nc, _ptr(out), nc, threads)
            if rc:
                raise MemoryError("oracle scratch allocation failed")
        return out


class _U64Tape(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("offsets", ctypes.c_void_p), ("count", ctypes.c_size_t)]


def reference_available() -> bool:
    return os.path.exists(REF_PATH)


def fingerprints(dimensions, texts, window_widths=None, seed=0):
    """(hashes, counts), uint32 [count, dimensions], from the oracle's restatement of the reference's Min-Hash."""
    data, offsets = texts
    offsets = np.ascontiguousarray(offsets, dtype=np.uint64)
    data = np.ascontiguousarray(data, dtype=np.uint8) if len(data) else np.zeros(1, dtype=np.uint8)
    count = len(offsets) - 1
    hashes = np.zeros((count, dimensions), dtype=np.uint32)
    counts = np.zeros((count, dimensions), dtype=np.uint32)
    widths = None if window_widths is None else np.ascontiguousarray(window_widths, dtype=np.uint64)
    lib = Port().lib
    lib.oracle_fingerprints_u64tape(ctypes.c_size_t(dimensions), None if widths is None else _ptr(widths),
                                    ctypes.c_size_t(0 if widths is None else len(widths)), ctypes.c_uint64(seed),
                                    _ptr(data), _ptr(offsets), ctypes.c_size_t(count), _ptr(hashes),
                                    ctypes.c_size_t(dimensions * 4), _ptr(counts), ctypes.c_size_t(dimensions * 4))
    return hashes, counts


class Reference:
    """The reference's own ``szs_*`` C-ABI, compiled from its sources (serial engines)."""

    def __init__(self, path: str | None = None):
        self.lib = ctypes.CDLL(path or REF_PATH)
        self._scope = ctypes.c_void_p()
        err = ctypes.c_char_p()
        if self.lib.szs_device_scope_init_default(ctypes.byref(self._scope), ctypes.byref(err)) != 0:
            raise RuntimeError(f"reference scope: {err.value}")

    def _engine(self, costs: Costs):
        engine, err = ctypes.c_void_p(), ctypes.c_char_p()
        if costs.kind == LEVENSHTEIN and costs.utf8:
            rc = self.lib.szs_levenshtein_distances_utf8_init(
                ctypes.c_int8(costs.match), ctypes.c_int8(costs.mismatch), ctypes.c_int8(costs.open),
                ctypes.c_int8(costs.extend), None, ctypes.c_int(CAP_SERIAL), ctypes.byref(engine), ctypes.byref(err))
            return engine, rc, "levenshtein_distances_utf8"
        if costs.kind == LEVENSHTEIN:
            rc = self.lib.szs_levenshtein_distances_init(
                ctypes.c_int8(costs.match), ctypes.c_int8(costs.mismatch), ctypes.c_int8(costs.open),
                ctypes.c_int8(costs.extend), None, ctypes.c_int(CAP_SERIAL), ctypes.byref(engine), ctypes.byref(err))
            return engine, rc, "levenshtein_distances"
        name = "needleman_wunsch_scores" if costs.kind == NEEDLEMAN_WUNSCH else "smith_waterman_scores"
        init = getattr(self.lib, f"szs_{name}_init")
        rc = init(ctypes.c_void_p(ctypes.addressof(costs.byte_to_class)),
                  ctypes.c_void_p(ctypes.addressof(costs.class_costs)), ctypes.c_int8(costs.open),
                  ctypes.c_int8(costs.extend), None, ctypes.c_int(CAP_SERIAL), ctypes.byref(engine), ctypes.byref(err))
        return engine, rc, name

    def cross(self, costs: Costs, queries, candidates=None) -> np.ndarray:
        engine, rc, name = self._engine(costs)
        if rc != 0:
            raise RuntimeError(f"reference init failed: {rc}")
        try:
            qd, qo = queries
            qo = np.ascontiguousarray(qo, dtype=np.uint64)
            qd = np.ascontiguousarray(qd, dtype=np.uint8) if len(qd) else np.zeros(1, dtype=np.uint8)
            q = _U64Tape(qd.ctypes.data, qo.ctypes.data, len(qo) - 1)
            if candidates is None:
                c_ptr, nc = None, len(qo) - 1
            else:
                cd, co = candidates
                co = np.ascontiguousarray(co, dtype=np.uint64)
                cd = np.ascontiguousarray(cd, dtype=np.uint8) if len(cd) else np.zeros(1, dtype=np.uint8)
                c = _U64Tape(cd.ctypes.data, co.ctypes.data, len(co) - 1)
                c_ptr, nc = ctypes.byref(c), len(co) - 1
            dtype = np.uint64 if costs.kind == LEVENSHTEIN else np.int64
            out = np.zeros((len(qo) - 1, nc), dtype=dtype)
            err = ctypes.c_char_p()
            fn = getattr(self.lib, f"szs_{name}_u64tape")
            rc = fn(engine, self._scope, ctypes.byref(q), c_ptr, ctypes.c_void_p(out.ctypes.data),
                    ctypes.c_size_t(max(nc, 1)), ctypes.byref(err))
            if rc != 0:
                raise RuntimeError(f"reference call failed: {rc} {err.value}")
            return out.astype(np.int64)
        finally:
            getattr(self.lib, f"szs_{name}_free")(engine)

    def fingerprints(self, dimensions, texts, window_widths=None, seed=0):
        """(hashes, counts) from the reference's `szs_fingerprints_u64tape` (rows `dimensions * 4` bytes apart)."""
        engine, err = ctypes.c_void_p(), ctypes.c_char_p()
        widths = None if window_widths is None else (ctypes.c_size_t * len(window_widths))(*window_widths)
        rc = self.lib.szs_fingerprints_init(ctypes.c_size_t(dimensions), ctypes.c_size_t(256), widths,
                                            ctypes.c_size_t(0 if window_widths is None else len(window_widths)),
                                            ctypes.c_uint64(seed), None, ctypes.c_int(CAP_SERIAL),
                                            ctypes.byref(engine), ctypes.byref(err))
        if rc != 0:
            raise RuntimeError(f"reference fingerprint init failed: {rc} {err.value}")
        try:
            data, offsets = texts
            offsets = np.ascontiguousarray(offsets, dtype=np.uint64)
            data = np.ascontiguousarray(data, dtype=np.uint8) if len(data) else np.zeros(1, dtype=np.uint8)
            tape = _U64Tape(data.ctypes.data, offsets.ctypes.data, len(offsets) - 1)
            hashes = np.zeros((len(offsets) - 1, dimensions), dtype=np.uint32)
            counts = np.zeros_like(hashes)
            rc = self.lib.szs_fingerprints_u64tape(engine, self._scope, ctypes.byref(tape),
                                                   ctypes.c_void_p(hashes.ctypes.data), ctypes.c_size_t(dimensions * 4),
                                                   ctypes.c_void_p(counts.ctypes.data), ctypes.c_size_t(dimensions * 4),
                                                   ctypes.byref(err))
            if rc != 0:
                raise RuntimeError(f"reference fingerprints failed: {rc} {err.value}")
            return hashes, counts
        finally:
            self.lib.szs_fingerprints_free(engine)

    def pairs(self, costs: Costs, first, second) -> np.ndarray:
        """One 1x1 call per pair, the way a pairwise caller drives the cross-product ABI."""
        (fd, fo), (sd, so) = first, second
        count = len(fo) - 1
        out = np.zeros(count, dtype=np.int64)
        for i in range(count):
            a = (fd[fo[i]:fo[i + 1]], np.array([0, fo[i + 1] - fo[i]], dtype=np.uint64))
            b = (sd[so[i]:so[i + 1]], np.array([0, so[i + 1] - so[i]], dtype=np.uint64))
            out[i] = self.cross(costs, a, b)[0, 0]
        return out

    def __del__(self):
        try:
            self.lib.szs_device_scope_free(self._scope)
        except Exception:
            pass
