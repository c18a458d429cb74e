"""Python face of the serving loop (``szs_gb300_server_*`` in include/stringzillas_gb300.h).

A ``Server`` owns one device arena and a few lanes; ``submit`` queues one request (a pairwise batch on any engine)
and returns a ``Ticket`` at once; ``Ticket.result()`` blocks until the request's scores are in its output array.
Requests that arrive while lanes are busy are merged into the next batch of the same engine (continuous batching).
The reference has no serving layer; its engines are called synchronously, one batch per call.
"""
from __future__ import annotations

import ctypes
import threading

import numpy as np

from . import _native
from ._native import lib

_SCHEDULES = {"batched": 0, "plain": 1}


def _u64_tape(strs):
    """(U64Tape, keep-alive) for a Strs; u32 offsets are widened on the host."""
    tape, bits = strs.tape()
    if bits == 64:
        return tape, (strs,)
    offsets = np.ascontiguousarray(strs._host_offsets()[strs._start:strs._start + len(strs) + 1], dtype=np.uint64)
    data = strs._data
    data_ptr = tape.data
    return _native.U64Tape(data_ptr, offsets.ctypes.data, len(strs)), (strs, offsets, data)


class Ticket:
    """One submitted request. ``result()`` waits for it (once) and returns the scores; ``info`` then holds the
    request's timings: ``admitted_ms`` and ``done_ms`` since submission, the batch it ran in and its cells."""

    def __init__(self, server, number, output, keep):
        self._server, self._number, self._output, self._keep = server, number, output, keep
        self._lock = threading.Lock()
        self._waited = False
        self.info = None

    def result(self):
        with self._lock:
            if not self._waited:
                info = _native.RequestInfo()
                err = ctypes.c_char_p()
                status = lib.szs_gb300_server_wait(self._server._handle, self._number, ctypes.byref(info),
                                                   ctypes.byref(err))
                self._waited = True
                self._keep = None
                self.info = {name: getattr(info, name) for name, _ in info._fields_}
                _native.raise_for(status, err.value, "serving request")
        return self._output


class Server:
    """``Server(gpu_device=0, arena_bytes=1 << 30, lanes=4, max_batch_pairs=1 << 22, max_batch_requests=0,
    schedule="batched", max_batch_cells=1 << 33, aging_ms=0)``.

    ``aging_ms > 0`` admits the smallest waiting request (by cells) first unless the oldest has waited that long;
    0 keeps arrival order.

    ``max_batch_requests=1, lanes=1, schedule="plain"`` gives the per-request form: every request on its own,
    one after another, with one plain launch each.
    """

    def __init__(self, gpu_device=0, arena_bytes=1 << 30, lanes=4, max_batch_pairs=1 << 22, max_batch_requests=0,
                 schedule="batched", max_batch_cells=1 << 33, aging_ms=0):
        config = _native.ServerConfig(int(gpu_device), int(arena_bytes), int(lanes), int(max_batch_pairs),
                                      int(max_batch_requests), _SCHEDULES[schedule], int(max_batch_cells),
                                      int(aging_ms))
        self._handle = ctypes.c_void_p()
        err = ctypes.c_char_p()
        status = lib.szs_gb300_server_init(ctypes.byref(config), ctypes.byref(self._handle), ctypes.byref(err))
        _native.raise_for(status, err.value, "server initialization")

    def submit(self, engine, first, second, out=None) -> Ticket:
        """Queues ``out[i] = engine's score(first[i], second[i])``; returns a Ticket immediately. Inputs must stay
        alive and unchanged until the ticket's result is taken (the Ticket keeps references to them)."""
        from . import _as_strs, _pointer_of
        first, second = _as_strs(first, "first"), _as_strs(second, "second")
        if len(first) != len(second):
            raise ValueError("pairwise inputs must have the same length")
        output = np.empty(len(first), dtype=engine._dtype) if out is None else out
        a_tape, a_keep = _u64_tape(first)
        b_tape, b_keep = _u64_tape(second)
        number = ctypes.c_uint64()
        err = ctypes.c_char_p()
        status = lib.szs_gb300_server_submit(self._handle, engine.handle, ctypes.byref(a_tape), ctypes.byref(b_tape),
                                             ctypes.c_void_p(_pointer_of(output) if len(first) else 0),
                                             ctypes.byref(number), ctypes.byref(err))
        _native.raise_for(status, err.value, "serving submit")
        return Ticket(self, number.value, output, (a_tape, b_tape, a_keep, b_keep, engine))

    def stats(self) -> dict:
        stats = _native.ServerStats()
        err = ctypes.c_char_p()
        _native.raise_for(lib.szs_gb300_server_get_stats(self._handle, ctypes.byref(stats), ctypes.byref(err)),
                          err.value, "server stats")
        return {name: getattr(stats, name) for name, _ in stats._fields_}

    def close(self):
        if getattr(self, "_handle", None) and self._handle.value:
            lib.szs_gb300_server_free(self._handle)
            self._handle = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        self.close()
