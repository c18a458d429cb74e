"""GB300-native batched Levenshtein / Needleman-Wunsch / Smith-Waterman scoring.

Drop-in for the scoring callables of the reference's ``stringzillas`` module
(python/stringzillas/similarities.c, python/README.md:351-393):

    LevenshteinDistances(match=0, mismatch=1, open=1, extend=1, capabilities=None)
    NeedlemanWunschScores(byte_to_class, class_substitution_costs, open=-1, extend=-1, capabilities=None)
    SmithWatermanScores(byte_to_class, class_substitution_costs, open=-1, extend=-1, capabilities=None)
    engine(queries, candidates=None, device=None, out=None) -> (len(queries), len(candidates)) matrix

Levenshtein results are ``uint64``, alignment scores ``int64``; ``candidates=None`` gives the symmetric
self-similarity matrix. Every call runs on the GPU through ``libszs_gb300.so``; there is no CPU fallback, so a
``DeviceScope(cpu_cores=...)`` is rejected with ``RuntimeError`` exactly as the reference rejects a CPU scope for a
CUDA engine. Extension (not in the reference): ``engine.pairwise(first, second)`` scores ``(first[i], second[i])``.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native
from ._native import lib

__all__ = [
    "Strs", "DeviceScope", "LevenshteinDistances", "LevenshteinDistancesUTF8", "NeedlemanWunschScores",
    "SmithWatermanScores", "Fingerprints", "to_device",
    "Server", "Ticket", "__version__", "__capabilities__",
]

__version__ = f"{lib.szs_version_major()}.{lib.szs_version_minor()}.{lib.szs_version_patch()}"


def _capability_names(mask: int) -> tuple:
    names = []
    for bit, name in ((_native.CAP_SERIAL, "serial"), (_native.CAP_PARALLEL, "parallel"),
                      (_native.CAP_CUDA, "cuda"), (_native.CAP_KEPLER, "kepler"), (_native.CAP_HOPPER, "hopper")):
        if mask & bit:
            names.append(name)
    return tuple(names)


__capabilities__ = _capability_names(lib.szs_capabilities())
__capabilities_str__ = ", ".join(__capabilities__)


class _DeviceBuffer:
    """Managed memory from ``szs_unified_alloc``, freed with the owning object."""

    def __init__(self, size: int):
        self.size = max(int(size), 1)
        self.ptr = lib.szs_unified_alloc(self.size)
        if not self.ptr:
            raise MemoryError("szs_unified_alloc failed")

    def view(self, dtype, count):
        buffer = (ctypes.c_ubyte * self.size).from_address(self.ptr)
        return np.frombuffer(buffer, dtype=dtype, count=count)

    def __del__(self):
        if getattr(self, "ptr", None):
            lib.szs_unified_free(self.ptr, self.size)
            self.ptr = None


def _pointer_of(array) -> int:
    """Address of a numpy array or of a tensor-like object (``data_ptr()``)."""
    if isinstance(array, np.ndarray):
        return array.ctypes.data
    if hasattr(array, "data_ptr"):
        return int(array.data_ptr())
    if hasattr(array, "__cuda_array_interface__"):
        return int(array.__cuda_array_interface__["data"][0])
    raise TypeError(f"unsupported buffer type {type(array).__name__}")


class Strs:
    """An Arrow-like tape of byte strings: contiguous ``data`` plus ``count + 1`` offsets.

    Stands in for the reference's ``stringzilla.Strs`` input container. Accepts a list of ``str``/``bytes``, a
    pyarrow string/binary array, or ``Strs.from_buffers(data, offsets)`` over numpy arrays or device tensors
    (``uint32``/``int32`` or ``uint64``/``int64`` offsets). Slices are views that keep the parent's offsets, so the
    first offset of a slice is generally not zero.
    """

    def __init__(self, items=None):
        self._as_bytes = False
        if items is None:
            items = []
        if hasattr(items, "buffers") and hasattr(items, "type"):  # pyarrow array
            self._from_arrow(items)
            return
        encoded = []
        for item in items:
            if isinstance(item, (bytes, bytearray, memoryview)):
                self._as_bytes = True
                encoded.append(bytes(item))
            elif isinstance(item, str):
                encoded.append(item.encode("utf-8"))
            else:
                raise TypeError(f"Strs items must be str or bytes, got {type(item).__name__}")
        lengths = np.fromiter((len(e) for e in encoded), dtype=np.uint64, count=len(encoded))
        offsets = np.zeros(len(encoded) + 1, dtype=np.uint64)
        np.cumsum(lengths, out=offsets[1:])
        data = np.frombuffer(b"".join(encoded), dtype=np.uint8) if encoded else np.zeros(0, dtype=np.uint8)
        self._set(data, offsets, 0, len(encoded))

    def _from_arrow(self, array):
        import pyarrow as pa
        if pa.types.is_large_string(array.type) or pa.types.is_large_binary(array.type):
            offset_dtype = np.int64
        elif pa.types.is_string(array.type) or pa.types.is_binary(array.type):
            offset_dtype = np.int32
        else:
            raise TypeError(f"unsupported pyarrow type {array.type}")
        if array.null_count:
            raise ValueError("null strings are not supported")
        self._as_bytes = pa.types.is_binary(array.type) or pa.types.is_large_binary(array.type)
        # Zero copy: both views alias Arrow's own buffers, and 32-bit offsets reach the `_u32tape` entry points as
        # they are (python/stringzillas/stringzillas.h:158-174 exports Arrow tapes the same way). A sliced array keeps
        # its parent's offsets, so the first offset is generally not zero.
        _, offsets_buffer, data_buffer = array.buffers()
        offsets = np.frombuffer(offsets_buffer, dtype=offset_dtype)[array.offset:array.offset + len(array) + 1]
        data = (np.frombuffer(data_buffer, dtype=np.uint8) if data_buffer is not None
                else np.zeros(0, dtype=np.uint8))
        self._set(data, offsets, 0, len(array))
        self._keep = array

    @classmethod
    def from_buffers(cls, data, offsets):
        """Wraps existing buffers without copying. ``offsets`` has ``count + 1`` entries."""
        self = cls.__new__(cls)
        self._as_bytes = True
        count = (offsets.shape[0] if hasattr(offsets, "shape") else len(offsets)) - 1
        self._set(data, offsets, 0, count)
        return self

    def _set(self, data, offsets, start, count):
        self._data, self._offsets, self._start, self._count = data, offsets, start, count

    def __len__(self):
        return self._count

    def _host_offsets(self):
        offsets = self._offsets
        if not isinstance(offsets, np.ndarray):
            offsets = offsets.cpu().numpy() if hasattr(offsets, "cpu") else np.asarray(offsets)
        return offsets

    def __getitem__(self, index):
        if isinstance(index, slice):
            start, stop, step = index.indices(self._count)
            if step != 1:
                raise ValueError("only contiguous slices are supported")
            view = Strs.__new__(Strs)
            view._as_bytes = self._as_bytes
            view._set(self._data, self._offsets, self._start + start, max(stop - start, 0))
            view._keep = self
            return view
        if index < 0:
            index += self._count
        if not 0 <= index < self._count:
            raise IndexError("Strs index out of range")
        offsets = self._host_offsets()
        data = self._data if isinstance(self._data, np.ndarray) else self._data.cpu().numpy()
        begin, end = int(offsets[self._start + index]), int(offsets[self._start + index + 1])
        raw = bytes(data[begin:end])
        return raw if self._as_bytes else raw.decode("utf-8")

    def __iter__(self):
        for i in range(self._count):
            yield self[i]

    def tape(self):
        """(tape struct, keep-alive) for the C-ABI. Chooses u32 or u64 offsets by the offsets' element size."""
        offsets = self._offsets
        itemsize = offsets.itemsize if isinstance(offsets, np.ndarray) else offsets.element_size()
        tape_type = _native.U32Tape if itemsize == 4 else _native.U64Tape
        data_ptr = _pointer_of(self._data) if (self._data.shape[0] if hasattr(self._data, "shape") else 1) else 0
        tape = tape_type(data_ptr or None, _pointer_of(offsets) + self._start * itemsize, self._count)
        return tape, itemsize * 8


def to_device(strs: Strs) -> Strs:
    """Moves a ``Strs`` tape into managed memory reachable by the GPU; returns the same object (as the reference's
    ``stringzillas.to_device`` does, python/stringzillas/stringzillas.c:171-233)."""
    if not isinstance(strs, Strs):
        raise TypeError("to_device expects a Strs object")
    offsets = strs._host_offsets()
    data = strs._data if isinstance(strs._data, np.ndarray) else strs._data.cpu().numpy()
    data_buffer = _DeviceBuffer(data.nbytes)
    offsets_buffer = _DeviceBuffer(offsets.nbytes)
    device_data = data_buffer.view(np.uint8, data.shape[0])
    device_offsets = offsets_buffer.view(offsets.dtype, offsets.shape[0])
    device_data[:] = data
    device_offsets[:] = offsets
    strs._data, strs._offsets = device_data, device_offsets
    strs._device_buffers = (data_buffer, offsets_buffer)
    return strs


class DeviceScope:
    """``DeviceScope(cpu_cores=None, gpu_device=None)`` (python/stringzillas/device_scope.c:17-61)."""

    def __init__(self, cpu_cores=None, gpu_device=None, stream=None):
        self.handle = ctypes.c_void_p()
        err = ctypes.c_char_p()
        if stream is not None:
            # Extension: run on a caller-owned CUDA stream (an int handle, or an object with `.cuda_stream`).
            handle = int(getattr(stream, "cuda_stream", stream))
            status = lib.szs_gb300_device_scope_init_stream(gpu_device or 0, ctypes.c_void_p(handle),
                                                            ctypes.byref(self.handle), ctypes.byref(err))
            self.description = f"GPU:{gpu_device or 0}:stream"
            self._stream = stream
            _native.raise_for(status, err.value, "DeviceScope initialization")
            return
        if cpu_cores is not None and gpu_device is not None:
            raise ValueError("Cannot specify both cpu_cores and gpu_device")
        if cpu_cores is not None:
            if not isinstance(cpu_cores, int) or isinstance(cpu_cores, bool):
                raise TypeError("cpu_cores must be an integer")
            status = lib.szs_device_scope_init_cpu_cores(cpu_cores, ctypes.byref(self.handle), ctypes.byref(err))
            self.description = "default" if cpu_cores == 1 else ("CPUs:all" if cpu_cores == 0 else f"CPUs:{cpu_cores}")
        elif gpu_device is not None:
            if not isinstance(gpu_device, int) or isinstance(gpu_device, bool):
                raise TypeError("gpu_device must be an integer")
            status = lib.szs_device_scope_init_gpu_device(gpu_device, ctypes.byref(self.handle), ctypes.byref(err))
            self.description = f"GPU:{gpu_device}"
        else:
            status = lib.szs_device_scope_init_default(ctypes.byref(self.handle), ctypes.byref(err))
            self.description = "default"
        _native.raise_for(status, err.value, "DeviceScope initialization")

    def __repr__(self):
        return f"DeviceScope({self.description})"

    def __del__(self):
        if getattr(self, "handle", None) and self.handle.value:
            lib.szs_device_scope_free(self.handle)
            self.handle = ctypes.c_void_p()


_default_scope = None


def _scope_handle(device):
    global _default_scope
    if device is None:
        if _default_scope is None:
            _default_scope = DeviceScope()
        return _default_scope.handle
    if not isinstance(device, DeviceScope):
        raise TypeError("device must be a DeviceScope instance")
    return device.handle


def _as_strs(obj, name):
    if isinstance(obj, Strs):
        return obj
    if isinstance(obj, (list, tuple)) or (hasattr(obj, "buffers") and hasattr(obj, "type")):
        return Strs(obj)
    raise TypeError(f"Expected stringzillas_gb300.Strs objects, got {type(obj).__name__} for {name}. "
                    "Convert using: Strs(your_string_list)")


class _Engine:
    _algo = ""
    _dtype = np.int64
    _name = ""

    def __init__(self):
        self.handle = ctypes.c_void_p()

    def _check_capabilities(self, capabilities):
        if capabilities is None or isinstance(capabilities, DeviceScope):
            return
        if not isinstance(capabilities, (tuple, list)) or not all(isinstance(c, str) for c in capabilities):
            raise TypeError("capabilities must be a tuple of strings or a DeviceScope")

    def __del__(self):
        if getattr(self, "handle", None) and self.handle.value:
            getattr(lib, f"szs_{self._algo}_free")(self.handle)
            self.handle = ctypes.c_void_p()

    def _output(self, rows, cols, out):
        if out is None:
            return np.empty((rows, cols), dtype=self._dtype), None
        if isinstance(out, np.ndarray):
            if out.ndim != 2:
                raise ValueError("out array must be 2-dimensional")
            if out.shape[0] < rows or out.shape[1] < cols:
                raise ValueError("out array is too small for results")
            if out.dtype != self._dtype:
                raise TypeError(f"out array must have {np.dtype(self._dtype).name} dtype")
            if out.strides[1] != 8:
                raise ValueError("out array rows must be contiguous (unit stride along columns)")
            return out, out.strides[0] // 8
        # A device tensor (e.g. torch.cuda) with row-major layout.
        if out.dim() != 2 or out.stride(1) != 1 or out.element_size() != 8:
            raise ValueError("out tensor must be 2-D, 8-byte elements, unit column stride")
        return out, out.stride(0)

    def __call__(self, queries, candidates=None, device=None, out=None):
        queries = _as_strs(queries, "queries")
        candidates = None if candidates is None else _as_strs(candidates, "candidates")
        rows = len(queries)
        cols = rows if candidates is None else len(candidates)
        result, stride = self._output(rows, cols, out)
        if stride is None:
            stride = cols
        if rows == 0 or cols == 0:
            return result
        q_tape, q_bits = queries.tape()
        c_tape, c_bits = (None, q_bits) if candidates is None else candidates.tape()
        if c_tape is not None and c_bits != q_bits:
            # Mixed offset widths: widen the narrower one.
            queries = Strs.from_buffers(queries._data, queries._host_offsets().astype(np.uint64))
            candidates = Strs.from_buffers(candidates._data, candidates._host_offsets().astype(np.uint64))
            q_tape, q_bits = queries.tape()
            c_tape, c_bits = candidates.tape()
        suffix = "_u32tape" if q_bits == 32 else "_u64tape"
        err = ctypes.c_char_p()
        fn = getattr(lib, f"szs_{self._algo}{suffix}")
        status = fn(self.handle, _scope_handle(device), ctypes.byref(q_tape),
                    None if c_tape is None else ctypes.byref(c_tape), ctypes.c_void_p(_pointer_of(result)),
                    stride, ctypes.byref(err))
        _native.raise_for(status, err.value, f"{self._name} computation")
        return result

    def pairwise(self, first, second, device=None, out=None):
        """Extension: ``out[i] = score(first[i], second[i])`` (no counterpart in the reference)."""
        first, second = _as_strs(first, "first"), _as_strs(second, "second")
        if len(first) != len(second):
            raise ValueError("pairwise inputs must have the same length")
        result = np.empty(len(first), dtype=self._dtype) if out is None else out
        if len(first) == 0:
            return result
        a_tape, a_bits = first.tape()
        b_tape, b_bits = second.tape()
        if a_bits != b_bits:
            first = Strs.from_buffers(first._data, first._host_offsets().astype(np.uint64))
            second = Strs.from_buffers(second._data, second._host_offsets().astype(np.uint64))
            a_tape, a_bits = first.tape()
            b_tape, b_bits = second.tape()
        suffix = "_pairwise_u32tape" if a_bits == 32 else "_pairwise_u64tape"
        err = ctypes.c_char_p()
        status = getattr(lib, f"szs_{self._algo}{suffix}")(
            self.handle, _scope_handle(device), ctypes.byref(a_tape), ctypes.byref(b_tape),
            ctypes.c_void_p(_pointer_of(result)), ctypes.byref(err))
        _native.raise_for(status, err.value, f"{self._name} computation")
        return result

    def set_schedule(self, schedule: str):
        """Extension: ``"batched"`` (default) or ``"plain"`` (one launch, one kernel shape, input order)."""
        code = {"batched": 0, "plain": 1}[schedule]
        err = ctypes.c_char_p()
        _native.raise_for(lib.szs_gb300_engine_set_schedule(self.handle, code, ctypes.byref(err)), err.value,
                          "set_schedule")

    def set_tuning(self, tuning=None):
        """Extension: per-length-bin choices (see ``szs_gb300_tuning_t``): a dict with any of ``packed_rows`` (16
        values), ``cell_bits`` (16 values), ``band_min_rows``, ``packed_warps`` (4 values),
        ``band_min_rows_packed``, ``pipeline_chunk_kb``, ``packed_step_cost`` (4 values), ``band_min_rows_few``,
        ``band_min_rows_compare``, ``band_wait_polls`` (the band kernels' wait bound, clamped to the built-in
        one) and ``short_max_rows`` (shorter sides up to this take the short-pair kernel; at most 128); None restores
        the built-in choices."""
        err = ctypes.c_char_p()
        if tuning is None:
            status = lib.szs_gb300_engine_set_tuning(self.handle, None, ctypes.byref(err))
        else:
            unknown = set(tuning) - {"packed_rows", "cell_bits", "band_min_rows", "packed_warps", "band_min_rows_packed",
                                     "pipeline_chunk_kb", "packed_step_cost", "band_min_rows_few",
                                     "band_min_rows_compare", "band_wait_polls", "short_max_rows"}
            if unknown:
                raise ValueError(f"unknown tuning fields {sorted(unknown)}")
            t = _native.Tuning()
            for name, size in (("packed_rows", 16), ("cell_bits", 16), ("packed_warps", 4), ("packed_step_cost", 4)):
                values = list(tuning.get(name, [0] * size))
                if len(values) != size:
                    raise ValueError(f"{name} needs {size} values")
                getattr(t, name)[:] = [int(v) for v in values]
            t.band_min_rows = int(tuning.get("band_min_rows", 0))
            t.band_min_rows_packed = int(tuning.get("band_min_rows_packed", 0))
            t.pipeline_chunk_kb = int(tuning.get("pipeline_chunk_kb", 0))
            t.band_min_rows_few = int(tuning.get("band_min_rows_few", 0))
            t.band_min_rows_compare = int(tuning.get("band_min_rows_compare", 0))
            t.band_wait_polls = int(tuning.get("band_wait_polls", 0))
            t.short_max_rows = int(tuning.get("short_max_rows", 0))
            status = lib.szs_gb300_engine_set_tuning(self.handle, ctypes.byref(t), ctypes.byref(err))
        _native.raise_for(status, err.value, "set_tuning")

    def get_tuning(self) -> dict:
        """Extension: the engine's current tuning (zeros mean built-in choices)."""
        t = _native.Tuning()
        err = ctypes.c_char_p()
        _native.raise_for(lib.szs_gb300_engine_get_tuning(self.handle, ctypes.byref(t), ctypes.byref(err)), err.value,
                          "get_tuning")
        return {"packed_rows": list(t.packed_rows), "cell_bits": list(t.cell_bits),
                "band_min_rows": t.band_min_rows, "packed_warps": list(t.packed_warps),
                "band_min_rows_packed": t.band_min_rows_packed, "pipeline_chunk_kb": t.pipeline_chunk_kb,
                "packed_step_cost": list(t.packed_step_cost), "band_min_rows_few": t.band_min_rows_few,
                "band_min_rows_compare": t.band_min_rows_compare, "band_wait_polls": t.band_wait_polls,
                "short_max_rows": t.short_max_rows}

    def stats(self) -> dict:
        """Extension: counters of the last call (device time, cells, pairs, launches)."""
        stats = _native.Stats()
        err = ctypes.c_char_p()
        _native.raise_for(lib.szs_gb300_engine_get_stats(self.handle, ctypes.byref(stats), ctypes.byref(err)),
                          err.value, "stats")
        return {name: getattr(stats, name) for name, _ in stats._fields_}

    @property
    def __capabilities__(self):
        return __capabilities__


def _int8(name, value):
    value = int(value)
    if value < -128 or value > 127:
        raise ValueError(f"{name} cost must fit in 8-bit signed integer")
    return value


class LevenshteinDistances(_Engine):
    """Byte-level edit distances; a gap of length k costs ``open + (k-1)*extend``; ``open == extend`` is linear."""

    _algo = "levenshtein_distances"
    _dtype = np.uint64
    _name = "Levenshtein distances"

    def __init__(self, match=0, mismatch=1, open=1, extend=1, capabilities=None):
        super().__init__()
        self._check_capabilities(capabilities)
        match, mismatch = _int8("match", match), _int8("mismatch", mismatch)
        open, extend = _int8("open", open), _int8("extend", extend)
        err = ctypes.c_char_p()
        status = lib.szs_levenshtein_distances_init(match, mismatch, open, extend, None, 0x7FFFFFFF,
                                                    ctypes.byref(self.handle), ctypes.byref(err))
        _native.raise_for(status, err.value, "Levenshtein distances initialization")
        self.description = f"{match},{mismatch},{open},{extend}"

    def __repr__(self):
        return f"LevenshteinDistances(match,mismatch,open,extend={self.description})"


class LevenshteinDistancesUTF8(LevenshteinDistances):
    """Edit distances over UTF-8 code points (``LevenshteinDistancesUTF8`` of the reference). Each call numbers the
    distinct code points of its batch on the device (one-byte codes up to 256 of them, 16-bit codes up to 65,536)."""

    _algo = "levenshtein_distances_utf8"
    _name = "UTF-8 Levenshtein distances"

    def __init__(self, match=0, mismatch=1, open=1, extend=1, capabilities=None):
        _Engine.__init__(self)
        self._check_capabilities(capabilities)
        match, mismatch = _int8("match", match), _int8("mismatch", mismatch)
        open, extend = _int8("open", open), _int8("extend", extend)
        err = ctypes.c_char_p()
        status = lib.szs_levenshtein_distances_utf8_init(match, mismatch, open, extend, None, 0x7FFFFFFF,
                                                         ctypes.byref(self.handle), ctypes.byref(err))
        _native.raise_for(status, err.value, "UTF-8 Levenshtein distances initialization")
        self.description = f"{match},{mismatch},{open},{extend}"

    def pairwise(self, first, second, device=None, out=None):
        """Extension: ``out[i] = distance(first[i], second[i])`` over code points."""
        algo = self._algo
        try:
            self._algo = "levenshtein_distances"  # the pairwise entry points serve every Levenshtein engine
            return super().pairwise(first, second, device=device, out=out)
        finally:
            self._algo = algo

    def __repr__(self):
        return f"LevenshteinDistancesUTF8(match,mismatch,open,extend={self.description})"


class _Alignment(_Engine):
    def __init__(self, byte_to_class=None, class_substitution_costs=None, open=-1, extend=-1, capabilities=None):
        super().__init__()
        if byte_to_class is None or class_substitution_costs is None:
            raise TypeError(f"{type(self).__name__} requires 'byte_to_class' and 'class_substitution_costs'")
        if not isinstance(byte_to_class, np.ndarray):
            raise TypeError("byte_to_class must be a NumPy array")
        if byte_to_class.ndim != 1 or byte_to_class.shape[0] != 256:
            raise ValueError("byte_to_class must be a 256-element array")
        if byte_to_class.dtype != np.uint8:
            raise TypeError("byte_to_class must have uint8 dtype")
        if not byte_to_class.flags.c_contiguous:
            raise ValueError("byte_to_class must be a C-contiguous array. Use np.ascontiguousarray() to convert.")
        if not isinstance(class_substitution_costs, np.ndarray):
            raise TypeError("class_substitution_costs must be a NumPy array")
        if class_substitution_costs.shape != (32, 32):
            raise ValueError("class_substitution_costs must be a 32x32 array")
        if class_substitution_costs.dtype != np.int8:
            raise TypeError("class_substitution_costs must have int8 dtype")
        if not class_substitution_costs.flags.c_contiguous:
            raise ValueError("class_substitution_costs must be a C-contiguous array. "
                             "Use np.ascontiguousarray() to convert.")
        self._check_capabilities(capabilities)
        open, extend = _int8("open", open), _int8("extend", extend)
        err = ctypes.c_char_p()
        status = getattr(lib, f"szs_{self._algo}_init")(
            byte_to_class.ctypes.data, class_substitution_costs.ctypes.data, open, extend, None, 0x7FFFFFFF,
            ctypes.byref(self.handle), ctypes.byref(err))
        _native.raise_for(status, err.value, f"{self._name} initialization")
        self.description = f"open={open},extend={extend}"

    @classmethod
    def dense(cls, substitution_matrix, open=-1, extend=-1, capabilities=None):
        """Extension: an engine over a dense 256 x 256 int8 table, ``substitution_matrix[a, b]`` = cost of aligning
        byte a of the first string with byte b of the second (no counterpart in the reference, which folds bytes
        into 32 classes). Calls over more than 32 distinct byte values score on the 32-bit routes."""
        if not isinstance(substitution_matrix, np.ndarray):
            raise TypeError("substitution_matrix must be a NumPy array")
        if substitution_matrix.shape != (256, 256):
            raise ValueError("substitution_matrix must be a 256x256 array")
        if substitution_matrix.dtype != np.int8:
            raise TypeError("substitution_matrix must have int8 dtype")
        table = np.ascontiguousarray(substitution_matrix)
        self = cls.__new__(cls)
        _Engine.__init__(self)
        self._check_capabilities(capabilities)
        open, extend = _int8("open", open), _int8("extend", extend)
        err = ctypes.c_char_p()
        status = getattr(lib, f"szs_gb300_{self._algo}_init_dense")(
            table.ctypes.data, open, extend, None, 0x7FFFFFFF, ctypes.byref(self.handle), ctypes.byref(err))
        _native.raise_for(status, err.value, f"{self._name} initialization")
        self.description = f"open={open},extend={extend}"
        return self


class NeedlemanWunschScores(_Alignment):
    """Global alignment scores (maximised); pass negative gap costs."""

    _algo = "needleman_wunsch_scores"
    _name = "Needleman-Wunsch scores"


class SmithWatermanScores(_Alignment):
    """Local alignment scores (maximised, never below 0); pass negative gap costs."""

    _algo = "smith_waterman_scores"
    _name = "Smith-Waterman scores"


class Fingerprints:
    """Min-Hash fingerprints: for every text and dimension, the low 32 bits of the minimum rolling hash over the
    text's windows of that dimension's width, and how many windows reach it (the reference's
    python/stringzillas/fingerprints.c:35-211). Texts shorter than a window give 0xFFFFFFFF and 0."""

    def __init__(self, ndim, window_widths=None, alphabet_size=256, seed=0, capabilities=None):
        _Engine._check_capabilities(None, capabilities)
        ndim = int(ndim)
        widths = None
        if window_widths is not None:
            if not isinstance(window_widths, np.ndarray):
                raise TypeError("window_widths must be a numpy array of uint64")
            if window_widths.dtype != np.uint64:
                raise TypeError("window_widths must have dtype uint64")
            if window_widths.ndim != 1:
                raise ValueError("window_widths must be a 1D array")
            if not window_widths.flags.c_contiguous:
                raise ValueError("window_widths must be a contiguous C-style array (no strides)")
            widths = window_widths
        self.handle = ctypes.c_void_p()
        err = ctypes.c_char_p()
        count = 0 if widths is None else len(widths)
        status = lib.szs_fingerprints_init(ndim, int(alphabet_size),
                                           None if widths is None else ctypes.c_void_p(widths.ctypes.data), count,
                                           ctypes.c_uint64(int(seed)), None, 0, ctypes.byref(self.handle),
                                           ctypes.byref(err))
        _native.raise_for(status, err.value, "Fingerprints initialization")
        self.ndim = ndim
        self._description = f"ndim={ndim},window_widths={count},alphabet_size={int(alphabet_size)},seed={int(seed)}"

    def __del__(self):
        if getattr(self, "handle", None) and self.handle.value:
            lib.szs_fingerprints_free(self.handle)
            self.handle = ctypes.c_void_p()

    def __repr__(self):
        return f"Fingerprints({self._description})"

    @property
    def __capabilities__(self):
        return __capabilities__

    def _outputs(self, rows, out):
        if out is None:
            return [np.empty((rows, self.ndim), dtype=np.uint32) for _ in range(2)]
        if not isinstance(out, (tuple, list)) or len(out) != 2:
            raise TypeError("out must be a (hashes, counts) pair")
        for array in out:
            if isinstance(array, np.ndarray):
                if array.ndim != 2 or array.dtype != np.uint32 or array.strides[1] != 4:
                    raise ValueError("out arrays must be 2-D uint32 with contiguous rows")
                shape = array.shape
            else:
                if array.dim() != 2 or array.element_size() != 4 or array.stride(1) != 1:
                    raise ValueError("out tensors must be 2-D, 4-byte elements, unit column stride")
                shape = tuple(array.shape)
            if shape[0] < rows or shape[1] < self.ndim:
                raise ValueError("out arrays are too small for results")
        return list(out)

    @staticmethod
    def _row_bytes(array):
        return array.strides[0] if isinstance(array, np.ndarray) else array.stride(0) * 4

    def __call__(self, texts, device=None, out=None):
        texts = _as_strs(texts, "texts")
        rows = len(texts)
        hashes, counts = self._outputs(rows, out)
        if rows == 0:
            return hashes, counts
        tape, bits = texts.tape()
        err = ctypes.c_char_p()
        fn = lib.szs_fingerprints_u32tape if bits == 32 else lib.szs_fingerprints_u64tape
        status = fn(self.handle, _scope_handle(device), ctypes.byref(tape), ctypes.c_void_p(_pointer_of(hashes)),
                    self._row_bytes(hashes), ctypes.c_void_p(_pointer_of(counts)), self._row_bytes(counts),
                    ctypes.byref(err))
        _native.raise_for(status, err.value, "Fingerprints computation")
        return hashes, counts

from .serving import Server, Ticket  # noqa: E402  (needs the engine classes above)
