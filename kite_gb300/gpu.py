"""ctypes binding of libkite_gpu.so (include/kite_gpu.h).

This is the Python face of the drop-in boundary: `Counter` mirrors the
reference's count worker seam (process_chunk / flush_all emitting
append_chunk records, src/count/worker.rs:196-449) and `merge` mirrors
build_merge_partition_chunk over all partitions (src/merge/mod.rs:198-214).
There is no CPU fallback: loading fails loudly if the CUDA library is
missing, and opening a context fails without a GPU.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

_LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libkite_gpu.so"
_lib = None

KITE_OK = 0
ERRORS = {
    -1: "KITE_ERR_CUDA", -2: "KITE_ERR_OOM", -3: "KITE_ERR_TIMEOUT", -4: "KITE_ERR_BAD_INPUT",
    -5: "KITE_ERR_COUNT_OVERFLOW", -6: "KITE_ERR_UNSUPPORTED", -7: "KITE_ERR_DEVICE", -8: "KITE_ERR_CALLBACK",
    -9: "KITE_ERR_STATE",
}
SPLIT_AUTO, SPLIT_SAMPLED, SPLIT_LEARNED = 0, 1, 2
ABI_VERSION = 2  # KITE_GPU_ABI_VERSION: the layouts of the structures below

EXPORTED = [
    "kite_gpu_abi_version", "kite_gpu_device_count", "kite_gpu_open", "kite_gpu_close", "kite_gpu_last_error",
    "kite_gpu_alloc_pinned", "kite_gpu_free_pinned", "kite_gpu_count_submit", "kite_gpu_wait_ticket",
    "kite_gpu_count_submit_device", "kite_gpu_count_finish", "kite_gpu_result_partition", "kite_gpu_merge",
    "kite_gpu_get_stats", "kite_gpu_synchronize", "kite_gpu_count_submit_sample",
    "kite_gpu_count_submit_device_sample", "kite_gpu_sample_totals", "kite_gpu_dump", "kite_gpu_histo",
    "kite_gpu_query",
]


class KiteGpuError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class Cfg(C.Structure):
    _fields_ = [("device", C.c_int), ("k", C.c_int), ("canonical", C.c_int), ("partitions", C.c_uint32),
                ("splitter_mode", C.c_int), ("imbalance_bound", C.c_double), ("arena_bytes", C.c_uint64),
                ("timeout_ms", C.c_uint32), ("stream", C.c_void_p), ("samples", C.c_uint32),
                ("tile_fill", C.c_double), ("scatter_shape", C.c_int), ("tile_wait_polls", C.c_uint32)]


class ChunkMeta(C.Structure):
    _fields_ = [("partition_id", C.c_uint32), ("codec", C.c_uint32), ("row_count", C.c_uint64),
                ("raw_bytes", C.c_uint64), ("key_min_lo", C.c_uint64 * 2), ("key_min_hi", C.c_uint64 * 2),
                ("key_max_lo", C.c_uint64 * 2), ("key_max_hi", C.c_uint64 * 2)]

    def as_dict(self) -> dict:
        lo = lambda a: int(a[0]) | (int(a[1]) << 64)  # noqa: E731
        return {"partition_id": self.partition_id, "codec": self.codec, "row_count": self.row_count,
                "raw_bytes": self.raw_bytes, "key_min": lo(self.key_min_lo), "key_max": lo(self.key_max_lo)}


class Stats(C.Structure):
    _fields_ = [("reads", C.c_uint64), ("bases", C.c_uint64), ("kmers", C.c_uint64), ("rows", C.c_uint64),
                ("payload_bytes", C.c_uint64), ("tiles", C.c_uint32), ("big_tiles", C.c_uint32),
                ("tiles_per_bucket", C.c_uint32), ("segments", C.c_uint32), ("tile_imbalance", C.c_double),
                ("splitter_used", C.c_int), ("stage_ms", C.c_double * 12), ("h2d_bytes", C.c_uint64),
                ("d2h_bytes", C.c_uint64), ("kernel_launches", C.c_uint64), ("mlp_loss", C.c_double),
                ("mlp_pred_imbalance", C.c_double), ("hist_pred_imbalance", C.c_double),
                ("range_imbalance", C.c_double), ("sort_fallbacks", C.c_uint64),
                ("split_levels", C.c_uint32), ("staged_scatter", C.c_uint32),
                ("mlp_reused", C.c_uint32), ("big_tile_keys", C.c_uint64), ("big_tile_rows", C.c_uint64),
                ("input_pieces", C.c_uint32)]

    def as_dict(self) -> dict:
        d = {f: getattr(self, f) for f, _ in self._fields_ if f != "stage_ms"}
        d["stage_ms"] = list(self.stage_ms)
        return d


class MergeInput(C.Structure):
    _fields_ = [("base", C.c_void_p), ("base_len", C.c_uint64), ("chunk_offset", C.POINTER(C.c_uint64)),
                ("chunk_len", C.POINTER(C.c_uint64)), ("chunk_rows", C.POINTER(C.c_uint64)),
                ("chunk_codec", C.POINTER(C.c_uint32)), ("part_first", C.POINTER(C.c_uint64)),
                ("part_count", C.POINTER(C.c_uint64)), ("has_min", C.c_int), ("has_max", C.c_int),
                ("min_count", C.c_uint32), ("max_count", C.c_uint32)]


EMIT = C.CFUNCTYPE(C.c_int, C.c_void_p, C.POINTER(ChunkMeta), C.POINTER(C.c_uint8), C.c_size_t)
HISTO = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_uint64, C.c_uint64)


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not _LIB_PATH.exists():
            raise RuntimeError(f"{_LIB_PATH} is missing: build the CUDA extension first (kite_gb300.build)")
        L = C.CDLL(str(_LIB_PATH))
        if L.kite_gpu_abi_version() != ABI_VERSION:
            raise RuntimeError(f"{_LIB_PATH} has C ABI {L.kite_gpu_abi_version()}, this binding {ABI_VERSION}: rebuild")
        L.kite_gpu_open.argtypes = [C.POINTER(Cfg), C.POINTER(C.c_void_p)]
        L.kite_gpu_close.argtypes = [C.c_void_p]
        L.kite_gpu_last_error.argtypes = [C.c_void_p]
        L.kite_gpu_last_error.restype = C.c_char_p
        L.kite_gpu_alloc_pinned.argtypes = [C.c_size_t]
        L.kite_gpu_alloc_pinned.restype = C.c_void_p
        L.kite_gpu_free_pinned.argtypes = [C.c_void_p]
        L.kite_gpu_count_submit.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t]
        L.kite_gpu_count_submit.restype = C.c_int64
        L.kite_gpu_wait_ticket.argtypes = [C.c_void_p, C.c_int64]
        L.kite_gpu_count_submit_device.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t]
        L.kite_gpu_count_finish.argtypes = [C.c_void_p, EMIT, C.c_void_p]
        L.kite_gpu_count_submit_sample.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_size_t]
        L.kite_gpu_count_submit_sample.restype = C.c_int64
        L.kite_gpu_count_submit_device_sample.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_size_t]
        L.kite_gpu_sample_totals.argtypes = [C.c_void_p, C.c_uint32, C.POINTER(C.c_uint64)]
        L.kite_gpu_result_partition.argtypes = [C.c_void_p, C.c_uint32, C.POINTER(ChunkMeta),
                                                C.POINTER(C.c_void_p), C.POINTER(C.c_size_t)]
        L.kite_gpu_merge.argtypes = [C.c_void_p, C.POINTER(MergeInput), C.c_int, EMIT, C.c_void_p]
        L.kite_gpu_dump.argtypes = [C.c_void_p, C.POINTER(MergeInput), EMIT, C.c_void_p]
        L.kite_gpu_histo.argtypes = [C.c_void_p, C.POINTER(MergeInput), HISTO, C.c_void_p]
        L.kite_gpu_query.argtypes = [C.c_void_p, C.POINTER(MergeInput), C.POINTER(C.c_uint64), C.c_size_t,
                                     C.POINTER(C.c_uint64)]
        L.kite_gpu_get_stats.argtypes = [C.c_void_p, C.POINTER(Stats)]
        L.kite_gpu_synchronize.argtypes = [C.c_void_p]
        _lib = L
    return _lib


def device_count() -> int:
    return lib().kite_gpu_device_count()


class Counter:
    """One GPU counting context (k, canonical, partitions fixed at open)."""

    def __init__(self, k: int, canonical: bool, partitions: int, device: int = 0,
                 splitter_mode: int = SPLIT_AUTO, imbalance_bound: float = 1.10, arena_bytes: int = 0,
                 timeout_ms: int = 0, stream: int | None = None, samples: int = 1, tile_fill: float = 0.0,
                 scatter_shape: int = 0, tile_wait_polls: int = 0):
        self._L = lib()
        cfg = Cfg(device, k, 1 if canonical else 0, partitions, splitter_mode, imbalance_bound, arena_bytes,
                  timeout_ms, C.c_void_p(stream) if stream else None, samples, tile_fill, scatter_shape,
                  tile_wait_polls)
        h = C.c_void_p()
        rc = self._L.kite_gpu_open(C.byref(cfg), C.byref(h))
        if rc != KITE_OK:
            raise KiteGpuError(rc, "kite_gpu_open failed")
        self._h = h
        self.k, self.canonical, self.partitions = k, canonical, partitions

    def _check(self, rc: int) -> int:
        if rc < 0:
            raise KiteGpuError(rc, self._L.kite_gpu_last_error(self._h).decode())
        return rc

    def submit(self, data) -> int:
        """Queue FASTQ bytes (bytes, bytearray, numpy uint8 array or (ptr, len))."""
        if isinstance(data, tuple):
            ptr, n = data
        else:
            buf = memoryview(data).cast("B")
            n = buf.nbytes
            ptr = C.addressof(C.c_uint8.from_buffer(buf)) if not buf.readonly else None
            if ptr is None:
                tmp = (C.c_uint8 * n).from_buffer_copy(buf)
                ptr = C.addressof(tmp)
                t = self._check(self._L.kite_gpu_count_submit(self._h, C.c_void_p(ptr), n))
                self._check(self._L.kite_gpu_wait_ticket(self._h, t))
                return t
        return self._check(self._L.kite_gpu_count_submit(self._h, C.c_void_p(ptr), n))

    def wait(self, ticket: int) -> None:
        self._check(self._L.kite_gpu_wait_ticket(self._h, ticket))

    def submit_device(self, ptr: int, n: int, sample: int = 0) -> None:
        self._check(self._L.kite_gpu_count_submit_device_sample(self._h, sample, C.c_void_p(ptr), n))

    def submit_sample(self, sample: int, ptr: int, n: int) -> int:
        """Queue n bytes at host address ptr for `sample` of a batched count."""
        return self._check(self._L.kite_gpu_count_submit_sample(self._h, sample, C.c_void_p(ptr), n))

    def sample_totals(self, sample: int) -> tuple:
        """(reads, bases, k-mers) of `sample` in the last finish."""
        out = (C.c_uint64 * 3)()
        self._check(self._L.kite_gpu_sample_totals(self._h, sample, out))
        return tuple(int(x) for x in out)

    def finish(self, collect: bool = True, callback=None, raw: bool = False, meta: bool = True) -> list:
        """Count the segment; returns [(meta dict, payload bytes)] per non-empty
        partition when collect, else keeps results on the device.  With raw and
        a callback, the callback gets (meta, host address, length) of the
        payload in the library's host buffer (valid during the call) instead of
        a copy; with meta False as well, (partition id, host address, length)."""
        out = []

        def _emit(user, m_ptr, data, n):
            try:
                if raw and callback is not None and not meta:
                    callback(m_ptr.contents.partition_id, C.cast(data, C.c_void_p).value, n)
                    return 0
                m = m_ptr.contents.as_dict()
                if raw and callback is not None:
                    callback(m, C.cast(data, C.c_void_p).value, n)
                    return 0
                payload = C.string_at(data, n)
                if callback is not None:
                    callback(m, payload)
                else:
                    out.append((m, payload))
                return 0
            except Exception:  # pragma: no cover - surfaced as KITE_ERR_CALLBACK
                return 1

        cb = EMIT(_emit) if collect else C.cast(None, EMIT)
        self._check(self._L.kite_gpu_count_finish(self._h, cb, None))
        return out

    def result_partition(self, p: int):
        m = ChunkMeta()
        ptr = C.c_void_p()
        n = C.c_size_t()
        self._check(self._L.kite_gpu_result_partition(self._h, p, C.byref(m), C.byref(ptr), C.byref(n)))
        return m.as_dict(), ptr.value, n.value

    def stats(self) -> dict:
        s = Stats()
        self._check(self._L.kite_gpu_get_stats(self._h, C.byref(s)))
        return s.as_dict()

    def synchronize(self) -> None:
        self._check(self._L.kite_gpu_synchronize(self._h))

    def merge(self, inputs: list, collect: bool = True, callback=None, bases: list | None = None) -> list:
        """inputs: list of kitefile.KiteImage; returns [(meta, payload)].
        With a callback, it gets (meta, host address, length) of each output
        chunk (valid during the call) and nothing is collected.  `bases`:
        optional host addresses holding each image's bytes (no copy)."""
        arr = (MergeInput * len(inputs))()
        keep = []
        for i, img in enumerate(inputs):
            mi, k = img.merge_input(bases[i] if bases else None)
            arr[i] = mi
            keep.append(k)
        out = []

        def _emit(user, meta, data, n):
            try:
                if callback is not None:
                    callback(meta.contents.as_dict(), C.cast(data, C.c_void_p).value, n)
                elif collect:
                    out.append((meta.contents.as_dict(), C.string_at(data, n)))
                return 0
            except Exception:  # pragma: no cover - surfaced as KITE_ERR_CALLBACK
                return 1

        cb = EMIT(_emit)
        self._check(self._L.kite_gpu_merge(self._h, arr, len(inputs), cb, None))
        return out

    def dump(self, image, callback=None, base: int | None = None) -> bytes:
        """`kite dump -o -` of one kitefile.KiteImage on the GPU: the TSV of
        every partition in order.  With a callback, it gets (meta, host
        address, length) of each partition's TSV (valid during the call) and
        nothing is returned.  `base`: optional host address holding the
        image's bytes (no copy)."""
        mi, keep = image.merge_input(base)
        parts = []

        def _emit(user, meta, data, n):
            try:
                if callback is not None:
                    callback(meta.contents.as_dict(), C.cast(data, C.c_void_p).value, n)
                else:
                    parts.append(C.string_at(data, n))
                return 0
            except Exception:  # pragma: no cover - surfaced as KITE_ERR_CALLBACK
                return 1

        cb = EMIT(_emit)
        self._check(self._L.kite_gpu_dump(self._h, C.byref(mi), cb, None))
        del keep
        return b"".join(parts)

    def histo(self, image, base: int | None = None) -> dict:
        """`kite histo` of one kitefile.KiteImage on the GPU: {count: keys}."""
        mi, keep = image.merge_input(base)
        out = {}

        def _emit(user, count, keys):
            out[int(count)] = int(keys)
            return 0

        cb = HISTO(_emit)
        self._check(self._L.kite_gpu_histo(self._h, C.byref(mi), cb, None))
        del keep
        return out

    def query(self, image, keys, base: int | None = None) -> list:
        """u64 counts of encoded keys (ints, or a numpy uint64 array for
        k <= 31; canonical where the database is) in one kitefile.KiteImage,
        0 when absent."""
        import numpy as np
        mi, keep = image.merge_input(base)
        n = len(keys)
        words = np.zeros(2 * max(n, 1), dtype=np.uint64)
        if n and isinstance(keys, np.ndarray) and keys.dtype == np.uint64:
            words[0:2 * n:2] = keys
        else:
            for i, key in enumerate(keys):
                words[2 * i] = key & (2 ** 64 - 1)
                words[2 * i + 1] = key >> 64
        out = np.zeros(max(n, 1), dtype=np.uint64)
        u64p = C.POINTER(C.c_uint64)
        self._check(self._L.kite_gpu_query(self._h, C.byref(mi), words.ctypes.data_as(u64p), n,
                                           out.ctypes.data_as(u64p)))
        del keep
        return out[:n].tolist()

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._L.kite_gpu_close(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
