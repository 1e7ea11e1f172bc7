"""ctypes binding of libkite_host.so (include/kite_host.h): the .kite writer
with the reference's staging/drain layout, the count planner, memory specs
and the CPU dump used to verify outputs."""
from __future__ import annotations

import ctypes as C
from pathlib import Path

from .gpu import ChunkMeta, EMIT

_LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libkite_host.so"
_lib = None

EXPORTED = [
    "kite_parse_memory_spec", "kite_resolve_memory_limit", "kite_count_passes_filter", "kite_host_last_error",
    "kite_derive_plan", "kite_suggest_write_lanes", "kite_writer_open", "kite_writer_append", "kite_writer_emit",
    "kite_writer_worker_drain", "kite_writer_finalize", "kite_writer_image", "kite_writer_close",
    "kite_reader_open", "kite_reader_open_image", "kite_reader_close", "kite_reader_header",
    "kite_reader_merge_input", "kite_dump_partition", "kite_detect_compression", "kite_input_open",
    "kite_input_next", "kite_input_max_chunk", "kite_input_close", "kite_sample_avg_read_len", "kite_synth_reads",
    "kite_input_set_threads", "kite_zstd_available", "kite_zstd_bound", "kite_zstd_chunk",
    "kite_synth_reads_var",
]


class HeaderInfo(C.Structure):
    _fields_ = [("k", C.c_int), ("canonical", C.c_int), ("partitions", C.c_uint32), ("key_width", C.c_uint16),
                ("codec_mask", C.c_uint16), ("has_min", C.c_int), ("has_max", C.c_int), ("min_count", C.c_uint32),
                ("max_count", C.c_uint32)]


class Plan(C.Structure):
    _fields_ = [("partitions", C.c_uint64), ("chunk_size_bytes", C.c_uint64), ("staging_bytes", C.c_uint64),
                ("worker_threads", C.c_uint64), ("local_flush_bytes", C.c_uint64), ("decomp_threads", C.c_uint64),
                ("writer_lanes", C.c_uint64), ("queue_depth", C.c_uint64), ("avg_read_len", C.c_double)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not _LIB_PATH.exists():
            raise RuntimeError(f"{_LIB_PATH} is missing: build first (kite_gb300.build)")
        L = C.CDLL(str(_LIB_PATH))
        L.kite_parse_memory_spec.argtypes = [C.c_char_p]
        L.kite_parse_memory_spec.restype = C.c_int64
        L.kite_host_last_error.restype = C.c_char_p
        L.kite_count_passes_filter.argtypes = [C.c_uint64, C.c_int, C.c_uint32, C.c_int, C.c_uint32]
        L.kite_derive_plan.argtypes = [C.c_uint64, C.c_double, C.c_int, C.c_int, C.c_uint64, C.c_uint64, C.c_uint64,
                                       C.c_int64, C.c_uint64, C.POINTER(Plan)]
        L.kite_suggest_write_lanes.argtypes = [C.c_uint64]
        L.kite_suggest_write_lanes.restype = C.c_uint64
        L.kite_writer_open.argtypes = [C.c_char_p, C.POINTER(HeaderInfo), C.c_uint64, C.c_uint64]
        L.kite_writer_open.restype = C.c_void_p
        L.kite_writer_append.argtypes = [C.c_void_p, C.POINTER(ChunkMeta), C.c_char_p, C.c_size_t]
        L.kite_writer_worker_drain.argtypes = [C.c_void_p]
        L.kite_writer_finalize.argtypes = [C.c_void_p, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
        L.kite_writer_image.argtypes = [C.c_void_p, C.POINTER(C.c_size_t)]
        L.kite_writer_image.restype = C.POINTER(C.c_uint8)
        L.kite_writer_close.argtypes = [C.c_void_p]
        L.kite_reader_open_image.argtypes = [C.c_char_p, C.c_size_t]
        L.kite_reader_open_image.restype = C.c_void_p
        L.kite_reader_open.argtypes = [C.c_char_p]
        L.kite_reader_open.restype = C.c_void_p
        L.kite_reader_close.argtypes = [C.c_void_p]
        L.kite_reader_header.argtypes = [C.c_void_p, C.POINTER(HeaderInfo), C.POINTER(C.c_uint64),
                                         C.POINTER(C.c_uint64)]
        L.kite_dump_partition.argtypes = [C.c_void_p, C.c_uint32, C.POINTER(C.c_void_p), C.POINTER(C.c_size_t),
                                          C.POINTER(C.c_size_t)]
        L.kite_dump_partition.restype = C.c_int64
        L.kite_detect_compression.argtypes = [C.c_char_p]
        L.kite_synth_reads.argtypes = [C.c_void_p, C.c_uint64, C.c_uint64, C.c_uint32, C.c_double, C.c_double,
                                       C.c_double, C.c_uint64, C.c_uint64, C.c_void_p, C.c_uint64, C.c_int]
        L.kite_synth_reads.restype = C.c_int64
        _lib = L
    return _lib


def err() -> str:
    return lib().kite_host_last_error().decode()


def parse_memory_spec(spec: str) -> int:
    v = lib().kite_parse_memory_spec(spec.encode())
    if v < 0:
        raise ValueError(err())
    return v


def count_passes_filter(count: int, min_count=None, max_count=None) -> bool:
    return bool(lib().kite_count_passes_filter(count, min_count is not None, min_count or 0,
                                                max_count is not None, max_count or 0))


def derive_plan(input_bytes: int, avg_read_len: float, compression: int, k: int, partitions: int, threads: int,
                memory: int, buffer_mb: int = -1, chunk_kmers: int = 0) -> dict:
    p = Plan()
    if lib().kite_derive_plan(input_bytes, avg_read_len, compression, k, partitions, threads, memory, buffer_mb,
                              chunk_kmers, C.byref(p)) != 0:
        raise ValueError(err())
    return p.as_dict()


class Writer:
    """In-memory (path None) or file .kite writer with the reference layout."""

    def __init__(self, path, k: int, canonical: bool, partitions: int, key_width: int, codec_mask: int,
                 staging_bytes: int, lanes: int, min_count=None, max_count=None):
        h = HeaderInfo(k, int(canonical), partitions, key_width, codec_mask, min_count is not None,
                       max_count is not None, min_count or 0, max_count or 0)
        self._L = lib()
        self._w = self._L.kite_writer_open(path.encode() if path else None, C.byref(h), staging_bytes, lanes)
        if not self._w:
            raise RuntimeError(err())

    def append(self, meta: dict, payload: bytes) -> None:
        m = ChunkMeta()
        m.partition_id = meta["partition_id"]
        m.codec = meta["codec"]
        m.row_count = meta["row_count"]
        m.raw_bytes = meta["raw_bytes"]
        m.key_min_lo[0] = meta["key_min"] & (2 ** 64 - 1)
        m.key_min_lo[1] = meta["key_min"] >> 64
        m.key_max_lo[0] = meta["key_max"] & (2 ** 64 - 1)
        m.key_max_lo[1] = meta["key_max"] >> 64
        if self._L.kite_writer_append(self._w, C.byref(m), payload, len(payload)) != 0:
            raise RuntimeError(err())

    def worker_drain(self) -> None:
        self._L.kite_writer_worker_drain(self._w)

    def finalize(self) -> tuple:
        tc, tr = C.c_uint64(), C.c_uint64()
        if self._L.kite_writer_finalize(self._w, C.byref(tc), C.byref(tr)) != 0:
            raise RuntimeError(err())
        return tc.value, tr.value

    def image(self) -> bytes:
        n = C.c_size_t()
        p = self._L.kite_writer_image(self._w, C.byref(n))
        if not p or n.value == 0:
            return b""
        # a sized array, not string_at (whose length is a C int: images pass 2 GB)
        return bytes((C.c_uint8 * n.value).from_address(C.addressof(p.contents)))

    def close(self) -> None:
        if self._w:
            self._L.kite_writer_close(self._w)
            self._w = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def read_chunks(path: str, chunk_size: int, threads: int = 0, collect: bool = True) -> list:
    """The FASTQ chunks the host reader produces for a file (plain, gzip or
    BGZF), in order; with collect False, only their lengths (the reader
    still writes every chunk into a buffer, as it fills a pinned one)."""
    L = lib()
    L.kite_input_open.restype = C.c_void_p
    L.kite_input_open.argtypes = [C.c_char_p, C.c_uint64]
    L.kite_input_next.restype = C.c_int64
    L.kite_input_next.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t]
    L.kite_input_max_chunk.restype = C.c_uint64
    L.kite_input_max_chunk.argtypes = [C.c_void_p]
    L.kite_input_set_threads.argtypes = [C.c_void_p, C.c_uint]
    L.kite_input_close.argtypes = [C.c_void_p]
    h = L.kite_input_open(str(path).encode(), chunk_size)
    if not h:
        raise RuntimeError(err())
    try:
        if threads:
            L.kite_input_set_threads(h, threads)
        cap = L.kite_input_max_chunk(h) + 64
        buf = C.create_string_buffer(cap)
        out = []
        while True:
            n = L.kite_input_next(h, buf, cap)
            if n < 0:
                raise RuntimeError(err())
            if n == 0:
                return out
            out.append(C.string_at(buf, n) if collect else n)
    finally:
        L.kite_input_close(h)


def dump_image(image: bytes) -> bytes:
    """kite dump -o - of a .kite image (CPU)."""
    L = lib()
    r = L.kite_reader_open_image(image, len(image))
    if not r:
        raise RuntimeError(err())
    h = HeaderInfo()
    L.kite_reader_header(r, C.byref(h), None, None)
    buf = C.c_void_p()
    cap = C.c_size_t(0)
    ln = C.c_size_t(0)
    try:
        for p in range(h.partitions):
            if L.kite_dump_partition(r, p, C.byref(buf), C.byref(cap), C.byref(ln)) < 0:
                raise RuntimeError(err())
        return C.string_at(buf, ln.value) if ln.value else b""
    finally:
        L.kite_reader_close(r)
        if buf.value:
            C.CDLL(None).free(buf)


def synth_reads(genome_codes, n_reads: int, read_len: int, sub_rate: float, n_rate: float, revcomp_frac: float,
                seed: int, first_index: int = 0, threads: int = 8) -> bytearray:
    import numpy as np
    g = np.ascontiguousarray(genome_codes, dtype=np.uint8)
    rec = 11 + 1 + read_len + 1 + 2 + read_len + 1
    out = bytearray(n_reads * rec)
    buf = (C.c_uint8 * len(out)).from_buffer(out)
    n = lib().kite_synth_reads(g.ctypes.data, len(g), n_reads, read_len, sub_rate, n_rate, revcomp_frac, seed,
                               first_index, C.addressof(buf), len(out), threads)
    if n < 0:
        raise RuntimeError(err())
    return out


def synth_reads_var(genome_codes, n_reads: int, len_lo: int, len_hi: int, sub_rate: float, seed: int,
                    first_index: int = 0, threads: int = 8) -> bytearray:
    """Reads of lengths uniform in [len_lo, len_hi] sampled from genome_codes
    (forward strand, substitutions only), multithreaded and deterministic."""
    import numpy as np
    g = np.ascontiguousarray(genome_codes, dtype=np.uint8)
    cap = n_reads * (2 * len_hi + 16)
    out = bytearray(cap)
    buf = (C.c_uint8 * len(out)).from_buffer(out)
    L = lib()
    L.kite_synth_reads_var.argtypes = [C.c_void_p, C.c_uint64, C.c_uint64, C.c_uint32, C.c_uint32, C.c_double,
                                       C.c_double, C.c_double, C.c_uint64, C.c_uint64, C.c_void_p, C.c_uint64,
                                       C.c_int]
    L.kite_synth_reads_var.restype = C.c_int64
    n = L.kite_synth_reads_var(g.ctypes.data, len(g), n_reads, len_lo, len_hi, sub_rate, 0.0, 0.0, seed,
                               first_index, C.addressof(buf), cap, threads)
    if n < 0:
        raise RuntimeError(err())
    del buf
    return out[:n]
