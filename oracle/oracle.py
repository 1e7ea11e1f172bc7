"""ctypes wrapper of the CPU oracle (oracle/_build/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg as the checker.  The product never imports it.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "liboracle.so"
CLI = BUILD / "kite_oracle"
_lib = None


def build() -> None:
    r = subprocess.run(["make", "-s", "-C", str(HERE)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        L = C.CDLL(str(LIB))
        L.orc_last_error.restype = C.c_char_p
        L.orc_parse_sequences.argtypes = [C.c_char_p, C.c_size_t, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64),
                                          C.c_size_t]
        L.orc_parse_sequences.restype = C.c_longlong
        L.orc_find_fastq_split.argtypes = [C.c_char_p, C.c_size_t]
        L.orc_find_fastq_split.restype = C.c_size_t
        L.orc_kmers.argtypes = [C.c_char_p, C.c_size_t, C.c_uint, C.c_int, C.c_int, C.POINTER(C.c_uint64),
                                C.c_size_t]
        L.orc_kmers.restype = C.c_size_t
        L.orc_bucket.argtypes = [C.c_uint64, C.c_uint64, C.c_int, C.c_uint]
        L.orc_bucket.restype = C.c_size_t
        L.orc_rle_u64.argtypes = [C.POINTER(C.c_uint64), C.c_size_t, C.POINTER(C.c_uint64), C.POINTER(C.c_uint32)]
        L.orc_rle_u64.restype = C.c_size_t
        L.orc_sort_u64.argtypes = [C.POINTER(C.c_uint64), C.c_size_t, C.c_uint]
        L.orc_encode_dvle.argtypes = [C.POINTER(C.c_uint64), C.POINTER(C.c_uint32), C.c_size_t, C.c_int,
                                      C.POINTER(C.c_uint8), C.c_size_t]
        L.orc_encode_dvle.restype = C.c_size_t
        L.orc_decode_kmer.argtypes = [C.c_uint64, C.c_uint64, C.c_uint, C.c_char_p]
        L.orc_loser_tree_u64.argtypes = [C.POINTER(C.c_uint64), C.POINTER(C.c_uint32), C.POINTER(C.c_size_t),
                                         C.c_size_t, C.POINTER(C.c_uint64), C.POINTER(C.c_uint32)]
        L.orc_loser_tree_u64.restype = C.c_size_t
        L.orc_merge_vectors_u64.argtypes = [C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), C.POINTER(C.c_size_t),
                                            C.c_size_t, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
        L.orc_merge_vectors_u64.restype = C.c_size_t
        L.orc_serialize_u64.argtypes = [C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), C.c_size_t,
                                        C.POINTER(C.c_uint8), C.c_size_t]
        L.orc_serialize_u64.restype = C.c_longlong
        L.orc_header_bytes.argtypes = [C.c_uint, C.c_int, C.c_uint, C.c_uint, C.c_uint, C.c_int, C.c_uint, C.c_int,
                                       C.c_uint, C.POINTER(C.c_uint8)]
        L.orc_header_parse.argtypes = [C.POINTER(C.c_uint8), C.c_size_t, C.POINTER(C.c_uint64)]
        L.orc_count_buffer.argtypes = [C.c_char_p, C.c_size_t, C.c_uint, C.c_int, C.c_size_t, C.c_size_t,
                                       C.c_size_t, C.POINTER(C.c_uint64)]
        L.orc_count_kite.argtypes = [C.c_char_p, C.c_size_t, C.c_uint, C.c_int, C.c_size_t, C.c_size_t, C.c_size_t,
                                     C.c_size_t, C.c_int, C.c_uint, C.c_int, C.c_uint, C.c_void_p, C.c_size_t,
                                     C.POINTER(C.c_uint64)]
        L.orc_count_kite.restype = C.c_longlong
        L.orc_dump_kite.argtypes = [C.c_char_p, C.c_size_t, C.c_void_p, C.c_size_t]
        L.orc_dump_kite.restype = C.c_longlong
        L.orc_merge_files.argtypes = [C.POINTER(C.c_char_p), C.c_size_t, C.c_size_t, C.c_void_p, C.c_size_t]
        L.orc_merge_files.restype = C.c_longlong
        L.orc_count_parts.argtypes = [C.c_char_p, C.c_size_t, C.c_uint, C.c_int, C.c_size_t, C.c_size_t, C.c_size_t,
                                      C.POINTER(C.c_void_p), C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
        L.orc_count_parts.restype = C.c_longlong
        L.orc_free.argtypes = [C.c_void_p]
        _lib = L
    return _lib


def err() -> str:
    return lib().orc_last_error().decode()


def count_kite(fastq: bytes, k: int, canonical: bool, partitions: int, staging_bytes: int = 16 << 20,
               lanes: int = 2, chunk_size: int = 64 << 20, min_count=None, max_count=None):
    """Single-worker count of an in-memory FASTQ; returns (.kite image, (reads, bases, kmers))."""
    L = lib()
    st = (C.c_uint64 * 3)()
    args = (fastq, len(fastq), k, 1 if canonical else 0, partitions, staging_bytes, lanes, chunk_size,
            0 if min_count is None else 1, min_count or 0, 0 if max_count is None else 1, max_count or 0)
    n = L.orc_count_kite(*args, None, 0, st)
    if n < 0:
        raise RuntimeError(err())
    buf = C.create_string_buffer(n)
    n2 = L.orc_count_kite(*args, buf, n, st)
    assert n2 == n
    return buf.raw[:n], (st[0], st[1], st[2])


def dump(image: bytes) -> bytes:
    L = lib()
    n = L.orc_dump_kite(image, len(image), None, 0)
    if n < 0:
        raise RuntimeError(err())
    buf = C.create_string_buffer(max(n, 1))
    L.orc_dump_kite(image, len(image), buf, n)
    return buf.raw[:n]


def merge_files(paths: list, lanes: int = 2) -> bytes:
    L = lib()
    arr = (C.c_char_p * len(paths))(*[str(p).encode() for p in paths])
    n = L.orc_merge_files(arr, len(paths), lanes, None, 0)
    if n < 0:
        raise RuntimeError(err())
    buf = C.create_string_buffer(n)
    L.orc_merge_files(arr, len(paths), lanes, buf, n)
    return buf.raw[:n]


def count_buffer(fastq: bytes, k: int, canonical: bool, partitions: int, workers: int,
                 chunk_size: int = 64 << 20) -> dict:
    """Timed multi-worker count to per-partition DVLE payloads (no file)."""
    L = lib()
    st = (C.c_uint64 * 7)()
    rc = L.orc_count_buffer(fastq, len(fastq), k, 1 if canonical else 0, partitions, workers, chunk_size, st)
    if rc != 0:
        raise RuntimeError(err())
    keys = ["reads", "bases", "kmers", "rows", "chunks", "payload_bytes", "ns"]
    return dict(zip(keys, list(st)))


class Parts:
    """Per-partition payloads of the single-worker count (orc_count_parts):
    meta[p] = (rows, bytes, key_min, key_max), payload(p) a memoryview."""

    def __init__(self, buf, total: int, meta, P: int, stats):
        self._buf = buf
        self.total = total
        self.P = P
        self.reads, self.bases, self.kmers, ns = stats
        self.seconds = ns / 1e9
        self.rows, self.bytes, self.key_min, self.key_max, self.offset = [], [], [], [], []
        off = 0
        for p in range(P):
            m = meta[6 * p:6 * p + 6]
            self.rows.append(m[0])
            self.bytes.append(m[1])
            self.key_min.append(m[2] | (m[3] << 64))
            self.key_max.append(m[4] | (m[5] << 64))
            self.offset.append(off)
            off += m[1]
        self._view = (C.c_uint8 * max(total, 1)).from_address(buf.value) if total else None

    def payload(self, p: int) -> memoryview:
        """A view of partition p's payload (valid until close); compare it
        through bytes() or numpy, not element by element."""
        if not self.bytes[p]:
            return memoryview(b"")
        return memoryview(self._view)[self.offset[p]:self.offset[p] + self.bytes[p]]

    def nonempty(self) -> list:
        return [p for p in range(self.P) if self.rows[p]]

    def close(self) -> None:
        if self._buf is not None and self._buf.value:
            lib().orc_free(self._buf)
        self._buf = None
        self._view = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def count_parts(fastq, k: int, canonical: bool, partitions: int, threads: int, chunk_size: int = 64 << 20) -> Parts:
    """Multi-threaded count with the single-worker count's per-partition
    payloads (deterministic).  `fastq` is bytes or any object exposing a
    buffer (bytearray, numpy array)."""
    L = lib()
    meta = (C.c_uint64 * (6 * partitions))()
    st = (C.c_uint64 * 4)()
    out = C.c_void_p()
    if isinstance(fastq, bytes):
        ptr, n = fastq, len(fastq)
    else:
        mv = memoryview(fastq).cast("B")
        n = mv.nbytes
        ptr = C.cast((C.c_char * n).from_buffer(mv) if not mv.readonly else C.c_char_p(bytes(mv)), C.c_char_p)
    total = L.orc_count_parts(ptr, n, k, 1 if canonical else 0, partitions, threads, chunk_size, C.byref(out), meta,
                              st)
    if total < 0:
        raise RuntimeError(err())
    return Parts(out, total, list(meta), partitions, list(st))


def merge_images(images: list, threads: int) -> dict:
    """Timed merge of in-memory .kite images with `threads` threads
    (orc_merge_images): rows in / out, payload bytes out, seconds."""
    L = lib()
    L.orc_merge_images.argtypes = [C.POINTER(C.c_char_p), C.POINTER(C.c_size_t), C.c_size_t, C.c_size_t,
                                   C.POINTER(C.c_uint64)]
    arr = (C.c_char_p * len(images))(*images)
    lens = (C.c_size_t * len(images))(*[len(x) for x in images])
    st = (C.c_uint64 * 4)()
    if L.orc_merge_images(arr, lens, len(images), threads, st) != 0:
        raise RuntimeError(err())
    return {"rows_in": st[0], "rows_out": st[1], "bytes_out": st[2], "seconds": st[3] / 1e9}
