"""Reader/writer helpers for the `.kite` (KX2) on-disk format in Python.

Layout (src/format/header.rs:62-92, src/format/bucket_dir.rs:6-147):
  128-byte header, data area, chunk index (128 B per chunk), partition table
  (40 B per partition), 24-byte footer "KX2FOOT!".
"""
from __future__ import annotations

import ctypes as C
import struct
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Chunk:
    partition_id: int
    codec: int
    file_offset: int
    encoded_bytes: int
    raw_bytes: int
    row_count: int
    key_min: int
    key_max: int


@dataclass
class KiteImage:
    data: bytes
    k: int = 0
    canonical: int = 0
    partitions: int = 0
    key_width: int = 0
    codec_mask: int = 0
    total_chunks: int = 0
    total_rows: int = 0
    min_count: int | None = None
    max_count: int | None = None
    chunks: list = field(default_factory=list)
    part_first: list = field(default_factory=list)
    part_count: list = field(default_factory=list)

    @classmethod
    def parse(cls, data: bytes) -> "KiteImage":
        if len(data) < 152 or data[:4] != b"KX2!":
            raise ValueError("not a .kite (KX2) image")
        (ver, k, canon, parts, kw, cm, _ck, cio, pto, fo, tc, tr) = struct.unpack_from("<HBBIHHIQQQQQ", data, 4)
        img = cls(data=data, k=k, canonical=canon, partitions=parts, key_width=kw, codec_mask=cm,
                  total_chunks=tc, total_rows=tr)
        res = data[60:128]
        if res[:4] == b"KMT1":
            flags, mn, mx = struct.unpack_from("<III", res, 4)
            img.min_count = mn if flags & 1 else None
            img.max_count = mx if flags & 2 else None
        if data[fo + 16:fo + 24] != b"KX2FOOT!":
            raise ValueError("invalid footer magic")
        n_chunks = (pto - cio) // 128
        for i in range(n_chunks):
            o = cio + 128 * i
            pid, codec, off, enc, raw, rows = struct.unpack_from("<IIQQQQ", data, o)
            kmin_lo = int.from_bytes(data[o + 40:o + 56], "little")
            kmax_lo = int.from_bytes(data[o + 72:o + 88], "little")
            img.chunks.append(Chunk(pid, codec, off, enc, raw, rows, kmin_lo, kmax_lo))
        for p in range(parts):
            first, cnt, _rows, _doff, _dbytes = struct.unpack_from("<QQQQQ", data, pto + 40 * p)
            img.part_first.append(first)
            img.part_count.append(cnt)
        return img

    def partition_chunks(self, p: int) -> list:
        return self.chunks[self.part_first[p]:self.part_first[p] + self.part_count[p]]

    def payload(self, c: Chunk) -> bytes:
        return self.data[c.file_offset:c.file_offset + c.encoded_bytes]

    def merge_input(self, base_address: int | None = None):
        """A kite_gpu_merge_input over this image (keeps the arrays alive).
        With base_address, the image bytes are read from that host address
        (e.g. a pinned copy of the image) instead of a private copy."""
        from .gpu import MergeInput
        n = len(self.chunks)
        arrs = {
            "off": np.array([c.file_offset for c in self.chunks], dtype=np.uint64),
            "len": np.array([c.encoded_bytes for c in self.chunks], dtype=np.uint64),
            "rows": np.array([c.row_count for c in self.chunks], dtype=np.uint64),
            "codec": np.array([c.codec for c in self.chunks], dtype=np.uint32),
            "first": np.array(self.part_first, dtype=np.uint64),
            "count": np.array(self.part_count, dtype=np.uint64),
        }
        buf = None
        if base_address is None:
            buf = (C.c_uint8 * len(self.data)).from_buffer_copy(self.data)
            base_address = C.addressof(buf)
        p64 = lambda a: a.ctypes.data_as(C.POINTER(C.c_uint64))  # noqa: E731
        mi = MergeInput(base_address, len(self.data), p64(arrs["off"]), p64(arrs["len"]), p64(arrs["rows"]),
                        arrs["codec"].ctypes.data_as(C.POINTER(C.c_uint32)), p64(arrs["first"]),
                        p64(arrs["count"]), 1 if self.min_count is not None else 0,
                        1 if self.max_count is not None else 0, self.min_count or 0, self.max_count or 0)
        _ = n
        return mi, (buf, arrs)


def read(path: str) -> KiteImage:
    with open(path, "rb") as f:
        return KiteImage.parse(f.read())
