"""FASTQ chunking for submission (host side).

Mirrors PlainChunkedReader/GzipChunkedReader::next_chunk
(src/count/decompress.rs:36-138): read chunk_size new bytes after the
carried tail, cut after the last 4k-th newline (find_fastq_split_4lines,
src/count/bgzf.rs:109-121), carry the rest.  A short read means EOF: the
final chunk is returned whole.
"""
from __future__ import annotations


def find_fastq_split(buf, start: int, end: int) -> int:
    """Offset (relative to start) just after the last 4k-th newline, or 0."""
    b = bytes(memoryview(buf)[start:end])
    total = b.count(b"\n")
    keep = total - total % 4
    if keep == 0:
        return 0
    pos = len(b)
    for _ in range(total - keep + 1):
        pos = b.rfind(b"\n", 0, pos)
    return pos + 1


def split_chunks(data, chunk_size: int) -> list[tuple[int, int]]:
    """(offset, length) of every chunk the reference's reader would produce."""
    n = len(data)
    out = []
    consumed = carry = 0
    while True:
        start = consumed - carry
        new = min(chunk_size, n - consumed)
        consumed += new
        length = carry + new
        if length == 0:
            break
        if new < chunk_size:
            out.append((start, length))
            break
        split = find_fastq_split(data, start, start + length)
        if split == 0 or split >= length:
            out.append((start, length))
            carry = 0
        else:
            out.append((start, split))
            carry = length - split
    return out
