"""Test helper: builds .kite images from explicit per-partition chunk rows
(DVLE or RAW payloads encoded here), through the host writer, so merge tests
can use multi-chunk partitions, RAW chunks, filters and huge counts."""
from kite_gb300 import host


def varint(v: int) -> bytes:
    out = bytearray()
    while True:
        b = v & 0x7F
        v >>= 7
        if v == 0:
            out.append(b)
            return bytes(out)
        out.append(b | 0x80)


def dvle(rows, wide: bool) -> bytes:
    kb = 16 if wide else 8
    k0, c0 = rows[0]
    out = bytearray(k0.to_bytes(kb, "little") + c0.to_bytes(4, "little"))
    prev = k0
    for k, c in rows[1:]:
        out += varint(k - prev) + varint(c)
        prev = k
    return bytes(out)


def raw(rows, wide: bool) -> bytes:
    kb = 16 if wide else 8
    return b"".join(k.to_bytes(kb, "little") + c.to_bytes(4, "little") for k, c in rows)


def bucket(key: int, P: int, wide: bool) -> int:
    bits = P.bit_length() - 1
    x = ((key & (2**64 - 1)) ^ (key >> 64)) if wide else key
    return ((x * 0x9E3779B97F4A7C15) & (2**64 - 1)) >> (64 - bits)


def build_image(k: int, canonical: bool, P: int, chunks, min_count=None, max_count=None, codec_mask=7,
                staging=16 << 20, lanes=2) -> bytes:
    """chunks: list of (partition, rows sorted by key, codec) appended in order."""
    wide = k > 31
    w = host.Writer(None, k, canonical, P, 128 if wide else 64, codec_mask, staging, lanes, min_count, max_count)
    for p, rows, codec in chunks:
        payload = dvle(rows, wide) if codec == 2 else raw(rows, wide)
        w.append({"partition_id": p, "codec": codec, "row_count": len(rows), "raw_bytes": len(payload),
                  "key_min": rows[0][0], "key_max": rows[-1][0]}, payload)
    w.worker_drain()
    w.finalize()
    img = w.image()
    w.close()
    return img
