"""Shared helpers for the GPU parity tests: run the CUDA path through the
C ABI and the oracle on the same bytes, compare partition payloads."""
from kite_gb300 import ingest
from kite_gb300.kitefile import KiteImage


def gpu_count(gpu, fastq: bytes, k: int, canonical: bool, P: int, chunk_size: int = 1 << 20, **kw):
    with gpu.Counter(k, canonical, P, **kw) as c:
        for o, l in ingest.split_chunks(fastq, chunk_size):
            c.submit(fastq[o:o + l])
        out = c.finish()
        st = c.stats()
    return out, st


def oracle_parts(orc, fastq: bytes, k: int, canonical: bool, P: int, chunk_size: int = 1 << 20):
    img, stats = orc.count_kite(fastq, k, canonical, P, chunk_size=chunk_size)
    ki = KiteImage.parse(img)
    parts = {}
    for p in range(P):
        ch = ki.partition_chunks(p)
        assert len(ch) <= 1
        if ch:
            parts[p] = (ch[0], ki.payload(ch[0]))
    return parts, stats, img


def assert_parity(gpu, orc, fastq: bytes, k: int, canonical: bool, P: int, chunk_size: int = 1 << 20, **kw):
    out, st = gpu_count(gpu, fastq, k, canonical, P, chunk_size, **kw)
    parts, (reads, bases, kmers), _ = oracle_parts(orc, fastq, k, canonical, P, chunk_size)
    assert (st["reads"], st["bases"], st["kmers"]) == (reads, bases, kmers)
    got = {m["partition_id"]: (m, payload) for m, payload in out}
    assert sorted(got) == sorted(parts), "non-empty partition sets differ"
    for p, (ch, payload) in parts.items():
        m, gp = got[p]
        assert m["row_count"] == ch.row_count, f"partition {p} rows"
        assert m["key_min"] == ch.key_min and m["key_max"] == ch.key_max, f"partition {p} key range"
        assert m["codec"] == ch.codec and m["raw_bytes"] == ch.raw_bytes
        assert gp == payload, f"partition {p} payload differs"
    return st
