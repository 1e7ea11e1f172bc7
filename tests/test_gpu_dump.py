"""GPU `kite dump` against the oracle's dump of the same .kite image: byte-
identical TSV (integer work: the bar is byte equality) for counts with one or
several chunks per partition, u64 and u128 keys, header min/max filters, RAW
chunks, sums above u32::MAX (saturated before the filter) and empty
partitions."""
import ctypes

import numpy as np
import pytest

from kite_gb300 import host, ingest, synth
from kite_gb300.kitefile import KiteImage
from kite_build import build_image, bucket

pytestmark = pytest.mark.gpu

U32 = 0xFFFFFFFF


def gpu_dump(gpu, img: bytes) -> bytes:
    ki = KiteImage.parse(img)
    with gpu.Counter(ki.k, bool(ki.canonical), ki.partitions) as c:
        return c.dump(ki)


def _kmer(v: int, k: int) -> bytes:
    return bytes(b"ACGT"[(v >> (2 * (k - 1 - i))) & 3] for i in range(k))


def _kmer_value(s: bytes) -> int:
    v = 0
    for ch in s:
        v = (v << 2) | b"ACGT".index(ch)
    return v


@pytest.mark.parametrize("k,canonical", [(1, False), (21, False), (31, True), (32, True), (63, True), (64, False)])
@pytest.mark.parametrize("flt", [(None, None), (2, None), (2, 40)])
def test_dump_of_counts(gpu, orc, k, canonical, flt):
    fq = synth.small_workload(seed=60 + k, n_reads=3000, genome_len=20_000)
    img, _ = orc.count_kite(fq, k, canonical, 16, min_count=flt[0], max_count=flt[1])
    a = gpu_dump(gpu, img)
    assert a == orc.dump(img)
    assert a == host.dump_image(img)


def test_dump_of_segmented_count(gpu, orc):
    # a small device arena cuts the count into segments: every partition then
    # holds several chunks whose keys overlap, summed by the dump
    fq = synth.small_workload(seed=5, n_reads=6000, genome_len=30_000)
    chunks = ingest.split_chunks(fq, 100_000)
    w = host.Writer(None, 25, True, 8, 64, 7, 16 << 20, 2, 2, None)
    segs = 0
    with gpu.Counter(25, True, 8, arena_bytes=256 * 1024) as c:
        for o, l in chunks:
            try:
                c.submit(fq[o:o + l])
            except gpu.KiteGpuError as e:
                assert e.code == -9
                for m, p in c.finish():
                    w.append(m, p)
                segs += 1
                c.submit(fq[o:o + l])
        for m, p in c.finish():
            w.append(m, p)
        segs += 1
    w.worker_drain()
    w.finalize()
    img = w.image()
    w.close()
    ki = KiteImage.parse(img)
    assert segs >= 2 and max(ki.part_count) >= 2
    assert gpu_dump(gpu, img) == orc.dump(img)


@pytest.mark.parametrize("wide", [False, True])
def test_dump_multichunk_and_raw(gpu, orc, wide):
    rng = np.random.default_rng(8)
    P, k = 8, (45 if wide else 25)
    keys = np.unique(rng.integers(0, 1 << 40, size=5000, dtype=np.uint64)).tolist()
    parts = {}
    for key in keys:
        parts.setdefault(bucket(int(key), P, wide), []).append(int(key))
    chunks = []
    for p, ks in sorted(parts.items()):
        for j in range(3):
            sel = sorted(set(ks[j::2] + ks[::3]))
            chunks.append((p, [(x, int(rng.integers(1, 9))) for x in sel], 1 if j == 2 else 2))
    for flt in ((None, None), (3, 12)):
        img = build_image(k, True, P, chunks, min_count=flt[0], max_count=flt[1])
        assert gpu_dump(gpu, img) == orc.dump(img)


@pytest.mark.parametrize("mx,present", [(None, True), (U32, True), (100, False)])
def test_dump_saturating_sum(gpu, orc, mx, present):
    # 0xFFFFFFFF + 5 saturates to 0xFFFFFFFF; the header max applies to that
    P = 4
    key = 100
    p = bucket(key, P, False)
    chunks = [(p, [(key, U32), (key + 1, 3)], 2), (p, [(key, 5)], 2), (bucket(7, P, False), [(7, 2)], 1)]
    img = build_image(21, False, P, chunks, max_count=mx)
    a = gpu_dump(gpu, img)
    assert a == orc.dump(img)
    assert _kmer(100, 21) == b"A" * 17 + b"CGCA"
    assert (_kmer(100, 21) + b"\t4294967295\n" in a) == present
    assert _kmer(101, 21) + b"\t3\n" in a


def test_dump_empty_and_sparse(gpu, orc):
    empty = build_image(21, False, 16, [])
    assert gpu_dump(gpu, empty) == b"" == orc.dump(empty)
    one = build_image(21, False, 16, [(bucket(9, 16, False), [(9, 1)], 2)])
    assert gpu_dump(gpu, one) == orc.dump(one) == b"A" * 19 + b"GC\t1\n"


def test_dump_tile_refinement_and_meta(gpu, orc):
    # tens of thousands of rows in a partition with clustered keys: several
    # merge tiles per partition; the emitted meta names each partition's
    # line count, bytes and first / last key
    P = 2
    rng = np.random.default_rng(3)
    base = [int(x) for x in np.unique(rng.integers(0, 1 << 20, size=60000))]
    a, b = {}, {}
    for key in base:
        p = bucket(key, P, False)
        a.setdefault(p, []).append((key, 1))
        b.setdefault(p, []).append((key, int(rng.integers(1, 1000))))
    img = build_image(21, False, P, [(p, r, 2) for p, r in sorted(a.items())] +
                      [(p, r, 2) for p, r in sorted(b.items())])
    ki = KiteImage.parse(img)
    metas = []
    with gpu.Counter(21, False, P) as c:
        c.dump(ki, callback=lambda m, addr, n: metas.append((m, ctypes.string_at(addr, n))))
        st = c.stats()
    assert b"".join(x for _, x in metas) == orc.dump(img)
    assert st["tiles"] > 2 * P
    for m, tsv in metas:
        lines = tsv.splitlines()
        assert m["row_count"] == len(lines) and m["raw_bytes"] == len(tsv) and m["codec"] == 0
        assert m["key_min"] == _kmer_value(lines[0].split(b"\t")[0])
        assert m["key_max"] == _kmer_value(lines[-1].split(b"\t")[0])


def test_dump_streams_groups(gpu, orc):
    # a TSV of ~0.8 GB leaves the device in several groups of whole
    # partitions through the two pinned staging halves (256 MB each)
    g = synth.genome_iid(np.random.default_rng(17), 20_000_000)
    fq = bytes(host.synth_reads(g, 300_000, 150, 0.01, 0.001, 0.5, seed=17))
    w = host.Writer(None, 31, True, 64, 64, 7, 16 << 20, 2)
    with gpu.Counter(31, True, 64) as c:
        c.submit(fq)
        for m, p in c.finish():
            w.append(m, p)
    w.worker_drain()
    w.finalize()
    img = w.image()
    w.close()
    with gpu.Counter(31, True, 64) as c:
        parts = []
        c.dump(KiteImage.parse(img), callback=lambda m, addr, n: parts.append(ctypes.string_at(addr, n)))
        st = c.stats()
    tsv = b"".join(parts)
    assert st["payload_bytes"] == len(tsv) > (600 << 20)
    assert tsv == orc.dump(img)
