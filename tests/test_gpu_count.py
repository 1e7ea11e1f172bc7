"""GPU count path vs the CPU oracle: bit-exact partition payloads (DVLE
bytes), row counts, key ranges and the reads/bases/kmers summary.  Integer
work: the bar is byte equality."""
import numpy as np
import pytest

from kite_gb300 import synth
from gpu_helpers import assert_parity, gpu_count

pytestmark = pytest.mark.gpu


EDGE = [
    b"",
    b"@r\nACGT\n+\nIIII\n",
    b"@r\nACGTNACGTTGCA\n+\nIIIIIIIIIIIII\n@s\n\n+\n\n@t\nacgtacgtACGTtt\n+\nIIIIIIIIIIIIII\n",
    b"@r\r\nACGTACGTAC\r\n+\r\nIIIIIIIIII\r\n",
    b"@r\nACGTACGTACGGATTACA\n+\nIIIIIIIIIIIIIIIIII\n@u\nGGGATTACAGATTACACC",  # unterminated seq line
    b"NOTFASTQ\nACGTACGT\n+\nIIIIIIII\n",  # chunk not starting with '@' is ignored
    b"@q\nACGTACGTAC\n+\n@IIIIIIIII\n@r\nTTTTGGGGCCCCAAAA\n+\nIIIIIIIIIIIIIIII\n",  # '@' in quality
]


@pytest.mark.parametrize("k,canonical", [(1, False), (3, True), (21, False), (31, True), (32, True), (33, False),
                                         (63, True), (64, False), (64, True)])
@pytest.mark.parametrize("case", range(len(EDGE)))
def test_edge_inputs(gpu, orc, case, k, canonical):
    assert_parity(gpu, orc, EDGE[case], k, canonical, 4)


@pytest.mark.parametrize("P", [2, 16, 256, 2048])
def test_partitions(gpu, orc, P):
    fq = synth.small_workload(seed=11, n_reads=3000, genome_len=20_000)
    assert_parity(gpu, orc, fq, 21, False, P)


@pytest.mark.parametrize("k,canonical", [(21, False), (31, True), (47, True), (63, True)])
def test_small_workload(gpu, orc, k, canonical):
    fq = synth.small_workload(seed=7, n_reads=20_000, genome_len=200_000)
    assert_parity(gpu, orc, fq, k, canonical, 16, chunk_size=300_000)


def test_tiled_buckets_u64(gpu, orc):
    # enough k-mers per bucket to need key-range tiles (and several chunks)
    fq = synth.small_workload(seed=1, n_reads=60_000, genome_len=1_000_000)
    st = assert_parity(gpu, orc, fq, 21, False, 2, chunk_size=1 << 20)
    assert st["tiles_per_bucket"] > 1


def test_tiled_single_level(gpu, orc):
    # up to 256 tiles per bucket: the split runs as one level
    fq = synth.small_workload(seed=3, n_reads=20_000, genome_len=400_000)
    st = assert_parity(gpu, orc, fq, 25, True, 8)
    assert 1 < st["tiles_per_bucket"] <= 256


def test_tiled_buckets_u128(gpu, orc):
    fq = synth.small_workload(seed=2, n_reads=40_000, genome_len=500_000)
    st = assert_parity(gpu, orc, fq, 63, True, 2, chunk_size=1 << 20)
    assert st["tiles_per_bucket"] > 1


def test_heavy_hitter_oversized_tile(gpu, orc):
    # poly-A reads: one key with a huge count fills a tile beyond on-chip capacity
    rng = np.random.default_rng(3)
    g = synth.genome_iid(rng, 50_000)
    fq = synth.reads_fixed(rng, g, 4000, 150, 0.0) + (b"@a\n" + b"A" * 150 + b"\n+\n" + b"I" * 150 + b"\n") * 3000
    st = assert_parity(gpu, orc, fq, 21, True, 2)
    assert st["big_tiles"] >= 1


def test_heavy_mixed_big_tile(gpu, orc):
    # a low-complexity region: few distinct keys, many copies, in a tiled bucket
    rng = np.random.default_rng(9)
    g = synth.genome_iid(rng, 400_000)
    g[:2000] = np.tile(np.array([0, 1], dtype=np.uint8), 1000)
    fq = synth.reads_fixed(rng, g, 40_000, 150, 0.0)
    fq += synth.reads_fixed(rng, g[:2200], 20_000, 150, 0.0)
    assert_parity(gpu, orc, fq, 31, False, 2)


def _rec(s: bytes) -> bytes:
    return b"@m\n" + s + b"\n+\n" + b"I" * len(s) + b"\n"


def _kmer(v: int, k: int) -> bytes:
    return bytes(b"ACGT"[(v >> (2 * (k - 1 - i))) & 3] for i in range(k))


@pytest.mark.parametrize("copies", [100, 300])
def test_mixed_bin(gpu, orc, copies):
    # Two distinct repeated keys that sit close together in one tile (k=21
    # forward keys 0 = A*21 and 2 = A*20+G share partition 0 of 2, and G*21
    # widens the tile's span so both fall in its first bin): 100 copies each
    # are ordered by counting inside the bin; 300 each make a large bin that
    # one warp sorts by extracting its distinct keys.
    fq = _rec(b"A" * 21) * copies + _rec(b"A" * 20 + b"G") * copies + _rec(b"G" * 21)
    rng = np.random.default_rng(11)
    fq += synth.reads_fixed(rng, synth.genome_iid(rng, 5000), 40, 60, 0.0)
    st = assert_parity(gpu, orc, fq, 21, False, 2)
    assert st["sort_fallbacks"] == 0


def test_large_tile_on_chip(gpu, orc):
    # 12,001 keys in partition 0: the tile holding the two repeated keys is
    # over the regular on-chip capacity (8192) but within twice it, so it
    # takes the double-capacity on-chip sort.
    # (sampled splitters: the learned ones cut the two keys apart)
    fq = _rec(b"A" * 21) * 6000 + _rec(b"A" * 20 + b"G") * 6000 + _rec(b"G" * 21)
    st = assert_parity(gpu, orc, fq, 21, False, 2, splitter_mode=gpu.SPLIT_SAMPLED)
    assert st["big_tiles"] >= 1


def test_large_bin_many_distinct(gpu, orc):
    # 40 distinct small keys of partition 0 (of 2), 10 copies each, share the
    # first bin of a tile widened by G*21: more distinct keys than one warp
    # extracts, so the tile takes the LSD fallback.
    from kite_build import bucket
    vals = [v for v in range(400) if bucket(v, 2, False) == 0][:40]
    fq = b"".join(_rec(_kmer(v, 21)) * 10 for v in vals) + _rec(b"G" * 21)
    st = assert_parity(gpu, orc, fq, 21, False, 2, splitter_mode=gpu.SPLIT_SAMPLED)
    assert st["sort_fallbacks"] >= 1


def test_dense_sequence_fallback(gpu, orc):
    # sequence lines with empty quality lines: close to one k-mer per FASTQ
    # byte, more than the staged-key capacity, so the extraction scatter runs
    rng = np.random.default_rng(12)
    seqs = [bytes(b"ACGT"[x] for x in rng.integers(0, 4, 2000)) for _ in range(50)]
    fq = b"".join(b"@d\n" + q + b"\n+\n\n" for q in seqs)
    assert_parity(gpu, orc, fq, 21, True, 16)


def test_segments_flush(gpu, orc):
    # a small arena forces several segments, so partitions hold several
    # chunks (one per segment, as the reference's worker flushes a segment
    # whenever its buffer fills): the summed counts, seen through the oracle's
    # `dump -o -` of a .kite image holding every chunk, must equal the dump of
    # the oracle's own count of the same reads
    from kite_gb300 import host, ingest
    fq = synth.small_workload(seed=5, n_reads=5000, genome_len=30_000)
    chunks = ingest.split_chunks(fq, 100_000)
    emitted = []
    with gpu.Counter(21, False, 8, arena_bytes=256 * 1024) as c:
        for o, l in chunks:
            try:
                c.submit(fq[o:o + l])
            except gpu.KiteGpuError as e:
                assert e.code == -9
                emitted += c.finish()
                c.submit(fq[o:o + l])
        emitted += c.finish()
        assert c.stats()["segments"] >= 2
    per_part = {}
    for m, _ in emitted:
        per_part[m["partition_id"]] = per_part.get(m["partition_id"], 0) + 1
    assert max(per_part.values()) >= 2
    w = host.Writer(None, 21, False, 8, 64, 7, 16 << 20, 2)
    for m, payload in emitted:
        w.append(m, payload)
    w.worker_drain()
    w.finalize()
    image = w.image()
    w.close()
    ref, _ = orc.count_kite(fq, 21, False, 8)
    got = orc.dump(image)
    assert got == orc.dump(ref) and got.count(b"\n") > 1000


@pytest.mark.parametrize("mode", ["sampled", "learned"])
def test_skewed_clustered_tiles(gpu, orc, mode):
    # AT-rich low-complexity keys (k=63, u128) in 2 partitions: hundreds of
    # key-range tiles per bucket, keys clustered inside them; thousands of
    # tiles have bins with many distinct keys and take the LSD fallback.
    # Bytes must match the oracle with either splitter method.
    fq = synth.skewed_workload(seed=6, n_reads=12_000, genome_len=400_000)
    sm = gpu.SPLIT_SAMPLED if mode == "sampled" else gpu.SPLIT_LEARNED
    st = assert_parity(gpu, orc, fq, 63, True, 2, splitter_mode=sm, imbalance_bound=100.0)
    assert st["tiles_per_bucket"] > 32



def test_tile_sort_bulk_load_timeout(gpu, orc):
    # the tile sort's first bounded wait for a tile's bulk load set to one
    # non-blocking test: the wait gives up, every CTA still waits for its copy
    # to land before it moves on, and the count returns KITE_ERR_TIMEOUT; the
    # device stays usable and a normal count afterwards is exact
    fq = synth.small_workload(seed=1, n_reads=20_000, genome_len=200_000)
    with gpu.Counter(21, False, 16, tile_wait_polls=1) as c:
        c.submit(fq)
        with pytest.raises(gpu.KiteGpuError) as e:
            c.finish()
        assert e.value.code == -3 and "bulk load" in str(e.value)
    assert_parity(gpu, orc, fq, 21, False, 16)
