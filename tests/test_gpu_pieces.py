"""Host chunks counted in input pieces: the chunks fall into up to eight runs,
each run's bucket scatter starts as soon as its last chunk is extracted (while
later chunks are still copying in), and the first key-range split level reads
every bucket as one run per piece.  Byte parity with the oracle through each
branch: pieces with key-range tiles (one and two split levels, u64 and u128
keys), pieces with one tile per bucket (the staged keys scattered again in
bucket order), staging over capacity (the scatter from the FASTQ, no pieces),
and device submissions (no pieces)."""
import numpy as np
import pytest

from kite_gb300 import ingest, synth
from gpu_helpers import assert_parity, oracle_parts

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def reads60k():
    return synth.small_workload(seed=21, n_reads=60_000, genome_len=1_000_000)


@pytest.mark.parametrize("chunk,pieces", [(256 << 10, 8), (8 << 20, 3)])
def test_pieces_tiled_u64(gpu, orc, reads60k, chunk, pieces):
    st = assert_parity(gpu, orc, reads60k, 31, True, 16, chunk_size=chunk)
    assert st["input_pieces"] == pieces and st["staged_scatter"] == 1
    assert st["tiles_per_bucket"] > 1 and st["split_levels"] == 1


def test_pieces_tiled_u128(gpu, orc, reads60k):
    st = assert_parity(gpu, orc, reads60k, 47, True, 4, chunk_size=1 << 20)
    assert st["input_pieces"] == 8 and st["tiles_per_bucket"] > 1


def test_pieces_two_split_levels(gpu, orc, reads60k):
    # a low tile fill: more than 1024 tiles per bucket, so the pieces are read
    # by the first of two split levels
    st = assert_parity(gpu, orc, reads60k, 25, False, 2, chunk_size=1 << 20, tile_fill=0.05)
    assert st["input_pieces"] == 8 and st["split_levels"] == 2


def test_pieces_one_tile_per_bucket(gpu, orc):
    fq = synth.small_workload(seed=22, n_reads=2000, genome_len=20_000)
    st = assert_parity(gpu, orc, fq, 21, True, 256, chunk_size=16 << 10)
    assert st["input_pieces"] == 8 and st["tiles_per_bucket"] == 1


def test_pieces_staging_over_capacity(gpu, orc):
    # empty quality lines: more k-mers than half a key per FASTQ byte, so the
    # staged keys overflow; the pieces' scatters stand down and the keys are
    # scattered from the FASTQ in bucket order
    rng = np.random.default_rng(5)
    acgt = np.frombuffer(b"ACGT", dtype=np.uint8)
    fq = b"".join(b"@\n" + acgt[rng.integers(0, 4, 200)].tobytes() + b"\n+\n\n" for _ in range(2000))
    st = assert_parity(gpu, orc, fq, 21, True, 16, chunk_size=64 << 10)
    assert st["staged_scatter"] == 0 and st["input_pieces"] == 1


def test_device_submissions_have_no_pieces(gpu, orc, reads60k):
    torch = pytest.importorskip("torch")
    chunk = 1 << 20
    # device chunks start on 16-byte boundaries
    layout = ingest.split_chunks(reads60k, chunk)
    offs, at = [], 0
    for _, l in layout:
        offs.append(at)
        at = (at + l + 15) & ~15
    host = bytearray(at)
    for (o, l), d in zip(layout, offs):
        host[d:d + l] = reads60k[o:o + l]
    dev = torch.frombuffer(host, dtype=torch.uint8).cuda()
    base = dev.data_ptr()
    with gpu.Counter(31, True, 16) as c:
        for (_, l), d in zip(layout, offs):
            c.submit_device(base + d, l)
        out = c.finish()
        st = c.stats()
    assert st["input_pieces"] == 1
    parts, _, _ = oracle_parts(orc, reads60k, 31, True, 16, chunk)
    got = {m["partition_id"]: payload for m, payload in out}
    assert sorted(got) == sorted(parts)
    assert all(got[p] == payload for p, (_, payload) in parts.items())
