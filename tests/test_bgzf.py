"""BGZF input (src/count/bgzf.rs): the host reader's chunks match the
oracle's restatement of decompress_bgzf_parallel (block headers scanned,
blocks inflated in parallel, output cut by find_fastq_split_near), the read
length sample matches sample_bgzf_input, and data that is not a BGZF block
yields no chunks.  CPU only."""
import ctypes as C
import struct
import zlib

import pytest

from kite_gb300 import host, synth


def bgzf_block(data: bytes) -> bytes:
    """One BGZF member: gzip header with the BC extra subfield, raw deflate,
    CRC32 and ISIZE (SAM/BAM specification, section 4.1)."""
    co = zlib.compressobj(6, zlib.DEFLATED, -15)
    comp = co.compress(data) + co.flush()
    bsize = 18 + len(comp) + 8 - 1
    head = struct.pack("<BBBBIBBHBBHH", 0x1F, 0x8B, 8, 4, 0, 0, 0xFF, 6, 0x42, 0x43, 2, bsize)
    return head + comp + struct.pack("<II", zlib.crc32(data) & 0xFFFFFFFF, len(data))


def write_bgzf(path, data: bytes, block: int = 65280, eof: bool = True) -> None:
    with open(path, "wb") as f:
        for o in range(0, len(data), block):
            f.write(bgzf_block(data[o:o + block]))
        if eof:
            f.write(bgzf_block(b""))


def oracle_chunk_lens(orc, path, chunk_size):
    L = orc.lib()
    L.orc_read_chunks.restype = C.c_int64
    L.orc_read_chunks.argtypes = [C.c_char_p, C.c_size_t, C.POINTER(C.c_uint64), C.c_size_t]
    cap = 1 << 16
    lens = (C.c_uint64 * cap)()
    n = L.orc_read_chunks(str(path).encode(), chunk_size, lens, cap)
    assert n >= 0, orc.err()
    return [int(lens[i]) for i in range(n)]


@pytest.fixture(scope="module")
def reads():
    return synth.small_workload(seed=31, n_reads=6000, genome_len=40_000)


@pytest.mark.parametrize("chunk_size", [100_000, 262_144, 1 << 20])
@pytest.mark.parametrize("block", [65280, 9000])
@pytest.mark.parametrize("threads", [1, 4, 16])  # 16: every host thread, as `kite count` uses
def test_chunks_match_oracle(orc, tmp_path, reads, chunk_size, block, threads):
    p = tmp_path / "r.fq.gz"
    write_bgzf(p, reads, block)
    got = host.read_chunks(p, chunk_size, threads)
    assert b"".join(got) == reads
    assert [len(c) for c in got] == oracle_chunk_lens(orc, p, chunk_size)
    for c in got[:-1]:
        assert c.count(b"\n") % 4 == 0 and c[:1] == b"@"


def test_detected_and_sampled_like_the_reference(orc, tmp_path, reads):
    p = tmp_path / "r.fq.gz"
    write_bgzf(p, reads, 20_000)
    L = host.lib()
    L.kite_detect_compression.argtypes = [C.c_char_p]
    assert L.kite_detect_compression(str(p).encode()) == 2  # KITE_INPUT_BGZF
    L.kite_sample_avg_read_len.restype = C.c_double
    L.kite_sample_avg_read_len.argtypes = [C.c_char_p, C.c_int]
    O = orc.lib()
    O.orc_sample_avg_read_len.restype = C.c_double
    O.orc_sample_avg_read_len.argtypes = [C.c_char_p]
    a = L.kite_sample_avg_read_len(str(p).encode(), 2)
    assert a == O.orc_sample_avg_read_len(str(p).encode()) and abs(a - 150.0) < 1e-9


def test_truncated_last_block_is_skipped(orc, tmp_path, reads):
    p = tmp_path / "t.fq.gz"
    write_bgzf(p, reads, 30_000, eof=False)
    raw = p.read_bytes()
    p.write_bytes(raw[:-10])  # the last block loses its tail
    got = host.read_chunks(p, 100_000)
    assert [len(c) for c in got] == oracle_chunk_lens(orc, p, 100_000)
    assert reads.startswith(b"".join(got)) and len(b"".join(got)) < len(reads)


def test_non_bgzf_data_yields_no_chunks(orc, tmp_path, reads, capfd):
    p = tmp_path / "bad.fq.gz"
    write_bgzf(p, reads, 30_000)
    p.write_bytes(p.read_bytes() + b"this is not a gzip member at all")
    assert host.read_chunks(p, 100_000) == []
    assert oracle_chunk_lens(orc, p, 100_000) == []
    err = capfd.readouterr().err
    assert "bgzf_decompress_error: Non-BGZF data at offset" in err


@pytest.mark.parametrize("kind", ["plain", "gzip"])
def test_plain_and_gzip_chunks_match_oracle(orc, tmp_path, reads, kind):
    import gzip
    p = tmp_path / ("r.fq" if kind == "plain" else "r.fq.gz")
    if kind == "plain":
        p.write_bytes(reads)
    else:
        with gzip.open(p, "wb", compresslevel=1) as f:
            f.write(reads)
    got = host.read_chunks(p, 100_000)
    assert b"".join(got) == reads
    assert [len(c) for c in got] == oracle_chunk_lens(orc, p, 100_000)


def test_block_with_wrong_isize(orc, tmp_path, reads):
    # a block whose trailer states the wrong output size still yields its
    # bytes (the trailer check fails after the data), as the reference's
    # decoder keeps what it read; the batch is assembled block by block
    raw = bytearray()
    blocks = [bgzf_block(reads[o:o + 30_000]) for o in range(0, len(reads), 30_000)]
    bad = bytearray(blocks[3])
    bad[-4:] = struct.pack("<I", 1234)
    blocks[3] = bytes(bad)
    for b in blocks:
        raw += b
    p = tmp_path / "w.fq.gz"
    p.write_bytes(bytes(raw))
    got = host.read_chunks(p, 100_000, 4)
    assert [len(c) for c in got] == oracle_chunk_lens(orc, p, 100_000)
    assert b"".join(got) == reads
