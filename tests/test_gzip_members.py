"""Multi-member gzip input: the members inflate in parallel and are handed
out in order, and the chunks are the serial reader's (the reference's
MultiGzDecoder stream cut by `next_chunk`, src/count/decompress.rs:36-81):
the same bytes and the same chunk lengths as the oracle's reader and as this
reader on one thread, for members of several sizes, false member headers
inside stored data, a corrupt member, bytes after the last member and a
truncated file.  CPU only."""
import ctypes as C
import gzip

import pytest

from kite_gb300 import host, synth


def oracle_chunk_lens(orc, path, chunk_size):
    L = orc.lib()
    L.orc_read_chunks.restype = C.c_int64
    L.orc_read_chunks.argtypes = [C.c_char_p, C.c_size_t, C.POINTER(C.c_uint64), C.c_size_t]
    cap = 1 << 16
    lens = (C.c_uint64 * cap)()
    n = L.orc_read_chunks(str(path).encode(), chunk_size, lens, cap)
    assert n >= 0, orc.err()
    return [int(lens[i]) for i in range(n)]


def members(data: bytes, piece: int, level: int = 1) -> bytes:
    return b"".join(gzip.compress(data[o:o + piece], compresslevel=level, mtime=0)
                    for o in range(0, len(data), piece))


@pytest.fixture(scope="module")
def reads():
    return synth.small_workload(seed=41, n_reads=12_000, genome_len=60_000)


def check(orc, path, data, chunk, threads_list=(1, 4, 16), compare_oracle=True):
    runs = {t: host.read_chunks(path, chunk, t) for t in threads_list}
    ref = runs[threads_list[0]]
    for t, got in runs.items():
        assert [len(c) for c in got] == [len(c) for c in ref], f"threads {t}"
        assert b"".join(got) == b"".join(ref), f"threads {t}"
    if data is not None:
        assert b"".join(ref) == data
    if compare_oracle:
        assert [len(c) for c in ref] == oracle_chunk_lens(orc, path, chunk)
    return ref


@pytest.mark.parametrize("piece", [40_000, 300_000, 1 << 20])
@pytest.mark.parametrize("chunk", [100_000, 1 << 20])
def test_members_match_serial_and_oracle(orc, tmp_path, reads, piece, chunk):
    p = tmp_path / "m.fq.gz"
    p.write_bytes(members(reads, piece))
    check(orc, p, reads, chunk)


def test_false_member_headers_in_stored_data(orc, tmp_path, reads):
    # a quality line holding a gzip member header, in members stored without
    # compression, so the header bytes appear in the file between members
    fake = bytes([0x1F, 0x8B, 0x08, 0x00, 0, 0, 0, 0, 0x04, 0xFF]) * 3
    rec = b"@fake\nACGTACGTAC\n+\n" + fake + b"\n"
    data = reads[:len(reads) // 3] + rec * 50 + reads[len(reads) // 3:]
    cut = data.index(rec) - 1000
    blob = members(data[:cut], 200_000) + members(data[cut:cut + 60_000], 20_000, level=0) + \
        members(data[cut + 60_000:], 200_000)
    p = tmp_path / "f.fq.gz"
    p.write_bytes(blob)
    assert blob.count(fake[:10]) >= 10
    check(orc, p, data, 100_000)


def test_corrupt_member(orc, tmp_path, reads):
    parts = [gzip.compress(reads[o:o + 100_000], compresslevel=1, mtime=0) for o in range(0, len(reads), 100_000)]
    bad = bytearray(parts[3])
    bad[len(bad) // 2] ^= 0xFF
    parts[3] = bytes(bad)
    p = tmp_path / "c.fq.gz"
    p.write_bytes(b"".join(parts))
    # the oracle's chunk reader reports the error instead of the chunks before it
    got = check(orc, p, None, 100_000, compare_oracle=False)
    assert 0 < sum(len(c) for c in got) < len(reads)


def test_bytes_after_last_member(orc, tmp_path, reads):
    p = tmp_path / "t.fq.gz"
    p.write_bytes(members(reads, 150_000) + bytes(64))
    check(orc, p, None, 100_000)


def test_truncated_file(orc, tmp_path, reads):
    blob = members(reads, 150_000)
    p = tmp_path / "x.fq.gz"
    p.write_bytes(blob[:len(blob) - 5000])
    got = check(orc, p, None, 100_000, compare_oracle=False)
    assert sum(len(c) for c in got) < len(reads)


def test_single_member(orc, tmp_path, reads):
    p = tmp_path / "s.fq.gz"
    p.write_bytes(gzip.compress(reads, compresslevel=6, mtime=0))
    check(orc, p, reads, 100_000)
