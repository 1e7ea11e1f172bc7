"""kite_gpu_count_rows_noalloc (the count entry point that allocates nothing)
against the context entry point (kite_gpu_count_submit + finish) on the same
chunk: rows must be identical (integer work, no tolerance), on two calls in a
row, with the second call on a different chunk as well.  Collected last so it
also runs after every other GPU test in the same process."""
import ctypes as C

import numpy as np
import pytest

from kite_gb300 import synth

MAX_BYTES = 512 * 1024
KITE_ERR_BAD_INPUT = -4
KITE_ERR_UNSUPPORTED = -6


def _fn(gpu):
    L = gpu.lib()
    f = L.kite_gpu_count_rows_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_int, C.c_int, C.c_int, C.c_uint32, C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p,
                  C.c_uint64, C.c_void_p, C.POINTER(C.c_uint64), C.c_void_p, C.c_uint32]
    return f


def _uleb(buf: bytes, i: int):
    v = s = 0
    while True:
        b = buf[i]
        i += 1
        v |= (b & 0x7F) << s
        s += 7
        if b < 0x80:
            return v, i


def _dvle_rows(payload: bytes, rows: int, wide: bool):
    kb = 16 if wide else 8
    key = int.from_bytes(payload[:kb], "little")
    out = [(key, int.from_bytes(payload[kb:kb + 4], "little"))]
    i = kb + 4
    for _ in range(rows - 1):
        d, i = _uleb(payload, i)
        c, i = _uleb(payload, i)
        key += d
        out.append((key, c))
    assert i == len(payload)
    return out


def context_rows(gpu, fastq: bytes, k: int, canonical: bool, P: int):
    """Rows per partition and totals from the context entry point."""
    with gpu.Counter(k, canonical, P) as c:
        c.submit(fastq)
        out = c.finish()
        st = c.stats()
    parts = {m["partition_id"]: _dvle_rows(payload, m["row_count"], k > 31) for m, payload in out}
    return parts, (st["reads"], st["bases"], st["kmers"], st["rows"])


def noalloc_rows(gpu, fastq: bytes, k: int, canonical: bool, P: int, max_rows: int | None = None):
    import torch
    f = _fn(gpu)
    kb = 16 if k > 31 else 8
    n = len(fastq)
    d_in = torch.frombuffer(bytearray(fastq) or bytearray(1), dtype=torch.uint8).to("cuda")
    cap = max(n, 1) if max_rows is None else max_rows
    d_keys = torch.empty(cap * kb, dtype=torch.uint8, device="cuda")
    d_counts = torch.empty(cap, dtype=torch.int32, device="cuda")
    d_prow = torch.full((P,), -1, dtype=torch.int32, device="cuda")
    totals = (C.c_uint64 * 4)()
    torch.cuda.synchronize()
    rc = f(0, k, 1 if canonical else 0, P, d_in.data_ptr(), n, d_keys.data_ptr(), d_counts.data_ptr(), cap,
           d_prow.data_ptr(), totals, None, 60000)
    tot = tuple(int(x) for x in totals)
    if rc != 0:
        return rc, None, tot
    rows = tot[3]
    words = d_keys.cpu().numpy()[:rows * kb].view(np.uint64).reshape(rows, kb // 8)
    counts = d_counts.cpu().numpy()[:rows].view(np.uint32)
    prow = d_prow.cpu().numpy().view(np.uint32)
    assert int(prow.sum()) == rows
    parts, o = {}, 0
    for p in range(P):
        r = int(prow[p])
        if r:
            if kb == 8:
                keys = [int(x) for x in words[o:o + r, 0]]
            else:
                keys = [int(lo) | (int(hi) << 64) for lo, hi in words[o:o + r]]
            parts[p] = list(zip(keys, (int(c) for c in counts[o:o + r])))
        o += r
    return rc, parts, tot


def _small_reads(seed: int, n_reads: int) -> bytes:
    rng = np.random.default_rng(seed)
    g = synth.genome_iid(rng, 20_000)
    return synth.reads_fixed(rng, g, n_reads, 150, 0.01, n_rate=0.002, revcomp_frac=0.5)


EDGE = (b"@r1\nACGTNacgtACGTACGTTTGACCAGTAGGACCAGGATTTACAGGGCACCCATACGATGACCAGGTTT\n+\n"
        + b"I" * 63 + b"\n@r2\n\n+\n\n@r3\nGGGGGGGGGGGGGGGGGGGGGGGGGGGGGGGGGGGGGGGGGGGGGGGGGGGGGGGGGGGGGGGGGGGGGGGGGG"
        + b"\n+\n" + b"I" * 74 + b"\n@r4\nACGTACGTACGTACGTACGTACGTACGTACGTACGTACGTACGTAC\r\n+\n" + b"I" * 47
        + b"\n@r5\nTTTTACGATCGATCGGGCTAGCTAGCATCGACTACGACTAGCATCAGCATCAGCATTACGACTAGCAGGGT")


CASES = [(21, True, 16), (31, False, 64), (45, True, 8), (64, True, 2), (17, True, 4096)]


@pytest.mark.gpu
@pytest.mark.parametrize("k,canonical,P", CASES)
def test_noalloc_matches_context_twice(gpu, k, canonical, P):
    a = _small_reads(7, 1500)
    b = EDGE
    assert len(a) <= MAX_BYTES
    ref_a = context_rows(gpu, a, k, canonical, P)
    ref_b = context_rows(gpu, b, k, canonical, P)
    for data, (parts, tot) in ((a, ref_a), (a, ref_a), (b, ref_b), (a, ref_a)):
        rc, got, gtot = noalloc_rows(gpu, data, k, canonical, P)
        assert rc == 0
        assert gtot == tot
        assert sorted(got) == sorted(parts)
        for p in parts:
            assert got[p] == parts[p], f"partition {p}"


@pytest.mark.gpu
def test_noalloc_empty_and_ignored_chunks(gpu):
    for data in (b"", b"ACGT\n+\nIIII\n", b"@only-a-header"):
        rc, got, tot = noalloc_rows(gpu, data, 21, True, 8)
        assert rc == 0 and got == {} and tot == (0, 0, 0, 0)


@pytest.mark.gpu
def test_noalloc_limits(gpu):
    import torch
    f = _fn(gpu)
    big = torch.zeros(MAX_BYTES + 1, dtype=torch.uint8, device="cuda")
    out = torch.empty(16, dtype=torch.uint8, device="cuda")
    prow = torch.empty(8, dtype=torch.int32, device="cuda")
    totals = (C.c_uint64 * 4)()
    rc = f(0, 21, 1, 8, big.data_ptr(), MAX_BYTES + 1, out.data_ptr(), out.data_ptr(), 1, prow.data_ptr(), totals,
           None, 60000)
    assert rc == KITE_ERR_UNSUPPORTED
    rc = f(0, 21, 1, 6, big.data_ptr(), 16, out.data_ptr(), out.data_ptr(), 1, prow.data_ptr(), totals, None, 60000)
    assert rc == KITE_ERR_BAD_INPUT  # partitions not a power of two
    data = _small_reads(9, 200)
    parts, tot = context_rows(gpu, data, 25, True, 8)
    rc, _, gtot = noalloc_rows(gpu, data, 25, True, 8, max_rows=10)
    assert rc == KITE_ERR_BAD_INPUT and gtot[3] == tot[3] > 10
    rc, got, gtot = noalloc_rows(gpu, data, 25, True, 8)
    assert rc == 0 and got == parts and gtot == tot


def _densest_cases():
    # 65,536 one-base records of 8 bytes: the most sequences a full chunk of
    # real reads holds, every one a k=1 k-mer
    one_base = b"@\nA\n+\nI\n" * (MAX_BYTES // 8)
    # 87,380 empty records (6 bytes) and one 8-byte record: the most sequence
    # lines a chunk can hold (a record spans four newlines)
    empties = b"@\n\n+\n\n" * 87_380 + b"@\nC\n+\nI\n"
    # one sequence line filling the chunk: the most k-mers (one per byte)
    rng = np.random.default_rng(31)
    seq = bytes(b"ACGT"[x] for x in rng.integers(0, 4, MAX_BYTES - 6))
    single = b"@\n" + seq + b"\n+\n\n"
    # short random reads of 2..9 bases
    recs = []
    n = 0
    while True:
        L = int(rng.integers(2, 10))
        r = b"@\n" + bytes(b"ACGT"[x] for x in rng.integers(0, 4, L)) + b"\n+\n" + b"I" * L + b"\n"
        if n + len(r) > MAX_BYTES - 8:
            break
        recs.append(r)
        n += len(r)
    short = b"".join(recs)
    short += b"@\n" + b"G" * ((MAX_BYTES - len(short) - 6) // 2) + b"\n+\n"
    short += b"I" * (MAX_BYTES - len(short) - 1) + b"\n"
    return {"one_base": one_base, "empties": empties, "single": single, "short": short}


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["one_base", "empties", "single", "short"])
@pytest.mark.parametrize("k,canonical,P", [(1, False, 2), (2, True, 4), (31, True, 64)])
def test_noalloc_full_size_chunks(gpu, name, k, canonical, P):
    # chunks of exactly KITE_NOALLOC_MAX_BYTES that reach the fixed bounds of
    # the scratch layout: the most sequences, the most k-mers, the most rows
    data = _densest_cases()[name]
    assert len(data) == MAX_BYTES
    parts, tot = context_rows(gpu, data, k, canonical, P)
    for _ in range(2):
        rc, got, gtot = noalloc_rows(gpu, data, k, canonical, P)
        assert rc == 0
        assert gtot == tot
        assert sorted(got) == sorted(parts)
        for p in parts:
            assert got[p] == parts[p], f"partition {p}"
