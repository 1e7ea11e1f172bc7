"""GPU `kite histo` and `kite query` against the oracle's restatements of
run_histo / run_query on the same .kite images: identical count -> frequency
tables (u64 sums of a partition's chunks, header filter on the sum, counts
above the on-chip bins and above u32::MAX) and identical u64 counts for
present and absent keys; the command lines' outputs byte for byte."""
import ctypes as C
import subprocess

import numpy as np
import pytest

from kite_gb300 import CLI, synth
from kite_gb300.kitefile import KiteImage
from kite_build import build_image, bucket

pytestmark = pytest.mark.gpu


def orc_histo(orc, img: bytes) -> dict:
    L = orc.lib()
    L.orc_histo_kite.restype = C.c_longlong
    L.orc_histo_kite.argtypes = [C.c_char_p, C.c_size_t, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), C.c_size_t]
    cap = 1 << 20
    a, b = (C.c_uint64 * cap)(), (C.c_uint64 * cap)()
    n = L.orc_histo_kite(img, len(img), a, b, cap)
    assert n >= 0, orc.err()
    return {int(a[i]): int(b[i]) for i in range(n)}


def orc_query(orc, img: bytes, keys: list) -> list:
    L = orc.lib()
    L.orc_query_kite.argtypes = [C.c_char_p, C.c_size_t, C.POINTER(C.c_uint64), C.c_size_t, C.POINTER(C.c_uint64)]
    arr = (C.c_uint64 * (2 * max(1, len(keys))))()
    for i, k in enumerate(keys):
        arr[2 * i], arr[2 * i + 1] = k & (2 ** 64 - 1), k >> 64
    out = (C.c_uint64 * max(1, len(keys)))()
    assert L.orc_query_kite(img, len(img), arr, len(keys), out) == 0, orc.err()
    return [int(out[i]) for i in range(len(keys))]


def gpu_histo(gpu, img):
    ki = KiteImage.parse(img)
    with gpu.Counter(ki.k, bool(ki.canonical), ki.partitions) as c:
        return c.histo(ki)


def gpu_query(gpu, img, keys):
    ki = KiteImage.parse(img)
    with gpu.Counter(ki.k, bool(ki.canonical), ki.partitions) as c:
        return c.query(ki, keys)


@pytest.mark.parametrize("k,canonical,flt", [(21, False, (None, None)), (31, True, (2, 40)), (63, True, (None, 5)),
                                             (64, False, (3, None))])
def test_histo_and_query_of_counts(gpu, orc, k, canonical, flt):
    fq = synth.small_workload(seed=80 + k, n_reads=4000, genome_len=15_000)
    img, _ = orc.count_kite(fq, k, canonical, 16, min_count=flt[0], max_count=flt[1])
    assert gpu_histo(gpu, img) == orc_histo(orc, img)
    ki = KiteImage.parse(img)
    rng = np.random.default_rng(k)
    present = []
    for ch in ki.chunks[:6]:
        present.append(ch.key_min)
        present.append(ch.key_max)
    absent = [int(x) for x in rng.integers(0, 2 ** 62, size=20, dtype=np.uint64)]
    keys = present + absent
    assert gpu_query(gpu, img, keys) == orc_query(orc, img, keys)
    assert all(c > 0 for c in gpu_query(gpu, img, present))


def test_histo_large_counts_and_multichunk(gpu, orc):
    # overlapping chunks summed in u64 (two u32-max counts exceed u32), counts
    # above the 1024 on-chip bins, RAW chunks, and the header max on the sum
    P = 8
    rng = np.random.default_rng(4)
    keys = sorted({int(x) for x in rng.integers(0, 1 << 40, size=4000)})
    parts = {}
    for key in keys:
        parts.setdefault(bucket(key, P, False), []).append(key)
    chunks = []
    for p, ks in sorted(parts.items()):
        for j in range(3):
            sel = ks[j::2] if j < 2 else ks[::3]
            rows = [(x, int(rng.choice([1, 2, 7, 1500, 70000, 0xFFFFFFFF]))) for x in sel]
            chunks.append((p, rows, 1 if j == 2 else 2))
    for mx in (None, 100000):
        img = build_image(25, True, P, chunks, max_count=mx)
        h = gpu_histo(gpu, img)
        assert h == orc_histo(orc, img)
        assert any(c > 0xFFFFFFFF for c in h) == (mx is None)
        assert gpu_query(gpu, img, keys[:300]) == orc_query(orc, img, keys[:300])


def run(args, check=True):
    r = subprocess.run([str(a) for a in args], capture_output=True)
    if check and r.returncode != 0:
        raise AssertionError(f"{args[0]} failed ({r.returncode}): {r.stderr.decode()[-2000:]}")
    return r


def test_cli_histo_and_query(gpu, orc, tmp_path):
    from pathlib import Path
    oracle_cli = Path(orc.__file__).resolve().parent / "_build" / "kite_oracle"
    files = []
    for i, (mn, mx) in enumerate(((None, None), (2, None), (None, 3))):
        fq = synth.small_workload(seed=90 + i, n_reads=3000, genome_len=12_000)
        img, _ = orc.count_kite(fq, 25, True, 16, min_count=mn, max_count=mx)
        f = tmp_path / f"s{i}.kite"
        f.write_bytes(img)
        files.append(f)
    run([CLI, "histo", "-i", *files, "-o", tmp_path / "g.tsv"])
    run([oracle_cli, "histo", "-i", *files, "-o", tmp_path / "o.tsv"])
    got = (tmp_path / "g.tsv").read_bytes()
    assert got == (tmp_path / "o.tsv").read_bytes() and got.startswith(b"count\ts0\ts1\ts2\n")
    run([CLI, "histo", "-i", *files, "-o", tmp_path / "gl.tsv", "--label", "a", "b", "c"])
    assert (tmp_path / "gl.tsv").read_bytes().startswith(b"count\ta\tb\tc\n")
    ki = KiteImage.parse(files[2].read_bytes())
    seq = "".join("ACGT"[(ki.chunks[0].key_min >> (2 * (24 - i))) & 3] for i in range(25))
    for q in (seq, seq.lower(), "A" * 25, "ACGT" * 6 + "C"):
        for f in (files[0], files[2]):
            a = run([CLI, "query", "-i", f, "-k", q]).stdout
            b = run([oracle_cli, "query", "-i", f, "-k", q]).stdout
            assert a == b and a.startswith(b"Kite Query\n")
    r = run([CLI, "query", "-i", files[0], "-k", "ACGT"], check=False)
    assert r.returncode != 0 and b"query k-mer length 4 does not match database k=25" in r.stderr
    r = run([CLI, "query", "-i", files[0], "-k", "N" * 25], check=False)
    assert r.returncode != 0 and b"query k-mer contains non-ACGT characters" in r.stderr


def test_histo_query_dump_of_segmented_u128_count(gpu, orc):
    # k=45 (u128 keys) counted in several segments (small arena): partitions
    # hold several chunks; histo, query and dump all sum them
    from kite_gb300 import host, ingest
    fq = synth.small_workload(seed=14, n_reads=5000, genome_len=25_000)
    w = host.Writer(None, 45, True, 8, 128, 7, 16 << 20, 2, None, 6)
    with gpu.Counter(45, True, 8, arena_bytes=256 * 1024) as c:
        for o, l in ingest.split_chunks(fq, 100_000):
            try:
                c.submit(fq[o:o + l])
            except gpu.KiteGpuError as e:
                assert e.code == -9
                for m, p in c.finish():
                    w.append(m, p)
                c.submit(fq[o:o + l])
        for m, p in c.finish():
            w.append(m, p)
    w.worker_drain()
    w.finalize()
    img = w.image()
    w.close()
    ki = KiteImage.parse(img)
    assert max(ki.part_count) >= 2
    assert gpu_histo(gpu, img) == orc_histo(orc, img)
    keys = [ch.key_min for ch in ki.chunks] + [ch.key_max for ch in ki.chunks] + [12345, 2 ** 80 + 7]
    assert gpu_query(gpu, img, keys) == orc_query(orc, img, keys)
    with gpu.Counter(45, True, 8) as c:
        assert c.dump(ki) == orc.dump(img)


def test_histo_query_empty(gpu, orc):
    img = build_image(21, False, 16, [])
    assert gpu_histo(gpu, img) == {} == orc_histo(orc, img)
    assert gpu_query(gpu, img, [0, 5, 2 ** 40]) == [0, 0, 0]
    assert gpu_query(gpu, img, []) == []
