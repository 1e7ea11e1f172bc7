"""The CUDA path against the oracle on the benchmark configurations' own
shapes and sizes (or slices of them large enough to reach the same kernel
paths): byte-identical .kite files through the command line, dump TSV
identity, and byte-identical partition payloads through the C ABI.

  C1  200,000 x 150 bp forward reads of a 1 Mbp genome, 0.5% subs, k=21
      non-canonical, 16 partitions: the whole configuration.
  C2  1,000,000 reads of the 10M-read workload (gzip FASTQ), k=31 canonical,
      --min 2 --max 1000000, 256 partitions; the same reads in 8 partitions
      (two split levels) and at tile loads that make tiles above the on-chip
      capacity.
  C4  200,000 x 250 bp reads of the skewed genome, k=63 canonical (u128),
      with sampled, learned and automatic splitters.
  C5  8 databases of 200,000-400,000 reads each of the 10M-read workload's
      shape, merged.
  C3  16 metagenome samples counted as one batch, every sample against the
      oracle's count of that sample alone.

Integer work: the bar is byte equality."""
import ctypes
import gzip
import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

from kite_gb300 import CLI, ingest, synth

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent
ORACLE = ROOT / "oracle" / "_build" / "kite_oracle"
THREADS = max(1, os.cpu_count() or 1)


def run(args):
    r = subprocess.run([str(a) for a in args], capture_output=True)
    if r.returncode != 0:
        raise AssertionError(f"{args[0]} {args[1]} failed ({r.returncode}): {r.stderr.decode()[-2000:]}")
    return r


def gpu_parts(gpu, fastq, k, canonical, P, chunk=64 << 20, **kw):
    """Partition payloads and stats of one GPU count through the C ABI."""
    with gpu.Counter(k, canonical, P, **kw) as c:
        for o, l in ingest.split_chunks(fastq, chunk):
            c.submit(memoryview(fastq)[o:o + l])
        out = c.finish()
        st = c.stats()
    return {m["partition_id"]: (m, p) for m, p in out}, st


def assert_same_parts(got: dict, ref, P: int, first: int = 0):
    """got: {partition id: (meta, payload)} (ids first .. first + P); ref: oracle.Parts."""
    want = [p for p in range(P) if ref.rows[p]]
    assert sorted(got) == [first + p for p in want], "non-empty partition sets differ"
    for p in want:
        m, payload = got[first + p]
        assert m["row_count"] == ref.rows[p], f"partition {p} rows"
        assert (m["key_min"], m["key_max"]) == (ref.key_min[p], ref.key_max[p]), f"partition {p} key range"
        assert m["raw_bytes"] == ref.bytes[p] == len(payload)
        assert payload == bytes(ref.payload(p)), f"partition {p} payload differs"


@pytest.fixture(scope="module")
def c2_reads():
    return bytes(synth.repeats_reads(1_000_000, seed=12, genome_seed=2))


@pytest.fixture(scope="module")
def c2_oracle(orc, c2_reads):
    return {P: orc.count_parts(c2_reads, 31, True, P, THREADS) for P in (8, 256)}


def test_c1_full_config_cli(gpu, orc, tmp_path):
    # the whole small configuration: .kite bytes at the reproducible layout
    # (-t 3: one count worker) and `dump -o -` TSV
    fq = tmp_path / "c1.fq"
    fq.write_bytes(synth.small_workload(seed=1, n_reads=200_000, genome_len=1_000_000))
    common = ["-i", fq, "-k", "21", "--canonical", "false", "--partitions", "16", "--memory", "64G", "-t", "3"]
    r = run([CLI, "count", "-o", tmp_path / "g.kite", *common])
    run([ORACLE, "count", "-o", tmp_path / "r.kite", *common])
    assert (tmp_path / "g.kite").read_bytes() == (tmp_path / "r.kite").read_bytes()
    assert b"kmers=26000000 " in r.stderr
    a = run([CLI, "dump", "-i", tmp_path / "g.kite", "-o", "-"]).stdout
    b = run([ORACLE, "dump", "-i", tmp_path / "r.kite", "-o", "-"]).stdout
    assert a == b and a.count(b"\n") > 3_000_000
    # every host thread count gives the same counts (the layout may differ)
    run([CLI, "count", "-o", tmp_path / "t.kite", *common[:-1], str(THREADS)])
    assert run([CLI, "dump", "-i", tmp_path / "t.kite", "-o", "-"]).stdout == b


def test_c2_slice_gzip_cli(gpu, orc, c2_reads, tmp_path):
    # 1M reads of the 10M-read workload from a gzip file, the configuration's
    # flags, 256 partitions
    gz = tmp_path / "c2.fq.gz"
    gz.write_bytes(gzip.compress(c2_reads, compresslevel=1))
    common = ["-i", gz, "-k", "31", "--canonical", "true", "--min", "2", "--max", "1000000",
              "--partitions", "256", "--memory", "64G", "-t", "3"]
    run([CLI, "count", "-o", tmp_path / "g.kite", *common])
    run([ORACLE, "count", "-o", tmp_path / "r.kite", *common])
    assert (tmp_path / "g.kite").read_bytes() == (tmp_path / "r.kite").read_bytes()
    a = run([CLI, "dump", "-i", tmp_path / "g.kite", "-o", "-"]).stdout
    b = run([ORACLE, "dump", "-i", tmp_path / "r.kite", "-o", "-"]).stdout
    assert a == b and len(a) > 0


def test_c2_slice_two_level_split(gpu, c2_reads, c2_oracle):
    # 8 partitions: ~14.5M keys per bucket need more than 1024 tiles, so the
    # key-range split runs in two levels
    got, st = gpu_parts(gpu, c2_reads, 31, True, 8, splitter_mode=gpu.SPLIT_SAMPLED)
    assert st["split_levels"] == 2 and st["tiles_per_bucket"] > 1024
    assert_same_parts(got, c2_oracle[8], 8)
    assert st["kmers"] == c2_oracle[8].kmers


@pytest.mark.parametrize("fill", [0.85, 1.6, 2.6])
def test_c2_slice_oversized_tiles(gpu, c2_reads, c2_oracle, fill):
    # tile loads above the on-chip capacity: 1.6 gives tiles between one and
    # two capacities (the double-capacity on-chip sort), 2.6 tiles above two
    # (LSD through global memory)
    got, st = gpu_parts(gpu, c2_reads, 31, True, 256, splitter_mode=gpu.SPLIT_SAMPLED, tile_fill=fill)
    assert_same_parts(got, c2_oracle[256], 256)
    if fill > 1.0:
        assert st["big_tiles"] > 0


@pytest.fixture(scope="module")
def c4_reads():
    return synth.skewed_workload(seed=14, n_reads=200_000)


@pytest.mark.parametrize("mode", ["sampled", "learned", "auto"])
def test_c4_slice_splitters(gpu, orc, c4_reads, mode):
    ref = orc.count_parts(c4_reads, 63, True, 256, THREADS)
    sm = {"sampled": gpu.SPLIT_SAMPLED, "learned": gpu.SPLIT_LEARNED, "auto": gpu.SPLIT_AUTO}[mode]
    got, st = gpu_parts(gpu, c4_reads, 63, True, 256, splitter_mode=sm)
    assert st["tiles_per_bucket"] > 1
    assert_same_parts(got, ref, 256)
    if mode == "sampled":
        assert st["splitter_used"] == gpu.SPLIT_SAMPLED


def test_c5_merge_eight_databases(gpu, orc, tmp_path):
    # 8 databases counted on the GPU from their own read samples (one genome),
    # then merged by the GPU command line and by the oracle's
    rng = np.random.default_rng(15)
    files = []
    for i, n in enumerate(rng.integers(200_000, 400_001, size=8)):
        fq = tmp_path / f"s{i}.fq"
        fq.write_bytes(synth.repeats_reads(int(n), seed=300 + i, genome_seed=2))
        out = tmp_path / f"s{i}.kite"
        flags = ["--min", "2", "--max", "1000000"] if i % 3 else ["--min", "2"]
        run([CLI, "count", "-i", fq, "-o", out, "-k", "31", "--canonical", "true", "--partitions", "256",
             "--memory", "64G", "-t", str(THREADS), *flags])
        fq.unlink()
        files.append(out)
    run([CLI, "merge", "-i", *files, "-o", tmp_path / "m.kite"])
    run([ORACLE, "merge", "-i", *files, "-o", tmp_path / "r.kite"])
    assert (tmp_path / "m.kite").read_bytes() == (tmp_path / "r.kite").read_bytes()
    a = run([CLI, "dump", "-i", tmp_path / "m.kite", "-o", "-"]).stdout
    b = run([ORACLE, "dump", "-i", tmp_path / "r.kite", "-o", "-"]).stdout
    assert a == b and len(a) > 0


def test_c3_batch_every_sample_vs_oracle(gpu, orc):
    # 16 uneven metagenome samples counted as one batch: the partitions of
    # sample s (ids s*P .. s*P+P-1) against the oracle's count of s alone
    samples = synth.metagenome_samples(seed=16, scale=0.02)
    P = 64
    bufs = [(ctypes.c_char * len(fq)).from_buffer_copy(fq) for fq in samples]
    with gpu.Counter(31, True, P, samples=len(samples), splitter_mode=gpu.SPLIT_SAMPLED) as c:
        for s, fq in enumerate(samples):
            for o, l in ingest.split_chunks(fq, 8 << 20):
                c.submit_sample(s, ctypes.addressof(bufs[s]) + o, l)
        c.synchronize()
        out = c.finish()
        totals = [c.sample_totals(s) for s in range(len(samples))]
    got = {m["partition_id"]: (m, p) for m, p in out}
    for s, fq in enumerate(samples):
        ref = orc.count_parts(fq, 31, True, P, THREADS)
        assert totals[s] == (ref.reads, ref.bases, ref.kmers)
        mine = {pid: v for pid, v in got.items() if s * P <= pid < (s + 1) * P}
        assert_same_parts(mine, ref, P, first=s * P)

