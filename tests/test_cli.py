"""The `kite` command line against the oracle's command line on the same
files: byte-identical .kite files (single-worker layout: -t 3), identical
dump TSV, identical merge output, and the reference's argument errors."""
import gzip
import subprocess
from pathlib import Path

import pytest

from kite_gb300 import CLI, synth

ROOT = Path(__file__).resolve().parent.parent
ORACLE = ROOT / "oracle" / "_build" / "kite_oracle"


def run(args, check=True):
    r = subprocess.run([str(a) for a in args], capture_output=True)
    if check and r.returncode != 0:
        raise AssertionError(f"{args[0]} failed ({r.returncode}): {r.stderr.decode()[-2000:]}")
    return r


@pytest.fixture(scope="module")
def fastq(tmp_path_factory, built):
    from test_bgzf import write_bgzf
    d = tmp_path_factory.mktemp("cli")
    fq = synth.small_workload(seed=21, n_reads=8000, genome_len=60_000)
    plain = d / "reads.fq"
    plain.write_bytes(fq)
    gz = d / "reads.fq.gz"
    with gzip.open(gz, "wb", compresslevel=1) as f:
        f.write(fq)
    bgzf = d / "reads.bgzf.fq.gz"
    write_bgzf(bgzf, fq, 30_000)
    return d, plain, gz, bgzf


@pytest.mark.gpu
@pytest.mark.parametrize("args", [
    ["-k", "21", "--partitions", "16"],
    ["-k", "31", "--canonical", "true", "--min", "2", "--max", "1000000"],
    ["-k", "31", "--canonical", "true", "--partitions", "64", "--buffer", "1"],
    ["-k", "55", "--canonical", "true", "--partitions", "32"],
])
@pytest.mark.parametrize("which", ["plain", "gz", "bgzf"])
def test_count_matches_oracle(gpu, orc, fastq, args, which):
    d, plain, gz, bgzf = fastq
    src = {"plain": plain, "gz": gz, "bgzf": bgzf}[which]
    out = d / f"gpu_{which}_{'_'.join(args).replace('-', '')}.kite"
    ref = d / f"ref_{which}_{'_'.join(args).replace('-', '')}.kite"
    common = ["-i", src, "--memory", "64G", "-t", "3", *args]
    r = run([CLI, "count", "-o", out, *common])
    run([ORACLE, "count", "-o", ref, *common])
    assert out.read_bytes() == ref.read_bytes()
    assert b"[kite count] summary reads=8000 " in r.stderr
    a = run([CLI, "dump", "-i", out, "-o", "-"]).stdout
    b = run([ORACLE, "dump", "-i", ref, "-o", "-"]).stdout
    assert a == b and len(a) > 0


@pytest.mark.gpu
def test_merge_matches_oracle(gpu, orc, tmp_path):
    files = []
    for i in range(3):
        fq = tmp_path / f"s{i}.fq"
        fq.write_bytes(synth.small_workload(seed=40 + i, n_reads=3000, genome_len=20_000))
        out = tmp_path / f"s{i}.kite"
        run([CLI, "count", "-i", fq, "-o", out, "-k", "25", "--canonical", "true", "--partitions", "16",
             "--memory", "8G", "-t", "2", "--min", "2"])
        files.append(out)
    run([CLI, "merge", "-i", *files, "-o", tmp_path / "m.kite"])
    run([ORACLE, "merge", "-i", *files, "-o", tmp_path / "r.kite"])
    assert (tmp_path / "m.kite").read_bytes() == (tmp_path / "r.kite").read_bytes()
    assert (tmp_path / "m.merge_report.md").exists()
    info = run([CLI, "info", "-i", tmp_path / "m.kite"]).stdout.decode()
    assert "min\t2" in info and "partitions\t16" in info


@pytest.mark.parametrize("args,msg", [
    (["-k", "0"], "invalid k-mer length"),
    (["-k", "129"], "invalid k-mer length"),
    (["--partitions", "3"], "must be a power of 2"),
    (["--min", "5", "--max", "2"], "--min must be less than or equal to --max"),
    (["-k", "21", "--mode", "tiny"], "possible values: fast, balanced, compact"),
])
def test_count_argument_errors(built, fastq, args, msg):
    d, plain, _, _ = fastq
    r = run([CLI, "count", "-i", plain, "-o", d / "x.kite", *args], check=False)
    assert r.returncode != 0 and msg.encode() in r.stderr


def test_count_output_name_error(built, fastq):
    d, plain, _, _ = fastq
    r = run([CLI, "count", "-i", plain, "-o", d / "x.bin"], check=False)
    assert r.returncode != 0 and b"output must end with .kite" in r.stderr


def test_info_marker_edit(built, orc, tmp_path):
    img, _ = orc.count_kite(synth.small_workload(seed=3, n_reads=500, genome_len=5000), 21, False, 4, min_count=2)
    p = tmp_path / "a.kite"
    p.write_bytes(img)
    run([CLI, "info", "-i", p, "--set-max", "9", "--clear-min"])
    out = run([CLI, "info", "-i", p]).stdout.decode()
    assert "min\tnone" in out and "max\t9" in out
    r = run([CLI, "info", "-i", p, "--set-min", "10"], check=False)
    assert r.returncode != 0 and b"must be <=" in r.stderr


def _zstd_chunks(image: bytes) -> int:
    from kite_gb300.kitefile import KiteImage
    return sum(1 for ch in KiteImage.parse(image).chunks if ch.codec & 4)


@pytest.mark.parametrize("mode", ["balanced", "compact"])
def test_zstd_modes_read_back(built, orc, tmp_path, mode):
    # the oracle's count with zstd "if smaller": the host reader decompresses
    # the zstd chunks and its dump equals the oracle's
    fq = tmp_path / "z.fq"
    fq.write_bytes(synth.small_workload(seed=23, n_reads=30_000, genome_len=200_000))
    out = tmp_path / "z.kite"
    run([ORACLE, "count", "-i", fq, "-o", out, "-k", "25", "--canonical", "true", "--partitions", "4",
         "--memory", "64G", "-t", "3", "--mode", mode])
    image = out.read_bytes()
    assert _zstd_chunks(image) > 0
    from kite_gb300 import host
    assert host.dump_image(image) == orc.dump(image)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["balanced", "compact"])
@pytest.mark.parametrize("k", [21, 31, 45])
def test_zstd_modes_match_oracle(gpu, orc, tmp_path, mode, k):
    # `kite count --mode balanced|compact`: byte-identical .kite files (the
    # same zstd library on both sides), identical dump, and a merge of zstd
    # inputs identical to the oracle's
    fq = tmp_path / "z.fq"
    fq.write_bytes(synth.small_workload(seed=24, n_reads=40_000, genome_len=300_000))
    common = ["-i", fq, "-k", str(k), "--canonical", "true", "--partitions", "8", "--memory", "64G", "-t", "3",
              "--mode", mode]
    run([CLI, "count", "-o", tmp_path / "g.kite", *common])
    run([ORACLE, "count", "-o", tmp_path / "r.kite", *common])
    g = (tmp_path / "g.kite").read_bytes()
    assert g == (tmp_path / "r.kite").read_bytes()
    assert _zstd_chunks(g) > 0
    a = run([CLI, "dump", "-i", tmp_path / "g.kite", "-o", "-"]).stdout
    assert a == run([ORACLE, "dump", "-i", tmp_path / "r.kite", "-o", "-"]).stdout and len(a) > 0
    run([CLI, "count", "-o", tmp_path / "f.kite", *common[:-1], "fast"])
    run([CLI, "merge", "-i", tmp_path / "g.kite", tmp_path / "f.kite", "-o", tmp_path / "m.kite"])
    run([ORACLE, "merge", "-i", tmp_path / "g.kite", tmp_path / "f.kite", "-o", tmp_path / "n.kite"])
    assert (tmp_path / "m.kite").read_bytes() == (tmp_path / "n.kite").read_bytes()
