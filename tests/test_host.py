"""Host-side logic vs the oracle (CPU only): writer layout, planner, memory
specs, count filter, dump, and that both C-ABI libraries export every
symbol their headers declare."""
import ctypes as C
import json
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

from kite_gb300 import host, synth
from kite_gb300.kitefile import KiteImage

ROOT = Path(__file__).resolve().parent.parent
GOLD = json.loads((Path(__file__).parent / "golden" / "reference_vectors.json").read_text())


def _declared(header: str) -> set:
    text = (ROOT / "include" / header).read_text()
    return set(re.findall(r"\b(kite_[a-z0-9_]+)\s*\(", text)) - {"kite_gpu_emit_fn"}


@pytest.mark.parametrize("lib,header", [("libkite_gpu.so", "kite_gpu.h"), ("libkite_host.so", "kite_host.h")])
def test_exports(built, lib, header):
    path = ROOT / "kite_gb300" / "_lib" / lib
    syms = subprocess.run(["nm", "-D", "--defined-only", str(path)], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\sT\s(kite_[a-z0-9_]+)", syms))
    missing = _declared(header) - exported
    assert not missing, f"{lib} lacks {sorted(missing)}"
    C.CDLL(str(path))  # loads without a GPU


def test_memory_spec(built, orc):
    c = GOLD["memory_spec"]
    for spec, val in c["ok"]:
        assert host.parse_memory_spec(spec) == val
    for spec in c["err"]:
        with pytest.raises(ValueError):
            host.parse_memory_spec(spec)


def test_count_filter(built):
    for count, mn, mx, ok in GOLD["count_filter"]["cases"]:
        assert host.count_passes_filter(count, mn, mx) == ok


def test_lanes(built):
    L = host.lib()
    assert [L.kite_suggest_write_lanes(w) for w in (1, 8, 9, 16, 17, 48, 64, 200)] == [2, 2, 2, 2, 3, 6, 6, 6]


@pytest.mark.parametrize("k", [21, 31, 51, 63])
@pytest.mark.parametrize("comp", [0, 1])
def test_planner_matches_oracle(built, orc, k, comp):
    L = orc.lib()
    L.orc_derive_plan.argtypes = [C.c_uint64, C.c_double, C.c_int, C.c_uint, C.c_uint64, C.c_uint64, C.c_uint64,
                                  C.c_longlong, C.c_uint64, C.POINTER(C.c_uint64)]
    rng = np.random.default_rng(k * 7 + comp)
    for _ in range(40):
        inb = int(rng.integers(1 << 20, 1 << 36))
        avg = float(rng.uniform(50, 300))
        parts = int(rng.choice([0, 0, 16, 256, 1024]))
        thr = int(rng.choice([1, 2, 3, 8, 16, 64]))
        mem = int(rng.choice([4, 16, 64, 256])) << 30
        buf = int(rng.choice([-1, -1, 0, 1, 4, 32]))
        out = (C.c_uint64 * 7)()
        rc = L.orc_derive_plan(inb, avg, comp, k, parts, thr, mem, buf, 0, out)
        if rc != 0:
            with pytest.raises(ValueError):
                host.derive_plan(inb, avg, comp, k, parts, thr, mem, buf)
            continue
        p = host.derive_plan(inb, avg, comp, k, parts, thr, mem, buf)
        assert [p["partitions"], p["chunk_size_bytes"], p["staging_bytes"], p["worker_threads"],
                p["local_flush_bytes"], p["decomp_threads"], p["writer_lanes"]] == list(out)


@pytest.mark.parametrize("staging,lanes", [(16 << 20, 2), (4096, 2), (65536, 2), (200_000, 2), (300, 6)])
def test_writer_layout_matches_oracle(built, orc, staging, lanes):
    """Replaying the oracle's single-worker append sequence through the host
    writer reproduces the oracle's .kite bytes, including staging drains."""
    fq = synth.small_workload(seed=4, n_reads=3000, genome_len=40_000)
    img, _ = orc.count_kite(fq, 21, False, 32, staging_bytes=staging, lanes=lanes)
    ki = KiteImage.parse(img)
    w = host.Writer(None, 21, False, 32, 64, 7, staging, lanes)
    for p in range(32):
        for ch in ki.partition_chunks(p):
            w.append({"partition_id": p, "codec": ch.codec, "row_count": ch.row_count, "raw_bytes": ch.raw_bytes,
                      "key_min": ch.key_min, "key_max": ch.key_max}, ki.payload(ch))
    w.worker_drain()
    w.finalize()
    assert w.image() == img


@pytest.mark.parametrize("staging,lanes", [(16 << 20, 1), (4096, 2), (65536, 4), (300, 3)])
def test_writer_file_lanes_match_oracle(built, orc, tmp_path, staging, lanes):
    """The file writer (staged buffers written by positional writes on its
    write lanes while appends go on) produces the oracle's .kite bytes."""
    fq = synth.small_workload(seed=5, n_reads=4000, genome_len=60_000)
    img, _ = orc.count_kite(fq, 21, False, 32, staging_bytes=staging, lanes=lanes)
    ki = KiteImage.parse(img)
    path = tmp_path / "w.kite"
    w = host.Writer(str(path), 21, False, 32, 64, 7, staging, lanes)
    for p in range(32):
        for ch in ki.partition_chunks(p):
            w.append({"partition_id": p, "codec": ch.codec, "row_count": ch.row_count, "raw_bytes": ch.raw_bytes,
                      "key_min": ch.key_min, "key_max": ch.key_max}, ki.payload(ch))
    w.worker_drain()
    w.finalize()
    w.close()
    assert path.read_bytes() == img


def test_dump_matches_oracle(built, orc):
    fq = synth.small_workload(seed=6, n_reads=2000, genome_len=20_000)
    for k, canon, mn, mx in [(21, False, None, None), (31, True, 2, None), (45, True, 2, 10)]:
        img, _ = orc.count_kite(fq, k, canon, 16, min_count=mn, max_count=mx)
        assert host.dump_image(img) == orc.dump(img)


def test_synth_reads_deterministic(built):
    g = synth.genome_iid(np.random.default_rng(1), 10_000)
    a = host.synth_reads(g, 1000, 150, 0.01, 0.001, 0.5, seed=9, threads=1)
    b = host.synth_reads(g, 1000, 150, 0.01, 0.001, 0.5, seed=9, threads=7)
    assert a == b and a.count(b"\n") == 4000
