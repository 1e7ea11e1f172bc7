"""The host library's threaded parts under ThreadSanitizer (CPU only): the
pipelined BGZF reader, the parallel gzip-member reader (including its fall
back to the serial reader on a corrupt member) and the writer's lanes, built
with -fsanitize=thread into a small driver over the C ABI.  No race report,
and the same bytes at every thread count."""
import gzip
import shutil
import struct
import subprocess
import zlib
from pathlib import Path

import pytest

from kite_gb300 import synth

ROOT = Path(__file__).resolve().parent.parent

DRIVER = r'''
#include "kite_host.h"
#include <cstdio>
#include <vector>
static long read_all(const char* path, unsigned threads) {
  kite_input* in = kite_input_open(path, 100000);
  if (!in) return -1;
  kite_input_set_threads(in, threads);
  const size_t cap = kite_input_max_chunk(in) + 64;
  std::vector<unsigned char> buf(cap);
  long tot = 0;
  for (;;) {
    const long n = (long)kite_input_next(in, buf.data(), cap);
    if (n <= 0) break;
    tot += n;
  }
  kite_input_close(in);
  return tot;
}
int main(int argc, char** argv) {
  for (int f = 1; f + 1 < argc; ++f)
    for (unsigned t : {1u, 4u, 8u}) printf("%s %u %ld\n", argv[f], t, read_all(argv[f], t));
  kite_header_info h{};
  h.k = 21; h.partitions = 32; h.key_width = 64; h.codec_mask = 7;
  kite_writer* w = kite_writer_open(argv[argc - 1], &h, 4096, 3);
  if (!w) return 2;
  std::vector<unsigned char> pay(50000, 7);
  for (int r = 0; r < 20; ++r)
    for (unsigned p = 0; p < 32; ++p) {
      kite_chunk_meta m{};
      m.partition_id = p; m.codec = 1; m.row_count = 10; m.raw_bytes = 1000 + p * 37;
      if (kite_writer_append(w, &m, pay.data(), 1000 + p * 37)) return 3;
    }
  uint64_t c = 0, rows = 0;
  if (kite_writer_worker_drain(w) || kite_writer_finalize(w, &c, &rows)) return 4;
  kite_writer_close(w);
  printf("writer %llu\n", (unsigned long long)c);
  return 0;
}
'''


def bgzf_block(data: bytes) -> bytes:
    co = zlib.compressobj(6, zlib.DEFLATED, -15)
    comp = co.compress(data) + co.flush()
    head = struct.pack("<BBBBIBBHBBHH", 0x1F, 0x8B, 8, 4, 0, 0, 0xFF, 6, 0x42, 0x43, 2, 18 + len(comp) + 8 - 1)
    return head + comp + struct.pack("<II", zlib.crc32(data) & 0xFFFFFFFF, len(data))


def test_threaded_host_parts_under_tsan(tmp_path):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no g++")
    drv = tmp_path / "drv.cpp"
    drv.write_text(DRIVER)
    exe = tmp_path / "drv"
    r = subprocess.run([cxx, "-O1", "-g", "-std=c++17", "-fsanitize=thread", "-DKITE_HAVE_ZLIB=1",
                        "-I", str(ROOT / "include"), "-I", str(ROOT / "kite_gb300" / "host"),
                        str(ROOT / "kite_gb300" / "host" / "kite_host.cpp"), str(drv), "-o", str(exe),
                        "-lz", "-lpthread", "-ldl"], capture_output=True, text=True)
    if r.returncode != 0:
        pytest.skip("no ThreadSanitizer build here: " + r.stderr[-300:])
    reads = synth.small_workload(seed=41, n_reads=30_000, genome_len=60_000)
    b = tmp_path / "b.fq.gz"
    b.write_bytes(b"".join(bgzf_block(reads[o:o + 65280]) for o in range(0, len(reads), 65280)) + bgzf_block(b""))
    m = tmp_path / "m.fq.gz"
    blob = b"".join(gzip.compress(reads[o:o + 200_000], compresslevel=1, mtime=0)
                    for o in range(0, len(reads), 200_000))
    m.write_bytes(blob)
    c = tmp_path / "c.fq.gz"
    bad = bytearray(blob)
    bad[len(bad) // 2] ^= 0xFF
    c.write_bytes(bytes(bad))
    run = subprocess.run([str(exe), str(b), str(m), str(c), str(tmp_path / "w.kite")], capture_output=True,
                         text=True, timeout=600, env={"TSAN_OPTIONS": "halt_on_error=0 exitcode=0"})
    assert "ThreadSanitizer" not in run.stderr, run.stderr[-3000:]
    assert run.returncode == 0, run.stderr[-2000:]
    got = {}
    for line in run.stdout.splitlines():
        parts = line.split()
        if len(parts) == 3:
            got.setdefault(parts[0], set()).add(int(parts[2]))
    assert got[str(b)] == {len(reads)} and got[str(m)] == {len(reads)}
    assert len(got[str(c)]) == 1 and 0 < next(iter(got[str(c)])) < len(reads)
    assert "writer 640" in run.stdout
