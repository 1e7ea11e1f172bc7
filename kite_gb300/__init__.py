"""kite_gb300 — GB300-native exact k-mer counting (drop-in for Kite's
`kite count` / `kite merge` path and its .kite format).

Native parts (built in-tree by kite_gb300.build):
  _lib/libkite_gpu.so   hand-written sm_103a kernels behind include/kite_gpu.h
  _lib/libkite_host.so  .kite writer/reader, planner, FASTQ ingest
  _lib/kite             the command line (count / merge / dump / info)
"""
from pathlib import Path

__version__ = "0.1.0"
PKG_DIR = Path(__file__).resolve().parent
LIB_DIR = PKG_DIR / "_lib"
CLI = LIB_DIR / "kite"
