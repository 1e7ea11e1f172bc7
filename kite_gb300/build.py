"""Builds the native parts of kite_gb300 in-tree.

Outputs (git-ignored, rebuilt on every machine):
  kite_gb300/_lib/libkite_gpu.so   CUDA kernels + C ABI (include/kite_gpu.h), sm_103a only
  kite_gb300/_lib/libkite_host.so  host library: .kite format, writer layout, reader,
                                   planner, FASTQ ingest, synthetic inputs (include/kite_host.h)
  kite_gb300/_lib/kite             the `kite count|merge|dump|info` command line

nvcc cross-compiles sm_103a without a GPU; translation units are compiled in
parallel and only when a source or header is newer than its object.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
HOST = PKG / "host"
INCLUDE = ROOT / "include"
BUILD = PKG / "_build"
LIB = PKG / "_lib"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _newer(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def _have_zlib(cxx: str) -> bool:
    r = subprocess.run([cxx, "-x", "c++", "-E", "-"], input="#include <zlib.h>\n", capture_output=True, text=True)
    return r.returncode == 0


def build(verbose: bool = False, jobs: int | None = None) -> dict:
    BUILD.mkdir(exist_ok=True)
    LIB.mkdir(exist_ok=True)
    nvcc = _nvcc()
    cxx = os.environ.get("CXX", "g++")
    zlib = _have_zlib(cxx)
    cu_headers = sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))
    host_headers = sorted(HOST.glob("*.h")) + sorted(INCLUDE.glob("*.h"))
    jobs = jobs or max(2, min(16, os.cpu_count() or 2))

    steps = []
    gpu_objs = []
    for src in sorted(CSRC.glob("*.cu")):
        obj = BUILD / (src.stem + ".o")
        gpu_objs.append(obj)
        if _newer(obj, [src, *cu_headers, Path(__file__)]):
            steps.append([nvcc, *ARCH, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
                          "-I", str(INCLUDE), "-I", str(CSRC), "-c", str(src), "-o", str(obj)])
    host_objs = []
    for src in sorted(HOST.glob("*.cpp")):
        if src.name == "kite_cli.cpp":
            continue
        obj = BUILD / ("host_" + src.stem + ".o")
        host_objs.append(obj)
        if _newer(obj, [src, *host_headers, Path(__file__)]):
            flags = ["-DKITE_HAVE_ZLIB=1"] if zlib else []
            steps.append([cxx, "-O3", "-std=c++17", "-fPIC", "-Wall", "-Wno-unused-function", *flags,
                          "-I", str(INCLUDE), "-I", str(HOST), "-c", str(src), "-o", str(obj)])
    cli_obj = BUILD / "host_kite_cli.o"
    cli_src = HOST / "kite_cli.cpp"
    if cli_src.exists() and _newer(cli_obj, [cli_src, *host_headers, Path(__file__)]):
        steps.append([cxx, "-O3", "-std=c++17", "-Wall", "-I", str(INCLUDE), "-I", str(HOST),
                      "-c", str(cli_src), "-o", str(cli_obj)])

    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        for fut in [ex.submit(_run, s) for s in steps]:
            fut.result()

    gpu_so = LIB / "libkite_gpu.so"
    if _newer(gpu_so, gpu_objs):
        _run([nvcc, *ARCH, "-shared", "-cudart", "shared", "-o", str(gpu_so), *map(str, gpu_objs)])
    host_so = LIB / "libkite_host.so"
    if host_objs and _newer(host_so, host_objs):
        _run([cxx, "-shared", "-o", str(host_so), *map(str, host_objs), *(["-lz"] if zlib else []), "-lpthread",
              "-ldl"])
    cli = LIB / "kite"
    if cli_src.exists() and _newer(cli, [cli_obj, host_so, gpu_so]):
        _run([cxx, "-o", str(cli), str(cli_obj), f"-L{LIB}", "-lkite_host", "-lkite_gpu",
              f"-Wl,-rpath,$ORIGIN", *(["-lz"] if zlib else []), "-lpthread", "-ldl"])
    if verbose:
        print(f"built {gpu_so}, {host_so}, {cli} (zlib={'yes' if zlib else 'no'})")
    return {"gpu": str(gpu_so), "host": str(host_so), "cli": str(cli), "zlib": zlib}


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
