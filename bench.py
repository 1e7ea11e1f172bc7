#!/usr/bin/env python
"""Benchmark: exact k-mer counting throughput on one GB300 (k-mers/s).

Workload (the 10M-read k=31 configuration): seeded 50 Mbp genome (80% i.i.d.
ACGT, 20% copies of 100 distinct 2 kbp repeat elements at 1% per-copy
divergence), 10,000,000 reads of 150 bp, strand 50/50, 1% substitutions,
0.1% N; k=31 canonical, 256 partitions (the planner's choice for this input),
sampled-histogram splitters.  One step = one full count of the whole input:
FASTQ bytes -> per-partition DVLE payloads of sorted (k-mer, count) rows.

  value  input already resident in HBM (kite_gpu_count_submit_device),
         device time of K steps from CUDA events on the counting stream.
  e2e    the same count through the C ABI from pinned host memory: H2D of
         the FASTQ and D2H of every partition payload inside the timed region.

--impl reference times the CPU restatement of the reference's count (the
oracle port: per-thread hash-bucket workers, sort, RLE, DVLE) on the host
cores on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

K = 31
CANONICAL = True
PARTITIONS = 256
READ_LEN = 150
CHUNK = 64 << 20
METRIC = "exact k-mers/s at k=31 (canonical, 10M x 150 bp reads)"
UNIT = "k-mers/s"


def gen_workload(n_reads: int, seed: int = 2, genome_seed: int | None = None):
    """Reads of the 10M-read workload's shape; the genome comes from
    genome_seed (default: seed), the reads from seed."""
    from kite_gb300 import synth
    return synth.repeats_reads(n_reads, seed=seed, genome_seed=genome_seed)


# --workload skewed: learned vs sampled splitters on skewed u128 keys: 20 Mbp
# genome whose first 30% is an AT-rich Markov chain (P(A)=P(T)=0.4), the rest
# uniform; 4M reads of 250 bp, 1% substitutions; k=63 canonical.
SKEWED = {"k": 63, "reads": 4_000_000, "read_len": 250,
          "metric": "exact k-mers/s at k=63 (canonical, 4M x 250 bp skewed reads)",
          "text": "4,000,000 x 250 bp reads, 20 Mbp genome (first 30% AT-rich Markov chain P(A)=P(T)=0.4, "
                  "rest uniform), 1% subs; k=63 canonical"}


def gen_skewed(n_reads: int, seed: int = 4):
    from kite_gb300 import synth
    return synth.skewed_workload(seed=seed, n_reads=n_reads)


def chunk_layout(data) -> list:
    from kite_gb300 import ingest
    return ingest.split_chunks(data, CHUNK)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict | None:
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in Path(self.path).read_text().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 9:
                rows.append(f)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in rows for n, v in zip(names, r[5:9]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def peaks() -> tuple:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured (MEASURED_PEAKS.json, copy burst)"
    return 6800.0, "fallback"


def stage_bytes(st: dict, fastq_bytes: int, w: int = 8) -> dict:
    """Algorithmic bytes per stage for one step (w = key bytes: 8 for k <= 31,
    16 above): the bytes each stage must read and write at minimum, per the
    kernels that ran."""
    N = st["kmers"]
    d = st["rows"]
    E = st["payload_bytes"]
    staged = st.get("staged_scatter", 0) == 1
    levels = st.get("split_levels", 1)
    return {
        0: ("k_newline_count", fastq_bytes),
        1: ("k_extract<hist>", fastq_bytes + (N * w if staged else 0)),
        2: ("k_bucket_scatter" if staged else "k_extract<scatter>", 2 * N * w if staged else fastq_bytes + N * w),
        3: ("k_split_hist+k_split_scatter", 3 * N * w * levels),
        4: ("k_tile_sort", N * w + d * (w + 4)),
        # tiles above the on-chip capacity: their keys in, their rows out
        5: ("k_big_tile_sort", st.get("big_tile_keys", 0) * w + st.get("big_tile_rows", 0) * (w + 4)),
        6: ("k_encode", d * (w + 4) + E),
    }


def ncu_traffic(kernel_family: str):
    """DRAM bytes per launch of the dominant kernel from the committed ncu
    summary (profiles/ncu_count_kernels.json), scaled to this workload."""
    p = ROOT / "profiles" / "ncu_count_kernels.json"
    if not p.exists():
        return None
    try:
        d = json.loads(p.read_text())
        ent = d["kernels"].get(kernel_family)
        return ent
    except Exception:
        return None


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if os.environ.get("KITE_BENCH_GLOO") is None else "gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def _reduce_device() -> str:
    import torch.distributed as dist
    return "cuda" if dist.get_backend() == "nccl" else "cpu"


def max_over_ranks(world, v: float) -> float:
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device=_reduce_device())
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(world, v: float) -> float:
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device=_reduce_device())
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def cpu_baseline(data, layout, reads_sample: int, threads: int, k: int = K, read_len: int = READ_LEN,
                 partitions: int = PARTITIONS) -> dict:
    """The oracle port of the reference's count (per-thread hash-bucket
    workers, sort, RLE, DVLE, writer) timed on the first reads_sample reads
    (all of them when reads_sample covers the workload)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle
    oracle.lib()
    # the first reads_sample records (fixed-length records)
    rec_len = 11 + 1 + read_len + 1 + 2 + read_len + 1
    n = min(len(data), reads_sample * rec_len)
    sample = bytes(memoryview(data)[:n])
    workers = max(1, threads - 2)  # reader + writer threads as in the reference plan
    r = oracle.count_buffer(sample, k, CANONICAL, partitions, workers)
    secs = r["ns"] / 1e9
    what = "the whole workload" if n == len(data) else "first"
    return {"value": r["kmers"] / secs, "unit": UNIT, "cores": workers, "kind": "port",
            "sample": f"{what} {n // rec_len:,} reads ({n / 1e6:.0f} MB) of the workload, {workers} worker threads",
            "seconds": secs, "kmers": r["kmers"], "full": n == len(data)}


def parity_full(collectors: dict, data, k: int, partitions: int) -> dict:
    """Byte comparison of the GPU's partition payloads with the oracle's
    (orc_count_parts: the single-worker count's payload of every partition,
    made with all host threads) on the whole workload.  collectors maps a
    submission path's name to count_collect(cb), which runs one GPU count
    calling cb(meta, host address, length) per partition.  Runs outside
    every timed region."""
    import ctypes as C
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle
    t0 = time.perf_counter()
    ref = oracle.count_parts(data, k, CANONICAL, partitions, os.cpu_count() or 1)
    t_oracle = time.perf_counter() - t0
    want = set(ref.nonempty())
    out = {"ok": True, "partitions_compared": 0, "rows": int(sum(ref.rows)), "payload_bytes": int(ref.total),
           "kmers": int(ref.kmers), "oracle_seconds": round(t_oracle, 2),
           "method": "GPU partition payloads (DVLE bytes, rows, key range) compared byte for byte with the "
                     "oracle's single-worker count of the whole workload, for each submission path",
           "paths": {}}
    for name, count_collect in collectors.items():
        seen, bad = set(), []

        def cb(m, addr, n):
            p = m["partition_id"]
            seen.add(p)
            same = (m["row_count"] == ref.rows[p] and n == ref.bytes[p] and m["key_min"] == ref.key_min[p]
                    and m["key_max"] == ref.key_max[p])
            if same and n:
                a = np.frombuffer((C.c_uint8 * n).from_address(addr), dtype=np.uint8)
                b = np.frombuffer(ref.payload(p), dtype=np.uint8)
                same = bool(np.array_equal(a, b))
            if not same:
                bad.append(p)

        count_collect(cb)
        ok = not bad and seen == want
        out["ok"] = out["ok"] and ok
        out["partitions_compared"] = max(out["partitions_compared"], len(seen))
        out["paths"][name] = ok
        if not ok:
            out.setdefault("mismatched_partitions", {})[name] = sorted(set(bad) | (seen ^ want))[:20]
    ref.close()
    return out


REF_MAX_STEPS, REF_MAX_WARMUP = 5, 1


def run_reference(args):
    """The oracle port of the reference's count on the host cores, on the
    GPU arm's whole workload (10M reads).  One step is a full count of it
    (several seconds), so at most REF_MAX_STEPS timed steps after at most
    REF_MAX_WARMUP warm-up steps run; the line says how many."""
    world, rank, _ = int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")), 0
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    reads = args.ref_reads or args.reads
    data = gen_workload(reads)
    steps, warmup = min(args.steps, REF_MAX_STEPS), min(args.warmup, REF_MAX_WARMUP)
    vals = []
    for i in range(warmup + steps):
        cb = cpu_baseline(data, None, reads, threads)
        if i >= warmup:
            vals.append(cb)
    v = statistics.median(c["value"] for c in vals)
    ms = statistics.median(c["seconds"] for c in vals) * 1e3
    full = vals[0]["full"] and reads == args.reads
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": steps,
            "warmup": warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u64", "data": "synthetic (seeded)", "impl": "reference",
            "config": {"workload": (f"the GPU arm's workload: {reads:,} x {READ_LEN} bp reads, 50 Mbp genome with "
                                    "20% repeats, 1% subs, 0.1% N, strand 50/50; k=31 canonical")
                       if full else f"same shape as the GPU arm, bounded sample of {reads:,} reads",
                       "reads": reads, "k": K, "canonical": CANONICAL, "partitions": PARTITIONS,
                       "same_config": full},
            "steps_requested": args.steps, "warmup_requested": args.warmup,
            "steps_note": f"one step is a full CPU count of the workload; timed steps capped at {REF_MAX_STEPS}, "
                          f"warm-up at {REF_MAX_WARMUP}",
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": vals[0]["cores"], "kind": "port",
                             "sample": vals[0]["sample"]},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


BATCH_METRIC = "aggregate k-mers/s, 16 metagenome samples counted as one batch (k=31 canonical)"


def run_batch_bench(args, world, rank, local):
    """16 samples of uneven size from a 64-species Zipf(1.2) metagenome
    (300 kbp i.i.d. genomes, reads 100-250 bp, 0.5% substitutions; read
    counts U[0.5M, 8M] x --batch-scale), k=31 canonical, 256 partitions per
    sample.  One step = all 16 samples counted in batched launch sequences (one,
    or --batch-groups G groups of samples at full read counts)
    (cfg.samples = 16) with the autotuned tile fill and scatter shape; the
    same samples counted by 16 sequential plain runs are timed beside it."""
    import torch
    from kite_gb300 import autotune, gpu, ingest, synth
    samples = synth.metagenome_samples(seed=3 + rank, scale=args.batch_scale, fast=True)
    S = len(samples)
    # device-resident copies, every chunk 16-byte aligned with 16 pad bytes
    chunks = []  # (sample, device offset, length)
    pos = 0
    for s, fq in enumerate(samples):
        for o, l in ingest.split_chunks(fq, CHUNK):
            chunks.append((s, o, pos, l))
            pos = (pos + l + 16 + 15) & ~15
    dev = torch.zeros(pos + 64, dtype=torch.uint8, device="cuda")
    for s, o, d, l in chunks:
        dev[d:d + l].copy_(torch.frombuffer(bytearray(samples[s][o:o + l]), dtype=torch.uint8))
    torch.cuda.synchronize()
    base = dev.data_ptr()
    stream = torch.cuda.current_stream()
    fastq_bytes = sum(len(x) for x in samples)

    # samples in --batch-groups contiguous groups, one launch sequence (one
    # finish) per group: at the full read counts the working buffers of all
    # 16 samples at once would not fit in HBM
    G = max(1, min(args.batch_groups, S))
    groups = [range(S * g // G, S * (g + 1) // G) for g in range(G)]

    def batched(c, cb=None):
        for grp in groups:
            for s, o, d, l in chunks:
                if s in grp:
                    c.submit_device(base + d, l, sample=s)
            if cb is None:
                c.finish(collect=False)
            else:
                c.finish(collect=True, callback=cb, raw=True)

    ctxs = {}  # one live context at a time: each holds the batch's working buffers

    def run_once(fill, shape):
        key = (fill, shape)
        if key not in ctxs:
            for old in ctxs.values():
                old.close()
            ctxs.clear()
            torch.cuda.synchronize()
            ctxs[key] = gpu.Counter(K, CANONICAL, PARTITIONS, device=local, splitter_mode=gpu.SPLIT_SAMPLED,
                                    samples=S, tile_fill=fill, scatter_shape=shape, stream=stream.cuda_stream)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        batched(ctxs[key])
        torch.cuda.synchronize()
        return time.perf_counter() - t0

    best, table = autotune.tune(run_once, reps=1)
    for c in ctxs.values():
        c.close()
    ctxs.clear()
    if args.autotune_out:
        autotune.record(args.autotune_out, best, table, "batch of 16 metagenome samples")
    c = gpu.Counter(K, CANONICAL, PARTITIONS, device=local, splitter_mode=gpu.SPLIT_SAMPLED, samples=S,
                    tile_fill=best["tile_fill"], scatter_shape=best["scatter_shape"], stream=stream.cuda_stream)
    for _ in range(args.warmup):
        batched(c)
    torch.cuda.synchronize()
    barrier(world)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    launches = 0
    for _ in range(args.steps):
        batched(c)
        launches += c.stats()["kernel_launches"]
    e1.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    ms = max_over_ranks(world, e0.elapsed_time(e1)) / args.steps
    per_sample = []
    kmers = 0
    # with --batch-parity, every sample's partitions (one more untimed pass)
    # against the oracle's count of that sample alone
    parity = None
    if args.batch_parity and rank == 0:
        import ctypes as Cc
        sys.path.insert(0, str(ROOT / "oracle"))
        import oracle
        got = {}

        def keep(m, addr, n):
            got[m["partition_id"]] = (m, bytes((Cc.c_uint8 * n).from_address(addr)) if n else b"")
        batched(c, keep)
        bad = []
        t0 = time.perf_counter()
        for s_ in range(S):
            ref = oracle.count_parts(samples[s_], K, CANONICAL, PARTITIONS, os.cpu_count() or 1)
            for p in range(PARTITIONS):
                g_ = got.get(s_ * PARTITIONS + p)
                if ref.rows[p] == 0:
                    if g_ is not None:
                        bad.append((s_, p))
                    continue
                if (g_ is None or g_[0]["row_count"] != ref.rows[p] or g_[0]["key_min"] != ref.key_min[p]
                        or g_[0]["key_max"] != ref.key_max[p] or g_[1] != bytes(ref.payload(p))):
                    bad.append((s_, p))
            ref.close()
        got.clear()
        parity = {"ok": not bad, "samples": S, "mismatched": bad[:10],
                  "oracle_seconds": round(time.perf_counter() - t0, 1),
                  "method": "every sample's partitions from the batched count compared byte for byte with the "
                            "oracle's single-worker count of that sample alone"}
    # per-sample totals of every group's finish
    for grp in groups:
        for s_, o, d, l in chunks:
            if s_ in grp:
                c.submit_device(base + d, l, sample=s_)
        c.finish(collect=False)
        for s_ in grp:
            per_sample.append(c.sample_totals(s_))
            kmers += per_sample[-1][2]
    c.close()
    # 16 sequential plain runs of the same samples (one context, one finish each)
    cp = gpu.Counter(K, CANONICAL, PARTITIONS, device=local, splitter_mode=gpu.SPLIT_SAMPLED,
                     tile_fill=best["tile_fill"], scatter_shape=best["scatter_shape"], stream=stream.cuda_stream)

    def sequential():
        for s in range(S):
            for t, o, d, l in chunks:
                if t == s:
                    cp.submit_device(base + d, l)
            cp.finish(collect=False)

    sequential()
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.steps):
        sequential()
    e1.record(stream)
    torch.cuda.synchronize()
    ms_seq = max_over_ranks(world, e0.elapsed_time(e1)) / args.steps
    cp.close()
    value = sum_over_ranks(world, kmers) / (ms / 1e3)
    if rank == 0:
        line = {"metric": BATCH_METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "u64", "data": "synthetic (seeded)",
                "config": {"workload": "16 samples of a 64-species Zipf(1.2) metagenome (300 kbp genomes), reads "
                                       f"100-250 bp, 0.5% subs, read counts U[0.5M, 8M] x {args.batch_scale}; "
                                       "k=31 canonical; 256 partitions per sample",
                           "samples": S, "fastq_bytes": fastq_bytes, "kmers_per_step": kmers,
                           "kmers_per_sample": [t[2] for t in per_sample],
                           "l2": "inputs larger than L2", "parallelism": f"replicas x{world}"},
                "sequential_plain": {"value": sum_over_ranks(world, kmers) / (ms_seq / 1e3), "unit": UNIT,
                                     "ms_per_step": ms_seq},
                "batched_over_sequential": ms_seq / ms, "groups": G, "parity": parity,
                "autotune": {"chosen": best, "table": table},
                "gpu_launches": launches}
        print(json.dumps(line))
    return 0


MERGE_METRIC = "merged input rows/s (8 .kite databases, k=31 canonical, 256 partitions)"


def run_merge_bench(args, world, rank, local):
    """8 .kite databases, each counted (on this GPU) from its own seeded
    sample of the 10M-read workload's shape with 2M-10M reads, merged by
    kite_gpu_merge: inputs in pinned host memory, outputs read in place.  One
    step = one full merge (H2D, decode, k-way merge with exact u32 summation,
    encode, D2H)."""
    import torch
    from kite_gb300 import gpu, host
    from kite_gb300.kitefile import KiteImage
    rng = np.random.default_rng(5)
    reads = [max(1000, int(x * args.merge_scale)) for x in rng.integers(2_000_000, 10_000_001, size=8)]
    images = []
    for i, nr in enumerate(reads):
        data = gen_workload(nr, seed=100 + i + 8 * rank, genome_seed=2)  # one genome, own reads
        layout = chunk_layout(data)
        pinned = torch.frombuffer(bytearray(data), dtype=torch.uint8).pin_memory()
        base = pinned.data_ptr()
        w = host.Writer(None, K, CANONICAL, PARTITIONS, 64, 7, 16 << 20, 2)
        with gpu.Counter(K, CANONICAL, PARTITIONS, device=local, arena_bytes=len(data) + (64 << 20)) as c:
            for o, l in layout:
                c.submit((base + o, l))
            for m, p in c.finish():
                w.append(m, p)
        w.finalize()
        images.append(w.image())
        w.close()
        del pinned, data
    kis = [KiteImage.parse(img) for img in images]
    pins = []
    for img in images:
        t = torch.empty(len(img), dtype=torch.uint8).pin_memory()
        t.numpy()[:] = np.frombuffer(img, dtype=np.uint8)
        pins.append(t)
    bases = [t.data_ptr() for t in pins]
    rows_in = sum(ki.total_rows for ki in kis)
    bytes_in = sum(len(img) for img in images)
    out_stats = {"rows": 0, "bytes": 0}

    def cb(meta, addr, n):
        out_stats["rows"] += meta["row_count"]
        out_stats["bytes"] += n

    c = gpu.Counter(K, CANONICAL, PARTITIONS, device=local)
    for _ in range(args.warmup):
        out_stats["rows"] = out_stats["bytes"] = 0
        c.merge(kis, callback=cb, bases=bases)
    torch.cuda.synchronize()
    barrier(world)
    stage = [0.0] * 10
    t0 = time.perf_counter()
    for _ in range(args.steps):
        out_stats["rows"] = out_stats["bytes"] = 0
        c.merge(kis, callback=cb, bases=bases)
        stage = [x + y for x, y in zip(stage, c.stats()["stage_ms"][:10])]
    c.synchronize()
    barrier(world)
    dt = max_over_ranks(world, (time.perf_counter() - t0) / args.steps)
    mst = c.stats()
    c.close()
    stage = [x / args.steps for x in stage]
    names = ["decode", "tile planning", "merge", "encode", "copy to host", "copy in (overlapped by the decode)",
             "planning: splitters (host wall)", "planning: first cut (host wall)", "planning: bisection (host wall)",
             "planning: tile lists (host wall)"]
    # algorithmic bytes per device stage: decode reads the payloads and
    # writes (key, u64 count) rows; the merge reads those and writes (key,
    # u32 count) rows; the encode reads those and writes the output payloads
    sbytes = {0: bytes_in + rows_in * 16, 2: rows_in * 16 + out_stats["rows"] * 12,
              3: out_stats["rows"] * 12 + out_stats["bytes"]}
    dom = max(sbytes, key=lambda i: stage[i])
    dev_ms = sum(stage[:4])
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        sys.path.insert(0, str(ROOT / "oracle"))
        import oracle
        r = oracle.merge_images(images, os.cpu_count() or 1)
        cpu = {"value": r["rows_in"] / r["seconds"], "unit": "rows/s", "cores": os.cpu_count() or 1, "kind": "port",
               "sample": "the same 8 images in memory: per partition load_partition_counts, the input filters, "
                         "merge_vectors_total and serialize_partition_chunk, partitions on all host threads",
               "seconds": round(r["seconds"], 3)}
    value = sum_over_ranks(world, rows_in) / dt
    peak, peak_src = peaks()
    algo = rows_in * 12 + out_stats["rows"] * 12  # decoded rows in + merged rows out, (key, count) as 8+4 B
    if rank == 0:
        line = {"metric": MERGE_METRIC, "value": value, "unit": "rows/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "u64", "data": "synthetic (seeded)",
                "config": {"workload": "8 .kite databases, each counted from its own seeded read sample "
                                       f"({min(reads):,}-{max(reads):,} reads) of the 10M-read workload's genome "
                                       "and read shape; k=31 canonical; "
                                       "256 partitions; merge with exact u32 summation",
                           "reads_per_db": reads, "rows_in": rows_in, "rows_out": out_stats["rows"],
                           "input_bytes": bytes_in, "output_bytes": out_stats["bytes"],
                           "parallelism": f"replicas x{world}"},
                "e2e": {"value": value, "unit": "rows/s", "h2d_bytes_per_step": bytes_in,
                        "d2h_bytes_per_step": out_stats["bytes"]},
                "device": {"value": rows_in / (dev_ms / 1e3), "unit": "rows/s", "ms_per_step": dev_ms,
                           "note": "the device stages only (decode, tile planning, merge, encode); the whole "
                                   "call adds the copies of the inputs in and the output out"},
                "stage_ms": {names[i]: round(stage[i], 3) for i in range(10)},
                "splitter_used": "learned" if mst["splitter_used"] == gpu.SPLIT_LEARNED else "sampled",
                "roofline": {"bound": "hbm", "kernel": names[dom],
                             "achieved": sbytes[dom] / (stage[dom] / 1e3) / 1e9, "peak": peak, "unit": "GB/s",
                             "frac": sbytes[dom] / (stage[dom] / 1e3) / 1e9 / peak, "traffic": None,
                             "peak_source": peak_src, "algorithmic_bytes": sbytes[dom], "kernel_ms": stage[dom],
                             "whole_call_gbs": algo / dt / 1e9},
                "cpu_baseline": cpu}
        print(json.dumps(line))
    return 0


INGEST_METRIC = "host ingest: decompressed FASTQ GB/s of the BGZF reader (parallel inflate)"


def _bgzf_bytes(data: bytes, block: int = 65280, level: int = 1) -> bytes:
    """BGZF members (gzip with the BC extra subfield) of 65,280-byte blocks."""
    import struct
    import zlib
    out = []
    for o in range(0, len(data), block):
        piece = data[o:o + block]
        co = zlib.compressobj(level, zlib.DEFLATED, -15)
        comp = co.compress(piece) + co.flush()
        head = struct.pack("<BBBBIBBHBBHH", 0x1F, 0x8B, 8, 4, 0, 0, 0xFF, 6, 0x42, 0x43, 2, 18 + len(comp) + 7)
        out.append(head + comp + struct.pack("<II", zlib.crc32(piece) & 0xFFFFFFFF, len(piece)))
    return b"".join(out)


def _gzip_members(data, piece: int = 64 << 20, level: int = 1) -> bytes:
    """Multi-member gzip of data (pieces compressed on all host threads; the
    readers decode it as one stream, as MultiGzDecoder does)."""
    import concurrent.futures as cf
    import gzip as gz
    mv = memoryview(data)
    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 1) as ex:
        parts = list(ex.map(lambda o: gz.compress(bytes(mv[o:o + piece]), compresslevel=level, mtime=0),
                            range(0, len(data), piece)))
    return b"".join(parts)


def _bgzf_parallel(data, block: int = 65280) -> bytes:
    import concurrent.futures as cf
    mv = memoryview(data)
    step = block * 512
    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 1) as ex:
        parts = list(ex.map(lambda o: _bgzf_bytes(bytes(mv[o:o + step]), block), range(0, len(data), step)))
    return b"".join(parts)


def e2e_cli_leg(data, local: int, partitions: int) -> dict:
    """The drop-in command end to end on this workload as configured: wall
    time of `kite count` (GPU) from a gzip file and from a BGZF copy of the
    same reads, including inflate, context setup and the .kite write,
    against the oracle's command line (the CPU restatement, all host cores)
    on the gzip file, and the serial gzip reader's own ceiling."""
    from kite_gb300 import CLI, host
    tmp = Path(tempfile.mkdtemp(prefix="kite_e2e_"))
    gzf, bgzf = tmp / "r.fq.gz", tmp / "r.bgzf.fq.gz"
    gzf.write_bytes(_gzip_members(data))
    bgzf.write_bytes(_bgzf_parallel(data))
    cores = os.cpu_count() or 1
    flags = ["-k", str(K), "--canonical", "true", "--min", "2", "--max", "1000000", "--partitions", str(partitions),
             "--memory", "64G", "-t", str(cores)]

    def timed(cmd):
        t0 = time.perf_counter()
        r = subprocess.run([str(c) for c in cmd], capture_output=True, text=True)
        dt = time.perf_counter() - t0
        if r.returncode != 0:
            raise RuntimeError(r.stderr[-2000:])
        return int(r.stderr.split("kmers=")[1].split()[0]), dt

    out = {}
    for name, path in (("gzip", gzf), ("bgzf", bgzf)):
        timed([CLI, "count", "-i", path, "-o", tmp / "g.kite", *flags, "--device", str(local)])  # warm file cache
        kmers, dt = timed([CLI, "count", "-i", path, "-o", tmp / "g.kite", *flags, "--device", str(local)])
        out[name] = {"kmers_per_s": kmers / dt, "seconds": round(dt, 3)}
    orc = ROOT / "oracle" / "_build" / "kite_oracle"
    kmers, dt = timed([orc, "count", "-i", gzf, "-o", tmp / "r.kite", *flags, "--workers", str(max(1, cores - 2))])
    out["oracle_cli_gzip"] = {"kmers_per_s": kmers / dt, "seconds": round(dt, 3), "cores": cores,
                              "kind": "port"}
    t0 = time.perf_counter()
    n = sum(host.read_chunks(gzf, 64 << 20, 1, collect=False))
    gz_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    nm = sum(host.read_chunks(gzf, 64 << 20, cores, collect=False))
    gm_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    nb = sum(host.read_chunks(bgzf, 64 << 20, cores, collect=False))
    bg_s = time.perf_counter() - t0
    # serial gzip: the reference's reader; the same file's members on every
    # host thread: this command's reader
    out["reader_ceiling"] = {"gzip_serial_gbs": round(n / gz_s / 1e9, 3), "gzip_kmers_per_s": kmers / gz_s,
                             "gzip_members_parallel_gbs": round(nm / gm_s / 1e9, 3),
                             "bgzf_gbs": round(nb / bg_s / 1e9, 3), "bgzf_kmers_per_s": kmers / bg_s,
                             "threads": cores}
    out["files"] = {"fastq_bytes": len(data), "gzip_bytes": gzf.stat().st_size, "bgzf_bytes": bgzf.stat().st_size,
                    "gzip": "multi-member gzip, level 1, 64 MiB members (kite count inflates the members in parallel; "
                            "a single-member file reads serially)", "bgzf": "65,280-byte blocks, level 1"}
    out["flags"] = " ".join(flags)
    for p in (gzf, bgzf, tmp / "g.kite", tmp / "r.kite"):
        if p.exists():
            p.unlink()
    tmp.rmdir()
    return out


def run_ingest_bench(args, world, rank, local):
    """Host ingest (the reader that feeds pinned buffers): decompressed GB/s of
    the BGZF reader at 1..N inflate threads against the serial gzip reader on
    the same reads, and the `kite count` command line end to end (file to
    .kite) on gzip and BGZF copies of the same FASTQ."""
    import gzip as gz
    from kite_gb300 import CLI, host
    if rank != 0:
        return 0
    n_reads = min(args.reads, 2_000_000)
    data = bytes(gen_workload(n_reads, seed=2))
    tmp = Path(tempfile.mkdtemp(prefix="kite_ingest_"))
    plain, gzf, bgzf = tmp / "r.fq", tmp / "r.fq.gz", tmp / "r.bgzf.fq.gz"
    plain.write_bytes(data)
    with gz.open(gzf, "wb", compresslevel=1) as f:
        f.write(data)
    bgzf.write_bytes(_bgzf_bytes(data))
    chunk = 64 << 20
    cores = os.cpu_count() or 1

    def reader_gbs(path, threads):
        best = 0.0
        for _ in range(max(1, args.steps)):
            t0 = time.perf_counter()
            n = sum(host.read_chunks(path, chunk, threads, collect=False))
            best = max(best, n / (time.perf_counter() - t0) / 1e9)
            assert n == len(data)
        return best

    gz_gbs = reader_gbs(gzf, 1)
    plain_gbs = reader_gbs(plain, 1)
    per_threads = {t: reader_gbs(bgzf, t) for t in sorted({1, 2, 4, 8, max(1, cores // 2), cores})}
    best_t = max(per_threads, key=per_threads.get)

    def cli_count(path):
        out = tmp / "o.kite"
        t0 = time.perf_counter()
        r = subprocess.run([str(CLI), "count", "-i", str(path), "-o", str(out), "-k", "31", "--canonical", "true",
                            "--partitions", str(PARTITIONS), "--memory", "64G", "--device", str(local)],
                           capture_output=True, text=True)
        dt = time.perf_counter() - t0
        if r.returncode != 0:
            raise RuntimeError(r.stderr[-2000:])
        kmers = int(r.stderr.split("kmers=")[1].split()[0])
        return kmers / dt, dt
    cli = {name: cli_count(p) for name, p in (("gzip", gzf), ("bgzf", bgzf), ("plain", plain))}
    line = {"metric": INGEST_METRIC, "value": per_threads[best_t], "unit": "GB/s", "n_gpus": world,
            "steps": args.steps, "warmup": 0, "ms_per_step": len(data) / per_threads[best_t] / 1e6,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8",
            "data": "synthetic (seeded)",
            "config": {"workload": f"{n_reads:,} reads of the 10M-read workload's shape ({len(data) / 1e9:.2f} GB "
                                   "FASTQ) as plain, gzip (level 1) and BGZF (65,280-byte blocks, level 1); "
                                   "64 MiB chunks", "host_cores": cores, "best_threads": best_t,
                       "parallelism": "host threads"},
            "bgzf_gbs_by_threads": {str(k): round(v, 3) for k, v in per_threads.items()},
            "gzip_serial_gbs": round(gz_gbs, 3), "plain_gbs": round(plain_gbs, 3),
            "cli_count_kmers_per_s": {k: v[0] for k, v in cli.items()},
            "cli_count_seconds": {k: round(v[1], 3) for k, v in cli.items()},
            "cpu_baseline": {"value": gz_gbs, "unit": "GB/s", "cores": 1, "kind": "port",
                             "sample": "the serial gzip reader (zlib gzread) on the same reads"}}
    print(json.dumps(line))
    for p in (plain, gzf, bgzf, tmp / "o.kite"):
        if p.exists():
            p.unlink()
    tmp.rmdir()
    return 0


DUMP_METRIC = "dump TSV lines/s (kite dump -o - of the 10M-read k=31 count)"


def run_dump_bench(args, world, rank, local):
    """kite dump of the 10M-read count's .kite image (counted once on this
    GPU, written in memory by the host writer): one step = one
    kite_gpu_dump call from the image in pinned host memory to the TSV of
    every partition in host memory (H2D, decode, per-partition merge with
    saturating sums, header filter, TSV formatting, D2H)."""
    import torch
    from kite_gb300 import gpu, host
    from kite_gb300.kitefile import KiteImage
    data = gen_workload(args.reads, seed=2 + rank)
    layout = chunk_layout(data)
    pinned = torch.frombuffer(bytearray(data), dtype=torch.uint8).pin_memory()
    base = pinned.data_ptr()
    w = host.Writer(None, K, CANONICAL, PARTITIONS, 64, 7, 16 << 20, 2, 2, 1_000_000)
    with gpu.Counter(K, CANONICAL, PARTITIONS, device=local, arena_bytes=len(data) + (64 << 20)) as c:
        for o, l in layout:
            c.submit((base + o, l))
        for m, p in c.finish():
            w.append(m, p)
    w.finalize()
    image = w.image()
    w.close()
    del pinned, data
    ki = KiteImage.parse(image)
    pin = torch.empty(len(image), dtype=torch.uint8).pin_memory()
    pin.numpy()[:] = np.frombuffer(image, dtype=np.uint8)
    out = {"lines": 0, "bytes": 0}

    def cb(meta, addr, n):
        out["lines"] += meta["row_count"]
        out["bytes"] += n

    c = gpu.Counter(K, CANONICAL, PARTITIONS, device=local)
    for _ in range(args.warmup):
        out["lines"] = out["bytes"] = 0
        c.dump(ki, callback=cb, base=pin.data_ptr())
    torch.cuda.synchronize()
    barrier(world)
    stage = [0.0] * 5
    launches = 0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        out["lines"] = out["bytes"] = 0
        c.dump(ki, callback=cb, base=pin.data_ptr())
        st = c.stats()
        launches += st["kernel_launches"]
        stage = [a + b for a, b in zip(stage, st["stage_ms"][:5])]
    c.synchronize()
    barrier(world)
    dt = max_over_ranks(world, (time.perf_counter() - t0) / args.steps)
    c.close()
    stage = [x / args.steps for x in stage]
    lines, tsv = out["lines"], out["bytes"]
    rows_in, payload = ki.total_rows, sum(ch.encoded_bytes for ch in ki.chunks)
    dev_ms = sum(stage[:4])
    value = sum_over_ranks(world, lines) / (dev_ms / 1e3)
    e2e = sum_over_ranks(world, lines) / dt
    # algorithmic bytes per stage: decode reads the payload and writes (key,
    # u64 count) rows; the merge reads those and writes (key, u32 count); the
    # formatting reads (key, count) and writes the TSV
    names = ["k_seg_decode", "tile planning", "k_merge_tiles<dump>", "k_tsv_tiles", "copy to host"]
    algo = {0: payload + rows_in * 16, 2: rows_in * 16 + lines * 12, 3: lines * 12 + tsv}
    dom = max(algo, key=lambda i: stage[i])
    peak, peak_src = peaks()
    achieved = algo[dom] / (stage[dom] / 1e3) / 1e9
    # kite histo and a batch of kite query lookups on the same image
    c = gpu.Counter(K, CANONICAL, PARTITIONS, device=local)
    c.histo(ki, base=pin.data_ptr())
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    hist = c.histo(ki, base=pin.data_ptr())
    histo_s = time.perf_counter() - t0
    hst = c.stats()
    rng = np.random.default_rng(7)
    present = np.array([ch.key_min for ch in ki.chunks] + [ch.key_max for ch in ki.chunks], dtype=np.uint64)
    qkeys = np.concatenate([np.tile(present, 500_000 // max(1, len(present))),
                            rng.integers(0, 2 ** 62, size=500_000, dtype=np.uint64)])
    c.query(ki, qkeys[:1000], base=pin.data_ptr())
    t0 = time.perf_counter()
    qc = c.query(ki, qkeys, base=pin.data_ptr())
    query_s = time.perf_counter() - t0
    c.close()
    tables = {"histo": {"rows_per_s": rows_in / histo_s, "seconds": histo_s, "bins": len(hist),
                        "stage_ms": {names[i]: round(hst["stage_ms"][i], 3) for i in range(3)}},
              "query": {"keys": len(qkeys), "keys_per_s": len(qkeys) / query_s, "seconds": query_s,
                        "found": sum(1 for x in qc if x)}}
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        sys.path.insert(0, str(ROOT / "oracle"))
        import oracle
        oracle.lib()
        # bounded sample: the image of a 1M-read count of the same workload
        sdata = bytes(gen_workload(1_000_000, seed=2))
        simg, _ = oracle.count_kite(sdata, K, CANONICAL, PARTITIONS, min_count=2, max_count=1_000_000)
        t1 = time.perf_counter()
        tsv_s = oracle.dump(simg)
        secs = time.perf_counter() - t1
        cpu = {"value": tsv_s.count(b"\n") / secs, "unit": "lines/s", "cores": 1, "kind": "port",
               "sample": "oracle dump of the .kite image of a 1M-read count of the same workload (1 thread)",
               "seconds": secs}
        import ctypes as C
        L = oracle.lib()
        L.orc_histo_kite.restype = C.c_longlong
        L.orc_histo_kite.argtypes = [C.c_char_p, C.c_size_t, C.c_void_p, C.c_void_p, C.c_size_t]
        t1 = time.perf_counter()
        L.orc_histo_kite(simg, len(simg), None, None, 0)
        hs = time.perf_counter() - t1
        tables["histo"]["cpu_baseline"] = {"rows_per_s": KiteImage.parse(simg).total_rows / hs, "seconds": hs,
                                           "sample": "oracle histo of the same 1M-read image (1 thread)"}
    if rank == 0:
        line = {"metric": DUMP_METRIC, "value": value, "unit": "lines/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": dev_ms, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "u64", "data": "synthetic (seeded)",
                "config": {"workload": f"kite dump of the .kite image of the {args.reads:,}-read count (k=31 "
                                       "canonical, 256 partitions, header min 2 / max 1,000,000)",
                           "rows_in": rows_in, "lines_out": lines, "image_bytes": len(image), "tsv_bytes": tsv,
                           "l2": "inputs larger than L2", "parallelism": f"replicas x{world}"},
                "e2e": {"value": e2e, "unit": "lines/s", "h2d_bytes_per_step": len(image), "d2h_bytes_per_step": tsv,
                        "ms_per_step": dt * 1e3},
                "gpu_launches": launches,
                "roofline": {"bound": "hbm", "kernel": names[dom], "achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": achieved / peak, "traffic": None, "peak_source": peak_src,
                             "algorithmic_bytes": algo[dom], "kernel_ms": stage[dom],
                             "stage_ms": {names[i]: round(stage[i], 3) for i in range(5)}},
                "cpu_baseline": cpu, "histo_query": tables}
        print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--reads", type=int, default=10_000_000)
    ap.add_argument("--ref-reads", type=int, default=0,
                    help="reads of the CPU baseline and the reference arm (0 = the whole workload)")
    ap.add_argument("--no-parity", action="store_true", help="skip the full-size comparison with the oracle")
    ap.add_argument("--no-cli", action="store_true", help="skip the command-line leg (gzip / BGZF files)")
    ap.add_argument("--batch-groups", type=int, default=1,
                    help="samples counted in this many launch sequences (one finish each)")
    ap.add_argument("--batch-parity", action="store_true",
                    help="compare every sample of the batch with the oracle (untimed)")
    ap.add_argument("--partitions", type=int, default=PARTITIONS)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-splitter-compare", action="store_true")
    ap.add_argument("--workload", default="repeats",
                    choices=["repeats", "skewed", "merge", "batch", "dump", "ingest"])
    ap.add_argument("--batch-scale", type=float, default=0.25, help="read-count scale of the batch samples")
    ap.add_argument("--autotune-out", default=None, help="write the batch autotuner's table here (JSON)")
    ap.add_argument("--merge-scale", type=float, default=1.0, help="read-count scale of the merge databases")
    ap.add_argument("--scatter-shape", type=int, default=0, choices=[0, 1, 2, 3],
                    help="key-range split scatter launch shape (0 = by digit count)")
    ap.add_argument("--tile-fill", type=float, default=0.0,
                    help="target tile load / on-chip capacity (0 = the library default)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)

    world, rank, local = dist_setup()
    import torch
    torch.cuda.set_device(local)
    from kite_gb300 import gpu
    if args.workload == "merge":
        return run_merge_bench(args, world, rank, local)
    if args.workload == "dump":
        return run_dump_bench(args, world, rank, local)
    if args.workload == "ingest":
        return run_ingest_bench(args, world, rank, local)
    if args.workload == "batch":
        return run_batch_bench(args, world, rank, local)

    skewed = args.workload == "skewed"
    kk = SKEWED["k"] if skewed else K
    metric = SKEWED["metric"] if skewed else METRIC
    if skewed and args.reads == 10_000_000:
        args.reads = SKEWED["reads"]
    if skewed:
        data = gen_skewed(args.reads, seed=4 + rank)
    else:
        data = gen_workload(args.reads, seed=2 + rank)  # each rank counts its own replica (weak scaling)
    layout = chunk_layout(data)
    total = len(data)
    # device-resident copy, every chunk at a 16-byte aligned offset, 16 pad bytes after each
    offs = []
    pos = 0
    for o, l in layout:
        offs.append(pos)
        pos = (pos + l + 16 + 15) & ~15
    dev = torch.zeros(pos + 64, dtype=torch.uint8, device="cuda")
    host_t = torch.frombuffer(data, dtype=torch.uint8)
    for (o, l), d in zip(layout, offs):
        dev[d:d + l].copy_(host_t[o:o + l])
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    base = dev.data_ptr()

    def device_step(c):
        for (o, l), d in zip(layout, offs):
            c.submit_device(base + d, l)
        c.finish(collect=False)

    c = gpu.Counter(kk, CANONICAL, args.partitions, device=local, splitter_mode=gpu.SPLIT_SAMPLED,
                    stream=stream.cuda_stream, scatter_shape=args.scatter_shape, tile_fill=args.tile_fill)
    for _ in range(args.warmup):
        device_step(c)
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    barrier(world)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    stage_sum = [0.0] * 12
    e0.record(stream)
    launches = 0
    for _ in range(args.steps):
        device_step(c)
        st = c.stats()
        launches += st["kernel_launches"]
        for i in range(12):
            stage_sum[i] += st["stage_ms"][i]
    e1.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    clk = clocks.stop()
    ms_total = e0.elapsed_time(e1)
    ms_total = max_over_ranks(world, ms_total)
    kmers = st["kmers"]
    value = sum_over_ranks(world, kmers * args.steps) / (ms_total / 1e3)

    # ---- roofline of the dominant kernel ----
    stages = stage_bytes(st, total, 8 if kk <= 31 else 16)
    avg_ms = {i: stage_sum[i] / args.steps for i in stages}
    dom = max(stages, key=lambda i: avg_ms[i])
    name, algo_bytes = stages[dom]
    peak, peak_src = peaks()
    achieved = algo_bytes / (avg_ms[dom] / 1e3) / 1e9
    tr = ncu_traffic(name)
    traffic = None
    try:
        traffic_src = json.loads((ROOT / "profiles" / "ncu_count_kernels.json").read_text())["source"] + \
            ", DRAM bytes per k-mer scaled to this step"
    except Exception:
        traffic_src = None
    if tr and tr.get("dram_bytes_per_key") is not None:
        # ncu DRAM bytes per k-mer from the committed 1M-read capture, scaled
        # to this step's k-mers (the split's figure is per level)
        traffic = tr["dram_bytes_per_key"] * kmers * (st.get("split_levels", 1) if tr.get("per_level") else 1)
    sort_ms = avg_ms[3] + avg_ms[4] + avg_ms[5]
    sort_bytes = stages[3][1] + stages[4][1]
    # the bytes a least-significant-digit radix sort with 16-bit digits would
    # move over the same keys (a histogram read of N·w, then a read and a
    # write of N·w per pass, p = ceil(2k / 16) passes) plus the run-length
    # pass (read N·w, write d·(w + 4)): the sort expressed as effective
    # bandwidth against the multi-pass method, over the measured split +
    # tile sort time
    w_key = 8 if kk <= 31 else 16
    p16 = -(-2 * kk // 16)
    lsd16_bytes = st["kmers"] * w_key * (1 + 2 * p16) + st["kmers"] * w_key + st["rows"] * (w_key + 4)
    roofline = {"bound": "hbm", "kernel": name, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic, "peak_source": peak_src,
                "traffic_source": traffic_src,
                "algorithmic_bytes": algo_bytes, "kernel_ms": avg_ms[dom],
                "sort_gbs": sort_bytes / (sort_ms / 1e3) / 1e9 if sort_ms > 0 else None,
                "sort_frac": (sort_bytes / (sort_ms / 1e3) / 1e9) / peak if sort_ms > 0 else None,
                "sort_lsd16_bytes": lsd16_bytes,
                "sort_lsd16_gbs": lsd16_bytes / (sort_ms / 1e3) / 1e9 if sort_ms > 0 else None,
                "sort_lsd16_frac": (lsd16_bytes / (sort_ms / 1e3) / 1e9) / peak if sort_ms > 0 else None,
                "stage_ms": {stages[i][0]: round(avg_ms[i], 4) for i in stages}}

    # ---- learned vs sampled splitters on the same input (identical output) ----
    splitters = None
    if not args.no_splitter_compare:
        cl = gpu.Counter(kk, CANONICAL, args.partitions, device=local, splitter_mode=gpu.SPLIT_LEARNED,
                         stream=stream.cuda_stream)
        device_step(cl)
        torch.cuda.synchronize()

        def timed_step(cc):
            a0 = torch.cuda.Event(enable_timing=True)
            a1 = torch.cuda.Event(enable_timing=True)
            a0.record(stream)
            device_step(cc)
            a1.record(stream)
            torch.cuda.synchronize()
            return a0.elapsed_time(a1) / 1e3

        # the same clock for both: CUDA events around one step each, three
        # interleaved steps per method, median
        t_s, t_l = [], []
        for _ in range(3):
            t_s.append(timed_step(c))
            sms = c.stats()["stage_ms"]
            t_l.append(timed_step(cl))
        ts, tl = statistics.median(t_s), statistics.median(t_l)
        stl = cl.stats()
        sml = stl["stage_ms"]
        cl.close()
        splitters = {"timing": "CUDA events around one device-resident step, median of 3 interleaved steps each",
                     "sampled": {"kmers_per_s": kmers / ts, "tile_imbalance": st["tile_imbalance"],
                                 "range_imbalance": st["range_imbalance"],
                                 "big_tiles": st["big_tiles"],
                                 "stage_ms": {stages[i][0]: round(sms[i], 3) for i in stages}},
                     "learned": {"kmers_per_s": kmers / tl, "tile_imbalance": stl["tile_imbalance"],
                                 "range_imbalance": stl["range_imbalance"], "model_reused": stl["mlp_reused"] == 1,
                                 "big_tiles": stl["big_tiles"], "mlp_loss": stl["mlp_loss"],
                                 "predicted_imbalance": stl["mlp_pred_imbalance"],
                                 "used": stl["splitter_used"] == gpu.SPLIT_LEARNED,
                                 "stage_ms": {stages[i][0]: round(sml[i], 3) for i in stages}}}

    # ---- e2e counter: the C ABI from pinned host memory ----
    pinned = torch.empty(total, dtype=torch.uint8).pin_memory()
    pinned.copy_(host_t)
    pbase = pinned.data_ptr()
    d2h = [0]
    ce = gpu.Counter(kk, CANONICAL, args.partitions, device=local, splitter_mode=gpu.SPLIT_SAMPLED,
                     scatter_shape=args.scatter_shape, tile_fill=args.tile_fill)

    # ---- the whole workload's output against the oracle (untimed), from
    # device-resident chunks and from the pinned host chunks ----
    parity = None
    if rank == 0 and not args.no_parity:
        def count_collect(cb):
            for (o, l), d in zip(layout, offs):
                c.submit_device(base + d, l)
            c.finish(collect=True, callback=cb, raw=True)
            torch.cuda.synchronize()

        def host_collect(cb):
            for o, l in layout:
                ce.submit((pbase + o, l))
            ce.finish(collect=True, callback=cb, raw=True)
            ce.synchronize()
        parity = parity_full({"device_chunks": count_collect, "host_chunks": host_collect}, data, kk,
                             args.partitions)

    e2e_parts = {"submit_s": 0.0, "finish_s": 0.0, "d2h_ms": 0.0, "stage_ms": [0.0] * 12}
    e2e_pieces = [0]

    def e2e_step(cc):
        t_a = time.perf_counter()
        for o, l in layout:
            cc.submit((pbase + o, l))
        t_b = time.perf_counter()
        e2e_parts["submit_s"] += t_b - t_a
        out_bytes = 0

        def cb(pid, addr, n):
            nonlocal out_bytes
            out_bytes += n
        cc.finish(collect=True, callback=cb, raw=True, meta=False)
        e2e_parts["finish_s"] += time.perf_counter() - t_b
        est = cc.stats()
        sm = est["stage_ms"]
        e2e_pieces[0] = est["input_pieces"]
        e2e_parts["d2h_ms"] += sm[7]
        e2e_parts["stage_ms"] = [a + b for a, b in zip(e2e_parts["stage_ms"], sm)]
        d2h[0] = out_bytes

    e2e_step(ce)
    ce.synchronize()
    for key in e2e_parts:
        e2e_parts[key] = [0.0] * 12 if key == "stage_ms" else 0.0
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step(ce)
    ce.synchronize()
    barrier(world)
    te = max_over_ranks(world, time.perf_counter() - t0)
    e2e_val = sum_over_ranks(world, kmers * args.steps) / te
    ce.close()
    c.close()

    cli = None
    if rank == 0 and world == 1 and not args.no_cli and not skewed:
        cli = e2e_cli_leg(data, local, args.partitions)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cb = cpu_baseline(data, layout, args.ref_reads or args.reads, os.cpu_count() or 1, kk,
                          SKEWED["read_len"] if skewed else READ_LEN, args.partitions)
        cpu = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")}

    if rank == 0:
        line = {"metric": metric, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_total / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "u128" if kk > 31 else "u64",
                "data": "synthetic (seeded)",
                "config": {"workload": (SKEWED["text"] if skewed else
                                        f"{args.reads:,} x {READ_LEN} bp reads, 50 Mbp genome with 20% repeats, "
                                        f"1% subs, 0.1% N, strand 50/50; k={K} canonical") +
                                       f"; {args.partitions} partitions; "
                                       "sampled-histogram splitters",
                           "reads": args.reads, "k": kk, "canonical": CANONICAL, "partitions": args.partitions,
                           "fastq_bytes": total, "kmers_per_step": kmers, "rows_per_step": st["rows"],
                           "payload_bytes_per_step": st["payload_bytes"],
                           "l2": "inputs larger than L2 (FASTQ and keys are GBs; no flush needed)",
                           "parallelism": f"replicas x{world}"},
                "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": total, "d2h_bytes_per_step": d2h[0],
                        "ms_per_step": te / args.steps * 1e3,
                        "submit_ms": e2e_parts["submit_s"] / args.steps * 1e3,
                        "finish_ms": e2e_parts["finish_s"] / args.steps * 1e3,
                        "d2h_ms": e2e_parts["d2h_ms"] / args.steps,
                        "input_pieces": e2e_pieces[0],
                        # device stages of the end-to-end count (the first two include waiting for the
                        # copies; with input pieces the bucket scatter runs inside the histogram stage)
                        "stage_ms": {stages[i][0]: round(e2e_parts["stage_ms"][i] / args.steps, 3) for i in stages},
                        # host wall time of the finish call's phases
                        "host_ms": {name: round(e2e_parts["stage_ms"][i] / args.steps, 3) for i, name in
                                    ((8, "copy in, extraction, bucket scatter"), (9, "split, sort, encode"),
                                     (10, "last payload copies"), (11, "emit calls"))}},
                "gpu_launches": launches, "roofline": roofline, "cpu_baseline": cpu, "clocks": clk,
                "parity": parity, "e2e_cli": cli,
                "splitters": splitters,
                "tiles": {"tiles": st["tiles"], "per_bucket": st["tiles_per_bucket"], "big": st["big_tiles"],
                          "imbalance": st["tile_imbalance"], "sort_fallbacks": st["sort_fallbacks"]}}
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
