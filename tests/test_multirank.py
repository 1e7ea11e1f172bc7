"""Multi-rank host logic on CPU (gloo, world size 2, launched by torchrun on
127.0.0.1): the bench's timing barrier and its max / sum reductions over
ranks, the reference arm under torchrun (rank 0 alone runs and prints one
line, the other rank exits 0 without work), and the premise of running
replicas with no data-path collective: counting input shards on separate
ranks and merging the shards' databases gives the count of the whole input
(the oracle on both sides)."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def launch(nproc: int, args: list, timeout: int = 600) -> subprocess.CompletedProcess:
    env = dict(os.environ, KITE_ROOT=str(ROOT), KITE_BENCH_GLOO="1", OMP_NUM_THREADS="1")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={nproc}",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()), *map(str, args)]
    return subprocess.run(cmd, capture_output=True, text=True, env=env, timeout=timeout, cwd=ROOT)


def json_lines(text: str) -> list:
    return [json.loads(x) for x in text.splitlines() if x.startswith("{")]


REDUCE = r'''
import json, os, sys
sys.path.insert(0, os.environ["KITE_ROOT"])
import bench
import torch.distributed as dist
world, rank, local = bench.dist_setup()
bench.barrier(world)
out = {"rank": rank, "world": world, "backend": dist.get_backend(),
       "max": bench.max_over_ranks(world, float(rank + 1)), "sum": bench.sum_over_ranks(world, float(rank + 1))}
bench.barrier(world)
with open(os.path.join(sys.argv[1], f"rank{rank}.json"), "w") as f:
    json.dump(out, f)
dist.destroy_process_group()
'''


def test_bench_rank_reductions(tmp_path):
    w = tmp_path / "reduce.py"
    w.write_text(REDUCE)
    r = launch(2, [w, tmp_path])
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [json.loads((tmp_path / f"rank{i}.json").read_text()) for i in range(2)]
    assert sorted(x["rank"] for x in lines) == [0, 1]
    for x in lines:
        assert x["world"] == 2 and x["backend"] == "gloo"
        assert x["max"] == 2.0 and x["sum"] == 3.0


def test_reference_arm_two_ranks(built):
    r = launch(2, ["bench.py", "--impl", "reference", "--gpus", 2, "--reads", 3000, "--steps", 1, "--warmup", 0])
    assert r.returncode == 0, r.stderr[-3000:]
    lines = json_lines(r.stdout)
    assert len(lines) == 1, r.stdout[-2000:]
    line = lines[0]
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"


SHARDS = r'''
import json, os, sys
root = os.environ["KITE_ROOT"]
sys.path.insert(0, root)
sys.path.insert(0, os.path.join(root, "oracle"))
import torch.distributed as dist
import oracle as orc
from kite_gb300 import ingest, synth
dist.init_process_group("gloo")
rank, world = dist.get_rank(), dist.get_world_size()
tmp = sys.argv[1]
fq = bytes(synth.small_workload(seed=31, n_reads=6000, genome_len=80_000))
chunks = ingest.split_chunks(fq, 64 << 10)
# this rank's shard: whole records, every world-th chunk
mine = b"".join(fq[o:o + l] for i, (o, l) in enumerate(chunks) if i % world == rank)
img, (reads, bases, kmers) = orc.count_kite(mine, 21, True, 16)
with open(os.path.join(tmp, f"shard{rank}.kite"), "wb") as f:
    f.write(img)
tot = [None] * world
dist.all_gather_object(tot, (reads, bases, kmers))
dist.barrier()
if rank == 0:
    merged = orc.merge_files([os.path.join(tmp, f"shard{r}.kite") for r in range(world)])
    whole, stats = orc.count_kite(fq, 21, True, 16)
    same = orc.dump(merged) == orc.dump(whole)
    sums = tuple(sum(t[i] for t in tot) for i in range(3))
    print(json.dumps({"chunks": len(chunks), "same_dump": same, "sums": list(sums), "whole": list(stats)}), flush=True)
dist.barrier()
dist.destroy_process_group()
'''


def test_shards_count_then_merge_equals_whole(built, tmp_path):
    w = tmp_path / "shards.py"
    w.write_text(SHARDS)
    r = launch(2, [w, tmp_path])
    assert r.returncode == 0, r.stderr[-3000:]
    lines = json_lines(r.stdout)
    assert len(lines) == 1
    out = lines[0]
    assert out["chunks"] >= 4
    assert out["same_dump"]
    assert out["sums"] == out["whole"]
