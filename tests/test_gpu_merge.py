"""GPU merge vs the oracle's restatement of `kite merge`: identical output
images (through the host writer), per-input filters before summing, multi-
chunk and RAW partitions, and the u32 overflow error naming the key."""
import numpy as np
import pytest

from kite_gb300 import host, synth
from kite_gb300.kitefile import KiteImage
from kite_build import build_image, bucket

pytestmark = pytest.mark.gpu


def gpu_merge_image(gpu, images, lanes=2):
    kis = [KiteImage.parse(x) for x in images]
    k0 = kis[0]
    mins = {ki.min_count for ki in kis}
    maxs = {ki.max_count for ki in kis}
    with gpu.Counter(k0.k, bool(k0.canonical), k0.partitions) as c:
        out = c.merge(kis)
    w = host.Writer(None, k0.k, bool(k0.canonical), k0.partitions, k0.key_width, 3, 16 << 20, lanes,
                    mins.pop() if len(mins) == 1 else None, maxs.pop() if len(maxs) == 1 else None)
    for m, payload in out:
        w.append(m, payload)
    w.finalize()
    return w.image()


def oracle_merge_image(orc, tmp_path, images, lanes=2):
    paths = []
    for i, img in enumerate(images):
        p = tmp_path / f"in{i}.kite"
        p.write_bytes(img)
        paths.append(p)
    return orc.merge_files(paths, lanes)


@pytest.mark.parametrize("k,canonical", [(21, False), (31, True), (45, True)])
@pytest.mark.parametrize("nin", [2, 3, 8])
def test_merge_counts(gpu, orc, tmp_path, k, canonical, nin):
    imgs = []
    for i in range(nin):
        fq = synth.small_workload(seed=30 + i, n_reads=1500 + 400 * i, genome_len=30_000)
        img, _ = orc.count_kite(fq, k, canonical, 16)
        imgs.append(img)
    assert gpu_merge_image(gpu, imgs) == oracle_merge_image(orc, tmp_path, imgs)


def test_merge_filters_before_summing(gpu, orc, tmp_path):
    fqs = [synth.small_workload(seed=50 + i, n_reads=3000, genome_len=10_000) for i in range(3)]
    imgs = [orc.count_kite(fqs[0], 21, True, 8, min_count=2)[0],
            orc.count_kite(fqs[1], 21, True, 8, min_count=3, max_count=40)[0],
            orc.count_kite(fqs[2], 21, True, 8)[0]]
    assert gpu_merge_image(gpu, imgs) == oracle_merge_image(orc, tmp_path, imgs)
    same = [orc.count_kite(f, 21, True, 8, min_count=2, max_count=50)[0] for f in fqs]
    a = gpu_merge_image(gpu, same)
    assert a == oracle_merge_image(orc, tmp_path, same)
    ki = KiteImage.parse(a)
    assert ki.min_count == 2 and ki.max_count == 50 and ki.codec_mask == 3


def _rows_by_partition(rng, nkeys, P, wide, maxkey):
    keys = np.unique(rng.integers(0, maxkey, size=nkeys, dtype=np.uint64)).tolist()
    parts = {}
    for key in keys:
        parts.setdefault(bucket(int(key), P, wide), []).append(int(key))
    return parts


@pytest.mark.parametrize("wide", [False, True])
def test_merge_multichunk_and_raw(gpu, orc, tmp_path, wide):
    """Inputs whose partitions hold several chunks with overlapping keys (as
    multi-worker counts write) and RAW chunks."""
    rng = np.random.default_rng(7)
    P = 8
    k = 45 if wide else 25
    imgs = []
    for i in range(3):
        parts = _rows_by_partition(rng, 6000, P, wide, 1 << 40)
        chunks = []
        for p, ks in sorted(parts.items()):
            # three overlapping chunks per partition
            for j in range(3):
                sel = sorted(set(ks[j::2] + ks[::3]))
                rows = [(x, int(rng.integers(1, 9))) for x in sel]
                chunks.append((p, rows, 1 if (i == 1 and j == 2) else 2))
        imgs.append(build_image(k, True, P, chunks, min_count=None if i else 4))
    assert gpu_merge_image(gpu, imgs) == oracle_merge_image(orc, tmp_path, imgs)


def test_merge_overflow_error(gpu, orc, tmp_path):
    P = 4
    big = 3_000_000_000
    a = build_image(21, False, P, [(bucket(100, P, False), [(100, big)], 2), (bucket(7, P, False), [(7, 5)], 2)])
    b = build_image(21, False, P, [(bucket(100, P, False), [(100, big)], 2)])
    with pytest.raises(RuntimeError) as e:
        oracle_merge_image(orc, tmp_path, [a, b])
    with pytest.raises(gpu.KiteGpuError) as g:
        gpu_merge_image(gpu, [a, b])
    assert g.value.code == -5
    assert str(e.value) in str(g.value) and "merged count exceeds u32 for key 100" in str(g.value)


def test_merge_tile_refinement(gpu, orc, tmp_path):
    # many rows in one partition with clustered keys force tile bisection
    P = 2
    rng = np.random.default_rng(3)
    base = [int(x) for x in np.unique(rng.integers(0, 1 << 20, size=30000))]
    chunks_a, chunks_b = {}, {}
    for key in base:
        p = bucket(key, P, False)
        chunks_a.setdefault(p, []).append((key, 1))
        chunks_b.setdefault(p, []).append((key, 2))
    a = build_image(21, False, P, [(p, r, 2) for p, r in sorted(chunks_a.items())])
    b = build_image(21, False, P, [(p, r, 2) for p, r in sorted(chunks_b.items())])
    assert gpu_merge_image(gpu, [a, b]) == oracle_merge_image(orc, tmp_path, [a, b])
