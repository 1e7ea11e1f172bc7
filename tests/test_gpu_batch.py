"""Batched count (cfg.samples > 1): every sample of a segment is counted by
one launch sequence; each sample's partitions must equal a plain count of
that sample alone (payload bytes, row counts, key ranges, totals)."""
import numpy as np
import pytest

from kite_gb300 import synth

pytestmark = pytest.mark.gpu


def _plain(gpu, fq: bytes, k: int, P: int):
    with gpu.Counter(k, True, P) as c:
        if fq:
            c.submit(fq)
        out = c.finish()
        st = c.stats()
    return {m["partition_id"]: (m, p) for m, p in out}, (st["reads"], st["bases"], st["kmers"])


def _samples():
    rng = np.random.default_rng(21)
    g = synth.genome_iid(rng, 300_000)
    return [
        synth.reads_fixed(rng, g, 6000, 150, 0.005),
        b"",  # an empty sample
        synth.reads_variable(rng, g, 4000, 100, 250, 0.005),
        synth.reads_fixed(rng, synth.genome_iid(rng, 50_000), 9000, 120, 0.01),
    ]


@pytest.mark.parametrize("k,P", [(21, 16), (31, 64), (45, 8)])
def test_batch_matches_plain_counts(gpu, k, P):
    samples = _samples()
    S = len(samples)
    with gpu.Counter(k, True, P, samples=S) as c:
        # queue out of sample order, in several chunks: blocks are grouped by sample
        from kite_gb300 import ingest
        bufs = []
        for s in (2, 0, 3, 1):
            fq = samples[s]
            for o, l in ingest.split_chunks(fq, 200_000):
                b = np.frombuffer(fq[o:o + l], dtype=np.uint8).copy()
                bufs.append(b)
                c.submit_sample(s, b.ctypes.data, len(b))
        out = c.finish()
        totals = [c.sample_totals(s) for s in range(S)]
    got = {m["partition_id"]: (m, p) for m, p in out}
    assert all(0 <= pid < S * P for pid in got)
    for s, fq in enumerate(samples):
        ref, ref_tot = _plain(gpu, fq, k, P)
        assert totals[s] == ref_tot, f"sample {s} totals"
        mine = {pid - s * P: v for pid, v in got.items() if s * P <= pid < (s + 1) * P}
        assert sorted(mine) == sorted(ref), f"sample {s} partitions"
        for p, (m, payload) in ref.items():
            gm, gp = mine[p]
            assert gm["row_count"] == m["row_count"] and gm["key_min"] == m["key_min"] and gm["key_max"] == m["key_max"]
            assert gp == payload, f"sample {s} partition {p}"


def test_batch_sample_index_checked(gpu):
    with gpu.Counter(21, True, 4, samples=2) as c:
        b = np.frombuffer(b"@r\nACGTACGTACGTACGTACGTACGT\n+\nIIIIIIIIIIIIIIIIIIIIIIII\n", dtype=np.uint8).copy()
        with pytest.raises(gpu.KiteGpuError):
            c.submit_sample(2, b.ctypes.data, len(b))
