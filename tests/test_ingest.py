"""Host-side chunking mirrors the reference reader (CPU)."""
import ctypes as C

import numpy as np

from kite_gb300 import ingest, synth


def test_split_matches_oracle_rule(orc):
    data = synth.small_workload(seed=3, n_reads=2000)
    for cs in (1000, 4096, 7777, 65536, len(data), len(data) + 1):
        chunks = ingest.split_chunks(data, cs)
        assert chunks[0][0] == 0 and sum(l for _, l in chunks) == len(data)
        for (o, l), (o2, _) in zip(chunks, chunks[1:]):
            assert o + l == o2
        for o, l in chunks[:-1]:
            # every non-final chunk ends after a 4k-th newline of itself
            assert data[o:o + l].count(b"\n") % 4 == 0
            assert orc.lib().orc_find_fastq_split(data[o:o + l], l) == l


def test_split_reference_vectors():
    d = b"@READ1\nACGT\n+\nIIII\n@READ2\nTTTT\n"
    assert ingest.find_fastq_split(d, 0, len(d)) == 19
    d2 = b"@READ1\nACGT\n+\nIIII\n@READ2\nTTTT\n+\nIIII\n"
    assert ingest.find_fastq_split(d2, 0, len(d2)) == 38
    assert ingest.find_fastq_split(b"@R\nAC\n", 0, 6) == 0
