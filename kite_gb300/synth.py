"""Seeded synthetic FASTQ inputs with the shapes of the benchmark workloads.

There are no public datasets on the machines this runs on; every input is
generated from a stated seed (numpy PCG64).  Records are
``@r<9-digit index>\\n<seq>\\n+\\n<qual>\\n`` with all qualities 'I'.

Workload shapes:
  small      1 Mbp i.i.d. genome, 200,000 x 150 bp forward reads, 0.5% subs, no N
  repeats    50 Mbp genome (80% i.i.d., 20% copies of 100 x 2 kbp repeat elements at
             1% per-copy divergence), 150 bp reads, strand 50/50, 1% subs, 0.1% N
  skewed     20 Mbp genome (first 30% AT-rich Markov chain with P(A)=P(T)=0.4),
             250 bp reads, 1% subs
  metagenome 64 species x 300 kbp, Zipf(1.2) abundances over a random permutation,
             read lengths uniform 100-250, 0.5% subs
"""
from __future__ import annotations

import numpy as np

_ASCII = np.frombuffer(b"ACGTN", dtype=np.uint8)


def genome_iid(rng: np.random.Generator, n: int) -> np.ndarray:
    return rng.integers(0, 4, size=n, dtype=np.uint8)


def genome_with_repeats(rng: np.random.Generator, n: int, n_elements: int = 100, elem_len: int = 2000,
                        repeat_frac: float = 0.2, divergence: float = 0.01) -> np.ndarray:
    g = genome_iid(rng, n)
    elems = rng.integers(0, 4, size=(n_elements, elem_len), dtype=np.uint8)
    n_copies = int(n * repeat_frac) // elem_len
    starts = np.sort(rng.choice(n // elem_len, size=n_copies, replace=False)) * elem_len
    which = rng.integers(0, n_elements, size=n_copies)
    for s, w in zip(starts, which):
        c = elems[w].copy()
        mut = rng.random(elem_len) < divergence
        c[mut] = (c[mut] + rng.integers(1, 4, size=int(mut.sum()), dtype=np.uint8)) % 4
        g[s:s + elem_len] = c
    return g


def genome_skewed(rng: np.random.Generator, n: int, low_frac: float = 0.3) -> np.ndarray:
    """First low_frac of the genome: AT-rich 4-state chain (P(A)=P(T)=0.4,
    P(C)=P(G)=0.1, each base drawn given the previous one with a 0.5 chance of
    repeating it), the rest uniform."""
    g = genome_iid(rng, n)
    m = int(n * low_frac)
    probs = np.array([0.4, 0.1, 0.1, 0.4])
    draws = rng.choice(4, size=m, p=probs).astype(np.uint8)
    keep = rng.random(m) < 0.5
    # a "repeat previous base" step makes it a Markov chain with the same marginal
    idx = np.arange(m)
    idx[keep] = 0
    idx = np.maximum.accumulate(idx)
    g[:m] = draws[idx]
    return g


def _mutate(rng, codes: np.ndarray, sub_rate: float) -> None:
    if sub_rate <= 0:
        return
    mut = rng.random(codes.shape) < sub_rate
    codes[mut] = (codes[mut] + rng.integers(1, 4, size=int(mut.sum()), dtype=np.uint8)) % 4


def reads_fixed(rng: np.random.Generator, genome: np.ndarray, n_reads: int, read_len: int, sub_rate: float,
                n_rate: float = 0.0, revcomp_frac: float = 0.0, first_index: int = 0) -> bytes:
    """FASTQ bytes of n_reads reads of read_len bases sampled uniformly."""
    starts = rng.integers(0, len(genome) - read_len + 1, size=n_reads)
    codes = genome[starts[:, None] + np.arange(read_len)[None, :]]
    if revcomp_frac > 0:
        minus = rng.random(n_reads) < revcomp_frac
        codes[minus] = 3 - codes[minus, ::-1]
    _mutate(rng, codes, sub_rate)
    seq = _ASCII[codes]
    if n_rate > 0:
        seq[rng.random(seq.shape) < n_rate] = ord("N")
    hdr_len = 11  # "@r" + 9 digits
    rec_len = hdr_len + 1 + read_len + 1 + 2 + read_len + 1
    out = np.empty((n_reads, rec_len), dtype=np.uint8)
    idx = np.arange(first_index, first_index + n_reads)
    out[:, 0] = ord("@")
    out[:, 1] = ord("r")
    for d in range(9):
        out[:, 2 + d] = ord("0") + (idx // 10 ** (8 - d)) % 10
    o = hdr_len
    out[:, o] = 10
    out[:, o + 1:o + 1 + read_len] = seq
    o += 1 + read_len
    out[:, o] = 10
    out[:, o + 1] = ord("+")
    out[:, o + 2] = 10
    out[:, o + 3:o + 3 + read_len] = ord("I")
    out[:, -1] = 10
    return out.tobytes()


def reads_variable(rng: np.random.Generator, genome: np.ndarray, n_reads: int, len_lo: int, len_hi: int,
                   sub_rate: float, first_index: int = 0) -> bytes:
    lens = rng.integers(len_lo, len_hi + 1, size=n_reads)
    parts = []
    for L in np.unique(lens):
        sel = np.nonzero(lens == L)[0]
        parts.append((sel, reads_fixed(rng, genome, len(sel), int(L), sub_rate, first_index=0)))
    # interleave back into read order: records of one length are contiguous
    # per group; the order of records does not change any count
    return b"".join(p for _, p in parts)


def small_workload(seed: int = 1, n_reads: int = 200_000, genome_len: int = 1_000_000) -> bytes:
    rng = np.random.default_rng(seed)
    g = genome_iid(rng, genome_len)
    return reads_fixed(rng, g, n_reads, 150, 0.005)


def repeats_workload(seed: int = 2, n_reads: int = 10_000_000, genome_len: int = 50_000_000,
                     batch: int = 1_000_000) -> bytes:
    rng = np.random.default_rng(seed)
    g = genome_with_repeats(rng, genome_len)
    parts = []
    for i in range(0, n_reads, batch):
        parts.append(reads_fixed(rng, g, min(batch, n_reads - i), 150, 0.01, n_rate=0.001, revcomp_frac=0.5,
                                 first_index=i))
    return b"".join(parts)


def skewed_workload(seed: int = 4, n_reads: int = 4_000_000, genome_len: int = 20_000_000,
                    batch: int = 500_000) -> bytes:
    rng = np.random.default_rng(seed)
    g = genome_skewed(rng, genome_len)
    parts = []
    for i in range(0, n_reads, batch):
        parts.append(reads_fixed(rng, g, min(batch, n_reads - i), 250, 0.01, first_index=i))
    return b"".join(parts)


def metagenome_samples(seed: int = 3, n_samples: int = 16, species: int = 64, species_len: int = 300_000,
                       reads_lo: int = 500_000, reads_hi: int = 8_000_000, scale: float = 1.0,
                       fast: bool = False) -> list:
    """Uneven samples of a Zipf(1.2) metagenome; `scale` shrinks read counts.
    fast: reads from the host library's multithreaded generator (same shape,
    another random stream), for the full read counts."""
    rng = np.random.default_rng(seed)
    genomes = [genome_iid(np.random.default_rng(seed * 1000 + s), species_len) for s in range(species)]
    out = []
    for si in range(n_samples):
        n = max(1, int(rng.integers(reads_lo, reads_hi + 1) * scale))
        ranks = rng.permutation(species) + 1
        w = 1.0 / ranks ** 1.2
        w /= w.sum()
        per = rng.multinomial(n, w)
        parts = []
        for s, c in enumerate(per):
            if c and fast:
                import os
                from . import host
                parts.append(host.synth_reads_var(genomes[s], int(c), 100, 250, 0.005,
                                                  seed=seed * 1_000_003 + si * 1009 + s,
                                                  threads=max(1, os.cpu_count() or 1)))
            elif c:
                parts.append(reads_variable(rng, genomes[s], int(c), 100, 250, 0.005))
        out.append(b"".join(parts))
    return out


_REPEAT_GENOMES: dict = {}


def repeats_reads(n_reads: int, seed: int = 2, genome_seed: int | None = None, threads: int = 0) -> bytearray:
    """Reads of the repeats workload's shape (150 bp, strand 50/50, 1% subs,
    0.1% N) from the 50 Mbp repeats genome of genome_seed (default: seed),
    generated by the host library's multi-threaded generator."""
    import os
    from . import host
    gs = seed if genome_seed is None else genome_seed
    if gs not in _REPEAT_GENOMES:
        _REPEAT_GENOMES.clear()
        _REPEAT_GENOMES[gs] = genome_with_repeats(np.random.default_rng(gs), 50_000_000)
    return host.synth_reads(_REPEAT_GENOMES[gs], n_reads, 150, 0.01, 0.001, 0.5, seed=seed,
                            threads=threads or max(1, os.cpu_count() or 1))
