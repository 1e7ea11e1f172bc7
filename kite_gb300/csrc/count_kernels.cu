// Count-path kernels: FASTQ line indexing, bit-parallel k-mer extraction with
// canonical min and N-splitting, hash-partition (bucket) scatter, and the
// key-range tile split that feeds the on-chip sort.
//
// Reference behaviour restated here:
//   parse_sequences          src/count/parser.rs:19-65   (sequence = line 1 mod 4 of a chunk
//                                                         that starts with '@')
//   BASE_ENCODE, KmerIter    src/count/kmer.rs:2-13, :241-267, :311-337
//   KmerWord::to_bucket      src/count/kmer.rs:67-71, :111-116
//   CountWorker::push_kmer   src/count/worker.rs:164-175 (replaced by a two-pass
//                            histogram + reservation scatter into bucket regions)
#include <cstdlib>

#include "kite_internal.h"

namespace kite {

static constexpr int kExtractThreads = 256;

// ---------------------------------------------------------------------------
// K1a: newlines per block (16-byte vector loads, SWAR byte compare).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_newline_count(const uint8_t* __restrict__ arena,
                                                       const BlockDesc* __restrict__ blocks,
                                                       unsigned long long* __restrict__ nl) {
  __shared__ unsigned red[34];
  const BlockDesc d = blocks[blockIdx.x];
  const uint64_t nvec = (d.end - d.start) >> 4;
  const uint4* v = reinterpret_cast<const uint4*>(arena + d.start);
  unsigned c = 0;
  for (uint64_t i = threadIdx.x; i < nvec; i += blockDim.x) {
    const uint4 w = v[i];
    c += __popc(__vcmpeq4(w.x, 0x0a0a0a0au)) + __popc(__vcmpeq4(w.y, 0x0a0a0a0au)) +
         __popc(__vcmpeq4(w.z, 0x0a0a0a0au)) + __popc(__vcmpeq4(w.w, 0x0a0a0a0au));
  }
  c >>= 3;  // each matching byte contributes 8 set bits
  for (uint64_t p = d.start + (nvec << 4) + threadIdx.x; p < d.end; p += blockDim.x) c += arena[p] == '\n';
  unsigned total;
  block_exclusive_scan<256, unsigned>(c, red, &total);
  if (threadIdx.x == 0) nl[blockIdx.x] = total;
}

void launch_newline_count(const uint8_t* arena, const BlockDesc* blocks, uint32_t nblocks,
                          unsigned long long* nl_out, cudaStream_t s) {
  if (nblocks) k_newline_count<<<nblocks, 256, 0, s>>>(arena, blocks, nl_out);
}

// Block descriptors from the chunk spans: one thread per block, its chunk by
// binary search over the spans' first blocks.
__global__ void k_make_blocks(const ChunkSpan* __restrict__ spans, uint32_t nspans, uint32_t blk, uint32_t nblocks,
                              BlockDesc* __restrict__ out) {
  const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nblocks) return;
  uint32_t lo = 0, hi = nspans;
  while (hi - lo > 1) {
    const uint32_t m = (lo + hi) >> 1;
    if (spans[m].first_block <= b) lo = m;
    else hi = m;
  }
  const ChunkSpan c = spans[lo];
  const uint64_t o = (uint64_t)(b - c.first_block) * blk;
  BlockDesc d;
  d.start = c.off + o;
  d.end = c.off + (o + blk < c.len ? o + blk : c.len);
  d.chunk_start = c.off;
  d.first_block = c.first_block;
  d.flags = c.flags;
  d.sample = c.sample;
  d.sample_first = c.sample_first;
  out[b] = d;
}

void launch_make_blocks(const ChunkSpan* spans, uint32_t nspans, uint32_t blk, uint32_t nblocks, BlockDesc* out,
                        cudaStream_t s) {
  if (nblocks) k_make_blocks<<<(nblocks + 255) / 256, 256, 0, s>>>(spans, nspans, blk, nblocks, out);
}

__device__ __forceinline__ uint64_t mix64(uint64_t x) {
  x ^= x >> 30;
  x *= 0xbf58476d1ce4e5b9ull;
  x ^= x >> 27;
  x *= 0x94d049bb133111ebull;
  x ^= x >> 31;
  return x;
}

// Per-block bucket counts: one row of the block x bucket count matrix when
// the host provides it (no atomics), else global atomics.
template <int NT, class T>
__device__ __forceinline__ void flush_hist(const ExtractParams<T>& p, const unsigned* hist, uint32_t P,
                                           uint32_t sample) {
  if (p.blk_counts) {
    unsigned* row = p.blk_counts + (size_t)(blockIdx.x + p.block_base) * P;
    for (uint32_t b = threadIdx.x; b < P; b += NT) row[b] = hist[b];
  } else {
    unsigned long long* cnt = p.bucket_count + (size_t)sample * P;
    for (uint32_t b = threadIdx.x; b < P; b += NT)
      if (hist[b]) atomicAdd(&cnt[b], (unsigned long long)hist[b]);
  }
}

// Reads / bases / k-mers of the CTA: one atomic per total per CTA.
// `red` holds 3 * NT / 32 values; ends with a barrier.
template <int NT>
__device__ __forceinline__ void flush_totals(CountTotals* tot, unsigned long long kmers, unsigned long long reads,
                                             unsigned long long bases, unsigned long long* red) {
  constexpr int NW = NT / 32;
  for (int o2 = 16; o2; o2 >>= 1) {
    kmers += __shfl_xor_sync(0xffffffffu, kmers, o2);
    reads += __shfl_xor_sync(0xffffffffu, reads, o2);
    bases += __shfl_xor_sync(0xffffffffu, bases, o2);
  }
  const int wid = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    red[wid] = kmers;
    red[NW + wid] = reads;
    red[2 * NW + wid] = bases;
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    unsigned long long v = 0;
    for (int w = 0; w < NW; ++w) v += red[threadIdx.x * NW + w];
    if (v) atomicAdd(threadIdx.x == 0 ? &tot->kmers : threadIdx.x == 1 ? &tot->reads : &tot->bases, v);
  }
  __syncthreads();
}

// Write offsets of the CTA inside every bucket region: from the scanned
// count matrix when there is one, else by global atomic reservation.
// Leaves base[b] = offset (~0 after an overflow) and hist[] zeroed.
template <int NT, class T>
__device__ __forceinline__ void reserve_ranges(const ExtractParams<T>& p, unsigned* hist, unsigned long long* base,
                                               uint32_t P, const BlockDesc& d) {
  const size_t g0 = (size_t)d.sample * P;  // this sample's first global bucket
  for (uint32_t b = threadIdx.x; b < P; b += NT) {
    const unsigned h = hist[b];
    unsigned long long r = 0;
    if (p.blk_offs)  // offset inside the sample's bucket region: this row minus the sample's first row
      r = p.blk_offs[(size_t)(blockIdx.x + p.block_base) * P + b] - p.blk_offs[(size_t)d.sample_first * P + b];
    else if (h) r = atomicAdd(&p.bucket_fill[g0 + b], (unsigned long long)h);
    if (h && r + h > p.bucket_count[g0 + b]) {
      dev_fail(p.status, KITE_DEV_REGION_OVERFLOW, b, (unsigned)r, h);
      r = ~0ull;
    }
    base[b] = r;
    hist[b] = 0;
  }
}

__host__ __device__ size_t extract64_smem_bytes(uint32_t partitions, bool scatter);

// A word's forward and reverse-complement code streams, shared with the warp.
struct CodeWords {
  uint64_t code, rcode;
};

size_t extract_smem_bytes(int key_bytes, uint32_t blk_bytes, uint32_t partitions, bool scatter) {
  (void)blk_bytes;
  const size_t b = extract64_smem_bytes(partitions, scatter);
  // the u64 histogram pass also shares every thread's three encoded words with its warp
  return key_bytes == 8 && !scatter ? ((b + 15) & ~(size_t)15) + (size_t)kExtractThreads * 3 * sizeof(CodeWords) : b;
}

// ---------------------------------------------------------------------------
// Bit-parallel extraction for k <= 31 (u64 keys).  Each thread owns 64 bytes
// of the block as two 32-byte words and also encodes the word before them.
// Per word, with byte-wise SIMD compares: 2-bit codes packed with the first
// byte in the top bits, the reverse-complement stream (field-reversed ~code),
// and bit masks of newlines and A/C/G/T bytes.  Line phase gives the
// sequence-line mask; a k-mer ending at byte e is valid when the k mask bits
// ending at e are all set, and its forward and reverse-complement values are
// two funnel shifts of the (previous word, word) pair.  Only valid ends are
// visited, so the cost is per k-mer, not per byte.
// ---------------------------------------------------------------------------
struct Word32 {
  uint64_t code;   // 2-bit codes, byte 0 in bits 63..62
  uint64_t rcode;  // complement codes in reverse byte order (byte 31 in bits 63..62)
  uint32_t nl;     // bit i: byte i is '\n'
  uint32_t vb;     // bit i: byte i is A/C/G/T in either case
};

// one bit per byte from a byte-wise 0x00/0xFF mask (byte j -> bit j)
__device__ __forceinline__ uint32_t byte_bits(uint32_t m) { return ((m & 0x01010101u) * 0x10204080u) >> 28; }

__device__ __forceinline__ Word32 encode_word(const uint4 a, const uint4 b) {
  const uint32_t x[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
  Word32 w;
  w.code = 0;
  w.nl = 0;
  w.vb = 0;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const uint32_t v = x[q];
    // A/a=0 C/c=1 G/g=2 T/t=3 from ASCII bits 1 and 2
    const uint32_t c4 = ((v >> 1) ^ (v >> 2)) & 0x03030303u;
    // a byte is a base when, case folded, it is the letter its code stands
    // for: a byte permute of "ACGT" with the codes as selectors
    const uint32_t x = c4 | (c4 >> 4);
    const uint32_t y = x & 0x00FF00FFu;
    const uint32_t valid = __vcmpeq4(v & 0xDFDFDFDFu, __byte_perm(0x54474341u, 0u, (y | (y >> 8)) & 0xFFFFu));
    const uint32_t p8 = (c4 * 0x40100401u) >> 24;  // byte 0's code in bits 7..6
    w.code |= (uint64_t)p8 << (56 - 8 * q);
    w.nl |= byte_bits(__vcmpeq4(v, 0x0a0a0a0au)) << (4 * q);
    w.vb |= byte_bits(valid) << (4 * q);
  }
  uint64_t r = __brevll(~w.code);
  w.rcode = ((r >> 1) & 0x5555555555555555ull) | ((r & 0x5555555555555555ull) << 1);
  return w;
}

// Sequence-line bytes of a word given the line phase at its first byte;
// advances the phase past the word.
__device__ __forceinline__ uint32_t seq_mask(uint32_t nl, unsigned& ph) {
  uint32_t seq = 0, m = nl;
  unsigned start = 0, p = ph;
  while (m) {
    const unsigned q = __ffs(m) - 1;
    if (p == 1) seq |= (uint32_t)((1ull << q) - (1ull << start));
    p = (p + 1) & 3u;
    start = q + 1;
    m &= m - 1;
  }
  if (p == 1) seq |= (uint32_t)((1ull << 32) - (1ull << start));
  ph = p;
  return seq;
}

// bit j set iff bits j .. j+k-1 of a are all set
__device__ __forceinline__ uint64_t runs_of(uint64_t a, uint32_t k) {
  uint64_t r = a;
  uint32_t len = 1;
  while (2 * len <= k) {
    r &= r >> len;
    len *= 2;
  }
  if (len < k) r &= r >> (k - len);
  return r;
}

// Visits every valid k-mer ending in word w (previous word pw): f(key, e).
template <class F>
__device__ __forceinline__ void word_kmers(uint32_t V, const Word32& pw, const Word32& w, uint32_t k, uint64_t mask,
                                           bool canonical, F&& f) {
  while (V) {
    const uint32_t e = __ffs(V) - 1;
    V &= V - 1;
    const uint32_t s = 2 * (31 - e);
    const uint64_t fwd = (s ? ((w.code >> s) | (pw.code << (64 - s))) : w.code) & mask;
    uint64_t key = fwd;
    if (canonical) {
      const uint32_t t = 2 * (33 + e - k);  // 4 .. 126
      const uint64_t rc = (t < 64 ? ((pw.rcode >> t) | (w.rcode << (64 - t))) : (w.rcode >> (t - 64))) & mask;
      key = rc < fwd ? rc : fwd;
    }
    f(key, e);
  }
}

__device__ __forceinline__ void load_word(const uint8_t* arena, uint64_t pos, uint64_t end, Word32& w,
                                          uint32_t& in_range) {
  uint4 a = make_uint4(0, 0, 0, 0), b = make_uint4(0, 0, 0, 0);
  // only 16-byte halves that start inside the block: at most 15 bytes past
  // its end, which the 16 pad bytes after every chunk cover
  if (pos < end) a = *reinterpret_cast<const uint4*>(arena + pos);
  if (pos + 16 < end) b = *reinterpret_cast<const uint4*>(arena + pos + 16);
  w = encode_word(a, b);
  in_range = pos >= end ? 0u : (end - pos >= 32 ? 0xFFFFFFFFu : (uint32_t)((1ull << (end - pos)) - 1));
}

// Extraction shared memory: [scatter bases P x 8] | histogram P x 4 | scan
// area 96 x 4 | (16-aligned) every warp's last word (8 x Word32) | (u64
// histogram pass) the threads' encoded words.
__host__ __device__ static size_t extract_xw_offset(uint32_t partitions, bool scatter) {
  return ((scatter ? (size_t)partitions * 8 : 0) + (size_t)partitions * 4 + 96 * 4 + 15) & ~(size_t)15;
}
__host__ __device__ size_t extract64_smem_bytes(uint32_t partitions, bool scatter) {
  return extract_xw_offset(partitions, scatter) + (size_t)(kExtractThreads / 32) * sizeof(Word32);
}

template <int MODE>
__global__ void __launch_bounds__(kExtractThreads, 6) k_extract64(ExtractParams<uint64_t> p) {
  constexpr int NT = kExtractThreads;
  extern __shared__ __align__(16) uint8_t sm[];
  const uint32_t P = p.partitions;
  unsigned long long* base = reinterpret_cast<unsigned long long*>(sm);
  unsigned* hist = reinterpret_cast<unsigned*>(sm + (MODE == 1 ? (size_t)P * 8 : 0));
  unsigned* scan_sm = hist + P;
  for (uint32_t b = threadIdx.x; b < P; b += NT) hist[b] = 0;

  const uint32_t bi = blockIdx.x + p.block_base;  // global block index
  const BlockDesc d = p.blocks[bi];
  const uint64_t e = d.end;
  const uint64_t ts = d.start + (uint64_t)threadIdx.x * 64;
  const bool chunk_ok = p.arena[d.chunk_start] == '@';  // src/count/parser.rs:27-29
  const uint32_t k = p.k;
  const uint64_t mask = (1ull << (2 * k)) - 1;
  const bool canon = p.canonical != 0;
  const uint32_t shift = p.shift;

  Word32 wp, w0, w1;
  uint32_t r0, r1;
  load_word(p.arena, ts, e, w0, r0);
  load_word(p.arena, ts + 32, e, w1, r1);
  w0.nl &= r0;
  w1.nl &= r1;
  // The word before ts is lane - 1's second word, the previous warp's last
  // one for lane 0; only the block's first thread encodes it itself.  (ts -
  // chunk_start is a multiple of 64: the word before is wholly inside the
  // chunk, or the thread starts the chunk.)
  const unsigned xlane = threadIdx.x & 31, xwid = threadIdx.x >> 5;
  Word32* xw = reinterpret_cast<Word32*>(sm + extract_xw_offset(P, MODE == 1));
  if (xlane == 31) xw[xwid] = w1;
  wp.code = __shfl_up_sync(0xffffffffu, w1.code, 1);
  wp.rcode = __shfl_up_sync(0xffffffffu, w1.rcode, 1);
  wp.nl = __shfl_up_sync(0xffffffffu, w1.nl, 1);
  wp.vb = __shfl_up_sync(0xffffffffu, w1.vb, 1);
  unsigned nl_total;
  const unsigned nl_before = block_exclusive_scan<NT, unsigned>(__popc(w0.nl) + __popc(w1.nl), scan_sm, &nl_total);
  const bool has_prev = ts > d.chunk_start && ts < e;
  if (xlane == 0) {
    if (xwid > 0) {
      wp = xw[xwid - 1];
    } else if (has_prev) {
      uint32_t rp;
      load_word(p.arena, ts - 32, ts, wp, rp);
    }
  }
  if (!has_prev) {
    wp.nl = 0;
    wp.vb = 0;
  }
  const unsigned long long line0 = p.block_nl_excl[bi] - p.block_nl_excl[d.first_block];
  unsigned ph = (unsigned)((line0 + nl_before) & 3ull);  // line phase at ts
  unsigned php = (ph - (unsigned)__popc(wp.nl)) & 3u;     // at ts - 32
  const uint32_t seqp = has_prev ? seq_mask(wp.nl, php) : 0u;
  const uint32_t seq0 = seq_mask(w0.nl, ph) & r0;
  const uint32_t seq1 = seq_mask(w1.nl, ph) & r1;
  const uint32_t okp = chunk_ok ? (seqp & wp.vb) : 0u;
  const uint32_t ok0 = chunk_ok ? (seq0 & w0.vb) : 0u;
  const uint32_t ok1 = chunk_ok ? (seq1 & w1.vb) : 0u;
  const uint32_t V0 = (uint32_t)(runs_of((uint64_t)okp | ((uint64_t)ok0 << 32), k) >> (33 - k));
  const uint32_t V1 = (uint32_t)(runs_of((uint64_t)ok0 | ((uint64_t)ok1 << 32), k) >> (33 - k));
  __syncthreads();  // hist zeroed

  if (MODE == 0) {
    unsigned long long kmers = __popc(V0) + __popc(V1);
    const bool sampling = p.sample != nullptr && (d.flags & 2u);
    // staged keys: this thread's run inside the block's reserved range
    uint64_t* out = nullptr;
    if (p.keys_stage) {
      unsigned tot;
      const unsigned before = block_exclusive_scan<NT, unsigned>((unsigned)kmers, scan_sm, &tot);
      unsigned long long* bb = reinterpret_cast<unsigned long long*>(scan_sm) + 40;
      if (threadIdx.x == 0) {
        unsigned long long at = tot ? atomicAdd(p.stage_counter, (unsigned long long)tot) : 0ull;
        if (at + tot > p.stage_cap) at = ~0ull;  // over capacity: the host takes the other scatter path
        *bb = at;
        p.blk_keys[2 * (size_t)bi] = at;
        p.blk_keys[2 * (size_t)bi + 1] = tot;
      }
      __syncthreads();
      if (*bb != ~0ull) out = p.keys_stage + *bb + before;
    }
    // The warp walks its words in thread order, one lane per end byte, so the
    // lanes share every sequence word's k-mers (a thread's own bytes may be
    // a quality line) and a word's keys go out as one coalesced run.
    const unsigned lane = threadIdx.x & 31;
    CodeWords* ws = reinterpret_cast<CodeWords*>(sm + ((extract64_smem_bytes(P, false) + 15) & ~(size_t)15)) +
                    (size_t)(threadIdx.x & ~31u) * 3;
    ws[3 * lane] = CodeWords{wp.code, wp.rcode};
    ws[3 * lane + 1] = CodeWords{w0.code, w0.rcode};
    ws[3 * lane + 2] = CodeWords{w1.code, w1.rcode};
    __syncwarp();
    const unsigned lt = (1u << lane) - 1u;
    const uint64_t wts = ts - (uint64_t)lane * 64;  // the warp's first byte
    uint64_t* wbase = nullptr;
    {
      const unsigned long long ob = out ? (unsigned long long)(out - p.keys_stage) : 0ull;
      const unsigned long long o0 = __shfl_sync(0xffffffffu, ob, 0);
      if (__shfl_sync(0xffffffffu, out ? 1u : 0u, 0)) wbase = p.keys_stage + o0;
    }
    // A lane's windows are fixed shifts of the (previous, current) word pair:
    // the forward k-mer is the low 64 bits of (pw.code:cw.code) >> sft and the
    // reverse complement the low 64 bits of (cw.rcode:pw.rcode) >> t, both
    // per-lane constants.  Each is two 32-bit funnel shifts of the 32-bit
    // words that the shift's word offset selects (chosen once per lane).
    const uint32_t sft = 2 * (31 - lane);     // 0 .. 62: word offset 0 or 1
    const bool f_hi = sft >= 32;
    const uint32_t fsh = sft & 31u;
    const uint32_t tr = 2 * (33 + lane - k);  // 4 .. 126: word offset 0 .. 3
    const uint32_t tq = tr >> 5, tsh = tr & 31u;
    unsigned run = 0;
    for (unsigned ls = __ballot_sync(0xffffffffu, (V0 | V1) != 0u); ls; ls &= ls - 1) {
      const int l = __ffs(ls) - 1;
      const unsigned lv[2] = {__shfl_sync(0xffffffffu, V0, l), __shfl_sync(0xffffffffu, V1, l)};
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const unsigned V = lv[h];
        if (V == 0u) continue;
        const bool act = (V >> lane) & 1u;
        uint64_t key = 0;
        if (act) {
          const CodeWords pw = ws[3 * l + h], cw = ws[3 * l + h + 1];
          const uint32_t c0 = (uint32_t)cw.code, c1 = (uint32_t)(cw.code >> 32);
          const uint32_t p0 = (uint32_t)pw.code, p1 = (uint32_t)(pw.code >> 32);
          const uint32_t a0 = f_hi ? c1 : c0, a1 = f_hi ? p0 : c1, a2 = f_hi ? p1 : p0;
          const uint64_t fwd =
              (((uint64_t)__funnelshift_r(a1, a2, fsh) << 32) | __funnelshift_r(a0, a1, fsh)) & mask;
          key = fwd;
          if (canon) {
            const uint32_t r0 = (uint32_t)pw.rcode, r1 = (uint32_t)(pw.rcode >> 32);
            const uint32_t r2 = (uint32_t)cw.rcode, r3 = (uint32_t)(cw.rcode >> 32);
            const uint32_t b0 = tq == 0 ? r0 : tq == 1 ? r1 : tq == 2 ? r2 : r3;
            const uint32_t b1 = tq == 0 ? r1 : tq == 1 ? r2 : tq == 2 ? r3 : 0u;
            const uint32_t b2 = tq == 0 ? r2 : tq == 1 ? r3 : 0u;
            const uint64_t rc =
                (((uint64_t)__funnelshift_r(b1, b2, tsh) << 32) | __funnelshift_r(b0, b1, tsh)) & mask;
            key = rc < fwd ? rc : fwd;
          }
          atomicAdd(&hist[bucket_of(key, shift)], 1u);
          if (wbase) wbase[run + __popc(V & lt)] = key;
        }
        if (sampling) {
          // the k-mers whose end position hashes into the sample: one
          // reservation per word
          const uint64_t pos = wts + (uint64_t)l * 64 + 32 * h + lane;
          const bool take = act && (mix64(pos) & p.sample_mask) == 0;
          const unsigned tb = __ballot_sync(0xffffffffu, take);
          if (tb) {
            const int ld = __ffs(tb) - 1;
            unsigned at = 0;
            if ((int)lane == ld) at = atomicAdd(p.sample_count, (unsigned)__popc(tb));
            at = __shfl_sync(0xffffffffu, at, ld) + __popc(tb & lt);
            if (take && at < p.sample_cap) p.sample[at] = key;
          }
        }
        run += __popc(V);
      }
    }
    // reads = starts of non-empty sequence-line runs; bases = sequence-line bytes
    unsigned long long reads = 0, bases = 0;
    if (chunk_ok) {
      bases = __popc(seq0) + __popc(seq1);
      reads = __popc(seq0 & ~((seq0 << 1) | (seqp >> 31))) + __popc(seq1 & ~((seq1 << 1) | (seq0 >> 31)));
    }
    __syncthreads();
    flush_hist<NT>(p, hist, P, d.sample);
    flush_totals<NT>(p.totals + d.sample, kmers, reads, bases, reinterpret_cast<unsigned long long*>(scan_sm));
  } else {
    auto count = [&](uint64_t key, uint32_t) { atomicAdd(&hist[bucket_of(key, shift)], 1u); };
    word_kmers(V0, wp, w0, k, mask, canon, count);
    word_kmers(V1, w0, w1, k, mask, canon, count);
    __syncthreads();
    reserve_ranges<NT>(p, hist, base, P, d);
    __syncthreads();
    auto write = [&](uint64_t key, uint32_t) {
      const uint32_t b = bucket_of(key, shift);
      const unsigned slot = atomicAdd(&hist[b], 1u);
      const unsigned long long r = base[b];
      if (r != ~0ull) p.keys_out[p.bucket_off[(size_t)d.sample * P + b] + r + slot] = key;
    };
    word_kmers(V0, wp, w0, k, mask, canon, write);
    word_kmers(V1, w0, w1, k, mask, canon, write);
  }
}

// ---------------------------------------------------------------------------
// The same for 32 <= k <= 64 (u128 keys): a k-mer ending in a word reaches up
// to two words back, so each thread also encodes the two words before its
// own; windows are funnel shifts of three packed words.
// ---------------------------------------------------------------------------
// bit j set iff bits j .. j+k-1 of a are all set
__device__ __forceinline__ u128 runs_of128(u128 a, uint32_t k) {
  u128 r = a;
  uint32_t len = 1;
  while (2 * len <= k) {
    r &= r >> len;
    len *= 2;
  }
  if (len < k) r &= r >> (k - len);
  return r;
}

// Visits every valid k-mer ending in word w (previous words p1, p2): f(key, e).
template <class F>
__device__ __forceinline__ void word_kmers128(uint32_t V, const Word32& p2, const Word32& p1, const Word32& w,
                                              uint32_t k, u128 mask, bool canonical, F&& f) {
  const u128 X = ((u128)p1.code << 64) | w.code;       // forward stream p1 | w (p2 above it)
  const u128 RL = ((u128)p1.rcode << 64) | p2.rcode;   // reverse stream R(w) | R(p1) | R(p2), low part
  const u128 RH = ((u128)w.rcode << 64) | p1.rcode;    // high part
  while (V) {
    const uint32_t e = __ffs(V) - 1;
    V &= V - 1;
    const uint32_t sft = 2 * (31 - e);  // 0 .. 62
    const u128 fwd = (sft ? ((X >> sft) | ((u128)p2.code << (128 - sft))) : X) & mask;
    u128 key = fwd;
    if (canonical) {
      const uint32_t t = 2 * (65 + e - k);  // 2 .. 128 for 32 <= k <= 64
      u128 rc;
      if (t < 64) rc = (RL >> t) | ((u128)w.rcode << (128 - t));
      else if (t < 128) rc = RH >> (t - 64);
      else rc = (u128)w.rcode;
      rc &= mask;
      key = rc < fwd ? rc : fwd;
    }
    f(key, e);
  }
}

template <int MODE>
__global__ void __launch_bounds__(kExtractThreads) k_extract128(ExtractParams<u128> p) {
  constexpr int NT = kExtractThreads;
  extern __shared__ __align__(16) uint8_t sm[];
  const uint32_t P = p.partitions;
  unsigned long long* base = reinterpret_cast<unsigned long long*>(sm);
  unsigned* hist = reinterpret_cast<unsigned*>(sm + (MODE == 1 ? (size_t)P * 8 : 0));
  unsigned* scan_sm = hist + P;
  for (uint32_t b = threadIdx.x; b < P; b += NT) hist[b] = 0;

  const uint32_t bi = blockIdx.x + p.block_base;  // global block index
  const BlockDesc d = p.blocks[bi];
  const uint64_t e = d.end;
  const uint64_t ts = d.start + (uint64_t)threadIdx.x * 64;
  const bool chunk_ok = p.arena[d.chunk_start] == '@';  // src/count/parser.rs:27-29
  const uint32_t k = p.k;
  const u128 mask = 2 * k == 128 ? ~u128(0) : ((u128(1) << (2 * k)) - u128(1));
  const bool canon = p.canonical != 0;
  const uint32_t shift = p.shift;

  Word32 wq, wp, w0, w1;
  uint32_t r0, r1, rp;
  // ts - chunk_start is a multiple of 64: the two words before are wholly
  // inside the chunk, or the thread starts the chunk
  const bool has_prev = ts > d.chunk_start && ts < e;
  load_word(p.arena, has_prev ? ts - 64 : ts, has_prev ? ts : ts, wq, rp);
  load_word(p.arena, has_prev ? ts - 32 : ts, has_prev ? ts : ts, wp, rp);
  if (!has_prev) {
    wq.nl = wq.vb = 0;
    wp.nl = wp.vb = 0;
  }
  load_word(p.arena, ts, e, w0, r0);
  load_word(p.arena, ts + 32, e, w1, r1);
  w0.nl &= r0;
  w1.nl &= r1;
  unsigned nl_total;
  const unsigned nl_before = block_exclusive_scan<NT, unsigned>(__popc(w0.nl) + __popc(w1.nl), scan_sm, &nl_total);
  const unsigned long long line0 = p.block_nl_excl[bi] - p.block_nl_excl[d.first_block];
  unsigned ph = (unsigned)((line0 + nl_before) & 3ull);                       // line phase at ts
  unsigned phq = (ph - (unsigned)__popc(wp.nl) - (unsigned)__popc(wq.nl)) & 3u;  // at ts - 64
  const uint32_t seqq = has_prev ? seq_mask(wq.nl, phq) : 0u;
  const uint32_t seqp = has_prev ? seq_mask(wp.nl, phq) : 0u;
  const uint32_t seq0 = seq_mask(w0.nl, ph) & r0;
  const uint32_t seq1 = seq_mask(w1.nl, ph) & r1;
  const uint32_t okq = chunk_ok ? (seqq & wq.vb) : 0u;
  const uint32_t okp = chunk_ok ? (seqp & wp.vb) : 0u;
  const uint32_t ok0 = chunk_ok ? (seq0 & w0.vb) : 0u;
  const uint32_t ok1 = chunk_ok ? (seq1 & w1.vb) : 0u;
  const uint32_t V0 =
      (uint32_t)(uint64_t)(runs_of128((u128)okq | ((u128)okp << 32) | ((u128)ok0 << 64), k) >> (65 - k));
  const uint32_t V1 =
      (uint32_t)(uint64_t)(runs_of128((u128)okp | ((u128)ok0 << 32) | ((u128)ok1 << 64), k) >> (65 - k));
  __syncthreads();  // hist zeroed

  if (MODE == 0) {
    unsigned long long kmers = __popc(V0) + __popc(V1);
    const bool sampling = p.sample != nullptr && (d.flags & 2u);
    u128* out = nullptr;
    if (p.keys_stage) {
      unsigned tot;
      const unsigned before = block_exclusive_scan<NT, unsigned>((unsigned)kmers, scan_sm, &tot);
      unsigned long long* bb = reinterpret_cast<unsigned long long*>(scan_sm) + 40;
      if (threadIdx.x == 0) {
        unsigned long long at = tot ? atomicAdd(p.stage_counter, (unsigned long long)tot) : 0ull;
        if (at + tot > p.stage_cap) at = ~0ull;  // over capacity: the host takes the other scatter path
        *bb = at;
        p.blk_keys[2 * (size_t)bi] = at;
        p.blk_keys[2 * (size_t)bi + 1] = tot;
      }
      __syncthreads();
      if (*bb != ~0ull) out = p.keys_stage + *bb + before;
    }
    auto emit = [&](u128 key, uint64_t pos) {
      atomicAdd(&hist[bucket_of(key, shift)], 1u);
      if (out) *out++ = key;
      if (sampling && (mix64(pos) & p.sample_mask) == 0) {
        const unsigned idx = atomicAdd(p.sample_count, 1u);
        if (idx < p.sample_cap) p.sample[idx] = key;
      }
    };
    word_kmers128(V0, wq, wp, w0, k, mask, canon, [&](u128 key, uint32_t b) { emit(key, ts + b); });
    word_kmers128(V1, wp, w0, w1, k, mask, canon, [&](u128 key, uint32_t b) { emit(key, ts + 32 + b); });
    unsigned long long reads = 0, bases = 0;
    if (chunk_ok) {
      bases = __popc(seq0) + __popc(seq1);
      reads = __popc(seq0 & ~((seq0 << 1) | (seqp >> 31))) + __popc(seq1 & ~((seq1 << 1) | (seq0 >> 31)));
    }
    __syncthreads();
    flush_hist<NT>(p, hist, P, d.sample);
    flush_totals<NT>(p.totals + d.sample, kmers, reads, bases, reinterpret_cast<unsigned long long*>(scan_sm));
  } else {
    auto count = [&](u128 key, uint32_t) { atomicAdd(&hist[bucket_of(key, shift)], 1u); };
    word_kmers128(V0, wq, wp, w0, k, mask, canon, count);
    word_kmers128(V1, wp, w0, w1, k, mask, canon, count);
    __syncthreads();
    reserve_ranges<NT>(p, hist, base, P, d);
    __syncthreads();
    auto write = [&](u128 key, uint32_t) {
      const uint32_t b = bucket_of(key, shift);
      const unsigned slot = atomicAdd(&hist[b], 1u);
      const unsigned long long r = base[b];
      if (r != ~0ull) p.keys_out[p.bucket_off[(size_t)d.sample * P + b] + r + slot] = key;
    };
    word_kmers128(V0, wq, wp, w0, k, mask, canon, write);
    word_kmers128(V1, wp, w0, w1, k, mask, canon, write);
  }
}

template <class T>
void launch_extract_hist(const ExtractParams<T>& p, uint32_t nblocks, cudaStream_t s) {
  const size_t smem = extract_smem_bytes(sizeof(T), p.blk_bytes, p.partitions, false);
  if constexpr (sizeof(T) == 8) {
    cudaFuncSetAttribute(k_extract64<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (nblocks)
      k_extract64<0><<<nblocks, kExtractThreads, smem, s>>>(reinterpret_cast<const ExtractParams<uint64_t>&>(p));
  } else {
    cudaFuncSetAttribute(k_extract128<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (nblocks) k_extract128<0><<<nblocks, kExtractThreads, smem, s>>>(p);
  }
}
template <class T>
void launch_extract_scatter(const ExtractParams<T>& p, uint32_t nblocks, cudaStream_t s) {
  const size_t smem = extract_smem_bytes(sizeof(T), p.blk_bytes, p.partitions, true);
  if constexpr (sizeof(T) == 8) {
    cudaFuncSetAttribute(k_extract64<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (nblocks)
      k_extract64<1><<<nblocks, kExtractThreads, smem, s>>>(reinterpret_cast<const ExtractParams<uint64_t>&>(p));
  } else {
    cudaFuncSetAttribute(k_extract128<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (nblocks) k_extract128<1><<<nblocks, kExtractThreads, smem, s>>>(p);
  }
}
template void launch_extract_hist<uint64_t>(const ExtractParams<uint64_t>&, uint32_t, cudaStream_t);
template void launch_extract_hist<u128>(const ExtractParams<u128>&, uint32_t, cudaStream_t);
template void launch_extract_scatter<uint64_t>(const ExtractParams<uint64_t>&, uint32_t, cudaStream_t);
template void launch_extract_scatter<u128>(const ExtractParams<u128>&, uint32_t, cudaStream_t);

// ---------------------------------------------------------------------------
// Key-range split: inside every hash bucket, route keys to S key-range tiles
// by the global splitters (tile of a key = number of splitters <= key).
// Tiles are laid out bucket-major, so each bucket's tiles stay contiguous and
// in key order.  One level handles D <= 1024 sub-ranges ("digits") per
// region; S > 1024 tiles take two levels (coarse ranges, then tiles inside
// each coarse range), so that every scatter writes to at most 1024
// destinations.  A digit's runs from consecutive batches of one part are
// adjacent, so partial sectors written by one batch are completed in L2 by the
// next before they reach DRAM.
// Each region is processed in G parts; part (r, g) owns the sub-range
// [off[(r*D+d)*G+g], +count) of digit d, so no two CTAs share a cursor and
// the only atomics are shared-memory ones.
// ---------------------------------------------------------------------------
static constexpr int kLutBits = 12, kLutSize = 1 << kLutBits;
static constexpr size_t kLutBytes = ((size_t)(kLutSize + 1) * 2 + 15) & ~(size_t)15;
static constexpr int kSplitThreads = 512;
static constexpr int kSplitUnroll = 8;
static constexpr uint32_t kMaxDigits = 1024;

// Loads region r's D-1 digit splitters and builds a table over the region's
// key range [lo, hi] (the splitters just outside it): lut[bin] = number of the
// region's splitters below the bin's first key.  Block-wide; ends with a barrier.
template <class T>
__device__ void load_digits(const TileSplitParams<T>& p, uint32_t r, T* spl, uint16_t* lut, T* lo_out,
                            uint32_t* shift_out) {
  const uint32_t nspl = p.D - 1;
  const long long base = (long long)p.spl_first + (long long)(r % p.spl_mod) * p.spl_region_stride;
  for (uint32_t i = threadIdx.x; i < nspl; i += blockDim.x) spl[i] = p.splitters[base + (long long)i * p.spl_step];
  const long long lo_i = base - (long long)p.spl_step, hi_i = base + (long long)nspl * p.spl_step;
  const T kmax = p.key_bits >= (uint32_t)KeyTraits<T>::kBits ? ~T(0) : ((T(1) << p.key_bits) - T(1));
  const T lo = lo_i >= 0 ? p.splitters[lo_i] : T(0);
  const T hi = hi_i < (long long)p.spl_total ? p.splitters[hi_i] : kmax;
  const T range = hi > lo ? T(hi - lo) : T(0);
  const int rb = range == T(0) ? 0 : KeyTraits<T>::kBits - clz_key(range);
  const uint32_t shift = rb > kLutBits ? (uint32_t)(rb - kLutBits) : 0u;
  __syncthreads();
  for (uint32_t bin = threadIdx.x; bin <= (uint32_t)kLutSize; bin += blockDim.x) {
    uint32_t v = nspl;
    if (bin < (uint32_t)kLutSize) {
      const T off = (T)bin << shift;
      if (off <= T(~T(0) - lo)) {
        const T start = lo + off;
        uint32_t a = 0, e = nspl;  // lower bound: splitters below start
        while (a < e) {
          const uint32_t m = (a + e) >> 1;
          if (spl[m] < start) a = m + 1;
          else e = m;
        }
        v = a;
      }
    }
    lut[bin] = (uint16_t)v;
  }
  __syncthreads();
  *lo_out = lo;
  *shift_out = shift;
}

// Digit of a key (>= lo): number of the region's splitters <= key, searched
// between the table entries of its bin and the next.
template <class T>
__device__ __forceinline__ uint32_t digit_of_key(const T* spl, const uint16_t* lut, T lo, uint32_t shift, T key) {
  const T rel = key > lo ? T(key - lo) : T(0);
  const T b = rel >> shift;
  const uint32_t bin = b >= (T)kLutSize ? (uint32_t)kLutSize - 1u : (uint32_t)(uint64_t)b;
  uint32_t a = lut[bin], e = lut[bin + 1];
  while (a < e) {
    const uint32_t m = (a + e) >> 1;
    if (spl[m] <= key) a = m + 1;
    else e = m;
  }
  return a;
}

// Keys of part g of region r: an even share of the region's run, or with
// input pieces, of its run in piece g / (G / pieces).
template <class T>
__device__ __forceinline__ void part_range(const TileSplitParams<T>& p, uint32_t r, uint32_t g, uint64_t* lo,
                                           uint64_t* hi) {
  uint32_t G = p.G, idx = r;
  if (p.pieces > 1) {
    G = p.G / p.pieces;
    const uint32_t q = g / G;
    g -= q * G;
    idx = q * p.R + r;
  }
  const uint64_t n = p.region_count[idx], base = p.region_off[idx];
  *lo = base + n * g / G;
  *hi = base + n * (g + 1) / G;
}

// Digit histogram of one part (shared-memory counters).
template <class T>
__global__ void __launch_bounds__(kSplitThreads) k_split_hist(TileSplitParams<T> p) {
  __shared__ T spl[kMaxDigits];
  __shared__ __align__(16) uint16_t lut[kLutBytes / 2];
  __shared__ unsigned hist[kMaxDigits];
  const uint32_t D = p.D, G = p.G;
  const uint32_t r = blockIdx.x / G, g = blockIdx.x % G;
  for (uint32_t i = threadIdx.x; i < D; i += kSplitThreads) hist[i] = 0;
  T lo;
  uint32_t sh;
  load_digits(p, r, spl, lut, &lo, &sh);
  uint64_t a, e;
  part_range(p, r, g, &a, &e);
  // kSplitUnroll independent loads in flight per thread before any use
  for (uint64_t i0 = a + threadIdx.x; i0 < e; i0 += (uint64_t)kSplitThreads * kSplitUnroll) {
    T key[kSplitUnroll];
#pragma unroll
    for (int u = 0; u < kSplitUnroll; ++u) {
      const uint64_t i = i0 + (uint64_t)u * kSplitThreads;
      key[u] = i < e ? p.keys_in[i] : T(0);
    }
#pragma unroll
    for (int u = 0; u < kSplitUnroll; ++u) {
      const uint64_t i = i0 + (uint64_t)u * kSplitThreads;
      if (i < e) {
        const uint32_t d = digit_of_key(spl, lut, lo, sh, key[u]);
        atomicAdd(&hist[d], 1u);
        if (p.dig) p.dig[i] = (uint16_t)d;
      }
    }
  }
  __syncthreads();
  for (uint32_t d = threadIdx.x; d < D; d += kSplitThreads) p.tile_count[((size_t)r * D + d) * G + g] = hist[d];
}

// Scatter of one part, a batch of BATCH keys at a time: the batch is ranked on
// chip by digit (shared-memory atomics over RADIX >= D digits; key order inside
// a tile does not matter) and staged in digit order behind each digit's keys
// held back from the previous batch.  Each digit's run is written up to its
// last 32-byte sector boundary with consecutive threads on consecutive
// addresses; the keys past the boundary (fewer than a sector) wait for the
// next batch.  Global writes therefore go out as whole sectors, except the
// first and last one of each digit in the part, even when a batch holds only a
// few keys per digit.
template <class T, int NT_, int IT_, int RADIX_>
struct ScatterSmem {
  static constexpr int NT = NT_, NW = NT / 32, IT = IT_, RADIX = RADIX_;
  static constexpr int BATCH = NT * IT;
  static constexpr int KPS = 32 / (int)sizeof(T);            // keys per sector
  static constexpr int STAGE = BATCH + RADIX * (KPS - 1);    // a batch and every digit's held-back keys
  static constexpr size_t o_stage = 0;
  static constexpr size_t o_dig = o_stage + (size_t)STAGE * sizeof(T);
  static constexpr size_t o_whist = (o_dig + (size_t)STAGE * 2 + 15) & ~(size_t)15;
  static constexpr size_t o_cur = o_whist + (size_t)RADIX * 4;
  static constexpr size_t o_dtot = o_cur + (size_t)RADIX * 8;
  static constexpr size_t o_dstart = o_dtot + (size_t)RADIX * 4;
  static constexpr size_t o_wr = o_dstart + (size_t)RADIX * 4;
  static constexpr size_t o_held = o_wr + (size_t)RADIX * 2;
  static constexpr size_t o_spl = (o_held + (size_t)RADIX + 15) & ~(size_t)15;
  static constexpr size_t o_lut = o_spl + (size_t)RADIX * sizeof(T);
  static constexpr size_t o_scan = o_lut + kLutBytes;
  static constexpr size_t total = o_scan + 64 * 4;
  static_assert(STAGE < 65536, "write counts are 16-bit");
};

template <class T, int NT, int IT, int RADIX>
__global__ void __launch_bounds__(NT, (IT * sizeof(T) > 64 ? 512 : 1024) / NT) k_split_scatter(TileSplitParams<T> p) {
  using L = ScatterSmem<T, NT, IT, RADIX>;
  constexpr int BATCH = L::BATCH, KPS = L::KPS;
  constexpr int PER = RADIX > NT ? RADIX / NT : 1;  // digits owned by each thread
  static_assert(RADIX <= NT || RADIX % NT == 0, "digits split evenly over the threads");
  extern __shared__ __align__(16) uint8_t sm[];
  T* stage = reinterpret_cast<T*>(sm + L::o_stage);
  uint16_t* dig16 = reinterpret_cast<uint16_t*>(sm + L::o_dig);
  unsigned* whist = reinterpret_cast<unsigned*>(sm + L::o_whist);
  unsigned long long* cur = reinterpret_cast<unsigned long long*>(sm + L::o_cur);
  unsigned* dtot = reinterpret_cast<unsigned*>(sm + L::o_dtot);      // held + new keys of the batch
  unsigned* dstart = reinterpret_cast<unsigned*>(sm + L::o_dstart);  // the digit's first stage slot
  uint16_t* wr = reinterpret_cast<uint16_t*>(sm + L::o_wr);          // keys written this batch
  uint8_t* held = sm + L::o_held;                                    // held-back keys ahead of the new ones
  T* spl = reinterpret_cast<T*>(sm + L::o_spl);
  uint16_t* lut = reinterpret_cast<uint16_t*>(sm + L::o_lut);
  unsigned* scan_sm = reinterpret_cast<unsigned*>(sm + L::o_scan);
  const uint32_t D = p.D, G = p.G;
  const uint32_t r = blockIdx.x / G, g = blockIdx.x % G;
  for (uint32_t d = threadIdx.x; d < (uint32_t)RADIX; d += NT) {
    cur[d] = d < D ? p.tile_off[((size_t)r * D + d) * G + g] : 0ull;
    whist[d] = 0;  // rank counters
    dtot[d] = 0;
    dstart[d] = 0;
    wr[d] = 0;
  }
  T lo = T(0);
  uint32_t sh = 0;
  if (p.dig) __syncthreads();  // the histogram pass left every digit
  else load_digits(p, r, spl, lut, &lo, &sh);  // ends with a barrier
  uint64_t a, e;
  part_range(p, r, g, &a, &e);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const unsigned pos0 = (unsigned)wid * 32u * IT + lane;
  const unsigned d0 = threadIdx.x * PER;
  for (uint64_t c0 = a; c0 < e; c0 += BATCH) {
    const unsigned cn = (unsigned)((e - c0) < (uint64_t)BATCH ? (e - c0) : (uint64_t)BATCH);
    T key[IT];
    unsigned dg[IT], rank[IT];
    bool valid[IT];
#pragma unroll
    for (int q = 0; q < IT; ++q) {
      const unsigned pos = pos0 + q * 32u;
      valid[q] = pos < cn;
      key[q] = valid[q] ? p.keys_in[c0 + pos] : T(0);
    }
    if (p.dig) {
#pragma unroll
      for (int q = 0; q < IT; ++q) dg[q] = valid[q] ? (unsigned)p.dig[c0 + pos0 + q * 32u] : 0u;
    } else {
#pragma unroll
      for (int q = 0; q < IT; ++q) dg[q] = valid[q] ? digit_of_key(spl, lut, lo, sh, key[q]) : 0u;
    }
#pragma unroll
    for (int q = 0; q < IT; ++q) rank[q] = valid[q] ? atomicAdd(&whist[dg[q]], 1u) : 0u;
    __syncthreads();
    // owned digits: the keys held back by the last batch (to registers), the
    // new totals and stage starts, and how many keys reach a sector boundary
    T hk[PER][KPS - 1];
    unsigned nh[PER], nt[PER], sum = 0;
#pragma unroll
    for (int j = 0; j < PER; ++j) {
      const unsigned d = d0 + j;
      nh[j] = nt[j] = 0;
      if (d < (unsigned)RADIX) {
        const unsigned w = wr[d];
        nh[j] = dtot[d] - w;
        const unsigned hs = dstart[d] + w;
#pragma unroll
        for (int k = 0; k < KPS - 1; ++k)
          if ((unsigned)k < nh[j]) hk[j][k] = stage[hs + k];
        cur[d] += w;
        nt[j] = nh[j] + whist[d];
        whist[d] = 0;
      }
      sum += nt[j];
    }
    unsigned total;
    unsigned ex = block_exclusive_scan<NT, unsigned>(sum, scan_sm, &total);
#pragma unroll
    for (int j = 0; j < PER; ++j) {
      const unsigned d = d0 + j;
      if (d < (unsigned)RADIX) {
        dstart[d] = ex;
        dtot[d] = nt[j];
        held[d] = (uint8_t)nh[j];
        const unsigned long long cb = cur[d];
        const unsigned long long B = (cb + nt[j]) & ~(unsigned long long)(KPS - 1);
        wr[d] = (uint16_t)(B > cb ? B - cb : 0ull);
        ex += nt[j];
      }
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < PER; ++j) {
      const unsigned d = d0 + j;
#pragma unroll
      for (int k = 0; k < KPS - 1; ++k)
        if ((unsigned)k < nh[j]) {
          stage[dstart[d] + k] = hk[j][k];
          dig16[dstart[d] + k] = (uint16_t)d;
        }
    }
#pragma unroll
    for (int q = 0; q < IT; ++q)
      if (valid[q]) {
        const unsigned at = dstart[dg[q]] + held[dg[q]] + rank[q];
        stage[at] = key[q];
        dig16[at] = (uint16_t)dg[q];
      }
    __syncthreads();
    for (unsigned i = threadIdx.x; i < total; i += NT) {
      const unsigned d = dig16[i], v = i - dstart[d];
      if (v < wr[d]) p.keys_out[cur[d] + v] = stage[i];
    }
    // no barrier: the next batch changes the stage and the digit state only
    // after its first barrier, which every thread reaches after this loop
  }
  __syncthreads();
  // the part's last keys of every digit (a partial sector)
#pragma unroll
  for (int j = 0; j < PER; ++j) {
    const unsigned d = d0 + j;
    if (d < (unsigned)RADIX)
      for (unsigned k = wr[d]; k < dtot[d]; ++k) p.keys_out[cur[d] + k] = stage[dstart[d] + k];
  }
}

// The same scatter when the histogram pass has left every key's digit: each
// digit's run leaves shared memory by one 1-D bulk copy (cp.async.bulk,
// shared -> global) issued by the digit's owner thread, instead of one store
// per key, and the stage holds keys only.  A bulk copy starts and ends on
// 16-byte boundaries at both addresses: runs end on sector boundaries (as
// above), a run of 8-byte keys starting at an odd key index sends its first
// key by a plain store, and the stage places every run on the parity of its
// global position (one pad slot per digit).  The owner waits for its copies
// to have read the stage before the next batch overwrites it.
template <class T, int NT_, int IT_, int RADIX_>
struct BulkScatterSmem {
  static constexpr int NT = NT_, IT = IT_, RADIX = RADIX_;
  static constexpr int BATCH = NT * IT;
  static constexpr int KPS = 32 / (int)sizeof(T);  // keys per sector
  static constexpr int PAD = sizeof(T) == 8 ? 1 : 0;
  static constexpr int STAGE = BATCH + RADIX * (KPS - 1) + RADIX * PAD;
  static constexpr size_t o_stage = 0;
  static constexpr size_t o_whist = ((size_t)STAGE * sizeof(T) + 15) & ~(size_t)15;
  static constexpr size_t o_cur = o_whist + (size_t)RADIX * 4;
  static constexpr size_t o_dtot = o_cur + (size_t)RADIX * 8;
  static constexpr size_t o_dstart = o_dtot + (size_t)RADIX * 4;
  static constexpr size_t o_wr = o_dstart + (size_t)RADIX * 4;
  static constexpr size_t o_held = o_wr + (size_t)RADIX * 2;
  static constexpr size_t o_scan = (o_held + (size_t)RADIX + 15) & ~(size_t)15;
  static constexpr size_t total = o_scan + 64 * 4;
  static_assert(STAGE < 65536, "write counts are 16-bit");
};

__device__ __forceinline__ void bulk_store_global(void* gdst, const void* ssrc, uint32_t bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(gdst),
               "r"((uint32_t)__cvta_generic_to_shared(ssrc)), "r"(bytes)
               : "memory");
}

template <class T, int NT, int IT, int RADIX>
__global__ void __launch_bounds__(NT, (IT * sizeof(T) > 64 ? 512 : 1024) / NT)
    k_split_scatter_bulk(TileSplitParams<T> p) {
  using L = BulkScatterSmem<T, NT, IT, RADIX>;
  constexpr int BATCH = L::BATCH, KPS = L::KPS;
  constexpr int PER = RADIX > NT ? RADIX / NT : 1;
  static_assert(RADIX <= NT || RADIX % NT == 0, "digits split evenly over the threads");
  extern __shared__ __align__(16) uint8_t sm[];
  T* stage = reinterpret_cast<T*>(sm + L::o_stage);
  unsigned* whist = reinterpret_cast<unsigned*>(sm + L::o_whist);
  unsigned long long* cur = reinterpret_cast<unsigned long long*>(sm + L::o_cur);
  unsigned* dtot = reinterpret_cast<unsigned*>(sm + L::o_dtot);
  unsigned* dstart = reinterpret_cast<unsigned*>(sm + L::o_dstart);
  uint16_t* wr = reinterpret_cast<uint16_t*>(sm + L::o_wr);
  uint8_t* held = sm + L::o_held;
  unsigned* scan_sm = reinterpret_cast<unsigned*>(sm + L::o_scan);
  const uint32_t D = p.D, G = p.G;
  const uint32_t r = blockIdx.x / G, g = blockIdx.x % G;
  for (uint32_t d = threadIdx.x; d < (uint32_t)RADIX; d += NT) {
    cur[d] = d < D ? p.tile_off[((size_t)r * D + d) * G + g] : 0ull;
    whist[d] = 0;  // rank counters
    dtot[d] = 0;
    dstart[d] = 0;
    wr[d] = 0;
  }
  __syncthreads();
  uint64_t a, e;
  part_range(p, r, g, &a, &e);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const unsigned pos0 = (unsigned)wid * 32u * IT + lane;
  const unsigned d0 = threadIdx.x * PER;
  T* out = p.keys_out;
  for (uint64_t c0 = a; c0 < e; c0 += BATCH) {
    const unsigned cn = (unsigned)((e - c0) < (uint64_t)BATCH ? (e - c0) : (uint64_t)BATCH);
    T key[IT];
    unsigned dg[IT], rank[IT];
    bool valid[IT];
#pragma unroll
    for (int q = 0; q < IT; ++q) {
      const unsigned pos = pos0 + q * 32u;
      valid[q] = pos < cn;
      key[q] = valid[q] ? p.keys_in[c0 + pos] : T(0);
      dg[q] = valid[q] ? (unsigned)p.dig[c0 + pos] : 0u;
    }
#pragma unroll
    for (int q = 0; q < IT; ++q) rank[q] = valid[q] ? atomicAdd(&whist[dg[q]], 1u) : 0u;
    asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");  // the last batch's copies have read the stage
    __syncthreads();
    // owned digits: the held-back keys (to registers), the new totals and
    // stage starts, and how many keys reach a sector boundary
    T hk[PER][KPS - 1];
    unsigned nh[PER], nt[PER], sum = 0;
#pragma unroll
    for (int j = 0; j < PER; ++j) {
      const unsigned d = d0 + j;
      nh[j] = nt[j] = 0;
      if (d < (unsigned)RADIX) {
        const unsigned w = wr[d];
        nh[j] = dtot[d] - w;
        const unsigned hs = dstart[d] + w;
#pragma unroll
        for (int k = 0; k < KPS - 1; ++k)
          if ((unsigned)k < nh[j]) hk[j][k] = stage[hs + k];
        cur[d] += w;
        nt[j] = nh[j] + whist[d];
        whist[d] = 0;
      }
      sum += nt[j] + L::PAD;
    }
    unsigned total;
    unsigned ex = block_exclusive_scan<NT, unsigned>(sum, scan_sm, &total);
#pragma unroll
    for (int j = 0; j < PER; ++j) {
      const unsigned d = d0 + j;
      if (d < (unsigned)RADIX) {
        const unsigned long long cb = cur[d];
        dstart[d] = L::PAD ? ex + (unsigned)((ex ^ (unsigned)cb) & 1u) : ex;
        dtot[d] = nt[j];
        held[d] = (uint8_t)nh[j];
        const unsigned long long B = (cb + nt[j]) & ~(unsigned long long)(KPS - 1);
        wr[d] = (uint16_t)(B > cb ? B - cb : 0ull);
        ex += nt[j] + L::PAD;
      }
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < PER; ++j) {
      const unsigned d = d0 + j;
#pragma unroll
      for (int k = 0; k < KPS - 1; ++k)
        if ((unsigned)k < nh[j]) stage[dstart[d] + k] = hk[j][k];
    }
#pragma unroll
    for (int q = 0; q < IT; ++q)
      if (valid[q]) stage[dstart[dg[q]] + held[dg[q]] + rank[q]] = key[q];
    __syncthreads();
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // the stage writes, before the copies read it
    bool issued = false;
#pragma unroll
    for (int j = 0; j < PER; ++j) {
      const unsigned d = d0 + j;
      if (d >= (unsigned)RADIX) continue;
      unsigned w = wr[d];
      if (!w) continue;
      unsigned long long cb = cur[d];
      unsigned s0 = dstart[d];
      if (L::PAD && (cb & 1ull)) {
        out[cb] = stage[s0];
        ++cb;
        ++s0;
        --w;
      }
      if (w) {
        bulk_store_global(out + cb, stage + s0, w * (uint32_t)sizeof(T));
        issued = true;
      }
    }
    if (issued) asm volatile("cp.async.bulk.commit_group;" ::: "memory");
  }
  asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
  __syncthreads();
  // the part's last keys of every digit (a partial sector)
#pragma unroll
  for (int j = 0; j < PER; ++j) {
    const unsigned d = d0 + j;
    if (d < (unsigned)RADIX)
      for (unsigned k = wr[d]; k < dtot[d]; ++k) out[cur[d] + k] = stage[dstart[d] + k];
  }
  asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");  // every copy done before the CTA's memory goes
}

// Bucket scatter of staged keys, one CTA per extraction block: batches of
// BATCH keys ranked on chip by partition (shared-memory atomics; order inside a
// partition does not matter), staged in partition order and written as runs at
// the block's offsets.
constexpr int kBsThreads = 256, kBsItems = 8, kBsBatch = kBsThreads * kBsItems;
template <class T>
struct BsSmem {
  static constexpr int NW = kBsThreads / 32;
  static constexpr size_t o_stage = 0;
  static constexpr size_t o_dig = o_stage + (size_t)kBsBatch * sizeof(T);
  static constexpr size_t o_whist = (o_dig + (size_t)kBsBatch + 15) & ~(size_t)15;
  static constexpr size_t o_cur = o_whist + (size_t)256 * NW * 4;
  static constexpr size_t o_dtot = o_cur + (size_t)256 * 8;
  static constexpr size_t o_dstart = o_dtot + (size_t)256 * 4;
  static constexpr size_t o_scan = o_dstart + (size_t)256 * 4;
  static constexpr size_t total = o_scan + 64 * 4;
};

template <class T>
__global__ void __launch_bounds__(kBsThreads, 4)
    k_bucket_scatter(const T* __restrict__ keys_stage, const unsigned long long* __restrict__ blk_keys,
                     const unsigned* __restrict__ blk_offs, const BlockDesc* __restrict__ blocks,
                     const unsigned long long* __restrict__ bucket_off, uint32_t P, uint32_t shift,
                     T* __restrict__ keys_out, const unsigned long long* __restrict__ stage_counter,
                     unsigned long long stage_cap) {
  using L = BsSmem<T>;
  constexpr int NT = kBsThreads, IT = kBsItems;
  extern __shared__ __align__(16) uint8_t sm[];
  T* stage = reinterpret_cast<T*>(sm + L::o_stage);
  uint8_t* dig8 = sm + L::o_dig;
  unsigned* whist = reinterpret_cast<unsigned*>(sm + L::o_whist);
  unsigned long long* cur = reinterpret_cast<unsigned long long*>(sm + L::o_cur);
  unsigned* dtot = reinterpret_cast<unsigned*>(sm + L::o_dtot);
  unsigned* dstart = reinterpret_cast<unsigned*>(sm + L::o_dstart);
  unsigned* scan_sm = reinterpret_cast<unsigned*>(sm + L::o_scan);
  const uint64_t a = blk_keys[2 * (size_t)blockIdx.x];
  const uint64_t n = blk_keys[2 * (size_t)blockIdx.x + 1];
  // an unstaged block (a == ~0), or staging over capacity anywhere so far:
  // the host scatters from the FASTQ instead
  if (n == 0 || a == ~0ull || (stage_counter && *stage_counter > stage_cap)) return;
  const BlockDesc d = blocks[blockIdx.x];
  const unsigned* row = blk_offs + (size_t)blockIdx.x * P;
  const unsigned* first = blk_offs + (size_t)d.sample_first * P;  // the sample's first block
  const unsigned long long* boff = bucket_off + (size_t)d.sample * P;
  for (uint32_t b = threadIdx.x; b < P; b += NT) cur[b] = boff[b] + (row[b] - first[b]);
  for (int b = threadIdx.x; b < 256; b += NT) whist[b] = 0;  // rank counters
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const unsigned pos0 = (unsigned)wid * 32u * IT + lane;
  for (uint64_t c0 = 0; c0 < n; c0 += kBsBatch) {
    const unsigned cn = (unsigned)((n - c0) < (uint64_t)kBsBatch ? (n - c0) : (uint64_t)kBsBatch);
    T key[IT];
    unsigned dg[IT], dest[IT];
    bool valid[IT];
#pragma unroll
    for (int q = 0; q < IT; ++q) {
      const unsigned pos = pos0 + q * 32u;
      valid[q] = pos < cn;
      key[q] = valid[q] ? keys_stage[a + c0 + pos] : T(0);
      dg[q] = valid[q] ? bucket_of(key[q], shift) : 0u;
    }
    atomic_rank<NT, IT, 256>(dg, valid, dest, whist, scan_sm, dtot, dstart);
#pragma unroll
    for (int q = 0; q < IT; ++q)
      if (valid[q]) {
        stage[dest[q]] = key[q];
        dig8[dest[q]] = (uint8_t)dg[q];
      }
    __syncthreads();
    for (unsigned i = threadIdx.x; i < cn; i += NT) {
      const unsigned d = dig8[i];
      keys_out[cur[d] + (i - dstart[d])] = stage[i];
    }
    __syncthreads();
    for (uint32_t b = threadIdx.x; b < P; b += NT) cur[b] += dtot[b];
    __syncthreads();
  }
}

template <class T>
void launch_bucket_scatter(const T* keys_stage, const unsigned long long* blk_keys, const unsigned* blk_offs,
                           const BlockDesc* blocks, const unsigned long long* bucket_off, uint32_t partitions,
                           uint32_t shift, uint32_t nblocks, T* keys_out, const unsigned long long* stage_counter,
                           unsigned long long stage_cap, cudaStream_t s) {
  const size_t smem = BsSmem<T>::total;
  cudaFuncSetAttribute(k_bucket_scatter<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (nblocks)
    k_bucket_scatter<T><<<nblocks, kBsThreads, smem, s>>>(keys_stage, blk_keys, blk_offs, blocks, bucket_off,
                                                          partitions, shift, keys_out, stage_counter, stage_cap);
}
template void launch_bucket_scatter<uint64_t>(const uint64_t*, const unsigned long long*, const unsigned*,
                                              const BlockDesc*, const unsigned long long*, uint32_t, uint32_t,
                                              uint32_t, uint64_t*, const unsigned long long*, unsigned long long,
                                              cudaStream_t);
template void launch_bucket_scatter<u128>(const u128*, const unsigned long long*, const unsigned*, const BlockDesc*,
                                          const unsigned long long*, uint32_t, uint32_t, uint32_t, u128*,
                                          const unsigned long long*, unsigned long long, cudaStream_t);

// Offsets of one input piece's bucket runs (bucket-major inside the piece,
// the piece after the earlier ones): an exclusive scan of the piece's bucket
// counts from *base, the counts added to the bucket totals, *base advanced.
__global__ void __launch_bounds__(256) k_piece_offsets(const unsigned long long* __restrict__ cnt, uint32_t P,
                                                       unsigned long long* __restrict__ base,
                                                       unsigned long long* __restrict__ off,
                                                       unsigned long long* __restrict__ bucket_count) {
  constexpr int NT = 256;
  __shared__ unsigned long long sm[NT / 32 + 2];
  const uint32_t per = (P + NT - 1) / NT, b0 = threadIdx.x * per;
  unsigned long long acc = 0;
  for (uint32_t j = 0; j < per; ++j)
    if (b0 + j < P) acc += cnt[b0 + j];
  const unsigned long long start = *base;  // every thread reads it before the barrier inside the scan
  unsigned long long total;
  unsigned long long at = start + block_exclusive_scan<NT, unsigned long long>(acc, sm, &total);
  for (uint32_t j = 0; j < per; ++j)
    if (b0 + j < P) {
      const unsigned long long c = cnt[b0 + j];
      off[b0 + j] = at;
      bucket_count[b0 + j] += c;
      at += c;
    }
  if (threadIdx.x == 0) *base = start + total;
}

void launch_piece_offsets(const unsigned long long* cnt, uint32_t partitions, unsigned long long* base,
                          unsigned long long* off, unsigned long long* bucket_count, cudaStream_t s) {
  k_piece_offsets<<<1, 256, 0, s>>>(cnt, partitions, base, off, bucket_count);
}

// Batched count: total of bucket b of sample t = the scanned matrix at the
// next sample's first block (or the column total) minus it at this sample's.
__global__ void k_sample_bucket_counts(const unsigned* __restrict__ m, const unsigned long long* __restrict__ col_total,
                                       const uint32_t* __restrict__ sample_first, uint32_t samples, uint32_t P,
                                       uint32_t nblocks, unsigned long long* __restrict__ bucket_count) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= samples * P) return;
  const uint32_t t = i / P, b = i % P;
  const uint32_t f = sample_first[t], nf = sample_first[t + 1];
  const unsigned long long lo = f < nblocks ? m[(size_t)f * P + b] : col_total[b];
  const unsigned long long hi = nf < nblocks ? m[(size_t)nf * P + b] : col_total[b];
  bucket_count[i] = hi - lo;
}

void launch_sample_bucket_counts(const unsigned* m, const unsigned long long* col_total, const uint32_t* sample_first,
                                 uint32_t samples, uint32_t partitions, uint32_t nblocks,
                                 unsigned long long* bucket_count, cudaStream_t s) {
  const uint32_t n = samples * partitions;
  if (n) k_sample_bucket_counts<<<(n + 255) / 256, 256, 0, s>>>(m, col_total, sample_first, samples, partitions, nblocks,
                                                              bucket_count);
}

// Tile list from the scanned part offsets: tile t = (b, j) starts at
// off[t*G] and ends where tile t+1 starts (the last at n_keys).
__global__ void k_make_tiles(const unsigned long long* __restrict__ off, uint32_t ntiles, uint32_t S, uint32_t G,
                             unsigned long long n_keys, TileDesc* __restrict__ tiles, uint32_t* __restrict__ lens) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntiles) return;
  const unsigned long long a = off[(size_t)t * G];
  const unsigned long long e = t + 1 < ntiles ? off[(size_t)(t + 1) * G] : n_keys;
  TileDesc d;
  d.start = a;
  d.len = (uint32_t)(e - a);
  d.bucket = t / S;
  tiles[t] = d;
  lens[t] = d.len;
}

// Region bounds of the next level from a level's scanned part offsets.
__global__ void k_region_bounds(const unsigned long long* __restrict__ off, uint32_t nreg, uint32_t G,
                                unsigned long long n_keys, unsigned long long* __restrict__ roff,
                                unsigned long long* __restrict__ rcnt) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nreg) return;
  const unsigned long long a = off[(size_t)t * G];
  const unsigned long long e = t + 1 < nreg ? off[(size_t)(t + 1) * G] : n_keys;
  roff[t] = a;
  rcnt[t] = e - a;
}

template <class T>
void launch_split_hist(const TileSplitParams<T>& p, cudaStream_t s) {
  if (p.R * p.G) k_split_hist<T><<<p.R * p.G, kSplitThreads, 0, s>>>(p);
}

template <class T, int NT_, int IT_, int RADIX_>
struct ScatterCfg {
  static constexpr int NT = NT_, IT = IT_, RADIX = RADIX_;
};

// Calls f(ScatterCfg<...>{}) for the scatter instance of D digits and launch
// shape 0..3 (threads x keys per thread; 0 picks 256 x 8 for up to 256 digits
// and 512 x 8 above: twice the keys per batch for four times the destinations).
template <class T, class F>
static void with_scatter_cfg(uint32_t D, int shape, F&& f) {
  constexpr int W = sizeof(T) == 8 ? 1 : 2;  // u128 keys: half the keys per thread
  auto by_radix = [&](auto cfg) {
    using C = decltype(cfg);
    if (D <= 16) f(ScatterCfg<T, C::NT, C::IT, 16>{});
    else if (D <= 256) f(ScatterCfg<T, C::NT, C::IT, 256>{});
    else f(ScatterCfg<T, C::NT, C::IT, 1024>{});
  };
  switch (shape) {
    case 1: by_radix(ScatterCfg<T, 256, 16 / W, 0>{}); break;
    case 2: by_radix(ScatterCfg<T, 512, 8 / W, 0>{}); break;
    case 3: by_radix(ScatterCfg<T, 512, 16 / W, 0>{}); break;
    default:
      if (D > 256) by_radix(ScatterCfg<T, 512, 8 / W, 0>{});
      else by_radix(ScatterCfg<T, 256, 8 / W, 0>{});
      break;
  }
}

template <class T>
void launch_split_scatter(const TileSplitParams<T>& p, int shape, cudaStream_t s) {
  with_scatter_cfg<T>(p.D, shape, [&](auto cfg) {
    using C = decltype(cfg);
    if (p.dig) {
      auto kern = k_split_scatter_bulk<T, C::NT, C::IT, C::RADIX>;
      const size_t smem = BulkScatterSmem<T, C::NT, C::IT, C::RADIX>::total;
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (p.R * p.G) kern<<<p.R * p.G, C::NT, smem, s>>>(p);
      return;
    }
    auto kern = k_split_scatter<T, C::NT, C::IT, C::RADIX>;
    const size_t smem = ScatterSmem<T, C::NT, C::IT, C::RADIX>::total;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (p.R * p.G) kern<<<p.R * p.G, C::NT, smem, s>>>(p);
  });
}

template <class T>
uint32_t split_scatter_slots(uint32_t D, int shape) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  with_scatter_cfg<T>(D, shape, [&](auto cfg) {
    using C = decltype(cfg);
    auto kern = k_split_scatter<T, C::NT, C::IT, C::RADIX>;
    const size_t smem = ScatterSmem<T, C::NT, C::IT, C::RADIX>::total;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, C::NT, smem);
  });
  return (uint32_t)std::max(1, sms) * (uint32_t)std::max(1, per_sm);
}

void launch_make_tiles(const unsigned long long* off, uint32_t ntiles, uint32_t S, uint32_t G,
                       unsigned long long n_keys, TileDesc* tiles, uint32_t* lens, cudaStream_t s) {
  if (ntiles) k_make_tiles<<<(ntiles + 255) / 256, 256, 0, s>>>(off, ntiles, S, G, n_keys, tiles, lens);
}

void launch_region_bounds(const unsigned long long* off, uint32_t nreg, uint32_t G, unsigned long long n_keys,
                          unsigned long long* roff, unsigned long long* rcnt, cudaStream_t s) {
  if (nreg) k_region_bounds<<<(nreg + 255) / 256, 256, 0, s>>>(off, nreg, G, n_keys, roff, rcnt);
}

template void launch_split_hist<uint64_t>(const TileSplitParams<uint64_t>&, cudaStream_t);
template void launch_split_hist<u128>(const TileSplitParams<u128>&, cudaStream_t);
template void launch_split_scatter<uint64_t>(const TileSplitParams<uint64_t>&, int, cudaStream_t);
template void launch_split_scatter<u128>(const TileSplitParams<u128>&, int, cudaStream_t);
template uint32_t split_scatter_slots<uint64_t>(uint32_t, int);
template uint32_t split_scatter_slots<u128>(uint32_t, int);

}  // namespace kite
