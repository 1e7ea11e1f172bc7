// Count-path kernels: FASTQ line indexing, rolling k-mer extraction with
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
#include "kite_internal.h"

namespace kite {

static constexpr int kHalo = 64;        // >= k-1 for every k <= 64
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

// ---------------------------------------------------------------------------
// Shared-memory byte layout of a block: block-relative byte rel = pos + kHalo
// - blk_start lives in segment rel >> pts (one thread's range of PT = 1 << pts
// bytes) at a stride of PT + 4 bytes, so the 32 lanes of a warp, each walking
// its own range, read 32 different banks.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t pidx(uint32_t rel, uint32_t pts) {
  return (rel >> pts) * ((1u << pts) + 4u) + (rel & ((1u << pts) - 1u));
}

// Rolling extraction over one thread's byte range.  Warm-up bytes before `ts`
// only seed the window; a newline resets it, so bytes of earlier lines never
// leak into a k-mer.
template <class T, class F>
__device__ __forceinline__ void roll_range(const uint8_t* sb, uint32_t pts, uint64_t blk_start, uint64_t ws,
                                           uint64_t ts, uint64_t te, unsigned phase, bool chunk_ok,
                                           const uint8_t* table, uint32_t k, bool canonical, F&& emit) {
  const T mask = (2 * k == (uint32_t)KeyTraits<T>::kBits) ? ~T(0) : ((T(1) << (2 * k)) - T(1));
  const unsigned rsh = 2 * (k - 1);
  T fwd = 0, rev = 0;
  uint32_t run = 0;
  unsigned ph = phase;
  for (uint64_t pos = ws; pos < te; ++pos) {
    const uint8_t b = sb[pidx((uint32_t)(pos + kHalo - blk_start), pts)];
    if (b == '\n') {
      fwd = 0;
      rev = 0;
      run = 0;
      if (pos >= ts) ph = (ph + 1) & 3;
      continue;
    }
    const uint8_t c = table[b];
    if (!chunk_ok || ph != 1 || c > 3) {
      fwd = 0;
      rev = 0;
      run = 0;
      continue;
    }
    fwd = ((fwd << 2) | T(c)) & mask;
    rev = (rev >> 2) | (T(c ^ 3) << rsh);
    if (++run >= k && pos >= ts) emit(canonical ? (fwd < rev ? fwd : rev) : fwd, pos);
  }
}

__device__ __forceinline__ uint64_t mix64(uint64_t x) {
  x ^= x >> 30;
  x *= 0xbf58476d1ce4e5b9ull;
  x ^= x >> 27;
  x *= 0x94d049bb133111ebull;
  x ^= x >> 31;
  return x;
}

__host__ __device__ __forceinline__ size_t padded_bytes(uint32_t blk_bytes) {
  const size_t pt = blk_bytes / kExtractThreads;
  const size_t segs = ((size_t)kHalo + blk_bytes + 16 + pt - 1) / pt;
  return (segs * (pt + 4) + 15) & ~(size_t)15;
}

size_t extract_smem_bytes(int key_bytes, uint32_t blk_bytes, uint32_t partitions, bool scatter) {
  (void)key_bytes;
  size_t o = padded_bytes(blk_bytes);
  if (scatter) o += (size_t)partitions * 8;  // reservation base (u64)
  o += (size_t)partitions * 4;               // histogram / cursor
  o += 34 * 4 + 256;                         // scan scratch + base table
  return o;
}

// MODE 0: histogram pass (bucket counts, totals, sampling).
// MODE 1: scatter pass (reserve bucket ranges, write keys).
template <class T, int MODE>
__global__ void __launch_bounds__(kExtractThreads) k_extract(ExtractParams<T> p) {
  constexpr int NT = kExtractThreads;
  extern __shared__ __align__(16) uint8_t sm[];
  const uint32_t P = p.partitions;
  uint8_t* sb = sm;
  size_t o = padded_bytes(p.blk_bytes);
  unsigned long long* base = reinterpret_cast<unsigned long long*>(sm + o);
  if (MODE == 1) o += (size_t)P * 8;
  unsigned* hist = reinterpret_cast<unsigned*>(sm + o);
  o += (size_t)P * 4;
  unsigned* scan_sm = reinterpret_cast<unsigned*>(sm + o);
  o += 34 * 4;
  uint8_t* table = sm + o;

  const BlockDesc d = p.blocks[blockIdx.x];
  const uint64_t s = d.start, e = d.end;
  const uint64_t hs = (s - d.chunk_start >= (uint64_t)kHalo) ? s - kHalo : d.chunk_start;
  const uint32_t PT = p.blk_bytes / NT;
  const uint32_t pts = 31 - __clz(PT);
  // coalesced 16-byte loads, stored as four 4-byte words (PT >= 4, so a word
  // never straddles a segment and its padded address stays 4-byte aligned)
  for (uint64_t w = (hs >> 4) + threadIdx.x; w < ((e + 15) >> 4); w += NT) {
    const uint4 v = reinterpret_cast<const uint4*>(p.arena)[w];
    const uint32_t rel = (uint32_t)(w * 16 + kHalo - s);
    *reinterpret_cast<uint32_t*>(sb + pidx(rel, pts)) = v.x;
    *reinterpret_cast<uint32_t*>(sb + pidx(rel + 4, pts)) = v.y;
    *reinterpret_cast<uint32_t*>(sb + pidx(rel + 8, pts)) = v.z;
    *reinterpret_cast<uint32_t*>(sb + pidx(rel + 12, pts)) = v.w;
  }
  for (int i = threadIdx.x; i < 256; i += NT) {
    uint8_t v = 255;
    if (i == 'A' || i == 'a') v = 0;
    else if (i == 'C' || i == 'c') v = 1;
    else if (i == 'G' || i == 'g') v = 2;
    else if (i == 'T' || i == 't') v = 3;
    table[i] = v;
  }
  for (uint32_t b = threadIdx.x; b < P; b += NT) hist[b] = 0;
  __syncthreads();

  const uint64_t ts = s + (uint64_t)threadIdx.x * PT;
  const uint64_t te = ts < e ? (ts + PT < e ? ts + PT : e) : ts;
  unsigned nl = 0;
  for (uint64_t pos = ts; pos < te; ++pos) nl += sb[pidx((uint32_t)(pos + kHalo - s), pts)] == '\n';
  unsigned nl_total;
  const unsigned nl_before = block_exclusive_scan<NT, unsigned>(nl, scan_sm, &nl_total);
  const unsigned long long line0 = p.block_nl_excl[blockIdx.x] - p.block_nl_excl[d.first_block];
  const unsigned phase = (unsigned)((line0 + nl_before) & 3ull);
  const bool chunk_ok = p.arena[d.chunk_start] == '@';  // src/count/parser.rs:27-29
  const uint64_t ws = (ts - hs >= p.k - 1) ? ts - (p.k - 1) : hs;
  const bool canon = p.canonical != 0;
  const uint32_t shift = p.shift;

  if (MODE == 0) {
    unsigned long long kmers = 0;
    const bool sampling = p.sample != nullptr && (d.flags & 2u);
    roll_range<T>(sb, pts, s, ws, ts, te, phase, chunk_ok, table, p.k, canon, [&](T key, uint64_t pos) {
      kmers++;
      atomicAdd(&hist[bucket_of(key, shift)], 1u);
      if (sampling && (mix64(pos) & p.sample_mask) == 0) {
        const unsigned idx = atomicAdd(p.sample_count, 1u);
        if (idx < p.sample_cap) p.sample[idx] = key;
      }
    });
    // reads / bases of this thread's range
    unsigned long long reads = 0, bases = 0;
    if (chunk_ok) {
      unsigned ph = phase;
      uint8_t prev = ts > d.chunk_start ? sb[pidx((uint32_t)(ts - 1 + kHalo - s), pts)] : (uint8_t)'\n';
      for (uint64_t pos = ts; pos < te; ++pos) {
        const uint8_t b = sb[pidx((uint32_t)(pos + kHalo - s), pts)];
        if (b == '\n') {
          ph = (ph + 1) & 3;
        } else if (ph == 1) {
          bases++;
          reads += prev == '\n';
        }
        prev = b;
      }
    }
    __syncthreads();
    for (uint32_t b = threadIdx.x; b < P; b += NT)
      if (hist[b]) atomicAdd(&p.bucket_count[b], (unsigned long long)hist[b]);
    // warp-aggregated totals
    for (int o2 = 16; o2; o2 >>= 1) {
      kmers += __shfl_xor_sync(0xffffffffu, kmers, o2);
      reads += __shfl_xor_sync(0xffffffffu, reads, o2);
      bases += __shfl_xor_sync(0xffffffffu, bases, o2);
    }
    if ((threadIdx.x & 31) == 0) {
      if (kmers) atomicAdd(&p.totals->kmers, kmers);
      if (reads) atomicAdd(&p.totals->reads, reads);
      if (bases) atomicAdd(&p.totals->bases, bases);
    }
  } else {
    roll_range<T>(sb, pts, s, ws, ts, te, phase, chunk_ok, table, p.k, canon,
                  [&](T key, uint64_t) { atomicAdd(&hist[bucket_of(key, shift)], 1u); });
    __syncthreads();
    for (uint32_t b = threadIdx.x; b < P; b += NT) {
      const unsigned h = hist[b];
      unsigned long long r = 0;
      if (h) {
        r = atomicAdd(&p.bucket_fill[b], (unsigned long long)h);
        if (r + h > p.bucket_count[b]) {
          dev_fail(p.status, KITE_DEV_REGION_OVERFLOW, b, (unsigned)r, h);
          r = ~0ull;
        }
      }
      base[b] = r;
      hist[b] = 0;
    }
    __syncthreads();
    roll_range<T>(sb, pts, s, ws, ts, te, phase, chunk_ok, table, p.k, canon, [&](T key, uint64_t) {
      const uint32_t b = bucket_of(key, shift);
      const unsigned slot = atomicAdd(&hist[b], 1u);
      const unsigned long long r = base[b];
      if (r != ~0ull) p.keys_out[p.bucket_off[b] + r + slot] = key;
    });
  }
}

template <class T>
void launch_extract_hist(const ExtractParams<T>& p, uint32_t nblocks, cudaStream_t s) {
  const size_t smem = extract_smem_bytes(sizeof(T), p.blk_bytes, p.partitions, false);
  cudaFuncSetAttribute(k_extract<T, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (nblocks) k_extract<T, 0><<<nblocks, kExtractThreads, smem, s>>>(p);
}
template <class T>
void launch_extract_scatter(const ExtractParams<T>& p, uint32_t nblocks, cudaStream_t s) {
  const size_t smem = extract_smem_bytes(sizeof(T), p.blk_bytes, p.partitions, true);
  cudaFuncSetAttribute(k_extract<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (nblocks) k_extract<T, 1><<<nblocks, kExtractThreads, smem, s>>>(p);
}
template void launch_extract_hist<uint64_t>(const ExtractParams<uint64_t>&, uint32_t, cudaStream_t);
template void launch_extract_hist<u128>(const ExtractParams<u128>&, uint32_t, cudaStream_t);
template void launch_extract_scatter<uint64_t>(const ExtractParams<uint64_t>&, uint32_t, cudaStream_t);
template void launch_extract_scatter<u128>(const ExtractParams<u128>&, uint32_t, cudaStream_t);

// ---------------------------------------------------------------------------
// Level-2 split: inside every hash bucket, route keys to S key-range tiles by
// the splitters (upper bound = number of splitters <= key).  Tiles are laid
// out bucket-major, so each bucket's tiles stay contiguous and in key order.
// Each bucket is cut into G parts; part (b, g) owns the sub-range
// [off[(b*S+j)*G+g], +cnt) of tile (b, j), so no two CTAs share a cursor and
// the only atomics are shared-memory ones.
// ---------------------------------------------------------------------------
// Tile of a key = number of splitters <= key.  A lookup table over the top
// kLutBits of the key gives the number of splitters below the key's bin; a
// short forward scan covers the splitters inside the bin (exact for any
// ascending splitters).
static constexpr int kLutBits = 12;

template <class T>
__device__ __forceinline__ uint32_t tile_of(const T* spl, const uint16_t* lut, uint32_t lut_shift, uint32_t S,
                                            T key) {
  uint32_t j = lut[(uint32_t)(uint64_t)(key >> lut_shift)];
  while (j + 1 < S && spl[j] <= key) ++j;
  return j;
}

// Loads the splitters and builds the table (block-wide; ends with a barrier).
template <class T>
__device__ __forceinline__ void load_splitters(const T* g_spl, uint32_t S, uint32_t key_bits, T* spl, uint16_t* lut,
                                               uint32_t* lut_shift) {
  for (uint32_t i = threadIdx.x; i + 1 < S; i += blockDim.x) spl[i] = g_spl[i];
  __syncthreads();
  const uint32_t L = key_bits < (uint32_t)kLutBits ? key_bits : (uint32_t)kLutBits;
  *lut_shift = key_bits - L;
  for (uint32_t bin = threadIdx.x; bin < (1u << L); bin += blockDim.x) {
    const T start = (T)bin << *lut_shift;
    uint32_t lo = 0, hi = S - 1;  // lower_bound over S-1 splitters
    while (lo < hi) {
      const uint32_t mid = (lo + hi) >> 1;
      if (spl[mid] < start) lo = mid + 1;
      else hi = mid;
    }
    lut[bin] = (uint16_t)lo;
  }
  __syncthreads();
}

static constexpr size_t kLutBytes = ((size_t)(1u << kLutBits) * 2 + 15) & ~(size_t)15;

static constexpr int kSplitThreads = 512;
static constexpr int kSplitUnroll = 8;

__device__ __forceinline__ void part_range(const unsigned long long* boff, const unsigned long long* bcnt,
                                           uint32_t b, uint32_t g, uint32_t G, uint64_t* lo, uint64_t* hi) {
  const uint64_t n = bcnt[b], base = boff[b];
  *lo = base + n * g / G;
  *hi = base + n * (g + 1) / G;
}

template <class T>
__global__ void __launch_bounds__(kSplitThreads) k_tile_hist(TileSplitParams<T> p) {
  extern __shared__ __align__(16) uint8_t sm[];
  const uint32_t S = p.S, G = p.G;
  T* spl = reinterpret_cast<T*>(sm);
  uint16_t* lut = reinterpret_cast<uint16_t*>(sm + (size_t)S * sizeof(T));
  unsigned* hist = reinterpret_cast<unsigned*>(sm + (size_t)S * sizeof(T) + kLutBytes);
  const uint32_t b = blockIdx.x / G, g = blockIdx.x % G;
  for (uint32_t i = threadIdx.x; i < S; i += blockDim.x) hist[i] = 0;
  uint32_t lsh;
  load_splitters(p.splitters, S, p.key_bits, spl, lut, &lsh);
  uint64_t lo, hi;
  part_range(p.bucket_off, p.bucket_count, b, g, G, &lo, &hi);
  // kSplitUnroll independent loads in flight per thread before any use
  for (uint64_t i0 = lo + threadIdx.x; i0 < hi; i0 += (uint64_t)kSplitThreads * kSplitUnroll) {
    T key[kSplitUnroll];
#pragma unroll
    for (int u = 0; u < kSplitUnroll; ++u) {
      const uint64_t i = i0 + (uint64_t)u * kSplitThreads;
      key[u] = i < hi ? p.keys_in[i] : T(0);
    }
#pragma unroll
    for (int u = 0; u < kSplitUnroll; ++u)
      if (i0 + (uint64_t)u * kSplitThreads < hi) atomicAdd(&hist[tile_of(spl, lut, lsh, S, key[u])], 1u);
  }
  __syncthreads();
  for (uint32_t j = threadIdx.x; j < S; j += blockDim.x)
    p.tile_count[((size_t)b * S + j) * G + g] = hist[j];
}

template <class T>
__global__ void __launch_bounds__(kSplitThreads) k_tile_scatter(TileSplitParams<T> p) {
  extern __shared__ __align__(16) uint8_t sm[];
  const uint32_t S = p.S, G = p.G;
  unsigned long long* base = reinterpret_cast<unsigned long long*>(sm);
  T* spl = reinterpret_cast<T*>(base + S);
  uint16_t* lut = reinterpret_cast<uint16_t*>(sm + (size_t)S * 8 + (size_t)S * sizeof(T));
  unsigned* cur = reinterpret_cast<unsigned*>(sm + (size_t)S * 8 + (size_t)S * sizeof(T) + kLutBytes);
  const uint32_t b = blockIdx.x / G, g = blockIdx.x % G;
  for (uint32_t j = threadIdx.x; j < S; j += blockDim.x) {
    base[j] = p.tile_off[((size_t)b * S + j) * G + g];
    cur[j] = 0;
  }
  uint32_t lsh;
  load_splitters(p.splitters, S, p.key_bits, spl, lut, &lsh);
  uint64_t lo, hi;
  part_range(p.bucket_off, p.bucket_count, b, g, G, &lo, &hi);
  for (uint64_t i0 = lo + threadIdx.x; i0 < hi; i0 += (uint64_t)kSplitThreads * kSplitUnroll) {
    T key[kSplitUnroll];
#pragma unroll
    for (int u = 0; u < kSplitUnroll; ++u) {
      const uint64_t i = i0 + (uint64_t)u * kSplitThreads;
      key[u] = i < hi ? p.keys_in[i] : T(0);
    }
#pragma unroll
    for (int u = 0; u < kSplitUnroll; ++u) {
      if (i0 + (uint64_t)u * kSplitThreads >= hi) break;
      const uint32_t j = tile_of(spl, lut, lsh, S, key[u]);
      const unsigned slot = atomicAdd(&cur[j], 1u);
      p.keys_out[base[j] + slot] = key[u];
    }
  }
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

size_t tile_split_smem(int key_bytes, uint32_t S, bool scatter) {
  return (scatter ? (size_t)S * 8 : 0) + (size_t)S * key_bytes + kLutBytes + (size_t)S * 4;
}

template <class T>
void launch_tile_hist(const TileSplitParams<T>& p, cudaStream_t s) {
  const size_t smem = tile_split_smem(sizeof(T), p.S, false);
  cudaFuncSetAttribute(k_tile_hist<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k_tile_hist<T><<<p.P * p.G, kSplitThreads, smem, s>>>(p);
}

template <class T>
void launch_tile_scatter(const TileSplitParams<T>& p, cudaStream_t s) {
  const size_t smem = tile_split_smem(sizeof(T), p.S, true);
  cudaFuncSetAttribute(k_tile_scatter<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k_tile_scatter<T><<<p.P * p.G, kSplitThreads, smem, s>>>(p);
}

void launch_make_tiles(const unsigned long long* off, uint32_t ntiles, uint32_t S, uint32_t G,
                       unsigned long long n_keys, TileDesc* tiles, uint32_t* lens, cudaStream_t s) {
  if (ntiles) k_make_tiles<<<(ntiles + 255) / 256, 256, 0, s>>>(off, ntiles, S, G, n_keys, tiles, lens);
}

template void launch_tile_hist<uint64_t>(const TileSplitParams<uint64_t>&, cudaStream_t);
template void launch_tile_hist<u128>(const TileSplitParams<u128>&, cudaStream_t);
template void launch_tile_scatter<uint64_t>(const TileSplitParams<uint64_t>&, cudaStream_t);
template void launch_tile_scatter<u128>(const TileSplitParams<u128>&, cudaStream_t);

}  // namespace kite
