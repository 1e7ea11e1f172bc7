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
// Rolling extraction over one thread's byte range.  `sb` is indexed by
// (pos + kHalo - blk_start).  Warm-up bytes before `ts` only seed the window;
// a newline resets it, so bytes of earlier lines never leak into a k-mer.
// ---------------------------------------------------------------------------
template <class T, class F>
__device__ __forceinline__ void roll_range(const uint8_t* sb, uint64_t blk_start, uint64_t ws, uint64_t ts,
                                           uint64_t te, unsigned phase, bool chunk_ok, const uint8_t* table,
                                           uint32_t k, bool canonical, F&& emit) {
  const T mask = (2 * k == (uint32_t)KeyTraits<T>::kBits) ? ~T(0) : ((T(1) << (2 * k)) - T(1));
  const unsigned rsh = 2 * (k - 1);
  T fwd = 0, rev = 0;
  uint32_t run = 0;
  unsigned ph = phase;
  for (uint64_t pos = ws; pos < te; ++pos) {
    const uint8_t b = sb[pos + kHalo - blk_start];
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

size_t extract_smem_bytes(int key_bytes, uint32_t blk_bytes, uint32_t partitions, bool scatter) {
  (void)key_bytes;
  size_t o = ((size_t)kHalo + blk_bytes + 16 + 15) & ~(size_t)15;
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
  size_t o = ((size_t)kHalo + p.blk_bytes + 16 + 15) & ~(size_t)15;
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
  for (uint64_t w = (hs >> 4) + threadIdx.x; w < ((e + 15) >> 4); w += NT)
    *reinterpret_cast<uint4*>(sb + (w * 16 + kHalo - s)) = reinterpret_cast<const uint4*>(p.arena)[w];
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

  const uint32_t PT = p.blk_bytes / NT;
  const uint64_t ts = s + (uint64_t)threadIdx.x * PT;
  const uint64_t te = ts < e ? (ts + PT < e ? ts + PT : e) : ts;
  unsigned nl = 0;
  for (uint64_t pos = ts; pos < te; ++pos) nl += sb[pos + kHalo - s] == '\n';
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
    roll_range<T>(sb, s, ws, ts, te, phase, chunk_ok, table, p.k, canon, [&](T key, uint64_t pos) {
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
      uint8_t prev = ts > d.chunk_start ? sb[ts - 1 + kHalo - s] : (uint8_t)'\n';
      for (uint64_t pos = ts; pos < te; ++pos) {
        const uint8_t b = sb[pos + kHalo - s];
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
    roll_range<T>(sb, s, ws, ts, te, phase, chunk_ok, table, p.k, canon,
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
    roll_range<T>(sb, s, ws, ts, te, phase, chunk_ok, table, p.k, canon, [&](T key, uint64_t) {
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
// ---------------------------------------------------------------------------
template <class T>
__device__ __forceinline__ uint32_t tile_of(const T* spl, uint32_t S, T key) {
  uint32_t j = 0;
  for (uint32_t step = S >> 1; step; step >>= 1)
    if (spl[j + step - 1] <= key) j += step;
  return j;
}

static constexpr int kSplitThreads = 256;

template <class T>
__global__ void __launch_bounds__(kSplitThreads) k_tile_hist(TileSplitParams<T> p) {
  extern __shared__ __align__(16) uint8_t sm[];
  const uint32_t S = p.S;
  T* spl = reinterpret_cast<T*>(sm);
  unsigned* hist = reinterpret_cast<unsigned*>(spl + S);
  const SliceDesc sl = p.slices[blockIdx.x];
  for (uint32_t i = threadIdx.x; i + 1 < S; i += blockDim.x) spl[i] = p.splitters[i];
  for (uint32_t i = threadIdx.x; i < S; i += blockDim.x) hist[i] = 0;
  __syncthreads();
  const T* src = p.keys_in + sl.start;
  for (uint32_t i = threadIdx.x; i < sl.len; i += blockDim.x) atomicAdd(&hist[tile_of(spl, S, src[i])], 1u);
  __syncthreads();
  unsigned long long* tc = p.tile_count + (size_t)sl.bucket * S;
  for (uint32_t j = threadIdx.x; j < S; j += blockDim.x)
    if (hist[j]) atomicAdd(&tc[j], (unsigned long long)hist[j]);
}

template <class T, int ITEMS>
__global__ void __launch_bounds__(kSplitThreads) k_tile_scatter(TileSplitParams<T> p) {
  extern __shared__ __align__(16) uint8_t sm[];
  const uint32_t S = p.S;
  unsigned long long* base = reinterpret_cast<unsigned long long*>(sm);
  T* spl = reinterpret_cast<T*>(base + S);
  unsigned* hist = reinterpret_cast<unsigned*>(spl + S);
  const SliceDesc sl = p.slices[blockIdx.x];
  for (uint32_t i = threadIdx.x; i + 1 < S; i += blockDim.x) spl[i] = p.splitters[i];
  for (uint32_t i = threadIdx.x; i < S; i += blockDim.x) hist[i] = 0;
  __syncthreads();
  const T* src = p.keys_in + sl.start;
  T key[ITEMS];
  uint32_t tj[ITEMS];
#pragma unroll
  for (int r = 0; r < ITEMS; ++r) {
    const uint32_t i = r * kSplitThreads + threadIdx.x;
    tj[r] = 0xffffffffu;
    if (i < sl.len) {
      key[r] = src[i];
      tj[r] = tile_of(spl, S, key[r]);
      atomicAdd(&hist[tj[r]], 1u);
    }
  }
  __syncthreads();
  const size_t tb = (size_t)sl.bucket * S;
  for (uint32_t j = threadIdx.x; j < S; j += blockDim.x) {
    const unsigned h = hist[j];
    unsigned long long r = 0;
    if (h) {
      r = atomicAdd(&p.tile_fill[tb + j], (unsigned long long)h);
      if (r + h > p.tile_count[tb + j]) {
        dev_fail(p.status, KITE_DEV_REGION_OVERFLOW, (unsigned)(tb + j), (unsigned)r, h);
        r = ~0ull;
      } else {
        r += p.tile_off[tb + j];
      }
    }
    base[j] = r;
    hist[j] = 0;
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < ITEMS; ++r) {
    if (tj[r] != 0xffffffffu) {
      const unsigned slot = atomicAdd(&hist[tj[r]], 1u);
      const unsigned long long b0 = base[tj[r]];
      if (b0 != ~0ull) p.keys_out[b0 + slot] = key[r];
    }
  }
}

template <class T>
void launch_tile_hist(const TileSplitParams<T>& p, uint32_t nslices, uint32_t, cudaStream_t s) {
  const size_t smem = (size_t)p.S * sizeof(T) + (size_t)p.S * 4;
  cudaFuncSetAttribute(k_tile_hist<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (nslices) k_tile_hist<T><<<nslices, kSplitThreads, smem, s>>>(p);
}

template <class T>
constexpr int split_items() { return sizeof(T) == 8 ? 16 : 8; }

uint32_t split_slice_keys(int key_bytes) { return kSplitThreads * (key_bytes == 8 ? 16 : 8); }

template <class T>
void launch_tile_scatter(const TileSplitParams<T>& p, uint32_t nslices, uint32_t, cudaStream_t s) {
  const size_t smem = (size_t)p.S * 8 + (size_t)p.S * sizeof(T) + (size_t)p.S * 4;
  cudaFuncSetAttribute(k_tile_scatter<T, split_items<T>()>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)smem);
  if (nslices) k_tile_scatter<T, split_items<T>()><<<nslices, kSplitThreads, smem, s>>>(p);
}
template void launch_tile_hist<uint64_t>(const TileSplitParams<uint64_t>&, uint32_t, uint32_t, cudaStream_t);
template void launch_tile_hist<u128>(const TileSplitParams<u128>&, uint32_t, uint32_t, cudaStream_t);
template void launch_tile_scatter<uint64_t>(const TileSplitParams<uint64_t>&, uint32_t, uint32_t, cudaStream_t);
template void launch_tile_scatter<u128>(const TileSplitParams<u128>&, uint32_t, uint32_t, cudaStream_t);

}  // namespace kite
