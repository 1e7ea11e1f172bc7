// On-chip tile sort + run-length reduction (the sort/RLE of a flushed bucket:
// radix_sort_u64_kmer / radix_sort_u128_kmer src/count/sorter.rs:67-93,
// :388-437, then rle_compress_typed :514-530 with u32 saturation).
//
// A tile is a key range of one hash bucket.  One CTA loads the whole tile into
// shared memory, orders it by a 16384-bin counting pass over its key span (bins
// holding several distinct keys are finished by a thread or a warp, rare
// pathological ones by LSD passes), then emits unique (key, count) rows in
// place and the tile's DVLE size for every row but the first.
#include "kite_internal.h"

namespace kite {

template <class T>
__device__ __forceinline__ T warp_min(T v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    const T w = shfl_xor_key(v, o);
    v = w < v ? w : v;
  }
  return v;
}
template <class T>
__device__ __forceinline__ T warp_max(T v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    const T w = shfl_xor_key(v, o);
    v = w > v ? w : v;
  }
  return v;
}

// Block-wide min and max of the thread values (smem needs 2*NW keys).
template <int NT, class T>
__device__ __forceinline__ void block_minmax(T& mn, T& mx, T* red) {
  constexpr int NW = NT / 32;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  mn = warp_min(mn);
  mx = warp_max(mx);
  if (lane == 0) {
    red[wid] = mn;
    red[NW + wid] = mx;
  }
  __syncthreads();
  mn = red[0];
  mx = red[NW];
  for (int w = 1; w < NW; ++w) {
    mn = red[w] < mn ? red[w] : mn;
    mx = red[NW + w] > mx ? red[NW + w] : mx;
  }
  __syncthreads();
}

template <class T>
__device__ __forceinline__ int varying_bits(T mn, T mx) {
  const T x = mn ^ mx;
  return x == T(0) ? 0 : KeyTraits<T>::kBits - clz_key(x);
}

template <class T>
struct TileSmem {
  static constexpr int NT = kTileThreads;
  static constexpr int ITEMS = tile_items<T>();
  static constexpr int CAP = NT * ITEMS;
  static constexpr int NW = NT / 32;
  static constexpr size_t buf_bytes = (size_t)CAP * sizeof(T);
  static constexpr size_t hist_bytes = (size_t)256 * NW * 4;
  static constexpr size_t head_bytes = ((size_t)(CAP + 1) * 2 + 15) & ~(size_t)15;
  static constexpr size_t misc_bytes = 64 * 8 + 2 * NW * sizeof(T) + 256 * 8;
  static constexpr size_t total = buf_bytes + hist_bytes + head_bytes + misc_bytes;
};

// Stable LSD passes over bits [lo_bit, nbits) of the n keys in buf (shared
// memory), 8-bit digits.
template <class T, int NT, int ITEMS>
__device__ __forceinline__ void smem_radix_sort(T* buf, unsigned n, int nbits, unsigned* warp_hist,
                                                unsigned* scan_sm, int lo_bit = 0) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  // spread the n keys over every warp: `items` rounds of 32 per warp
  const int items = (int)((n + NT - 1) / NT);
  const unsigned pos0 = (unsigned)wid * 32u * (unsigned)items + lane;
  for (int shift = lo_bit; shift < nbits; shift += 8) {
    T key[ITEMS];
    unsigned dig[ITEMS], dest[ITEMS];
    bool valid[ITEMS];
#pragma unroll
    for (int r = 0; r < ITEMS; ++r) {
      const unsigned pos = pos0 + r * 32u;
      valid[r] = r < items && pos < n;
      key[r] = valid[r] ? buf[pos] : T(0);
      dig[r] = digit_of(key[r], shift);
    }
    block_rank<NT, ITEMS, 256>(dig, valid, dest, warp_hist, scan_sm, nullptr, nullptr, items);
#pragma unroll
    for (int r = 0; r < ITEMS; ++r)
      if (valid[r]) buf[dest[r]] = key[r];
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Tile sort by binning.  One CTA per tile of n <= CAP keys:
//  1. load the tile into shared memory (one bulk copy), then count the keys per bin:
//     bin = (key - lo) >> s with 16384 bins spanning the tile's key range
//     [lo, hi] (its splitters);
//  2. an exclusive scan of the bin counts; then the keys themselves are
//     scattered into bin order (every thread first takes its keys from the
//     staged tile into registers, so none is overwritten before it is read).
//     Bins are key-ordered; order inside a bin is arbitrary, so every later
//     pass reads shared memory directly;
//  3. a bin holding more than one distinct key is found where two different
//     neighbours share it, and marked (a shared bit per bin);
//  4. a marked bin of at most kSmallBin keys (typically two colliding
//     k-mers) is insertion-sorted by the thread owning its bit; a larger one
//     (typically a repeated k-mer and a colliding one) by the warp owning its
//     bit word.  Up to 32 keys sit one per lane: lanes with equal keys find
//     each other by a match, and each key's new position is the copies of
//     the smaller distinct keys plus its equal predecessors.  A larger bin
//     has its distinct keys extracted in ascending order with their counts
//     and is rewritten with them (equal keys are interchangeable).  A bin of
//     more than kMaxDistinct distinct keys is ranked by counting when it
//     holds at most kMaxMixed keys and otherwise sends the tile to LSD passes;
//  5. run-length reduction over the sorted keys: head flags by warp ballots,
//     rows written to global memory over the tile's keys (u32 counts; a tile
//     holds fewer than 2^32 keys, so no count saturates here).
// ---------------------------------------------------------------------------
// 16384 bins with 16-bit counters packed two to a word (a tile holds at most
// 16384 keys, so no half carries into the other)
constexpr int kBinBits = 14, kBins = 1 << kBinBits;
constexpr unsigned kSmallBin = 16;     // marked bins a single thread sorts
constexpr unsigned kMaxMixed = 256;    // largest bin ranked by counting when it has many distinct keys
constexpr unsigned kMaxDistinct = 32;  // distinct keys a warp extracts from one large bin
constexpr int kLoadBatch = 8;          // global loads a thread keeps in flight

// MULT = 1: the regular tile (8192 u64 / 4096 u128 keys, two CTAs per SM);
// MULT = 2: twice that, with twice the threads, for the oversized tiles (one
// CTA per SM).
template <class T, int MULT>
struct BinSmem {
  static constexpr int NT = kTileThreads * MULT;
  static constexpr int ITEMS = tile_items<T>();
  static constexpr int CAP = NT * ITEMS;
  static constexpr int NW = NT / 32;
  // the keys, plus 16 bytes: the bulk copy of a tile starts at the 16-byte
  // boundary at or below its first key
  static constexpr size_t buf_bytes = (size_t)CAP * sizeof(T) + 16;
  // bin counters; later the u16 run heads (CAP + 1 entries), or the LSD
  // fallback's per-warp digit histograms (256 * NW counters)
  static constexpr size_t head_need = ((size_t)(CAP + 1) * 2 + 15) & ~(size_t)15;
  static constexpr size_t bin_bytes = ((size_t)kBins * 2 > head_need ? (size_t)kBins * 2 : head_need) + 16;
  static constexpr size_t fbit_bytes = kBins / 8;
  static constexpr unsigned MAXLARGE = CAP / (kSmallBin + 1) + 1;  // marked bins above kSmallBin keys
  static constexpr size_t misc_bytes = 64 * 8 + 16 + ((MAXLARGE * 2 + 15) & ~(size_t)15) + 16;  // + mbarrier
  static constexpr size_t total = buf_bytes + bin_bytes + fbit_bytes + misc_bytes;
  static_assert((size_t)(CAP + 1) * 2 <= bin_bytes, "run heads must fit the bin area");
  static_assert((size_t)256 * NW * 4 <= bin_bytes, "LSD histograms must fit the bin area");
  static_assert(kBins / 2 % (4 * NT) == 0, "bin scan takes whole uint4 groups");
  static_assert(CAP <= 65535, "bin offsets fit 16 bits");
  static_assert(kBins % (32 * NW) == 0, "every warp owns whole words of bin marks");
  static_assert(kBins % NT == 0 && kBins / NT <= 32 && 32 % (kBins / NT) == 0, "every thread owns bin marks in one word");
};

template <class T>
__device__ __forceinline__ unsigned bin_of(T key, T mn, int s) {
  return (unsigned)(uint64_t)((key - mn) >> s);
}

// Packed 16-bit bin counters: bin b is half (b & 1) of word b >> 1.
__device__ __forceinline__ unsigned bin_add(unsigned* bins, unsigned b) {
  const unsigned sh = (b & 1u) << 4;
  return (atomicAdd(&bins[b >> 1], 1u << sh) >> sh) & 0xffffu;
}
__device__ __forceinline__ unsigned bin_get(const unsigned* bins, unsigned b) {
  return (bins[b >> 1] >> ((b & 1u) << 4)) & 0xffffu;
}

template <class T>
__device__ __forceinline__ unsigned match_key(T v) {
  unsigned eq = __match_any_sync(0xffffffffu, (unsigned long long)(uint64_t)v);
  if (sizeof(T) > 8) eq &= __match_any_sync(0xffffffffu, (unsigned long long)hi64(v));
  return eq;
}

// One warp orders buf[a, a + m), m <= 32, one key per lane: a key's new
// position is the copies of the smaller distinct keys (one shuffle per
// distinct key, from its lowest lane) plus its equal predecessors.
template <class T>
__device__ __forceinline__ void warp_match_sort(T* buf, unsigned a, unsigned m, unsigned lane) {
  const bool act = lane < m;
  const T mine = act ? buf[a + lane] : T(0);
  const unsigned amask = m >= 32 ? 0xffffffffu : ((1u << m) - 1u);
  const unsigned eq = match_key(mine) & amask;
  const unsigned leaders = __ballot_sync(0xffffffffu, act && (unsigned)(__ffs(eq) - 1) == lane);
  const unsigned cnt = __popc(eq);
  unsigned less = 0;
  for (unsigned L = leaders; L; L &= L - 1) {
    const int l = __ffs(L) - 1;
    const T kl = shfl_key(mine, l);
    const unsigned cl = __shfl_sync(0xffffffffu, cnt, l);
    less += kl < mine ? cl : 0u;
  }
  const unsigned pos = a + less + __popc(eq & ((1u << lane) - 1u));
  __syncwarp();
  if (act) buf[pos] = mine;
  __syncwarp();
}

// One warp orders buf[a, a + m), m <= kMaxMixed, by counting: each key's new
// position is the number of smaller keys plus the equal keys before it.
template <class T>
__device__ __forceinline__ void warp_count_sort(T* buf, unsigned a, unsigned m, unsigned lane) {
  constexpr int R = kMaxMixed / 32;
  T key[R];
  unsigned rk[R];
#pragma unroll
  for (int i = 0; i < R; ++i) {
    const unsigned q = lane + 32u * i;
    key[i] = q < m ? buf[a + q] : T(0);
    rk[i] = 0;
  }
  for (unsigned t = 0; t < m; ++t) {
    const T v = buf[a + t];
#pragma unroll
    for (int i = 0; i < R; ++i) rk[i] += (unsigned)(v < key[i]) | ((unsigned)(v == key[i]) & (unsigned)(t < lane + 32u * i));
  }
  __syncwarp();
#pragma unroll
  for (int i = 0; i < R; ++i)
    if (lane + 32u * i < m) buf[a + rk[i]] = key[i];
  __syncwarp();
}

// One warp orders buf[a, a + m) by extracting its distinct keys in ascending
// order with their counts and rewriting the range with them.  False (range
// untouched) when the range holds more than kMaxDistinct distinct keys.
template <class T>
__device__ __forceinline__ bool warp_distinct_sort(T* buf, unsigned a, unsigned m, unsigned lane) {
  const unsigned e = a + m;
  T myv = T(0), cur = T(0);
  unsigned myc = 0, U = 0;
  bool have = false;
  for (;;) {
    // smallest key above `cur` in the range, and its number of copies
    T best = T(0);
    unsigned cnt = 0;
    for (unsigned j = a + lane; j < e; j += 32) {
      const T v = buf[j];
      if (have && !(cur < v)) continue;
      if (cnt == 0 || v < best) {
        best = v;
        cnt = 1;
      } else if (v == best) {
        ++cnt;
      }
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      const T ob = shfl_xor_key(best, o);
      const unsigned oc = __shfl_xor_sync(0xffffffffu, cnt, o);
      if (oc && (cnt == 0 || ob < best)) {
        best = ob;
        cnt = oc;
      } else if (oc && ob == best) {
        cnt += oc;
      }
    }
    if (cnt == 0) break;
    if (U == kMaxDistinct) return false;
    if (lane == U) {
      myv = best;
      myc = cnt;
    }
    ++U;
    cur = best;
    have = true;
  }
  __syncwarp();
  unsigned off = a;
  for (unsigned u = 0; u < U; ++u) {
    const T v = shfl_key(myv, (int)u);
    const unsigned c = __shfl_sync(0xffffffffu, myc, (int)u);
    for (unsigned t = lane; t < c; t += 32) buf[off + t] = v;
    off += c;
  }
  __syncwarp();
  return true;
}

// ---- bulk (TMA) copy of a tile's keys into shared memory, completed on an
// mbarrier (PTX cp.async.bulk / mbarrier) ----
__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  // earlier generic-proxy accesses to the destination come before the copy
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               ::"r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}
// Waits for phase `parity` of the barrier, giving up after `limit` polls
// (each a try_wait, which may suspend the thread for a while); limit 1 is a
// single non-blocking test.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t limit) {
  if (limit == 1) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return done != 0;
  }
  for (uint32_t it = 0; it < limit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}
constexpr uint32_t kBulkWaitPolls = 1u << 18;                // a bulk copy from device memory ends long before
constexpr uint32_t kBulkDrainPolls = 1u << 26;               // after a timeout: the copy must leave shared memory
constexpr unsigned long long kBulkTimeoutFlag = 1ull << 40;  // added to the sort statistics on a timeout

template <class T, int MULT>
__device__ __forceinline__ void sort_tile(uint32_t tid, T* __restrict__ keys, uint32_t* __restrict__ counts,
                                          const TileDesc* __restrict__ tiles, TileOut<T>* __restrict__ tout,
                                          unsigned long long* fallbacks, const TileRanges<T>& rg) {
  using L = BinSmem<T, MULT>;
  constexpr int NT = L::NT, NW = L::NW, ITEMS = L::ITEMS;
  extern __shared__ __align__(16) uint8_t sm[];
  T* buf = reinterpret_cast<T*>(sm);
  unsigned* bins = reinterpret_cast<unsigned*>(sm + L::buf_bytes);
  unsigned* fbits = reinterpret_cast<unsigned*>(sm + L::buf_bytes + L::bin_bytes);
  unsigned long long* scan64 = reinterpret_cast<unsigned long long*>(sm + L::buf_bytes + L::bin_bytes + L::fbit_bytes);
  unsigned* scan_sm = reinterpret_cast<unsigned*>(scan64);
  unsigned* misc = reinterpret_cast<unsigned*>(scan64 + 64);  // [0] LSD fallback, [1] large bins
  unsigned short* large = reinterpret_cast<unsigned short*>(misc + 4);
  uint64_t* bar = reinterpret_cast<uint64_t*>(sm + L::total - 16);

  const TileDesc td = tiles[tid];
  const unsigned n = td.len;
  if (n > (unsigned)L::CAP) return;  // oversized tiles take a larger path
  if (n == 0) {
    if (threadIdx.x == 0) {
      TileOut<T> o;
      o.first_key = o.last_key = T(0);
      o.rows = 0;
      o.first_count = 0;
      o.rest_bytes = 0;
      tout[tid] = o;
    }
    return;
  }
  T* g = keys + td.start;
  uint32_t* gc = counts + td.start;
  // the tile's key range from its splitters
  const uint32_t tl = rg.S > 1 ? (rg.tile0 + tid) % rg.S : 0u;
  const T mn = tl > 0 ? rg.spl[tl - 1] : T(0);
  T mx = rg.kmax;
  if (tl + 1 < rg.S) {
    const T e = rg.spl[tl];
    mx = e > mn ? T(e - T(1)) : mn;
  }
  const int rb = mx == mn ? 0 : KeyTraits<T>::kBits - clz_key(T(mx - mn));
  const int s = rb > kBinBits ? rb - kBinBits : 0;
  auto bin_at = [&](T key) -> unsigned {  // clamped: a key outside the range cannot leave the table
    const unsigned b = key < mn ? 0u : bin_of(key, mn, s);
    return b < (unsigned)kBins ? b : (unsigned)kBins - 1u;
  };

  // ---- 1. bulk load with the bin histogram; 2. scan, key scatter into bin order ----
  // The tile's keys arrive by one bulk copy of the 16-byte aligned span that
  // holds them (key buffers are allocated with slack past their end), while
  // the threads clear the bins.
  const uintptr_t ga = reinterpret_cast<uintptr_t>(g);
  const uintptr_t s0 = ga & ~(uintptr_t)15, s1 = (ga + (uintptr_t)n * sizeof(T) + 15) & ~(uintptr_t)15;
  const T* tk = reinterpret_cast<const T*>(sm + (ga - s0));  // the tile's keys in shared memory
  if (threadIdx.x == 0) mbar_init(bar);
  for (int b = threadIdx.x; b < kBins / 2; b += NT) bins[b] = 0;
  for (int b = threadIdx.x; b < kBins / 32; b += NT) fbits[b] = 0;
  if (threadIdx.x < 4) misc[threadIdx.x] = 0;
  __syncthreads();
  if (threadIdx.x == 0) bulk_load(sm, reinterpret_cast<const void*>(s0), (uint32_t)(s1 - s0), bar);
  const bool arrived = mbar_wait(bar, 0, rg.wait_polls ? rg.wait_polls : kBulkWaitPolls);
  if (__syncthreads_or(!arrived)) {
    // the wait gave up: report, wait (with a far larger bound) until the copy
    // has landed so that no write to this CTA's shared memory is still in
    // flight when it moves on, and leave the tile empty (the count fails)
    if (threadIdx.x == 0) {
      mbar_wait(bar, 0, kBulkDrainPolls);
      if (fallbacks) atomicAdd(fallbacks, kBulkTimeoutFlag);
      TileOut<T> o;  // an empty tile for the link and encode kernels that follow
      o.first_key = o.last_key = T(0);
      o.rows = 0;
      o.first_count = 0;
      o.rest_bytes = 0;
      tout[tid] = o;
    }
    __syncthreads();
    return;
  }
  for (unsigned i = threadIdx.x; i < n; i += NT) bin_add(bins, bin_at(tk[i]));
  __syncthreads();
  {
    constexpr int G = kBins / 2 / (4 * NT);  // uint4 groups (8 bins each) per thread
    uint4* b4 = reinterpret_cast<uint4*>(bins) + threadIdx.x * G;
    uint4 x[G];
    unsigned sum = 0;
#pragma unroll
    for (int j = 0; j < G; ++j) {
      x[j] = b4[j];
      const unsigned w2 = x[j].x + x[j].y + x[j].z + x[j].w;  // both halves, no carry across
      sum += (w2 & 0xffffu) + (w2 >> 16);
    }
    unsigned tot;
    unsigned pre = block_exclusive_scan<NT, unsigned>(sum, scan_sm, &tot);
    // each word becomes (start of its even bin) | (start of its odd bin) << 16
    auto put = [&](unsigned w) {
      const unsigned r = pre | ((pre + (w & 0xffffu)) << 16);
      pre += (w & 0xffffu) + (w >> 16);
      return r;
    };
#pragma unroll
    for (int j = 0; j < G; ++j) {
      uint4 y;
      y.x = put(x[j].x);
      y.y = put(x[j].y);
      y.z = put(x[j].z);
      y.w = put(x[j].w);
      b4[j] = y;
    }
  }
  __syncthreads();
  {
    // every thread takes its keys from the staged tile before any is
    // overwritten, then scatters them into bin order
    T v[ITEMS];
#pragma unroll
    for (int u = 0; u < ITEMS; ++u) {
      const unsigned i = threadIdx.x + u * NT;
      v[u] = i < n ? tk[i] : T(0);
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < ITEMS; ++u)
      if (threadIdx.x + u * NT < n) buf[bin_add(bins, bin_at(v[u]))] = v[u];
  }
  __syncthreads();
  // bin_get(b) is now the end of bin b; its start is the end of bin b - 1 (0 for b = 0)

  // ---- 3. mark the bins holding more than one distinct key ----
  for (unsigned p = threadIdx.x + 1; p < n; p += NT) {
    const T a = buf[p], b = buf[p - 1];
    if (a != b) {
      const unsigned ba = bin_at(a);
      if (bin_at(b) == ba) {
        const unsigned bit = 1u << (ba & 31);
        if (!(atomicOr(&fbits[ba >> 5], bit) & bit)) {
          const unsigned m = bin_get(bins, ba) - (ba ? bin_get(bins, ba - 1) : 0u);
          if (m > kSmallBin) large[atomicAdd(&misc[1], 1u)] = (unsigned short)ba;
        }
      }
    }
  }
  __syncthreads();

  // ---- 4. order the marked bins: small ones by the thread owning their
  // bits, the listed larger ones by the warps in turn ----
  {
    constexpr int BPT = kBins / NT;
    const unsigned lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const unsigned b0 = threadIdx.x * BPT;
    for (unsigned bits = (fbits[b0 >> 5] >> (b0 & 31)) & (BPT == 32 ? 0xffffffffu : ((1u << BPT) - 1u)); bits;
         bits &= bits - 1) {
      const unsigned bb = b0 + (__ffs(bits) - 1);
      const unsigned a = bb ? bin_get(bins, bb - 1) : 0u, e = bin_get(bins, bb);
      if (e - a > kSmallBin) continue;
      for (unsigned j = a + 1; j < e; ++j) {
        const T v = buf[j];
        unsigned q = j;
        while (q > a) {
          const T w = buf[q - 1];
          if (!(v < w)) break;
          buf[q] = w;
          --q;
        }
        buf[q] = v;
      }
    }
    const unsigned nlarge = misc[1];
    for (unsigned li = wid; li < nlarge; li += NW) {
      const unsigned bb = large[li];
      const unsigned a = bb ? bin_get(bins, bb - 1) : 0u, m = bin_get(bins, bb) - a;
      if (m <= 32) warp_match_sort(buf, a, m, lane);
      else if (!warp_distinct_sort(buf, a, m, lane)) {
        if (m <= kMaxMixed) warp_count_sort(buf, a, m, lane);
        else if (lane == 0) misc[0] = 1;
      }
    }
  }
  __syncthreads();
  if (misc[0]) {
    // a large bin of many distinct keys: full LSD over the varying bits, in place
    if (threadIdx.x == 0 && fallbacks) atomicAdd(fallbacks, 1ull);
    smem_radix_sort<T, NT, ITEMS>(buf, n, varying_bits(mn, mx), bins, scan_sm, 0);
  }

  // ---- 5. run-length reduction over the sorted keys ----
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const unsigned rounds = (n + NT - 1) / NT;
  const unsigned w0 = (unsigned)wid * 32u * rounds;
  unsigned hmask = 0, cnt = 0;
  for (unsigned r = 0; r < rounds; ++r) {
    const unsigned p = w0 + r * 32u + lane;
    bool h = false;
    if (p < n) h = p == 0 || buf[p] != buf[p - 1];
    hmask |= (unsigned)h << r;
    cnt += __popc(__ballot_sync(0xffffffffu, h));
  }
  unsigned U;
  unsigned u = block_exclusive_scan<NT, unsigned>(lane == 0 ? cnt : 0u, scan_sm, &U);
  u = __shfl_sync(0xffffffffu, u, 0);
  unsigned short* head = reinterpret_cast<unsigned short*>(bins);
  const unsigned lt = (1u << lane) - 1u;
  for (unsigned r = 0; r < rounds; ++r) {
    const bool h = (hmask >> r) & 1u;
    const unsigned bal = __ballot_sync(0xffffffffu, h);
    if (h) head[u + __popc(bal & lt)] = (unsigned short)(w0 + r * 32u + lane);
    u += __popc(bal);
  }
  if (threadIdx.x == 0) head[U] = (unsigned short)n;
  __syncthreads();
  unsigned long long rest = 0;
  // a warp takes 32 consecutive rows: the next row's start and the previous
  // row's key come from the neighbouring lanes (the warp's ends read them)
  for (unsigned v0 = threadIdx.x - (unsigned)lane; v0 < U; v0 += NT) {
    const unsigned v = v0 + (unsigned)lane;
    const bool act = v < U;
    const unsigned i = act ? (unsigned)head[v] : 0u;
    const T key = act ? buf[i] : T(0);
    unsigned nxt = __shfl_down_sync(0xffffffffu, i, 1);
    if (lane == 31 || v + 1 >= U) nxt = act ? (unsigned)head[v + 1] : 0u;
    T prev = shfl_up_key(key, 1);
    if (lane == 0 && act && v > 0) prev = buf[head[v - 1]];
    if (act) {
      const unsigned c = nxt - i;
      g[v] = key;
      gc[v] = c;
      if (v > 0) rest += (unsigned long long)(varint_len(T(key - prev)) + varint_len((uint64_t)c));
    }
  }
  unsigned long long rest_total;
  block_exclusive_scan<NT, unsigned long long>(rest, scan64, &rest_total);
  if (threadIdx.x == 0) {
    if (MULT > 1 && fallbacks) atomicAdd(&fallbacks[1], (unsigned long long)U);  // rows of tiles above capacity
    TileOut<T> o;
    o.first_key = buf[head[0]];
    o.first_count = (unsigned)head[1] - head[0];
    o.last_key = buf[head[U - 1]];
    o.rows = U;
    o.rest_bytes = rest_total;
    tout[tid] = o;
  }
}

// One CTA per tile: tile blockIdx.x (+ the launch's first) or ids[blockIdx.x];
// with a device count, CTAs walk ids[0 .. *nids) in turn.
template <class T, int MULT>
__global__ void __launch_bounds__(kTileThreads * MULT, MULT == 1 ? 2 : 1)
    k_tile_sort(T* __restrict__ keys, uint32_t* __restrict__ counts, const TileDesc* __restrict__ tiles,
                const uint32_t* __restrict__ ids, const unsigned* __restrict__ nids, TileOut<T>* __restrict__ tout,
                unsigned long long* fallbacks, TileRanges<T> rg) {
  if (nids) {
    const unsigned cnt = *nids;
    for (unsigned i = blockIdx.x; i < cnt; i += gridDim.x) {
      sort_tile<T, MULT>(ids[i], keys, counts, tiles, tout, fallbacks, rg);
      __syncthreads();  // shared memory is reused by the next tile
    }
  } else {
    sort_tile<T, MULT>(ids ? ids[blockIdx.x] : blockIdx.x, keys, counts, tiles, tout, fallbacks, rg);
  }
}

template <class T, int MULT>
static void tile_sort_with(T* keys, uint32_t* counts, const TileDesc* tiles, const uint32_t* ids,
                           const unsigned* nids, uint32_t n, TileOut<T>* out, unsigned long long* fallbacks,
                           TileRanges<T> rg, cudaStream_t s) {
  const size_t smem = BinSmem<T, MULT>::total;
  cudaFuncSetAttribute(k_tile_sort<T, MULT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaFuncSetAttribute(k_tile_sort<T, MULT>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  if (n) k_tile_sort<T, MULT><<<n, BinSmem<T, MULT>::NT, smem, s>>>(keys, counts, tiles, ids, nids, out, fallbacks, rg);
}

template <class T>
void launch_tile_sort(T* keys, uint32_t* counts, const TileDesc* tiles, uint32_t ntiles, TileOut<T>* out,
                      unsigned long long* fallbacks, TileRanges<T> rg, cudaStream_t s) {
  tile_sort_with<T, 1>(keys, counts, tiles, nullptr, nullptr, ntiles, out, fallbacks, rg, s);
}
template <class T>
void launch_tile_sort_large(T* keys, uint32_t* counts, const TileDesc* tiles, const uint32_t* ids, uint32_t nids,
                            const unsigned* nids_dev, TileOut<T>* out, unsigned long long* fallbacks,
                            TileRanges<T> rg, cudaStream_t s) {
  tile_sort_with<T, 2>(keys, counts, tiles, ids, nids_dev, nids, out, fallbacks, rg, s);
}
template void launch_tile_sort<uint64_t>(uint64_t*, uint32_t*, const TileDesc*, uint32_t, TileOut<uint64_t>*,
                                         unsigned long long*, TileRanges<uint64_t>, cudaStream_t);
template void launch_tile_sort<u128>(u128*, uint32_t*, const TileDesc*, uint32_t, TileOut<u128>*, unsigned long long*,
                                     TileRanges<u128>, cudaStream_t);
template void launch_tile_sort_large<uint64_t>(uint64_t*, uint32_t*, const TileDesc*, const uint32_t*, uint32_t,
                                               const unsigned*, TileOut<uint64_t>*, unsigned long long*,
                                               TileRanges<uint64_t>, cudaStream_t);
template void launch_tile_sort_large<u128>(u128*, uint32_t*, const TileDesc*, const uint32_t*, uint32_t,
                                           const unsigned*, TileOut<u128>*, unsigned long long*, TileRanges<u128>,
                                           cudaStream_t);

// ---------------------------------------------------------------------------
// Oversized tiles: one CTA, LSD passes through global memory.  Each pass
// histograms the digit, then walks the tile in CAP-key chunks, ranks each
// chunk stably on chip and appends every digit group at its running offset.
// Then a chunked run-length reduction with carries between chunks.
// ---------------------------------------------------------------------------
template <class T>
__device__ __forceinline__ void big_sort_tile(uint32_t tid, T* __restrict__ keys, uint32_t* __restrict__ counts,
                                              T* __restrict__ scratch, const TileDesc* __restrict__ tiles,
                                              TileOut<T>* __restrict__ tout, DevStatus* st,
                                              unsigned long long* sstats) {
  using L = TileSmem<T>;
  constexpr int NT = L::NT, ITEMS = L::ITEMS, CAP = L::CAP;
  extern __shared__ __align__(16) uint8_t sm[];
  unsigned* warp_hist = reinterpret_cast<unsigned*>(sm + L::buf_bytes);
  unsigned long long* scan64 = reinterpret_cast<unsigned long long*>(sm + L::buf_bytes + L::hist_bytes + L::head_bytes);
  unsigned* scan_sm = reinterpret_cast<unsigned*>(scan64);
  T* red = reinterpret_cast<T*>(scan64 + 64);
  unsigned long long* run_off = reinterpret_cast<unsigned long long*>(red + 2 * L::NW);  // 256
  unsigned* dtot = reinterpret_cast<unsigned*>(sm + L::buf_bytes + L::hist_bytes);        // 256 (head area)
  unsigned* dstart = dtot + 256;                                                          // 256

  const TileDesc td = tiles[tid];
  const unsigned long long n = td.len;
  T* src = keys + td.start;
  T* dst = scratch + td.start;

  T mn = ~T(0), mx = T(0);
  for (unsigned long long i = threadIdx.x; i < n; i += NT) {
    const T v = src[i];
    mn = v < mn ? v : mn;
    mx = v > mx ? v : mx;
  }
  block_minmax<NT>(mn, mx, red);
  if (mn == mx) {  // one key fills the tile: a single row
    if (threadIdx.x == 0) {
      if (sstats) atomicAdd(&sstats[1], 1ull);
      keys[td.start] = mn;
      counts[td.start] = n > 0xffffffffull ? 0xffffffffu : (uint32_t)n;
      TileOut<T> o;
      o.first_key = o.last_key = mn;
      o.rows = 1;
      o.first_count = counts[td.start];
      o.rest_bytes = 0;
      tout[tid] = o;
    }
    return;
  }
  const int nbits = varying_bits(mn, mx);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const unsigned pos0 = (unsigned)wid * 32u * ITEMS + lane;
  for (int shift = 0; shift < nbits; shift += 8) {
    // digit histogram
    for (int d = threadIdx.x; d < 256; d += NT) warp_hist[d] = 0;
    __syncthreads();
    for (unsigned long long i = threadIdx.x; i < n; i += NT) atomicAdd(&warp_hist[digit_of(src[i], shift)], 1u);
    __syncthreads();
    if (threadIdx.x == 0) {
      unsigned long long acc = 0;
      for (int d = 0; d < 256; ++d) {
        run_off[d] = acc;
        acc += warp_hist[d];
      }
    }
    __syncthreads();
    for (unsigned long long c0 = 0; c0 < n; c0 += CAP) {
      const unsigned cn = (unsigned)((n - c0) < (unsigned long long)CAP ? (n - c0) : CAP);
      T key[ITEMS];
      unsigned dig[ITEMS], dest[ITEMS];
      bool valid[ITEMS];
#pragma unroll
      for (int r = 0; r < ITEMS; ++r) {
        const unsigned pos = pos0 + r * 32u;
        valid[r] = pos < cn;
        key[r] = valid[r] ? src[c0 + pos] : T(0);
        dig[r] = digit_of(key[r], shift);
      }
      block_rank<NT, ITEMS, 256>(dig, valid, dest, warp_hist, scan_sm, dtot, dstart);
#pragma unroll
      for (int r = 0; r < ITEMS; ++r)
        if (valid[r]) dst[run_off[dig[r]] + (dest[r] - dstart[dig[r]])] = key[r];
      __syncthreads();
      for (int d = threadIdx.x; d < 256; d += NT) run_off[d] += dtot[d];
      __syncthreads();
    }
    T* t = src;
    src = dst;
    dst = t;
  }
  // Run-length reduction of the sorted keys in src (keys or scratch).
  // Pass A: unique keys to keys[start+u], head positions to counts[start+u].
  T* ok = keys + td.start;
  uint32_t* oc = counts + td.start;
  unsigned long long U = 0;
  for (unsigned long long c0 = 0; c0 < n; c0 += CAP) {
    const unsigned cn = (unsigned)((n - c0) < (unsigned long long)CAP ? (n - c0) : CAP);
    const unsigned b0 = threadIdx.x * ITEMS;
    T kv[ITEMS];
    bool hd[ITEMS];
    unsigned nh = 0;
#pragma unroll
    for (int r = 0; r < ITEMS; ++r) {
      const unsigned i = b0 + r;
      hd[r] = false;
      if (i < cn) {
        const unsigned long long gi = c0 + i;
        kv[r] = src[gi];
        hd[r] = gi == 0 || kv[r] != src[gi - 1];
        nh += hd[r];
      }
    }
    unsigned tot;
    unsigned long long u = U + block_exclusive_scan<NT, unsigned>(nh, scan_sm, &tot);
    __syncthreads();
#pragma unroll
    for (int r = 0; r < ITEMS; ++r)
      if (hd[r]) {
        ok[u] = kv[r];
        oc[u] = (uint32_t)(c0 + b0 + r);
        u++;
      }
    U += tot;
    __syncthreads();
  }
  // Pass B: head positions -> counts (saturating u32), DVLE rest bytes.
  unsigned long long rest = 0;
  for (unsigned long long c0 = 0; c0 < U; c0 += CAP) {
    const unsigned cn = (unsigned)((U - c0) < (unsigned long long)CAP ? (U - c0) : CAP);
    unsigned long long cnt[ITEMS];
    T kv[ITEMS], kp[ITEMS];
#pragma unroll
    for (int r = 0; r < ITEMS; ++r) {
      const unsigned i = threadIdx.x + r * NT;
      cnt[r] = 0;
      if (i < cn) {
        const unsigned long long v = c0 + i;
        const unsigned long long h0 = oc[v];
        const unsigned long long h1 = (v + 1 < U) ? (unsigned long long)oc[v + 1] : n;
        cnt[r] = h1 - h0;
        kv[r] = ok[v];
        kp[r] = v > 0 ? ok[v - 1] : T(0);
      }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < ITEMS; ++r) {
      const unsigned i = threadIdx.x + r * NT;
      if (i < cn) {
        const unsigned long long v = c0 + i;
        const uint32_t c = cnt[r] > 0xffffffffull ? 0xffffffffu : (uint32_t)cnt[r];
        oc[v] = c;
        if (v > 0) rest += (unsigned long long)(varint_len(kv[r] - kp[r]) + varint_len((uint64_t)c));
      }
    }
    __syncthreads();
  }
  unsigned long long rest_total;
  block_exclusive_scan<NT, unsigned long long>(rest, scan64, &rest_total);
  if (threadIdx.x == 0) {
    if (sstats) atomicAdd(&sstats[1], U);
    TileOut<T> o;
    o.first_key = ok[0];
    o.first_count = oc[0];
    o.last_key = ok[U - 1];
    o.rows = (uint32_t)U;
    o.rest_bytes = rest_total;
    tout[tid] = o;
  }
  (void)st;
}

// One CTA per listed tile, or (device count) CTAs walking the list in turn.
template <class T>
__global__ void __launch_bounds__(kTileThreads, 1)
    k_big_tile_sort(T* __restrict__ keys, uint32_t* __restrict__ counts, T* __restrict__ scratch,
                    const TileDesc* __restrict__ tiles, const uint32_t* __restrict__ big_ids,
                    const unsigned* __restrict__ nids, TileOut<T>* __restrict__ tout, DevStatus* st,
                    unsigned long long* sstats) {
  if (nids) {
    const unsigned cnt = *nids;
    for (unsigned i = blockIdx.x; i < cnt; i += gridDim.x) {
      big_sort_tile<T>(big_ids[i], keys, counts, scratch, tiles, tout, st, sstats);
      __syncthreads();  // shared memory is reused by the next tile
    }
  } else {
    big_sort_tile<T>(big_ids[blockIdx.x], keys, counts, scratch, tiles, tout, st, sstats);
  }
}

template <class T>
void launch_big_tile_sort(T* keys, uint32_t* counts, T* scratch, const TileDesc* tiles, const uint32_t* big_ids,
                          uint32_t nbig, const unsigned* nbig_dev, TileOut<T>* out, DevStatus* st,
                          unsigned long long* sort_stats, cudaStream_t s) {
  const size_t smem = TileSmem<T>::total;
  cudaFuncSetAttribute(k_big_tile_sort<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (nbig)
    k_big_tile_sort<T><<<nbig, kTileThreads, smem, s>>>(keys, counts, scratch, tiles, big_ids, nbig_dev, out, st,
                                                         sort_stats);
}
template void launch_big_tile_sort<uint64_t>(uint64_t*, uint32_t*, uint64_t*, const TileDesc*, const uint32_t*,
                                             uint32_t, const unsigned*, TileOut<uint64_t>*, DevStatus*,
                                             unsigned long long*, cudaStream_t);
template void launch_big_tile_sort<u128>(u128*, uint32_t*, u128*, const TileDesc*, const uint32_t*, uint32_t,
                                         const unsigned*, TileOut<u128>*, DevStatus*, unsigned long long*,
                                         cudaStream_t);

// Oversized tiles listed on the device, per bucket group: group g (buckets
// gb[g] .. gb[g+1]) lists its tiles above the on-chip capacity (up to twice
// it) from ids[gb[g] * S] on and those above twice it from ids2[gb[g] * S] on,
// with the counts in cnt[2g] and cnt[2g + 1].  Also the tile statistics:
// stats[0] largest tile, [1] keys, [2] non-empty tiles, [3] keys in the tiles
// above capacity, range[t] keys in tile index t of every bucket.
__global__ void k_tile_lists(const uint32_t* __restrict__ lens, uint32_t ntiles, uint32_t S,
                             const uint32_t* __restrict__ gb, uint32_t NG, uint32_t cap, uint32_t* __restrict__ ids,
                             uint32_t* __restrict__ ids2, unsigned* __restrict__ cnt,
                             unsigned long long* __restrict__ stats, unsigned long long* __restrict__ range) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntiles) return;
  const uint32_t len = lens[t];
  if (len == 0) return;
  const uint32_t b = t / S;
  uint32_t g = 0;
  while (g + 1 < NG && gb[g + 1] <= b) ++g;
  if (len > 2 * cap) ids2[(size_t)gb[g] * S + atomicAdd(&cnt[2 * g + 1], 1u)] = t;
  else if (len > cap) ids[(size_t)gb[g] * S + atomicAdd(&cnt[2 * g], 1u)] = t;
  if (len > cap) atomicAdd(&stats[3], (unsigned long long)len);
  atomicMax(&stats[0], (unsigned long long)len);
  atomicAdd(&stats[1], (unsigned long long)len);
  atomicAdd(&stats[2], 1ull);
  atomicAdd(&range[t % S], (unsigned long long)len);
}

void launch_tile_lists(const uint32_t* lens, uint32_t ntiles, uint32_t S, const uint32_t* gb, uint32_t NG,
                       uint32_t cap, uint32_t* ids, uint32_t* ids2, unsigned* cnt, unsigned long long* stats,
                       unsigned long long* range, cudaStream_t s) {
  if (ntiles)
    k_tile_lists<<<(ntiles + 255) / 256, 256, 0, s>>>(lens, ntiles, S, gb, NG, cap, ids, ids2, cnt, stats, range);
}

}  // namespace kite
