// Shared device helpers for the GB300 k-mer counting kernels.
//
// Keys are the reference's k-mer words: u64 for k <= 31 and u128 for
// 32 <= k <= 64 (run_count dispatch, src/count/mod.rs:232-238).  Everything
// here is integer work; nothing uses tensor cores.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

typedef unsigned __int128 u128;

namespace kite {

// Device status word: kernels record the first failure here instead of
// trapping (host reads it after each stage).
struct DevStatus {
  unsigned int code;    // 0 = ok, else KITE_DEV_* below
  unsigned int a, b, c; // detail words
};
enum : unsigned int {
  KITE_DEV_OK = 0,
  KITE_DEV_STAGE_OVERFLOW = 1,  // a CTA staging buffer would overflow
  KITE_DEV_REGION_OVERFLOW = 2, // a bucket/tile region reservation overran
  KITE_DEV_TILE_OVERFLOW = 3,   // a tile larger than the on-chip capacity reached the tile sort
  KITE_DEV_BAD_INPUT = 4,
  KITE_DEV_ENCODE_OVERFLOW = 5,
  KITE_DEV_COUNT_OVERFLOW = 6,  // merged count exceeds u32 (merge path)
  KITE_DEV_SHORT_VARINTS = 7,   // a DVLE chunk holds fewer varints than its rows need (merge path)
};

__device__ __forceinline__ void dev_fail(DevStatus* st, unsigned code, unsigned a = 0, unsigned b = 0,
                                         unsigned c = 0) {
  if (atomicCAS(&st->code, 0u, code) == 0u) {
    st->a = a;
    st->b = b;
    st->c = c;
  }
}

// ---------------------------------------------------------------------------
// Key traits
// ---------------------------------------------------------------------------
template <class T> struct KeyTraits;
template <> struct KeyTraits<uint64_t> {
  static constexpr int kBytes = 8;
  static constexpr int kBits = 64;
  static constexpr int kEntry = 12;  // on-disk (key, count) entry size
};
template <> struct KeyTraits<u128> {
  static constexpr int kBytes = 16;
  static constexpr int kBits = 128;
  static constexpr int kEntry = 20;
};

// Fibonacci hash partition (src/count/kmer.rs:67-71, :111-116).
// `shift` = 64 - log2(partitions), always < 64 because partitions >= 2.
__device__ __forceinline__ uint32_t bucket_of(uint64_t key, uint32_t shift) {
  return (uint32_t)((key * 0x9E3779B97F4A7C15ull) >> shift);
}
__device__ __forceinline__ uint32_t bucket_of(u128 key, uint32_t shift) {
  return bucket_of((uint64_t)key ^ (uint64_t)(key >> 64), shift);
}

__device__ __forceinline__ int clz_key(uint64_t v) { return __clzll((long long)v); }
__device__ __forceinline__ int clz_key(u128 v) {
  uint64_t hi = (uint64_t)(v >> 64);
  return hi ? __clzll((long long)hi) : 64 + __clzll((long long)(uint64_t)v);
}

// LEB128 length of an unsigned value (write_varint_u64/u128,
// src/format/run_block.rs:9-35): max(1, ceil(bits/7)).
__device__ __forceinline__ int varint_len(uint64_t v) {
  int bits = 64 - __clzll((long long)v);
  return bits == 0 ? 1 : (bits + 6) / 7;
}
__device__ __forceinline__ int varint_len(u128 v) {
  int bits = 128 - clz_key(v);
  return bits == 0 ? 1 : (bits + 6) / 7;
}

__host__ __device__ __forceinline__ uint64_t hi64(uint64_t) { return 0; }
__host__ __device__ __forceinline__ uint64_t hi64(u128 v) { return (uint64_t)(v >> 64); }

template <class T>
__device__ __forceinline__ T make_key(uint64_t lo, uint64_t hi);
template <>
__device__ __forceinline__ uint64_t make_key<uint64_t>(uint64_t lo, uint64_t) { return lo; }
template <>
__device__ __forceinline__ u128 make_key<u128>(uint64_t lo, uint64_t hi) { return ((u128)hi << 64) | (u128)lo; }

// Warp shuffles of a key (one or two 64-bit moves).
template <class T>
__device__ __forceinline__ T shfl_key(T v, int src) {
  const uint64_t lo = __shfl_sync(0xffffffffu, (unsigned long long)(uint64_t)v, src);
  const uint64_t hi = sizeof(T) == 8 ? 0 : __shfl_sync(0xffffffffu, (unsigned long long)hi64(v), src);
  return make_key<T>(lo, hi);
}
template <class T>
__device__ __forceinline__ T shfl_up_key(T v, int d) {
  const uint64_t lo = __shfl_up_sync(0xffffffffu, (unsigned long long)(uint64_t)v, d);
  const uint64_t hi = sizeof(T) == 8 ? 0 : __shfl_up_sync(0xffffffffu, (unsigned long long)hi64(v), d);
  return make_key<T>(lo, hi);
}
template <class T>
__device__ __forceinline__ T shfl_xor_key(T v, int m) {
  const uint64_t lo = __shfl_xor_sync(0xffffffffu, (unsigned long long)(uint64_t)v, m);
  const uint64_t hi = sizeof(T) == 8 ? 0 : __shfl_xor_sync(0xffffffffu, (unsigned long long)hi64(v), m);
  return make_key<T>(lo, hi);
}

template <class T>
__device__ __forceinline__ unsigned digit_of(T key, int shift) {
  return (unsigned)(uint64_t)(key >> shift) & 0xffu;
}

// ---------------------------------------------------------------------------
// Block-wide exclusive scan of one unsigned value per thread.  `smem` holds at
// least 32 entries.  Returns the exclusive prefix; *total gets the block sum.
// ---------------------------------------------------------------------------
template <int NT, class V>
__device__ __forceinline__ V block_exclusive_scan(V x, V* smem, V* total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  V inc = x;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    V y = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += y;
  }
  if (lane == 31) smem[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    V w = lane < NT / 32 ? smem[lane] : V(0);
    V wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      V y = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += y;
    }
    if (lane < NT / 32) smem[lane] = wi - w;
    if (lane == NT / 32 - 1) smem[NT / 32] = wi;
  }
  __syncthreads();
  V res = smem[wid] + inc - x;
  *total = smem[NT / 32];
  __syncthreads();
  return res;
}

// ---------------------------------------------------------------------------
// Block-wide digit ranking by shared-memory atomics (not stable: order inside
// a digit is arbitrary).  `cnt` holds RADIX zeroed counters and is left
// zeroed; digit_total / digit_start get the batch's per-digit counts and
// exclusive starts; dest[r] = position of item r in digit-major order.  With
// RADIX > NT each thread scans RADIX / NT consecutive counters.
// ---------------------------------------------------------------------------
template <int NT, int ITEMS, int RADIX>
__device__ __forceinline__ void atomic_rank(const unsigned (&digit)[ITEMS], const bool (&valid)[ITEMS],
                                            unsigned (&dest)[ITEMS], unsigned* cnt, unsigned* scan_smem,
                                            unsigned* digit_total, unsigned* digit_start) {
  static_assert(RADIX <= NT || RADIX % NT == 0, "counters split evenly over the threads");
  constexpr int PER = RADIX > NT ? RADIX / NT : 1;
#pragma unroll
  for (int r = 0; r < ITEMS; ++r) dest[r] = valid[r] ? atomicAdd(&cnt[digit[r]], 1u) : 0u;
  __syncthreads();
  const int d0 = threadIdx.x * PER;
  unsigned v[PER], sum = 0;
#pragma unroll
  for (int j = 0; j < PER; ++j) {
    v[j] = d0 + j < RADIX ? cnt[d0 + j] : 0u;
    sum += v[j];
  }
  unsigned total;
  unsigned ex = block_exclusive_scan<NT, unsigned>(sum, scan_smem, &total);
#pragma unroll
  for (int j = 0; j < PER; ++j)
    if (d0 + j < RADIX) {
      digit_start[d0 + j] = ex;
      digit_total[d0 + j] = v[j];
      cnt[d0 + j] = 0;
      ex += v[j];
    }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < ITEMS; ++r)
    if (valid[r]) dest[r] += digit_start[digit[r]];
}

// ---------------------------------------------------------------------------
// Stable block-wide digit ranking (the LSD radix step used on chip).
//
// Items are owned in "warp-striped" order: warp w owns the contiguous
// position range [w*32*ITEMS, (w+1)*32*ITEMS), and in round r lane l holds
// position w*32*ITEMS + r*32 + l.  For each valid item the routine returns
// its destination index in the stable digit-sorted order.  warp_hist needs
// RADIX*NW unsigned ints of shared memory, scan_smem at least 33 entries.
// Digits of invalid items are ignored.  __match_any_sync groups lanes with
// equal digits; the group leader advances the warp's running digit count.
// ---------------------------------------------------------------------------
template <int NT, int ITEMS, int RADIX>
__device__ __forceinline__ void block_rank(const unsigned (&digit)[ITEMS], const bool (&valid)[ITEMS],
                                           unsigned (&dest)[ITEMS], unsigned* warp_hist, unsigned* scan_smem,
                                           unsigned* digit_total /* RADIX entries or nullptr */,
                                           unsigned* digit_start /* RADIX entries or nullptr */,
                                           int items = ITEMS /* rounds in use (block-uniform) */) {
  constexpr int NW = NT / 32;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const unsigned lt = (1u << lane) - 1u;
  unsigned* wh = warp_hist + wid * RADIX;
  for (int d = lane; d < RADIX; d += 32) wh[d] = 0;
  __syncwarp();
#pragma unroll
  for (int r = 0; r < ITEMS; ++r) {
    if (r >= items) break;
    const unsigned d = valid[r] ? digit[r] : (unsigned)RADIX;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const unsigned before = __popc(peers & lt);
    unsigned base = 0;
    if (d < (unsigned)RADIX) base = wh[d];
    __syncwarp();
    if (d < (unsigned)RADIX && before == 0) wh[d] = base + __popc(peers);
    __syncwarp();
    dest[r] = base + before;
  }
  __syncthreads();
  // Exclusive scan over (digit major, warp minor).  RADIX*NW entries, each
  // thread takes a contiguous run of E entries.
  constexpr int TOTAL = RADIX * NW;
  constexpr int E = (TOTAL + NT - 1) / NT;
  unsigned vals[E];
  unsigned run = 0;
#pragma unroll
  for (int i = 0; i < E; ++i) {
    const int e = threadIdx.x * E + i;
    unsigned v = 0;
    if (e < TOTAL) v = warp_hist[(e % NW) * RADIX + e / NW];
    vals[i] = v;
    run += v;
  }
  unsigned total;
  unsigned pre = block_exclusive_scan<NT, unsigned>(run, scan_smem, &total);
  // write back exclusive prefixes (safe: all reads above completed before the
  // scan's barriers)
#pragma unroll
  for (int i = 0; i < E; ++i) {
    const int e = threadIdx.x * E + i;
    if (e < TOTAL) {
      const int w = e % NW, d = e / NW;
      warp_hist[w * RADIX + d] = pre;
      if (w == 0 && digit_start) digit_start[d] = pre;
    }
    pre += vals[i];
  }
  __syncthreads();
  if (digit_total) {
    for (int d = threadIdx.x; d < RADIX; d += NT) {
      const unsigned next = (d + 1 < RADIX) ? warp_hist[d + 1] : total;  // warp 0 entry of next digit
      digit_total[d] = next - warp_hist[d];
    }
  }
#pragma unroll
  for (int r = 0; r < ITEMS; ++r)
    if (valid[r]) dest[r] += warp_hist[wid * RADIX + digit[r]];
  __syncthreads();
}

}  // namespace kite
