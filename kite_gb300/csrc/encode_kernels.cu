// DVLE encoding of every hash bucket's rows into one payload per partition
// (encode_dvle_u64 / encode_dvle_u128, src/format/run_block.rs:70-95:
// first key raw LE + count u32 LE, then LEB128(key delta) + LEB128(count)).
//
// Tiles of a bucket are in key order, so a bucket's payload is the
// concatenation of its tiles' encodings; only the first row of each tile needs
// the previous tile's last key.
#include "kite_internal.h"

namespace kite {

// One warp per bucket: walks the bucket's S tiles 32 at a time, links each
// non-empty tile to the last key of the previous non-empty tile, and computes
// tile byte offsets, row totals and the bucket's min/max key.
template <class T>
__global__ void k_tile_link(const TileOut<T>* __restrict__ tout, uint32_t P, uint32_t S,
                            const uint32_t* __restrict__ tile_first, unsigned long long* __restrict__ tile_boff,
                            T* __restrict__ tile_prev, BucketMeta* __restrict__ meta) {
  const int lane = threadIdx.x & 31;
  const uint32_t b = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (b >= P) return;
  // tiles of bucket b: [t0, t0 + S) (fixed S) or [tile_first[b], tile_first[b+1])
  const size_t t0 = tile_first ? tile_first[b] : (size_t)b * S;
  if (tile_first) S = tile_first[b + 1] - tile_first[b];
  bool have_prev = false;
  T prev = T(0), kmin = T(0);
  unsigned long long boff = 0, rows = 0;
  const unsigned lt = (1u << lane) - 1u;
  for (uint32_t j0 = 0; j0 < S; j0 += 32) {
    const uint32_t j = j0 + lane;
    TileOut<T> o;
    o.first_key = o.last_key = T(0);
    o.rows = 0;
    o.first_count = 0;
    o.rest_bytes = 0;
    if (j < S) o = tout[t0 + j];
    const bool ne = o.rows > 0;
    const unsigned ball = __ballot_sync(0xffffffffu, ne);
    // previous non-empty lane's last key
    const unsigned below = ball & lt;
    const int src_lane = below ? 31 - __clz(below) : 0;
    const T lk = o.last_key;
    const T from_lane = shfl_key(lk, src_lane);
    const bool has_p = below ? true : have_prev;
    const T p = below ? from_lane : prev;
    unsigned long long bytes = 0;
    if (ne) {
      const int first = has_p ? varint_len((T)(o.first_key - p)) + varint_len((uint64_t)o.first_count)
                              : KeyTraits<T>::kEntry;
      bytes = (unsigned long long)first + o.rest_bytes;
    }
    // warp inclusive scan of bytes and rows
    unsigned long long inc = bytes, rinc = ne ? o.rows : 0;
    for (int d = 1; d < 32; d <<= 1) {
      const unsigned long long y = __shfl_up_sync(0xffffffffu, inc, d);
      const unsigned long long ry = __shfl_up_sync(0xffffffffu, rinc, d);
      if (lane >= d) {
        inc += y;
        rinc += ry;
      }
    }
    if (j < S) {
      tile_boff[t0 + j] = boff + inc - bytes;
      tile_prev[t0 + j] = p;
    }
    // first non-empty tile overall gives kmin
    if (!have_prev && ball) {
      const int fl = __ffs(ball) - 1;
      kmin = shfl_key(o.first_key, fl);
    }
    if (ball) {
      const int ll = 31 - __clz(ball);
      prev = shfl_key(lk, ll);
      have_prev = true;
    }
    boff += __shfl_sync(0xffffffffu, inc, 31);
    rows += __shfl_sync(0xffffffffu, rinc, 31);
  }
  if (lane == 0) {
    BucketMeta m;
    m.rows = rows;
    m.bytes = boff;
    m.byte_off = 0;
    m.kmin_lo = (unsigned long long)kmin;
    m.kmin_hi = hi64(kmin);
    m.kmax_lo = (unsigned long long)prev;
    m.kmax_hi = hi64(prev);
    meta[b] = m;
  }
}

template <class T>
void launch_tile_link(const TileOut<T>* tout, uint32_t P, uint32_t S, unsigned long long* tile_boff, T* tile_prev,
                      BucketMeta* meta, cudaStream_t s) {
  const unsigned threads = 256;
  const unsigned blocks = (unsigned)(((size_t)P * 32 + threads - 1) / threads);
  k_tile_link<T><<<blocks, threads, 0, s>>>(tout, P, S, nullptr, tile_boff, tile_prev, meta);
}

template <class T>
void launch_tile_link_ranges(const TileOut<T>* tout, uint32_t P, const uint32_t* tile_first,
                             unsigned long long* tile_boff, T* tile_prev, BucketMeta* meta, cudaStream_t s) {
  const unsigned threads = 256;
  const unsigned blocks = (unsigned)(((size_t)P * 32 + threads - 1) / threads);
  k_tile_link<T><<<blocks, threads, 0, s>>>(tout, P, 0, tile_first, tile_boff, tile_prev, meta);
}
template void launch_tile_link_ranges<uint64_t>(const TileOut<uint64_t>*, uint32_t, const uint32_t*,
                                                unsigned long long*, uint64_t*, BucketMeta*, cudaStream_t);
template void launch_tile_link_ranges<u128>(const TileOut<u128>*, uint32_t, const uint32_t*, unsigned long long*,
                                            u128*, BucketMeta*, cudaStream_t);
template void launch_tile_link<uint64_t>(const TileOut<uint64_t>*, uint32_t, uint32_t, unsigned long long*,
                                         uint64_t*, BucketMeta*, cudaStream_t);
template void launch_tile_link<u128>(const TileOut<u128>*, uint32_t, uint32_t, unsigned long long*, u128*,
                                     BucketMeta*, cudaStream_t);

// Exclusive scan of bucket byte sizes into byte_off (single CTA; P <= 1<<16).
// With a mirror (pinned host memory mapped into the device's address space),
// the finished records are also written there, so the host reads them when
// the kernel has completed without a copy that would queue on a copy engine.
__global__ void __launch_bounds__(1024) k_bucket_offsets(BucketMeta* meta, uint32_t P, BucketMeta* mirror) {
  __shared__ unsigned long long sm[34];
  unsigned long long carry = 0;
  for (uint32_t b0 = 0; b0 < P; b0 += 1024) {
    const uint32_t b = b0 + threadIdx.x;
    const unsigned long long v = b < P ? meta[b].bytes : 0;
    unsigned long long tot;
    const unsigned long long ex = block_exclusive_scan<1024, unsigned long long>(v, sm, &tot);
    if (b < P) {
      meta[b].byte_off = carry + ex;
      if (mirror) mirror[b] = meta[b];
    }
    carry += tot;
  }
}

void launch_bucket_offsets(BucketMeta* meta, uint32_t P, BucketMeta* host_mirror, cudaStream_t s) {
  k_bucket_offsets<<<1, 1024, 0, s>>>(meta, P, host_mirror);
}

template <class T>
__device__ __forceinline__ int put_varint(uint8_t* o, T v) {
  int n = 0;
  for (;;) {
    const uint8_t b = (uint8_t)(v & T(0x7f));
    v >>= 7;
    if (v == T(0)) {
      o[n++] = b;
      return n;
    }
    o[n++] = b | 0x80;
  }
}

// One CTA per tile, 1024 rows at a time, each thread four consecutive rows
// (the previous row's key from the thread's own registers for all but its
// first): per-row sizes, one block scan per round, each thread's rows'
// bytes assembled in shared memory, then written out with consecutive
// threads on consecutive aligned 4-byte words (whole sectors, not one
// scattered byte store per row byte).
constexpr int kEncThreads = 256, kEncRows = 4, kEncRound = kEncThreads * kEncRows;
template <class T>
__global__ void __launch_bounds__(kEncThreads) k_encode(const T* __restrict__ keys, const uint32_t* __restrict__ counts,
                                                        const TileDesc* __restrict__ tiles,
                                                        const TileOut<T>* __restrict__ tout,
                                                        const unsigned long long* __restrict__ tile_boff,
                                                        const T* __restrict__ tile_prev,
                                                        const BucketMeta* __restrict__ meta, uint8_t* __restrict__ out,
                                                        unsigned long long out_cap, DevStatus* st) {
  // largest row: LEB128 of a key delta plus LEB128 of a u32 count, or the raw first row
  constexpr int kRowMax = (KeyTraits<T>::kBits + 6) / 7 + 5;
  __shared__ unsigned long long sm[34];
  __shared__ uint8_t chunk[kEncRound * kRowMax];
  const uint32_t t = blockIdx.x;
  const TileOut<T> o = tout[t];
  if (o.rows == 0) return;
  const TileDesc td = tiles[t];
  const unsigned long long base = meta[td.bucket].byte_off + tile_boff[t];
  const bool first_in_bucket = tile_boff[t] == 0;
  const T tprev = tile_prev[t];
  const T* k = keys + td.start;
  const uint32_t* c = counts + td.start;
  unsigned long long run = 0;
  unsigned* scan32 = reinterpret_cast<unsigned*>(sm);
  for (uint32_t r0 = 0; r0 < o.rows; r0 += kEncRound) {
    const uint32_t rb = r0 + threadIdx.x * kEncRows;  // the thread's first row
    T key[kEncRows];
    uint32_t cnt[kEncRows];
    int sz[kEncRows];
    unsigned mine = 0;
    T p = rb < o.rows ? (rb == 0 ? tprev : k[rb - 1]) : T(0);
#pragma unroll
    for (int i = 0; i < kEncRows; ++i) {
      const uint32_t r = rb + i;
      key[i] = T(0);
      cnt[i] = 0;
      sz[i] = 0;
      if (r < o.rows) {
        key[i] = k[r];
        cnt[i] = c[r];
        sz[i] = (r == 0 && first_in_bucket) ? KeyTraits<T>::kEntry
                                            : varint_len((T)(key[i] - p)) + varint_len((uint64_t)cnt[i]);
        p = key[i];
      }
      mine += (unsigned)sz[i];
    }
    unsigned tot;
    unsigned ex = block_exclusive_scan<kEncThreads, unsigned>(mine, scan32, &tot);
    {
      T q = rb < o.rows ? (rb == 0 ? tprev : k[rb - 1]) : T(0);
      uint8_t* w = chunk + ex;
#pragma unroll
      for (int i = 0; i < kEncRows; ++i) {
        const uint32_t r = rb + i;
        if (r >= o.rows) break;
        if (r == 0 && first_in_bucket) {
          for (int j = 0; j < (int)sizeof(T); ++j) w[j] = (uint8_t)(key[i] >> (8 * j));
          for (int j = 0; j < 4; ++j) w[sizeof(T) + j] = (uint8_t)(cnt[i] >> (8 * j));
        } else {
          const int n1 = put_varint<T>(w, (T)(key[i] - q));
          put_varint<uint64_t>(w + n1, (uint64_t)cnt[i]);
        }
        w += sz[i];
        q = key[i];
      }
    }
    __syncthreads();
    const unsigned long long at = base + run;
    if (at + tot > out_cap) {
      if (threadIdx.x == 0) dev_fail(st, KITE_DEV_ENCODE_OVERFLOW, t, r0, 0);
    } else {
      // 4-byte stores on 4-byte aligned addresses; the unaligned head and
      // tail bytes one by one
      uint8_t* dst = out + at;
      const unsigned head = (unsigned)((4u - ((uintptr_t)dst & 3u)) & 3u);
      if (tot < head + 8u) {
        for (unsigned i = threadIdx.x; i < tot; i += kEncThreads) dst[i] = chunk[i];
      } else {
        const unsigned body = (tot - head) & ~3u, tail = tot - head - body;
        if (threadIdx.x < head) dst[threadIdx.x] = chunk[threadIdx.x];
        if (threadIdx.x < tail) dst[head + body + threadIdx.x] = chunk[head + body + threadIdx.x];
        uint32_t* dw = reinterpret_cast<uint32_t*>(dst + head);
        for (unsigned i = threadIdx.x; i < body / 4; i += kEncThreads) {
          const uint8_t* bb = chunk + head + 4 * i;
          dw[i] = (uint32_t)bb[0] | ((uint32_t)bb[1] << 8) | ((uint32_t)bb[2] << 16) | ((uint32_t)bb[3] << 24);
        }
      }
    }
    __syncthreads();  // the chunk is refilled next round
    run += tot;
  }
}

template <class T>
void launch_encode(const T* keys, const uint32_t* counts, const TileDesc* tiles, const TileOut<T>* tout,
                   const unsigned long long* tile_boff, const T* tile_prev, const BucketMeta* meta, uint32_t ntiles,
                   uint8_t* out, unsigned long long out_cap, DevStatus* st, cudaStream_t s) {
  if (ntiles)
    k_encode<T><<<ntiles, kEncThreads, 0, s>>>(keys, counts, tiles, tout, tile_boff, tile_prev, meta, out, out_cap,
                                                st);
}
template void launch_encode<uint64_t>(const uint64_t*, const uint32_t*, const TileDesc*, const TileOut<uint64_t>*,
                                      const unsigned long long*, const uint64_t*, const BucketMeta*, uint32_t,
                                      uint8_t*, unsigned long long, DevStatus*, cudaStream_t);
template void launch_encode<u128>(const u128*, const uint32_t*, const TileDesc*, const TileOut<u128>*,
                                  const unsigned long long*, const u128*, const BucketMeta*, uint32_t, uint8_t*,
                                  unsigned long long, DevStatus*, cudaStream_t);

}  // namespace kite
