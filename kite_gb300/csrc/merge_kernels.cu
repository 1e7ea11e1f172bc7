// GPU `kite merge`: decode every input chunk, k-way merge per partition with
// exact count summation, DVLE re-encode.
//
// Reference semantics restated (src/merge/mod.rs:198-214 and
// src/kiteops/mod.rs:433-859):
//   load_partition_counts   every chunk of one input's partition decoded
//                           (DVLE or RAW), equal keys summed in u64 (saturating)
//   apply_reader_filter     that input's header min/max, on the per-input sum
//   merge_vectors_total     union over inputs, u64 saturating sums
//   serialize_partition_chunk  a total above u32::MAX is an error naming the key;
//                           otherwise one DVLE chunk per non-empty partition.
//
// GPU structure:
//   decode    payload bytes cut into 8 KiB segments, one warp each;
//             per-segment varint terminator counts and parity sums,
//             per-stream scans on the device, then a pass that writes
//             (key, u64 count) rows.  A
//             "stream" is one chunk.
//   tiles     key-range tiles per partition from global splitters, refined by
//             bisection until every tile fits on chip; each stream is
//             binary-searched for the tile edges.
//   merge     one CTA per tile: rows of all its streams into shared memory,
//             merged ranks by binary search (ties broken by stream order),
//             per-input sums, filter, cross-input sums, overflow check.
//   encode    the count path's DVLE link + encode kernels.
//
// The same decode / tile / merge stages serve `kite dump` (one input):
//   LoserTreeMerger src/dump/loser_tree.rs:141-175  the chunks of a partition
//                           merged by key, equal keys summed with saturating
//                           u32 adds (= the u64 sum clamped to u32::MAX)
//   stream_partition_slabs src/dump/merge.rs:282-428  header min/max applied
//                           to that summed count, then one TSV line per row
//   decode_kmer_any src/dump/decoder.rs:27-50  the key's 2-bit codes MSB
//                           first as ACGT, "<kmer>\t<count>\n"
// with a formatting pass in place of the DVLE encode.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "merge.h"
#include "kite_internal.h"
#include "splitters.h"

namespace kite {

namespace {

constexpr uint32_t kSeg = 8192;          // decode segment bytes (one warp each)
constexpr int kMergeThreads = 512;
constexpr uint32_t kMergeCap = 4096;      // rows per merge tile
constexpr uint32_t kMaxTileStreams = 256; // streams per tile (inputs x chunks)
constexpr int kTsvThreads = 256;          // rows per formatting round
constexpr uint32_t kHistBins = 1024;      // histo: counts below this binned on chip, larger ones listed

// What the merge kernel makes of each merged key group.
enum MergeMode : int {
  kModeMerge = 0,  // kite merge: per-input filter, u64 sums, u32 overflow recorded
  kModeDump = 1,   // kite dump: sum clamped to u32, then the header filter; TSV byte counts
  kModeHisto = 2,  // kite histo: per-input filter on the u64 sum, then count -> frequency
  kModeRows = 3,   // kite query: every key with its u64 sum, no filter
};

// Outputs of the histo and query modes.
struct MergeAux {
  unsigned long long* hist;      // kHistBins frequencies (histo)
  unsigned long long* spill;     // counts >= kHistBins, one entry per key (histo)
  unsigned long long* spill_n;   // entries written to spill
  unsigned long long spill_cap;
  unsigned long long* counts64;  // u64 sum of every output row (query)
  uint32_t line_k;               // k, for TSV line lengths (dump)
};

// Decimal digits of a count.
__host__ __device__ __forceinline__ unsigned dec_digits(uint32_t v) {
  unsigned d = 1;
  for (uint32_t p = 10; d < 10 && v >= p; p *= 10) ++d;
  return d;
}

struct StreamDesc {
  uint64_t byte_off;   // payload offset in the device byte buffer
  uint64_t byte_len;
  uint64_t row_off;    // first row in the decoded arrays
  uint64_t rows;
  uint32_t codec;
  uint32_t input;
  uint32_t partition;
  uint32_t head;       // raw head bytes (12 or 20) for DVLE, 0 for RAW
};

struct SegDesc {
  uint64_t start, end;  // byte range (device buffer offsets) inside the stream's varint area
  uint32_t stream;
  uint32_t first;       // 1 if first segment of the stream
};

struct InputFilter {
  uint32_t has_min, has_max, min_count, max_count;
};

// One entry of a tile's stream list.
struct TileStream {
  uint64_t lo, hi;      // row range [lo, hi) (absolute row indices)
  uint32_t input;
  uint32_t pad;
};

struct MergeTile {
  uint64_t out_off;     // output row base (reserved = rows in)
  uint32_t first_ts;    // index into TileStream list
  uint32_t nts;
  uint32_t rows_in;
  uint32_t partition;
};

__device__ __forceinline__ bool is_term(uint8_t b) { return (b & 0x80u) == 0; }

// Warp shuffle-up of a 64- or 128-bit value, a wrapping inclusive warp sum,
// and a broadcast from one lane.
template <class T>
__device__ __forceinline__ T shfl_up_t(T v, int d) {
  if constexpr (sizeof(T) == 8) {
    return (T)__shfl_up_sync(0xffffffffu, (unsigned long long)v, d);
  } else {
    const unsigned long long lo = __shfl_up_sync(0xffffffffu, (unsigned long long)v, d);
    const unsigned long long hi = __shfl_up_sync(0xffffffffu, (unsigned long long)(v >> 64), d);
    return ((T)hi << 64) | (T)lo;
  }
}
template <class T>
__device__ __forceinline__ T warp_incl_sum(T v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const T y = shfl_up_t(v, o);
    if (lane >= o) v += y;
  }
  return v;
}
template <class T>
__device__ __forceinline__ T warp_bcast_t(T v, int src) {
  if constexpr (sizeof(T) == 8) {
    return (T)__shfl_sync(0xffffffffu, (unsigned long long)v, src);
  } else {
    const unsigned long long lo = __shfl_sync(0xffffffffu, (unsigned long long)v, src);
    const unsigned long long hi = __shfl_sync(0xffffffffu, (unsigned long long)(v >> 64), src);
    return ((T)hi << 64) | (T)lo;
  }
}
template <class T>
__device__ __forceinline__ T warp_sum_t(T v) {
  return warp_bcast_t(warp_incl_sum(v), 31);
}

// ---- warp-cooperative DVLE decode ----------------------------------------------
// A segment (kSeg bytes of one stream's varint area) is decoded by one warp in
// rounds of 512 bytes: every lane loads 16 bytes (one coalesced 512-byte load
// per warp) into a per-warp shared-memory window that also holds the 32 bytes
// before the round, marks the terminator bytes (top bit clear) and decodes
// the varints whose terminator lies in its own 16 bytes, reading back to the
// previous terminator in the window (a varint is at most 19 bytes).  A varint
// belongs to the segment holding its terminator; the stream's bytes before
// its varint area (the raw head row) bound the first varint.  A final varint
// without a terminator at the stream's end belongs to the last segment.
constexpr int kDecWarps = 8;                    // warps per decode CTA
constexpr uint32_t kRound = 512;                // bytes per warp round
constexpr uint32_t kWinBytes = kRound + 32;     // window: 32 bytes before the round + the round

struct DecWindow {
  uint8_t b[kWinBytes];
};

// Terminator bits of 16 bytes (bit i: byte i has its top bit clear).
__device__ __forceinline__ uint32_t term_bits16(uint4 w) {
  auto m4 = [](uint32_t x) {
    const uint32_t t = ~x & 0x80808080u;
    return ((t >> 7) & 1u) | ((t >> 14) & 2u) | ((t >> 21) & 4u) | ((t >> 28) & 8u);
  };
  return m4(w.x) | (m4(w.y) << 4) | (m4(w.z) << 8) | (m4(w.w) << 12);
}

// Loads the round at `base` (16-byte aligned) into the window: bytes
// [base - 32, base + 512); blocks at or beyond lim_pad (the padded end of
// the byte buffer) and before byte 0 read as zero.
__device__ __forceinline__ void load_round(const uint8_t* __restrict__ bytes, uint64_t base, uint64_t lim_pad,
                                           DecWindow* win, uint32_t lane) {
  uint4* wv = reinterpret_cast<uint4*>(win->b);
  const uint64_t o = base + 16ull * lane;
  uint4 v = make_uint4(0, 0, 0, 0);
  if (o < lim_pad) v = *reinterpret_cast<const uint4*>(bytes + o);
  wv[2 + lane] = v;
  if (lane < 2) {
    uint4 p = make_uint4(0, 0, 0, 0);
    if (base >= 32) p = *reinterpret_cast<const uint4*>(bytes + base - 32 + 16 * lane);
    wv[lane] = p;
  }
  __syncwarp();
}

// The value of the varint ending at window byte t (32 <= t < 48) of the
// lane's 48-byte view: bytes from one past the previous boundary bit of
// `bound` below t up to t.
template <class T>
__device__ __forceinline__ T varint_at(const DecWindow* win, uint64_t bound, uint32_t lane_off, int t) {
  const uint64_t below = bound & ((1ull << t) - 1ull);
  const int start = below ? 64 - __clzll(below) : 0;
  T val = 0;
  unsigned sh = 0;
  for (int j = start; j <= t; ++j) {
    const uint8_t b = win->b[lane_off + j];
    if (sh < (unsigned)KeyTraits<T>::kBits) val |= (T)(b & 0x7f) << sh;
    sh += 7;
  }
  return val;
}

// Per lane and round: `bound` marks over the lane's 48-byte view (window
// bytes [16 lane, 16 lane + 48) = stream bytes base - 32 + 16 lane + i) the
// terminators and every byte before the varint area (so the first varint
// starts at the area); `own` marks the terminators of the lane's own 16 bytes
// (view bits 32..47) inside [seg_lo, seg_hi).
__device__ __forceinline__ void round_masks(const DecWindow* win, uint32_t lane, uint64_t base, uint64_t area,
                                            uint64_t seg_lo, uint64_t seg_hi, uint64_t& bound, uint32_t& own) {
  const uint4* wv = reinterpret_cast<const uint4*>(win->b);
  const uint64_t t0 = term_bits16(wv[lane]), t1 = term_bits16(wv[lane + 1]), t2 = term_bits16(wv[lane + 2]);
  bound = t0 | (t1 << 16) | (t2 << 32);
  const uint64_t ob = base + 16ull * lane;  // stream byte of view bit 32
  const int64_t nb = (int64_t)(32 + area) - (int64_t)ob;  // view bits below the varint area
  if (nb > 0) bound |= nb >= 48 ? 0xFFFFFFFFFFFFull : ((1ull << nb) - 1ull);
  const int64_t lo = (int64_t)seg_lo - (int64_t)ob, hi = (int64_t)seg_hi - (int64_t)ob;
  uint32_t keep = 0xFFFFu;
  if (lo > 0) keep &= lo >= 16 ? 0u : ~((1u << lo) - 1u);
  if (hi < 16) keep &= hi <= 0 ? 0u : ((1u << hi) - 1u);
  own = (uint32_t)t2 & keep;
}

// Pass A, one warp per segment: the varints the segment owns, and the
// wrapping sums of those at even / odd positions within the segment (which
// of the two are key deltas follows from the parity of the segment's first
// varint index, known after the per-stream scan).
template <class T>
__global__ void __launch_bounds__(32 * kDecWarps)
    k_seg_pass_a(const uint8_t* __restrict__ bytes, uint64_t lim_pad, const SegDesc* __restrict__ segs,
                 uint32_t nseg, const StreamDesc* __restrict__ streams, uint32_t* __restrict__ terms,
                 T* __restrict__ sum_even, T* __restrict__ sum_odd) {
  __shared__ __align__(16) DecWindow wins[kDecWarps];
  const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const uint32_t si = blockIdx.x * kDecWarps + wid;
  if (si >= nseg) return;
  DecWindow* win = &wins[wid];
  const SegDesc d = segs[si];
  const StreamDesc sd = streams[d.stream];
  const uint64_t area = sd.byte_off + sd.head, lim = sd.byte_off + sd.byte_len;
  uint32_t n = 0;  // varints owned so far (the same in every lane)
  T se = 0, so = 0;
  for (uint64_t base = d.start & ~15ull; base < d.end; base += kRound) {
    load_round(bytes, base, lim_pad, win, lane);
    uint64_t bound;
    uint32_t own;
    round_masks(win, lane, base, area, d.start, d.end, bound, own);
    const uint32_t c = __popc(own);
    uint32_t incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= (uint32_t)o) incl += y;
    }
    uint32_t idx = n + incl - c;
    for (uint32_t m = own; m; m &= m - 1, ++idx) {
      const T v = varint_at<T>(win, bound, 16 * lane, 32 + __ffs(m) - 1);
      if (idx & 1u) so += v;
      else se += v;
    }
    n += __shfl_sync(0xffffffffu, incl, 31);
    __syncwarp();
  }
  // a final varint without its terminator (the stream ends inside it)
  if (d.end == lim && lim > area && lane == 0 && !is_term(bytes[lim - 1])) {
    uint64_t p = lim;
    while (p > area && !is_term(bytes[p - 1])) --p;
    T val = 0;
    unsigned sh = 0;
    for (uint64_t q = p; q < lim; ++q) {
      if (sh < (unsigned)KeyTraits<T>::kBits) val |= (T)(bytes[q] & 0x7f) << sh;
      sh += 7;
    }
    if (n & 1u) so += val;
    else se += val;
    ++n;
  }
  n = __shfl_sync(0xffffffffu, n, 0);
  se = warp_sum_t(se);
  so = warp_sum_t(so);
  if (lane == 0) {
    terms[si] = n;
    sum_even[si] = se;
    sum_odd[si] = so;
  }
}

// Per stream of the list sids (one warp each): first varint index and start
// key of every segment [seg_first, seg_end) of the stream (exclusive scans of
// the terminator counts and of the delta sums), and the check that the stream
// holds the 2 * (rows - 1) varints its rows need.
template <class T>
__global__ void k_stream_seg_scan(const uint32_t* __restrict__ terms, const T* __restrict__ sum_even,
                                  const T* __restrict__ sum_odd, const uint32_t* __restrict__ seg_first,
                                  const uint32_t* __restrict__ seg_end, const StreamDesc* __restrict__ streams,
                                  const T* __restrict__ first_keys, const uint32_t* __restrict__ sids, uint32_t nsid,
                                  unsigned long long* __restrict__ vstart, T* __restrict__ kstart, DevStatus* st) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t w = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  if (w >= nsid) return;
  const uint32_t si = sids[w];
  const StreamDesc sd = streams[si];
  const uint32_t f = seg_first[si], e = seg_end[si];
  unsigned long long cv = 0;
  T ck = f < e ? first_keys[si] : T(0);
  for (uint32_t b = f; b < e; b += 32) {
    const uint32_t s = b + lane;
    const unsigned long long t = s < e ? terms[s] : 0ull;
    const unsigned long long ti = warp_incl_sum<unsigned long long>(t);
    const unsigned long long v = cv + ti - t;
    T dv = 0;
    if (s < e) dv = (v & 1ull) ? sum_odd[s] : sum_even[s];
    const T di = warp_incl_sum(dv);
    if (s < e) {
      vstart[s] = v;
      kstart[s] = ck + (di - dv);
    }
    cv += __shfl_sync(0xffffffffu, ti, 31);
    ck += warp_bcast_t(di, 31);
  }
  if (lane == 0 && sd.head && sd.rows && cv < 2 * (sd.rows - 1)) dev_fail(st, KITE_DEV_SHORT_VARINTS, si);
}

// Pass B, one warp per segment: (key, u64 count) rows of the varints the
// segment owns.  Varint index v (within the stream's varint area): even =
// key delta of row v/2+1, odd = count of row (v-1)/2+1.  Keys are the running
// wrapping sum of the deltas (as the reference's wrapping_add), from the
// segment's start key: each round a warp scan of the lanes' delta sums.
template <class T>
__global__ void __launch_bounds__(32 * kDecWarps)
    k_seg_rows(const uint8_t* __restrict__ bytes, uint64_t lim_pad, const SegDesc* __restrict__ segs,
               uint32_t nseg, const StreamDesc* __restrict__ streams, const unsigned long long* __restrict__ vstart,
               const T* __restrict__ kstart, T* __restrict__ keys, unsigned long long* __restrict__ counts) {
  __shared__ __align__(16) DecWindow wins[kDecWarps];
  const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const uint32_t si = blockIdx.x * kDecWarps + wid;
  if (si >= nseg) return;
  DecWindow* win = &wins[wid];
  const SegDesc d = segs[si];
  const StreamDesc sd = streams[d.stream];
  const uint64_t area = sd.byte_off + sd.head, lim = sd.byte_off + sd.byte_len;
  const unsigned long long nvar = sd.rows ? 2ull * (sd.rows - 1) : 0ull;
  unsigned long long v0 = vstart[si];  // stream varint index of the segment's next owned varint
  T key = kstart[si];                  // key before that varint
  for (uint64_t base = d.start & ~15ull; base < d.end; base += kRound) {
    load_round(bytes, base, lim_pad, win, lane);
    uint64_t bound;
    uint32_t own;
    round_masks(win, lane, base, area, d.start, d.end, bound, own);
    const uint32_t c = __popc(own);
    uint32_t incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= (uint32_t)o) incl += y;
    }
    const unsigned long long vl = v0 + incl - c;  // index of the lane's first owned varint
    // the lane's key deltas (kept: a lane owns at most 16 varints, so at most
    // 8 deltas, the j-th owned varint's delta in slot j / 2 whichever parity
    // the lane starts on), then the key before each lane's first (warp scan)
    T dsum = 0;
    T dv[8];
    {
      uint32_t m = own;
      unsigned long long v = vl;
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        if (m) {
          const int t = __ffs(m) - 1;
          m &= m - 1;
          if ((v & 1ull) == 0 && v < nvar) {
            dv[j >> 1] = varint_at<T>(win, bound, 16 * lane, 32 + t);
            dsum += dv[j >> 1];
          }
          ++v;
        }
      }
    }
    const T dincl = warp_incl_sum(dsum);
    T k = key + (dincl - dsum);
    {
      uint32_t m = own;
      unsigned long long v = vl;
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        if (m == 0 || v >= nvar) break;  // bytes after the last row are ignored, as the reference decodes row_count rows
        const int t = __ffs(m) - 1;
        m &= m - 1;
        if ((v & 1ull) == 0) {
          k += dv[j >> 1];
          keys[sd.row_off + v / 2 + 1] = k;
        } else {
          counts[sd.row_off + (v - 1) / 2 + 1] = (unsigned long long)(uint64_t)varint_at<T>(win, bound, 16 * lane, 32 + t);
        }
        ++v;
      }
    }
    key += warp_bcast_t(dincl, 31);
    v0 += __shfl_sync(0xffffffffu, incl, 31);
    __syncwarp();
  }
  if (d.end == lim && lim > area && lane == 0 && !is_term(bytes[lim - 1]) && v0 < nvar) {
    uint64_t p = lim;
    while (p > area && !is_term(bytes[p - 1])) --p;
    T val = 0;
    unsigned sh = 0;
    for (uint64_t q = p; q < lim; ++q) {
      if (sh < (unsigned)KeyTraits<T>::kBits) val |= (T)(bytes[q] & 0x7f) << sh;
      sh += 7;
    }
    if ((v0 & 1ull) == 0) keys[sd.row_off + v0 / 2 + 1] = key + val;
    else counts[sd.row_off + (v0 - 1) / 2 + 1] = (unsigned long long)(uint64_t)val;
  }
}

// Head row of every DVLE stream of the list sids.
template <class T>
__global__ void k_stream_heads(const uint8_t* __restrict__ bytes, const StreamDesc* __restrict__ streams,
                               const uint32_t* __restrict__ sids, uint32_t nsid, T* __restrict__ keys,
                               unsigned long long* __restrict__ counts, T* __restrict__ first_keys) {
  const uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= nsid) return;
  const uint32_t i = sids[w];
  const StreamDesc sd = streams[i];
  if (sd.rows == 0 || sd.head == 0) return;
  const uint8_t* p = bytes + sd.byte_off;
  T k = 0;
  for (int b = 0; b < (int)sizeof(T); ++b) k |= (T)p[b] << (8 * b);
  uint32_t c = 0;
  for (int b = 0; b < 4; ++b) c |= (uint32_t)p[sizeof(T) + b] << (8 * b);
  keys[sd.row_off] = k;
  counts[sd.row_off] = c;
  first_keys[i] = k;
}

template <class T>
__global__ void k_raw_rows(const uint8_t* __restrict__ bytes, const StreamDesc* __restrict__ streams,
                           const uint32_t* __restrict__ raw_ids, uint32_t nraw, T* __restrict__ keys,
                           unsigned long long* __restrict__ counts) {
  // one CTA per RAW stream
  if (blockIdx.x >= nraw) return;
  const StreamDesc sd = streams[raw_ids[blockIdx.x]];
  const uint32_t es = sizeof(T) + 4;
  for (uint64_t r = threadIdx.x; r < sd.rows; r += blockDim.x) {
    const uint8_t* p = bytes + sd.byte_off + r * es;
    T k = 0;
    for (int b = 0; b < (int)sizeof(T); ++b) k |= (T)p[b] << (8 * b);
    uint32_t c = 0;
    for (int b = 0; b < 4; ++b) c |= (uint32_t)p[sizeof(T) + b] << (8 * b);
    keys[sd.row_off + r] = k;
    counts[sd.row_off + r] = c;
  }
}

// lower_bound of `key` in the sorted rows [lo, hi) of the decoded key array.
template <class T>
__global__ void k_lower_bound(const T* __restrict__ keys, const uint64_t* __restrict__ qlo,
                              const uint64_t* __restrict__ qhi, const T* __restrict__ qkey, uint32_t nq,
                              uint64_t* __restrict__ out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nq) return;
  uint64_t lo = qlo[i], hi = qhi[i];
  const T key = qkey[i];
  while (lo < hi) {
    const uint64_t mid = lo + (hi - lo) / 2;
    if (keys[mid] < key) lo = mid + 1;
    else hi = mid;
  }
  out[i] = lo;
}

// Row position of every splitter in every stream: pos[s * (S + 1) + j] is
// lower_bound(spl[j - 1]) in stream s's rows for 1 <= j < S, the stream's
// first row for j = 0 and its end for j = S.
template <class T>
__global__ void k_range_positions(const T* __restrict__ keys, const StreamDesc* __restrict__ streams, uint32_t nst,
                                  const T* __restrict__ spl, uint32_t S, uint64_t* __restrict__ pos) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint64_t)nst * (S + 1)) return;
  const uint32_t si = (uint32_t)(i / (S + 1)), j = (uint32_t)(i % (S + 1));
  const StreamDesc sd = streams[si];
  uint64_t lo = sd.row_off, hi = sd.row_off + sd.rows;
  if (j == 0 || j == S) {
    pos[i] = j == 0 ? lo : hi;
    return;
  }
  const T key = spl[j - 1];
  while (lo < hi) {
    const uint64_t mid = lo + (hi - lo) / 2;
    if (keys[mid] < key) lo = mid + 1;
    else hi = mid;
  }
  pos[i] = lo;
}

template <class T>
__global__ void k_sample_rows(const T* __restrict__ keys, uint64_t nrows, uint32_t nsample, T* __restrict__ out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nsample) return;
  out[i] = keys[(uint64_t)((unsigned __int128)i * nrows / nsample)];
}

template <class T>
struct MergeSmem {
  static constexpr size_t keys = (size_t)kMergeCap * sizeof(T);
  static constexpr size_t cnts = (size_t)kMergeCap * 8;
  static constexpr size_t tag = (size_t)kMergeCap * 2;
  static constexpr size_t perm = (size_t)kMergeCap * 2 * 2;  // two index arrays (merge rounds ping-pong)
  static constexpr size_t head = (size_t)(kMergeCap + 1) * 2;
  // every region starts 16-byte aligned (misc holds 8-byte scan values)
  static constexpr size_t seg = ((size_t)(kMaxTileStreams + 1) * 4 + kMaxTileStreams * 4 + 15) & ~(size_t)15;
  static constexpr size_t misc = 64 * 8;
  static constexpr size_t hist = (size_t)kHistBins * 4;  // histo mode: per-CTA bins of the small counts
  static constexpr size_t total = keys + cnts + tag + perm + ((head + 15) & ~(size_t)15) + seg + misc + hist;
};

// MODE kModeMerge: `kite merge` (per-input filter on the per-input sum, u64
// totals, overflow above u32 recorded).  kModeDump: `kite dump` of one input
// (the sum clamped to u32 first, the header filter on the clamped count;
// rest_bytes of a tile = its TSV bytes, lines of k + 2 + digits).
// kModeHisto: `kite histo` of one input (load_partition_counts' u64 sum,
// apply_reader_filter_to_rows on it, then the count's frequency; no rows
// written).  kModeRows: `kite query` (every key with its u64 sum in
// aux.counts64, no filter).
template <class T, int MODE>
__global__ void __launch_bounds__(kMergeThreads) k_merge_tiles(
    const T* __restrict__ keys, const unsigned long long* __restrict__ counts, const MergeTile* __restrict__ tiles,
    const TileStream* __restrict__ ts, const InputFilter* __restrict__ filt, T* __restrict__ out_keys,
    uint32_t* __restrict__ out_counts, TileOut<T>* __restrict__ tout, unsigned long long* __restrict__ overflow,
    DevStatus* st, MergeAux aux) {
  constexpr bool DUMP = MODE == kModeDump;
  using L = MergeSmem<T>;
  constexpr int NT = kMergeThreads;
  extern __shared__ __align__(16) uint8_t sm[];
  T* sk = reinterpret_cast<T*>(sm);
  unsigned long long* sc = reinterpret_cast<unsigned long long*>(sm + L::keys);
  uint16_t* stag = reinterpret_cast<uint16_t*>(sm + L::keys + L::cnts);
  uint16_t* perm_a = reinterpret_cast<uint16_t*>(sm + L::keys + L::cnts + L::tag);
  uint16_t* perm_b = perm_a + kMergeCap;
  uint16_t* head = reinterpret_cast<uint16_t*>(sm + L::keys + L::cnts + L::tag + L::perm);
  uint32_t* sstart = reinterpret_cast<uint32_t*>(sm + L::keys + L::cnts + L::tag + L::perm +
                                                 ((L::head + 15) & ~(size_t)15));
  uint32_t* sinput = sstart + kMaxTileStreams + 1;
  unsigned long long* misc = reinterpret_cast<unsigned long long*>(reinterpret_cast<uint8_t*>(sstart) + L::seg);
  unsigned* hbin = reinterpret_cast<unsigned*>(reinterpret_cast<uint8_t*>(misc) + L::misc);

  const MergeTile mt = tiles[blockIdx.x];
  const uint32_t nts = mt.nts, n = mt.rows_in;
  if (n == 0 || nts == 0) {
    if (threadIdx.x == 0) {
      TileOut<T> o{};
      tout[blockIdx.x] = o;
    }
    return;
  }
  if (n > kMergeCap || nts > kMaxTileStreams) {
    dev_fail(st, KITE_DEV_TILE_OVERFLOW, blockIdx.x, n, nts);
    return;
  }
  if (threadIdx.x < 32) {
    // stream starts inside the tile: warp 0 scans the stream lengths
    uint32_t carry = 0;
    const uint32_t lane = threadIdx.x;
    for (uint32_t i0 = 0; i0 < nts; i0 += 32) {
      const uint32_t i = i0 + lane;
      uint32_t len = 0;
      if (i < nts) {
        const TileStream t = ts[mt.first_ts + i];
        len = (uint32_t)(t.hi - t.lo);
        sinput[i] = t.input;
      }
      uint32_t incl = len;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= (uint32_t)o) incl += y;
      }
      if (i < nts) sstart[i] = carry + incl - len;
      carry += __shfl_sync(0xffffffffu, incl, 31);
    }
    if (lane == 0) sstart[nts] = carry;
  }
  if (MODE == kModeHisto)
    for (uint32_t b = threadIdx.x; b < kHistBins; b += NT) hbin[b] = 0;
  __syncthreads();
  // load the rows of every stream: row r of the tile belongs to the last
  // stream starting at or before it
  for (uint32_t r = threadIdx.x; r < n; r += NT) {
    uint32_t lo = 0, hi = nts - 1;
    while (lo < hi) {
      const uint32_t mid = (lo + hi + 1) >> 1;
      if (sstart[mid] <= r) lo = mid;
      else hi = mid - 1;
    }
    const uint64_t src = ts[mt.first_ts + lo].lo + (r - sstart[lo]);
    sk[r] = keys[src];
    sc[r] = counts[src];
    stag[r] = (uint16_t)lo;
  }
  __syncthreads();
  // Merged order of the rows (ties in stream order): the sorted streams are
  // merged pairwise in rounds, run 2p with run 2p + 1, each round a merge
  // path (Green, McColl and Bader, 2012): thread t takes output positions
  // [t * PER, t * PER + PER) of the tile, finds where that range starts in
  // both runs of its pair by a diagonal binary search, then merges
  // sequentially.  Stable (equal keys: the earlier run first), so a group of
  // equal keys keeps stream order, i.e. input order, then chunk order.
  constexpr uint32_t PER = kMergeCap / NT;
  uint16_t* perm = perm_a;
  {
    uint16_t* src = perm_a;
    uint16_t* dst = perm_b;
    for (uint32_t r = threadIdx.x; r < n; r += NT) src[r] = (uint16_t)r;
    __syncthreads();
    for (uint32_t w = 1; w < nts; w <<= 1) {
      const uint32_t q0 = threadIdx.x * PER;
      if (q0 < n) {
        // the pair holding output q0: pairs start at stream multiples of 2w;
        // the last pair whose first row is <= q0 (empty pairs are passed over)
        uint32_t p = 0;
        {
          uint32_t lo = 0, hi = (nts + 2 * w - 1) / (2 * w) - 1;
          while (lo < hi) {
            const uint32_t mid = (lo + hi + 1) >> 1;
            if (sstart[min(mid * 2 * w, nts)] <= q0) lo = mid;
            else hi = mid - 1;
          }
          p = lo;
        }
        uint32_t q = q0;
        const uint32_t qend = min(q0 + PER, n);
        while (q < qend) {
          const uint32_t a0 = sstart[min(p * 2 * w, nts)], a1 = sstart[min(p * 2 * w + w, nts)],
                         b1 = sstart[min(p * 2 * w + 2 * w, nts)];
          const uint32_t la = a1 - a0, lb = b1 - a1, d = q - a0;
          // i = rows of run A among the pair's first d outputs
          uint32_t lo = d > lb ? d - lb : 0, hi = d < la ? d : la;
          while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (sk[src[a0 + mid]] <= sk[src[a1 + d - 1 - mid]]) lo = mid + 1;
            else hi = mid;
          }
          uint32_t i = lo, j = d - lo;
          const uint32_t stop = min(qend, b1);
          for (; q < stop; ++q) {
            const bool take_a = i < la && (j >= lb || sk[src[a0 + i]] <= sk[src[a1 + j]]);
            dst[q] = take_a ? src[a0 + i++] : src[a1 + j++];
          }
          ++p;  // the range continues in the next pair
        }
      }
      __syncthreads();
      uint16_t* t = src;
      src = dst;
      dst = t;
    }
    perm = src;
  }
  // key-group heads in merged order
  const uint32_t q0 = threadIdx.x * PER;
  uint32_t nh = 0;
#pragma unroll
  for (int i = 0; i < PER; ++i) {
    const uint32_t q = q0 + i;
    if (q < n && (q == 0 || sk[perm[q]] != sk[perm[q - 1]])) nh++;
  }
  unsigned G;
  unsigned* scan32 = reinterpret_cast<unsigned*>(misc);
  unsigned g = block_exclusive_scan<NT, unsigned>(nh, scan32, &G);
#pragma unroll
  for (int i = 0; i < PER; ++i) {
    const uint32_t q = q0 + i;
    if (q < n && (q == 0 || sk[perm[q]] != sk[perm[q - 1]])) head[g++] = (uint16_t)q;
  }
  if (threadIdx.x == 0) head[G] = (uint16_t)n;
  __syncthreads();
  // per group: per-input sums (u64 saturating), input filter, total.  Each
  // thread takes a run of consecutive groups (at most PER: G <= n <= the
  // capacity), keeping their totals in registers; one block scan compacts
  // the present ones in group order, and their keys go to shared memory for
  // the DVLE sizes: over the row counts (read by then) for u64 keys, over the
  // row keys for u128 (whose group keys are then kept in registers).
  constexpr bool KEEP_KEYS = sizeof(T) > 8;
  unsigned long long rest = 0;
  T first_key = T(0), last_key = T(0);
  uint32_t first_count = 0;
  unsigned* scan_b = scan32 + 40;
  const uint32_t gpt = (G + NT - 1) / NT;
  const uint32_t g_lo = min(G, threadIdx.x * gpt), g_hi = min(G, g_lo + gpt);
  T gkey[PER];
  unsigned long long gtot[PER];
  uint32_t pmask = 0, npres = 0;
#pragma unroll
  for (int i = 0; i < PER; ++i) {
    gkey[i] = T(0);
    gtot[i] = 0;
    const uint32_t gi = g_lo + i;
    if (gi < g_hi) {
      const uint32_t a = head[gi], b = head[gi + 1];
      if (KEEP_KEYS) gkey[i] = sk[perm[a]];
      bool present = false;
      unsigned long long total = 0;
      uint32_t cur_in = 0xffffffffu;
      unsigned long long part = 0;
      for (uint32_t q = a; q <= b; ++q) {
        const uint32_t in = q < b ? sinput[stag[perm[q]]] : 0xfffffffeu;
        if (in != cur_in) {
          if (cur_in != 0xffffffffu) {
            const InputFilter f = filt[cur_in];
            const unsigned long long eff = DUMP && part > 0xffffffffull ? 0xffffffffull : part;
            const bool ok = MODE == kModeRows ||
                            (!(f.has_min && eff < f.min_count) && !(f.has_max && eff > f.max_count));
            if (ok) {
              total = (total > ~0ull - part) ? ~0ull : total + part;
              present = true;
            }
          }
          cur_in = in;
          part = 0;
        }
        if (q < b) {
          const unsigned long long c = sc[perm[q]];
          part = (part > ~0ull - c) ? ~0ull : part + c;
        }
      }
      gtot[i] = total;
      if (present) {
        pmask |= 1u << i;
        ++npres;
      }
    }
  }
  __syncthreads();  // every row count (and for u128 every row key) has been read
  unsigned tot;
  const unsigned base = block_exclusive_scan<NT, unsigned>(npres, scan_b, &tot);
  T* outk = KEEP_KEYS ? sk : reinterpret_cast<T*>(sc);  // the present groups' keys in output order
  if (!KEEP_KEYS) {
#pragma unroll
    for (int i = 0; i < PER; ++i)
      if ((pmask >> i) & 1u) gkey[i] = sk[perm[head[g_lo + i]]];
  }
  {
    unsigned o = base;
#pragma unroll
    for (int i = 0; i < PER; ++i) {
      if (!((pmask >> i) & 1u)) continue;
      const unsigned long long total = gtot[i];
      if (MODE == kModeHisto) {
        if (total < kHistBins) {
          atomicAdd(&hbin[total], 1u);
        } else {
          const unsigned long long j = atomicAdd(aux.spill_n, 1ull);
          if (j < aux.spill_cap) aux.spill[j] = total;
        }
      } else {
        if (MODE == kModeMerge && total > 0xffffffffull)
          atomicMin(overflow, ((unsigned long long)blockIdx.x << 32) | (unsigned long long)o);
        const uint32_t c32 = total > 0xffffffffull ? 0xffffffffu : (uint32_t)total;
        out_keys[mt.out_off + o] = gkey[i];
        out_counts[mt.out_off + o] = c32;
        if (MODE == kModeRows) aux.counts64[mt.out_off + o] = total;
        if (o == 0) misc[60] = c32;
      }
      outk[o] = gkey[i];
      ++o;
    }
  }
  __syncthreads();
  if (MODE == kModeMerge || MODE == kModeDump) {
    // DVLE sizes of the rows after the tile's first (TSV line sizes for dump)
    unsigned o = base;
#pragma unroll
    for (int i = 0; i < PER; ++i) {
      if (!((pmask >> i) & 1u)) continue;
      const uint32_t cc = gtot[i] > 0xffffffffull ? 0xffffffffu : (uint32_t)gtot[i];
      if (DUMP) rest += aux.line_k + 2 + dec_digits(cc);
      else if (o > 0) rest += (unsigned long long)(varint_len((T)(gkey[i] - outk[o - 1])) + varint_len((uint64_t)cc));
      ++o;
    }
  }
  if (MODE != kModeHisto && threadIdx.x == 0 && tot) {
    first_key = outk[0];
    first_count = (uint32_t)misc[60];
    last_key = outk[tot - 1];
  }
  const unsigned long long out_base = tot;
  if (MODE == kModeHisto) {
    // the CTA's small-count bins into the global histogram
    for (uint32_t b = threadIdx.x; b < kHistBins; b += NT)
      if (hbin[b]) atomicAdd(&aux.hist[b], (unsigned long long)hbin[b]);
  }
  unsigned long long rest_total;
  block_exclusive_scan<NT, unsigned long long>(rest, misc + 8, &rest_total);
  if (threadIdx.x == 0) {
    TileOut<T> o;
    o.first_key = first_key;
    o.last_key = last_key;
    o.rows = (uint32_t)out_base;
    o.first_count = first_count;
    o.rest_bytes = rest_total;
    tout[blockIdx.x] = o;
  }
}

// TSV lines of one merged tile: rows in rounds of kTsvThreads, each round's
// lines assembled in shared memory (block scan of the line lengths), then
// stored as one contiguous run of bytes at the tile's output offset.
template <class T>
__global__ void __launch_bounds__(kTsvThreads) k_tsv_tiles(const T* __restrict__ keys,
                                                           const uint32_t* __restrict__ counts,
                                                           const MergeTile* __restrict__ tiles,
                                                           const TileOut<T>* __restrict__ tout,
                                                           const unsigned long long* __restrict__ tboff, uint32_t k,
                                                           uint8_t* __restrict__ out) {
  constexpr int NT = kTsvThreads;
  extern __shared__ __align__(16) uint8_t sm[];
  unsigned* scan = reinterpret_cast<unsigned*>(sm);
  char* buf = reinterpret_cast<char*>(sm + 256);
  const uint64_t base = tiles[blockIdx.x].out_off;
  const uint32_t rows = tout[blockIdx.x].rows;
  unsigned long long dst = tboff[blockIdx.x];
  for (uint32_t r0 = 0; r0 < rows; r0 += NT) {
    const uint32_t r = r0 + threadIdx.x;
    T key = T(0);
    uint32_t c = 0;
    unsigned len = 0;
    if (r < rows) {
      key = keys[base + r];
      c = counts[base + r];
      len = k + 2 + dec_digits(c);
    }
    unsigned tot;
    const unsigned o = block_exclusive_scan<NT, unsigned>(len, scan, &tot);
    if (len) {
      char* p = buf + o;
      for (uint32_t i = 0; i < k; ++i) p[i] = "ACGT"[(unsigned)(key >> (2 * (k - 1 - i))) & 3u];
      p[k] = '\t';
      uint32_t v = c;
      for (unsigned i = len - 2; i > k; --i) {
        p[i] = (char)('0' + v % 10);
        v /= 10;
      }
      p[len - 1] = '\n';
    }
    __syncthreads();
    // 4-byte stores on 4-byte aligned addresses; the unaligned head and tail
    // bytes one by one
    uint8_t* d8 = out + dst;
    const unsigned head = (unsigned)((4u - ((uintptr_t)d8 & 3u)) & 3u);
    if (tot < head + 8u) {
      for (unsigned i = threadIdx.x; i < tot; i += NT) d8[i] = (uint8_t)buf[i];
    } else {
      const unsigned body = (tot - head) & ~3u, tail = tot - head - body;
      if (threadIdx.x < head) d8[threadIdx.x] = (uint8_t)buf[threadIdx.x];
      if (threadIdx.x < tail) d8[head + body + threadIdx.x] = (uint8_t)buf[head + body + threadIdx.x];
      uint32_t* dw = reinterpret_cast<uint32_t*>(d8 + head);
      for (unsigned i = threadIdx.x; i < body / 4; i += NT) {
        const uint8_t* b = reinterpret_cast<const uint8_t*>(buf) + head + 4 * i;
        dw[i] = (uint32_t)b[0] | ((uint32_t)b[1] << 8) | ((uint32_t)b[2] << 16) | ((uint32_t)b[3] << 24);
      }
    }
    dst += tot;
    __syncthreads();
  }
}

// kite query lookups: key q of partition qp[q] in the merged rows of that
// partition's non-empty tiles (tile_first / tile_key0 / tile_off / tile_rows,
// first keys ascending within a partition); its u64 sum, 0 when absent.
template <class T>
__global__ void k_query_rows(const T* __restrict__ keys, const unsigned long long* __restrict__ counts64,
                             const uint32_t* __restrict__ tile_first, const T* __restrict__ tile_key0,
                             const unsigned long long* __restrict__ tile_off, const uint32_t* __restrict__ tile_rows,
                             const T* __restrict__ qk, const uint32_t* __restrict__ qp, uint32_t nq,
                             unsigned long long* __restrict__ out) {
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq) return;
  const T key = qk[q];
  const uint32_t p = qp[q];
  uint32_t lo = tile_first[p], hi = tile_first[p + 1];
  // last tile whose first key is <= key
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (tile_key0[mid] <= key) lo = mid + 1;
    else hi = mid;
  }
  unsigned long long c = 0;
  if (lo > tile_first[p]) {
    const uint32_t t = lo - 1;
    unsigned long long a = tile_off[t], b = a + tile_rows[t];
    while (a < b) {
      const unsigned long long mid = a + (b - a) / 2;
      if (keys[mid] < key) a = mid + 1;
      else b = mid;
    }
    if (a < tile_off[t] + tile_rows[t] && keys[a] == key) c = counts64[a];
  }
  out[q] = c;
}

template <class T>
struct Key128 {
  static unsigned __int128 to(T v) { return (unsigned __int128)v; }
};

// ---- host side -----------------------------------------------------------------
// A device buffer of the call: its own allocation, or a slot of the
// context's pool (kept after the call).
struct Dev {
  MergePoolSlot own;
  MergePoolSlot* sl = &own;
  void* p = nullptr;
  size_t cap = 0;
  Dev() = default;
  Dev(MergePool* pool, int slot) : sl(pool ? &pool->slot[slot] : &own) {}
  Dev(const Dev&) = delete;
  Dev& operator=(const Dev&) = delete;
  bool ensure(size_t b) {
    if (b > sl->cap) {
      cudaFree(sl->p);
      sl->p = nullptr;
      sl->cap = 0;
      if (cudaMalloc(&sl->p, b + 256) != cudaSuccess) return false;
      sl->cap = b + 256;
    }
    p = sl->p;
    cap = sl->cap;
    return true;
  }
  ~Dev() {
    if (sl == &own) cudaFree(own.p);
  }
  template <class U> U* as() { return static_cast<U*>(p); }
};

template <class T>
int merge_typed(uint32_t P, uint32_t key_bits, const kite_gpu_merge_input* in, int n, cudaStream_t s,
                uint32_t timeout_ms, int mode, kite_gpu_emit_fn emit, void* user, std::string* msg,
                kite_gpu_stats* stat, const StagingFn& staging, const MergeExtra* ex) {
  const bool dump = mode == kModeDump;
  auto fail = [&](int code, const std::string& m) {
    *msg = m;
    return code;
  };
#define MCU(call)                                                                      \
  do {                                                                                 \
    cudaError_t _e = (call);                                                           \
    if (_e != cudaSuccess) return fail(KITE_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e)); \
  } while (0)
  auto sync = [&]() { return bounded_sync(s, timeout_ms); };
  const uint32_t head_bytes = sizeof(T) + 4;
  // stage timing: [0] decode, [1] tile planning, [2] merge, [3] encode or
  // TSV formatting, [4] copy of the output to the host (events 0-3 back to
  // back, then 4-6 around the last two stages)
  cudaEvent_t sev[7];
  for (auto& e : sev)
    if (cudaEventCreate(&e) != cudaSuccess) return fail(KITE_ERR_CUDA, "event create");
  struct EvGuard {
    cudaEvent_t* e;
    ~EvGuard() {
      for (int i = 0; i < 7; ++i) cudaEventDestroy(e[i]);
    }
  } ev_guard{sev};
  for (int i = 0; i < 12; ++i) stat->stage_ms[i] = 0;
  // ---- streams (one per input chunk), bytes to the device ----
  std::vector<StreamDesc> streams;
  std::vector<uint64_t> in_base(n);
  uint64_t total_bytes = 0, total_rows = 0;
  std::vector<std::pair<uint64_t, uint64_t>> in_span(n);  // file [lo, hi) of payload bytes
  for (int i = 0; i < n; ++i) {
    uint64_t lo = UINT64_MAX, hi = 0;
    uint64_t nch = 0;
    for (uint32_t p = 0; p < P; ++p) nch = std::max<uint64_t>(nch, in[i].part_first[p] + in[i].part_count[p]);
    for (uint64_t c = 0; c < nch; ++c) {
      lo = std::min(lo, in[i].chunk_offset[c]);
      hi = std::max(hi, in[i].chunk_offset[c] + in[i].chunk_len[c]);
    }
    if (nch == 0) lo = hi = 0;
    if (hi > in[i].base_len) return fail(KITE_ERR_BAD_INPUT, "chunk out of bounds in input #" + std::to_string(i + 1));
    in_span[i] = {lo, hi};
    in_base[i] = total_bytes;
    total_bytes += (hi - lo + 15) & ~15ull;
  }
  for (uint32_t p = 0; p < P; ++p)
    for (int i = 0; i < n; ++i)
      for (uint64_t c = in[i].part_first[p]; c < in[i].part_first[p] + in[i].part_count[p]; ++c) {
        const uint32_t codec = in[i].chunk_codec[c];
        if (codec & KITE_CODEC_ZSTD) return fail(KITE_ERR_UNSUPPORTED, "zstd chunks are not supported by the GPU merge");
        StreamDesc sd{};
        sd.byte_off = in_base[i] + in[i].chunk_offset[c] - in_span[i].first;
        sd.byte_len = in[i].chunk_len[c];
        sd.rows = in[i].chunk_rows[c];
        sd.row_off = total_rows;
        sd.codec = codec;
        sd.input = (uint32_t)i;
        sd.partition = p;
        sd.head = (codec & KITE_CODEC_DVLE) ? head_bytes : 0;
        if (sd.rows && (codec & KITE_CODEC_DVLE) && sd.byte_len < head_bytes)
          return fail(KITE_ERR_BAD_INPUT, sizeof(T) == 8 ? "u64 DVLE payload too small" : "u128 DVLE payload too small");
        if (sd.rows && !(codec & KITE_CODEC_DVLE) && sd.byte_len < sd.rows * head_bytes)
          return fail(KITE_ERR_BAD_INPUT, "raw row payload truncated");
        total_rows += sd.rows;
        streams.push_back(sd);
      }
  stat->h2d_bytes += total_bytes;
  MergePool* pool = ex ? ex->pool : nullptr;
  Dev d_bytes(pool, 0), d_streams(pool, 1), d_segs(pool, 2), d_terms(pool, 3), d_vstart(pool, 4), d_dsum(pool, 5),
      d_dsum2(pool, 6), d_sfirst(pool, 7), d_send(pool, 8), d_sids(pool, 9), d_kstart(pool, 10), d_keys(pool, 11),
      d_counts(pool, 12), d_first(pool, 13), d_raw(pool, 14);
  if (!d_bytes.ensure(total_bytes + 64)) return fail(KITE_ERR_OOM, "device bytes");
  // ---- decode segments, grouped by input: each input's bytes come in on a
  // side stream and its segments are decoded as soon as they have landed, so
  // the copies of the later inputs overlap the decode of the earlier ones ----
  std::vector<SegDesc> segs;
  std::vector<uint32_t> raw_ids;
  std::vector<uint32_t> seg_first(streams.size(), 0), seg_end(streams.size(), 0);
  std::vector<uint32_t> sids;                                   // DVLE streams with rows, input by input
  std::vector<uint32_t> in_seg(n + 1, 0), in_sid(n + 1, 0);     // per input: its segment and stream-id ranges
  {
    std::vector<std::vector<uint32_t>> by_input(n);
    for (uint32_t si = 0; si < streams.size(); ++si) by_input[streams[si].input].push_back(si);
    for (int i = 0; i < n; ++i) {
      in_seg[i] = (uint32_t)segs.size();
      in_sid[i] = (uint32_t)sids.size();
      for (uint32_t si : by_input[i]) {
        const StreamDesc& sd = streams[si];
        seg_first[si] = seg_end[si] = (uint32_t)segs.size();
        if (sd.rows == 0) continue;
        if (sd.head == 0) {
          raw_ids.push_back(si);
          continue;
        }
        sids.push_back(si);
        const uint64_t a = sd.byte_off + sd.head, e = sd.byte_off + sd.byte_len;
        for (uint64_t o = a; o < e; o += kSeg) segs.push_back(SegDesc{o, std::min(o + kSeg, e), si, o == a ? 1u : 0u});
        seg_end[si] = (uint32_t)segs.size();
      }
    }
    in_seg[n] = (uint32_t)segs.size();
    in_sid[n] = (uint32_t)sids.size();
  }
  const uint32_t nseg = (uint32_t)segs.size(), nst = (uint32_t)streams.size(), nsid = (uint32_t)sids.size();
  if (!d_streams.ensure(nst * sizeof(StreamDesc) + 8) || !d_segs.ensure(nseg * sizeof(SegDesc) + 8) ||
      !d_terms.ensure(nseg * 4 + 8) || !d_vstart.ensure(nseg * 8 + 8) || !d_dsum.ensure(nseg * sizeof(T) + 16) ||
      !d_dsum2.ensure(nseg * sizeof(T) + 16) || !d_kstart.ensure(nseg * sizeof(T) + 16) ||
      !d_keys.ensure(total_rows * sizeof(T) + 16) || !d_counts.ensure(total_rows * 8 + 16) ||
      !d_first.ensure(nst * sizeof(T) + 16) || !d_raw.ensure(raw_ids.size() * 4 + 8) ||
      !d_sfirst.ensure(nst * 4 + 8) || !d_send.ensure(nst * 4 + 8) || !d_sids.ensure(nsid * 4 + 8))
    return fail(KITE_ERR_OOM, "merge decode buffers");
  MCU(cudaMemcpyAsync(d_streams.p, streams.data(), nst * sizeof(StreamDesc), cudaMemcpyHostToDevice, s));
  if (nseg) MCU(cudaMemcpyAsync(d_segs.p, segs.data(), nseg * sizeof(SegDesc), cudaMemcpyHostToDevice, s));
  if (nst) {
    MCU(cudaMemcpyAsync(d_sfirst.p, seg_first.data(), nst * 4, cudaMemcpyHostToDevice, s));
    MCU(cudaMemcpyAsync(d_send.p, seg_end.data(), nst * 4, cudaMemcpyHostToDevice, s));
  }
  if (nsid) MCU(cudaMemcpyAsync(d_sids.p, sids.data(), nsid * 4, cudaMemcpyHostToDevice, s));
  if (!raw_ids.empty())
    MCU(cudaMemcpyAsync(d_raw.p, raw_ids.data(), raw_ids.size() * 4, cudaMemcpyHostToDevice, s));
  int launches = 0;
  DevStatus* dst = nullptr;
  MCU(cudaMallocAsync(&dst, sizeof(DevStatus), s));
  MCU(cudaMemsetAsync(dst, 0, sizeof(DevStatus), s));
  // copy lane: the side stream, one landing event per input, timing events
  // around the copies ([0], [1]) and around each input's decode ([2 + 2i],
  // [3 + 2i]: recorded after the wait, so they time the kernels only)
  struct CopyLane {
    cudaStream_t cs = nullptr;
    std::vector<cudaEvent_t> ev, tev;
    ~CopyLane() {
      for (auto e : ev) cudaEventDestroy(e);
      for (auto e : tev) cudaEventDestroy(e);
      if (cs) cudaStreamDestroy(cs);
    }
  } cl;
  MCU(cudaStreamCreateWithFlags(&cl.cs, cudaStreamNonBlocking));
  cl.ev.resize(n, nullptr);
  for (int i = 0; i < n; ++i) MCU(cudaEventCreateWithFlags(&cl.ev[i], cudaEventDisableTiming));
  cl.tev.resize(2 + 2 * (size_t)n, nullptr);
  for (auto& e : cl.tev) MCU(cudaEventCreate(&e));
  MCU(cudaEventRecord(sev[0], s));
  MCU(cudaEventRecord(cl.tev[0], cl.cs));
  for (int i = 0; i < n; ++i) {
    if (in_span[i].second > in_span[i].first)
      MCU(cudaMemcpyAsync(d_bytes.as<uint8_t>() + in_base[i], in[i].base + in_span[i].first,
                          in_span[i].second - in_span[i].first, cudaMemcpyHostToDevice, cl.cs));
    MCU(cudaEventRecord(cl.ev[i], cl.cs));
  }
  MCU(cudaEventRecord(cl.tev[1], cl.cs));
  const uint64_t lim_pad = total_bytes + 64;  // every aligned 16-byte block below this is readable
  for (int i = 0; i < n; ++i) {
    MCU(cudaStreamWaitEvent(s, cl.ev[i], 0));
    MCU(cudaEventRecord(cl.tev[2 + 2 * i], s));
    const uint32_t s0 = in_seg[i], ns = in_seg[i + 1] - in_seg[i];
    const uint32_t q0 = in_sid[i], nq = in_sid[i + 1] - in_sid[i];
    if (nq) {
      k_stream_heads<T><<<(nq + 255) / 256, 256, 0, s>>>(d_bytes.as<uint8_t>(), d_streams.as<StreamDesc>(),
                                                         d_sids.as<uint32_t>() + q0, nq, d_keys.as<T>(),
                                                         d_counts.as<unsigned long long>(), d_first.as<T>());
      launches++;
    }
    if (ns) {
      // DVLE varints: pass A (per-segment counts and parity sums), the
      // per-stream scans, pass B (rows); no host round trip
      const unsigned gsegs = (ns + kDecWarps - 1) / kDecWarps;
      k_seg_pass_a<T><<<gsegs, 32 * kDecWarps, 0, s>>>(d_bytes.as<uint8_t>(), lim_pad, d_segs.as<SegDesc>() + s0, ns,
                                                       d_streams.as<StreamDesc>(), d_terms.as<uint32_t>() + s0,
                                                       d_dsum.as<T>() + s0, d_dsum2.as<T>() + s0);
      k_stream_seg_scan<T><<<(nq + 7) / 8, 256, 0, s>>>(d_terms.as<uint32_t>(), d_dsum.as<T>(), d_dsum2.as<T>(),
                                                        d_sfirst.as<uint32_t>(), d_send.as<uint32_t>(),
                                                        d_streams.as<StreamDesc>(), d_first.as<T>(),
                                                        d_sids.as<uint32_t>() + q0, nq,
                                                        d_vstart.as<unsigned long long>(), d_kstart.as<T>(), dst);
      k_seg_rows<T><<<gsegs, 32 * kDecWarps, 0, s>>>(d_bytes.as<uint8_t>(), lim_pad, d_segs.as<SegDesc>() + s0, ns,
                                                     d_streams.as<StreamDesc>(), d_vstart.as<unsigned long long>() + s0,
                                                     d_kstart.as<T>() + s0, d_keys.as<T>(),
                                                     d_counts.as<unsigned long long>());
      launches += 3;
    }
    MCU(cudaEventRecord(cl.tev[3 + 2 * i], s));
  }
  if (!raw_ids.empty()) {
    k_raw_rows<T><<<(unsigned)raw_ids.size(), 256, 0, s>>>(d_bytes.as<uint8_t>(), d_streams.as<StreamDesc>(),
                                                           d_raw.as<uint32_t>(), (uint32_t)raw_ids.size(),
                                                           d_keys.as<T>(), d_counts.as<unsigned long long>());
    launches++;
  }
  DevStatus hdec{};
  MCU(cudaMemcpyAsync(&hdec, dst, sizeof hdec, cudaMemcpyDeviceToHost, s));
  MCU(cudaEventRecord(sev[1], s));
  // planning phases, host wall clock (the decode's kernels run meanwhile until
  // the first wait): [6] splitters, [7] first cut, [8] bisection, [9] tile lists
  auto wall = []() { return std::chrono::steady_clock::now(); };
  auto ms_since = [](std::chrono::steady_clock::time_point a) {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - a).count();
  };
  auto tp0 = wall();
  // ---- tiles: global splitters from a row sample, refined by bisection ----
  std::vector<uint32_t> part_first_stream(P + 1, 0);
  {
    uint32_t si = 0;
    for (uint32_t p = 0; p < P; ++p) {
      part_first_stream[p] = si;
      while (si < nst && streams[si].partition == p) si++;
    }
    part_first_stream[P] = nst;
  }
  // tiles of three quarters of the on-chip capacity on average (the
  // refinement below splits the few that the cut leaves above it): the merge
  // kernel's cost per tile is mostly fixed (stream scan, merge rounds,
  // barriers), so fuller tiles cost less per row
  uint32_t S = 1;
  {
    const double want = (double)total_rows / ((double)P * 0.75 * kMergeCap);
    if (want > 1.0) S = (uint32_t)std::min(4096.0, std::ceil(want));
  }
  std::vector<T> spl;
  Dev d_spl;
  if (S > 1 && total_rows) {
    const uint32_t ns = (uint32_t)std::min<uint64_t>(total_rows, 1u << 20);
    Dev d_sample, d_hist;
    if (!d_sample.ensure(ns * sizeof(T)) || !d_spl.ensure(S * sizeof(T)) || !d_hist.ensure(65536 * 4))
      return fail(KITE_ERR_OOM, "merge splitters");
    k_sample_rows<T><<<(ns + 255) / 256, 256, 0, s>>>(d_keys.as<T>(), total_rows, ns, d_sample.as<T>());
    // sampling every m-th row of the concatenated streams is a uniform sample
    // of the key multiset; key bits from the input k
    launches += 1 + compute_hist_splitters<T>(d_sample.as<T>(), ns, key_bits, S, d_spl.as<T>(),
                                              d_hist.as<unsigned>(), s);
    stat->splitter_used = KITE_SPLIT_SAMPLED;
    if (ex && ex->mlp && ex->splitter_mode != KITE_SPLIT_SAMPLED) {
      // the learned CDF of the row sample cuts the merged key range; kept
      // when its predicted max/mean tile load is the lower one (LEARNED: always)
      double hist_imb = 0.0;
      if (predict_imbalance<T>(ex->mlp, d_sample.as<T>(), ns, d_spl.as<T>(), S, s, timeout_ms, &hist_imb))
        return fail(KITE_ERR_TIMEOUT, "merge splitter evaluation did not finish");
      Dev d_spl2;
      if (!d_spl2.ensure(S * sizeof(T))) return fail(KITE_ERR_OOM, "merge splitters");
      MlpReport rep;
      if (mlp_splitters<T>(ex->mlp, d_sample.as<T>(), ns, key_bits, S, d_spl2.as<T>(), s, timeout_ms, &rep))
        return fail(KITE_ERR_CUDA, "learned splitter training failed");
      launches += 1 + rep.launches;
      stat->hist_pred_imbalance = hist_imb;
      stat->mlp_pred_imbalance = rep.pred_imbalance;
      stat->mlp_loss = rep.loss;
      stat->mlp_reused = rep.reused ? 1u : 0u;
      if (rep.pred_imbalance < 1e29 && (ex->splitter_mode == KITE_SPLIT_LEARNED || rep.pred_imbalance < hist_imb)) {
        MCU(cudaMemcpyAsync(d_spl.p, d_spl2.p, (S - 1) * sizeof(T), cudaMemcpyDeviceToDevice, s));
        stat->splitter_used = KITE_SPLIT_LEARNED;
      }
      if (sync()) return fail(KITE_ERR_TIMEOUT, "merge splitter wait");
    }
    spl.resize(S - 1);
    MCU(cudaMemcpyAsync(spl.data(), d_spl.p, (S - 1) * sizeof(T), cudaMemcpyDeviceToHost, s));
  } else {
    S = 1;
  }
  stat->stage_ms[6] = ms_since(tp0);
  auto tp1 = wall();
  // ---- first cut on the device: the row position of every splitter in every
  // stream (one binary search each), read back as one matrix
  const size_t SP = (size_t)S + 1;
  std::vector<uint64_t> pos((size_t)nst * SP);
  if (nst && S > 1) {
    Dev d_pos;
    if (!d_pos.ensure(pos.size() * 8)) return fail(KITE_ERR_OOM, "merge range positions");
    const uint64_t nq = pos.size();
    k_range_positions<T><<<(unsigned)((nq + 255) / 256), 256, 0, s>>>(d_keys.as<T>(), d_streams.as<StreamDesc>(), nst,
                                                                     d_spl.as<T>(), S, d_pos.as<uint64_t>());
    launches++;
    MCU(cudaMemcpyAsync(pos.data(), d_pos.p, nq * 8, cudaMemcpyDeviceToHost, s));
    if (sync()) return fail(KITE_ERR_TIMEOUT, "merge range wait");
  } else {
    if (sync()) return fail(KITE_ERR_TIMEOUT, "merge splitter wait");
    for (uint32_t si = 0; si < nst; ++si) {
      pos[si * SP] = streams[si].row_off;
      pos[si * SP + 1] = streams[si].row_off + streams[si].rows;
    }
  }
  // A finished range: partition, low key, and the offset of its per-stream
  // [lo, hi) row positions in dlo / dhi (one entry per stream of the
  // partition).  Ranges above the on-chip capacity are bisected by key.
  struct Done {
    uint32_t p;
    T lo;
    uint64_t off;
  };
  struct Range {
    uint32_t p;
    T lo, hi;
    bool open_hi;
  };
  // First cut, partitions in parallel on the host threads: each range that
  // fits on chip becomes a finished range of its partition, the rest go to
  // the bisection below.
  const unsigned hthreads = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
  auto parallel_parts = [&](auto&& fn) {
    std::vector<std::thread> th;
    for (unsigned t = 0; t < hthreads; ++t)
      th.emplace_back([&, t]() {
        for (uint32_t p = t; p < P; p += hthreads) fn(p);
      });
    for (auto& x : th) x.join();
  };
  struct PartCut {
    std::vector<Done> done;
    std::vector<uint64_t> dlo, dhi;
    std::vector<Range> work;
  };
  std::vector<PartCut> cut(P);
  parallel_parts([&](uint32_t p) {
    PartCut& c = cut[p];
    const uint32_t f = part_first_stream[p], nstr = part_first_stream[p + 1] - f;
    if (!nstr) return;
    for (uint32_t j = 0; j < S; ++j) {
      const T lo = j ? spl[j - 1] : T(0);
      const bool open_hi = j + 1 == S;
      const T hi = open_hi ? T(0) : spl[j];
      if (!open_hi && hi <= lo) continue;  // empty (repeated splitter)
      uint64_t rows = 0;
      for (uint32_t k2 = 0; k2 < nstr; ++k2) rows += pos[(f + k2) * SP + j + 1] - pos[(f + k2) * SP + j];
      if (rows == 0) continue;
      if (rows <= kMergeCap && nstr <= kMaxTileStreams) {
        c.done.push_back(Done{p, lo, (uint64_t)c.dlo.size()});
        for (uint32_t k2 = 0; k2 < nstr; ++k2) {
          c.dlo.push_back(pos[(f + k2) * SP + j]);
          c.dhi.push_back(pos[(f + k2) * SP + j + 1]);
        }
      } else {
        c.work.push_back(Range{p, lo, hi, open_hi});
      }
    }
  });
  stat->stage_ms[7] = ms_since(tp1);
  auto tp2 = wall();
  std::vector<Done> done;  // ranges finished by the bisection (offsets into dlo / dhi)
  std::vector<uint64_t> dlo, dhi;
  std::vector<Range> work;
  for (uint32_t p = 0; p < P; ++p) work.insert(work.end(), cut[p].work.begin(), cut[p].work.end());
  std::vector<uint64_t>().swap(pos);
  // the decode's status arrived with the sync above
  if (hdec.code == KITE_DEV_SHORT_VARINTS)
    return fail(KITE_ERR_BAD_INPUT, sizeof(T) == 8 ? "invalid u64 DVLE delta" : "invalid u128 DVLE delta");
  Dev d_qlo, d_qhi, d_qkey, d_qout;
  std::vector<uint64_t> lp, hp;
  for (int round = 0; !work.empty() && round < 200; ++round) {
    // queries: for every range and stream, lower_bound(lo) and lower_bound(hi)
    std::vector<uint64_t> qlo, qhi;
    std::vector<T> qkey;
    for (auto& r : work)
      for (uint32_t si = part_first_stream[r.p]; si < part_first_stream[r.p + 1]; ++si) {
        const uint64_t a = streams[si].row_off, b = a + streams[si].rows;
        qlo.push_back(a);
        qhi.push_back(b);
        qkey.push_back(r.lo);
        qlo.push_back(a);
        qhi.push_back(b);
        qkey.push_back(r.open_hi ? T(0) : r.hi);
      }
    const uint32_t nq = (uint32_t)qlo.size();
    if (!d_qlo.ensure(nq * 8) || !d_qhi.ensure(nq * 8) || !d_qkey.ensure(nq * sizeof(T)) || !d_qout.ensure(nq * 8))
      return fail(KITE_ERR_OOM, "merge tile queries");
    MCU(cudaMemcpyAsync(d_qlo.p, qlo.data(), nq * 8, cudaMemcpyHostToDevice, s));
    MCU(cudaMemcpyAsync(d_qhi.p, qhi.data(), nq * 8, cudaMemcpyHostToDevice, s));
    MCU(cudaMemcpyAsync(d_qkey.p, qkey.data(), nq * sizeof(T), cudaMemcpyHostToDevice, s));
    k_lower_bound<T><<<(nq + 255) / 256, 256, 0, s>>>(d_keys.as<T>(), d_qlo.as<uint64_t>(), d_qhi.as<uint64_t>(),
                                                      d_qkey.as<T>(), nq, d_qout.as<uint64_t>());
    launches++;
    std::vector<uint64_t> qout(nq);
    MCU(cudaMemcpyAsync(qout.data(), d_qout.p, nq * 8, cudaMemcpyDeviceToHost, s));
    if (sync()) return fail(KITE_ERR_TIMEOUT, "merge tile wait");
    std::vector<Range> next;
    size_t q = 0;
    for (auto& r : work) {
      uint64_t rows = 0;
      lp.clear();
      hp.clear();
      for (uint32_t si = part_first_stream[r.p]; si < part_first_stream[r.p + 1]; ++si) {
        const uint64_t a = qout[q++], b0 = qout[q++];
        const uint64_t b = r.open_hi ? streams[si].row_off + streams[si].rows : b0;
        lp.push_back(a);
        hp.push_back(b);
        rows += b - a;
      }
      const uint32_t nstr = part_first_stream[r.p + 1] - part_first_stream[r.p];
      const T hi_eff = r.open_hi ? (sizeof(T) == 8 ? (T)~0ull : ~T(0)) : r.hi;
      if (rows > kMergeCap && hi_eff - r.lo > T(1)) {
        const T mid = r.lo + (hi_eff - r.lo) / 2;
        Range a = r, b = r;
        a.hi = mid;
        a.open_hi = false;
        b.lo = mid;
        next.push_back(a);
        next.push_back(b);
      } else {
        if (rows > kMergeCap || nstr > kMaxTileStreams)
          return fail(KITE_ERR_UNSUPPORTED, "merge tile cannot be split below the on-chip capacity");
        if (rows) {
          done.push_back(Done{r.p, r.lo, (uint64_t)dlo.size()});
          dlo.insert(dlo.end(), lp.begin(), lp.end());
          dhi.insert(dhi.end(), hp.begin(), hp.end());
        }
      }
    }
    work.swap(next);
  }
  if (!work.empty()) return fail(KITE_ERR_UNSUPPORTED, "merge tile refinement did not converge");
  stat->stage_ms[8] = ms_since(tp2);
  auto tp3 = wall();
  // ---- tile lists: per partition (in parallel) its finished ranges in key
  // order, then the partitions concatenated with their offsets ----
  std::vector<std::vector<Done>> refined(P);
  for (const Done& d : done) refined[d.p].push_back(d);
  struct PartTiles {
    std::vector<MergeTile> mts;
    std::vector<TileStream> tss;
    uint64_t rows = 0;
  };
  std::vector<PartTiles> pt(P);
  parallel_parts([&](uint32_t p) {
    PartTiles& o = pt[p];
    PartCut& c = cut[p];
    std::vector<Done>& rf = refined[p];
    std::sort(rf.begin(), rf.end(), [](const Done& a, const Done& b) { return a.lo < b.lo; });
    const uint32_t f = part_first_stream[p], nstr = part_first_stream[p + 1] - f;
    size_t i = 0, r = 0;
    while (i < c.done.size() || r < rf.size()) {
      const bool from_cut = r >= rf.size() || (i < c.done.size() && c.done[i].lo < rf[r].lo);
      const Done& d = from_cut ? c.done[i++] : rf[r++];
      const uint64_t* lo_v = from_cut ? c.dlo.data() : dlo.data();
      const uint64_t* hi_v = from_cut ? c.dhi.data() : dhi.data();
      MergeTile mt{};
      mt.out_off = o.rows;  // relative to the partition until concatenated
      mt.first_ts = (uint32_t)o.tss.size();
      mt.partition = p;
      uint64_t rows = 0;
      for (uint32_t k2 = 0; k2 < nstr; ++k2) {
        const uint64_t lo = lo_v[d.off + k2], hi = hi_v[d.off + k2];
        if (hi == lo) continue;
        o.tss.push_back(TileStream{lo, hi, streams[f + k2].input, 0});
        rows += hi - lo;
      }
      mt.nts = (uint32_t)(o.tss.size() - mt.first_ts);
      mt.rows_in = (uint32_t)rows;
      o.rows += rows;
      o.mts.push_back(mt);
    }
    std::vector<Done>().swap(c.done);
    std::vector<uint64_t>().swap(c.dlo);
    std::vector<uint64_t>().swap(c.dhi);
  });
  // the partitions' offsets, then every partition's tiles and stream ranges
  // written in place in parallel, the stream ranges straight into pinned
  // memory for their copy to the device
  std::vector<MergeTile> mts;
  std::vector<TileDesc> tds;
  std::vector<uint32_t> tile_first(P + 1, 0);
  std::vector<uint64_t> ts_first(P + 1, 0), row_first(P + 1, 0);
  for (uint32_t p = 0; p < P; ++p) {
    tile_first[p + 1] = tile_first[p] + (uint32_t)pt[p].mts.size();
    ts_first[p + 1] = ts_first[p] + pt[p].tss.size();
    row_first[p + 1] = row_first[p] + pt[p].rows;
  }
  const uint64_t out_off = row_first[P];
  const size_t nts_all = (size_t)ts_first[P];
  mts.resize(tile_first[P]);
  tds.resize(tile_first[P]);
  std::vector<TileStream> tss_own;
  TileStream* tss = nullptr;
  if (pool) {
    MergePoolSlot& hs = pool->host;
    const size_t need = nts_all * sizeof(TileStream) + 64;
    if (hs.cap < need) {
      if (hs.p) cudaFreeHost(hs.p);
      hs.p = nullptr;
      hs.cap = 0;
      if (cudaMallocHost(&hs.p, need) != cudaSuccess) return fail(KITE_ERR_OOM, "merge tile lists (pinned)");
      hs.cap = need;
    }
    tss = static_cast<TileStream*>(hs.p);
  } else {
    tss_own.resize(nts_all + 1);
    tss = tss_own.data();
  }
  parallel_parts([&](uint32_t p) {
    PartTiles& o = pt[p];
    const uint32_t t0 = tile_first[p], s0 = (uint32_t)ts_first[p];
    for (size_t i = 0; i < o.mts.size(); ++i) {
      MergeTile mt = o.mts[i];
      mt.out_off += row_first[p];
      mt.first_ts += s0;
      tds[t0 + i] = TileDesc{mt.out_off, 0, p};
      mts[t0 + i] = mt;
    }
    if (!o.tss.empty()) std::memcpy(tss + s0, o.tss.data(), o.tss.size() * sizeof(TileStream));
    PartTiles().mts.swap(o.mts);
    PartTiles().tss.swap(o.tss);
  });
  stat->stage_ms[9] = ms_since(tp3);
  const uint32_t ntiles = (uint32_t)mts.size();
  std::vector<InputFilter> filt(n);
  for (int i = 0; i < n; ++i)
    filt[i] = InputFilter{(uint32_t)in[i].has_min, (uint32_t)in[i].has_max, in[i].min_count, in[i].max_count};
  Dev d_mt(pool, 15), d_ts(pool, 16), d_filt(pool, 17), d_okeys(pool, 18), d_ocounts(pool, 19), d_tout(pool, 20),
      d_over(pool, 21), d_tds(pool, 22), d_tf(pool, 23), d_boff(pool, 24), d_prev(pool, 25), d_meta(pool, 26),
      d_out(pool, 27);
  if (!d_mt.ensure(ntiles * sizeof(MergeTile) + 8) || !d_ts.ensure(nts_all * sizeof(TileStream) + 8) ||
      !d_filt.ensure(n * sizeof(InputFilter)) || !d_okeys.ensure(out_off * sizeof(T) + 16) ||
      !d_ocounts.ensure(out_off * 4 + 16) || !d_tout.ensure(ntiles * sizeof(TileOut<T>) + 16) ||
      !d_over.ensure(8) || !d_tds.ensure(ntiles * sizeof(TileDesc) + 8) || !d_tf.ensure((P + 1) * 4) ||
      !d_boff.ensure(ntiles * 8 + 8) || !d_prev.ensure(ntiles * sizeof(T) + 16) || !d_meta.ensure(P * sizeof(BucketMeta)))
    return fail(KITE_ERR_OOM, "merge tile buffers");
  if (ntiles) {
    MCU(cudaMemcpyAsync(d_mt.p, mts.data(), ntiles * sizeof(MergeTile), cudaMemcpyHostToDevice, s));
    MCU(cudaMemcpyAsync(d_ts.p, tss, nts_all * sizeof(TileStream), cudaMemcpyHostToDevice, s));
  }
  MCU(cudaMemcpyAsync(d_filt.p, filt.data(), n * sizeof(InputFilter), cudaMemcpyHostToDevice, s));
  MCU(cudaMemsetAsync(d_over.p, 0xff, 8, s));
  const size_t smem = MergeSmem<T>::total;
  auto kmerge = mode == kModeDump    ? k_merge_tiles<T, kModeDump>
                : mode == kModeHisto ? k_merge_tiles<T, kModeHisto>
                : mode == kModeRows  ? k_merge_tiles<T, kModeRows>
                                     : k_merge_tiles<T, kModeMerge>;
  cudaFuncSetAttribute(kmerge, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  MergeAux aux{};
  aux.line_k = key_bits / 2;
  Dev d_hist, d_spill, d_c64;
  if (mode == kModeHisto) {
    if (!d_hist.ensure((kHistBins + 1) * 8) || !d_spill.ensure(out_off * 8 + 8)) return fail(KITE_ERR_OOM, "histo buffers");
    MCU(cudaMemsetAsync(d_hist.p, 0, (kHistBins + 1) * 8, s));
    aux.hist = d_hist.as<unsigned long long>();
    aux.spill_n = aux.hist + kHistBins;
    aux.spill = d_spill.as<unsigned long long>();
    aux.spill_cap = out_off;
  }
  if (mode == kModeRows) {
    if (!d_c64.ensure(out_off * 8 + 8)) return fail(KITE_ERR_OOM, "query buffers");
    aux.counts64 = d_c64.as<unsigned long long>();
  }
  if (mode == kModeMerge && ntiles) {
    // ---- merge, encode and copy-out pipelined over partition groups: group
    // g's payload copies to the host (on the input copy lane, idle by now)
    // while group g + 1 merges.  The offsets kernel writes each group's
    // partition records into mapped pinned memory, so the host sizes the
    // group's encode without a copy that would queue on a copy engine. ----
    const uint32_t NG = std::min<uint32_t>(8, P);
    std::vector<uint32_t> pb(NG + 1);
    for (uint32_t g = 0; g <= NG; ++g) pb[g] = (uint32_t)((uint64_t)P * g / NG);
    if (NG == 8 && P >= 64) {
      // tapering groups (weights 6,6,6,6,6,5,3,2 of 40): the last copy-out,
      // which nothing overlaps, carries about a twentieth of the output
      static const uint32_t cw[9] = {0, 6, 12, 18, 24, 30, 35, 38, 40};
      for (uint32_t g = 0; g <= NG; ++g) pb[g] = (uint32_t)((uint64_t)P * cw[g] / 40);
    }
    MCU(cudaMemcpyAsync(d_tds.p, tds.data(), ntiles * sizeof(TileDesc), cudaMemcpyHostToDevice, s));
    MCU(cudaMemcpyAsync(d_tf.p, tile_first.data(), (P + 1) * 4, cudaMemcpyHostToDevice, s));
    if (!d_over.ensure((size_t)NG * 8)) return fail(KITE_ERR_OOM, "merge tile buffers");
    MCU(cudaMemsetAsync(d_over.p, 0xff, (size_t)NG * 8, s));  // per group: its first overflowing row
    struct HostMem {
      void* p = nullptr;
      ~HostMem() {
        if (p) cudaFreeHost(p);
      }
    } hmm;
    MCU(cudaMallocHost(&hmm.p, (size_t)P * sizeof(BucketMeta)));
    BucketMeta* hm = static_cast<BucketMeta*>(hmm.p);
    BucketMeta* hm_dev = nullptr;
    MCU(cudaHostGetDevicePointer(reinterpret_cast<void**>(&hm_dev), hm, 0));
    // output buffers: the inputs' payload size to start with (a merged
    // partition's rows are at most its inputs' rows); a group that needs more
    // grows them once every queued encode and copy has finished
    uint64_t cap = std::max<uint64_t>(total_bytes, 1ull << 20) + 16;
    if (!d_out.ensure(cap)) return fail(KITE_ERR_OOM, "merge output");
    uint8_t* hout = staging ? staging(cap) : nullptr;
    std::unique_ptr<uint8_t[]> hown;
    if (!hout) {
      hown.reset(new (std::nothrow) uint8_t[cap]);
      if (!hown) return fail(KITE_ERR_OOM, "merge output host buffer");
      hout = hown.get();
    }
    DevStatus* est = nullptr;
    MCU(cudaMallocAsync(&est, sizeof(DevStatus), s));
    MCU(cudaMemsetAsync(est, 0, sizeof(DevStatus), s));
    struct Evs {
      std::vector<cudaEvent_t> e;
      ~Evs() {
        for (auto x : e) cudaEventDestroy(x);
      }
    } gv;
    gv.e.resize(7 * (size_t)NG, nullptr);
    for (auto& e : gv.e) MCU(cudaEventCreate(&e));
    cudaEvent_t* ge = gv.e.data();  // per group: merge, merged, linked | encode start, end | copy start, end
    MCU(cudaEventRecord(sev[2], s));
    auto queue_merge = [&](uint32_t g) -> cudaError_t {
      const uint32_t pa = pb[g], pe = pb[g + 1], ta = tile_first[pa], tb = tile_first[pe];
      cudaEventRecord(ge[7 * g], s);
      if (tb > ta)
        kmerge<<<tb - ta, kMergeThreads, smem, s>>>(d_keys.as<T>(), d_counts.as<unsigned long long>(),
                                                    d_mt.as<MergeTile>() + ta, d_ts.as<TileStream>(),
                                                    d_filt.as<InputFilter>(), d_okeys.as<T>(), d_ocounts.as<uint32_t>(),
                                                    d_tout.as<TileOut<T>>() + ta, d_over.as<unsigned long long>() + g,
                                                    dst, aux);
      cudaEventRecord(ge[7 * g + 1], s);
      if (pe > pa) {
        launch_tile_link_ranges<T>(d_tout.as<TileOut<T>>(), pe - pa, d_tf.as<uint32_t>() + pa,
                                   d_boff.as<unsigned long long>(), d_prev.as<T>(), d_meta.as<BucketMeta>() + pa, s);
        launch_bucket_offsets(d_meta.as<BucketMeta>() + pa, pe - pa, hm_dev + pa, s);
      }
      cudaEventRecord(ge[7 * g + 2], s);
      return cudaGetLastError();
    };
    std::vector<uint64_t> gbase(NG, 0);
    uint64_t total_out = 0, out_rows = 0;
    MCU(queue_merge(0));
    for (uint32_t g = 0; g < NG; ++g) {
      if (g + 1 < NG) MCU(queue_merge(g + 1));
      launches += 3;
      if (bounded_event_wait(ge[7 * g + 2], timeout_ms)) return fail(KITE_ERR_TIMEOUT, "merge group wait");
      const uint32_t pa = pb[g], pe = pb[g + 1], ta = tile_first[pa], tb = tile_first[pe];
      uint64_t gbytes = 0;
      for (uint32_t p = pa; p < pe; ++p) {
        gbytes += hm[p].bytes;
        out_rows += hm[p].rows;
      }
      if (total_out + gbytes + 16 > cap) {
        // every earlier group's bytes are on the host once the copy lane is
        // idle: the device buffer is replaced, the host one grown with them
        if (bounded_sync(s, timeout_ms) || bounded_sync(cl.cs, timeout_ms))
          return fail(KITE_ERR_TIMEOUT, "merge output wait");
        const uint64_t ncap = total_out + gbytes + 16 + (total_out + gbytes) / 4;
        if (!d_out.ensure(ncap)) return fail(KITE_ERR_OOM, "merge output");
        std::unique_ptr<uint8_t[]> nh(new (std::nothrow) uint8_t[ncap]);
        if (!nh) return fail(KITE_ERR_OOM, "merge output host buffer");
        std::memcpy(nh.get(), hout, total_out);
        hown = std::move(nh);
        hout = hown.get();
        cap = ncap;
      }
      gbase[g] = total_out;
      MCU(cudaEventRecord(ge[7 * g + 3], s));
      // k_encode places a partition's bytes at its record's offset (relative
      // to the group) plus the tile's: the group's slice of the output
      if (tb > ta)
        launch_encode<T>(d_okeys.as<T>(), d_ocounts.as<uint32_t>(), d_tds.as<TileDesc>() + ta,
                         d_tout.as<TileOut<T>>() + ta, d_boff.as<unsigned long long>() + ta, d_prev.as<T>() + ta,
                         d_meta.as<BucketMeta>(), tb - ta, d_out.as<uint8_t>() + total_out, gbytes, est, s);
      MCU(cudaEventRecord(ge[7 * g + 4], s));
      MCU(cudaStreamWaitEvent(cl.cs, ge[7 * g + 4], 0));
      MCU(cudaEventRecord(ge[7 * g + 5], cl.cs));
      if (gbytes)
        MCU(cudaMemcpyAsync(hout + total_out, d_out.as<uint8_t>() + total_out, gbytes, cudaMemcpyDeviceToHost, cl.cs));
      MCU(cudaEventRecord(ge[7 * g + 6], cl.cs));
      total_out += gbytes;
    }
    MCU(cudaEventRecord(sev[3], s));
    std::vector<unsigned long long> overs(NG);
    DevStatus hst{}, hest{};
    MCU(cudaMemcpyAsync(&hst, dst, sizeof hst, cudaMemcpyDeviceToHost, s));
    MCU(cudaMemcpyAsync(&hest, est, sizeof hest, cudaMemcpyDeviceToHost, s));
    MCU(cudaMemcpyAsync(overs.data(), d_over.p, (size_t)NG * 8, cudaMemcpyDeviceToHost, s));
    if (bounded_sync(s, timeout_ms) || bounded_sync(cl.cs, timeout_ms)) return fail(KITE_ERR_TIMEOUT, "merge wait");
    cudaFreeAsync(dst, s);
    cudaFreeAsync(est, s);
    if (hst.code) {
      char b[160];
      snprintf(b, sizeof b, "merge: device status %u (%u, %u, %u)", hst.code, hst.a, hst.b, hst.c);
      return fail(hst.code == KITE_DEV_BAD_INPUT ? KITE_ERR_BAD_INPUT : KITE_ERR_DEVICE, b);
    }
    for (uint32_t g = 0; g < NG; ++g) {
      if (overs[g] == ~0ull) continue;
      // first overflowing row in (partition, key) order: name its key like the reference
      const uint32_t t = tile_first[pb[g]] + (uint32_t)(overs[g] >> 32), r = (uint32_t)(overs[g] & 0xffffffffu);
      T key{};
      MCU(cudaMemcpy(&key, d_okeys.as<T>() + mts[t].out_off + r, sizeof(T), cudaMemcpyDeviceToHost));
      unsigned __int128 v = (unsigned __int128)key;
      std::string ks;
      if (v == 0) ks = "0";
      while (v) {
        ks.insert(ks.begin(), (char)('0' + (int)(v % 10)));
        v /= 10;
      }
      return fail(KITE_ERR_COUNT_OVERFLOW, "merged count exceeds u32 for key " + ks);
    }
    if (hest.code) return fail(KITE_ERR_DEVICE, "merge encode failed");
    // stage times: decode, planning and the input copy as the other modes;
    // merge, link + offsets + encode, and the copy-out summed over the groups
    {
      static const int pairs[2][2] = {{0, 1}, {1, 2}};
      float ms = 0;
      for (int i = 0; i < 2; ++i)
        if (cudaEventElapsedTime(&ms, sev[pairs[i][0]], sev[pairs[i][1]]) == cudaSuccess) stat->stage_ms[i] = ms;
      float dec = 0;
      for (int i = 0; i < n; ++i)
        if (cudaEventElapsedTime(&ms, cl.tev[2 + 2 * i], cl.tev[3 + 2 * i]) == cudaSuccess) dec += ms;
      stat->stage_ms[0] = dec;
      if (cudaEventElapsedTime(&ms, cl.tev[0], cl.tev[1]) == cudaSuccess) stat->stage_ms[5] = ms;
      double mg = 0, en = 0, cp = 0;
      for (uint32_t g = 0; g < NG; ++g) {
        if (cudaEventElapsedTime(&ms, ge[7 * g], ge[7 * g + 1]) == cudaSuccess) mg += ms;
        if (cudaEventElapsedTime(&ms, ge[7 * g + 1], ge[7 * g + 2]) == cudaSuccess) en += ms;
        if (cudaEventElapsedTime(&ms, ge[7 * g + 3], ge[7 * g + 4]) == cudaSuccess) en += ms;
        if (cudaEventElapsedTime(&ms, ge[7 * g + 5], ge[7 * g + 6]) == cudaSuccess) cp += ms;
      }
      stat->stage_ms[2] = mg;
      stat->stage_ms[3] = en;
      stat->stage_ms[4] = cp;
    }
    stat->d2h_bytes += total_out;
    stat->rows = out_rows;
    stat->payload_bytes = total_out;
    stat->tiles = ntiles;
    stat->kernel_launches = launches;
    uint64_t tmax = 0, tsum = 0, tne = 0;
    for (auto& m : mts)
      if (m.rows_in) {
        tmax = std::max<uint64_t>(tmax, m.rows_in);
        tsum += m.rows_in;
        tne++;
      }
    stat->tile_imbalance = tne ? (double)tmax / ((double)tsum / tne) : 0.0;
    if (!emit) return KITE_OK;
    for (uint32_t g = 0; g < NG; ++g)
      for (uint32_t p = pb[g]; p < pb[g + 1]; ++p) {
        const BucketMeta& m = hm[p];
        if (!m.rows) continue;
        kite_chunk_meta cm{};
        cm.partition_id = p;
        cm.codec = KITE_CODEC_DVLE;
        cm.row_count = m.rows;
        cm.raw_bytes = m.bytes;
        cm.key_min_lo[0] = m.kmin_lo;
        cm.key_min_lo[1] = m.kmin_hi;
        cm.key_max_lo[0] = m.kmax_lo;
        cm.key_max_lo[1] = m.kmax_hi;
        if (emit(user, &cm, hout + gbase[g] + m.byte_off, (size_t)m.bytes))
          return fail(KITE_ERR_CALLBACK, "emit callback aborted");
      }
    return KITE_OK;
  }
  MCU(cudaEventRecord(sev[2], s));
  if (ntiles) {
    kmerge<<<ntiles, kMergeThreads, smem, s>>>(d_keys.as<T>(), d_counts.as<unsigned long long>(),
                                               d_mt.as<MergeTile>(), d_ts.as<TileStream>(), d_filt.as<InputFilter>(),
                                               d_okeys.as<T>(), d_ocounts.as<uint32_t>(), d_tout.as<TileOut<T>>(),
                                               d_over.as<unsigned long long>(), dst, aux);
    launches++;
  }
  MCU(cudaEventRecord(sev[3], s));
  DevStatus hst{};
  unsigned long long over = 0;
  std::vector<TileOut<T>> htout(ntiles);
  MCU(cudaMemcpyAsync(&hst, dst, sizeof hst, cudaMemcpyDeviceToHost, s));
  MCU(cudaMemcpyAsync(&over, d_over.p, 8, cudaMemcpyDeviceToHost, s));
  if (ntiles) MCU(cudaMemcpyAsync(htout.data(), d_tout.p, ntiles * sizeof(TileOut<T>), cudaMemcpyDeviceToHost, s));
  if (sync()) return fail(KITE_ERR_TIMEOUT, "merge wait");
  cudaFreeAsync(dst, s);
  if (hst.code) {
    char b[160];
    snprintf(b, sizeof b, "%s: device status %u (%u, %u, %u)", dump ? "dump" : "merge", hst.code, hst.a, hst.b,
             hst.c);
    return fail(hst.code == KITE_DEV_BAD_INPUT ? KITE_ERR_BAD_INPUT : KITE_ERR_DEVICE, b);
  }
  auto stage_times = [&]() {
    static const int pairs[5][2] = {{0, 1}, {1, 2}, {2, 3}, {4, 5}, {5, 6}};
    float ms = 0;
    for (int i = 0; i < 5; ++i)
      if (cudaEventElapsedTime(&ms, sev[pairs[i][0]], sev[pairs[i][1]]) == cudaSuccess) stat->stage_ms[i] = ms;
    // [0] the decode kernels alone (the wait for each input's bytes left
    // out), [5] the copies of the inputs in, which the decode overlaps
    float dec = 0;
    for (int i = 0; i < n; ++i)
      if (cudaEventElapsedTime(&ms, cl.tev[2 + 2 * i], cl.tev[3 + 2 * i]) == cudaSuccess) dec += ms;
    stat->stage_ms[0] = dec;
    if (cudaEventElapsedTime(&ms, cl.tev[0], cl.tev[1]) == cudaSuccess) stat->stage_ms[5] = ms;
  };
  stat->tiles = ntiles;
  if (mode == kModeHisto) {
    // ---- count -> frequency: the small bins, then the listed large counts ----
    std::vector<unsigned long long> hb(kHistBins + 1);
    MCU(cudaMemcpyAsync(hb.data(), d_hist.p, (kHistBins + 1) * 8, cudaMemcpyDeviceToHost, s));
    if (sync()) return fail(KITE_ERR_TIMEOUT, "histo wait");
    const unsigned long long ns = std::min<unsigned long long>(hb[kHistBins], out_off);
    std::vector<unsigned long long> big(ns);
    MCU(cudaEventRecord(sev[4], s));
    if (ns) MCU(cudaMemcpyAsync(big.data(), d_spill.p, ns * 8, cudaMemcpyDeviceToHost, s));
    MCU(cudaEventRecord(sev[5], s));
    MCU(cudaEventRecord(sev[6], s));
    if (sync()) return fail(KITE_ERR_TIMEOUT, "histo wait");
    stage_times();
    std::sort(big.begin(), big.end());
    uint64_t keys_out = 0;
    for (uint32_t b = 0; b < kHistBins; ++b) keys_out += hb[b];
    stat->rows = keys_out + ns;
    stat->kernel_launches = launches;
    if (!ex || !ex->histo) return KITE_OK;
    for (uint32_t b = 0; b < kHistBins; ++b)
      if (hb[b] && ex->histo(ex->user, b, hb[b])) return fail(KITE_ERR_CALLBACK, "histo callback aborted");
    for (size_t i = 0; i < big.size();) {
      size_t j = i;
      while (j < big.size() && big[j] == big[i]) ++j;
      if (ex->histo(ex->user, big[i], j - i)) return fail(KITE_ERR_CALLBACK, "histo callback aborted");
      i = j;
    }
    return KITE_OK;
  }
  if (mode == kModeRows) {
    // ---- query lookups over the non-empty tiles of each partition ----
    std::vector<uint32_t> qtf(P + 1, 0), qrows;
    std::vector<T> qkey0;
    std::vector<unsigned long long> qoff;
    for (uint32_t p = 0; p < P; ++p) {
      qtf[p] = (uint32_t)qrows.size();
      for (uint32_t t = tile_first[p]; t < tile_first[p + 1]; ++t)
        if (htout[t].rows) {
          qkey0.push_back(htout[t].first_key);
          qoff.push_back(mts[t].out_off);
          qrows.push_back(htout[t].rows);
        }
    }
    qtf[P] = (uint32_t)qrows.size();
    const uint32_t nq = (uint32_t)ex->nq, nt = (uint32_t)qrows.size();
    std::vector<T> qk(nq);
    std::vector<uint32_t> qp(nq);
    for (uint32_t q = 0; q < nq; ++q) {
      qk[q] = (T)(((unsigned __int128)ex->keys[2 * q + 1] << 64) | ex->keys[2 * q]);
      qp[q] = ex->parts[q];
    }
    Dev d_qtf, d_qk0, d_qoff, d_qrows, d_qk, d_qp, d_qout;
    if (!d_qtf.ensure((P + 1) * 4) || !d_qk0.ensure(nt * sizeof(T) + 16) || !d_qoff.ensure(nt * 8 + 8) ||
        !d_qrows.ensure(nt * 4 + 8) || !d_qk.ensure(nq * sizeof(T) + 16) || !d_qp.ensure(nq * 4 + 8) ||
        !d_qout.ensure(nq * 8 + 8))
      return fail(KITE_ERR_OOM, "query buffers");
    MCU(cudaMemcpyAsync(d_qtf.p, qtf.data(), (P + 1) * 4, cudaMemcpyHostToDevice, s));
    if (nt) {
      MCU(cudaMemcpyAsync(d_qk0.p, qkey0.data(), nt * sizeof(T), cudaMemcpyHostToDevice, s));
      MCU(cudaMemcpyAsync(d_qoff.p, qoff.data(), nt * 8, cudaMemcpyHostToDevice, s));
      MCU(cudaMemcpyAsync(d_qrows.p, qrows.data(), nt * 4, cudaMemcpyHostToDevice, s));
    }
    MCU(cudaEventRecord(sev[4], s));
    if (nq) {
      MCU(cudaMemcpyAsync(d_qk.p, qk.data(), nq * sizeof(T), cudaMemcpyHostToDevice, s));
      MCU(cudaMemcpyAsync(d_qp.p, qp.data(), nq * 4, cudaMemcpyHostToDevice, s));
      k_query_rows<T><<<(nq + 255) / 256, 256, 0, s>>>(d_okeys.as<T>(), d_c64.as<unsigned long long>(),
                                                       d_qtf.as<uint32_t>(), d_qk0.as<T>(),
                                                       d_qoff.as<unsigned long long>(), d_qrows.as<uint32_t>(),
                                                       d_qk.as<T>(), d_qp.as<uint32_t>(), nq,
                                                       d_qout.as<unsigned long long>());
      launches++;
    }
    MCU(cudaEventRecord(sev[5], s));
    if (nq) MCU(cudaMemcpyAsync(ex->counts_out, d_qout.p, nq * 8, cudaMemcpyDeviceToHost, s));
    MCU(cudaEventRecord(sev[6], s));
    if (sync()) return fail(KITE_ERR_TIMEOUT, "query wait");
    MCU(cudaGetLastError());
    stage_times();
    stat->kernel_launches = launches;
    return KITE_OK;
  }
  if (dump) {
    // ---- TSV: tile byte offsets in (partition, key) order, then formatting ----
    std::vector<unsigned long long> tboff(ntiles + 1);
    std::vector<uint64_t> prow(P, 0), pbytes(P, 0);
    unsigned long long acc = 0;
    uint64_t out_rows = 0;
    for (uint32_t t = 0; t < ntiles; ++t) {
      tboff[t] = acc;
      acc += htout[t].rest_bytes;
      prow[mts[t].partition] += htout[t].rows;
      pbytes[mts[t].partition] += htout[t].rest_bytes;
      out_rows += htout[t].rows;
    }
    tboff[ntiles] = acc;
    if (!d_boff.ensure((ntiles + 1) * 8) || !d_out.ensure(acc + 16)) return fail(KITE_ERR_OOM, "dump output");
    if (ntiles && acc) MCU(cudaMemcpyAsync(d_boff.p, tboff.data(), (ntiles + 1) * 8, cudaMemcpyHostToDevice, s));
    MCU(cudaEventRecord(sev[4], s));
    if (ntiles && acc) {
      const size_t tsm = 256 + (size_t)kTsvThreads * (key_bits / 2 + 12);
      k_tsv_tiles<T><<<ntiles, kTsvThreads, tsm, s>>>(d_okeys.as<T>(), d_ocounts.as<uint32_t>(), d_mt.as<MergeTile>(),
                                                      d_tout.as<TileOut<T>>(), d_boff.as<unsigned long long>(),
                                                      key_bits / 2, d_out.as<uint8_t>());
      launches++;
    }
    MCU(cudaEventRecord(sev[5], s));
    stat->d2h_bytes += emit ? acc : 0;
    stat->rows = out_rows;
    stat->payload_bytes = acc;
    stat->tiles = ntiles;
    stat->kernel_launches = launches;
    if (!emit || acc == 0) {
      MCU(cudaEventRecord(sev[6], s));
      if (sync()) return fail(KITE_ERR_TIMEOUT, "dump wait");
      MCU(cudaGetLastError());
      stage_times();
      return KITE_OK;
    }
    // ---- copy-out in groups of whole partitions through two pinned halves:
    // group i+2 is queued once group i has been emitted, so the copy of the
    // next group overlaps the callback's work on this one
    uint64_t maxpart = 0;
    for (uint32_t p = 0; p < P; ++p) maxpart = std::max(maxpart, pbytes[p]);
    const uint64_t half = std::max<uint64_t>(std::min<uint64_t>(acc, 256ull << 20), maxpart);
    std::vector<uint32_t> gfirst{0};  // first partition of every group
    std::vector<uint64_t> goff{0};
    {
      uint64_t g = 0, off = 0;
      for (uint32_t p = 0; p < P; ++p) {
        if (g + pbytes[p] > half) {
          gfirst.push_back(p);
          goff.push_back(off);
          g = 0;
        }
        g += pbytes[p];
        off += pbytes[p];
      }
      gfirst.push_back(P);
      goff.push_back(off);
    }
    const uint32_t ngroups = (uint32_t)gfirst.size() - 1;
    uint8_t* stage = staging ? staging(ngroups > 1 ? 2 * half : half) : nullptr;
    std::unique_ptr<uint8_t[]> fallback;
    if (!stage) {
      // no pinned staging offered: one pageable buffer for everything
      fallback.reset(new (std::nothrow) uint8_t[acc]);
      if (!fallback) return fail(KITE_ERR_OOM, "dump host buffer");
    }
    auto group_dst = [&](uint32_t g) { return stage ? stage + (g & 1) * half : fallback.get() + goff[g]; };
    cudaEvent_t cev[2];
    for (auto& e : cev)
      if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return fail(KITE_ERR_CUDA, "event");
    struct CevGuard {
      cudaEvent_t* e;
      ~CevGuard() {
        cudaEventDestroy(e[0]);
        cudaEventDestroy(e[1]);
      }
    } cev_guard{cev};
    auto queue_copy = [&](uint32_t g) -> cudaError_t {
      const uint64_t n = goff[g + 1] - goff[g];
      cudaError_t e = n ? cudaMemcpyAsync(group_dst(g), d_out.as<uint8_t>() + goff[g], n, cudaMemcpyDeviceToHost, s)
                        : cudaSuccess;
      if (e == cudaSuccess) e = cudaEventRecord(cev[g & 1], s);
      return e;
    };
    MCU(queue_copy(0));
    if (ngroups > 1) MCU(queue_copy(1));
    for (uint32_t g = 0; g < ngroups; ++g) {
      const int w = bounded_event_wait(cev[g & 1], timeout_ms);
      if (w) return fail(w == -3 ? KITE_ERR_TIMEOUT : KITE_ERR_CUDA, "dump copy wait");
      const uint8_t* src = group_dst(g);
      uint64_t off = 0;
      for (uint32_t p = gfirst[g]; p < gfirst[g + 1]; ++p) {
        if (!prow[p]) continue;
        // key range of the partition's lines: first row of its first non-empty
        // tile, last row of its last one
        kite_chunk_meta cm{};
        cm.partition_id = p;
        cm.codec = 0;
        cm.row_count = prow[p];
        cm.raw_bytes = pbytes[p];
        bool first = true;
        for (uint32_t t = tile_first[p]; t < tile_first[p + 1]; ++t) {
          if (!htout[t].rows) continue;
          const unsigned __int128 a = (unsigned __int128)htout[t].first_key, b = (unsigned __int128)htout[t].last_key;
          if (first) {
            cm.key_min_lo[0] = (uint64_t)a;
            cm.key_min_lo[1] = (uint64_t)(a >> 64);
            first = false;
          }
          cm.key_max_lo[0] = (uint64_t)b;
          cm.key_max_lo[1] = (uint64_t)(b >> 64);
        }
        if (emit(user, &cm, src + off, (size_t)pbytes[p])) return fail(KITE_ERR_CALLBACK, "emit callback aborted");
        off += pbytes[p];
      }
      if (g + 2 < ngroups) MCU(queue_copy(g + 2));
    }
    MCU(cudaEventRecord(sev[6], s));
    if (sync()) return fail(KITE_ERR_TIMEOUT, "dump wait");
    MCU(cudaGetLastError());
    stage_times();
    return KITE_OK;
  }
  if (over != ~0ull) {
    // first overflowing row in (partition, key) order: name its key like the reference
    const uint32_t t = (uint32_t)(over >> 32), r = (uint32_t)(over & 0xffffffffu);
    T key{};
    MCU(cudaMemcpyAsync(&key, d_okeys.as<T>() + mts[t].out_off + r, sizeof(T), cudaMemcpyDeviceToHost, s));
    if (sync()) return fail(KITE_ERR_TIMEOUT, "merge wait");
    unsigned __int128 v = (unsigned __int128)key;
    std::string ks;
    if (v == 0) ks = "0";
    while (v) {
      ks.insert(ks.begin(), (char)('0' + (int)(v % 10)));
      v /= 10;
    }
    return fail(KITE_ERR_COUNT_OVERFLOW, "merged count exceeds u32 for key " + ks);
  }
  // ---- encode: per partition, tiles in key order ----
  for (uint32_t t = 0; t < ntiles; ++t) tds[t].len = htout[t].rows;
  if (ntiles) MCU(cudaMemcpyAsync(d_tds.p, tds.data(), ntiles * sizeof(TileDesc), cudaMemcpyHostToDevice, s));
  MCU(cudaMemcpyAsync(d_tf.p, tile_first.data(), (P + 1) * 4, cudaMemcpyHostToDevice, s));
  launch_tile_link_ranges<T>(d_tout.as<TileOut<T>>(), P, d_tf.as<uint32_t>(), d_boff.as<unsigned long long>(),
                             d_prev.as<T>(), d_meta.as<BucketMeta>(), s);
  launch_bucket_offsets(d_meta.as<BucketMeta>(), P, nullptr, s);
  launches += 2;
  std::vector<BucketMeta> meta(P);
  MCU(cudaMemcpyAsync(meta.data(), d_meta.p, P * sizeof(BucketMeta), cudaMemcpyDeviceToHost, s));
  if (sync()) return fail(KITE_ERR_TIMEOUT, "merge wait");
  uint64_t out_bytes = 0, out_rows = 0;
  for (auto& m : meta) {
    out_bytes += m.bytes;
    out_rows += m.rows;
  }
  if (!d_out.ensure(out_bytes + 16)) return fail(KITE_ERR_OOM, "merge output");
  DevStatus* est = nullptr;
  MCU(cudaMallocAsync(&est, sizeof(DevStatus), s));
  MCU(cudaMemsetAsync(est, 0, sizeof(DevStatus), s));
  MCU(cudaEventRecord(sev[4], s));
  launch_encode<T>(d_okeys.as<T>(), d_ocounts.as<uint32_t>(), d_tds.as<TileDesc>(), d_tout.as<TileOut<T>>(),
                   d_boff.as<unsigned long long>(), d_prev.as<T>(), d_meta.as<BucketMeta>(), ntiles,
                   d_out.as<uint8_t>(), out_bytes, est, s);
  launches++;
  MCU(cudaEventRecord(sev[5], s));
  // the output to the host: through the caller's pinned staging when given
  // (a copy at full link speed), else into ordinary host memory
  uint8_t* hout = staging ? staging(out_bytes + 16) : nullptr;
  std::unique_ptr<uint8_t[]> hown;
  if (!hout) {
    hown.reset(new (std::nothrow) uint8_t[out_bytes + 16]);
    if (!hown) return fail(KITE_ERR_OOM, "merge output host buffer");
    hout = hown.get();
  }
  if (out_bytes) MCU(cudaMemcpyAsync(hout, d_out.p, out_bytes, cudaMemcpyDeviceToHost, s));
  MCU(cudaEventRecord(sev[6], s));
  MCU(cudaMemcpyAsync(&hst, est, sizeof hst, cudaMemcpyDeviceToHost, s));
  if (sync()) return fail(KITE_ERR_TIMEOUT, "merge wait");
  stage_times();
  cudaFreeAsync(est, s);
  if (hst.code) return fail(KITE_ERR_DEVICE, "merge encode failed");
  stat->d2h_bytes += out_bytes;
  stat->rows = out_rows;
  stat->payload_bytes = out_bytes;
  stat->tiles = ntiles;
  stat->kernel_launches = launches;
  uint64_t tmax = 0, tsum = 0, tne = 0;
  for (auto& m : mts)
    if (m.rows_in) {
      tmax = std::max<uint64_t>(tmax, m.rows_in);
      tsum += m.rows_in;
      tne++;
    }
  stat->tile_imbalance = tne ? (double)tmax / ((double)tsum / tne) : 0.0;
  if (!emit) return KITE_OK;
  for (uint32_t p = 0; p < P; ++p) {
    const BucketMeta& m = meta[p];
    if (!m.rows) continue;
    kite_chunk_meta cm{};
    cm.partition_id = p;
    cm.codec = KITE_CODEC_DVLE;
    cm.row_count = m.rows;
    cm.raw_bytes = m.bytes;
    cm.key_min_lo[0] = m.kmin_lo;
    cm.key_min_lo[1] = m.kmin_hi;
    cm.key_max_lo[0] = m.kmax_lo;
    cm.key_max_lo[1] = m.kmax_hi;
    if (emit(user, &cm, hout + m.byte_off, (size_t)m.bytes)) return fail(KITE_ERR_CALLBACK, "emit callback aborted");
  }
  return KITE_OK;
#undef MCU
}

}  // namespace

int merge_run(int k, uint32_t partitions, const kite_gpu_merge_input* inputs, int n, cudaStream_t s,
              uint32_t timeout_ms, int mode, kite_gpu_emit_fn emit, void* user, std::string* msg,
              kite_gpu_stats* st, const StagingFn& staging, const MergeExtra* ex) {
  if (k <= 31)
    return merge_typed<uint64_t>(partitions, 2 * k, inputs, n, s, timeout_ms, mode, emit, user, msg, st, staging,
                                 ex);
  return merge_typed<u128>(partitions, 2 * k, inputs, n, s, timeout_ms, mode, emit, user, msg, st, staging, ex);
}

}  // namespace kite
