// kite_gpu_count_rows_noalloc: exact k-mer counting of one small FASTQ chunk
// that allocates nothing.
//
// Some callers cannot allocate device memory when they want a count: a
// process whose framework has already reserved the device's memory for its
// own caching pool, or a loop that counts small read batches between other
// GPU work and cannot accept the device-wide synchronisation that cudaMalloc
// and cudaFree imply, nor an out-of-memory failure half way through a run.
// The context API (kite_gpu_open) grows its buffers on demand with cudaMalloc;
// this entry point works only in g_noalloc_scratch below, a fixed array in
// this file's device data, and writes its results into buffers the caller
// already owns.
//
// Limits and sharing:
//  * at most KITE_NOALLOC_MAX_BYTES (512 KiB) of FASTQ per call; a larger
//    chunk is rejected with KITE_ERR_UNSUPPORTED before any launch.
//  * the array (kScratchBytes, about 21 MiB) exists once per device in the
//    process.  Every call on a device uses the same array, so calls that
//    overlap on the GPU (two host threads, or two streams without ordering
//    between them) race and corrupt each other's results: serialise them.
//  * the first call on a device looks the array's address up with
//    cudaGetSymbolAddress (which also loads this module on that device); make
//    that first call before any stream capture begins.  The address is kept
//    with the id of the device's context and looked up again when a new
//    context replaces it (after cudaDeviceReset, for example).
//  * the call returns once the work has finished, waiting at most timeout_ms.
//
// The kernels are a small-input variant of the context path: one pass finds
// the sequence lines, one rolls the k-mers (KmerIter::next,
// src/count/kmer.rs:241-267 and :311-337), the keys are grouped by their
// Fibonacci-hash partition (src/count/kmer.rs:67-71, :111-116), and one CTA
// per partition sorts its keys through global memory and reduces them to
// (key, count) rows, as the reference's flush_bucket does per bucket
// (src/count/worker.rs:296-449).
#include <algorithm>
#include <chrono>
#include <cstring>
#include <mutex>
#include <thread>
#include <tuple>
#include <utility>

#include "kite_gpu.h"
#include "kite_internal.h"

namespace kite {
namespace na {

constexpr uint32_t kMaxBytes = KITE_NOALLOC_MAX_BYTES;
constexpr uint32_t kMaxSeq = kMaxBytes / 4 + 2;  // a record spans at least four newlines
constexpr uint32_t kMaxParts = 65536;
constexpr uint32_t kPiece = 256;  // bases per extraction piece
constexpr int kMaxDevices = 64;
constexpr int kSortThreads = 512;

struct Counters {
  unsigned long long reads, bases, kmers;
  unsigned int nseq, npieces, nkeys, nrows;
  unsigned int status, pad;
};

constexpr size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }
constexpr size_t kOffKeysA = 0;
constexpr size_t kOffKeysB = align256(kOffKeysA + (size_t)kMaxBytes * 16);
constexpr size_t kOffCounts = align256(kOffKeysB + (size_t)kMaxBytes * 16);
constexpr size_t kOffSeqStart = align256(kOffCounts + (size_t)kMaxBytes * 4);
constexpr size_t kOffSeqEnd = align256(kOffSeqStart + (size_t)kMaxSeq * 4);
constexpr size_t kOffPieceOff = align256(kOffSeqEnd + (size_t)kMaxSeq * 4);
constexpr size_t kOffBucketCount = align256(kOffPieceOff + (size_t)(kMaxSeq + 1) * 4);
constexpr size_t kOffBucketFill = align256(kOffBucketCount + (size_t)kMaxParts * 4);
constexpr size_t kOffBucketOff = align256(kOffBucketFill + (size_t)kMaxParts * 4);
constexpr size_t kOffBucketRows = align256(kOffBucketOff + (size_t)(kMaxParts + 1) * 4);
constexpr size_t kOffRowOff = align256(kOffBucketRows + (size_t)kMaxParts * 4);
constexpr size_t kOffCounters = align256(kOffRowOff + (size_t)(kMaxParts + 1) * 4);
constexpr size_t kScratchBytes = align256(kOffCounters + sizeof(Counters));

// Typed views of the scratch array.
struct View {
  uint8_t* s;
  template <class T> __device__ T* keys_a() const { return reinterpret_cast<T*>(s + kOffKeysA); }
  template <class T> __device__ T* keys_b() const { return reinterpret_cast<T*>(s + kOffKeysB); }
  __device__ uint32_t* counts() const { return reinterpret_cast<uint32_t*>(s + kOffCounts); }
  __device__ uint32_t* seq_start() const { return reinterpret_cast<uint32_t*>(s + kOffSeqStart); }
  __device__ uint32_t* seq_end() const { return reinterpret_cast<uint32_t*>(s + kOffSeqEnd); }
  __device__ uint32_t* piece_off() const { return reinterpret_cast<uint32_t*>(s + kOffPieceOff); }
  __device__ uint32_t* bucket_count() const { return reinterpret_cast<uint32_t*>(s + kOffBucketCount); }
  __device__ uint32_t* bucket_fill() const { return reinterpret_cast<uint32_t*>(s + kOffBucketFill); }
  __device__ uint32_t* bucket_off() const { return reinterpret_cast<uint32_t*>(s + kOffBucketOff); }
  __device__ uint32_t* bucket_rows() const { return reinterpret_cast<uint32_t*>(s + kOffBucketRows); }
  __device__ uint32_t* row_off() const { return reinterpret_cast<uint32_t*>(s + kOffRowOff); }
  __device__ Counters* counters() const { return reinterpret_cast<Counters*>(s + kOffCounters); }
};

}  // namespace na
}  // namespace kite

// The only working memory of kite_gpu_count_rows_noalloc (one per device).
static __device__ __align__(256) unsigned char g_noalloc_scratch[kite::na::kScratchBytes];

namespace kite {
namespace na {
namespace {

// A/a=0, C/c=1, G/g=2, T/t=3, anything else 4 (src/count/kmer.rs:2-13).
__device__ __forceinline__ uint32_t base_code(uint8_t c) {
  switch (c) {
    case 'A': case 'a': return 0;
    case 'C': case 'c': return 1;
    case 'G': case 'g': return 2;
    case 'T': case 't': return 3;
    default: return 4;
  }
}

// Sequence lines of the chunk (parse_sequences, src/count/parser.rs:19-65):
// line 4r+1 of the chunk is sequence r; a final sequence line without its
// newline runs to the end; a chunk that does not start with '@' yields
// nothing (the worker ignores the parse error, src/count/worker.rs:217).
// Also the piece offsets of every sequence, and the reads / bases totals.
// One CTA.
__global__ void __launch_bounds__(1024) k_lines(const uint8_t* __restrict__ d, uint32_t len, uint8_t* scr) {
  constexpr uint32_t kPer = 16, kWin = 1024 * kPer;
  __shared__ unsigned sm[40];
  __shared__ unsigned long long sm64[40];
  const View v{scr};
  Counters* c = v.counters();
  uint32_t* ss = v.seq_start();
  uint32_t* se = v.seq_end();
  uint32_t* po = v.piece_off();
  if (len == 0 || d[0] != '@') {
    if (threadIdx.x == 0) {
      c->nseq = 0;
      c->npieces = 0;
      po[0] = 0;
    }
    return;
  }
  unsigned carry = 0;  // newlines before the current window
  for (uint32_t w0 = 0; w0 < len; w0 += kWin) {
    const uint32_t b = w0 + threadIdx.x * kPer;
    const uint32_t e = min(b + kPer, len);
    unsigned cnt = 0;
    for (uint32_t i = b; i < e; ++i) cnt += d[i] == '\n';
    unsigned tot;
    unsigned line = carry + block_exclusive_scan<1024, unsigned>(cnt, sm, &tot);
    for (uint32_t i = b; i < e; ++i) {
      if (d[i] != '\n') continue;
      if ((line & 3u) == 0) ss[line >> 2] = i + 1;  // header ends: sequence starts
      else if ((line & 3u) == 1) se[line >> 2] = i;
      ++line;
    }
    carry += tot;
  }
  const unsigned nl = carry;
  const unsigned nseq = nl ? (nl + 3) / 4 : 0;
  if (threadIdx.x == 0 && (nl & 3u) == 1) se[nl >> 2] = len;
  __syncthreads();
  unsigned pcarry = 0;
  unsigned long long reads = 0, bases = 0;
  for (uint32_t s0 = 0; s0 < nseq; s0 += 1024) {
    const uint32_t s = s0 + threadIdx.x;
    unsigned pieces = 0;
    if (s < nseq) {
      const uint32_t L = se[s] - ss[s];
      pieces = (L + kPiece - 1) / kPiece;
      reads += L > 0;
      bases += L;
    }
    unsigned tot;
    const unsigned ex = block_exclusive_scan<1024, unsigned>(pieces, sm, &tot);
    if (s < nseq) po[s] = pcarry + ex;
    pcarry += tot;
  }
  unsigned long long rt, bt;
  block_exclusive_scan<1024, unsigned long long>(reads, sm64, &rt);
  block_exclusive_scan<1024, unsigned long long>(bases, sm64, &bt);
  if (threadIdx.x == 0) {
    po[nseq] = pcarry;
    c->nseq = nseq;
    c->npieces = pcarry;
    c->reads = rt;
    c->bases = bt;
  }
}

// Rolling k-mers, one piece of up to kPiece bases per thread: the piece
// emits the k-mers that END inside it and starts rolling k-1 bases earlier
// (clamped to the sequence start), so every k-mer is emitted exactly once.
// A first pass counts, one atomic reserves the slots, a second pass writes
// the keys and the partition histogram.
template <class T>
__global__ void __launch_bounds__(256) k_extract(const uint8_t* __restrict__ d, uint32_t k, uint32_t canonical,
                                                 uint32_t shift, uint8_t* scr) {
  const View v{scr};
  Counters* c = v.counters();
  const uint32_t npieces = c->npieces, nseq = c->nseq;
  const uint32_t* ss = v.seq_start();
  const uint32_t* se = v.seq_end();
  const uint32_t* po = v.piece_off();
  T* keys = v.keys_a<T>();
  uint32_t* bcount = v.bucket_count();
  const T mask = (2 * k == (uint32_t)KeyTraits<T>::kBits) ? ~T(0) : ((T(1) << (2 * k)) - T(1));
  const uint32_t rshift = 2 * (k - 1);
  unsigned long long kmers = 0;
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < npieces; q += gridDim.x * blockDim.x) {
    uint32_t lo = 0, hi = nseq - 1;  // last sequence with po[s] <= q
    while (lo < hi) {
      const uint32_t mid = (lo + hi + 1) >> 1;
      if (po[mid] <= q) lo = mid;
      else hi = mid - 1;
    }
    const uint32_t s0 = ss[lo];
    const uint32_t ps = s0 + (q - po[lo]) * kPiece;
    const uint32_t pe = min(ps + kPiece, se[lo]);
    const uint32_t r0 = (ps - s0 >= k - 1) ? ps - (k - 1) : s0;
    uint32_t n = 0, valid = 0;
    for (uint32_t i = r0; i < pe; ++i) {
      if (base_code(d[i]) > 3) {
        valid = 0;
        continue;
      }
      ++valid;
      n += (valid >= k && i >= ps);
    }
    if (n == 0) continue;
    const uint32_t at = atomicAdd(&c->nkeys, n);
    if (at + n > kMaxBytes) {
      atomicCAS(&c->status, 0u, 1u);
      continue;
    }
    T fwd = 0, rev = 0;
    valid = 0;
    uint32_t o = at;
    for (uint32_t i = r0; i < pe; ++i) {
      const uint32_t b = base_code(d[i]);
      if (b > 3) {
        fwd = 0;
        rev = 0;
        valid = 0;
        continue;
      }
      fwd = ((fwd << 2) | T(b)) & mask;
      rev = (rev >> 2) | (T(b ^ 3u) << rshift);
      ++valid;
      if (valid >= k && i >= ps) {
        const T key = canonical ? (fwd < rev ? fwd : rev) : fwd;
        keys[o++] = key;
        atomicAdd(&bcount[bucket_of(key, shift)], 1u);
      }
    }
    kmers += n;
  }
  for (int m = 16; m; m >>= 1) kmers += __shfl_xor_sync(0xffffffffu, kmers, m);
  if ((threadIdx.x & 31) == 0 && kmers) atomicAdd(&c->kmers, kmers);
}

// Exclusive scan of n counters into out[0..n], out[n] = total.  One CTA.
__global__ void __launch_bounds__(1024) k_scan(const uint32_t* __restrict__ in, uint32_t n,
                                               uint32_t* __restrict__ out) {
  __shared__ unsigned sm[40];
  unsigned carry = 0;
  for (uint32_t i0 = 0; i0 < n; i0 += 1024) {
    const uint32_t i = i0 + threadIdx.x;
    const unsigned x = i < n ? in[i] : 0u;
    unsigned tot;
    const unsigned ex = block_exclusive_scan<1024, unsigned>(x, sm, &tot);
    if (i < n) out[i] = carry + ex;
    carry += tot;
  }
  if (threadIdx.x == 0) out[n] = carry;
}

// Keys grouped by partition: keys_a -> keys_b at the partition offsets.
template <class T>
__global__ void __launch_bounds__(256) k_scatter(uint32_t shift, uint8_t* scr) {
  const View v{scr};
  const uint32_t n = min(v.counters()->nkeys, kMaxBytes);
  const T* a = v.keys_a<T>();
  T* b = v.keys_b<T>();
  const uint32_t* off = v.bucket_off();
  uint32_t* fill = v.bucket_fill();
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const T key = a[i];
    const uint32_t bk = bucket_of(key, shift);
    const uint32_t pos = off[bk] + atomicAdd(&fill[bk], 1u);
    if (pos < kMaxBytes) b[pos] = key;
  }
}

// One CTA per partition: LSD radix sort of its keys through global memory
// (8-bit digits over the bits that vary, each chunk of CAP keys ranked stably
// on chip), then the run-length reduction to (key, count) rows written to
// keys_a / counts at the partition's offset, and the partition's row count.
template <class T>
__global__ void __launch_bounds__(kSortThreads) k_sort_rle(uint8_t* scr) {
  constexpr int NT = kSortThreads, ITEMS = tile_items<T>(), CAP = NT * ITEMS, NW = NT / 32;
  __shared__ unsigned warp_hist[256 * NW];
  __shared__ unsigned scan_sm[40];
  __shared__ unsigned dtot[256], dstart[256];
  __shared__ unsigned long long run_off[256];
  __shared__ T red_mn[NW], red_mx[NW];
  const View v{scr};
  const uint32_t bk = blockIdx.x;
  const uint32_t n = v.bucket_count()[bk];
  if (n == 0) {
    if (threadIdx.x == 0) v.bucket_rows()[bk] = 0;
    return;
  }
  const uint32_t off = v.bucket_off()[bk];
  T* src = v.keys_b<T>() + off;
  T* dst = v.keys_a<T>() + off;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;

  T mn = ~T(0), mx = T(0);
  for (uint32_t i = threadIdx.x; i < n; i += NT) {
    const T x = src[i];
    mn = x < mn ? x : mn;
    mx = x > mx ? x : mx;
  }
  for (int m = 16; m; m >>= 1) {
    const T a = shfl_xor_key(mn, m), b = shfl_xor_key(mx, m);
    mn = a < mn ? a : mn;
    mx = b > mx ? b : mx;
  }
  if (lane == 0) {
    red_mn[wid] = mn;
    red_mx[wid] = mx;
  }
  __syncthreads();
  mn = red_mn[0];
  mx = red_mx[0];
  for (int w = 1; w < NW; ++w) {
    mn = red_mn[w] < mn ? red_mn[w] : mn;
    mx = red_mx[w] > mx ? red_mx[w] : mx;
  }
  const int nbits = mn == mx ? 0 : KeyTraits<T>::kBits - clz_key(T(mn ^ mx));
  const unsigned pos0 = (unsigned)wid * 32u * ITEMS + lane;
  for (int sh = 0; sh < nbits; sh += 8) {
    for (int d = threadIdx.x; d < 256; d += NT) dtot[d] = 0;
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < n; i += NT) atomicAdd(&dtot[digit_of(src[i], sh)], 1u);
    __syncthreads();
    if (threadIdx.x == 0) {
      unsigned long long acc = 0;
      for (int d = 0; d < 256; ++d) {
        run_off[d] = acc;
        acc += dtot[d];
      }
    }
    __syncthreads();
    for (uint32_t c0 = 0; c0 < n; c0 += CAP) {
      const uint32_t cn = min(n - c0, (uint32_t)CAP);
      T key[ITEMS];
      unsigned dig[ITEMS], dest[ITEMS];
      bool valid[ITEMS];
#pragma unroll
      for (int r = 0; r < ITEMS; ++r) {
        const unsigned pos = pos0 + r * 32u;
        valid[r] = pos < cn;
        key[r] = valid[r] ? src[c0 + pos] : T(0);
        dig[r] = digit_of(key[r], sh);
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
  // Run-length reduction of the sorted keys in src.  Unique keys go to
  // keys_a at the partition offset (in place when src is keys_a: the u-th
  // head is written only after the whole chunk holding position u was read,
  // and u never passes the position being read).  Pass A stores the head
  // positions in counts, pass B turns them into run lengths.
  T* ok = v.keys_a<T>() + off;
  uint32_t* oc = v.counts() + off;
  uint32_t U = 0;
  for (uint32_t c0 = 0; c0 < n; c0 += CAP) {
    const uint32_t cn = min(n - c0, (uint32_t)CAP);
    const uint32_t b0 = threadIdx.x * ITEMS;
    T kv[ITEMS];
    bool hd[ITEMS];
    unsigned nh = 0;
#pragma unroll
    for (int r = 0; r < ITEMS; ++r) {
      const uint32_t i = b0 + r;
      hd[r] = false;
      if (i < cn) {
        const uint32_t gi = c0 + i;
        kv[r] = src[gi];
        hd[r] = gi == 0 || kv[r] != src[gi - 1];
        nh += hd[r];
      }
    }
    unsigned tot;
    uint32_t u = U + block_exclusive_scan<NT, unsigned>(nh, scan_sm, &tot);
#pragma unroll
    for (int r = 0; r < ITEMS; ++r)
      if (hd[r]) {
        ok[u] = kv[r];
        oc[u] = c0 + b0 + r;
        u++;
      }
    U += tot;
    __syncthreads();
  }
  for (uint32_t c0 = 0; c0 < U; c0 += CAP) {
    const uint32_t cn = min(U - c0, (uint32_t)CAP);
    uint32_t cnt[ITEMS];
#pragma unroll
    for (int r = 0; r < ITEMS; ++r) {
      const uint32_t i = threadIdx.x + r * NT;
      cnt[r] = 0;
      if (i < cn) {
        const uint32_t q = c0 + i;
        cnt[r] = ((q + 1 < U) ? oc[q + 1] : n) - oc[q];
      }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < ITEMS; ++r) {
      const uint32_t i = threadIdx.x + r * NT;
      if (i < cn) oc[c0 + i] = cnt[r];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) v.bucket_rows()[bk] = U;
}

// One CTA per partition: copies its rows to the caller's arrays at the
// partition's row offset (rows past max_rows are dropped; the host reports
// the shortfall) and stores the partition's row count.
template <class T>
__global__ void __launch_bounds__(256) k_emit(uint8_t* scr, uint32_t P, T* __restrict__ out_keys,
                                              uint32_t* __restrict__ out_counts, unsigned long long max_rows,
                                              uint32_t* __restrict__ part_rows) {
  const View v{scr};
  const uint32_t bk = blockIdx.x;
  const uint32_t rows = v.bucket_rows()[bk];
  const unsigned long long ro = v.row_off()[bk];
  const uint32_t off = v.bucket_off()[bk];
  const T* ok = v.keys_a<T>() + off;
  const uint32_t* oc = v.counts() + off;
  for (uint32_t i = threadIdx.x; i < rows; i += blockDim.x) {
    if (ro + i >= max_rows) break;
    out_keys[ro + i] = ok[i];
    out_counts[ro + i] = oc[i];
  }
  if (threadIdx.x == 0) {
    part_rows[bk] = rows;
    if (bk == 0) v.counters()->nrows = v.row_off()[P];
  }
}

// Per device: the scratch array's address and the SM count, and the CUDA
// context they belong to.  A context that is destroyed and made again (for
// example after cudaDeviceReset) loads this module afresh, so its array can
// sit elsewhere: the entry is looked up again whenever the device's current
// context has another id.
struct DeviceEntry {
  unsigned long long ctx_id = 0;
  uint8_t* scratch = nullptr;
  uint32_t sms = 0;
};
std::mutex g_mu;
DeviceEntry g_dev[kMaxDevices];

typedef int (*CtxGetCurrentFn)(void**);
typedef int (*CtxGetIdFn)(void*, unsigned long long*);

// Id of the calling thread's current context (0 when it cannot be had).
unsigned long long current_ctx_id() {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  static bool looked = false;
  if (!looked) {
    looked = true;
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<CtxGetCurrentFn>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<CtxGetIdFn>(f);
  }
  if (!get_current || !get_id) return 0;
  void* ctx = nullptr;
  unsigned long long id = 0;
  if (get_current(&ctx) != 0 || !ctx || get_id(ctx, &id) != 0) return 0;
  return id;
}

// Address of this device's scratch array and its SM count, with that device
// current: looked up on the first call in each context of the device (on
// every call when the context id is unavailable).
int device_entry(int device, uint8_t** scratch, uint32_t* sms) {
  std::lock_guard<std::mutex> lock(g_mu);
  DeviceEntry& d = g_dev[device];
  const unsigned long long id = current_ctx_id();
  if (!d.scratch || id == 0 || id != d.ctx_id) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) return KITE_ERR_CUDA;
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || n < 1)
      return KITE_ERR_CUDA;
    d.scratch = static_cast<uint8_t*>(p);
    d.sms = (uint32_t)n;
    d.ctx_id = id;
  }
  *scratch = d.scratch;
  *sms = d.sms;
  return KITE_OK;
}

// Launches kernel f and returns the error of this launch alone (a launch
// error the caller had left pending is neither reported nor cleared).
template <class... KArgs, class... Args, size_t... I>
cudaError_t launch_impl(void (*f)(KArgs...), dim3 g, dim3 b, cudaStream_t s, std::index_sequence<I...>,
                        Args... args) {
  std::tuple<KArgs...> t(static_cast<KArgs>(args)...);
  void* p[sizeof...(KArgs) + 1] = {static_cast<void*>(&std::get<I>(t))...};
  return cudaLaunchKernel(reinterpret_cast<const void*>(f), g, b, p, 0, s);
}
template <class... KArgs, class... Args>
cudaError_t launch(void (*f)(KArgs...), dim3 g, dim3 b, cudaStream_t s, Args... args) {
  static_assert(sizeof...(KArgs) == sizeof...(Args), "kernel argument count");
  return launch_impl(f, g, b, s, std::index_sequence_for<KArgs...>{}, args...);
}

// Polls the stream until its work is done; no event or other object is made.
int wait_idle(cudaStream_t s, uint32_t timeout_ms) {
  const auto deadline = std::chrono::steady_clock::now() + std::chrono::milliseconds(timeout_ms);
  for (int spins = 0;; ++spins) {
    const cudaError_t q = cudaStreamQuery(s);
    if (q == cudaSuccess) return KITE_OK;
    if (q != cudaErrorNotReady) return KITE_ERR_CUDA;
    if (std::chrono::steady_clock::now() > deadline) return KITE_ERR_TIMEOUT;
    if (spins > 64) std::this_thread::sleep_for(std::chrono::microseconds(50));
  }
}

template <class T>
int run(uint8_t* scr, uint32_t sms, uint32_t k, bool canonical, uint32_t P, const uint8_t* d_fastq, uint32_t len,
        void* d_keys, uint32_t* d_counts, uint64_t max_rows, uint32_t* d_part_rows, uint64_t* totals,
        cudaStream_t s, uint32_t timeout_ms) {
  // What accumulates across threads starts at zero on every call.
  if (cudaMemsetAsync(scr + kOffBucketCount, 0, (size_t)P * 4, s) != cudaSuccess ||
      cudaMemsetAsync(scr + kOffBucketFill, 0, (size_t)P * 4, s) != cudaSuccess ||
      cudaMemsetAsync(scr + kOffCounters, 0, sizeof(Counters), s) != cudaSuccess)
    return KITE_ERR_CUDA;
  uint32_t log2p = 0;
  while ((1u << log2p) < P) ++log2p;
  const uint32_t shift = 64 - log2p;
  const uint32_t max_pieces = len / 4 + 2 + len / kPiece;
  // grid-stride kernels: four CTAs per SM at most
  const uint32_t g_pieces = std::min<uint32_t>((max_pieces + 255) / 256, 4 * sms);
  const uint32_t g_keys = std::min<uint32_t>(std::max<uint32_t>(len, 1) / 256 + 1, 4 * sms);
  uint32_t* const bucket_count = reinterpret_cast<uint32_t*>(scr + kOffBucketCount);
  uint32_t* const bucket_off = reinterpret_cast<uint32_t*>(scr + kOffBucketOff);
  uint32_t* const bucket_rows = reinterpret_cast<uint32_t*>(scr + kOffBucketRows);
  uint32_t* const row_off = reinterpret_cast<uint32_t*>(scr + kOffRowOff);
  const cudaError_t le[7] = {
      launch(k_lines, 1, 1024, s, d_fastq, len, scr),
      launch(k_extract<T>, g_pieces, 256, s, d_fastq, k, canonical ? 1u : 0u, shift, scr),
      launch(k_scan, 1, 1024, s, bucket_count, P, bucket_off),
      launch(k_scatter<T>, g_keys, 256, s, shift, scr),
      launch(k_sort_rle<T>, P, kSortThreads, s, scr),
      launch(k_scan, 1, 1024, s, bucket_rows, P, row_off),
      launch(k_emit<T>, P, 256, s, scr, P, static_cast<T*>(d_keys), d_counts, (unsigned long long)max_rows,
             d_part_rows)};
  for (const cudaError_t e : le)
    if (e != cudaSuccess) return KITE_ERR_CUDA;
  int rc = wait_idle(s, timeout_ms);
  if (rc) return rc;
  Counters hc;
  if (cudaMemcpyAsync(&hc, scr + kOffCounters, sizeof hc, cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return KITE_ERR_CUDA;
  rc = wait_idle(s, timeout_ms);
  if (rc) return rc;
  totals[0] = hc.reads;
  totals[1] = hc.bases;
  totals[2] = hc.kmers;
  totals[3] = hc.nrows;
  if (hc.status) return KITE_ERR_DEVICE;
  if (hc.nrows > max_rows) return KITE_ERR_BAD_INPUT;
  return KITE_OK;
}

}  // namespace
}  // namespace na
}  // namespace kite

extern "C" int kite_gpu_count_rows_noalloc(int device, int k, int canonical, uint32_t partitions,
                                           const uint8_t* d_fastq, size_t len, void* d_keys, uint32_t* d_counts,
                                           uint64_t max_rows, uint32_t* d_partition_rows, uint64_t* totals,
                                           void* stream, uint32_t timeout_ms) {
  using namespace kite::na;
  if (!totals) return KITE_ERR_BAD_INPUT;
  for (int i = 0; i < 4; ++i) totals[i] = 0;
  if (k < 1 || k > 64 || partitions < 2 || partitions > kMaxParts || (partitions & (partitions - 1)) ||
      !d_partition_rows || (max_rows && (!d_keys || !d_counts)) || (len && !d_fastq) || device < 0 ||
      device >= kMaxDevices)
    return KITE_ERR_BAD_INPUT;
  if (len > kMaxBytes) return KITE_ERR_UNSUPPORTED;
  int prev = 0;
  if (cudaGetDevice(&prev) != cudaSuccess) return KITE_ERR_CUDA;
  // with the device current its primary context is initialised, so the
  // context id below is that of the context the kernels will run in
  if (cudaSetDevice(device) != cudaSuccess) return KITE_ERR_CUDA;
  uint8_t* scr = nullptr;
  uint32_t sms = 0;
  int rc = device_entry(device, &scr, &sms);
  if (rc == KITE_OK) {
    const cudaStream_t s = static_cast<cudaStream_t>(stream);
    const uint32_t t = timeout_ms ? timeout_ms : 600000u;
    rc = k <= 31 ? run<uint64_t>(scr, sms, (uint32_t)k, canonical != 0, partitions, d_fastq, (uint32_t)len,
                                 d_keys, d_counts, max_rows, d_partition_rows, totals, s, t)
                 : run<u128>(scr, sms, (uint32_t)k, canonical != 0, partitions, d_fastq, (uint32_t)len, d_keys,
                             d_counts, max_rows, d_partition_rows, totals, s, t);
  }
  if (prev != device) cudaSetDevice(prev);
  return rc;
}
