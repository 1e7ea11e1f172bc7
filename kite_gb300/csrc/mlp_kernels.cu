// Learned CDF over the k-mer key space: a small FP32 MLP trained on the GPU
// by hand-written forward / backward / Adam kernels, then inverted into
// tile splitters.  No counterpart in the reference: it only moves tile
// boundaries, so counts stay exact whatever it predicts.
//
// Model.  Let V(key) be the top 48 of the 2k key bits; its top 16 bits are the
// key's bin b, the next 32 bits its place inside the bin.  With C(b) and m(b)
// the sample counts below and inside bin b (from the sample histogram),
//     F(key) = ( C(b) + m(b) * g(V(key)) ) / n
// where g is the MLP: 48 features in {0,1} -> 64 ReLU -> 64 ReLU -> 1.  The
// histogram places the mass of every bin; the network learns how that mass is
// spread inside a bin, which is what a histogram cannot resolve when one bin
// holds more than a tile's share of keys (low-complexity, AT-rich k-mers).
// Loss = mean over the sample of (F_hat - rank/n)^2, i.e. the global CDF
// error, so heavy bins dominate training.
//
// Splitter j: the bin holding quantile j/S from the histogram, then a
// bit-by-bit search of g inside the bin for the within-bin target.  The
// predicted max/mean tile load of the sample decides between these splitters
// and the histogram ones.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "mlp.h"
#include "kite_internal.h"

namespace kite {

static constexpr int kIn = 48, kH = 64;
static constexpr int kBinBits = 16, kSubBits = 32;
static constexpr uint32_t kTrainRows = 1u << 20;  // training rows taken from the sorted key sample
static constexpr int kParams = kIn * kH + kH + kH * kH + kH + kH + 1;

// parameter offsets
static constexpr int oW1 = 0, oB1 = oW1 + kIn * kH, oW2 = oB1 + kH, oB2 = oW2 + kH * kH, oW3 = oB2 + kH,
                     oB3 = oW3 + kH;

struct MlpModel {
  float* params = nullptr;  // device
  float* grads = nullptr;
  float* m = nullptr;
  float* v = nullptr;
  float* feats = nullptr;   // [n, kIn]
  float* target = nullptr;  // [n] within-bin fraction
  float* scale = nullptr;   // [n] m(b)/n
  float* loss = nullptr;    // [1]
  uint32_t cap = 0;
  void* keys_sorted = nullptr;
  size_t keys_cap = 0;
  unsigned* tile_hits = nullptr;
  uint32_t tile_cap = 0;
  uint32_t* batch_idx = nullptr;
  unsigned* hist = nullptr;   // [65536] sample histogram, then inclusive cumulative
  unsigned* hist2 = nullptr;  // [65536] the same over the sorted training subset
  float last_loss = 0;
  double last_pred_imbalance = 0;
  bool trained = false;
  uint32_t trained_key_bits = 0;
};

MlpModel* mlp_create() { return new MlpModel(); }

void mlp_destroy(MlpModel* m) {
  if (!m) return;
  cudaFree(m->params);
  cudaFree(m->grads);
  cudaFree(m->m);
  cudaFree(m->v);
  cudaFree(m->feats);
  cudaFree(m->target);
  cudaFree(m->scale);
  cudaFree(m->loss);
  cudaFree(m->keys_sorted);
  cudaFree(m->tile_hits);
  cudaFree(m->batch_idx);
  cudaFree(m->hist);
  cudaFree(m->hist2);
  delete m;
}

// ---- 48-bit view of a key ---------------------------------------------------
template <class T>
__device__ __forceinline__ uint64_t view48(T key, uint32_t key_bits) {
  return key_bits >= 48 ? (uint64_t)(key >> (key_bits - 48)) : ((uint64_t)key << (48 - key_bits));
}

template <class T>
__global__ void k_bin_hist(const T* __restrict__ keys, uint32_t n, uint32_t key_bits, unsigned* __restrict__ hist) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) atomicAdd(&hist[(uint32_t)(view48(keys[i], key_bits) >> kSubBits)], 1u);
}

// inclusive cumulative counts, one CTA
__global__ void __launch_bounds__(1024) k_cum(unsigned* __restrict__ h) {
  __shared__ unsigned sm[34];
  unsigned carry = 0;
  for (uint32_t b0 = 0; b0 < (1u << kBinBits); b0 += 1024) {
    const unsigned v = h[b0 + threadIdx.x];
    unsigned tot;
    const unsigned ex = block_exclusive_scan<1024, unsigned>(v, sm, &tot);
    h[b0 + threadIdx.x] = carry + ex + v;
    carry += tot;
  }
}

// Training rows from every `stride`-th key of the sorted sample of n keys:
// row j describes key i = j * stride (its rank among the n keys).
template <class T>
__global__ void k_make_features(const T* __restrict__ sorted, uint32_t n, uint32_t rows, uint32_t stride,
                                uint32_t key_bits, const unsigned* __restrict__ cum, float* __restrict__ feats,
                                float* __restrict__ target, float* __restrict__ scale) {
  const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= rows) return;
  const uint32_t i = j * stride;
  const uint64_t v = view48(sorted[i], key_bits);
  const uint32_t b = (uint32_t)(v >> kSubBits);
  const unsigned hi = cum[b], lo = b ? cum[b - 1] : 0u;
  const float m = (float)(hi - lo);
  float* f = feats + (size_t)j * kIn;
#pragma unroll
  for (int q = 0; q < kIn; ++q) f[q] = (float)((v >> (kIn - 1 - q)) & 1ull);
  target[j] = ((float)(i - lo) + 0.5f) / m;
  scale[j] = m / (float)n;
}

// ---- forward + backward ------------------------------------------------------
// One CTA handles kB samples: forward per sample (activations kept in shared
// memory, feature-major with a padded stride so lanes hit distinct banks),
// then weight-parallel gradient sums over the CTA's samples (no atomics
// inside the CTA), one global atomicAdd per parameter per CTA.
// Per-sample loss: (scale * (y - target))^2 / batch (scale = 1 without array).
static constexpr int kB = 128;        // samples per CTA (== threads)
static constexpr int kLd = kB + 1;    // padded row stride
static constexpr size_t kFbSmem = (size_t)(kParams + kIn * kLd + 3 * kH * kLd + kB) * sizeof(float);

__global__ void __launch_bounds__(kB) k_fwd_bwd(const float* __restrict__ params, const float* __restrict__ feats,
                                                const float* __restrict__ target, const float* __restrict__ scale,
                                                const uint32_t* __restrict__ idx, uint32_t batch,
                                                float* __restrict__ grads, float* __restrict__ loss) {
  extern __shared__ float sm[];
  float* P = sm;                       // parameters
  float* X = P + kParams;              // [kIn][kLd]
  float* H1 = X + kIn * kLd;           // [kH][kLd]  (relu output)
  float* H2 = H1 + kH * kLd;           // [kH][kLd]
  float* D = H2 + kH * kLd;            // [kH][kLd]  reused: d2 then d1 (pre-activation grads)
  float* DY = D + kH * kLd;            // [kB]
  const int t = threadIdx.x;
  for (int i = t; i < kParams; i += kB) P[i] = params[i];
  const uint32_t b = blockIdx.x * kB + t;
  const bool live = b < batch;
  const uint32_t s = live ? idx[b] : 0;
  for (int i = 0; i < kIn; ++i) X[i * kLd + t] = live ? feats[(size_t)s * kIn + i] : 0.f;
  __syncthreads();
  for (int j = 0; j < kH; ++j) {
    float a = P[oB1 + j];
    for (int i = 0; i < kIn; ++i) a += P[oW1 + j * kIn + i] * X[i * kLd + t];
    H1[j * kLd + t] = a > 0.f ? a : 0.f;
  }
  float y = P[oB3];
  for (int j = 0; j < kH; ++j) {
    float a = P[oB2 + j];
    for (int i = 0; i < kH; ++i) a += P[oW2 + j * kH + i] * H1[i * kLd + t];
    const float h = a > 0.f ? a : 0.f;
    H2[j * kLd + t] = h;
    y += P[oW3 + j] * h;
  }
  const float sc = live ? (scale ? scale[s] : 1.f) : 0.f;
  const float e = live ? sc * (y - target[s]) : 0.f;
  const float dy = live ? 2.f * e * sc / (float)batch : 0.f;
  DY[t] = dy;
  for (int j = 0; j < kH; ++j) D[j * kLd + t] = H2[j * kLd + t] > 0.f ? dy * P[oW3 + j] : 0.f;
  __syncthreads();
  for (int w = t; w < kH * kH + kH + kH + 1; w += kB) {
    float g = 0.f;
    if (w < kH * kH) {
      const int j = w / kH, i = w % kH;
      for (int q = 0; q < kB; ++q) g += D[j * kLd + q] * H1[i * kLd + q];
      atomicAdd(&grads[oW2 + w], g);
    } else if (w < kH * kH + kH) {
      const int j = w - kH * kH;
      for (int q = 0; q < kB; ++q) g += D[j * kLd + q];
      atomicAdd(&grads[oB2 + j], g);
    } else if (w < kH * kH + 2 * kH) {
      const int j = w - kH * kH - kH;
      for (int q = 0; q < kB; ++q) g += DY[q] * H2[j * kLd + q];
      atomicAdd(&grads[oW3 + j], g);
    } else {
      for (int q = 0; q < kB; ++q) g += DY[q];
      atomicAdd(&grads[oB3], g);
    }
  }
  float d1[kH];
  for (int i = 0; i < kH; ++i) d1[i] = 0.f;
  for (int j = 0; j < kH; ++j) {
    const float dj = D[j * kLd + t];
    if (dj != 0.f)
      for (int i = 0; i < kH; ++i) d1[i] += dj * P[oW2 + j * kH + i];
  }
  __syncthreads();
  for (int i = 0; i < kH; ++i) D[i * kLd + t] = H1[i * kLd + t] > 0.f ? d1[i] : 0.f;
  __syncthreads();
  for (int w = t; w < kIn * kH + kH; w += kB) {
    float g = 0.f;
    if (w < kIn * kH) {
      const int j = w / kIn, i = w % kIn;
      for (int q = 0; q < kB; ++q) g += D[j * kLd + q] * X[i * kLd + q];
      atomicAdd(&grads[oW1 + w], g);
    } else {
      const int j = w - kIn * kH;
      for (int q = 0; q < kB; ++q) g += D[j * kLd + q];
      atomicAdd(&grads[oB1 + j], g);
    }
  }
  float l = e * e / (float)batch;
  for (int o = 16; o; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
  if ((t & 31) == 0 && l != 0.f) atomicAdd(loss, l);
}

__global__ void k_adam(float* __restrict__ p, float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       float lr, float b1, float b2, float eps, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kParams) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  g[i] = 0.f;
}

// Batch indices: a strided walk (stride coprime to n) over the sample.
__global__ void k_batch_idx(uint32_t* idx, uint32_t batch, uint32_t n, uint32_t start, uint32_t stride) {
  const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < batch) idx[b] = (uint32_t)(((uint64_t)(start + b) * stride) % n);
}

// One warp per splitter j: bin from the cumulative histogram, then the
// largest 32-bit sub-position whose predicted within-bin fraction stays below
// the target; the splitter is the first key of the next 48-bit cell.  Lane l
// holds hidden units l and l + 32 (weights transposed in shared memory so the
// lanes read consecutive words); every sum runs over its inputs in index
// order, one fused multiply-add at a time, so each lane's arithmetic is that of
// a plain sequential forward pass.
template <class T>
__global__ void __launch_bounds__(256) k_invert(const float* __restrict__ params, const unsigned* __restrict__ cum,
                                                uint32_t n, uint32_t S, uint32_t key_bits, T* __restrict__ spl) {
  extern __shared__ float P[];  // W1 as [input][hidden], W2 as [input][output]; biases and w3 as given
  for (int i = threadIdx.x; i < kParams; i += blockDim.x) {
    float v = params[i];
    int at = i;
    if (i < oB1) at = oW1 + (i % kIn) * kH + i / kIn;                        // W1[j][i] -> [i][j]
    else if (i >= oW2 && i < oB2) at = oW2 + ((i - oW2) % kH) * kH + (i - oW2) / kH;  // W2[j][i] -> [i][j]
    P[at] = v;
  }
  __syncthreads();
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t j = (blockIdx.x * blockDim.x + threadIdx.x) / 32 + 1;
  if (j >= S) return;
  const double q = (double)n * j / S;  // sample rank at the cut
  uint32_t lo = 0, hi = (1u << kBinBits) - 1;
  while (lo < hi) {  // first bin whose inclusive cumulative count exceeds q
    const uint32_t mid = (lo + hi) >> 1;
    if ((double)cum[mid] > q) hi = mid;
    else lo = mid + 1;
  }
  const uint32_t b = lo;
  const double below = b ? cum[b - 1] : 0.0, mass = (double)cum[b] - below;
  const float u = mass > 0 ? (float)((q - below) / mass) : 1.f;
  uint32_t sub = 0;
  for (int bit = kSubBits - 1; bit >= 0; --bit) {
    const uint32_t cand = sub | (1u << bit);
    const uint64_t v = ((uint64_t)b << kSubBits) | cand;
    float a0 = P[oB1 + lane], a1 = P[oB1 + lane + 32];
#pragma unroll
    for (int i = 0; i < kIn; ++i) {
      const float xi = (float)((v >> (kIn - 1 - i)) & 1ull);
      a0 += P[oW1 + i * kH + lane] * xi;
      a1 += P[oW1 + i * kH + lane + 32] * xi;
    }
    const float h0 = a0 > 0.f ? a0 : 0.f, h1 = a1 > 0.f ? a1 : 0.f;
    float c0 = P[oB2 + lane], c1 = P[oB2 + lane + 32];
#pragma unroll 8
    for (int i = 0; i < 32; ++i) {
      const float hv = __shfl_sync(0xffffffffu, h0, i);
      c0 += P[oW2 + i * kH + lane] * hv;
      c1 += P[oW2 + i * kH + lane + 32] * hv;
    }
#pragma unroll 8
    for (int i = 0; i < 32; ++i) {
      const float hv = __shfl_sync(0xffffffffu, h1, i);
      c0 += P[oW2 + (i + 32) * kH + lane] * hv;
      c1 += P[oW2 + (i + 32) * kH + lane + 32] * hv;
    }
    const float r0 = c0 > 0.f ? c0 : 0.f, r1 = c1 > 0.f ? c1 : 0.f;
    float y = P[oB3];
#pragma unroll 8
    for (int i = 0; i < 32; ++i) y += P[oW3 + i] * __shfl_sync(0xffffffffu, r0, i);
#pragma unroll 8
    for (int i = 0; i < 32; ++i) y += P[oW3 + 32 + i] * __shfl_sync(0xffffffffu, r1, i);
    if (y <= u) sub = cand;
  }
  if (lane != 0) return;
  const uint64_t cell = (((uint64_t)b << kSubBits) | sub) + 1;  // first cell above
  T s;
  if (key_bits >= 48) {
    s = cell >= (1ull << 48) ? ((key_bits == (uint32_t)KeyTraits<T>::kBits) ? ~T(0) : (T(1) << key_bits) - T(1))
                             : (T)cell << (key_bits - 48);
  } else {
    s = (T)((cell + ((1ull << (48 - key_bits)) - 1)) >> (48 - key_bits));
  }
  spl[j - 1] = s;
}

template <class T>
__global__ void __launch_bounds__(256) k_tile_hits(const T* __restrict__ sample, uint32_t n,
                                                   const T* __restrict__ spl, uint32_t S,
                                                   unsigned* __restrict__ hits) {
  extern __shared__ __align__(16) uint8_t smraw[];
  unsigned* h = reinterpret_cast<unsigned*>(smraw);  // S counters of this CTA
  for (uint32_t t = threadIdx.x; t < S; t += blockDim.x) h[t] = 0;
  __syncthreads();
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    // tile = number of the S - 1 splitters <= key (any S)
    const T x = sample[i];
    uint32_t lo = 0, hi = S - 1;
    while (lo < hi) {
      const uint32_t mid = (lo + hi) >> 1;
      if (spl[mid] <= x) lo = mid + 1;
      else hi = mid;
    }
    atomicAdd(&h[lo], 1u);
  }
  __syncthreads();
  for (uint32_t t = threadIdx.x; t < S; t += blockDim.x)
    if (h[t]) atomicAdd(&hits[t], h[t]);
}

// Sorts the n splitters in place: one CTA, a bitonic network in shared
// memory over the next power of two (padded with the all-ones key).
template <class T>
__global__ void __launch_bounds__(1024) k_sort_splitters(T* spl, uint32_t n) {
  extern __shared__ __align__(16) uint8_t smraw[];
  T* v = reinterpret_cast<T*>(smraw);
  uint32_t np2 = 1;
  while (np2 < n) np2 <<= 1;
  for (uint32_t i = threadIdx.x; i < np2; i += blockDim.x) v[i] = i < n ? spl[i] : ~T(0);
  __syncthreads();
  for (uint32_t k = 2; k <= np2; k <<= 1)
    for (uint32_t j = k >> 1; j; j >>= 1) {
      for (uint32_t i = threadIdx.x; i < np2; i += blockDim.x) {
        const uint32_t l = i ^ j;
        if (l > i) {
          const T a = v[i], b = v[l];
          if (((i & k) == 0) == (b < a)) {
            v[i] = b;
            v[l] = a;
          }
        }
      }
      __syncthreads();
    }
  for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) spl[i] = v[i];
}

template <class T>
static size_t splitter_sort_smem(uint32_t n) {
  uint32_t np2 = 1;
  while (np2 < n) np2 <<= 1;
  const size_t bytes = (size_t)np2 * sizeof(T);
  cudaFuncSetAttribute(k_sort_splitters<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  return bytes;
}

// Bitonic sort of the sample in device memory (padded to a power of two
// with the all-ones key, which sorts last and is dropped).
template <class T>
__global__ void k_pad(T* keys, const T* src, uint32_t n, uint32_t np2) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < np2) keys[i] = i < n ? src[i] : ~T(0);
}

template <class T>
__global__ void k_bitonic_step(T* keys, uint32_t np2, uint32_t j, uint32_t k) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np2) return;
  const uint32_t l = i ^ j;
  if (l <= i) return;
  const T a = keys[i], b = keys[l];
  const bool up = (i & k) == 0;
  if ((a > b) == up) {
    keys[i] = b;
    keys[l] = a;
  }
}

namespace {

template <class T>
int sort_sample(MlpModel* m, const T* d_sample, uint32_t n, cudaStream_t s, T** out) {
  uint32_t np2 = 1, launches = 1;
  while (np2 < n) np2 <<= 1;
  const size_t bytes = (size_t)np2 * sizeof(T);
  if (m->keys_cap < bytes) {
    cudaFree(m->keys_sorted);
    if (cudaMalloc(&m->keys_sorted, bytes) != cudaSuccess) return -1;
    m->keys_cap = bytes;
  }
  T* keys = static_cast<T*>(m->keys_sorted);
  const uint32_t blocks = (np2 + 255) / 256;
  k_pad<T><<<blocks, 256, 0, s>>>(keys, d_sample, n, np2);
  for (uint32_t k = 2; k <= np2; k <<= 1)
    for (uint32_t j = k >> 1; j > 0; j >>= 1) {
      k_bitonic_step<T><<<blocks, 256, 0, s>>>(keys, np2, j, k);
      launches++;
    }
  *out = keys;
  return (int)launches;
}

}  // namespace

template <class T>
int predict_imbalance(MlpModel* m, const T* d_sample, uint32_t n, const T* d_spl, uint32_t S, cudaStream_t s,
                      uint32_t timeout_ms, double* out) {
  *out = 0.0;
  if (n == 0 || S < 2) return 0;
  if (m->tile_cap < S) {
    cudaFree(m->tile_hits);
    if (cudaMalloc(&m->tile_hits, (size_t)S * 4) != cudaSuccess) return 1;
    m->tile_cap = S;
  }
  cudaMemsetAsync(m->tile_hits, 0, (size_t)S * 4, s);
  const uint32_t grid = std::min<uint32_t>((n + 255) / 256, 4 * 152);
  k_tile_hits<T><<<grid, 256, (size_t)S * 4, s>>>(d_sample, n, d_spl, S, m->tile_hits);
  std::vector<unsigned> h(S);
  cudaMemcpyAsync(h.data(), m->tile_hits, (size_t)S * 4, cudaMemcpyDeviceToHost, s);
  if (bounded_sync(s, timeout_ms)) return 1;
  unsigned mx = 0;
  for (unsigned v : h) mx = std::max(mx, v);
  *out = (double)mx / ((double)n / S);
  return 0;
}
template int predict_imbalance<uint64_t>(MlpModel*, const uint64_t*, uint32_t, const uint64_t*, uint32_t,
                                         cudaStream_t, uint32_t, double*);
template int predict_imbalance<u128>(MlpModel*, const u128*, uint32_t, const u128*, uint32_t, cudaStream_t,
                                     uint32_t, double*);

int mlp_train(MlpModel* m, uint32_t n, int steps, uint32_t batch, float lr, cudaStream_t s, uint32_t timeout_ms,
              float* final_loss, int* launches);

template <class T>
int mlp_splitters(MlpModel* m, const T* d_sample, uint32_t n, uint32_t key_bits, uint32_t S, T* d_spl,
                  cudaStream_t s, uint32_t timeout_ms, MlpReport* rep) {
  *rep = MlpReport{};
  rep->pred_imbalance = 1e30;
  if (!m || n < 4 * S || n < 1024) return 0;  // too few samples to learn from
  if (!m->hist && cudaMalloc(&m->hist, sizeof(unsigned) << kBinBits) != cudaSuccess) return 1;
  if (!m->hist2 && cudaMalloc(&m->hist2, sizeof(unsigned) << kBinBits) != cudaSuccess) return 1;
  // cumulative bin histogram of the whole sample (its order does not matter)
  cudaMemsetAsync(m->hist, 0, sizeof(unsigned) << kBinBits, s);
  k_bin_hist<T><<<(n + 255) / 256, 256, 0, s>>>(d_sample, n, key_bits, m->hist);
  k_cum<<<1, 1024, 0, s>>>(m->hist);
  rep->launches += 2;
  const size_t smem = kParams * sizeof(float);
  cudaFuncSetAttribute(k_invert<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (m->trained && m->trained_key_bits == key_bits) {
    // the within-bin shape learned on an earlier segment, over this sample's histogram
    k_invert<T><<<(uint32_t)(((size_t)(S - 1) * 32 + 255) / 256), 256, smem, s>>>(m->params, m->hist, n, S, key_bits, d_spl);
    k_sort_splitters<T><<<1, 1024, splitter_sort_smem<T>(S - 1), s>>>(d_spl, S - 1);
    rep->launches += 3;
    double pred = 0;
    if (predict_imbalance<T>(m, d_sample, n, d_spl, S, s, timeout_ms, &pred)) return 1;
    if (pred <= m->last_pred_imbalance * 1.05) {
      rep->pred_imbalance = pred;
      rep->loss = m->last_loss;
      rep->reused = true;
      return cudaGetLastError() == cudaSuccess ? 0 : 1;
    }
  }
  // training rows: the within-bin ranks of a sorted subset of at most
  // kTrainRows keys (the sample fills in no particular order)
  const uint32_t rows = n < kTrainRows ? n : kTrainRows;
  T* sorted = nullptr;
  const int sl = sort_sample<T>(m, d_sample, rows, s, &sorted);
  if (sl < 0) return 1;
  rep->launches += sl;
  if (m->cap < rows) {
    cudaFree(m->feats);
    cudaFree(m->target);
    cudaFree(m->scale);
    if (cudaMalloc(&m->feats, (size_t)rows * kIn * sizeof(float)) != cudaSuccess) return 1;
    if (cudaMalloc(&m->target, (size_t)rows * sizeof(float)) != cudaSuccess) return 1;
    if (cudaMalloc(&m->scale, (size_t)rows * sizeof(float)) != cudaSuccess) return 1;
    m->cap = rows;
  }
  cudaMemsetAsync(m->hist2, 0, sizeof(unsigned) << kBinBits, s);
  k_bin_hist<T><<<(rows + 255) / 256, 256, 0, s>>>(sorted, rows, key_bits, m->hist2);
  k_cum<<<1, 1024, 0, s>>>(m->hist2);
  k_make_features<T><<<(rows + 255) / 256, 256, 0, s>>>(sorted, rows, rows, 1, key_bits, m->hist2, m->feats,
                                                         m->target, m->scale);
  rep->launches += 3;
  const int steps = 400;
  int tl = 0;
  if (mlp_train(m, rows, steps, 8192, 2e-3f, s, timeout_ms, &rep->loss, &tl)) return 1;
  rep->launches += tl;
  k_invert<T><<<(uint32_t)(((size_t)(S - 1) * 32 + 255) / 256), 256, smem, s>>>(m->params, m->hist, n, S, key_bits, d_spl);
  k_sort_splitters<T><<<1, 1024, splitter_sort_smem<T>(S - 1), s>>>(d_spl, S - 1);
  rep->launches += 2;
  if (predict_imbalance<T>(m, d_sample, n, d_spl, S, s, timeout_ms, &rep->pred_imbalance)) return 1;
  rep->launches += 1;
  m->last_loss = rep->loss;
  m->last_pred_imbalance = rep->pred_imbalance;
  m->trained = true;
  m->trained_key_bits = key_bits;
  return cudaGetLastError() == cudaSuccess ? 0 : 1;
}
template int mlp_splitters<uint64_t>(MlpModel*, const uint64_t*, uint32_t, uint32_t, uint32_t, uint64_t*,
                                     cudaStream_t, uint32_t, MlpReport*);
template int mlp_splitters<u128>(MlpModel*, const u128*, uint32_t, uint32_t, uint32_t, u128*, cudaStream_t, uint32_t,
                                 MlpReport*);

// Trains on m->feats / m->target / m->scale (n samples) with Adam; fixed init.
int mlp_train(MlpModel* m, uint32_t n, int steps, uint32_t batch, float lr, cudaStream_t s, uint32_t timeout_ms,
              float* final_loss, int* launches) {
  if (!m->params) {
    if (cudaMalloc(&m->params, kParams * sizeof(float)) != cudaSuccess) return 1;
    cudaMalloc(&m->grads, kParams * sizeof(float));
    cudaMalloc(&m->m, kParams * sizeof(float));
    cudaMalloc(&m->v, kParams * sizeof(float));
    cudaMalloc(&m->loss, sizeof(float) * 2);
    cudaMalloc(&m->batch_idx, (size_t)65536 * 4);
  }
  std::vector<float> p(kParams, 0.f);
  uint64_t st = 0x2545F4914F6CDD1Dull;
  auto rnd = [&]() {
    st = st * 6364136223846793005ull + 1442695040888963407ull;
    return ((double)(st >> 11) / 9007199254740992.0) * 2.0 - 1.0;
  };
  for (int i = 0; i < kIn * kH; ++i) p[oW1 + i] = (float)(rnd() * std::sqrt(6.0 / kIn));
  for (int i = 0; i < kH * kH; ++i) p[oW2 + i] = (float)(rnd() * std::sqrt(6.0 / kH));
  for (int i = 0; i < kH; ++i) p[oW3 + i] = (float)(rnd() * std::sqrt(3.0 / kH));
  for (int i = 0; i < kH; ++i) p[oB1 + i] = 0.01f;
  for (int i = 0; i < kH; ++i) p[oB2 + i] = 0.01f;
  p[oB3] = 0.5f;
  cudaMemcpyAsync(m->params, p.data(), kParams * sizeof(float), cudaMemcpyHostToDevice, s);
  cudaMemsetAsync(m->grads, 0, kParams * sizeof(float), s);
  cudaMemsetAsync(m->m, 0, kParams * sizeof(float), s);
  cudaMemsetAsync(m->v, 0, kParams * sizeof(float), s);
  batch = std::min(std::min(batch, n), 65536u);
  auto gcd = [](uint32_t a, uint32_t b) {
    while (b) {
      uint32_t t = a % b;
      a = b;
      b = t;
    }
    return a;
  };
  uint32_t stride = 2654435761u % n;
  if (stride == 0) stride = 1;
  while (gcd(stride, n) != 1) stride++;
  cudaFuncSetAttribute(k_fwd_bwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kFbSmem);
  const float b1 = 0.9f, b2 = 0.999f;
  double c1 = 1, c2 = 1;
  for (int t = 0; t < steps; ++t) {
    k_batch_idx<<<(batch + 255) / 256, 256, 0, s>>>(m->batch_idx, batch, n, (uint32_t)((uint64_t)t * batch % n),
                                                    stride);
    cudaMemsetAsync(m->loss, 0, sizeof(float), s);
    k_fwd_bwd<<<(batch + kB - 1) / kB, kB, kFbSmem, s>>>(m->params, m->feats, m->target, m->scale, m->batch_idx,
                                                        batch, m->grads, m->loss);
    c1 *= b1;
    c2 *= b2;
    const float decay = t > steps * 3 / 4 ? 0.2f : (t > steps / 2 ? 0.5f : 1.0f);
    k_adam<<<(kParams + 255) / 256, 256, 0, s>>>(m->params, m->grads, m->m, m->v, lr * decay, b1, b2, 1e-8f,
                                                 (float)(1 - c1), (float)(1 - c2));
  }
  *launches = 3 * steps;
  float l = 0;
  cudaMemcpyAsync(&l, m->loss, sizeof(float), cudaMemcpyDeviceToHost, s);
  if (bounded_sync(s, timeout_ms)) return 1;
  if (final_loss) *final_loss = l;
  return cudaGetLastError() == cudaSuccess ? 0 : 1;
}

}  // namespace kite

// ---- test hooks (C ABI, no counterpart in the reference) -------------------------
// One forward + backward of the learned-CDF network over n samples (unit
// scale) against a given parameter vector, so tests can check the
// hand-written gradients against a CPU float64 reference.
extern "C" int kite_mlp_grad_check(const float* params, const float* feats, const float* target, uint32_t n,
                                   float* grads_out, float* loss_out) {
  using namespace kite;
  float *dp, *df, *dt, *dg, *dl;
  uint32_t* di;
  cudaMalloc(&dp, kParams * 4);
  cudaMalloc(&df, (size_t)n * kIn * 4);
  cudaMalloc(&dt, (size_t)n * 4);
  cudaMalloc(&dg, kParams * 4);
  cudaMalloc(&dl, 4);
  cudaMalloc(&di, (size_t)n * 4);
  std::vector<uint32_t> id(n);
  for (uint32_t i = 0; i < n; ++i) id[i] = i;
  cudaMemcpy(dp, params, kParams * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(df, feats, (size_t)n * kIn * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(dt, target, (size_t)n * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(di, id.data(), (size_t)n * 4, cudaMemcpyHostToDevice);
  cudaMemset(dg, 0, kParams * 4);
  cudaMemset(dl, 0, 4);
  cudaFuncSetAttribute(k_fwd_bwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kFbSmem);
  k_fwd_bwd<<<(n + kB - 1) / kB, kB, kFbSmem>>>(dp, df, dt, nullptr, di, n, dg, dl);
  cudaError_t e = cudaDeviceSynchronize();
  cudaMemcpy(grads_out, dg, kParams * 4, cudaMemcpyDeviceToHost);
  cudaMemcpy(loss_out, dl, 4, cudaMemcpyDeviceToHost);
  cudaFree(dp);
  cudaFree(df);
  cudaFree(dt);
  cudaFree(dg);
  cudaFree(dl);
  cudaFree(di);
  return e == cudaSuccess ? 0 : -1;
}

extern "C" int kite_mlp_param_count(void) { return kite::kParams; }
extern "C" int kite_mlp_input_count(void) { return kite::kIn; }
