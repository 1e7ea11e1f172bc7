// Learned CDF over the k-mer key space: a small FP32 MLP trained on the GPU
// by hand-written forward / backward / Adam kernels, then inverted into
// tile splitters.  No counterpart in the reference: it only moves tile
// boundaries, so counts stay exact whatever it predicts.
//
// Model: x = the top 32 bits of the 2k-bit key (below the fixed zero bits),
// as 32 features in {0,1};  h1 = relu(W1 x + b1) (64);  h2 = relu(W2 h1 + b2)
// (64);  y = w3 . h2 + b3  ~  CDF(key) in [0,1].  Loss = mean (y - rank/n)^2
// over the sampled keys (ranks from a sort of the sample).  The CDF is
// inverted by a bit-by-bit search per splitter, which only needs y to be
// non-decreasing to be exact and stays well defined otherwise; splitters are
// sorted afterwards.  The predicted max/mean tile load on the sample decides
// between these splitters and the histogram fallback.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "mlp.h"
#include "kite_internal.h"

namespace kite {

static constexpr int kIn = 32, kH = 64;
static constexpr int kParams = kIn * kH + kH + kH * kH + kH + kH + 1;  // 6337

// parameter offsets
static constexpr int oW1 = 0, oB1 = oW1 + kIn * kH, oW2 = oB1 + kH, oB2 = oW2 + kH * kH, oW3 = oB2 + kH,
                     oB3 = oW3 + kH;

struct MlpModel {
  float* params = nullptr;  // device
  float* grads = nullptr;
  float* m = nullptr;
  float* v = nullptr;
  float* feats = nullptr;   // [n, kIn]
  float* target = nullptr;  // [n]
  float* loss = nullptr;    // [1]
  uint32_t cap = 0;
  void* keys_sorted = nullptr;
  size_t keys_cap = 0;
  unsigned* tile_hits = nullptr;
  uint32_t tile_cap = 0;
  uint32_t* batch_idx = nullptr;
  float last_loss = 0;
  double last_pred_imbalance = 0;
  double last_hist_imbalance = 0;
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
  cudaFree(m->loss);
  cudaFree(m->keys_sorted);
  cudaFree(m->tile_hits);
  cudaFree(m->batch_idx);
  delete m;
}

// ---- features ---------------------------------------------------------------
template <class T>
__device__ __forceinline__ void key_features(T key, uint32_t key_bits, float* f) {
  // top 32 bits of the key_bits-wide value
  const int sh = (int)key_bits - kIn;
  const uint32_t top = sh >= 0 ? (uint32_t)(uint64_t)(key >> sh) : (uint32_t)(uint64_t)(key << (-sh));
#pragma unroll
  for (int i = 0; i < kIn; ++i) f[i] = (float)((top >> (kIn - 1 - i)) & 1u);
}

template <class T>
__global__ void k_make_features(const T* __restrict__ sorted, uint32_t n, uint32_t key_bits, float* __restrict__ feats,
                                float* __restrict__ target) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  key_features(sorted[i], key_bits, feats + (size_t)i * kIn);
  target[i] = ((float)i + 0.5f) / (float)n;
}

// ---- forward + backward ------------------------------------------------------
// One CTA handles kB samples: forward per sample (activations kept in shared
// memory, feature-major with a padded stride so lanes hit distinct banks),
// then weight-parallel gradient sums over the CTA's samples (no atomics
// inside the CTA), one global atomicAdd per parameter per CTA.
static constexpr int kB = 128;        // samples per CTA (== threads)
static constexpr int kLd = kB + 1;    // padded row stride
static constexpr size_t kFbSmem = (size_t)(kParams + kIn * kLd + 3 * kH * kLd + kB) * sizeof(float);

__global__ void __launch_bounds__(kB) k_fwd_bwd(const float* __restrict__ params, const float* __restrict__ feats,
                                                const float* __restrict__ target, const uint32_t* __restrict__ idx,
                                                uint32_t batch, float* __restrict__ grads, float* __restrict__ loss) {
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
  // forward
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
  const float e = live ? y - target[s] : 0.f;
  const float dy = live ? 2.f * e / (float)batch : 0.f;
  DY[t] = dy;
  // d2 = dy * w3 masked by relu
  for (int j = 0; j < kH; ++j) D[j * kLd + t] = H2[j * kLd + t] > 0.f ? dy * P[oW3 + j] : 0.f;
  __syncthreads();
  // grads of layer 3 and layer 2 (weight-parallel over the CTA's samples)
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
  // d1 = W2^T d2 masked by relu (per sample)
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
  // grads of layer 1
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
  // loss
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

// Batch index generator: a fixed-stride walk through a permutation-free
// shuffle (i * stride + offset mod n with stride coprime to n).
__global__ void k_batch_idx(uint32_t* idx, uint32_t batch, uint32_t n, uint32_t start, uint32_t stride) {
  const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < batch) idx[b] = (uint32_t)(((uint64_t)(start + b) * stride) % n);
}

// ---- inference: forward one key ---------------------------------------------
__device__ float mlp_eval(const float* __restrict__ P, const float* x) {
  float h1[kH];
  for (int j = 0; j < kH; ++j) {
    float a = P[oB1 + j];
#pragma unroll
    for (int i = 0; i < kIn; ++i) a += P[oW1 + j * kIn + i] * x[i];
    h1[j] = a > 0.f ? a : 0.f;
  }
  float y = P[oB3];
  for (int j = 0; j < kH; ++j) {
    float a = P[oB2 + j];
    for (int i = 0; i < kH; ++i) a += P[oW2 + j * kH + i] * h1[i];
    y += P[oW3 + j] * (a > 0.f ? a : 0.f);
  }
  return y;
}

// One thread per splitter: bit-by-bit search for the largest key whose
// predicted CDF stays below j/S (the model sees the top 32 bits; lower bits
// of the splitter stay 0).
template <class T>
__global__ void k_invert(const float* __restrict__ params, uint32_t S, uint32_t key_bits, T* __restrict__ spl) {
  extern __shared__ float P[];
  for (int i = threadIdx.x; i < kParams; i += blockDim.x) P[i] = params[i];
  __syncthreads();
  const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (j >= S) return;
  const float q = (float)j / (float)S;
  uint32_t top = 0;
  float x[kIn];
  for (int bit = kIn - 1; bit >= 0; --bit) {
    const uint32_t cand = top | (1u << bit);
#pragma unroll
    for (int i = 0; i < kIn; ++i) x[i] = (float)((cand >> (kIn - 1 - i)) & 1u);
    if (mlp_eval(P, x) <= q) top = cand;
  }
  // splitter = first key of the next 32-bit cell
  const int sh = (int)key_bits - kIn;
  T s;
  if (top == 0xffffffffu) s = sh >= 0 ? ((T)1 << key_bits) - T(1) : (T)top;
  else s = sh >= 0 ? ((T)(top + 1u) << sh) : (T)((top + 1u) >> (-sh));
  spl[j - 1] = s;
}

// Predicted per-tile load on the sample (sorted) for given splitters.
template <class T>
__global__ void k_tile_hits(const T* __restrict__ sample, uint32_t n, const T* __restrict__ spl, uint32_t S,
                            unsigned* __restrict__ hits) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t j = 0;
  for (uint32_t step = S >> 1; step; step >>= 1)
    if (spl[j + step - 1] <= sample[i]) j += step;
  atomicAdd(&hits[j], 1u);
}

// Sorts the splitters in place (odd-even transposition in one CTA).
template <class T>
__global__ void k_sort_splitters(T* spl, uint32_t n) {
  for (uint32_t round = 0; round < n; ++round) {
    for (uint32_t i = 2 * threadIdx.x + (round & 1); i + 1 < n; i += 2 * blockDim.x) {
      const T a = spl[i], b = spl[i + 1];
      if (b < a) {
        spl[i] = b;
        spl[i + 1] = a;
      }
    }
    __syncthreads();
  }
}

// ---- host driver ----------------------------------------------------------------
namespace {

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

template <class T>
void sort_sample(MlpModel* m, const T* d_sample, uint32_t n, cudaStream_t s, T** out) {
  uint32_t np2 = 1;
  while (np2 < n) np2 <<= 1;
  const size_t bytes = (size_t)np2 * sizeof(T);
  if (m->keys_cap < bytes) {
    cudaFree(m->keys_sorted);
    cudaMalloc(&m->keys_sorted, bytes);
    m->keys_cap = bytes;
  }
  T* keys = static_cast<T*>(m->keys_sorted);
  const uint32_t blocks = (np2 + 255) / 256;
  k_pad<T><<<blocks, 256, 0, s>>>(keys, d_sample, n, np2);
  for (uint32_t k = 2; k <= np2; k <<= 1)
    for (uint32_t j = k >> 1; j > 0; j >>= 1) k_bitonic_step<T><<<blocks, 256, 0, s>>>(keys, np2, j, k);
  *out = keys;
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
  k_tile_hits<T><<<(n + 255) / 256, 256, 0, s>>>(d_sample, n, d_spl, S, m->tile_hits);
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
  T* sorted = nullptr;
  sort_sample<T>(m, d_sample, n, s, &sorted);
  uint32_t np2 = 1, lg = 0;
  while (np2 < n) {
    np2 <<= 1;
    lg++;
  }
  rep->launches += 1 + (int)(lg * (lg + 1) / 2);
  if (m->cap < n) {
    cudaFree(m->feats);
    cudaFree(m->target);
    if (cudaMalloc(&m->feats, (size_t)n * kIn * sizeof(float)) != cudaSuccess) return 1;
    if (cudaMalloc(&m->target, (size_t)n * sizeof(float)) != cudaSuccess) return 1;
    m->cap = n;
  }
  k_make_features<T><<<(n + 255) / 256, 256, 0, s>>>(sorted, n, key_bits, m->feats, m->target);
  rep->launches += 1;
  int steps = 400;
  if (const char* e = getenv("KITE_MLP_STEPS")) steps = std::max(1, atoi(e));
  int tl = 0;
  if (mlp_train(m, n, steps, 8192, 3e-3f, s, timeout_ms, &rep->loss, &tl)) return 1;
  rep->launches += tl;
  const size_t smem = kParams * sizeof(float);
  cudaFuncSetAttribute(k_invert<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k_invert<T><<<(S + 127) / 128, 128, smem, s>>>(m->params, S, key_bits, d_spl);
  k_sort_splitters<T><<<1, 1024, 0, s>>>(d_spl, S - 1);
  rep->launches += 2;
  if (predict_imbalance<T>(m, sorted, n, d_spl, S, s, timeout_ms, &rep->pred_imbalance)) return 1;
  rep->launches += 1;
  m->last_loss = rep->loss;
  m->last_pred_imbalance = rep->pred_imbalance;
  return cudaGetLastError() == cudaSuccess ? 0 : 1;
}
template int mlp_splitters<uint64_t>(MlpModel*, const uint64_t*, uint32_t, uint32_t, uint32_t, uint64_t*,
                                     cudaStream_t, uint32_t, MlpReport*);
template int mlp_splitters<u128>(MlpModel*, const u128*, uint32_t, uint32_t, uint32_t, u128*, cudaStream_t, uint32_t,
                                 MlpReport*);

// Trains on m->feats / m->target (n samples) with Adam; deterministic init.
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
  // He-style init from a fixed LCG; output bias 0.5
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
  uint32_t* idx = m->batch_idx;
  // stride coprime with n
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
    k_batch_idx<<<(batch + 255) / 256, 256, 0, s>>>(idx, batch, n, (uint32_t)((uint64_t)t * batch % n), stride);
    cudaMemsetAsync(m->loss, 0, sizeof(float), s);
    k_fwd_bwd<<<(batch + kB - 1) / kB, kB, kFbSmem, s>>>(m->params, m->feats, m->target, idx, batch, m->grads,
                                                        m->loss);
    c1 *= b1;
    c2 *= b2;
    const float decay = t > steps / 2 ? 0.3f : 1.0f;
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
// Forward + backward of one batch against a given parameter vector, so tests can
// check the hand-written gradients against a CPU float64 reference.
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
  k_fwd_bwd<<<(n + kB - 1) / kB, kB, kFbSmem>>>(dp, df, dt, di, n, dg, dl);
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
