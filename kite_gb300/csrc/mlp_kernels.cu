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

// ---- forward + backward (one sample per thread, weights in shared memory) ---
// Gradients are accumulated per CTA in shared memory, then added to global.
__global__ void __launch_bounds__(256) k_fwd_bwd(const float* __restrict__ params, const float* __restrict__ feats,
                                                 const float* __restrict__ target, const uint32_t* __restrict__ idx,
                                                 uint32_t batch, float* __restrict__ grads, float* __restrict__ loss) {
  extern __shared__ float sp[];  // params | grads
  float* sg = sp + kParams;
  for (int i = threadIdx.x; i < kParams; i += blockDim.x) {
    sp[i] = params[i];
    sg[i] = 0.f;
  }
  __syncthreads();
  const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
  float lsum = 0.f;
  if (b < batch) {
    const uint32_t s = idx[b];
    float x[kIn];
#pragma unroll
    for (int i = 0; i < kIn; ++i) x[i] = feats[(size_t)s * kIn + i];
    float h1[kH], h2[kH];
    for (int j = 0; j < kH; ++j) {
      float a = sp[oB1 + j];
#pragma unroll
      for (int i = 0; i < kIn; ++i) a += sp[oW1 + j * kIn + i] * x[i];
      h1[j] = a > 0.f ? a : 0.f;
    }
    for (int j = 0; j < kH; ++j) {
      float a = sp[oB2 + j];
      for (int i = 0; i < kH; ++i) a += sp[oW2 + j * kH + i] * h1[i];
      h2[j] = a > 0.f ? a : 0.f;
    }
    float y = sp[oB3];
    for (int j = 0; j < kH; ++j) y += sp[oW3 + j] * h2[j];
    const float e = y - target[s];
    lsum = e * e;
    const float dy = 2.f * e / (float)batch;
    // layer 3
    atomicAdd(&sg[oB3], dy);
    float d2[kH];
    for (int j = 0; j < kH; ++j) {
      atomicAdd(&sg[oW3 + j], dy * h2[j]);
      d2[j] = h2[j] > 0.f ? dy * sp[oW3 + j] : 0.f;
    }
    // layer 2
    float d1[kH];
    for (int i = 0; i < kH; ++i) d1[i] = 0.f;
    for (int j = 0; j < kH; ++j) {
      if (d2[j] == 0.f) continue;
      atomicAdd(&sg[oB2 + j], d2[j]);
      for (int i = 0; i < kH; ++i) {
        if (h1[i] > 0.f) atomicAdd(&sg[oW2 + j * kH + i], d2[j] * h1[i]);
        d1[i] += d2[j] * sp[oW2 + j * kH + i];
      }
    }
    // layer 1
    for (int j = 0; j < kH; ++j) {
      const float g = h1[j] > 0.f ? d1[j] : 0.f;
      if (g == 0.f) continue;
      atomicAdd(&sg[oB1 + j], g);
#pragma unroll
      for (int i = 0; i < kIn; ++i)
        if (x[i] != 0.f) atomicAdd(&sg[oW1 + j * kIn + i], g * x[i]);
    }
  }
  // loss
  for (int o = 16; o; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
  if ((threadIdx.x & 31) == 0 && lsum != 0.f) atomicAdd(loss, lsum / (float)batch);
  __syncthreads();
  for (int i = threadIdx.x; i < kParams; i += blockDim.x)
    if (sg[i] != 0.f) atomicAdd(&grads[i], sg[i]);
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

template <class T>
void sort_sample(MlpModel* m, const T* d_sample, uint32_t n, cudaStream_t s, T** out) {
  // copy to the model's buffer and sort it with the on-chip tile machinery
  // when small, else on the host (the sample is at most 2^20 keys)
  const size_t bytes = (size_t)n * sizeof(T);
  if (m->keys_cap < bytes) {
    cudaFree(m->keys_sorted);
    cudaMalloc(&m->keys_sorted, bytes);
    m->keys_cap = bytes;
  }
  std::vector<T> h(n);
  cudaMemcpyAsync(h.data(), d_sample, bytes, cudaMemcpyDeviceToHost, s);
  cudaStreamSynchronize(s);
  std::sort(h.begin(), h.end());
  cudaMemcpyAsync(m->keys_sorted, h.data(), bytes, cudaMemcpyHostToDevice, s);
  cudaStreamSynchronize(s);
  *out = static_cast<T*>(m->keys_sorted);
}

double imbalance_on_sample(MlpModel* m, const void* sorted, uint32_t n, const void* spl, uint32_t S, int key_bytes,
                           cudaStream_t s) {
  if (m->tile_cap < S) {
    cudaFree(m->tile_hits);
    cudaMalloc(&m->tile_hits, (size_t)S * 4);
    m->tile_cap = S;
  }
  cudaMemsetAsync(m->tile_hits, 0, (size_t)S * 4, s);
  if (key_bytes == 8)
    k_tile_hits<uint64_t><<<(n + 255) / 256, 256, 0, s>>>((const uint64_t*)sorted, n, (const uint64_t*)spl, S,
                                                          m->tile_hits);
  else
    k_tile_hits<u128><<<(n + 255) / 256, 256, 0, s>>>((const u128*)sorted, n, (const u128*)spl, S, m->tile_hits);
  std::vector<unsigned> h(S);
  cudaMemcpyAsync(h.data(), m->tile_hits, (size_t)S * 4, cudaMemcpyDeviceToHost, s);
  cudaStreamSynchronize(s);
  unsigned mx = 0;
  for (unsigned v : h) mx = std::max(mx, v);
  return n ? (double)mx / ((double)n / S) : 0.0;
}

}  // namespace

int mlp_train(MlpModel* m, const float* feats_host_or_null, uint32_t n, int steps, uint32_t batch, float lr,
              cudaStream_t s, float* final_loss);

template <class T>
int mlp_splitters(MlpModel* m, const T* d_sample, uint32_t n, uint32_t key_bits, uint32_t S, T* d_spl, double bound,
                  cudaStream_t s, bool* used) {
  *used = false;
  if (!m || n < 4 * S || n < 1024) return 0;  // too few samples to learn from
  T* sorted = nullptr;
  sort_sample<T>(m, d_sample, n, s, &sorted);
  if (m->cap < n) {
    cudaFree(m->feats);
    cudaFree(m->target);
    cudaMalloc(&m->feats, (size_t)n * kIn * sizeof(float));
    cudaMalloc(&m->target, (size_t)n * sizeof(float));
    m->cap = n;
  }
  k_make_features<T><<<(n + 255) / 256, 256, 0, s>>>(sorted, n, key_bits, m->feats, m->target);
  float loss = 0;
  if (mlp_train(m, nullptr, n, 400, 8192, 3e-3f, s, &loss)) return 1;
  m->last_loss = loss;
  const size_t smem = kParams * sizeof(float);
  cudaFuncSetAttribute(k_invert<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k_invert<T><<<(S + 127) / 128, 128, smem, s>>>(m->params, S, key_bits, d_spl);
  k_sort_splitters<T><<<1, 1024, 0, s>>>(d_spl, S - 1);
  const double imb = imbalance_on_sample(m, sorted, n, d_spl, S, sizeof(T), s);
  m->last_pred_imbalance = imb;
  *used = imb <= bound;
  return cudaGetLastError() == cudaSuccess ? 0 : 1;
}
template int mlp_splitters<uint64_t>(MlpModel*, const uint64_t*, uint32_t, uint32_t, uint32_t, uint64_t*, double,
                                     cudaStream_t, bool*);
template int mlp_splitters<u128>(MlpModel*, const u128*, uint32_t, uint32_t, uint32_t, u128*, double, cudaStream_t,
                                 bool*);

// Trains on m->feats / m->target (n samples) with Adam; deterministic init.
int mlp_train(MlpModel* m, const float* feats_host, uint32_t n, int steps, uint32_t batch, float lr, cudaStream_t s,
              float* final_loss) {
  (void)feats_host;
  if (!m->params) {
    cudaMalloc(&m->params, kParams * sizeof(float));
    cudaMalloc(&m->grads, kParams * sizeof(float));
    cudaMalloc(&m->m, kParams * sizeof(float));
    cudaMalloc(&m->v, kParams * sizeof(float));
    cudaMalloc(&m->loss, sizeof(float) * 2);
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
  batch = std::min(batch, n);
  uint32_t* idx = nullptr;
  cudaMallocAsync(&idx, (size_t)batch * 4, s);
  // stride coprime with n
  uint32_t stride = 2654435761u % n;
  auto gcd = [](uint32_t a, uint32_t b) {
    while (b) {
      uint32_t t = a % b;
      a = b;
      b = t;
    }
    return a;
  };
  if (stride == 0) stride = 1;
  while (gcd(stride, n) != 1) stride++;
  const size_t smem = 2 * kParams * sizeof(float);
  cudaFuncSetAttribute(k_fwd_bwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  const float b1 = 0.9f, b2 = 0.999f;
  double c1 = 1, c2 = 1;
  for (int t = 0; t < steps; ++t) {
    k_batch_idx<<<(batch + 255) / 256, 256, 0, s>>>(idx, batch, n, (uint32_t)((uint64_t)t * batch % n), stride);
    cudaMemsetAsync(m->loss, 0, sizeof(float), s);
    k_fwd_bwd<<<(batch + 255) / 256, 256, smem, s>>>(m->params, m->feats, m->target, idx, batch, m->grads, m->loss);
    c1 *= b1;
    c2 *= b2;
    const float decay = t > steps / 2 ? 0.3f : 1.0f;
    k_adam<<<(kParams + 255) / 256, 256, 0, s>>>(m->params, m->grads, m->m, m->v, lr * decay, b1, b2, 1e-8f,
                                                 (float)(1 - c1), (float)(1 - c2));
  }
  float l = 0;
  cudaMemcpyAsync(&l, m->loss, sizeof(float), cudaMemcpyDeviceToHost, s);
  cudaFreeAsync(idx, s);
  cudaStreamSynchronize(s);
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
  const size_t smem = 2 * kParams * sizeof(float);
  cudaFuncSetAttribute(k_fwd_bwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k_fwd_bwd<<<(n + 255) / 256, 256, smem>>>(dp, df, dt, di, n, dg, dl);
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
