// Learned CDF over the k-mer key space: a small FP32 network trained on the
// GPU by hand-written forward / backward / Adam kernels, then inverted into
// tile splitters.  No counterpart in the reference: it only moves tile
// boundaries, so counts stay exact whatever it predicts.
//
// Key view.  V(key) = the top 48 of the 2k key bits (zero-padded below for
// k < 24), bits x_0 (most significant) .. x_47.  The top 16 bits are the
// key's bin b.
//
// Model: a two-stage learned index over V.
//  Stage 1 (counts of the counter's key sample, up to 2^22 keys of the
//   segment's first chunk): C(b), m(b) = sample keys below / inside bin b;
//   every heavy bin (more than an eighth of a tile's share of the sample)
//   also gets counts of its 256 sub-cells (the next 8 bits), and every heavy
//   sub-cell counts of its own next 8 bits.
//  Stage 2 (the network): an autoregressive density over the bits below the
//   bin: for each bit i >= 16 it predicts P(x_i = 1 | x_0 .. x_{i-1}).  The
//   network is a masked MLP (48 inputs -> 64 ReLU -> 64 ReLU -> 32 logits):
//   hidden unit k has degree d(k) = 16 + k/2 and sees only inputs i < d(k)
//   (first layer) or first-layer units of degree <= d(k) (second layer), and
//   output o (bit 16 + o) sees only second-layer units of degree <= 16 + o,
//   so each output depends on the bits above its own (Germain et al., MADE,
//   2015).  The within-cell CDF it defines,
//       g(V) = sum over set bits i of V below the cell of
//              P(prefix x_0..x_{i-1}) * P(x_i = 0 | prefix)  / P(cell),
//   is monotone in V by construction (it is the distribution function of a
//   proper distribution over the bits), and it inverts exactly by
//   arithmetic decoding, bit by bit.
//  F(key) = (C(b) [+ the sub-cell counts below, heavy bins] + m * g(V)) / n.
// Training: maximum likelihood (binary cross-entropy of every bit i >= 16
// given the bits above it) over the whole sample, minibatches of 8192 keys
// drawn by a hash of (step, index), Adam.  The training steps are captured once as a CUDA graph (the step
// counter lives on the device) and replayed.
//
// Splitter j: the bin (and heavy bins' sub-cell) holding quantile j/S of the
// sample from the stage-1 counts, then the bits below it decoded from the
// network's conditionals so that g reaches the quantile's within-cell
// fraction.  The predicted max/mean tile load of the sample decides between
// these splitters and the histogram ones.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "mlp.h"
#include "kite_internal.h"

namespace kite {

static constexpr int kIn = 48, kH = 64, kB0 = 16, kOut = kIn - kB0;  // 32 predicted bits
static constexpr int kBinBits = 16;
static constexpr int kSubBits = 8;           // sub-cells of a heavy bin
static constexpr int kSubCells = 1 << kSubBits;
static constexpr int kParams = kIn * kH + kH + kH * kH + kH + kOut * kH + kOut;
static constexpr uint32_t kBatch = 8192;
static constexpr int kTrainSteps = 4000;
static constexpr int kStepsPerGraph = 50;
static constexpr float kLr = 3e-3f;

// parameter offsets: W1 [kH][kIn], b1, W2 [kH][kH], b2, W3 [kOut][kH], b3
static constexpr int oW1 = 0, oB1 = oW1 + kIn * kH, oW2 = oB1 + kH, oB2 = oW2 + kH * kH, oW3 = oB2 + kH,
                     oB3 = oW3 + kOut * kH;

// Degrees and masks.  Hidden unit k (either layer) has degree 16 + k/2.
__host__ __device__ constexpr int deg_of(int k) { return kB0 + k / 2; }
// first layer: unit j sees inputs i < deg(j)
__host__ __device__ constexpr int w1_inputs(int j) { return deg_of(j); }
// second layer: unit k sees first-layer units j with deg(j) <= deg(k), i.e. j <= (k | 1)
__host__ __device__ constexpr int w2_inputs(int k) { return (k | 1) + 1; }
// output o (bit 16 + o) sees second-layer units k with deg(k) <= 16 + o, i.e. k < 2o + 2
__host__ __device__ constexpr int w3_inputs(int o) { return 2 * o + 2 < kH ? 2 * o + 2 : kH; }
__host__ __device__ constexpr bool param_live(int p) {
  return p < oB1   ? (p % kIn) < w1_inputs(p / kIn)
         : p < oW2 ? true
         : p < oB2 ? ((p - oW2) % kH) < w2_inputs((p - oW2) / kH)
         : p < oW3 ? true
         : p < oB3 ? ((p - oW3) % kH) < w3_inputs((p - oW3) / kH)
                   : true;
}

struct MlpModel {
  float* params = nullptr;  // device
  float* grads = nullptr;
  float* m = nullptr;
  float* v = nullptr;
  float* loss = nullptr;     // [0] running sum of the step, [1] last step's loss
  unsigned* step = nullptr;  // training step counter (device)
  uint64_t* views = nullptr; // 48-bit views of the sample keys
  uint32_t views_cap = 0;
  unsigned* tile_hits = nullptr;
  uint32_t tile_cap = 0;
  unsigned* hist = nullptr;      // [65536] sample counts per bin, then inclusive cumulative
  int* heavy_idx = nullptr;      // [65536] heavy-bin slot or -1
  unsigned* sub = nullptr;       // [heavy slots][256] sub-cell counts, then inclusive cumulative
  unsigned* nheavy = nullptr;    // [2] heavy bins, heavy sub-cells
  uint32_t sub_cap = 0;          // heavy slots allocated
  int* heavy2_idx = nullptr;     // [heavy slots][256] second-level slot of a heavy sub-cell, or -1
  unsigned* sub2 = nullptr;      // [second-level slots][256] counts of a heavy sub-cell's next 8 bits
  cudaStream_t cap_stream = nullptr;
  cudaGraphExec_t graph = nullptr;
  uint32_t graph_n = 0;          // the sample size the graph was captured for
  float last_loss = 0;
  double last_pred_imbalance = 0;
  bool trained = false;
  uint32_t trained_key_bits = 0;
};

MlpModel* mlp_create() { return new MlpModel(); }

void mlp_destroy(MlpModel* m) {
  if (!m) return;
  if (m->graph) cudaGraphExecDestroy(m->graph);
  if (m->cap_stream) cudaStreamDestroy(m->cap_stream);
  cudaFree(m->params);
  cudaFree(m->grads);
  cudaFree(m->m);
  cudaFree(m->v);
  cudaFree(m->loss);
  cudaFree(m->step);
  cudaFree(m->views);
  cudaFree(m->tile_hits);
  cudaFree(m->hist);
  cudaFree(m->heavy_idx);
  cudaFree(m->sub);
  cudaFree(m->nheavy);
  cudaFree(m->heavy2_idx);
  cudaFree(m->sub2);
  delete m;
}

// ---- 48-bit view of a key ---------------------------------------------------
template <class T>
__device__ __forceinline__ uint64_t view48(T key, uint32_t key_bits) {
  return key_bits >= 48 ? (uint64_t)(key >> (key_bits - 48)) : ((uint64_t)key << (48 - key_bits));
}
__device__ __forceinline__ float bit_of(uint64_t v, int i) { return (float)((v >> (kIn - 1 - i)) & 1ull); }
// splitmix64 finalizer: the minibatch of step t draws sample mix64(t, b) mod n
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// ---- stage 1 ----------------------------------------------------------------
template <class T>
__global__ void k_views(const T* __restrict__ keys, uint32_t n, uint32_t key_bits, uint64_t* __restrict__ views,
                        unsigned* __restrict__ hist) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint64_t v = view48(keys[i], key_bits);
    views[i] = v;
    atomicAdd(&hist[(uint32_t)(v >> (kIn - kBinBits))], 1u);
  }
}

// Heavy bins (count > thr) get a slot; the rest -1.  Slots beyond `cap` are
// not given (those bins are treated as light).
__global__ void k_heavy(const unsigned* __restrict__ hist, unsigned thr, uint32_t cap, int* __restrict__ heavy_idx,
                        unsigned* __restrict__ nheavy) {
  const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= (1u << kBinBits)) return;
  int slot = -1;
  if (hist[b] > thr) {
    const unsigned s = atomicAdd(nheavy, 1u);
    if (s < cap) slot = (int)s;
  }
  heavy_idx[b] = slot;
}

__global__ void k_sub_hist(const uint64_t* __restrict__ views, uint32_t n, const int* __restrict__ heavy_idx,
                           unsigned* __restrict__ sub) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint64_t v = views[i];
    const int h = heavy_idx[(uint32_t)(v >> (kIn - kBinBits))];
    if (h >= 0) atomicAdd(&sub[(size_t)h * kSubCells + (uint32_t)((v >> (kIn - kBinBits - kSubBits)) & (kSubCells - 1))], 1u);
  }
}

// Heavy sub-cells (count > thr) of the heavy bins get a second-level slot:
// one thread per (slot, sub-cell), on the raw counts.
__global__ void k_heavy2(const unsigned* __restrict__ sub, const unsigned* __restrict__ nheavy, uint32_t cap,
                         unsigned thr, int* __restrict__ heavy2_idx, unsigned* __restrict__ nheavy2) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t nh = min(*nheavy, cap);
  if (i >= cap * kSubCells) return;
  int slot = -1;
  if (i / kSubCells < nh && sub[i] > thr) {
    const unsigned s2 = atomicAdd(nheavy2, 1u);
    if (s2 < cap) slot = (int)s2;
  }
  heavy2_idx[i] = slot;
}

__global__ void k_sub2_hist(const uint64_t* __restrict__ views, uint32_t n, const int* __restrict__ heavy_idx,
                            const int* __restrict__ heavy2_idx, unsigned* __restrict__ sub2) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint64_t v = views[i];
    const int h = heavy_idx[(uint32_t)(v >> (kIn - kBinBits))];
    if (h < 0) continue;
    const int h2 = heavy2_idx[(size_t)h * kSubCells + (uint32_t)((v >> (kIn - kBinBits - kSubBits)) & (kSubCells - 1))];
    if (h2 >= 0)
      atomicAdd(&sub2[(size_t)h2 * kSubCells + (uint32_t)((v >> (kIn - kBinBits - 2 * kSubBits)) & (kSubCells - 1))],
                1u);
  }
}

// inclusive cumulative counts of every heavy slot's sub-cells: one warp each
__global__ void k_sub_cum(unsigned* __restrict__ sub, const unsigned* __restrict__ nheavy, uint32_t cap) {
  const uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) / 32, lane = threadIdx.x & 31;
  const uint32_t nh = min(*nheavy, cap);
  if (w >= nh) return;
  unsigned* c = sub + (size_t)w * kSubCells;
  unsigned carry = 0;
  for (int b0 = 0; b0 < kSubCells; b0 += 32) {
    unsigned x = c[b0 + lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= (uint32_t)o) x += y;
    }
    c[b0 + lane] = x + carry;
    carry += __shfl_sync(0xffffffffu, x, 31);
  }
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

// ---- forward + backward ------------------------------------------------------
// One CTA handles kB samples (one per thread): the forward pass per sample
// with activations kept in shared memory (feature-major, padded stride), then
// weight-parallel gradient sums over the CTA's samples (live weights only;
// masked ones stay zero), one global atomicAdd per weight per CTA.
// Loss = mean over the batch and the 32 predicted bits of the binary
// cross-entropy.  Sample s of the batch is views[idx(s)], idx either given
// (idx != null) or drawn by a hash of (training step *step, b, seed).
static constexpr int kB = 128;        // samples per CTA (== threads)
static constexpr int kLd = kB + 1;    // padded row stride
static constexpr size_t kFbSmem = (size_t)(kParams + kIn * kLd + 3 * kH * kLd + kOut * kLd) * sizeof(float);

__global__ void __launch_bounds__(kB) k_fwd_bwd(const float* __restrict__ params, const uint64_t* __restrict__ views,
                                                const uint32_t* __restrict__ idx, const unsigned* __restrict__ step,
                                                uint32_t n, uint32_t seed, uint32_t batch,
                                                float* __restrict__ grads, float* __restrict__ loss) {
  extern __shared__ float sm[];
  float* P = sm;                      // parameters
  float* X = P + kParams;             // [kIn][kLd]
  float* H1 = X + kIn * kLd;          // [kH][kLd]  relu outputs
  float* H2 = H1 + kH * kLd;          // [kH][kLd]
  float* D = H2 + kH * kLd;           // [kH][kLd]  pre-activation gradients: layer 2, then layer 1
  float* DY = D + kH * kLd;           // [kOut][kLd] logit gradients
  const int t = threadIdx.x;
  for (int i = t; i < kParams; i += kB) P[i] = params[i];
  const uint32_t b = blockIdx.x * kB + t;
  const bool live = b < batch;
  uint32_t s = 0;
  if (live) {
    if (idx) s = idx[b];
    else s = (uint32_t)(mix64(((uint64_t)(*step) << 32) + b + ((uint64_t)seed << 20)) % n);
  }
  const uint64_t v = live ? views[s] : 0ull;
  for (int i = 0; i < kIn; ++i) X[i * kLd + t] = bit_of(v, i);
  __syncthreads();
  for (int j = 0; j < kH; ++j) {
    float a = P[oB1 + j];
    for (int i = 0; i < w1_inputs(j); ++i) a += P[oW1 + j * kIn + i] * X[i * kLd + t];
    H1[j * kLd + t] = a > 0.f ? a : 0.f;
  }
  for (int k = 0; k < kH; ++k) {
    float a = P[oB2 + k];
    for (int j = 0; j < w2_inputs(k); ++j) a += P[oW2 + k * kH + j] * H1[j * kLd + t];
    H2[k * kLd + t] = a > 0.f ? a : 0.f;
  }
  const float inv = live ? 1.f / ((float)batch * (float)kOut) : 0.f;
  float l = 0.f;
  for (int o = 0; o < kOut; ++o) {
    float a = P[oB3 + o];
    for (int k = 0; k < w3_inputs(o); ++k) a += P[oW3 + o * kH + k] * H2[k * kLd + t];
    const float x = X[(kB0 + o) * kLd + t];
    const float p = 1.f / (1.f + __expf(-a));
    DY[o * kLd + t] = (p - x) * inv;
    // binary cross-entropy from the logit: max(a, 0) - x a + log(1 + e^-|a|)
    l += (fmaxf(a, 0.f) - x * a + log1pf(__expf(-fabsf(a)))) * inv;
  }
  for (int k = 0; k < kH; ++k) {
    float g = 0.f;
    for (int o = k / 2; o < kOut; ++o) g += DY[o * kLd + t] * P[oW3 + o * kH + k];
    D[k * kLd + t] = H2[k * kLd + t] > 0.f ? g : 0.f;
  }
  __syncthreads();
  // second and third layer gradients
  for (int w = t; w < kH * kH + kH + kOut * kH + kOut; w += kB) {
    float g = 0.f;
    if (w < kH * kH) {
      const int k = w / kH, j = w % kH;
      if (j >= w2_inputs(k)) continue;
      for (int q = 0; q < kB; ++q) g += D[k * kLd + q] * H1[j * kLd + q];
      atomicAdd(&grads[oW2 + w], g);
    } else if (w < kH * kH + kH) {
      const int k = w - kH * kH;
      for (int q = 0; q < kB; ++q) g += D[k * kLd + q];
      atomicAdd(&grads[oB2 + k], g);
    } else if (w < kH * kH + kH + kOut * kH) {
      const int r = w - kH * kH - kH, o = r / kH, k = r % kH;
      if (k >= w3_inputs(o)) continue;
      for (int q = 0; q < kB; ++q) g += DY[o * kLd + q] * H2[k * kLd + q];
      atomicAdd(&grads[oW3 + r], g);
    } else {
      const int o = w - kH * kH - kH - kOut * kH;
      for (int q = 0; q < kB; ++q) g += DY[o * kLd + q];
      atomicAdd(&grads[oB3 + o], g);
    }
  }
  // first layer pre-activation gradients (D is rewritten after every thread
  // has used the second layer's)
  float d1[kH];
#pragma unroll
  for (int j = 0; j < kH; ++j) d1[j] = 0.f;
  for (int k = 0; k < kH; ++k) {
    const float dk = D[k * kLd + t];
    const int lim = w2_inputs(k);
    if (dk != 0.f) {
#pragma unroll
      for (int j = 0; j < kH; ++j)
        if (j < lim) d1[j] += dk * P[oW2 + k * kH + j];
    }
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < kH; ++j) D[j * kLd + t] = H1[j * kLd + t] > 0.f ? d1[j] : 0.f;
  __syncthreads();
  for (int w = t; w < kIn * kH + kH; w += kB) {
    float g = 0.f;
    if (w < kIn * kH) {
      const int j = w / kIn, i = w % kIn;
      if (i >= w1_inputs(j)) continue;
      for (int q = 0; q < kB; ++q) g += D[j * kLd + q] * X[i * kLd + q];
      atomicAdd(&grads[oW1 + w], g);
    } else {
      const int j = w - kIn * kH;
      for (int q = 0; q < kB; ++q) g += D[j * kLd + q];
      atomicAdd(&grads[oB1 + j], g);
    }
  }
  for (int o = 16; o; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
  if ((t & 31) == 0 && l != 0.f) atomicAdd(loss, l);
}

// Adam step of the whole parameter vector by one CTA: the step number, the
// learning rate schedule (halved after half the steps, x0.2 after three
// quarters) and the bias corrections come from the device step counter,
// which the CTA then advances; the step's loss moves to loss[1].
__global__ void __launch_bounds__(1024) k_adam(float* __restrict__ p, float* __restrict__ g, float* __restrict__ m,
                                               float* __restrict__ v, unsigned* __restrict__ step,
                                               float* __restrict__ loss, uint32_t total_steps, float lr0) {
  const unsigned t = *step;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const float c1 = 1.f - powf(b1, (float)(t + 1)), c2 = 1.f - powf(b2, (float)(t + 1));
  const float lr = lr0 * (t > total_steps * 3 / 4 ? 0.2f : (t > total_steps / 2 ? 0.5f : 1.0f));
  for (int i = threadIdx.x; i < kParams; i += blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    g[i] = 0.f;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    *step = t + 1;
    loss[1] = loss[0];
    loss[0] = 0.f;
  }
}

// ---- inversion ---------------------------------------------------------------
// One warp per splitter j: the bin holding sample rank q = n j / S from the
// cumulative counts; for a heavy bin also its sub-cell; then the remaining
// bits decoded from the network: with the interval [lo, lo + P) of the
// within-cell fraction covered by the current prefix, bit i is 0 when the
// target u < lo + P * P(x_i = 0 | prefix).  Lane l holds hidden units l and
// l + 32; sums run over their inputs in index order.  The splitter is the
// first key of the next 48-bit cell.
template <class T>
__global__ void __launch_bounds__(256) k_invert(const float* __restrict__ params, const unsigned* __restrict__ cum,
                                                const int* __restrict__ heavy_idx, const unsigned* __restrict__ sub,
                                                const int* __restrict__ heavy2_idx, const unsigned* __restrict__ sub2,
                                                uint32_t n, uint32_t S, uint32_t key_bits, T* __restrict__ spl) {
  extern __shared__ float P[];  // W1 as [input][hidden], W2 as [input][output]; the rest as given
  for (int i = threadIdx.x; i < kParams; i += blockDim.x) {
    int at = i;
    if (i < oB1) at = oW1 + (i % kIn) * kH + i / kIn;                                   // W1[j][i] -> [i][j]
    else if (i >= oW2 && i < oB2) at = oW2 + ((i - oW2) % kH) * kH + (i - oW2) / kH;   // W2[k][j] -> [j][k]
    P[at] = params[i];
  }
  __syncthreads();
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t j = (blockIdx.x * blockDim.x + threadIdx.x) / 32 + 1;
  if (j >= S) return;
  const double q = (double)n * j / S;  // sample rank at the cut
  uint32_t lo_b = 0, hi_b = (1u << kBinBits) - 1;
  while (lo_b < hi_b) {  // first bin whose inclusive cumulative count exceeds q
    const uint32_t mid = (lo_b + hi_b) >> 1;
    if ((double)cum[mid] > q) hi_b = mid;
    else lo_b = mid + 1;
  }
  const uint32_t b = lo_b;
  double below = b ? cum[b - 1] : 0.0, mass = (double)cum[b] - below;
  uint64_t v = (uint64_t)b << (kIn - kBinBits);
  int first = kB0;
  const int h = heavy_idx[b];
  if (h >= 0 && mass > 0) {
    const unsigned* c = sub + (size_t)h * kSubCells;
    const double r = q - below;
    uint32_t a = 0, e = kSubCells - 1;
    while (a < e) {
      const uint32_t mid = (a + e) >> 1;
      if ((double)c[mid] > r) e = mid;
      else a = mid + 1;
    }
    const double sb = a ? c[a - 1] : 0.0;
    below += sb;
    mass = (double)c[a] - sb;
    v |= (uint64_t)a << (kIn - kBinBits - kSubBits);
    first = kB0 + kSubBits;
    const int h2 = heavy2_idx[(size_t)h * kSubCells + a];
    if (h2 >= 0 && mass > 0) {  // a heavy sub-cell: its next 8 bits from counts too
      const unsigned* c2 = sub2 + (size_t)h2 * kSubCells;
      const double r2 = q - below;
      uint32_t a2 = 0, e2 = kSubCells - 1;
      while (a2 < e2) {
        const uint32_t mid = (a2 + e2) >> 1;
        if ((double)c2[mid] > r2) e2 = mid;
        else a2 = mid + 1;
      }
      const double sb2 = a2 ? c2[a2 - 1] : 0.0;
      below += sb2;
      mass = (double)c2[a2] - sb2;
      v |= (uint64_t)a2 << (kIn - kBinBits - 2 * kSubBits);
      first = kB0 + 2 * kSubBits;
    }
  }
  const double u = mass > 0 ? (q - below) / mass : 1.0;
  double lo = 0.0, width = 1.0;
  for (int i = first; i < kIn; ++i) {
    // forward pass of the prefix v (bits below i are zero and unseen by output i)
    float a0 = P[oB1 + lane], a1 = P[oB1 + lane + 32];
    for (int x = 0; x < w1_inputs((int)lane + 32) && x < i; ++x) {
      const float xi = bit_of(v, x);
      if (x < w1_inputs((int)lane)) a0 += P[oW1 + x * kH + lane] * xi;
      a1 += P[oW1 + x * kH + lane + 32] * xi;
    }
    const float h0 = a0 > 0.f ? a0 : 0.f, h1 = a1 > 0.f ? a1 : 0.f;
    float c0 = P[oB2 + lane], c1 = P[oB2 + lane + 32];
    for (int x = 0; x < 32; ++x) {
      const float hv = __shfl_sync(0xffffffffu, h0, x);
      if (x < w2_inputs((int)lane)) c0 += P[oW2 + x * kH + lane] * hv;
      c1 += P[oW2 + x * kH + lane + 32] * hv;  // every first-layer unit x < 32 is below lane + 32's limit
    }
    for (int x = 0; x < 32; ++x) {
      const float hv = __shfl_sync(0xffffffffu, h1, x);
      if (x + 32 < w2_inputs((int)lane + 32)) c1 += P[oW2 + (x + 32) * kH + lane + 32] * hv;
    }
    const float r0 = c0 > 0.f ? c0 : 0.f, r1 = c1 > 0.f ? c1 : 0.f;
    const int o = i - kB0;
    float y = 0.f;
    for (int x = 0; x < 32; ++x) {
      const float a = __shfl_sync(0xffffffffu, r0, x);
      if (x < w3_inputs(o)) y += P[oW3 + o * kH + x] * a;
    }
    for (int x = 0; x < 32; ++x) {
      const float a = __shfl_sync(0xffffffffu, r1, x);
      if (x + 32 < w3_inputs(o)) y += P[oW3 + o * kH + x + 32] * a;
    }
    y += P[oB3 + o];
    const double p0 = width * (1.0 / (1.0 + exp((double)y)));  // P(bit 0) share of the interval
    if (u >= lo + p0) {
      v |= 1ull << (kIn - 1 - i);
      lo += p0;
      width -= p0;
    } else {
      width = p0;
    }
  }
  if (lane != 0) return;
  const uint64_t cell = v + 1;  // first cell above
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
  int sms = 152;
  int dev = 0;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const uint32_t grid = std::min<uint32_t>((n + 255) / 256, 4 * (uint32_t)std::max(sms, 1));
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

namespace {

uint32_t coprime_stride(uint32_t n) {
  auto gcd = [](uint32_t a, uint32_t b) {
    while (b) {
      const uint32_t t = a % b;
      a = b;
      b = t;
    }
    return a;
  };
  uint32_t stride = 2654435761u % n;
  if (stride == 0) stride = 1;
  while (gcd(stride, n) != 1) stride++;
  return stride;
}

// Initial parameters (fixed seed): He-scaled normal weights for the hidden
// layers, small output weights, zero biases; masked weights are zero and stay
// zero (their gradients are never formed).
std::vector<float> initial_params() {
  std::vector<float> p(kParams, 0.f);
  uint64_t st = 0x2545F4914F6CDD1Dull;
  auto uni = [&]() {
    st = st * 6364136223846793005ull + 1442695040888963407ull;
    return ((double)(st >> 11) + 0.5) / 9007199254740992.0;
  };
  auto normal = [&]() { return std::sqrt(-2.0 * std::log(uni())) * std::cos(6.283185307179586 * uni()); };
  for (int i = 0; i < oB1; ++i) p[oW1 + i] = (float)(normal() * std::sqrt(2.0 / kIn));
  for (int i = 0; i < kH * kH; ++i) p[oW2 + i] = (float)(normal() * std::sqrt(2.0 / kH));
  for (int i = 0; i < kOut * kH; ++i) p[oW3 + i] = (float)(normal() * 0.01);
  for (int i = 0; i < kParams; ++i)
    if (!param_live(i)) p[i] = 0.f;
  return p;
}

int ensure_training_buffers(MlpModel* m) {
  if (m->params) return 0;
  if (cudaMalloc(&m->params, kParams * sizeof(float)) != cudaSuccess) return 1;
  if (cudaMalloc(&m->grads, kParams * sizeof(float)) != cudaSuccess) return 1;
  if (cudaMalloc(&m->m, kParams * sizeof(float)) != cudaSuccess) return 1;
  if (cudaMalloc(&m->v, kParams * sizeof(float)) != cudaSuccess) return 1;
  if (cudaMalloc(&m->loss, 2 * sizeof(float)) != cudaSuccess) return 1;
  if (cudaMalloc(&m->step, sizeof(unsigned)) != cudaSuccess) return 1;
  return 0;
}

// kStepsPerGraph training steps (forward/backward + Adam each) captured as a
// graph on the model's own stream, for a sample of n views.
int capture_steps(MlpModel* m, uint32_t n) {
  if (m->graph && m->graph_n == n) return 0;
  if (m->graph) {
    cudaGraphExecDestroy(m->graph);
    m->graph = nullptr;
  }
  if (!m->cap_stream && cudaStreamCreateWithFlags(&m->cap_stream, cudaStreamNonBlocking) != cudaSuccess) return 1;
  const uint32_t batch = std::min(kBatch, n);
  const uint32_t stride = coprime_stride(n);
  cudaFuncSetAttribute(k_fwd_bwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kFbSmem);
  cudaGraph_t g = nullptr;
  if (cudaStreamBeginCapture(m->cap_stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return 1;
  for (int i = 0; i < kStepsPerGraph; ++i) {
    k_fwd_bwd<<<(batch + kB - 1) / kB, kB, kFbSmem, m->cap_stream>>>(m->params, m->views, nullptr, m->step, n,
                                                                      stride, batch, m->grads, m->loss);
    k_adam<<<1, 1024, 0, m->cap_stream>>>(m->params, m->grads, m->m, m->v, m->step, m->loss, kTrainSteps, kLr);
  }
  if (cudaStreamEndCapture(m->cap_stream, &g) != cudaSuccess) return 1;
  const cudaError_t e = cudaGraphInstantiate(&m->graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    m->graph = nullptr;
    return 1;
  }
  m->graph_n = n;
  return 0;
}

// Trains from the initial parameters on the n views; returns the number of
// graph launches + setup copies, or -1 on failure.
int train(MlpModel* m, uint32_t n, cudaStream_t s, uint32_t timeout_ms, float* final_loss) {
  if (ensure_training_buffers(m) || capture_steps(m, n)) return -1;
  const std::vector<float> p = initial_params();
  cudaMemcpyAsync(m->params, p.data(), kParams * sizeof(float), cudaMemcpyHostToDevice, s);
  cudaMemsetAsync(m->grads, 0, kParams * sizeof(float), s);
  cudaMemsetAsync(m->m, 0, kParams * sizeof(float), s);
  cudaMemsetAsync(m->v, 0, kParams * sizeof(float), s);
  cudaMemsetAsync(m->loss, 0, 2 * sizeof(float), s);
  cudaMemsetAsync(m->step, 0, sizeof(unsigned), s);
  int launches = 0;
  for (int i = 0; i < kTrainSteps; i += kStepsPerGraph) {
    if (cudaGraphLaunch(m->graph, s) != cudaSuccess) return -1;
    launches++;
  }
  float l[2] = {0.f, 0.f};
  cudaMemcpyAsync(l, m->loss, sizeof l, cudaMemcpyDeviceToHost, s);
  if (bounded_sync(s, timeout_ms)) return -1;
  if (final_loss) *final_loss = l[1];
  return launches;
}

}  // namespace

template <class T>
int mlp_splitters(MlpModel* m, const T* d_sample, uint32_t n, uint32_t key_bits, uint32_t S, T* d_spl,
                  cudaStream_t s, uint32_t timeout_ms, MlpReport* rep) {
  *rep = MlpReport{};
  rep->pred_imbalance = 1e30;
  if (!m || n < 4 * S || n < 1024) return 0;  // too few samples to learn from
  // ---- stage 1: bin counts and heavy bins' sub-cell counts of the sample
  const uint32_t heavy_cap = 8 * S + 8;  // cells above an eighth of a tile: at most 8 S of them per level
  if (!m->hist && cudaMalloc(&m->hist, sizeof(unsigned) << kBinBits) != cudaSuccess) return 1;
  if (!m->heavy_idx && cudaMalloc(&m->heavy_idx, sizeof(int) << kBinBits) != cudaSuccess) return 1;
  if (!m->nheavy && cudaMalloc(&m->nheavy, 2 * sizeof(unsigned)) != cudaSuccess) return 1;
  if (m->sub_cap < heavy_cap) {
    cudaFree(m->sub);
    cudaFree(m->sub2);
    cudaFree(m->heavy2_idx);
    m->sub = m->sub2 = nullptr;
    m->heavy2_idx = nullptr;
    m->sub_cap = 0;
    if (cudaMalloc(&m->sub, (size_t)heavy_cap * kSubCells * sizeof(unsigned)) != cudaSuccess ||
        cudaMalloc(&m->sub2, (size_t)heavy_cap * kSubCells * sizeof(unsigned)) != cudaSuccess ||
        cudaMalloc(&m->heavy2_idx, (size_t)heavy_cap * kSubCells * sizeof(int)) != cudaSuccess)
      return 1;
    m->sub_cap = heavy_cap;
  }
  if (m->views_cap < n) {
    cudaFree(m->views);
    m->views = nullptr;
    m->views_cap = 0;
    if (m->graph) {  // the captured steps read the old buffer
      cudaGraphExecDestroy(m->graph);
      m->graph = nullptr;
    }
    if (cudaMalloc(&m->views, (size_t)n * sizeof(uint64_t)) != cudaSuccess) return 1;
    m->views_cap = n;
  }
  int sms = 152, dev = 0;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const uint32_t grid = std::min<uint32_t>((n + 255) / 256, 8 * (uint32_t)std::max(sms, 1));
  cudaMemsetAsync(m->hist, 0, sizeof(unsigned) << kBinBits, s);
  cudaMemsetAsync(m->nheavy, 0, 2 * sizeof(unsigned), s);
  cudaMemsetAsync(m->sub, 0, (size_t)heavy_cap * kSubCells * sizeof(unsigned), s);
  cudaMemsetAsync(m->sub2, 0, (size_t)heavy_cap * kSubCells * sizeof(unsigned), s);
  k_views<T><<<grid, 256, 0, s>>>(d_sample, n, key_bits, m->views, m->hist);
  // cells holding more than an eighth of a tile's share of the sample are
  // counted one level (8 bits) deeper, twice at most
  const unsigned thr = (unsigned)((double)n / (8.0 * S));
  k_heavy<<<(1u << kBinBits) / 256, 256, 0, s>>>(m->hist, thr, heavy_cap, m->heavy_idx, m->nheavy);
  k_sub_hist<<<grid, 256, 0, s>>>(m->views, n, m->heavy_idx, m->sub);
  k_heavy2<<<(uint32_t)(((size_t)heavy_cap * kSubCells + 255) / 256), 256, 0, s>>>(
      m->sub, m->nheavy, heavy_cap, thr, m->heavy2_idx, m->nheavy + 1);
  k_sub2_hist<<<grid, 256, 0, s>>>(m->views, n, m->heavy_idx, m->heavy2_idx, m->sub2);
  k_sub_cum<<<(heavy_cap * 32 + 255) / 256, 256, 0, s>>>(m->sub, m->nheavy, heavy_cap);
  k_sub_cum<<<(heavy_cap * 32 + 255) / 256, 256, 0, s>>>(m->sub2, m->nheavy + 1, heavy_cap);
  k_cum<<<1, 1024, 0, s>>>(m->hist);
  rep->launches += 8;
  const size_t smem = kParams * sizeof(float);
  cudaFuncSetAttribute(k_invert<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  const uint32_t inv_grid = (uint32_t)(((size_t)(S - 1) * 32 + 255) / 256);
  if (m->trained && m->trained_key_bits == key_bits) {
    // the bit conditionals learned on an earlier segment, over this sample's counts
    k_invert<T><<<inv_grid, 256, smem, s>>>(m->params, m->hist, m->heavy_idx, m->sub, m->heavy2_idx, m->sub2, n, S,
                                            key_bits, d_spl);
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
  // ---- stage 2: train the network on every sample key
  const int tl = train(m, n, s, timeout_ms, &rep->loss);
  if (tl < 0) return 1;
  rep->launches += tl;
  k_invert<T><<<inv_grid, 256, smem, s>>>(m->params, m->hist, m->heavy_idx, m->sub, m->heavy2_idx, m->sub2, n, S,
                                            key_bits, d_spl);
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

}  // namespace kite

// ---- test hooks (C ABI, no counterpart in the reference) -------------------------
// One forward + backward of the learned-CDF network over n keys' 48-bit views
// against a given parameter vector (masked weights must be zero), so tests
// can check the hand-written gradients against a CPU float64 reference.
// Returns 0, or -1 on a CUDA failure.
extern "C" int kite_mlp_grad_check(const float* params, const uint64_t* views, uint32_t n, float* grads_out,
                                   float* loss_out) {
  using namespace kite;
  float *dp = nullptr, *dg = nullptr, *dl = nullptr;
  uint64_t* dv = nullptr;
  uint32_t* di = nullptr;
  cudaError_t e = cudaMalloc(&dp, kParams * 4);
  if (e == cudaSuccess) e = cudaMalloc(&dv, (size_t)n * 8);
  if (e == cudaSuccess) e = cudaMalloc(&dg, kParams * 4);
  if (e == cudaSuccess) e = cudaMalloc(&dl, 4);
  if (e == cudaSuccess) e = cudaMalloc(&di, (size_t)n * 4);
  if (e == cudaSuccess) {
    std::vector<uint32_t> id(n);
    for (uint32_t i = 0; i < n; ++i) id[i] = i;
    cudaMemcpy(dp, params, kParams * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(dv, views, (size_t)n * 8, cudaMemcpyHostToDevice);
    cudaMemcpy(di, id.data(), (size_t)n * 4, cudaMemcpyHostToDevice);
    cudaMemset(dg, 0, kParams * 4);
    cudaMemset(dl, 0, 4);
    cudaFuncSetAttribute(k_fwd_bwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kFbSmem);
    k_fwd_bwd<<<(n + kB - 1) / kB, kB, kFbSmem>>>(dp, dv, di, nullptr, n, 1, n, dg, dl);
    e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(grads_out, dg, kParams * 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(loss_out, dl, 4, cudaMemcpyDeviceToHost);
  }
  cudaFree(dp);
  cudaFree(dv);
  cudaFree(dg);
  cudaFree(dl);
  cudaFree(di);
  return e == cudaSuccess ? 0 : -1;
}

extern "C" int kite_mlp_param_count(void) { return kite::kParams; }
extern "C" int kite_mlp_input_count(void) { return kite::kIn; }

// Fits the learned CDF to n 48-bit key views (host array) for S tiles, as
// the count path does (stage-1 counts, training, inversion), and returns the
// trained parameters and the S - 1 splitter cells (48-bit views of the
// splitters) so tests can check the inversion against a CPU evaluation of the
// same network.  Returns 0, or -1 on failure.
extern "C" int kite_mlp_fit(const uint64_t* views, uint32_t n, uint32_t S, float* params_out, uint64_t* cells_out,
                            double* pred_imbalance) {
  using namespace kite;
  MlpModel* m = mlp_create();
  uint64_t *dv = nullptr, *ds = nullptr;
  int rc = -1;
  if (cudaMalloc(&dv, (size_t)n * 8) == cudaSuccess && cudaMalloc(&ds, (size_t)S * 8) == cudaSuccess &&
      cudaMemcpy(dv, views, (size_t)n * 8, cudaMemcpyHostToDevice) == cudaSuccess) {
    MlpReport rep;
    if (mlp_splitters<uint64_t>(m, dv, n, 48, S, ds, nullptr, 600000, &rep) == 0 &&
        cudaDeviceSynchronize() == cudaSuccess &&
        cudaMemcpy(params_out, m->params, kParams * 4, cudaMemcpyDeviceToHost) == cudaSuccess &&
        cudaMemcpy(cells_out, ds, (size_t)(S - 1) * 8, cudaMemcpyDeviceToHost) == cudaSuccess) {
      if (pred_imbalance) *pred_imbalance = rep.pred_imbalance;
      rc = 0;
    }
  }
  cudaFree(dv);
  cudaFree(ds);
  mlp_destroy(m);
  return rc;
}
