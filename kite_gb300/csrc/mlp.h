// Learned CDF over the k-mer key space (FP32 MLP trained on the GPU by
// hand-written forward/backward kernels).  Internal.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "kite_common.cuh"

namespace kite {

struct MlpModel;
MlpModel* mlp_create();
void mlp_destroy(MlpModel* m);

struct MlpReport {
  int launches = 0;
  float loss = 0.f;
  double pred_imbalance = 0.0;  // max/mean tile load of the sample under the learned splitters
  bool reused = false;          // the model trained on an earlier segment was kept (no training)
};

// Trains the CDF on the sampled keys and writes S-1 ascending splitters to
// d_spl.  A model already trained in this context (same key width) is tried
// first on the new sample and kept when its predicted imbalance is within 5%
// of what it reached when trained; otherwise it is retrained.  Returns 0 on
// success (report filled), non-zero on a CUDA failure or timeout.  Fewer than
// 1024 samples (or 4 per tile): nothing is trained and report->pred_imbalance
// is +inf.
template <class T>
int mlp_splitters(MlpModel* m, const T* d_sample, uint32_t n, uint32_t key_bits, uint32_t S, T* d_spl,
                  cudaStream_t s, uint32_t timeout_ms, MlpReport* report);

// max/mean tile load of `n` sample keys under S-1 splitters (bounded wait).
template <class T>
int predict_imbalance(MlpModel* m, const T* d_sample, uint32_t n, const T* d_spl, uint32_t S, cudaStream_t s,
                      uint32_t timeout_ms, double* out);

}  // namespace kite
