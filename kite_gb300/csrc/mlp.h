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

// Trains the CDF on the sampled keys and writes S-1 splitters.  *used is set
// to false (and nothing is written) when the predicted max/mean tile load on
// the sample exceeds `bound`: the caller then falls back to the sampled
// histogram splitters.
template <class T>
int mlp_splitters(MlpModel* m, const T* d_sample, uint32_t n, uint32_t key_bits, uint32_t S, T* d_spl, double bound,
                  cudaStream_t s, bool* used);

}  // namespace kite
