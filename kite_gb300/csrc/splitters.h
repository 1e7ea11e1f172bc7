// Splitter producers (sampled histogram, learned CDF).  Internal.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "kite_common.cuh"

namespace kite {

// S-1 ascending splitters from a 2^16-bin histogram of the sampled keys'
// top bits (key_bits = 2k).  With no sample, splitters cut [0, 2^key_bits)
// uniformly.
// Returns the number of kernels launched.
template <class T>
int compute_hist_splitters(const T* d_sample, uint32_t nsample, uint32_t key_bits, uint32_t S, T* d_spl,
                           unsigned* d_hist, cudaStream_t s);

}  // namespace kite
