// GPU k-way merge of .kite inputs (kite merge).  Internal.
#pragma once

#include <cstdint>
#include <functional>
#include <string>
#include <cuda_runtime.h>

#include "kite_gpu.h"

namespace kite {

// Pinned host staging of at least the given bytes (nullptr if it cannot be had).
using StagingFn = std::function<uint8_t*(size_t)>;

// k selects the key width (u64 for k <= 31, else u128) and the splitter key
// bits.  dump: one input, TSV lines per partition instead of DVLE chunks,
// copied out through `staging` in groups of whole partitions.
int merge_run(int k, uint32_t partitions, const kite_gpu_merge_input* inputs, int n, cudaStream_t s,
              uint32_t timeout_ms, bool dump, kite_gpu_emit_fn emit, void* user, std::string* msg,
              kite_gpu_stats* st, const StagingFn& staging = nullptr);

}  // namespace kite
