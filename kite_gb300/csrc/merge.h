// GPU k-way merge of .kite inputs (kite merge).  Internal.
#pragma once

#include <cstdint>
#include <string>
#include <cuda_runtime.h>

#include "kite_gpu.h"

namespace kite {

// k selects the key width (u64 for k <= 31, else u128) and the splitter key
// bits.  dump: one input, TSV lines per partition instead of DVLE chunks.
int merge_run(int k, uint32_t partitions, const kite_gpu_merge_input* inputs, int n, cudaStream_t s,
              uint32_t timeout_ms, bool dump, kite_gpu_emit_fn emit, void* user, std::string* msg,
              kite_gpu_stats* st);

}  // namespace kite
