// GPU k-way merge of .kite inputs (kite merge).  Internal.
#pragma once

#include <cstdint>
#include <functional>
#include <string>
#include <cuda_runtime.h>

#include "kite_gpu.h"
#include "mlp.h"

namespace kite {

// Pinned host staging of at least the given bytes (nullptr if it cannot be had).
using StagingFn = std::function<uint8_t*(size_t)>;

// Modes of merge_run (the merge kernel's kModeMerge / kModeDump / kModeHisto / kModeRows).
enum : int { kMergeModeMerge = 0, kMergeModeDump = 1, kMergeModeHisto = 2, kMergeModeQuery = 3 };

// Device buffers of the merge path kept by a context across calls (grown,
// never shrunk), so repeated merges, dumps and queries do not pay for
// allocating and freeing gigabytes every call.
struct MergePoolSlot {
  void* p = nullptr;
  size_t cap = 0;
};
struct MergePool {
  static constexpr int kSlots = 32;
  MergePoolSlot slot[kSlots];
  MergePoolSlot host;  // pinned host memory: the tile stream lists on their way to the device
  MergePool() = default;
  MergePool(const MergePool&) = delete;
  MergePool& operator=(const MergePool&) = delete;
  ~MergePool() {
    for (auto& s : slot) cudaFree(s.p);
    if (host.p) cudaFreeHost(host.p);
  }
};

// Inputs and outputs of the histo and query modes.
struct MergeExtra {
  kite_gpu_histo_fn histo = nullptr;  // histo: called per count in ascending order
  void* user = nullptr;
  const uint64_t* keys = nullptr;     // query: (lo, hi) words per key
  const uint32_t* parts = nullptr;    // query: partition of each key
  size_t nq = 0;
  uint64_t* counts_out = nullptr;     // query: u64 sum per key, 0 when absent
  MlpModel* mlp = nullptr;            // learned CDF for the tile cut (null: sampled histogram only)
  int splitter_mode = 0;              // KITE_SPLIT_*: AUTO keeps whichever predicts the lower imbalance
  MergePool* pool = nullptr;          // the context's buffers (null: allocated and freed by the call)
};

// k selects the key width (u64 for k <= 31, else u128) and the splitter key
// bits.  Dump: one input, TSV lines per partition instead of DVLE chunks,
// copied out through `staging` in groups of whole partitions.  Histo and
// query: one input, results through `ex`.
int merge_run(int k, uint32_t partitions, const kite_gpu_merge_input* inputs, int n, cudaStream_t s,
              uint32_t timeout_ms, int mode, kite_gpu_emit_fn emit, void* user, std::string* msg,
              kite_gpu_stats* st, const StagingFn& staging = nullptr, const MergeExtra* ex = nullptr);

}  // namespace kite
