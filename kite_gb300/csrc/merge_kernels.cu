// GPU merge (placeholder until the merge kernels land).
#include "merge.h"

namespace kite {

int merge_run(int, uint32_t, const kite_gpu_merge_input*, int, cudaStream_t, uint32_t, kite_gpu_emit_fn, void*,
              std::string* msg, kite_gpu_stats*) {
  *msg = "merge not built yet";
  return KITE_ERR_UNSUPPORTED;
}

}  // namespace kite
