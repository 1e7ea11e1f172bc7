// Device-wide exclusive prefix sum over u64 (reduce-then-scan, no inter-CTA
// waiting).  Used for bucket/tile region offsets and newline prefixes.
#include <chrono>
#include <thread>

#include "kite_internal.h"

namespace kite {

static constexpr int kScanThreads = 256;
static constexpr int kScanItems = 16;
static constexpr size_t kScanTile = (size_t)kScanThreads * kScanItems;

__global__ void __launch_bounds__(kScanThreads) k_scan_reduce(const unsigned long long* __restrict__ in, size_t n,
                                                              unsigned long long* __restrict__ sums) {
  __shared__ unsigned long long sm[34];
  const size_t base = blockIdx.x * kScanTile;
  unsigned long long acc = 0;
  for (int i = 0; i < kScanItems; ++i) {
    const size_t idx = base + (size_t)i * kScanThreads + threadIdx.x;
    if (idx < n) acc += in[idx];
  }
  unsigned long long total;
  block_exclusive_scan<kScanThreads, unsigned long long>(acc, sm, &total);
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// Scans one tile per CTA in blocked order and adds the tile offset.
__global__ void __launch_bounds__(kScanThreads) k_scan_tile(const unsigned long long* __restrict__ in,
                                                            unsigned long long* __restrict__ out, size_t n,
                                                            const unsigned long long* __restrict__ offs) {
  __shared__ unsigned long long sm[34];
  const size_t base = blockIdx.x * kScanTile + (size_t)threadIdx.x * kScanItems;
  unsigned long long v[kScanItems];
  unsigned long long acc = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    v[i] = (base + i < n) ? in[base + i] : 0ull;
    acc += v[i];
  }
  unsigned long long total;
  unsigned long long pre = block_exclusive_scan<kScanThreads, unsigned long long>(acc, sm, &total);
  if (offs) pre += offs[blockIdx.x];
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    if (base + i < n) out[base + i] = pre;
    pre += v[i];
  }
}

// ---- column offsets of a row-major u32 count matrix (rows = blocks) ----
static constexpr uint32_t kColRows = 256;  // rows per group

// Column sums of each group of kColRows rows.
__global__ void __launch_bounds__(256) k_col_group_sums(const unsigned* __restrict__ m, uint32_t rows, uint32_t cols,
                                                        unsigned long long* __restrict__ gsum) {
  const uint32_t g = blockIdx.y;
  const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cols) return;
  const uint32_t r0 = g * kColRows, r1 = min(rows, r0 + kColRows);
  unsigned long long acc = 0;
  for (uint32_t r = r0; r < r1; ++r) acc += m[(size_t)r * cols + c];
  gsum[(size_t)g * cols + c] = acc;
}

// Exclusive scan of the group sums down each column; column totals.
__global__ void __launch_bounds__(256) k_col_group_scan(unsigned long long* __restrict__ gsum, uint32_t groups,
                                                        uint32_t cols, unsigned long long* __restrict__ total) {
  const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cols) return;
  unsigned long long acc = 0;
  // 16 groups loaded before any is rewritten, so the loads are in flight together
  constexpr uint32_t kB = 16;
  for (uint32_t g = 0; g < groups; g += kB) {
    unsigned long long v[kB];
#pragma unroll
    for (uint32_t j = 0; j < kB; ++j) v[j] = g + j < groups ? gsum[(size_t)(g + j) * cols + c] : 0ull;
#pragma unroll
    for (uint32_t j = 0; j < kB; ++j)
      if (g + j < groups) {
        gsum[(size_t)(g + j) * cols + c] = acc;
        acc += v[j];
      }
  }
  total[c] = acc;
}

// Rows of each group turned into running column offsets, in place.
__global__ void __launch_bounds__(256) k_col_offsets(unsigned* __restrict__ m, uint32_t rows, uint32_t cols,
                                                     const unsigned long long* __restrict__ gsum) {
  const uint32_t g = blockIdx.y;
  const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cols) return;
  const uint32_t r0 = g * kColRows, r1 = min(rows, r0 + kColRows);
  unsigned acc = (unsigned)gsum[(size_t)g * cols + c];
  // 16 rows loaded before any is rewritten, so the loads are in flight together
  constexpr uint32_t kB = 16;
  for (uint32_t r = r0; r < r1; r += kB) {
    unsigned v[kB];
#pragma unroll
    for (uint32_t j = 0; j < kB; ++j) v[j] = r + j < r1 ? m[(size_t)(r + j) * cols + c] : 0u;
#pragma unroll
    for (uint32_t j = 0; j < kB; ++j)
      if (r + j < r1) {
        m[(size_t)(r + j) * cols + c] = acc;
        acc += v[j];
      }
  }
}

int count_matrix_offsets(unsigned* m, uint32_t rows, uint32_t cols, unsigned long long* gsum,
                         unsigned long long* col_total, cudaStream_t s) {
  if (rows == 0 || cols == 0) return 0;
  const uint32_t groups = (rows + kColRows - 1) / kColRows;
  const dim3 grid((cols + 255) / 256, groups);
  k_col_group_sums<<<grid, 256, 0, s>>>(m, rows, cols, gsum);
  k_col_group_scan<<<(cols + 255) / 256, 256, 0, s>>>(gsum, groups, cols, col_total);
  k_col_offsets<<<grid, 256, 0, s>>>(m, rows, cols, gsum);
  return 3;
}

size_t scan_tmp_elems(size_t n) {
  size_t tiles = (n + kScanTile - 1) / kScanTile;
  if (tiles <= 1) return 1;
  return tiles + scan_tmp_elems(tiles);
}

int exclusive_scan_u64(const unsigned long long* in, unsigned long long* out, size_t n, unsigned long long* tmp,
                       cudaStream_t s) {
  if (n == 0) return 0;
  const size_t tiles = (n + kScanTile - 1) / kScanTile;
  if (tiles == 1) {
    k_scan_tile<<<1, kScanThreads, 0, s>>>(in, out, n, nullptr);
    return 1;
  }
  k_scan_reduce<<<(unsigned)tiles, kScanThreads, 0, s>>>(in, n, tmp);
  const int inner = exclusive_scan_u64(tmp, tmp, tiles, tmp + tiles, s);
  k_scan_tile<<<(unsigned)tiles, kScanThreads, 0, s>>>(in, out, n, tmp);
  return inner + 2;
}

int bounded_sync(cudaStream_t s, uint32_t timeout_ms) {
  cudaEvent_t e;
  if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return -1;
  if (cudaEventRecord(e, s) != cudaSuccess) {
    cudaEventDestroy(e);
    return -1;
  }
  const int rc = bounded_event_wait(e, timeout_ms);
  cudaEventDestroy(e);
  return rc;
}

int bounded_event_wait(cudaEvent_t e, uint32_t timeout_ms) {
  const auto deadline = std::chrono::steady_clock::now() + std::chrono::milliseconds(timeout_ms);
  int rc = 0;
  for (int spins = 0;; ++spins) {
    const cudaError_t q = cudaEventQuery(e);
    if (q == cudaSuccess) break;
    if (q != cudaErrorNotReady) {
      rc = -1;
      break;
    }
    if (std::chrono::steady_clock::now() > deadline) {
      rc = -3;
      break;
    }
    if (spins > 64) std::this_thread::sleep_for(std::chrono::microseconds(50));
  }
  return rc;
}

}  // namespace kite
