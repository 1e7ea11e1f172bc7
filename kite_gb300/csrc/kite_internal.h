// Internal launch interface between the C-ABI orchestration (kite_gpu.cu) and
// the kernel translation units.  Not part of the public ABI.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "kite_common.cuh"

namespace kite {

// One extraction work block: a byte range of one submitted chunk.
struct BlockDesc {
  uint64_t start;         // first byte (arena offset), 16-byte aligned
  uint64_t end;           // one past the last byte
  uint64_t chunk_start;   // arena offset of the chunk's first byte
  uint32_t first_block;   // index of the chunk's first block
  uint32_t flags;         // bit 1: block of the segment's first chunk (key sample source)
  uint32_t sample;        // sample of a batched count (0 otherwise): its buckets are sample*P .. sample*P+P-1
  uint32_t sample_first;  // index of the sample's first block (blocks of a sample are contiguous)
};

// One chunk's run of extraction blocks (the block descriptors are made on
// the device from these).
struct ChunkSpan {
  uint64_t off, len;      // arena offset and length of the chunk
  uint32_t first_block;   // index of its first block
  uint32_t flags;         // copied to its blocks
  uint32_t sample;        // sample of a batched count
  uint32_t sample_first;  // index of the sample's first block
};

// A key-range tile: the on-chip sort unit.
struct TileDesc {
  uint64_t start;   // key index of the tile's first key
  uint32_t len;     // keys in the tile
  uint32_t bucket;
};

// Per-tile results of the sort + run-length reduction.
template <class T>
struct TileOut {
  T first_key, last_key;
  uint32_t rows;        // unique keys
  uint32_t first_count;
  uint64_t rest_bytes;  // DVLE bytes of rows 1..rows-1 (deltas inside the tile)
};

struct CountTotals {
  unsigned long long reads, bases, kmers, samples;
};

template <class T>
struct ExtractParams {
  const uint8_t* arena;
  const BlockDesc* blocks;
  const unsigned long long* block_nl_excl;  // newlines before each block, counted from its chunk's start
  uint32_t block_base;   // the launch's first block: block index = blockIdx.x + block_base
  uint32_t k;
  uint32_t canonical;
  uint32_t shift;        // 64 - log2(partitions)
  uint32_t partitions;   // per sample; global bucket arrays hold samples * partitions entries
  uint32_t blk_bytes;
  // histogram pass
  unsigned long long* bucket_count;  // [samples * partitions]
  CountTotals* totals;               // [samples]
  T* sample;                         // may be null
  unsigned int* sample_count;
  uint32_t sample_cap;
  uint32_t sample_mask;              // keep positions whose mixed hash & mask == 0
  // per-block bucket counts [blocks][partitions]: the histogram pass writes
  // them (instead of atomics on bucket_count) and, scanned per bucket, they
  // become each block's write offsets inside the bucket regions; null = atomics
  unsigned* blk_counts;
  const unsigned* blk_offs;
  // histogram pass, optional: every block's keys, in block-local order, to
  // keys_stage at a position reserved on stage_counter; blk_keys[2*b] = that
  // position, blk_keys[2*b+1] = the block's key count (null = not written)
  T* keys_stage;
  unsigned long long stage_cap;          // keys keys_stage holds; a block past it writes nothing
  unsigned long long* stage_counter;
  unsigned long long* blk_keys;
  // scatter pass
  const unsigned long long* bucket_off;  // [partitions] region start (key index)
  unsigned long long* bucket_fill;       // [partitions]
  T* keys_out;
  DevStatus* status;
};

// One level of the key-range split.  Region r (a hash bucket, or one coarse
// key range of a bucket) is cut into D <= 256 digits by D-1 of the global
// splitters: spl[spl_first + (r % spl_mod) * spl_region_stride + i * spl_step]
// for i < D-1 (spl_total splitters in all).  Each region is processed in G
// parts.
template <class T>
struct TileSplitParams {
  const T* keys_in;
  T* keys_out;
  const unsigned long long* region_off;    // [R] first key of each region
  const unsigned long long* region_count;  // [R]
  const T* splitters;     // spl_total ascending keys
  uint32_t spl_total;
  uint32_t R;             // regions
  uint32_t D;             // digits per region (2..256)
  uint32_t G;             // parts per region
  uint32_t spl_first, spl_step, spl_mod, spl_region_stride;
  uint32_t key_bits;      // 2k: significant key bits
  unsigned long long* tile_count;       // [R*D*G] (digit-major, part-minor)
  const unsigned long long* tile_off;   // exclusive scan of tile_count
  uint16_t* dig;  // or null; else every key's digit, parallel to keys_in: the histogram writes it, the scatter reads it
  // 0/1: region r's keys are one run at region_off[r].  pieces > 1: keys_in
  // holds `pieces` input pieces one after another, each bucket-major, and
  // region r has one run per piece at region_off[q * R + r] (count
  // region_count[q * R + r]); parts g of the region belong to piece
  // g / (G / pieces).
  uint32_t pieces;
};

// ---- launchers (count_kernels.cu) ----
void launch_make_blocks(const ChunkSpan* spans, uint32_t nspans, uint32_t blk, uint32_t nblocks, BlockDesc* out,
                        cudaStream_t s);
void launch_newline_count(const uint8_t* arena, const BlockDesc* blocks, uint32_t nblocks,
                          unsigned long long* nl_out, cudaStream_t s);
template <class T>
void launch_extract_hist(const ExtractParams<T>& p, uint32_t nblocks, cudaStream_t s);
template <class T>
void launch_extract_scatter(const ExtractParams<T>& p, uint32_t nblocks, cudaStream_t s);
// Scatter of the staged keys of every block into the bucket regions
// (partitions <= 256): keys of block b go to bucket_off[k] + blk_offs[b][k]
// onwards, ranked on chip so that writes are coalesced.
// stage_counter (or null): the launch does nothing when the staging counter
// is above stage_cap (some block's keys were not staged).
template <class T>
void launch_bucket_scatter(const T* keys_stage, const unsigned long long* blk_keys, const unsigned* blk_offs,
                           const BlockDesc* blocks, const unsigned long long* bucket_off, uint32_t partitions,
                           uint32_t shift, uint32_t nblocks, T* keys_out, const unsigned long long* stage_counter,
                           unsigned long long stage_cap, cudaStream_t s);
// One input piece's bucket runs: off[b] = *base + the piece's counts of the
// buckets below b; bucket_count[b] += cnt[b]; then *base += the piece's
// total.  One CTA (partitions <= 1024).
void launch_piece_offsets(const unsigned long long* cnt, uint32_t partitions, unsigned long long* base,
                          unsigned long long* off, unsigned long long* bucket_count, cudaStream_t s);
// Batched count: bucket totals of every (sample, bucket) from the scanned
// count matrix m (rows = blocks, cols = partitions), col_total = column sums.
void launch_sample_bucket_counts(const unsigned* m, const unsigned long long* col_total, const uint32_t* sample_first,
                                 uint32_t samples, uint32_t partitions, uint32_t nblocks,
                                 unsigned long long* bucket_count, cudaStream_t s);
template <class T>
void launch_split_hist(const TileSplitParams<T>& p, cudaStream_t s);
template <class T>
void launch_split_scatter(const TileSplitParams<T>& p, int shape, cudaStream_t s);  // shape 0..3: threads x keys
template <class T>
uint32_t split_scatter_slots(uint32_t D, int shape);  // resident scatter CTAs on the device
void launch_make_tiles(const unsigned long long* off, uint32_t ntiles, uint32_t S, uint32_t G,
                       unsigned long long n_keys, TileDesc* tiles, uint32_t* lens, cudaStream_t s);
void launch_region_bounds(const unsigned long long* off, uint32_t nreg, uint32_t G, unsigned long long n_keys,
                          unsigned long long* roff, unsigned long long* rcnt, cudaStream_t s);
size_t extract_smem_bytes(int key_bytes, uint32_t blk_bytes, uint32_t partitions, bool scatter);

// ---- scan.cu ----
// Exclusive scan of n u64 values (in may equal out).  `tmp` needs
// scan_tmp_elems(n) entries.
size_t scan_tmp_elems(size_t n);
// Returns the number of kernels launched.
int exclusive_scan_u64(const unsigned long long* in, unsigned long long* out, size_t n,
                       unsigned long long* tmp, cudaStream_t s);
// Column sums / offsets of a rows x cols u32 count matrix (row-major):
// after count_matrix_offsets, m[r][c] = sum of m[0..r)[c] (in place) and
// col_total[c] = the column sum.  `gsum` needs ceil(rows/256)*cols u64.
// Column totals must stay below 2^32.  Returns the number of launches.
int count_matrix_offsets(unsigned* m, uint32_t rows, uint32_t cols, unsigned long long* gsum,
                         unsigned long long* col_total, cudaStream_t s);
// Waits for the work queued on s, polling with a deadline: 0 ok, -1 CUDA
// error, -3 timeout.
int bounded_sync(cudaStream_t s, uint32_t timeout_ms);
// Waits for one recorded event: 0, -1 (CUDA error) or -3 (timeout).
int bounded_event_wait(cudaEvent_t e, uint32_t timeout_ms);

// ---- sort_kernels.cu ----
constexpr int kTileThreads = 512;
template <class T> __host__ __device__ constexpr int tile_items() { return sizeof(T) == 8 ? 16 : 8; }
template <class T> __host__ __device__ constexpr uint32_t tile_capacity() { return (uint32_t)(kTileThreads * tile_items<T>()); }

// Key range of every tile: tile t of a bucket holds the keys in
// [spl[t-1], spl[t]) (0 and kmax close the ends), S tiles per bucket; tile
// index of a launch's tile i = tile0 + i.
template <class T>
struct TileRanges {
  const T* spl;
  uint32_t S;
  uint32_t tile0;
  T kmax;
  uint32_t wait_polls;  // bound of the first wait for a tile's bulk load (1: a single non-blocking test)
};

// `fallbacks` (device counters): [0] tiles that took the LSD fallback (plus
// 2^40 for a tile whose bulk load did not complete), [1] rows of the tiles
// above the on-chip capacity (double-capacity and global-memory sorts).
template <class T>
void launch_tile_sort(T* keys, uint32_t* counts, const TileDesc* tiles, uint32_t ntiles, TileOut<T>* out,
                      unsigned long long* fallbacks, TileRanges<T> rg, cudaStream_t s);
// Tiles of tile_capacity < len <= 2 * tile_capacity, listed in ids: the same
// on-chip sort with twice the shared memory (one CTA per SM).  With nids_dev,
// the list's length is on the device and the nids CTAs walk it in turn.
template <class T>
void launch_tile_sort_large(T* keys, uint32_t* counts, const TileDesc* tiles, const uint32_t* ids, uint32_t nids,
                            const unsigned* nids_dev, TileOut<T>* out, unsigned long long* fallbacks,
                            TileRanges<T> rg, cudaStream_t s);
// Oversized tiles (more keys than 2 * tile_capacity): one CTA per tile, LSD
// passes through global memory with `scratch` (>= largest tile keys); with
// nbig_dev as above; sort_stats[1] gains the rows they make.
template <class T>
void launch_big_tile_sort(T* keys, uint32_t* counts, T* scratch, const TileDesc* tiles, const uint32_t* big_ids,
                          uint32_t nbig, const unsigned* nbig_dev, TileOut<T>* out, DevStatus* st,
                          unsigned long long* sort_stats, cudaStream_t s);
// Per bucket group, the tiles above capacity (lists and counts on the
// device) and the tile statistics; see k_tile_lists.
void launch_tile_lists(const uint32_t* lens, uint32_t ntiles, uint32_t S, const uint32_t* gb, uint32_t NG,
                       uint32_t cap, uint32_t* ids, uint32_t* ids2, unsigned* cnt, unsigned long long* stats,
                       unsigned long long* range, cudaStream_t s);

// ---- encode_kernels.cu ----
struct BucketMeta {
  unsigned long long rows;
  unsigned long long bytes;
  unsigned long long byte_off;
  unsigned long long kmin_lo, kmin_hi, kmax_lo, kmax_hi;
};
template <class T>
void launch_tile_link(const TileOut<T>* tout, uint32_t P, uint32_t S, unsigned long long* tile_boff, T* tile_prev,
                      BucketMeta* meta, cudaStream_t s);
template <class T>
void launch_encode(const T* keys, const uint32_t* counts, const TileDesc* tiles, const TileOut<T>* tout,
                   const unsigned long long* tile_boff, const T* tile_prev, const BucketMeta* meta, uint32_t ntiles,
                   uint8_t* out, unsigned long long out_cap, DevStatus* st, cudaStream_t s);
// Same, with variable tile ranges per bucket: tiles of b are [tile_first[b], tile_first[b+1]).
template <class T>
void launch_tile_link_ranges(const TileOut<T>* tout, uint32_t P, const uint32_t* tile_first,
                             unsigned long long* tile_boff, T* tile_prev, BucketMeta* meta, cudaStream_t s);
// host_mirror: optional device address of mapped pinned host memory that
// receives a copy of the P finished records
void launch_bucket_offsets(BucketMeta* meta, uint32_t P, BucketMeta* host_mirror, cudaStream_t s);

}  // namespace kite
