/*
 * kite_gpu.h — C ABI of the GB300 exact k-mer counting library
 * (libkite_gpu.so, hand-written sm_103a CUDA kernels).
 *
 * The reference (jiehua1995/Kite v0.7.5) is a monolithic Rust binary with no
 * FFI.  These entry points replace its internal counting and merging seams,
 * and keep their argument meaning:
 *
 *   kite_gpu_count_submit   <- CountWorker::process_chunk(&[u8])
 *                              src/count/worker.rs:196 (a chunk starts at a
 *                              FASTQ record boundary, src/count/bgzf.rs:109-121;
 *                              a chunk not starting with '@' contributes
 *                              nothing, src/count/worker.rs:217)
 *   kite_gpu_count_finish   <- CountWorker::flush_all src/count/worker.rs:284
 *                              + flush_bucket :296-449 (sort, RLE, DVLE)
 *   kite_gpu_emit_fn        <- ConcurrentKiteWriter::append_chunk
 *                              src/count/writer.rs:285-348 (same fields)
 *   kite_gpu_merge          <- build_merge_partition_chunk
 *                              src/merge/mod.rs:198-214 over all partitions
 *                              (load_partition_counts, per-input filter,
 *                              merge_vectors_total, serialize_partition_chunk
 *                              src/kiteops/mod.rs:433-859)
 *   kite_gpu_histo          <- run_histo src/histo/mod.rs:16-169 (one input)
 *   kite_gpu_query          <- run_query src/query/mod.rs:15-96 (many keys)
 *   kite_gpu_dump           <- run_dump src/dump/mod.rs:183-520 through
 *                              stream_partition_slabs src/dump/merge.rs:282-428
 *                              (LoserTreeMerger src/dump/loser_tree.rs:141-175,
 *                              decode_kmer_any src/dump/decoder.rs:27-50)
 *
 * Conventions: every function returns 0 (KITE_OK) or a negative KITE_ERR_*
 * code; no exception crosses the ABI; a context owns all of its device memory
 * and streams; one host thread drives one context; every host-side wait is
 * bounded by cfg.timeout_ms and returns KITE_ERR_TIMEOUT instead of hanging.
 * There is no CPU fallback: without a usable CUDA device kite_gpu_open fails.
 */
#ifndef KITE_GPU_H
#define KITE_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define KITE_GPU_ABI_VERSION 2  /* 2: kite_gpu_stats.input_pieces */

enum {
  KITE_OK = 0,
  KITE_ERR_CUDA = -1,           /* a CUDA runtime call failed */
  KITE_ERR_OOM = -2,            /* device or pinned allocation failed */
  KITE_ERR_TIMEOUT = -3,        /* a bounded wait ran out */
  KITE_ERR_BAD_INPUT = -4,      /* invalid argument or malformed payload */
  KITE_ERR_COUNT_OVERFLOW = -5, /* merged count exceeds u32 (merge) */
  KITE_ERR_UNSUPPORTED = -6,    /* k > 64, unknown codec, ... */
  KITE_ERR_DEVICE = -7,         /* a kernel reported a failure status */
  KITE_ERR_CALLBACK = -8,       /* the emit callback returned non-zero */
  KITE_ERR_STATE = -9           /* call out of order */
};

enum { KITE_SPLIT_AUTO = 0, KITE_SPLIT_SAMPLED = 1, KITE_SPLIT_LEARNED = 2 };

/* Codec bits of a chunk (src/format/run_block.rs:1-3). */
enum { KITE_CODEC_RAW = 1, KITE_CODEC_DVLE = 2, KITE_CODEC_ZSTD = 4 };

typedef struct kite_gpu_ctx kite_gpu_ctx;

typedef struct {
  int device;                /* CUDA device ordinal */
  int k;                     /* 1..64 (u64 keys for k <= 31, u128 for 32..64) */
  int canonical;             /* 0 or 1 */
  uint32_t partitions;       /* power of two >= 2: hash buckets of the .kite file */
  int splitter_mode;         /* KITE_SPLIT_* : how key-range tiles are cut */
  double imbalance_bound;    /* learned splitters fall back above this max/mean (0 = 1.10) */
  uint64_t arena_bytes;      /* FASTQ bytes held on device before a flush (0 = auto) */
  uint32_t timeout_ms;       /* bound on every host-side wait (0 = 600000) */
  void* stream;              /* optional cudaStream_t to run on (NULL = own stream) */
  uint32_t samples;          /* batched count: samples per segment (0 = 1); see kite_gpu_count_submit_sample */
  double tile_fill;          /* target tile load as a fraction of on-chip capacity (0 = 0.85) */
  int scatter_shape;         /* key-range split scatter launch shape 0..3 (0 = 256 threads x 8 keys) */
  uint32_t tile_wait_polls;  /* bound of the tile sort's first wait for a tile's bulk load (0 = 2^18 polls);
                                1 gives up unless the copy has already landed (tests of the timeout path:
                                the count then returns KITE_ERR_TIMEOUT) */
} kite_gpu_cfg;

/* One emitted chunk: the arguments of ConcurrentKiteWriter::append_chunk. */
typedef struct {
  uint32_t partition_id;
  uint32_t codec;            /* KITE_CODEC_DVLE for u64/u128 keys */
  uint64_t row_count;
  uint64_t raw_bytes;        /* payload length (fast mode: no zstd) */
  uint64_t key_min_lo[2];    /* u128 key_min_lo as (low 64, high 64) */
  uint64_t key_min_hi[2];    /* u128 key_min_hi (0 for k <= 64) */
  uint64_t key_max_lo[2];
  uint64_t key_max_hi[2];
} kite_chunk_meta;

/* Called once per non-empty partition, in ascending partition order.  `data`
 * is valid only during the call.  Return 0 to continue, non-zero to abort
 * (the API call then returns KITE_ERR_CALLBACK). */
typedef int (*kite_gpu_emit_fn)(void* user, const kite_chunk_meta* meta, const uint8_t* data, size_t len);

typedef struct {
  uint64_t reads, bases, kmers;      /* the summary line fields (src/count/mod.rs:598-612) */
  uint64_t rows, payload_bytes;      /* unique (key,count) rows and DVLE bytes of the last finish */
  uint32_t tiles, big_tiles, tiles_per_bucket, segments;
  double tile_imbalance;             /* max / mean keys per non-empty tile */
  int splitter_used;                 /* KITE_SPLIT_SAMPLED or KITE_SPLIT_LEARNED */
  double stage_ms[12];               /* count: [0..7] device time per stage (events: newline count, histogram
                                        pass, bucket scatter, split, tile sort, large tiles, encode, payload
                                        copy to the host); host wall time [8] until the bucket counts are back
                                        (the copy in), [9] split + sort + encode, [10] the last payload copies
                                        after that, [11] the emit calls.  Merge: see kite_gpu_merge */
  uint64_t h2d_bytes, d2h_bytes;
  uint64_t kernel_launches;          /* kernels this library launched in the last finish */
  double mlp_loss, mlp_pred_imbalance, hist_pred_imbalance; /* learned-splitter diagnostics */
  double range_imbalance;            /* max / mean keys per key range (summed over partitions) */
  uint64_t sort_fallbacks;           /* tiles whose on-chip sort fell back to LSD passes (a large bin of distinct keys) */
  uint32_t split_levels;             /* key-range split passes over the keys (0, 1 or 2) */
  uint32_t staged_scatter;           /* 1: keys staged by the histogram pass, then a ranked bucket scatter */
  uint32_t mlp_reused;               /* 1: the learned CDF of an earlier segment was kept (no training) */
  uint64_t big_tile_keys;            /* keys in tiles above the on-chip capacity */
  uint64_t big_tile_rows;            /* unique rows those tiles reduced to */
  uint32_t input_pieces;             /* host chunks: runs of chunks whose bucket scatter ran while later chunks
                                        were still copying in (1 = one scatter after the last chunk) */
} kite_gpu_stats;

/* Merge input: one .kite file's partition table, with payloads in host memory
 * (e.g. an mmap of the file).  Chunks of partition p are chunk_meta[first[p]
 * .. first[p]+count[p]) and their payload bytes start at base + file_offset. */
typedef struct {
  const uint8_t* base;               /* file image */
  uint64_t base_len;
  const uint64_t* chunk_offset;      /* per chunk: file offset of the payload */
  const uint64_t* chunk_len;         /* per chunk: encoded bytes */
  const uint64_t* chunk_rows;        /* per chunk: row count */
  const uint32_t* chunk_codec;       /* per chunk: codec bits */
  const uint64_t* part_first;        /* per partition: first chunk index */
  const uint64_t* part_count;        /* per partition: number of chunks */
  int has_min, has_max;              /* header count filters (src/format/header.rs:30-31) */
  uint32_t min_count, max_count;
} kite_gpu_merge_input;

int kite_gpu_abi_version(void);
int kite_gpu_device_count(void);

int kite_gpu_open(const kite_gpu_cfg* cfg, kite_gpu_ctx** out);
void kite_gpu_close(kite_gpu_ctx* ctx);
const char* kite_gpu_last_error(const kite_gpu_ctx* ctx);

/* Page-locked host buffers for submit (faster, truly asynchronous copies). */
void* kite_gpu_alloc_pinned(size_t bytes);
void kite_gpu_free_pinned(void* p);

/* Queue one FASTQ chunk (host memory).  Returns a ticket >= 0; the buffer may
 * be reused after kite_gpu_wait_ticket(ticket) returns.  Returns
 * KITE_ERR_STATE if the device arena is full: call kite_gpu_count_finish to
 * flush the counted segment, then submit again. */
int64_t kite_gpu_count_submit(kite_gpu_ctx* ctx, const uint8_t* fastq, size_t len);
int kite_gpu_wait_ticket(kite_gpu_ctx* ctx, int64_t ticket);

/* Register chunks that already live in device memory (no copy).  Each chunk
 * start must be 16-byte aligned and 16 readable bytes must follow the last
 * chunk.  Used by benchmarks that time the kernels on HBM-resident input. */
int kite_gpu_count_submit_device(kite_gpu_ctx* ctx, const uint8_t* d_fastq, size_t len);

/* Batched count (no counterpart in the reference, which runs one input per
 * process): with cfg.samples = S > 1, chunks are queued for sample s < S and
 * every sample of the segment is counted by one launch sequence.  Keys of
 * sample s fall in partitions s*cfg.partitions + p (p = the reference's
 * partition of the key), so the finish emits each sample's partitions as one
 * contiguous range, ascending; kite_gpu_sample_totals gives each sample's
 * reads, bases and k-mers of the last finish.  The plain submit calls queue
 * for sample 0. */
int64_t kite_gpu_count_submit_sample(kite_gpu_ctx* ctx, uint32_t sample, const uint8_t* fastq, size_t len);
int kite_gpu_count_submit_device_sample(kite_gpu_ctx* ctx, uint32_t sample, const uint8_t* d_fastq, size_t len);
int kite_gpu_sample_totals(kite_gpu_ctx* ctx, uint32_t sample, uint64_t totals[3]);

/* Count everything submitted since the last finish: emit one DVLE chunk per
 * non-empty partition (ascending), then reset for the next segment.  With
 * emit == NULL the results stay on the device (kite_gpu_result_*). */
int kite_gpu_count_finish(kite_gpu_ctx* ctx, kite_gpu_emit_fn emit, void* user);

/* Results of the last finish kept on device: partition metadata and the
 * device address of its payload. */
int kite_gpu_result_partition(kite_gpu_ctx* ctx, uint32_t partition, kite_chunk_meta* meta,
                              const uint8_t** device_payload, size_t* len);

/* K-way merge of n inputs (same k, canonical, partitions and key width):
 * per-input header filter before summing, u64 sums, u32 overflow is an error
 * (KITE_ERR_COUNT_OVERFLOW, message names the key), one DVLE chunk per
 * non-empty partition, emitted in partition order (after every partition has
 * been merged, so an overflow emits nothing).  The context keeps the device
 * buffers of merge, dump, histo and query between calls (grown when a call
 * needs more, released by kite_gpu_close). */
int kite_gpu_merge(kite_gpu_ctx* ctx, const kite_gpu_merge_input* inputs, int n, kite_gpu_emit_fn emit,
                   void* user);

/* `kite dump` of one .kite input (same k, canonical, partitions and key width
 * as the context): per partition, its chunks merged by key with saturating
 * u32 sums of equal keys, the header min/max applied to the summed count,
 * then one line "<kmer>\t<count>\n" per key in ascending key order (k bases,
 * 2-bit codes most significant first as A, C, G, T).  emit is called once per
 * partition that has lines, in ascending partition order, with meta
 * {partition_id, codec 0, row_count = lines, raw_bytes = TSV bytes, key_min /
 * key_max = its first and last key} and the TSV bytes (valid during the
 * call).  stats.stage_ms[0..5]: decode kernels, tile planning, merge,
 * formatting, copy to the host, copy of the input in (which the decode
 * overlaps); [6..9] the host wall time of the planning's phases (splitters,
 * first cut, bisection, tile lists). */
int kite_gpu_dump(kite_gpu_ctx* ctx, const kite_gpu_merge_input* input, kite_gpu_emit_fn emit, void* user);

/* Called once per count value with the number of keys that have it. */
typedef int (*kite_gpu_histo_fn)(void* user, uint64_t count, uint64_t keys);

/* `kite histo` of one .kite input: per partition its chunks summed by key in
 * u64 (saturating; load_partition_counts src/kiteops/mod.rs:433-473), the
 * header min/max applied to that sum (apply_reader_filter_to_rows :103-108),
 * then the frequency of every count; emit is called for each count present,
 * ascending. */
int kite_gpu_histo(kite_gpu_ctx* ctx, const kite_gpu_merge_input* input, kite_gpu_histo_fn emit, void* user);

/* `kite query` for n keys at once (already encoded, canonical where the
 * database is: keys[2i] low and keys[2i+1] high 64 bits, high 0 for k <= 31):
 * counts[i] = the u64 sum of key i over its partition's chunks, 0 when absent
 * (no header filter; the caller reports it, as run_query does).  Only the
 * partitions the keys fall in are decoded. */
int kite_gpu_query(kite_gpu_ctx* ctx, const kite_gpu_merge_input* input, const uint64_t* keys, size_t n,
                   uint64_t* counts);

int kite_gpu_get_stats(kite_gpu_ctx* ctx, kite_gpu_stats* out);

/* Device-side timing of the last count/merge, summed per kernel family. */
int kite_gpu_synchronize(kite_gpu_ctx* ctx);

/* Largest FASTQ chunk kite_gpu_count_rows_noalloc accepts. */
#define KITE_NOALLOC_MAX_BYTES (512u * 1024u)

/* Counts one small FASTQ chunk that already lives in device memory, without
 * allocating anything: no context, no cudaMalloc / cudaFree, no pinned host
 * buffer.  It has no counterpart in the reference.  It is meant for callers
 * that cannot allocate device memory at the moment they count: a process
 * whose framework already reserved the device's memory for its own pool, or
 * a loop counting small read batches between other GPU work that must not
 * take the device-wide synchronisation of cudaMalloc / cudaFree.
 *
 * Same counting rules as kite_gpu_count_submit + kite_gpu_count_finish on one
 * chunk (a chunk not starting with '@' counts nothing).  Results go to the
 * caller's device arrays, grouped by partition in ascending order, keys
 * ascending inside a partition: d_keys gets the keys (8-byte little-endian
 * words for k <= 31, 16-byte words for k >= 32; aligned to the word size),
 * d_counts their counts, d_partition_rows[partitions] the rows of each
 * partition; totals[4] (host) gets reads, bases, k-mers and rows.
 *
 * Working memory is one fixed array of about 21 MiB in this library's device
 * data, one per device, which every call on that device shares: calls that
 * overlap on the GPU race and corrupt each other's results, so serialise them
 * (and after KITE_ERR_TIMEOUT, wait for `stream` before the next call).  The
 * first call on a device looks the array up (cudaGetSymbolAddress, with that
 * device current); make it before any stream capture starts.  Runs on
 * `stream` (NULL = the default stream) of `device`, restores the caller's
 * current device, and returns when the work is done (at most timeout_ms;
 * 0 = 600000).  Errors: KITE_ERR_UNSUPPORTED when len exceeds
 * KITE_NOALLOC_MAX_BYTES (nothing runs); KITE_ERR_BAD_INPUT for invalid
 * arguments, or when the rows exceed max_rows (totals[3] then gives the rows
 * needed). */
int kite_gpu_count_rows_noalloc(int device, int k, int canonical, uint32_t partitions, const uint8_t* d_fastq,
                                size_t len, void* d_keys, uint32_t* d_counts, uint64_t max_rows,
                                uint32_t* d_partition_rows, uint64_t* totals, void* stream, uint32_t timeout_ms);

#ifdef __cplusplus
}
#endif

#endif /* KITE_GPU_H */
