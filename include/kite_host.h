/*
 * kite_host.h — host-side C ABI of libkite_host.so: the .kite (KX2) writer
 * and reader, the count planner, FASTQ ingest and the TSV dump.  These are
 * the pieces around the GPU counting path that make it a drop-in for the
 * reference's `kite count` / `kite merge` / `kite dump`.
 *
 *   kite_writer_*           <- ConcurrentKiteWriter src/count/writer.rs:51-495
 *                              (staging per partition, high/low watermark drain,
 *                              finalize: chunk index, partition table, footer,
 *                              header rewrite).  kite_writer_emit has the
 *                              kite_gpu_emit_fn signature.
 *   kite_derive_plan        <- derive_heuristic_plan src/count/mod.rs:624-864
 *   kite_parse_memory_spec  <- parse_memory_spec src/runtime.rs:6-54
 *   kite_count_passes_filter<- count_passes_filter src/kiteops/mod.rs:44-56
 *   kite_reader_*           <- KiteReader::open src/dump/reader.rs:43-155,
 *                              run_data_for_decode :162-186 (zstd chunks)
 *   kite_zstd_chunk         <- CountWorker::flush_bucket's zstd "if smaller"
 *                              src/count/worker.rs:340-374, :452-501
 *   kite_dump_partition     <- stream_partition_slabs src/dump/merge.rs:282-428
 *   kite_input_*            <- detect_compression src/count/reader.rs:22-51,
 *                              Plain/GzipChunkedReader src/count/decompress.rs:36-138
 */
#ifndef KITE_HOST_H
#define KITE_HOST_H

#include <stddef.h>
#include <stdint.h>

#include "kite_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- small helpers ------------------------------------------------------ */
int64_t kite_parse_memory_spec(const char* spec); /* bytes, or -1 (message in kite_host_last_error) */
int64_t kite_resolve_memory_limit(const char* spec_or_null);
int kite_count_passes_filter(uint64_t count, int has_min, uint32_t min_count, int has_max, uint32_t max_count);
const char* kite_host_last_error(void);

/* ---- planner ------------------------------------------------------------- */
enum { KITE_INPUT_PLAIN = 0, KITE_INPUT_GZIP = 1, KITE_INPUT_BGZF = 2 };
typedef struct {
  uint64_t partitions, chunk_size_bytes, staging_bytes, worker_threads, local_flush_bytes, decomp_threads,
      writer_lanes, queue_depth;
  double avg_read_len;
} kite_plan;
int kite_derive_plan(uint64_t input_bytes, double avg_read_len, int compression, int k, uint64_t partitions,
                     uint64_t total_threads, uint64_t memory_bytes, int64_t buffer_mb, uint64_t chunk_kmers,
                     kite_plan* out);
uint64_t kite_suggest_write_lanes(uint64_t workers);

/* ---- writer -------------------------------------------------------------- */
typedef struct kite_writer kite_writer;
typedef struct {
  int k, canonical;
  uint32_t partitions;
  uint16_t key_width, codec_mask;
  int has_min, has_max;
  uint32_t min_count, max_count;
} kite_header_info;
/* path NULL: keep the image in memory (kite_writer_image). */
kite_writer* kite_writer_open(const char* path, const kite_header_info* h, uint64_t staging_bytes,
                              uint64_t write_lanes);
int kite_writer_append(kite_writer* w, const kite_chunk_meta* meta, const uint8_t* data, size_t len);
int kite_writer_emit(void* w, const kite_chunk_meta* meta, const uint8_t* data, size_t len);
int kite_writer_worker_drain(kite_writer* w); /* CountWorker::flush_all's drain loop */
int kite_writer_finalize(kite_writer* w, uint64_t* total_chunks, uint64_t* total_rows);
const uint8_t* kite_writer_image(kite_writer* w, size_t* len);
void kite_writer_close(kite_writer* w);

/* ---- reader + dump ------------------------------------------------------- */
typedef struct kite_reader kite_reader;
kite_reader* kite_reader_open(const char* path);
kite_reader* kite_reader_open_image(const uint8_t* data, size_t len); /* copies */
void kite_reader_close(kite_reader* r);
int kite_reader_header(const kite_reader* r, kite_header_info* h, uint64_t* total_chunks, uint64_t* total_rows);
/* Fills a kite_gpu_merge_input that points into the reader's image. */
int kite_reader_merge_input(const kite_reader* r, kite_gpu_merge_input* mi);
/* Appends the TSV lines of one partition ("<kmer>\t<count>\n", segments
 * summed with saturating u32, header filter applied). Returns bytes or -1. */
int64_t kite_dump_partition(const kite_reader* r, uint32_t partition, char** buf, size_t* cap, size_t* len);

/* ---- zstd "if smaller" (count --mode balanced | compact) ------------------ */
/* CountWorker::flush_bucket src/count/worker.rs:340-374 with its heuristics
 * compression_level_for / min_compression_input_bytes /
 * min_compression_savings_bytes :452-501: one chunk's DVLE payload is
 * zstd-compressed at base_level (balanced 2, compact 5, raised by the
 * heuristics, at most 6) when it is large enough, and the compressed bytes
 * are kept only when they save enough.  Returns the compressed length written
 * to out (the chunk then carries codec | KITE_CODEC_ZSTD, raw_bytes = len),
 * 0 to keep the payload as it is, -1 on error.  out needs
 * kite_zstd_bound(len) bytes.  zstd is the system's libzstd.so.1, loaded at
 * run time; kite_zstd_available says whether it loaded.  Readers decompress
 * zstd chunks when a file is opened (kite_reader_*). */
int kite_zstd_available(void);
size_t kite_zstd_bound(size_t len);
int64_t kite_zstd_chunk(int k, int base_level, const kite_chunk_meta* meta, const uint8_t* payload, size_t len,
                        uint8_t* out, size_t cap);

/* ---- input --------------------------------------------------------------- */
int kite_detect_compression(const char* path); /* KITE_INPUT_* or -1 */
typedef struct kite_input kite_input;
kite_input* kite_input_open(const char* path, uint64_t chunk_size);
/* Next FASTQ-aligned chunk into dst (capacity >= chunk_size + carry); returns
 * its length, 0 at end, -1 on error. */
int64_t kite_input_next(kite_input* in, uint8_t* dst, size_t cap);
uint64_t kite_input_max_chunk(const kite_input* in);
/* Inflate threads of a BGZF input and of a multi-member gzip input (its
 * members inflate in parallel; default half the host's cores).  Plain input
 * and single-member gzip ignore it. */
int kite_input_set_threads(kite_input* in, unsigned threads);
void kite_input_close(kite_input* in);
double kite_sample_avg_read_len(const char* path, int compression);

/* ---- synthetic inputs ------------------------------------------------------ */
/* Seeded FASTQ generator (same record shape as kite_gb300.synth): reads of a
 * fixed length sampled from `genome` (2-bit codes), with substitutions, N and
 * reverse complements; multithreaded, deterministic for a given seed.
 * Returns bytes written (n_reads * record length). */
int64_t kite_synth_reads(const uint8_t* genome, uint64_t genome_len, uint64_t n_reads, uint32_t read_len,
                         double sub_rate, double n_rate, double revcomp_frac, uint64_t seed, uint64_t first_index,
                         uint8_t* out, uint64_t cap, int threads);
/* The same with read lengths uniform in [len_lo, len_hi], records back to back. */
int64_t kite_synth_reads_var(const uint8_t* genome, uint64_t genome_len, uint64_t n_reads, uint32_t len_lo,
                             uint32_t len_hi, double sub_rate, double n_rate, double revcomp_frac, uint64_t seed,
                             uint64_t first_index, uint8_t* out, uint64_t cap, int threads);

#ifdef __cplusplus
}
#endif

#endif /* KITE_HOST_H */
