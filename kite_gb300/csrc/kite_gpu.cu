// C-ABI implementation of libkite_gpu.so: context, device arena, the staged
// count pipeline and result emission.  See include/kite_gpu.h for the
// contract and the reference seams each entry point replaces.
//
// Count pipeline of one segment (everything submitted since the last finish):
//   K1  newline count per 16 KiB block + scan        -> line phase at each block
//   K2  extract (histogram pass): rolling canonical k-mers, hash-bucket counts,
//       reads/bases/kmers, key sample from the segment's first chunk
//   K3  extract (scatter pass): k-mers into their hash-bucket regions
//   K3b tile split: each bucket cut into key-range tiles by splitters
//   K4  tile sort + run-length reduction on chip (oversized tiles: K4b)
//   K7  DVLE encode of every bucket's rows into one payload per partition
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <cmath>
#include <vector>

#include "kite_gpu.h"
#include "kite_internal.h"
#include "merge.h"
#include "splitters.h"
#include "mlp.h"

using namespace kite;

namespace {

struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
  cudaError_t ensure(size_t bytes) {
    if (bytes <= cap) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    size_t want = bytes + bytes / 8 + 256;
    cudaError_t e = cudaMalloc(&p, want);
    if (e != cudaSuccess) {
      p = nullptr;
      return e;
    }
    cap = want;
    return cudaSuccess;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
  template <class U> U* as() const { return static_cast<U*>(p); }
};

struct HostBuf {
  void* p = nullptr;
  size_t cap = 0;
  cudaError_t ensure(size_t bytes) {
    if (bytes <= cap) return cudaSuccess;
    if (p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
    size_t want = bytes + bytes / 8 + 256;
    cudaError_t e = cudaMallocHost(&p, want);
    if (e != cudaSuccess) {
      p = nullptr;
      return e;
    }
    cap = want;
    return cudaSuccess;
  }
  void release() {
    if (p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
  }
  template <class U> U* as() const { return static_cast<U*>(p); }
};

struct Chunk {
  uint64_t off;  // offset from the arena base
  uint64_t len;
  uint32_t sample;  // batched count: the sample it belongs to
};

enum Stage { ST_LINES = 0, ST_HIST, ST_SCATTER, ST_SPLIT, ST_SORT, ST_BIG, ST_ENCODE, ST_D2H, ST_COUNT };

// Bucket groups of the sort / encode / copy-out pipeline.
constexpr uint32_t kSortGroups = 8;
// Host chunks: runs of chunks whose bucket scatter runs while later chunks copy in.
constexpr uint32_t kMaxPieces = 8;

}  // namespace

struct kite_gpu_ctx {
  kite_gpu_cfg cfg{};
  std::string err;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  cudaStream_t copy_stream = nullptr;
  cudaStream_t aux_stream = nullptr;   // highest priority: splitters beside the bucket scatter, encodes beside the next sort
  MergePool merge_pool;                // merge / dump / histo / query device buffers, kept across calls
  cudaEvent_t spl_ready = nullptr;

  // FASTQ arena (host submissions are copied here)
  DevBuf arena;
  uint64_t arena_used = 0;
  const uint8_t* ext_base = nullptr;  // device submissions: caller-owned base
  bool ext_mode = false;
  std::vector<Chunk> chunks;
  std::vector<cudaEvent_t> ticket_events;
  int64_t next_ticket = 0;

  // scratch
  DevBuf blocks, nl, scan_tmp, bucket_count, bucket_off, bucket_fill, totals, status;
  DevBuf keys_a, keys_b, counts, sample, sample_count, splitters, splitters2, hist16;
  DevBuf tile_count, tile_off, tile_fill, tiles, big_ids, tile_out, tile_boff, tile_prev, meta, out;
  DevBuf lvl_count, lvl_off, reg_off, reg_cnt, sort_stats, blk_mat, blk_gsum, blk_keys, stage_ctr;
  DevBuf col_total, sample_first, spans, digits, tile_lists, piece_off, piece_cnt, piece_base;
  HostBuf h_blocks, h_small, h_tiles, h_out, h_meta, h_dump;
  std::vector<cudaEvent_t> ev;   // stage events
  std::vector<cudaEvent_t> gev;  // sort / encode / copy-out events, 8 per bucket group

  // results of the last finish
  std::vector<BucketMeta> res_meta;
  uint64_t res_bytes = 0;
  bool res_on_host = false;  // the payload was copied to h_out while encoding
  std::vector<uint64_t> sample_totals;  // reads, bases, k-mers per sample of the last finish
  kite_gpu_stats stats{};
  MlpModel* mlp = nullptr;
};

namespace {

int fail(kite_gpu_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

#define KCU(call)                                                                       \
  do {                                                                                  \
    cudaError_t _e = (call);                                                            \
    if (_e != cudaSuccess)                                                              \
      return fail(ctx, _e == cudaErrorMemoryAllocation ? KITE_ERR_OOM : KITE_ERR_CUDA, \
                  std::string(#call) + ": " + cudaGetErrorString(_e));                  \
  } while (0)

// Bounded wait for all work queued on `s`.
// Waits (bounded by cfg.timeout_ms) for a recorded event.
int wait_event(kite_gpu_ctx* ctx, cudaEvent_t e) {
  const auto deadline = std::chrono::steady_clock::now() + std::chrono::milliseconds(ctx->cfg.timeout_ms);
  int spins = 0;
  for (;;) {
    cudaError_t q = cudaEventQuery(e);
    if (q == cudaSuccess) return KITE_OK;
    if (q != cudaErrorNotReady) return fail(ctx, KITE_ERR_CUDA, std::string("stream wait: ") + cudaGetErrorString(q));
    if (std::chrono::steady_clock::now() > deadline)
      return fail(ctx, KITE_ERR_TIMEOUT, "device work did not finish within timeout_ms");
    if (++spins > 64) std::this_thread::sleep_for(std::chrono::microseconds(50));
  }
}

int wait_stream(kite_gpu_ctx* ctx, cudaStream_t s) {
  cudaEvent_t e;
  KCU(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  KCU(cudaEventRecord(e, s));
  const int rc = wait_event(ctx, e);
  cudaEventDestroy(e);
  return rc;
}

int check_status(kite_gpu_ctx* ctx, const char* where) {
  DevStatus st{};
  KCU(cudaMemcpyAsync(&st, ctx->status.p, sizeof st, cudaMemcpyDeviceToHost, ctx->stream));
  int rc = wait_stream(ctx, ctx->stream);
  if (rc) return rc;
  if (st.code != KITE_DEV_OK) {
    char buf[256];
    snprintf(buf, sizeof buf, "%s: device status %u (%u, %u, %u)", where, st.code, st.a, st.b, st.c);
    return fail(ctx, KITE_ERR_DEVICE, buf);
  }
  return KITE_OK;
}

uint32_t log2u(uint64_t v) {
  uint32_t r = 0;
  while ((1ull << r) < v) r++;
  return r;
}

const uint8_t* arena_base(kite_gpu_ctx* ctx) {
  return ctx->ext_mode ? ctx->ext_base : ctx->arena.as<const uint8_t>();
}

void reset_segment(kite_gpu_ctx* ctx) {
  ctx->chunks.clear();
  ctx->arena_used = 0;
  ctx->ext_mode = false;
  ctx->ext_base = nullptr;
}

// to_host: copy each bucket group's payload to the pinned host buffer as soon
// as it is encoded.
template <class T>
int run_count(kite_gpu_ctx* ctx, bool to_host) {
  cudaStream_t s = ctx->stream;
  const uint32_t P = ctx->cfg.partitions;                  // per sample
  const uint32_t NS = ctx->cfg.samples ? ctx->cfg.samples : 1;
  const uint32_t PT = P * NS;                               // buckets of the segment (sample-major)
  const uint32_t k = (uint32_t)ctx->cfg.k;
  const uint32_t CAP = tile_capacity<T>();
  auto& st = ctx->stats;
  const uint64_t prev_h2d = st.h2d_bytes, prev_d2h = st.d2h_bytes;
  const uint32_t prev_segments = st.segments;
  std::memset(&st, 0, sizeof st);
  st.hist_pred_imbalance = -1.0;
  st.h2d_bytes = prev_h2d;
  st.d2h_bytes = prev_d2h;
  st.segments = prev_segments + 1;
  // nothing of this count starts before the side stream's work of an earlier
  // call (which an error return may have left in flight) is done
  KCU(cudaEventRecord(ctx->spl_ready, ctx->aux_stream));
  KCU(cudaStreamWaitEvent(s, ctx->spl_ready, 0));
  for (auto& e : ctx->ev) cudaEventRecord(e, s);  // reset so unused stages read 0
  KCU(cudaEventRecord(ctx->ev[0], s));
  // host wall phases: [8] until the bucket counts are on the host (the copy
  // in), [9] the split, sort and encode queued and done on the stream, [10]
  // the last payload copies after that; [11] (finish) the emit calls
  using clk = std::chrono::steady_clock;
  const auto wall0 = clk::now();
  auto wall_ms = [](clk::time_point a, clk::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
  };

  // ---- blocks -------------------------------------------------------------
  uint32_t blk = 16384;  // 256 threads x 64 bytes
  while (blk > 1024 && extract_smem_bytes(sizeof(T), blk, P, true) > 200 * 1024) blk >>= 1;
  if (extract_smem_bytes(sizeof(T), blk, P, true) > 220 * 1024)
    return fail(ctx, KITE_ERR_UNSUPPORTED, "partition count too large for the extraction kernel");
  // blocks in sample order (chunks of one sample keep their submission order)
  std::vector<size_t> order(ctx->chunks.size());
  for (size_t c = 0; c < order.size(); ++c) order[c] = c;
  std::stable_sort(order.begin(), order.end(),
                   [&](size_t a, size_t b) { return ctx->chunks[a].sample < ctx->chunks[b].sample; });
  std::vector<uint32_t> sample_first(NS + 1, 0xFFFFFFFFu);
  struct Span {
    size_t chunk;
    uint32_t first, n;
  };
  std::vector<Span> spans;  // each chunk's blocks, in block order
  std::vector<ChunkSpan> cspans;
  uint64_t chunk0_len = 0;
  uint32_t nblocks = 0;
  for (size_t c : order) {
    const Chunk& ch = ctx->chunks[c];
    if (ch.len == 0) continue;
    const uint32_t first = nblocks;
    if (first == 0) chunk0_len = ch.len;
    if (sample_first[ch.sample] == 0xFFFFFFFFu) sample_first[ch.sample] = first;
    const uint32_t nb = (uint32_t)((ch.len + blk - 1) / blk);
    cspans.push_back(ChunkSpan{ch.off, ch.len, first, first == 0 ? 2u : 0u, ch.sample, sample_first[ch.sample]});
    spans.push_back(Span{c, first, nb});
    nblocks += nb;
  }
  // samples without blocks start where the next one does
  sample_first[NS] = nblocks;
  for (int t = (int)NS - 1; t >= 0; --t)
    if (sample_first[t] == 0xFFFFFFFFu) sample_first[t] = sample_first[t + 1];
  ctx->sample_totals.assign((size_t)NS * 3, 0);
  if (nblocks == 0) {
    ctx->res_meta.assign(PT, BucketMeta{});
    ctx->res_bytes = 0;
    return KITE_OK;
  }
  KCU(ctx->h_blocks.ensure(cspans.size() * sizeof(ChunkSpan)));
  std::memcpy(ctx->h_blocks.p, cspans.data(), cspans.size() * sizeof(ChunkSpan));
  KCU(ctx->spans.ensure(cspans.size() * sizeof(ChunkSpan)));
  KCU(cudaMemcpyAsync(ctx->spans.p, ctx->h_blocks.p, cspans.size() * sizeof(ChunkSpan), cudaMemcpyHostToDevice, s));
  KCU(ctx->blocks.ensure((size_t)nblocks * sizeof(BlockDesc)));
  launch_make_blocks(ctx->spans.as<ChunkSpan>(), (uint32_t)cspans.size(), blk, nblocks, ctx->blocks.as<BlockDesc>(), s);
  st.kernel_launches += 1;
  KCU(ctx->nl.ensure((size_t)nblocks * 8));
  KCU(ctx->scan_tmp.ensure(scan_tmp_elems(std::max<size_t>((size_t)nblocks, (size_t)PT * 4096)) * 8 + 64));
  KCU(ctx->status.ensure(sizeof(DevStatus)));
  KCU(cudaMemsetAsync(ctx->status.p, 0, sizeof(DevStatus), s));
  const uint8_t* base = arena_base(ctx);

  // ---- K1 newline count + K2 histogram pass -------------------------------
  const uint32_t sample_cap = 1u << 22;
  KCU(ctx->bucket_count.ensure((size_t)PT * 8));
  KCU(ctx->totals.ensure(NS * sizeof(CountTotals)));
  KCU(ctx->sample.ensure((size_t)sample_cap * sizeof(T)));
  KCU(ctx->sample_count.ensure(8));
  KCU(cudaMemsetAsync(ctx->bucket_count.p, 0, (size_t)PT * 8, s));
  KCU(cudaMemsetAsync(ctx->totals.p, 0, NS * sizeof(CountTotals), s));
  KCU(cudaMemsetAsync(ctx->sample_count.p, 0, 8, s));
  // keep ~2^22 of the first chunk's k-mer positions (about one k-mer per 2.5 bytes)
  uint64_t est = std::max<uint64_t>(chunk0_len * 2 / 5, 1);
  uint32_t mask = 0;
  while ((est >> log2u((uint64_t)mask + 1)) > sample_cap && mask < (1u << 30)) mask = mask * 2 + 1;
  ExtractParams<T> ep{};
  ep.arena = base;
  ep.blocks = ctx->blocks.as<BlockDesc>();
  ep.block_nl_excl = ctx->nl.as<unsigned long long>();
  ep.k = k;
  ep.canonical = ctx->cfg.canonical ? 1u : 0u;
  ep.shift = 64 - log2u(P);
  ep.partitions = P;
  ep.blk_bytes = blk;
  ep.bucket_count = ctx->bucket_count.as<unsigned long long>();
  ep.totals = ctx->totals.as<CountTotals>();
  ep.sample = ctx->sample.as<T>();
  ep.sample_count = ctx->sample_count.as<unsigned int>();
  ep.sample_cap = sample_cap;
  ep.sample_mask = mask;
  ep.status = ctx->status.as<DevStatus>();
  // per-block bucket counts in a blocks x buckets matrix (no contended
  // atomics), scanned per bucket into each block's write offsets
  const uint64_t groups = ((uint64_t)nblocks + 255) / 256;
  const bool use_matrix = (uint64_t)nblocks * P * 4 <= (2ull << 30) && groups <= 65535;
  if (use_matrix) {
    KCU(ctx->blk_mat.ensure((size_t)nblocks * P * 4));
    KCU(ctx->blk_gsum.ensure((size_t)groups * P * 8));
    ep.blk_counts = ctx->blk_mat.as<unsigned>();
  }
  // u64 keys and at most 256 partitions: the histogram pass also stages every
  // block's keys (capacity: half a key per FASTQ byte; more than that and the
  // extraction scatter runs instead), then an on-chip ranked scatter moves
  // them to the bucket regions
  uint64_t fastq_bytes = 0;
  for (const Chunk& ch : ctx->chunks) fastq_bytes += ch.len;
  const bool stage_keys = use_matrix && P <= 256;
  const uint64_t stage_cap = fastq_bytes / 2 + 1024;
  if (stage_keys) {
    const uint64_t cap = stage_cap;
    KCU(ctx->keys_b.ensure(cap * sizeof(T)));
    KCU(ctx->blk_keys.ensure((size_t)nblocks * 16));
    KCU(ctx->stage_ctr.ensure(8));
    KCU(cudaMemsetAsync(ctx->stage_ctr.p, 0, 8, s));
    ep.keys_stage = ctx->keys_b.as<T>();
    ep.stage_cap = cap;
    ep.stage_counter = ctx->stage_ctr.as<unsigned long long>();
    ep.blk_keys = ctx->blk_keys.as<unsigned long long>();
  }
  // Host chunks: each chunk's newline count, scan and histogram pass start
  // as soon as that chunk's copy has landed, so the copies of later chunks
  // overlap the extraction of earlier ones.  Newline prefixes are counted
  // from each chunk's start, which is all the extraction reads of them.
  const bool overlap = !ctx->ext_mode && spans.size() > 1 && ctx->ticket_events.size() == ctx->chunks.size();
  // Input pieces (host chunks of one sample, staged keys): the chunks fall
  // into NP runs, and each run's bucket scatter follows its last chunk's
  // extraction, while later chunks are still copying in.  The key array
  // then holds the pieces one after another, each bucket-major inside, and
  // the first split level reads every bucket as one run per piece.  Until the
  // key total is known, the key array is sized for a full staging buffer.
  const uint32_t NP = (overlap && NS == 1 && stage_keys) ? std::min<uint32_t>(kMaxPieces, (uint32_t)spans.size()) : 1;
  std::vector<uint32_t> piece_first(NP + 1, 0);  // first block of each piece
  if (NP > 1) {
    KCU(ctx->piece_off.ensure((size_t)NP * P * 8));
    KCU(ctx->piece_cnt.ensure((size_t)NP * P * 8));
    KCU(ctx->piece_base.ensure(8));
    KCU(cudaMemsetAsync(ctx->piece_base.p, 0, 8, s));
    KCU(ctx->keys_a.ensure(stage_cap * sizeof(T)));
  }
  unsigned long long* nl = ctx->nl.as<unsigned long long>();
  auto wait_all_copies = [&]() -> cudaError_t {
    cudaEvent_t dep;
    cudaError_t e = cudaEventCreateWithFlags(&dep, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventRecord(dep, ctx->copy_stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, dep, 0);
    cudaEventDestroy(dep);
    return e;
  };
  if (overlap) {
    KCU(cudaEventRecord(ctx->ev[1], s));  // the newline stage folds into the histogram stage
    uint32_t piece = 0;
    for (size_t i = 0; i < spans.size(); ++i) {
      const Span& sp = spans[i];
      KCU(cudaStreamWaitEvent(s, ctx->ticket_events[sp.chunk], 0));
      launch_newline_count(base, ctx->blocks.as<BlockDesc>() + sp.first, sp.n, nl + sp.first, s);
      st.kernel_launches += 1 + exclusive_scan_u64(nl + sp.first, nl + sp.first, sp.n,
                                                   ctx->scan_tmp.as<unsigned long long>(), s);
      ep.block_base = sp.first;
      launch_extract_hist<T>(ep, sp.n, s);
      st.kernel_launches += 1;
      if (NP > 1 && i + 1 == (size_t)(piece + 1) * spans.size() / NP) {
        // the piece's blocks: offsets inside the piece, the piece's bucket
        // runs after the earlier pieces, and its staged keys scattered there
        const uint32_t r0 = piece_first[piece], rows = sp.first + sp.n - r0;
        unsigned* m = ctx->blk_mat.as<unsigned>() + (size_t)r0 * P;
        unsigned long long* pc = ctx->piece_cnt.as<unsigned long long>() + (size_t)piece * P;
        unsigned long long* po = ctx->piece_off.as<unsigned long long>() + (size_t)piece * P;
        st.kernel_launches += count_matrix_offsets(m, rows, P, ctx->blk_gsum.as<unsigned long long>(), pc, s);
        launch_piece_offsets(pc, P, ctx->piece_base.as<unsigned long long>(), po,
                             ctx->bucket_count.as<unsigned long long>(), s);
        launch_bucket_scatter<T>(ctx->keys_b.as<T>(), ctx->blk_keys.as<unsigned long long>() + 2 * (size_t)r0, m,
                                 ctx->blocks.as<BlockDesc>() + r0, po, P, ep.shift, rows, ctx->keys_a.as<T>(),
                                 ctx->stage_ctr.as<unsigned long long>(), stage_cap, s);
        st.kernel_launches += 2;
        piece_first[++piece] = sp.first + sp.n;
      }
    }
    ep.block_base = 0;
    KCU(wait_all_copies());
  } else {
    KCU(wait_all_copies());
    launch_newline_count(base, ctx->blocks.as<BlockDesc>(), nblocks, nl, s);
    st.kernel_launches += 1 + exclusive_scan_u64(nl, nl, nblocks, ctx->scan_tmp.as<unsigned long long>(), s);
    KCU(cudaEventRecord(ctx->ev[1], s));
    launch_extract_hist<T>(ep, nblocks, s);
    st.kernel_launches += 1;
  }
  if (use_matrix && NP == 1) {
    // column totals straight into the bucket counts for one sample; per
    // (sample, bucket) totals from the sample boundaries for a batch
    KCU(ctx->col_total.ensure((size_t)P * 8));
    st.kernel_launches += count_matrix_offsets(ctx->blk_mat.as<unsigned>(), nblocks, P,
                                               ctx->blk_gsum.as<unsigned long long>(),
                                               NS == 1 ? ctx->bucket_count.as<unsigned long long>()
                                                       : ctx->col_total.as<unsigned long long>(), s);
    if (NS > 1) {
      KCU(ctx->sample_first.ensure((NS + 1) * 4));
      KCU(cudaMemcpyAsync(ctx->sample_first.p, sample_first.data(), (NS + 1) * 4, cudaMemcpyHostToDevice, s));
      launch_sample_bucket_counts(ctx->blk_mat.as<unsigned>(), ctx->col_total.as<unsigned long long>(),
                                  ctx->sample_first.as<uint32_t>(), NS, P, nblocks,
                                  ctx->bucket_count.as<unsigned long long>(), s);
      st.kernel_launches += 1;
    }
  }
  KCU(cudaGetLastError());
  KCU(cudaEventRecord(ctx->ev[2], s));

  // bring bucket counts, totals and the sample count to the host
  // host copies: bucket counts, per-sample totals, sample count, staged keys
  const size_t o_tot = (size_t)PT * 8, o_ns = o_tot + NS * sizeof(CountTotals), o_stg = o_ns + 8;
  const size_t o_pc = o_stg + 8, pc_bytes = NP > 1 ? (size_t)NP * P * 8 : 0;
  const size_t small_bytes = o_pc + pc_bytes;
  // then the bucket offsets and (pieces) the pieces' runs in bucket order
  KCU(ctx->h_small.ensure(small_bytes + (size_t)PT * 8 + pc_bytes));
  uint8_t* hs = ctx->h_small.as<uint8_t>();
  if (NP > 1) KCU(cudaMemcpyAsync(hs + o_pc, ctx->piece_cnt.p, pc_bytes, cudaMemcpyDeviceToHost, s));
  KCU(cudaMemcpyAsync(hs, ctx->bucket_count.p, (size_t)PT * 8, cudaMemcpyDeviceToHost, s));
  KCU(cudaMemcpyAsync(hs + o_tot, ctx->totals.p, NS * sizeof(CountTotals), cudaMemcpyDeviceToHost, s));
  KCU(cudaMemcpyAsync(hs + o_ns, ctx->sample_count.p, 4, cudaMemcpyDeviceToHost, s));
  if (stage_keys) KCU(cudaMemcpyAsync(hs + o_stg, ctx->stage_ctr.p, 8, cudaMemcpyDeviceToHost, s));
  int rc = wait_stream(ctx, s);
  if (rc) return rc;
  const auto wall1 = clk::now();
  uint64_t staged = ~0ull;
  if (stage_keys) std::memcpy(&staged, hs + o_stg, 8);
  std::vector<uint64_t> bcount(PT);
  std::memcpy(bcount.data(), hs, (size_t)PT * 8);
  std::vector<CountTotals> tot(NS);
  std::memcpy(tot.data(), hs + o_tot, NS * sizeof(CountTotals));
  uint32_t nsample = 0;
  std::memcpy(&nsample, hs + o_ns, 4);
  nsample = std::min(nsample, sample_cap);
  for (uint32_t t = 0; t < NS; ++t) {
    st.reads += tot[t].reads;
    st.bases += tot[t].bases;
    st.kmers += tot[t].kmers;
    ctx->sample_totals[3 * t] = tot[t].reads;
    ctx->sample_totals[3 * t + 1] = tot[t].bases;
    ctx->sample_totals[3 * t + 2] = tot[t].kmers;
  }
  const uint64_t N = st.kmers;
  if (N == 0) {
    ctx->res_meta.assign(PT, BucketMeta{});
    ctx->res_bytes = 0;
    return KITE_OK;
  }

  // ---- K3 scatter pass ----------------------------------------------------
  std::vector<uint64_t> boff(PT);
  uint64_t acc = 0, maxb = 0;
  for (uint32_t b = 0; b < PT; ++b) {
    boff[b] = acc;
    acc += bcount[b];
    maxb = std::max(maxb, bcount[b]);
  }
  std::memcpy(hs + small_bytes, boff.data(), (size_t)PT * 8);
  KCU(ctx->bucket_off.ensure((size_t)PT * 8));
  KCU(ctx->bucket_fill.ensure((size_t)PT * 8));
  KCU(cudaMemcpyAsync(ctx->bucket_off.p, hs + small_bytes, (size_t)PT * 8, cudaMemcpyHostToDevice, s));
  KCU(cudaMemsetAsync(ctx->bucket_fill.p, 0, (size_t)PT * 8, s));
  KCU(ctx->keys_a.ensure(N * sizeof(T)));
  KCU(ctx->keys_b.ensure(N * sizeof(T)));
  KCU(ctx->counts.ensure(N * 4));
  ep.bucket_off = ctx->bucket_off.as<unsigned long long>();
  ep.bucket_fill = ctx->bucket_fill.as<unsigned long long>();
  ep.keys_out = ctx->keys_a.as<T>();
  ep.blk_counts = nullptr;
  ep.blk_offs = (use_matrix && maxb < (1ull << 32)) ? ctx->blk_mat.as<unsigned>() : nullptr;
  const bool staged_ok = stage_keys && ep.blk_offs && staged == N && N <= stage_cap;
  // pieces > 1: the keys lie piece after piece (their scatters ran with the extraction)
  uint32_t pieces = 1;
  const uint64_t* pcnt = reinterpret_cast<const uint64_t*>(hs + o_pc);
  uint64_t maxpc = maxb;  // the largest run of one bucket in one piece
  if (NP > 1 && staged_ok) {
    st.staged_scatter = 1;
    pieces = NP;
    maxpc = 0;
    for (size_t i = 0; i < (size_t)NP * P; ++i) maxpc = std::max<uint64_t>(maxpc, pcnt[i]);
  } else if (staged_ok) {
    st.staged_scatter = 1;
    launch_bucket_scatter<T>(ctx->keys_b.as<T>(), ctx->blk_keys.as<unsigned long long>(), ep.blk_offs,
                             ctx->blocks.as<BlockDesc>(), ctx->bucket_off.as<unsigned long long>(), P, ep.shift,
                             nblocks, ctx->keys_a.as<T>(), nullptr, 0, s);
    st.kernel_launches += 1;
  } else {
    // from the FASTQ again; with pieces the matrix holds offsets inside each
    // piece, so the keys take their places by atomics
    if (NP > 1) ep.blk_offs = nullptr;
    ep.keys_stage = nullptr;
    launch_extract_scatter<T>(ep, nblocks, s);
    st.kernel_launches += 1;
  }
  st.input_pieces = pieces;
  KCU(cudaGetLastError());
  KCU(cudaEventRecord(ctx->ev[3], s));

  // ---- K3b tile split -----------------------------------------------------
  // Tiles per bucket: the largest bucket's keys over the target tile load
  // (cfg.tile_fill of the on-chip capacity), rounded up to a multiple of 32
  // for one split level (up to 1024 tiles); beyond that a power of two, so
  // that the two levels divide it evenly.
  const double fill = std::min(4.0, std::max(0.05, ctx->cfg.tile_fill));
  uint32_t S = 1;
  if ((double)maxb > fill * CAP) {
    const double want = std::ceil((double)maxb / (fill * CAP));
    if (want <= 1024.0) {
      S = std::min<uint32_t>(1024, ((uint32_t)want + 31) & ~31u);
    } else {
      S = 2048;
      while ((double)S < want && S < 4096) S <<= 1;
    }
  }
  st.tiles_per_bucket = S;
  if (S == 1 && pieces > 1) {
    // one tile per bucket reads each bucket as one run: the staged keys are
    // scattered again, piece q's run of bucket b after the earlier pieces' runs
    uint64_t* at = reinterpret_cast<uint64_t*>(hs + small_bytes + (size_t)PT * 8);
    for (uint32_t b = 0; b < P; ++b) {
      uint64_t o = boff[b];
      for (uint32_t q = 0; q < NP; ++q) {
        at[(size_t)q * P + b] = o;
        o += pcnt[(size_t)q * P + b];
      }
    }
    KCU(cudaMemcpyAsync(ctx->piece_off.p, at, pc_bytes, cudaMemcpyHostToDevice, s));
    for (uint32_t q = 0; q < NP; ++q) {
      const uint32_t r0 = piece_first[q];
      launch_bucket_scatter<T>(ctx->keys_b.as<T>(), ctx->blk_keys.as<unsigned long long>() + 2 * (size_t)r0,
                               ctx->blk_mat.as<unsigned>() + (size_t)r0 * P, ctx->blocks.as<BlockDesc>() + r0,
                               ctx->piece_off.as<unsigned long long>() + (size_t)q * P, P, ep.shift,
                               piece_first[q + 1] - r0, ctx->keys_a.as<T>(), nullptr, 0, s);
      st.kernel_launches += 1;
    }
    pieces = 1;
    maxpc = maxb;
  }
  T* sorted = ctx->keys_a.as<T>();
  T* scratch = ctx->keys_b.as<T>();
  const T* tile_spl = nullptr;  // the splitters that cut every bucket into its S tiles
  std::vector<TileDesc> ht;  // one tile per bucket (S == 1): made on the host
  uint32_t dev_tiles = 0;    // S > 1: the tiles made on the device
  if (S == 1) {
    for (uint32_t b = 0; b < PT; ++b) ht.push_back(TileDesc{boff[b], (uint32_t)bcount[b], b});
  } else {
    // Splitters: SAMPLED = histogram only; LEARNED = train the CDF and keep
    // it unless its predicted max/mean tile load exceeds imbalance_bound AND
    // the histogram's prediction is lower (then the histogram); AUTO =
    // histogram unless its own prediction exceeds the bound, then as LEARNED.
    KCU(ctx->splitters.ensure((size_t)S * sizeof(T)));
    KCU(ctx->splitters2.ensure((size_t)S * sizeof(T)));
    KCU(ctx->hist16.ensure((size_t)65536 * 4));
    const int mode = ctx->cfg.splitter_mode;
    const double bound = ctx->cfg.imbalance_bound;
    T* hist_spl = ctx->splitters.as<T>();
    T* mlp_spl = ctx->splitters2.as<T>();
    double hist_imb = -1.0;
    // The splitters depend only on the key sample, complete since the bucket
    // counts were read back: they are made on the side stream, so their
    // evaluations (which wait on the host) overlap the bucket scatter; the
    // split waits for them through an event.
    const cudaStream_t ss = ctx->aux_stream;
    if (mode != KITE_SPLIT_LEARNED) {
      st.kernel_launches +=
          compute_hist_splitters<T>(ctx->sample.as<T>(), nsample, 2 * k, S, hist_spl, ctx->hist16.as<unsigned>(), ss);
      if (mode == KITE_SPLIT_AUTO) {
        if (predict_imbalance<T>(ctx->mlp, ctx->sample.as<T>(), nsample, hist_spl, S, ss, ctx->cfg.timeout_ms,
                                 &hist_imb))
          return fail(ctx, KITE_ERR_TIMEOUT, "splitter evaluation did not finish");
        st.kernel_launches += 1;
      }
    }
    bool learned = false;
    if (mode == KITE_SPLIT_LEARNED || (mode == KITE_SPLIT_AUTO && hist_imb > bound)) {
      MlpReport rep;
      if (mlp_splitters<T>(ctx->mlp, ctx->sample.as<T>(), nsample, 2 * k, S, mlp_spl, ss, ctx->cfg.timeout_ms, &rep))
        return fail(ctx, KITE_ERR_CUDA, "learned splitter training failed");
      st.kernel_launches += rep.launches;
      st.mlp_loss = rep.loss;
      st.mlp_pred_imbalance = rep.pred_imbalance;
      st.mlp_reused = rep.reused ? 1u : 0u;
      learned = rep.pred_imbalance <= bound;
      if (!learned && mode == KITE_SPLIT_LEARNED) {
        st.kernel_launches += compute_hist_splitters<T>(ctx->sample.as<T>(), nsample, 2 * k, S, hist_spl,
                                                        ctx->hist16.as<unsigned>(), ss);
        if (predict_imbalance<T>(ctx->mlp, ctx->sample.as<T>(), nsample, hist_spl, S, ss, ctx->cfg.timeout_ms,
                                 &hist_imb))
          return fail(ctx, KITE_ERR_TIMEOUT, "splitter evaluation did not finish");
        st.kernel_launches += 1;
      }
      // above the bound the network still wins when the histogram predicts worse
      if (!learned && hist_imb >= 0.0 && rep.pred_imbalance < hist_imb) learned = true;
    }
    st.hist_pred_imbalance = hist_imb;
    st.splitter_used = learned ? KITE_SPLIT_LEARNED : KITE_SPLIT_SAMPLED;
    const T* chosen = learned ? mlp_spl : hist_spl;
    tile_spl = chosen;
    KCU(cudaEventRecord(ctx->spl_ready, ss));
    KCU(cudaStreamWaitEvent(s, ctx->spl_ready, 0));
    // Split into tiles: one level of S digits when S <= 1024, else coarse
    // ranges of 1024 tiles first, then the tiles inside each coarse range.
    // G parts per region (parts of >= 32K keys, G <= 64): the fewest parts
    // whose CTAs fill the scatter's resident slots in whole waves, as far as
    // a 2% gain in the used fraction of the last wave goes.
    auto parts = [&](uint64_t regions, uint64_t max_region, uint32_t D) {
      const uint64_t slots = split_scatter_slots<T>(D, ctx->cfg.scatter_shape);
      const uint64_t gmax = std::min<uint64_t>(64, std::max<uint64_t>(1, max_region / 32768));
      uint64_t best = 1;
      double best_used = 0.0;
      for (uint64_t g = 1; g <= gmax; ++g) {
        const uint64_t ctas = regions * g;
        const double used = (double)ctas / (double)(((ctas + slots - 1) / slots) * slots);
        if (used > best_used + 0.02) {
          best = g;
          best_used = used;
        }
      }
      return (uint32_t)best;
    };
    const uint32_t D2 = std::min<uint32_t>(S, 1024), D1 = S / D2;
    st.split_levels = D1 > 1 ? 2 : 1;
    const size_t nt = (size_t)PT * S;
    TileSplitParams<T> tp{};
    tp.splitters = chosen;
    tp.spl_total = S - 1;
    tp.key_bits = 2 * k;
    tp.spl_step = 1;
    tp.spl_mod = 1;
    uint32_t G = 1;
    T* level_in = ctx->keys_a.as<T>();
    T* level_out = ctx->keys_b.as<T>();
    if (D1 > 1) {
      // level 1: buckets -> (bucket, coarse range); coarse splitter c is tile splitter (c+1)*D2-1
      const uint32_t G1 = pieces * parts((uint64_t)PT * pieces, maxpc, D1);
      const size_t n1 = (size_t)PT * D1 * G1;
      KCU(ctx->lvl_count.ensure(n1 * 8));
      KCU(ctx->lvl_off.ensure(n1 * 8));
      KCU(ctx->reg_off.ensure((size_t)PT * D1 * 8));
      KCU(ctx->reg_cnt.ensure((size_t)PT * D1 * 8));
      KCU(ctx->scan_tmp.ensure(scan_tmp_elems(n1) * 8 + 64));
      TileSplitParams<T> t1 = tp;
      t1.keys_in = level_in;
      t1.keys_out = level_out;
      t1.region_off = (pieces > 1 ? ctx->piece_off : ctx->bucket_off).as<unsigned long long>();
      t1.region_count = (pieces > 1 ? ctx->piece_cnt : ctx->bucket_count).as<unsigned long long>();
      t1.pieces = pieces;
      t1.R = PT;
      t1.D = D1;
      t1.G = G1;
      t1.spl_first = D2 - 1;
      t1.spl_step = D2;
      t1.spl_region_stride = 0;
      t1.tile_count = ctx->lvl_count.as<unsigned long long>();
      t1.tile_off = ctx->lvl_off.as<unsigned long long>();
      launch_split_hist<T>(t1, s);
      st.kernel_launches += 3 + exclusive_scan_u64(t1.tile_count, ctx->lvl_off.as<unsigned long long>(), n1,
                                                   ctx->scan_tmp.as<unsigned long long>(), s);
      launch_split_scatter<T>(t1, ctx->cfg.scatter_shape, s);
      launch_region_bounds(t1.tile_off, PT * D1, G1, N, ctx->reg_off.as<unsigned long long>(),
                           ctx->reg_cnt.as<unsigned long long>(), s);
      // level 2: (bucket, coarse c) -> tiles c*D2 .. c*D2+D2-1
      G = parts((uint64_t)PT * D1, (maxb + D1 - 1) / D1 * 2, D2);
      tp.region_off = ctx->reg_off.as<unsigned long long>();
      tp.region_count = ctx->reg_cnt.as<unsigned long long>();
      tp.R = PT * D1;
      tp.spl_first = 0;
      tp.spl_mod = D1;
      tp.spl_region_stride = D2;
      std::swap(level_in, level_out);
    } else {
      G = pieces * parts((uint64_t)PT * pieces, maxpc, D2);
      tp.region_off = (pieces > 1 ? ctx->piece_off : ctx->bucket_off).as<unsigned long long>();
      tp.region_count = (pieces > 1 ? ctx->piece_cnt : ctx->bucket_count).as<unsigned long long>();
      tp.pieces = pieces;
      tp.R = PT;
      tp.spl_first = 0;
      tp.spl_region_stride = 0;
    }
    const size_t ntg = nt * G;
    KCU(ctx->tile_count.ensure(ntg * 8));
    KCU(ctx->tile_off.ensure(ntg * 8));
    KCU(ctx->scan_tmp.ensure(scan_tmp_elems(ntg) * 8 + 64));
    tp.keys_in = level_in;
    tp.keys_out = level_out;
    tp.D = D2;
    tp.G = G;
    tp.tile_count = ctx->tile_count.as<unsigned long long>();
    tp.tile_off = ctx->tile_off.as<unsigned long long>();
    // the last level's digits: computed once by the histogram, read by the scatter
    KCU(ctx->digits.ensure(N * 2));
    tp.dig = ctx->digits.as<uint16_t>();
    launch_split_hist<T>(tp, s);
    st.kernel_launches += 3 + exclusive_scan_u64(tp.tile_count, ctx->tile_off.as<unsigned long long>(), ntg,
                                                 ctx->scan_tmp.as<unsigned long long>(), s);
    launch_split_scatter<T>(tp, ctx->cfg.scatter_shape, s);
    KCU(ctx->tiles.ensure(nt * sizeof(TileDesc)));
    KCU(ctx->tile_fill.ensure(nt * 4));
    launch_make_tiles(ctx->tile_off.as<unsigned long long>(), (uint32_t)nt, S, G, N, ctx->tiles.as<TileDesc>(),
                      ctx->tile_fill.as<uint32_t>(), s);
    KCU(cudaGetLastError());
    // the tile lengths stay on the device: the oversized tiles are listed
    // there and the sort follows without a host round trip
    dev_tiles = (uint32_t)nt;
    sorted = level_out;
    scratch = level_in;
  }
  KCU(cudaEventRecord(ctx->ev[4], s));
  const uint32_t ntiles = dev_tiles ? dev_tiles : (uint32_t)ht.size();
  const uint32_t Sl = ntiles / PT;  // tiles per bucket
  const T kmax = 2 * k >= (uint32_t)KeyTraits<T>::kBits ? ~T(0) : ((T(1) << (2 * k)) - T(1));
  // Bucket groups: each group's tiles are sorted, linked and encoded in turn,
  // so one group's payload copies to the host while the next one sorts.
  const uint32_t NG = std::min<uint32_t>(kSortGroups, PT);
  std::vector<uint32_t> gb(NG + 1);  // first bucket of each group
  for (uint32_t g = 0; g <= NG; ++g) gb[g] = (uint32_t)((uint64_t)PT * g / NG);
  if (NG == 8 && PT >= 64) {
    // tapering groups (weights 6,6,6,6,6,5,3,2 of 40): the last copy to the
    // host, which nothing overlaps, carries a twentieth of the payload
    static const uint32_t cw[9] = {0, 6, 12, 18, 24, 30, 35, 38, 40};
    for (uint32_t g = 0; g <= NG; ++g) gb[g] = (uint32_t)((uint64_t)PT * cw[g] / 40);
  }
  // Oversized tiles, group by group: those sorted on chip at twice the
  // capacity (list A) and those sorted through global memory (list B).  From
  // device-made tiles the lists are made on the device (group g's entries
  // from index gb[g] * S, counts lcnt[2g], lcnt[2g+1]) and walked by a fixed
  // grid; from host tiles on the host, one CTA per listed tile.
  std::vector<uint32_t> big, gbig(NG + 1, 0), glarge(NG, 0);
  KCU(ctx->big_ids.ensure((size_t)2 * ntiles * 4 + 8));
  uint32_t* ids_a = ctx->big_ids.as<uint32_t>();
  uint32_t* ids_b = ids_a + ntiles;
  unsigned* lcnt = nullptr;
  const size_t lhead = (size_t)(2 * NG + 8) * 8;  // counts, then the group bounds
  const size_t lbytes = lhead + (size_t)(4 + S) * 8;
  if (dev_tiles) {
    KCU(ctx->tile_lists.ensure(lbytes + 64));
    lcnt = ctx->tile_lists.as<unsigned>();
    // [0] largest tile, [1] keys, [2] non-empty tiles, [3] keys in tiles above
    // capacity, then the S range sums
    unsigned long long* lstats = reinterpret_cast<unsigned long long*>(ctx->tile_lists.as<uint8_t>() + lhead);
    KCU(cudaMemsetAsync(ctx->tile_lists.p, 0, lbytes, s));
    uint32_t* dgb = reinterpret_cast<uint32_t*>(lcnt + 2 * NG);
    KCU(ctx->h_tiles.ensure(lbytes + 64));
    std::memcpy(ctx->h_tiles.p, gb.data(), (NG + 1) * 4);
    KCU(cudaMemcpyAsync(dgb, ctx->h_tiles.p, (NG + 1) * 4, cudaMemcpyHostToDevice, s));
    launch_tile_lists(ctx->tile_fill.as<uint32_t>(), ntiles, S, dgb, NG, CAP, ids_a, ids_b, lcnt, lstats, lstats + 4,
                      s);
    st.kernel_launches += 1;
    st.tiles = ntiles;
  } else {
    for (uint32_t g = 0; g < NG; ++g) {
      gbig[g] = (uint32_t)big.size();
      for (uint32_t t = gb[g] * Sl; t < gb[g + 1] * Sl; ++t)
        if (ht[t].len > CAP && ht[t].len <= 2 * CAP) big.push_back(t);
      glarge[g] = (uint32_t)big.size() - gbig[g];
      for (uint32_t t = gb[g] * Sl; t < gb[g + 1] * Sl; ++t)
        if (ht[t].len > 2 * CAP) big.push_back(t);
    }
    gbig[NG] = (uint32_t)big.size();
    uint64_t tmax = 0, tsum = 0, tne = 0;
    for (uint32_t t = 0; t < ntiles; ++t)
      if (ht[t].len) {
        tmax = std::max<uint64_t>(tmax, ht[t].len);
        tsum += ht[t].len;
        tne++;
      }
    st.tiles = ntiles;
    st.big_tiles = (uint32_t)big.size();
    for (uint32_t t : big) st.big_tile_keys += ht[t].len;
    st.tile_imbalance = tne ? (double)tmax / ((double)tsum / (double)tne) : 0.0;
    st.range_imbalance = 1.0;  // one tile per bucket
    KCU(ctx->h_tiles.ensure(ht.size() * sizeof(TileDesc) + big.size() * 4 + 64));
    std::memcpy(ctx->h_tiles.p, ht.data(), ht.size() * sizeof(TileDesc));
    KCU(ctx->tiles.ensure(ht.size() * sizeof(TileDesc)));
    KCU(cudaMemcpyAsync(ctx->tiles.p, ctx->h_tiles.p, ht.size() * sizeof(TileDesc), cudaMemcpyHostToDevice, s));
    if (!big.empty()) {
      uint8_t* hb2 = ctx->h_tiles.as<uint8_t>() + ht.size() * sizeof(TileDesc);
      std::memcpy(hb2, big.data(), big.size() * 4);
      KCU(cudaMemcpyAsync(ids_a, hb2, big.size() * 4, cudaMemcpyHostToDevice, s));
    }
  }
  int sm_count = 0;
  cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, ctx->cfg.device);
  const uint32_t walk_grid = (uint32_t)std::max(1, sm_count);
  KCU(ctx->tile_out.ensure((size_t)ntiles * sizeof(TileOut<T>)));
  KCU(ctx->sort_stats.ensure(16));
  KCU(cudaMemsetAsync(ctx->sort_stats.p, 0, 16, s));
  KCU(ctx->tile_boff.ensure((size_t)ntiles * 8));
  KCU(ctx->tile_prev.ensure((size_t)ntiles * sizeof(T)));
  KCU(ctx->meta.ensure((size_t)PT * sizeof(BucketMeta)));
  KCU(ctx->h_meta.ensure((size_t)PT * sizeof(BucketMeta)));
  // payload buffers: the previous payload size or 2.25 bytes per k-mer to
  // start with; grown, keeping what is written, when a group needs more
  KCU(ctx->out.ensure(std::max<uint64_t>(ctx->res_bytes, N * 9 / 4) + 16));
  if (to_host) KCU(ctx->h_out.ensure(std::max<uint64_t>(ctx->res_bytes, N * 9 / 4) + 16));
  ctx->res_on_host = false;
  ctx->res_meta.assign(PT, BucketMeta{});
  st.kernel_launches += 1 + (uint64_t)NG * 3 + (uint64_t)NG * 3;  // memset, per group: sort, link, offsets, encode
  for (uint32_t g = 0; g < NG; ++g)
    st.kernel_launches += dev_tiles ? 2 : (glarge[g] ? 1 : 0) + (gbig[g + 1] - gbig[g] > glarge[g] ? 1 : 0);
  cudaEvent_t* gev = ctx->gev.data();  // per group: sort, large, link | encode | copy start/end
  TileOut<T>* tout = ctx->tile_out.as<TileOut<T>>();
  BucketMeta* meta = ctx->meta.as<BucketMeta>();
  BucketMeta* hmeta = ctx->h_meta.as<BucketMeta>();
  // the device's address of the pinned records (mapped host memory): the
  // offsets kernel writes them there, and nothing queues on a copy engine
  // behind the previous group's payload copy
  BucketMeta* hmeta_dev = nullptr;
  KCU(cudaHostGetDevicePointer(reinterpret_cast<void**>(&hmeta_dev), hmeta, 0));

  // ---- K4 tile sort + RLE, K5 link and byte offsets (one group) --------------
  auto queue_sort = [&](uint32_t g) -> cudaError_t {
    const uint32_t t0 = gb[g] * Sl, nt = (gb[g + 1] - gb[g]) * Sl, nb = gb[g + 1] - gb[g];
    cudaEventRecord(gev[8 * g], s);
    launch_tile_sort<T>(sorted, ctx->counts.as<uint32_t>(), ctx->tiles.as<TileDesc>() + t0, nt, tout + t0,
                        ctx->sort_stats.as<unsigned long long>(), TileRanges<T>{tile_spl, Sl, t0, kmax, ctx->cfg.tile_wait_polls}, s);
    cudaEventRecord(gev[8 * g + 1], s);
    if (dev_tiles) {
      launch_tile_sort_large<T>(sorted, ctx->counts.as<uint32_t>(), ctx->tiles.as<TileDesc>(), ids_a + t0, walk_grid,
                                lcnt + 2 * g, tout, ctx->sort_stats.as<unsigned long long>(),
                                TileRanges<T>{tile_spl, Sl, 0, kmax, ctx->cfg.tile_wait_polls}, s);
      launch_big_tile_sort<T>(sorted, ctx->counts.as<uint32_t>(), scratch, ctx->tiles.as<TileDesc>(), ids_b + t0,
                              walk_grid, lcnt + 2 * g + 1, tout, ctx->status.as<DevStatus>(),
                              ctx->sort_stats.as<unsigned long long>(), s);
    } else {
      launch_tile_sort_large<T>(sorted, ctx->counts.as<uint32_t>(), ctx->tiles.as<TileDesc>(), ids_a + gbig[g],
                                glarge[g], nullptr, tout, ctx->sort_stats.as<unsigned long long>(),
                                TileRanges<T>{tile_spl, Sl, 0, kmax, ctx->cfg.tile_wait_polls}, s);
      launch_big_tile_sort<T>(sorted, ctx->counts.as<uint32_t>(), scratch, ctx->tiles.as<TileDesc>(),
                              ids_a + gbig[g] + glarge[g], gbig[g + 1] - gbig[g] - glarge[g], nullptr, tout,
                              ctx->status.as<DevStatus>(), ctx->sort_stats.as<unsigned long long>(), s);
    }
    cudaEventRecord(gev[8 * g + 2], s);
    // ---- K5: per-bucket tile links, byte offsets from the group's start
    launch_tile_link<T>(tout + t0, nb, Sl, ctx->tile_boff.as<unsigned long long>() + t0, ctx->tile_prev.as<T>() + t0,
                        meta + gb[g], s);
    launch_bucket_offsets(meta + gb[g], nb, hmeta_dev + gb[g], s);
    cudaEventRecord(gev[8 * g + 3], s);
    return cudaGetLastError();
  };
  // With copies to the host, the encodes run on the highest-priority side
  // stream, each behind its group's sort and offsets, so group g's encode and
  // then its copy start as soon as the host has read the group's sizes,
  // beside the sort of group g+1 rather than after it.  Results kept on the
  // device encode in line on the counting stream (nothing waits on them there,
  // and the sorts keep the SMs to themselves).
  const cudaStream_t es = to_host ? ctx->aux_stream : s;
  // Grows a payload buffer to `need` bytes keeping its first `keep` bytes
  // (after every queued encode and copy has finished).
  auto grow_out = [&](uint64_t need, uint64_t keep) -> int {
    int r = wait_stream(ctx, s);
    if (!r) r = wait_stream(ctx, es);
    if (!r) r = wait_stream(ctx, ctx->copy_stream);
    if (r) return r;
    if (need > ctx->out.cap) {
      DevBuf nb;
      KCU(nb.ensure(need));
      if (keep) KCU(cudaMemcpy(nb.p, ctx->out.p, keep, cudaMemcpyDeviceToDevice));
      ctx->out.release();
      ctx->out = nb;
    }
    if (to_host && need > ctx->h_out.cap) {
      HostBuf nb;
      KCU(nb.ensure(need));
      if (keep) std::memcpy(nb.p, ctx->h_out.p, keep);
      ctx->h_out.release();
      ctx->h_out = nb;
    }
    return KITE_OK;
  };

  uint64_t total_bytes = 0, rows = 0;
  float ms_sort = 0, ms_big = 0, ms_enc = 0, ms_d2h = 0;
  KCU(queue_sort(0));
  for (uint32_t g = 0; g < NG; ++g) {
    if (g + 1 < NG) KCU(queue_sort(g + 1));
    rc = wait_event(ctx, gev[8 * g + 3]);
    if (rc) return rc;
    const uint32_t t0 = gb[g] * Sl, nt = (gb[g + 1] - gb[g]) * Sl;
    uint64_t gbytes = 0;
    for (uint32_t b = gb[g]; b < gb[g + 1]; ++b) {
      BucketMeta m = hmeta[b];
      gbytes += m.bytes;
      rows += m.rows;
      m.byte_off += total_bytes;
      ctx->res_meta[b] = m;
    }
    if (total_bytes + gbytes + 16 > ctx->out.cap || (to_host && total_bytes + gbytes + 16 > ctx->h_out.cap)) {
      rc = grow_out(total_bytes + gbytes + 16 + (total_bytes + gbytes) / 4, total_bytes);
      if (rc) return rc;
    }
    // ---- K7 DVLE encode of the group, then its copy to the host
    KCU(cudaStreamWaitEvent(es, gev[8 * g + 3], 0));
    cudaEventRecord(gev[8 * g + 4], es);
    launch_encode<T>(sorted, ctx->counts.as<uint32_t>(), ctx->tiles.as<TileDesc>() + t0, tout + t0,
                     ctx->tile_boff.as<unsigned long long>() + t0, ctx->tile_prev.as<T>() + t0, meta, nt,
                     ctx->out.as<uint8_t>() + total_bytes, gbytes, ctx->status.as<DevStatus>(), es);
    cudaEventRecord(gev[8 * g + 5], es);
    KCU(cudaGetLastError());
    if (to_host) {
      KCU(cudaStreamWaitEvent(ctx->copy_stream, gev[8 * g + 5], 0));
      cudaEventRecord(gev[8 * g + 6], ctx->copy_stream);
      if (gbytes)
        KCU(cudaMemcpyAsync(ctx->h_out.as<uint8_t>() + total_bytes, ctx->out.as<uint8_t>() + total_bytes, gbytes,
                            cudaMemcpyDeviceToHost, ctx->copy_stream));
      cudaEventRecord(gev[8 * g + 7], ctx->copy_stream);
    }
    total_bytes += gbytes;
  }
  // the counting stream takes up the encodes again
  KCU(cudaStreamWaitEvent(s, gev[8 * (NG - 1) + 5], 0));
  KCU(cudaEventRecord(ctx->ev[7], s));
  KCU(cudaMemcpyAsync(ctx->h_small.p, ctx->sort_stats.p, 16, cudaMemcpyDeviceToHost, s));
  if (dev_tiles) KCU(cudaMemcpyAsync(ctx->h_tiles.p, ctx->tile_lists.p, lbytes, cudaMemcpyDeviceToHost, s));
  rc = wait_stream(ctx, s);
  const auto wall2 = clk::now();
  if (!rc && to_host) rc = wait_stream(ctx, ctx->copy_stream);
  if (rc) return rc;
  st.stage_ms[8] = wall_ms(wall0, wall1);
  st.stage_ms[9] = wall_ms(wall1, wall2);
  st.stage_ms[10] = wall_ms(wall2, clk::now());
  std::memcpy(&st.sort_fallbacks, ctx->h_small.p, 8);
  std::memcpy(&st.big_tile_rows, ctx->h_small.as<uint8_t>() + 8, 8);
  // the tile sort adds 2^40 to its statistics when a tile's bulk load did not complete
  if (st.sort_fallbacks >> 40) return fail(ctx, KITE_ERR_TIMEOUT, "tile sort: a bulk load of a tile did not complete");
  if (dev_tiles) {
    const unsigned* hc = ctx->h_tiles.as<unsigned>();
    const unsigned long long* hs2 = reinterpret_cast<const unsigned long long*>(ctx->h_tiles.as<uint8_t>() + lhead);
    uint32_t nbig = 0;
    for (uint32_t g = 0; g < 2 * NG; ++g) nbig += hc[g];
    st.big_tiles = nbig;
    st.tile_imbalance = hs2[2] ? (double)hs2[0] / ((double)hs2[1] / (double)hs2[2]) : 0.0;
    unsigned long long rmax = 0;
    for (uint32_t t = 0; t < S; ++t) rmax = std::max(rmax, hs2[4 + t]);
    st.big_tile_keys = hs2[3];
    st.range_imbalance = (double)rmax / ((double)N / S);
  }
  rc = check_status(ctx, "count");
  if (rc) return rc;
  for (uint32_t g = 0; g < NG; ++g) {
    float a = 0, b = 0, c = 0, d = 0;
    cudaEventElapsedTime(&a, gev[8 * g], gev[8 * g + 1]);
    cudaEventElapsedTime(&b, gev[8 * g + 1], gev[8 * g + 2]);
    cudaEventElapsedTime(&c, gev[8 * g + 2], gev[8 * g + 3]);
    cudaEventElapsedTime(&d, gev[8 * g + 4], gev[8 * g + 5]);
    ms_sort += a;
    ms_big += b;
    ms_enc += c + d;
    if (to_host) {
      float e = 0;
      cudaEventElapsedTime(&e, gev[8 * g + 6], gev[8 * g + 7]);
      ms_d2h += e;
    }
  }
  ctx->res_bytes = total_bytes;
  ctx->res_on_host = to_host;
  if (to_host) st.d2h_bytes += total_bytes;
  st.rows = rows;
  st.payload_bytes = total_bytes;
  // stage times
  static const int map[4] = {ST_LINES, ST_HIST, ST_SCATTER, ST_SPLIT};
  for (int i = 0; i < 4; ++i) {
    float ms = 0;
    cudaEventElapsedTime(&ms, ctx->ev[i], ctx->ev[i + 1]);
    st.stage_ms[map[i]] = ms;
  }
  st.stage_ms[ST_SORT] = ms_sort;
  st.stage_ms[ST_BIG] = ms_big;
  st.stage_ms[ST_ENCODE] = ms_enc;
  st.stage_ms[ST_D2H] = ms_d2h;
  return KITE_OK;
}

int emit_results(kite_gpu_ctx* ctx, kite_gpu_emit_fn emit, void* user) {
  if (!emit) return KITE_OK;
  const uint32_t P = (uint32_t)ctx->res_meta.size();
  if (ctx->res_bytes && !ctx->res_on_host) {
    KCU(ctx->h_out.ensure(ctx->res_bytes));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, ctx->stream);
    KCU(cudaMemcpyAsync(ctx->h_out.p, ctx->out.p, ctx->res_bytes, cudaMemcpyDeviceToHost, ctx->stream));
    cudaEventRecord(e1, ctx->stream);
    int rc = wait_stream(ctx, ctx->stream);
    if (rc) return rc;
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    ctx->stats.stage_ms[ST_D2H] = ms;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    ctx->stats.d2h_bytes += ctx->res_bytes;
  }
  for (uint32_t b = 0; b < P; ++b) {
    const BucketMeta& m = ctx->res_meta[b];
    if (m.rows == 0) continue;
    kite_chunk_meta cm{};
    cm.partition_id = b;
    cm.codec = KITE_CODEC_DVLE;
    cm.row_count = m.rows;
    cm.raw_bytes = m.bytes;
    cm.key_min_lo[0] = m.kmin_lo;
    cm.key_min_lo[1] = m.kmin_hi;
    cm.key_max_lo[0] = m.kmax_lo;
    cm.key_max_lo[1] = m.kmax_hi;
    if (emit(user, &cm, ctx->h_out.as<uint8_t>() + m.byte_off, (size_t)m.bytes) != 0)
      return fail(ctx, KITE_ERR_CALLBACK, "emit callback aborted");
  }
  return KITE_OK;
}

}  // namespace

// ============================================================================
// C ABI
// ============================================================================
extern "C" {

int kite_gpu_abi_version(void) { return KITE_GPU_ABI_VERSION; }

int kite_gpu_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) return 0;
  return n;
}

const char* kite_gpu_last_error(const kite_gpu_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

void* kite_gpu_alloc_pinned(size_t bytes) {
  void* p = nullptr;
  if (cudaMallocHost(&p, bytes ? bytes : 1) != cudaSuccess) return nullptr;
  return p;
}
void kite_gpu_free_pinned(void* p) {
  if (p) cudaFreeHost(p);
}

int kite_gpu_open(const kite_gpu_cfg* cfg, kite_gpu_ctx** out) {
  if (!cfg || !out) return KITE_ERR_BAD_INPUT;
  *out = nullptr;
  if (cfg->k < 1 || cfg->k > 64) return KITE_ERR_UNSUPPORTED;
  if (cfg->partitions < 2 || (cfg->partitions & (cfg->partitions - 1)) || cfg->partitions > 65536)
    return KITE_ERR_BAD_INPUT;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0 || cfg->device < 0 || cfg->device >= ndev)
    return KITE_ERR_CUDA;
  if (cudaSetDevice(cfg->device) != cudaSuccess) return KITE_ERR_CUDA;
  kite_gpu_ctx* ctx = new kite_gpu_ctx();
  ctx->cfg = *cfg;
  if (ctx->cfg.timeout_ms == 0) ctx->cfg.timeout_ms = 600000;
  if (ctx->cfg.imbalance_bound <= 0) ctx->cfg.imbalance_bound = 1.10;
  if (ctx->cfg.samples == 0) ctx->cfg.samples = 1;
  if ((uint64_t)ctx->cfg.samples * ctx->cfg.partitions > (1u << 20)) {
    delete ctx;
    return KITE_ERR_BAD_INPUT;
  }
  if (ctx->cfg.tile_fill <= 0) ctx->cfg.tile_fill = 0.85;
  if (cfg->stream) {
    ctx->stream = (cudaStream_t)cfg->stream;
  } else {
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
      delete ctx;
      return KITE_ERR_CUDA;
    }
    ctx->own_stream = true;
  }
  // The splitter stream has the highest priority: its small kernels take SMs
  // as the bucket scatter's CTAs retire instead of waiting for its last wave.
  int prio_least = 0, prio_greatest = 0;
  cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest);
  if (cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithPriority(&ctx->aux_stream, cudaStreamNonBlocking, prio_greatest) != cudaSuccess ||
      cudaEventCreateWithFlags(&ctx->spl_ready, cudaEventDisableTiming) != cudaSuccess) {
    delete ctx;
    return KITE_ERR_CUDA;
  }
  ctx->ev.resize(9);
  for (auto& e : ctx->ev) cudaEventCreate(&e);
  ctx->gev.resize(8 * kSortGroups);
  for (auto& e : ctx->gev) cudaEventCreate(&e);
  if (ctx->cfg.arena_bytes == 0) {
    size_t fr = 0, to = 0;
    cudaMemGetInfo(&fr, &to);
    ctx->cfg.arena_bytes = std::max<uint64_t>(fr / 8, 64ull << 20);
  }
  ctx->mlp = mlp_create();
  *out = ctx;
  return KITE_OK;
}

void kite_gpu_close(kite_gpu_ctx* ctx) {
  if (!ctx) return;
  cudaStreamSynchronize(ctx->stream);
  cudaStreamSynchronize(ctx->copy_stream);
  cudaStreamSynchronize(ctx->aux_stream);
  for (auto e : ctx->ticket_events) cudaEventDestroy(e);
  for (auto e : ctx->ev) cudaEventDestroy(e);
  for (auto e : ctx->gev) cudaEventDestroy(e);
  DevBuf* bufs[] = {&ctx->arena, &ctx->blocks, &ctx->nl, &ctx->scan_tmp, &ctx->bucket_count, &ctx->bucket_off,
                    &ctx->bucket_fill, &ctx->totals, &ctx->status, &ctx->keys_a, &ctx->keys_b, &ctx->counts,
                    &ctx->sample, &ctx->sample_count, &ctx->splitters, &ctx->splitters2, &ctx->hist16,
                    &ctx->tile_count, &ctx->tile_off, &ctx->tile_fill, &ctx->tiles, &ctx->big_ids,
                    &ctx->tile_out, &ctx->tile_boff, &ctx->tile_prev, &ctx->meta, &ctx->out,
                    &ctx->lvl_count, &ctx->lvl_off, &ctx->reg_off, &ctx->reg_cnt, &ctx->sort_stats,
                    &ctx->blk_mat, &ctx->blk_gsum, &ctx->blk_keys, &ctx->stage_ctr,
                    &ctx->col_total, &ctx->sample_first, &ctx->spans, &ctx->digits, &ctx->tile_lists,
                    &ctx->piece_off, &ctx->piece_cnt, &ctx->piece_base};
  for (DevBuf* b : bufs) b->release();
  ctx->h_blocks.release();
  ctx->h_small.release();
  ctx->h_tiles.release();
  ctx->h_out.release();
  ctx->h_meta.release();
  ctx->h_dump.release();
  mlp_destroy(ctx->mlp);
  if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
  cudaStreamDestroy(ctx->copy_stream);
  cudaStreamDestroy(ctx->aux_stream);
  cudaEventDestroy(ctx->spl_ready);
  delete ctx;
}

int64_t kite_gpu_count_submit_sample(kite_gpu_ctx* ctx, uint32_t sample, const uint8_t* fastq, size_t len) {
  if (!ctx || (!fastq && len)) return KITE_ERR_BAD_INPUT;
  if (sample >= (ctx->cfg.samples ? ctx->cfg.samples : 1u))
    return fail(ctx, KITE_ERR_BAD_INPUT, "sample index beyond cfg.samples");
  if (ctx->ext_mode) return fail(ctx, KITE_ERR_STATE, "host and device submissions cannot mix in one segment");
  if (len == 0) return ctx->next_ticket++;
  cudaSetDevice(ctx->cfg.device);  // the caller's thread may not be the one that opened the context
  const uint64_t off = (ctx->arena_used + 15) & ~15ull;
  if (off + len + 16 > ctx->cfg.arena_bytes) {
    if (ctx->chunks.empty() && len + 16 > ctx->cfg.arena_bytes)
      return fail(ctx, KITE_ERR_BAD_INPUT, "chunk larger than the device arena");
    return fail(ctx, KITE_ERR_STATE, "device arena full: finish the segment first");
  }
  // the copy stream waits for earlier compute on the arena (a finish may be in flight)
  cudaEvent_t dep;
  KCU(cudaEventCreateWithFlags(&dep, cudaEventDisableTiming));
  KCU(cudaEventRecord(dep, ctx->stream));
  KCU(cudaStreamWaitEvent(ctx->copy_stream, dep, 0));
  cudaEventDestroy(dep);
  if (off + len + 16 > ctx->arena.cap) {
    // grow geometrically up to arena_bytes, keeping the bytes already queued
    uint64_t want = std::max<uint64_t>(off + len + 16, std::max<uint64_t>(ctx->arena.cap * 2, 64ull << 20));
    want = std::min<uint64_t>(want, ctx->cfg.arena_bytes);
    void* np = nullptr;
    KCU(cudaMalloc(&np, want));
    if (ctx->arena_used) {
      KCU(cudaMemcpyAsync(np, ctx->arena.p, ctx->arena_used, cudaMemcpyDeviceToDevice, ctx->copy_stream));
      KCU(cudaStreamSynchronize(ctx->copy_stream));
    }
    if (ctx->arena.p) cudaFree(ctx->arena.p);
    ctx->arena.p = np;
    ctx->arena.cap = want;
  }
  KCU(cudaMemcpyAsync(ctx->arena.as<uint8_t>() + off, fastq, len, cudaMemcpyHostToDevice, ctx->copy_stream));
  // zero the 16 pad bytes after the chunk (vector loads may read them)
  KCU(cudaMemsetAsync(ctx->arena.as<uint8_t>() + off + len, 0, 16, ctx->copy_stream));
  cudaEvent_t e;
  KCU(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  KCU(cudaEventRecord(e, ctx->copy_stream));
  ctx->ticket_events.push_back(e);
  ctx->chunks.push_back(Chunk{off, len, sample});
  ctx->arena_used = off + len;
  ctx->stats.h2d_bytes += len;
  return ctx->next_ticket++;
}

int kite_gpu_wait_ticket(kite_gpu_ctx* ctx, int64_t ticket) {
  if (!ctx) return KITE_ERR_BAD_INPUT;
  // tickets complete in order on the copy stream; waiting for the stream is
  // a superset of waiting for this ticket
  (void)ticket;
  return wait_stream(ctx, ctx->copy_stream);
}

int64_t kite_gpu_count_submit(kite_gpu_ctx* ctx, const uint8_t* fastq, size_t len) {
  return kite_gpu_count_submit_sample(ctx, 0, fastq, len);
}

int kite_gpu_count_submit_device_sample(kite_gpu_ctx* ctx, uint32_t sample, const uint8_t* d_fastq, size_t len) {
  if (!ctx || (!d_fastq && len)) return KITE_ERR_BAD_INPUT;
  if (sample >= (ctx->cfg.samples ? ctx->cfg.samples : 1u))
    return fail(ctx, KITE_ERR_BAD_INPUT, "sample index beyond cfg.samples");
  if (!ctx->ext_mode && !ctx->chunks.empty())
    return fail(ctx, KITE_ERR_STATE, "host and device submissions cannot mix in one segment");
  if (((uintptr_t)d_fastq) & 15) return fail(ctx, KITE_ERR_BAD_INPUT, "device chunk must be 16-byte aligned");
  if (len == 0) return KITE_OK;
  if (!ctx->ext_mode) {
    ctx->ext_mode = true;
    ctx->ext_base = d_fastq;
  }
  if (d_fastq < ctx->ext_base) return fail(ctx, KITE_ERR_BAD_INPUT, "device chunks must not precede the first one");
  ctx->chunks.push_back(Chunk{(uint64_t)(d_fastq - ctx->ext_base), len, sample});
  return KITE_OK;
}

int kite_gpu_count_submit_device(kite_gpu_ctx* ctx, const uint8_t* d_fastq, size_t len) {
  return kite_gpu_count_submit_device_sample(ctx, 0, d_fastq, len);
}

int kite_gpu_sample_totals(kite_gpu_ctx* ctx, uint32_t sample, uint64_t* totals) {
  if (!ctx || !totals) return KITE_ERR_BAD_INPUT;
  if ((size_t)sample * 3 + 3 > ctx->sample_totals.size()) return fail(ctx, KITE_ERR_BAD_INPUT, "no such sample in the last finish");
  for (int i = 0; i < 3; ++i) totals[i] = ctx->sample_totals[(size_t)sample * 3 + i];
  return KITE_OK;
}

int kite_gpu_count_finish(kite_gpu_ctx* ctx, kite_gpu_emit_fn emit, void* user) {
  if (!ctx) return KITE_ERR_BAD_INPUT;
  cudaSetDevice(ctx->cfg.device);
  int rc = ctx->cfg.k <= 31 ? run_count<uint64_t>(ctx, emit != nullptr) : run_count<u128>(ctx, emit != nullptr);
  const auto t0 = std::chrono::steady_clock::now();
  if (rc == KITE_OK) rc = emit_results(ctx, emit, user);
  ctx->stats.stage_ms[11] = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  for (auto e : ctx->ticket_events) cudaEventDestroy(e);
  ctx->ticket_events.clear();
  reset_segment(ctx);
  return rc;
}

int kite_gpu_result_partition(kite_gpu_ctx* ctx, uint32_t partition, kite_chunk_meta* meta,
                              const uint8_t** device_payload, size_t* len) {
  if (!ctx || partition >= ctx->res_meta.size()) return KITE_ERR_BAD_INPUT;
  const BucketMeta& m = ctx->res_meta[partition];
  if (meta) {
    std::memset(meta, 0, sizeof *meta);
    meta->partition_id = partition;
    meta->codec = KITE_CODEC_DVLE;
    meta->row_count = m.rows;
    meta->raw_bytes = m.bytes;
    meta->key_min_lo[0] = m.kmin_lo;
    meta->key_min_lo[1] = m.kmin_hi;
    meta->key_max_lo[0] = m.kmax_lo;
    meta->key_max_lo[1] = m.kmax_hi;
  }
  if (device_payload) *device_payload = ctx->out.as<uint8_t>() + m.byte_off;
  if (len) *len = (size_t)m.bytes;
  return KITE_OK;
}

int kite_gpu_get_stats(kite_gpu_ctx* ctx, kite_gpu_stats* out) {
  if (!ctx || !out) return KITE_ERR_BAD_INPUT;
  *out = ctx->stats;
  return KITE_OK;
}

int kite_gpu_synchronize(kite_gpu_ctx* ctx) {
  if (!ctx) return KITE_ERR_BAD_INPUT;
  int rc = wait_stream(ctx, ctx->copy_stream);
  if (!rc) rc = wait_stream(ctx, ctx->aux_stream);
  if (rc) return rc;
  return wait_stream(ctx, ctx->stream);
}

int kite_gpu_merge(kite_gpu_ctx* ctx, const kite_gpu_merge_input* inputs, int n, kite_gpu_emit_fn emit, void* user) {
  if (!ctx || !inputs || n <= 0) return KITE_ERR_BAD_INPUT;
  cudaSetDevice(ctx->cfg.device);
  std::string msg;
  MergeExtra ex;
  ex.mlp = ctx->mlp;
  ex.splitter_mode = ctx->cfg.splitter_mode;
  ex.pool = &ctx->merge_pool;
  auto staging = [ctx](size_t bytes) -> uint8_t* {
    return ctx->h_dump.ensure(bytes) == cudaSuccess ? ctx->h_dump.as<uint8_t>() : nullptr;
  };
  int rc = merge_run(ctx->cfg.k, ctx->cfg.partitions, inputs, n, ctx->stream, ctx->cfg.timeout_ms,
                     kMergeModeMerge, emit, user, &msg, &ctx->stats, staging, &ex);
  if (rc) ctx->err = msg;
  return rc;
}

int kite_gpu_dump(kite_gpu_ctx* ctx, const kite_gpu_merge_input* input, kite_gpu_emit_fn emit, void* user) {
  if (!ctx || !input) return KITE_ERR_BAD_INPUT;
  cudaSetDevice(ctx->cfg.device);
  std::string msg;
  auto staging = [ctx](size_t bytes) -> uint8_t* {
    return ctx->h_dump.ensure(bytes) == cudaSuccess ? ctx->h_dump.as<uint8_t>() : nullptr;
  };
  MergeExtra ex;
  ex.pool = &ctx->merge_pool;
  int rc = merge_run(ctx->cfg.k, ctx->cfg.partitions, input, 1, ctx->stream, ctx->cfg.timeout_ms, kMergeModeDump,
                     emit, user, &msg, &ctx->stats, staging, &ex);
  if (rc) ctx->err = msg;
  return rc;
}

int kite_gpu_histo(kite_gpu_ctx* ctx, const kite_gpu_merge_input* input, kite_gpu_histo_fn emit, void* user) {
  if (!ctx || !input) return KITE_ERR_BAD_INPUT;
  cudaSetDevice(ctx->cfg.device);
  std::string msg;
  MergeExtra ex;
  ex.histo = emit;
  ex.user = user;
  ex.pool = &ctx->merge_pool;
  int rc = merge_run(ctx->cfg.k, ctx->cfg.partitions, input, 1, ctx->stream, ctx->cfg.timeout_ms, kMergeModeHisto,
                     nullptr, nullptr, &msg, &ctx->stats, nullptr, &ex);
  if (rc) ctx->err = msg;
  return rc;
}

int kite_gpu_query(kite_gpu_ctx* ctx, const kite_gpu_merge_input* input, const uint64_t* keys, size_t n,
                   uint64_t* counts) {
  if (!ctx || !input || (n && (!keys || !counts))) return KITE_ERR_BAD_INPUT;
  cudaSetDevice(ctx->cfg.device);
  const uint32_t P = ctx->cfg.partitions;
  unsigned bits = 0;
  while ((1u << bits) < P) ++bits;
  // partition of every key (KmerWord::to_bucket src/count/kmer.rs:67-71,
  // :111-116: u128 keys fold their halves first); only those are decoded
  std::vector<uint32_t> parts(n);
  std::vector<uint64_t> pfirst(P), pcount(P, 0);
  for (size_t i = 0; i < n; ++i) {
    const uint64_t x = ctx->cfg.k <= 31 ? keys[2 * i] : (keys[2 * i] ^ keys[2 * i + 1]);
    parts[i] = bits ? (uint32_t)((x * 0x9E3779B97F4A7C15ull) >> (64 - bits)) : 0u;
  }
  for (uint32_t p = 0; p < P; ++p) pfirst[p] = input->part_first[p];
  for (size_t i = 0; i < n; ++i) pcount[parts[i]] = input->part_count[parts[i]];
  kite_gpu_merge_input sub = *input;
  sub.part_first = pfirst.data();
  sub.part_count = pcount.data();
  std::string msg;
  MergeExtra ex;
  ex.keys = keys;
  ex.parts = parts.data();
  ex.nq = n;
  ex.counts_out = counts;
  ex.pool = &ctx->merge_pool;
  int rc = merge_run(ctx->cfg.k, P, &sub, 1, ctx->stream, ctx->cfg.timeout_ms, kMergeModeQuery, nullptr, nullptr,
                     &msg, &ctx->stats, nullptr, &ex);
  if (rc) ctx->err = msg;
  return rc;
}

}  // extern "C"
