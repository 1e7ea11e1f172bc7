// `kite` command line: count / merge / dump / info with the reference's flags
// (CountArgs src/cli.rs:137-229, DumpArgs :238-282, MergeArgs :416-451) on the
// GB300 path.  Counting and merging run on the GPU through include/kite_gpu.h;
// the .kite layout comes from the host writer (include/kite_host.h).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <csignal>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <sys/stat.h>
#include <unistd.h>
#include <thread>
#include <vector>

#include "kite_gpu.h"
#include "kite_host.h"

namespace {

struct Fail {
  std::string msg;
};

[[noreturn]] void die(const std::string& m) { throw Fail{m}; }

std::string opt_str(bool has, uint32_t v) { return has ? std::to_string(v) : "none"; }

struct Args {
  std::vector<std::string> pos;
  std::vector<std::pair<std::string, std::string>> kv;
};

bool parse_bool(const std::string& v) {
  if (v == "true") return true;
  if (v == "false") return false;
  die("invalid value '" + v + "' for '--canonical <BOOL>'\n  [possible values: true, false]");
}

uint64_t parse_u64(const std::string& flag, const std::string& v) {
  if (v.empty() || v.find_first_not_of("0123456789") != std::string::npos)
    die("invalid value '" + v + "' for '" + flag + "': invalid digit found in string");
  return strtoull(v.c_str(), nullptr, 10);
}

double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

void print_command(const char* cmd, int argc, char** argv) {
  std::string s = "kite";
  for (int i = 1; i < argc; ++i) {
    s += ' ';
    s += argv[i];
  }
  fprintf(stderr, "[kite %s] Command: %s\n", cmd, s.c_str());
}

// ---------------------------------------------------------------------------
// count
// ---------------------------------------------------------------------------
// Chunks of one segment for --mode balanced | compact: copied out of the
// GPU's emit callback, compressed in parallel (kite_zstd_chunk: the
// reference's zstd "if smaller"), appended to the writer in their emit order.
struct ZstdSegment {
  kite_writer* w;
  int k, level;
  unsigned threads;
  struct Item {
    kite_chunk_meta meta;
    std::vector<uint8_t> data, z;
    int64_t zlen;
  };
  std::vector<Item> items;
  static int collect(void* user, const kite_chunk_meta* meta, const uint8_t* data, size_t len) {
    auto* s = static_cast<ZstdSegment*>(user);
    s->items.push_back(Item{*meta, std::vector<uint8_t>(data, data + len), {}, 0});
    return 0;
  }
  int flush() {
    std::atomic<size_t> next(0);
    std::atomic<int> failed(0);
    auto work = [&]() {
      for (size_t i; (i = next.fetch_add(1)) < items.size();) {
        Item& it = items[i];
        it.z.resize(kite_zstd_bound(it.data.size()) + 16);
        it.zlen = kite_zstd_chunk(k, level, &it.meta, it.data.data(), it.data.size(), it.z.data(), it.z.size());
        if (it.zlen < 0) failed = 1;
      }
    };
    std::vector<std::thread> th;
    for (unsigned t = 0; t < std::max(1u, threads); ++t) th.emplace_back(work);
    for (auto& t : th) t.join();
    if (failed) return -1;
    for (Item& it : items) {
      int r;
      if (it.zlen > 0) {
        kite_chunk_meta m = it.meta;
        m.codec |= KITE_CODEC_ZSTD;
        m.raw_bytes = it.data.size();
        r = kite_writer_append(w, &m, it.z.data(), (size_t)it.zlen);
      } else {
        r = kite_writer_append(w, &it.meta, it.data.data(), it.data.size());
      }
      if (r != 0) return -1;
    }
    items.clear();
    return 0;
  }
};

int cmd_count(int argc, char** argv) {
  std::string in, out, mem, mode = "fast", splitters = "auto";
  int k = 21, device = 0;
  bool canonical = false, has_min = false, has_max = false;
  uint32_t mn = 0, mx = 0;
  uint64_t threads = 0, partitions = 0, chunk_kmers = 0;
  int64_t buffer_mb = -1;
  for (int i = 2; i < argc; ++i) {
    std::string a = argv[i];
    auto val = [&]() -> std::string {
      if (i + 1 >= argc) die("a value is required for '" + a + "' but none was supplied");
      return argv[++i];
    };
    if (a == "-i" || a == "--input") in = val();
    else if (a == "-o" || a == "--output") out = val();
    else if (a == "-k" || a == "--kmer") k = (int)parse_u64(a, val());
    else if (a == "--canonical") canonical = parse_bool(val());
    else if (a == "--min") { has_min = true; mn = (uint32_t)parse_u64(a, val()); }
    else if (a == "--max") { has_max = true; mx = (uint32_t)parse_u64(a, val()); }
    else if (a == "--mode") mode = val();
    else if (a == "-t" || a == "--threads") threads = parse_u64(a, val());
    else if (a == "--partitions") partitions = parse_u64(a, val());
    else if (a == "--chunk-kmers") chunk_kmers = parse_u64(a, val());
    else if (a == "--memory") mem = val();
    else if (a == "--buffer") buffer_mb = (int64_t)parse_u64(a, val());
    else if (a == "-p" || a == "--progress" || a == "--test-mode") continue;
    else if (a == "--splitters") splitters = val();
    else if (a == "--device") device = (int)parse_u64(a, val());
    else die("unexpected argument '" + a + "' found");
  }
  if (in.empty() || out.empty()) die("the following required arguments were not provided: --input, --output");
  print_command("count", argc, argv);
  // run_count validation, src/count/mod.rs:210-230
  if (k < 1 || k > 128)
    die("invalid k-mer length: --k must be between 1 and 128.\nGot: " + std::to_string(k) + "\nExample: --k 21");
  if (partitions != 0 && (partitions & (partitions - 1)))
    die("invalid partition count: --partitions must be a power of 2 because kite uses partition bits for "
        "routing.\nGot: " + std::to_string(partitions) + "\nExamples: 256, 512, 1024");
  if (has_min && has_max && mn > mx)
    die("invalid count filter range: --min must be less than or equal to --max.\nGot: --min " + std::to_string(mn) +
        " --max " + std::to_string(mx));
  if (k > 64) die("k > 64 (256-bit keys) is not supported by the GPU counting path");
  if (partitions == 1) die("invalid partition count: --partitions 1 leaves no partition bits for routing");
  // CountMode::zstd_level src/cli.rs:11-19
  int zstd_level = 0;
  if (mode == "balanced") zstd_level = 2;
  else if (mode == "compact") zstd_level = 5;
  else if (mode != "fast")
    die("invalid value '" + mode + "' for '--mode <MODE>'\n  [possible values: fast, balanced, compact]");
  if (zstd_level && !kite_zstd_available())
    die("--mode " + mode + " needs zstd (libzstd.so.1), which could not be loaded; use --mode fast");
  const bool to_null = out == "/dev/null";
  if (!to_null && (out.size() < 5 || out.compare(out.size() - 5, 5, ".kite") != 0))
    die("invalid count output path: output must end with .kite, or be /dev/null for benchmark runs.\nGot: " + out +
        "\nExample: -o result.kite");
  int split_mode = splitters == "sampled" ? KITE_SPLIT_SAMPLED : splitters == "learned" ? KITE_SPLIT_LEARNED
                                                                                          : KITE_SPLIT_AUTO;
  const int64_t memb = kite_resolve_memory_limit(mem.empty() ? nullptr : mem.c_str());
  if (memb < 0) die(kite_host_last_error());
  const int comp = kite_detect_compression(in.c_str());
  if (comp < 0) die(kite_host_last_error());
  struct stat sst;
  if (stat(in.c_str(), &sst) != 0) die("failed to open input FASTQ.\nInput: " + in);
  const uint64_t total_threads = threads ? threads : std::max(1u, std::thread::hardware_concurrency());
  const double avg = partitions == 0 ? kite_sample_avg_read_len(in.c_str(), comp) : 150.0;
  kite_plan plan{};
  if (kite_derive_plan((uint64_t)sst.st_size, avg, comp, k, partitions, total_threads, (uint64_t)memb, buffer_mb,
                       chunk_kmers, &plan) != 0)
    die(kite_host_last_error());
  const double t0 = now_s();
  kite_header_info h{};
  h.k = k;
  h.canonical = canonical;
  h.partitions = (uint32_t)plan.partitions;
  h.key_width = k <= 31 ? 64 : 128;
  h.codec_mask = 7;  // RAW|DVLE|ZSTD, as count always writes (src/count/mod.rs:255)
  h.has_min = has_min;
  h.min_count = mn;
  h.has_max = has_max;
  h.max_count = mx;
  kite_writer* w = kite_writer_open(to_null ? nullptr : out.c_str(), &h, plan.staging_bytes, plan.writer_lanes);
  if (!w) die(kite_host_last_error());
  const char* comp_name[] = {"plain", "gzip", "bgzf"};
  fprintf(stderr, "[kite count] input:       %s\n[kite count] output:      %s\n", in.c_str(), out.c_str());
  fprintf(stderr, "[kite count] compression: %s\n", comp_name[comp]);
  fprintf(stderr, "[kite count] k=%d, canonical=%s, partitions=%llu, min=%s, max=%s\n", k,
          canonical ? "true" : "false", (unsigned long long)plan.partitions, opt_str(has_min, mn).c_str(),
          opt_str(has_max, mx).c_str());
  fprintf(stderr, "[kite count] mode=%s, codec=%s, device=cuda:%d\n", mode.c_str(),
          zstd_level ? "dvle+zstd-if-smaller" : "dvle-only", device);

  kite_gpu_cfg cfg{};
  cfg.device = device;
  cfg.k = k;
  cfg.canonical = canonical;
  cfg.partitions = (uint32_t)plan.partitions;
  cfg.splitter_mode = split_mode;
  kite_input* input = kite_input_open(in.c_str(), plan.chunk_size_bytes);
  if (!input) die(kite_host_last_error());
  // BGZF inflate threads: the plan's split keeps most host threads for
  // counting workers, but here the GPU counts, so every host thread inflates
  // (the split changes nothing in the output; the plan's sizes still apply)
  kite_input_set_threads(input, (unsigned)std::max<uint64_t>(plan.decomp_threads, total_threads));
  // pinned ring: the host inflates/reads chunk i+1 while chunk i is copied
  const int NBUF = 3;
  const size_t cap = (size_t)kite_input_max_chunk(input) + 64;
  std::vector<uint8_t*> ring(NBUF, nullptr);
  std::vector<int64_t> ticket(NBUF, -1);
  // The GPU context and the pinned ring are set up on a second thread while
  // this one reads the first chunks into host memory (at most kEarly of them).
  kite_gpu_ctx* ctx = nullptr;
  int rc = KITE_OK;
  bool ring_ok = true;
  std::atomic<bool> ready{false};
  std::thread setup([&]() {
    rc = kite_gpu_open(&cfg, &ctx);
    if (rc == KITE_OK)
      for (auto& b : ring) {
        b = static_cast<uint8_t*>(kite_gpu_alloc_pinned(cap));
        if (!b) ring_ok = false;
      }
    ready.store(true, std::memory_order_release);
  });
  constexpr size_t kEarly = 16;
  std::vector<std::pair<std::unique_ptr<uint8_t[]>, size_t>> early;
  bool input_done = false;
  while (!ready.load(std::memory_order_acquire) && early.size() < kEarly) {
    std::unique_ptr<uint8_t[]> b(new uint8_t[cap]);
    const int64_t n = kite_input_next(input, b.get(), cap);
    if (n < 0) {
      setup.join();
      die(kite_host_last_error());
    }
    if (n == 0) {
      input_done = true;
      break;
    }
    early.emplace_back(std::move(b), (size_t)n);
  }
  setup.join();
  if (rc != KITE_OK) die("failed to open the GPU counting context (code " + std::to_string(rc) + ")");
  if (!ring_ok) die("failed to allocate pinned host buffers");
  uint64_t reads = 0, bases = 0, kmers = 0;
  // balanced / compact: every chunk of the segment through zstd "if smaller"
  // on the host threads, then appended in partition order
  ZstdSegment zseg{w, k, zstd_level, (unsigned)total_threads, {}};
  auto finish_segment = [&]() {
    int r = zstd_level ? kite_gpu_count_finish(ctx, ZstdSegment::collect, &zseg)
                       : kite_gpu_count_finish(ctx, kite_writer_emit, w);
    if (r == KITE_OK && zstd_level && zseg.flush() != 0) die(kite_host_last_error());
    if (r != KITE_OK) die(std::string("GPU count failed: ") + kite_gpu_last_error(ctx));
    kite_gpu_stats st{};
    kite_gpu_get_stats(ctx, &st);
    reads += st.reads;
    bases += st.bases;
    kmers += st.kmers;
  };
  auto submit = [&](const uint8_t* p, size_t n) -> int64_t {
    int64_t t = kite_gpu_count_submit(ctx, p, n);
    if (t == KITE_ERR_STATE) {  // device arena full: count this segment first
      finish_segment();
      t = kite_gpu_count_submit(ctx, p, n);
    }
    if (t < 0) die(std::string("submit failed: ") + kite_gpu_last_error(ctx));
    return t;
  };
  // the early chunks: a copy from pageable memory has left the buffer when
  // the submit returns
  for (auto& b : early) {
    submit(b.first.get(), b.second);
    b.first.reset();
  }
  for (int slot = 0; !input_done; slot = (slot + 1) % NBUF) {
    if (ticket[slot] >= 0 && kite_gpu_wait_ticket(ctx, ticket[slot]) != KITE_OK)
      die(std::string("copy wait failed: ") + kite_gpu_last_error(ctx));
    const int64_t n = kite_input_next(input, ring[slot], cap);
    if (n < 0) die(kite_host_last_error());
    if (n == 0) break;
    ticket[slot] = submit(ring[slot], (size_t)n);
  }
  finish_segment();
  if (kite_writer_worker_drain(w) != 0) die(kite_host_last_error());
  uint64_t chunks = 0, rows = 0;
  if (kite_writer_finalize(w, &chunks, &rows) != 0) die(kite_host_last_error());
  kite_gpu_stats st{};
  kite_gpu_get_stats(ctx, &st);
  kite_input_close(input);
  for (auto b : ring) kite_gpu_free_pinned(b);
  kite_gpu_close(ctx);
  kite_writer_close(w);
  const double el = now_s() - t0;
  if (has_min || has_max)
    fprintf(stderr,
            "[kite count] header filter markers saved: min=%s, max=%s (raw k-mers are retained in the .kite file)\n",
            opt_str(has_min, mn).c_str(), opt_str(has_max, mx).c_str());
  fprintf(stderr,
          "[kite count] summary reads=%llu bases=%llu kmers=%llu raw_rows_written=%llu chunks=%llu header_min=%s "
          "header_max=%s elapsed=%.3fs\n",
          (unsigned long long)reads, (unsigned long long)bases, (unsigned long long)kmers, (unsigned long long)rows,
          (unsigned long long)chunks, opt_str(has_min, mn).c_str(), opt_str(has_max, mx).c_str(), el);
  fprintf(stderr, "[kite count] gpu tiles=%u per_bucket=%u big=%u imbalance=%.3f splitters=%s segments=%u\n",
          st.tiles, st.tiles_per_bucket, st.big_tiles, st.tile_imbalance,
          st.splitter_used == KITE_SPLIT_LEARNED ? "learned" : "sampled", st.segments);
  fprintf(stderr, "[kite count] done in %.3fs (%s, %llu chunks, %llu rows)\n", el, out.c_str(),
          (unsigned long long)chunks, (unsigned long long)rows);
  return 0;
}

// ---------------------------------------------------------------------------
// merge (run_merge src/merge/mod.rs:22-191)
// ---------------------------------------------------------------------------
int cmd_merge(int argc, char** argv) {
  std::vector<std::string> ins;
  std::string out;
  uint64_t threads = 0;
  int device = 0;
  for (int i = 2; i < argc; ++i) {
    std::string a = argv[i];
    if (a == "-i" || a == "--input") {
      while (i + 1 < argc && argv[i + 1][0] != '-') ins.push_back(argv[++i]);
    } else if ((a == "-o" || a == "--output") && i + 1 < argc) {
      out = argv[++i];
    } else if ((a == "-t" || a == "--threads") && i + 1 < argc) {
      threads = parse_u64(a, argv[++i]);
    } else if (a == "--device" && i + 1 < argc) {
      device = (int)parse_u64(a, argv[++i]);
    } else if (a == "-p" || a == "--progress" || a == "--test-mode") {
      continue;
    } else {
      die("unexpected argument '" + a + "' found");
    }
  }
  if (ins.size() < 2) die("2 values required for '--input <FILE> <FILE>...' but " + std::to_string(ins.size()) +
                          " was provided");
  if (out.empty()) die("the following required arguments were not provided: --output <FILE>");
  print_command("merge", argc, argv);
  const double t0 = now_s();
  fprintf(stderr, "[kite merge] inputs=%zu, output=%s\n", ins.size(), out.c_str());
  std::vector<kite_reader*> rs;
  std::vector<kite_header_info> hs;
  for (auto& p : ins) {
    kite_reader* r = kite_reader_open(p.c_str());
    if (!r) die("failed to open " + p + "\n\nCaused by:\n    " + kite_host_last_error());
    kite_header_info h{};
    kite_reader_header(r, &h, nullptr, nullptr);
    rs.push_back(r);
    hs.push_back(h);
  }
  // ensure_compatible_with_names src/kiteops/mod.rs:217-271
  auto name = [&](size_t i) { return "input #" + std::to_string(i + 1) + " (" + ins[i] + ")"; };
  for (size_t i = 1; i < hs.size(); ++i) {
    if (hs[i].k != hs[0].k)
      die("incompatible .kite inputs: " + name(i) + " has k=" + std::to_string(hs[i].k) + ", but " + name(0) +
          " has k=" + std::to_string(hs[0].k) + ".\nAll input .kite files must use the same k.");
    if ((hs[i].canonical != 0) != (hs[0].canonical != 0))
      die("incompatible .kite inputs: " + name(i) + " has a different canonical mode than " + name(0) +
          ".\nAll input .kite files must agree on canonical mode.");
    if (hs[i].partitions != hs[0].partitions)
      die("incompatible .kite inputs: " + name(i) + " has partitions=" + std::to_string(hs[i].partitions) +
          ", but " + name(0) + " has partitions=" + std::to_string(hs[0].partitions) +
          ".\nAll input .kite files must use the same partition count.");
    if (hs[i].key_width != hs[0].key_width)
      die("incompatible .kite inputs: " + name(i) + " has key_width=" + std::to_string(hs[i].key_width) + ", but " +
          name(0) + " has key_width=" + std::to_string(hs[0].key_width) +
          ".\nAll input .kite files must use the same key width.");
  }
  if (hs[0].key_width != 64 && hs[0].key_width != 128) die("merge of 256-bit keys is not supported on the GPU path");
  kite_header_info oh = hs[0];
  oh.codec_mask = 3;  // DVLE|RAW (src/merge/mod.rs:108)
  bool same_min = true, same_max = true;
  for (auto& h : hs) {
    same_min = same_min && h.has_min == hs[0].has_min && (!h.has_min || h.min_count == hs[0].min_count);
    same_max = same_max && h.has_max == hs[0].has_max && (!h.has_max || h.max_count == hs[0].max_count);
  }
  oh.has_min = same_min && hs[0].has_min;
  oh.has_max = same_max && hs[0].has_max;
  const uint64_t lanes = kite_suggest_write_lanes(std::max(1u, std::thread::hardware_concurrency()));
  kite_writer* w = kite_writer_open(out.c_str(), &oh, 16ull << 20, lanes);
  if (!w) die(kite_host_last_error());
  kite_gpu_cfg cfg{};
  cfg.device = device;
  cfg.k = oh.k;
  cfg.canonical = oh.canonical;
  cfg.partitions = oh.partitions;
  kite_gpu_ctx* ctx = nullptr;
  if (kite_gpu_open(&cfg, &ctx) != KITE_OK) die("failed to open the GPU merge context");
  std::vector<kite_gpu_merge_input> mi(rs.size());
  for (size_t i = 0; i < rs.size(); ++i) kite_reader_merge_input(rs[i], &mi[i]);
  int rc = kite_gpu_merge(ctx, mi.data(), (int)mi.size(), kite_writer_emit, w);
  if (rc != KITE_OK) die(kite_gpu_last_error(ctx));
  uint64_t chunks = 0, rows = 0;
  if (kite_writer_finalize(w, &chunks, &rows) != 0) die(kite_host_last_error());
  kite_writer_close(w);
  kite_gpu_close(ctx);
  const double el = now_s() - t0;
  // merge report (write_merge_report src/merge/mod.rs:226-301)
  std::string stem = out, parent;
  size_t slash = out.find_last_of('/');
  if (slash != std::string::npos) {
    parent = out.substr(0, slash + 1);
    stem = out.substr(slash + 1);
  }
  size_t dot = stem.find_last_of('.');
  if (dot != std::string::npos && dot > 0) stem = stem.substr(0, dot);
  const std::string report = parent + stem + ".merge_report.md";
  if (FILE* f = fopen(report.c_str(), "w")) {
    const uint64_t wt = threads ? threads : std::max(1u, std::thread::hardware_concurrency());
    fprintf(f, "# Kite Merge Report\n\n## Summary\n\n| Field | Value |\n|---|---:|\n");
    fprintf(f, "| Inputs | %zu |\n| Output rows | %llu |\n| Output chunks | %llu |\n| Partitions | %u |\n",
            ins.size(), (unsigned long long)rows, (unsigned long long)chunks, oh.partitions);
    fprintf(f, "| Threads requested | %llu |\n| Worker threads used | %llu |\n| Elapsed seconds | %.3f |\n\n",
            (unsigned long long)threads, (unsigned long long)wt, el);
    fprintf(f, "## Compatibility\n\n| Field | Value |\n|---|---:|\n| k | %d |\n| Canonical | %s |\n| Key width | %u |\n\n",
            oh.k, oh.canonical ? "true" : "false", oh.key_width);
    fprintf(f, "## Downstream Filter Semantics\n\nInput header min/max filters are applied before merge. The output "
               "header retains a min or max marker only when all inputs share the same marker.\n\n");
    fprintf(f, "- Output min: %s\n- Output max: %s\n\n", opt_str(oh.has_min, oh.min_count).c_str(),
            opt_str(oh.has_max, oh.max_count).c_str());
    fprintf(f, "## Inputs\n\n| # | Path | k | Canonical | Partitions | Key width | Rows | Chunks | Min | Max |\n");
    fprintf(f, "|---:|---|---:|---:|---:|---:|---:|---:|---:|---:|\n");
    for (size_t i = 0; i < rs.size(); ++i) {
      uint64_t tc = 0, tr = 0;
      kite_reader_header(rs[i], nullptr, &tc, &tr);
      fprintf(f, "| %zu | `%s` | %d | %s | %u | %u | %llu | %llu | %s | %s |\n", i + 1, ins[i].c_str(), hs[i].k,
              hs[i].canonical ? "true" : "false", hs[i].partitions, hs[i].key_width, (unsigned long long)tr,
              (unsigned long long)tc, opt_str(hs[i].has_min, hs[i].min_count).c_str(),
              opt_str(hs[i].has_max, hs[i].max_count).c_str());
    }
    fprintf(f, "\n## Output\n\n- File: `%s`\n- Report: `%s`\n", out.c_str(), report.c_str());
    fclose(f);
  }
  for (auto r : rs) kite_reader_close(r);
  fprintf(stderr, "[kite merge] wrote %llu rows across %llu chunks in %.3fs (report=%s)\n", (unsigned long long)rows,
          (unsigned long long)chunks, el, report.c_str());
  return 0;
}

// ---------------------------------------------------------------------------
// dump (run_dump src/dump/mod.rs:183-520): partitions in order, TSV lines,
// merged, filtered and formatted on the GPU (kite_gpu_dump)
// ---------------------------------------------------------------------------
int dump_write(void* user, const kite_chunk_meta*, const uint8_t* data, size_t len) {
  return fwrite(data, 1, len, static_cast<FILE*>(user)) == len ? 0 : 1;
}

int cmd_dump(int argc, char** argv) {
  std::string in, out;
  int device = 0;
  for (int i = 2; i < argc; ++i) {
    std::string a = argv[i];
    if ((a == "-i" || a == "--input") && i + 1 < argc) in = argv[++i];
    else if ((a == "-o" || a == "--output") && i + 1 < argc) out = argv[++i];
    else if (a == "--device" && i + 1 < argc) device = (int)parse_u64(a, argv[++i]);
    else if ((a == "-t" || a == "--threads" || a == "--buffer") && i + 1 < argc) ++i;
    else if (a == "-p" || a == "--progress" || a == "--test-mode") continue;
    else die("unexpected argument '" + a + "' found");
  }
  if (in.empty() || out.empty()) die("the following required arguments were not provided: --input, --output");
  print_command("dump", argc, argv);
  kite_reader* r = kite_reader_open(in.c_str());
  if (!r) die(kite_host_last_error());
  kite_header_info h{};
  uint64_t tc = 0, tr = 0;
  kite_reader_header(r, &h, &tc, &tr);
  fprintf(stderr, "[kite dump] opening: %s\n[kite dump] output:  %s\n", in.c_str(), out.c_str());
  fprintf(stderr, "[kite dump] k=%d, partitions=%u, total_chunks=%llu\n", h.k, h.partitions, (unsigned long long)tc);
  fprintf(stderr, "[kite dump] header filters min=%s, max=%s\n", opt_str(h.has_min, h.min_count).c_str(),
          opt_str(h.has_max, h.max_count).c_str());
  if (h.key_width != 64 && h.key_width != 128) die("dump of 256-bit keys is not supported on the GPU path");
  FILE* f = out == "-" ? stdout : fopen(out.c_str(), "wb");
  if (!f) die("failed to create " + out);
  const double t0 = now_s();
  kite_gpu_cfg cfg{};
  cfg.device = device;
  cfg.k = h.k;
  cfg.canonical = h.canonical;
  cfg.partitions = h.partitions;
  kite_gpu_ctx* ctx = nullptr;
  if (kite_gpu_open(&cfg, &ctx) != KITE_OK) die("failed to open the GPU dump context");
  kite_gpu_merge_input mi{};
  kite_reader_merge_input(r, &mi);
  const int rc = kite_gpu_dump(ctx, &mi, dump_write, f);
  if (rc == KITE_ERR_CALLBACK) die("write failed");
  if (rc != KITE_OK) die(kite_gpu_last_error(ctx));
  kite_gpu_close(ctx);
  if (f == stdout) fflush(stdout);
  else fclose(f);
  kite_reader_close(r);
  fprintf(stderr, "[kite dump] done in %.3fs\n", now_s() - t0);
  return 0;
}

// ---------------------------------------------------------------------------
// info (run_info src/info/mod.rs:14): header summary; --set/--clear-min/max
// rewrite the header markers in place (update_count_filters_in_file
// src/format/header.rs:166-183)
// ---------------------------------------------------------------------------
int cmd_info(int argc, char** argv) {
  std::string in;
  bool set_min = false, set_max = false, clear_min = false, clear_max = false;
  uint32_t nmin = 0, nmax = 0;
  for (int i = 2; i < argc; ++i) {
    std::string a = argv[i];
    if ((a == "-i" || a == "--input") && i + 1 < argc) in = argv[++i];
    else if (a == "--set-min" && i + 1 < argc) { set_min = true; nmin = (uint32_t)parse_u64(a, argv[++i]); }
    else if (a == "--set-max" && i + 1 < argc) { set_max = true; nmax = (uint32_t)parse_u64(a, argv[++i]); }
    else if (a == "--clear-min") clear_min = true;
    else if (a == "--clear-max") clear_max = true;
    else die("unexpected argument '" + a + "' found");
  }
  if (set_min && clear_min) die("--set-min and --clear-min cannot be used together");
  if (set_max && clear_max) die("--set-max and --clear-max cannot be used together");
  kite_reader* r = kite_reader_open(in.c_str());
  if (!r) die(kite_host_last_error());
  kite_header_info h{};
  uint64_t tc = 0, tr = 0;
  kite_reader_header(r, &h, &tc, &tr);
  kite_reader_close(r);
  if (set_min || set_max || clear_min || clear_max) {
    kite_header_info nh = h;
    if (clear_min) nh.has_min = 0;
    else if (set_min) { nh.has_min = 1; nh.min_count = nmin; }
    if (clear_max) nh.has_max = 0;
    else if (set_max) { nh.has_max = 1; nh.max_count = nmax; }
    if (nh.has_min && nh.has_max && nh.min_count > nh.max_count)
      die("header min (" + std::to_string(nh.min_count) + ") must be <= header max (" + std::to_string(nh.max_count) + ")");
    FILE* f = fopen(in.c_str(), "r+b");
    if (!f) die("failed to open " + in);
    uint8_t res[68] = {0};
    if (nh.has_min || nh.has_max) {
      memcpy(res, "KMT1", 4);
      uint32_t flags = (nh.has_min ? 1u : 0u) | (nh.has_max ? 2u : 0u);
      uint32_t mn = nh.has_min ? nh.min_count : 0, mx = nh.has_max ? nh.max_count : 0;
      memcpy(res + 4, &flags, 4);
      memcpy(res + 8, &mn, 4);
      memcpy(res + 12, &mx, 4);
    }
    fseek(f, 60, SEEK_SET);
    fwrite(res, 1, 68, f);
    fclose(f);
    fprintf(stderr, "[kite info] updated header count filters: min=%s, max=%s\n",
            opt_str(nh.has_min, nh.min_count).c_str(), opt_str(nh.has_max, nh.max_count).c_str());
    h = nh;
  }
  printf("file\t%s\nk\t%d\ncanonical\t%s\npartitions\t%u\nkey_width\t%u\ncodec_mask\t%u\ntotal_chunks\t%llu\n"
         "total_rows\t%llu\nmin\t%s\nmax\t%s\n",
         in.c_str(), h.k, h.canonical ? "true" : "false", h.partitions, h.key_width, h.codec_mask,
         (unsigned long long)tc, (unsigned long long)tr, opt_str(h.has_min, h.min_count).c_str(),
         opt_str(h.has_max, h.max_count).c_str());
  return 0;
}

void on_sigint(int) {
  static const char msg[] = "\n[kite] interrupted\n";
  (void)!write(2, msg, sizeof msg - 1);
  _exit(130);
}

}  // namespace

// ---------------------------------------------------------------------------
// histo (run_histo src/histo/mod.rs:16-169): per input, counts summed per key
// over its chunks, header filter, count -> frequency on the GPU
// (kite_gpu_histo); one row per count over all inputs, one column per input.
// Labels: --label, else file names without the suffixes of
// infer_sample_labels (src/kiteops/mod.rs:123-165).
// ---------------------------------------------------------------------------
std::string label_from_path(const std::string& path, size_t index) {
  const size_t slash = path.find_last_of('/');
  std::string name = slash == std::string::npos ? path : path.substr(slash + 1);
  for (const char* suf : {".fastq.gz", ".fq.gz", ".fastq", ".fq", ".kite", ".tsv", ".txt", ".gz"}) {
    const size_t l = strlen(suf);
    if (name.size() >= l && name.compare(name.size() - l, l, suf) == 0) {
      name.resize(name.size() - l);
      break;
    }
  }
  return name.empty() ? "sample" + std::to_string(index + 1) : name;
}

int histo_add(void* user, uint64_t count, uint64_t keys) {
  (*static_cast<std::map<uint64_t, uint64_t>*>(user))[count] = keys;
  return 0;
}

int cmd_histo(int argc, char** argv) {
  std::vector<std::string> ins, labels;
  std::string out;
  int device = 0;
  for (int i = 2; i < argc; ++i) {
    std::string a = argv[i];
    if (a == "-i" || a == "--input") {
      while (i + 1 < argc && argv[i + 1][0] != '-') ins.push_back(argv[++i]);
    } else if (a == "--label") {
      while (i + 1 < argc && argv[i + 1][0] != '-') labels.push_back(argv[++i]);
    } else if ((a == "-o" || a == "--output") && i + 1 < argc) out = argv[++i];
    else if (a == "--device" && i + 1 < argc) device = (int)parse_u64(a, argv[++i]);
    else if ((a == "-t" || a == "--threads") && i + 1 < argc) ++i;
    else if (a == "-p" || a == "--progress" || a == "--test-mode") continue;
    else die("unexpected argument '" + a + "' found");
  }
  if (ins.empty() || out.empty()) die("the following required arguments were not provided: --input, --output");
  if (!labels.empty() && labels.size() != ins.size())
    die("--label count (" + std::to_string(labels.size()) + ") must match input count (" +
        std::to_string(ins.size()) + ")");
  if (labels.empty())
    for (size_t i = 0; i < ins.size(); ++i) labels.push_back(label_from_path(ins[i], i));
  print_command("histo", argc, argv);
  const double t0 = now_s();
  std::vector<std::map<uint64_t, uint64_t>> hs(ins.size());
  std::map<uint64_t, int> bins;
  for (size_t i = 0; i < ins.size(); ++i) {
    kite_reader* r = kite_reader_open(ins[i].c_str());
    if (!r) die(kite_host_last_error());
    kite_header_info h{};
    uint64_t tc = 0, tr = 0;
    kite_reader_header(r, &h, &tc, &tr);
    if (h.key_width != 64 && h.key_width != 128) die("histo of 256-bit keys is not supported on the GPU path");
    kite_gpu_cfg cfg{};
    cfg.device = device;
    cfg.k = h.k;
    cfg.canonical = h.canonical;
    cfg.partitions = h.partitions;
    kite_gpu_ctx* ctx = nullptr;
    if (kite_gpu_open(&cfg, &ctx) != KITE_OK) die("failed to open the GPU histo context");
    kite_gpu_merge_input mi{};
    kite_reader_merge_input(r, &mi);
    if (kite_gpu_histo(ctx, &mi, histo_add, &hs[i]) != KITE_OK) die(kite_gpu_last_error(ctx));
    kite_gpu_close(ctx);
    kite_reader_close(r);
    for (auto& kv : hs[i]) bins[kv.first] = 1;
  }
  FILE* f = out == "-" ? stdout : fopen(out.c_str(), "wb");
  if (!f) die("failed to create " + out);
  fprintf(f, "count");
  for (auto& l : labels) fprintf(f, "\t%s", l.c_str());
  fprintf(f, "\n");
  for (auto& b : bins) {
    fprintf(f, "%llu", (unsigned long long)b.first);
    for (auto& h : hs) {
      auto it = h.find(b.first);
      fprintf(f, "\t%llu", (unsigned long long)(it == h.end() ? 0 : it->second));
    }
    fprintf(f, "\n");
  }
  if (f == stdout) fflush(stdout);
  else fclose(f);
  fprintf(stderr, "[kite histo] done in %.3fs (bins=%zu, output=%s)\n", now_s() - t0, bins.size(), out.c_str());
  return 0;
}

// ---------------------------------------------------------------------------
// query (run_query src/query/mod.rs:15-96): encode_query_kmer
// (src/kiteops/mod.rs:302-348: length k, ACGT only, canonical if the
// database is), its partition, its summed count (kite_gpu_query), and the
// report with the header filter's outcome.
// ---------------------------------------------------------------------------
int cmd_query(int argc, char** argv) {
  std::string in, kmer;
  int device = 0;
  for (int i = 2; i < argc; ++i) {
    std::string a = argv[i];
    if ((a == "-i" || a == "--input") && i + 1 < argc) in = argv[++i];
    else if ((a == "-k" || a == "--kmer") && i + 1 < argc) kmer = argv[++i];
    else if (a == "--device" && i + 1 < argc) device = (int)parse_u64(a, argv[++i]);
    else if (a == "--test-mode") continue;
    else die("unexpected argument '" + a + "' found");
  }
  if (in.empty() || kmer.empty()) die("the following required arguments were not provided: --input, --kmer");
  print_command("query", argc, argv);
  fprintf(stderr, "[kite query] opening: %s\n[kite query] query:   %s\n", in.c_str(), kmer.c_str());
  const double t0 = now_s();
  kite_reader* r = kite_reader_open(in.c_str());
  if (!r) die(kite_host_last_error());
  kite_header_info h{};
  uint64_t tc = 0, tr = 0;
  kite_reader_header(r, &h, &tc, &tr);
  if (h.key_width != 64 && h.key_width != 128) die("query of 256-bit keys is not supported on the GPU path");
  if (kmer.size() != (size_t)h.k)
    die("query k-mer length " + std::to_string(kmer.size()) + " does not match database k=" + std::to_string(h.k));
  unsigned __int128 fwd = 0, rev = 0;
  for (size_t i = 0; i < kmer.size(); ++i) {
    const char c = kmer[i];
    const char* pos = strchr("ACGT", c >= 'a' && c <= 'z' ? c - 32 : c);
    if (!pos || c == 0) die("query k-mer contains non-ACGT characters");
    const unsigned b = (unsigned)(pos - "ACGT");
    fwd = (fwd << 2) | b;
    rev |= (unsigned __int128)(3 - b) << (2 * i);
  }
  const unsigned __int128 key = h.canonical && rev < fwd ? rev : fwd;
  const uint64_t kw[2] = {(uint64_t)key, (uint64_t)(key >> 64)};
  unsigned bits = 0;
  while ((1u << bits) < h.partitions) ++bits;
  const uint64_t x = h.key_width == 64 ? kw[0] : (kw[0] ^ kw[1]);
  const uint64_t part = bits ? (x * 0x9E3779B97F4A7C15ull) >> (64 - bits) : 0;
  kite_gpu_cfg cfg{};
  cfg.device = device;
  cfg.k = h.k;
  cfg.canonical = h.canonical;
  cfg.partitions = h.partitions;
  kite_gpu_ctx* ctx = nullptr;
  if (kite_gpu_open(&cfg, &ctx) != KITE_OK) die("failed to open the GPU query context");
  kite_gpu_merge_input mi{};
  kite_reader_merge_input(r, &mi);
  uint64_t count = 0;
  if (kite_gpu_query(ctx, &mi, kw, 1, &count) != KITE_OK) die(kite_gpu_last_error(ctx));
  kite_gpu_close(ctx);
  std::string ks(h.k, 'A');
  for (int i = 0; i < h.k; ++i) ks[i] = "ACGT"[(unsigned)(key >> (2 * (h.k - 1 - i))) & 3u];
  const bool pass = !(h.has_min && count < h.min_count) && !(h.has_max && count > h.max_count);
  printf("Kite Query\n  Database:           %s\n  Query:              %s\n  Partition:          %llu\n"
         "  Count:              %llu\n  Header Min Count:   %s\n  Header Max Count:   %s\n  Header Filter:      %s\n",
         in.c_str(), ks.c_str(), (unsigned long long)part, (unsigned long long)count,
         opt_str(h.has_min, h.min_count).c_str(), opt_str(h.has_max, h.max_count).c_str(),
         count == 0 ? "not present" : (pass ? "included" : "excluded from downstream analysis/output"));
  fflush(stdout);
  kite_reader_close(r);
  fprintf(stderr, "[kite query] done in %.3fs\n", now_s() - t0);
  return 0;
}

int main(int argc, char** argv) {
  std::signal(SIGINT, on_sigint);  // ctrl-c exits 130 (src/main.rs:21-25)
  if (argc < 2) {
    fprintf(stderr, "Usage: kite <count|merge|dump|histo|query|info> [OPTIONS]\n");
    return 2;
  }
  const std::string cmd = argv[1];
  try {
    if (cmd == "count") return cmd_count(argc, argv);
    if (cmd == "merge") return cmd_merge(argc, argv);
    if (cmd == "dump") return cmd_dump(argc, argv);
    if (cmd == "info") return cmd_info(argc, argv);
    if (cmd == "histo") return cmd_histo(argc, argv);
    if (cmd == "query") return cmd_query(argc, argv);
    fprintf(stderr, "error: unrecognized subcommand '%s'\n", cmd.c_str());
    return 2;
  } catch (const Fail& f) {
    fprintf(stderr, "Error: %s\n", f.msg.c_str());
    return 1;
  }
}
