// kite_oracle.cpp — TEST INFRASTRUCTURE, NOT PRODUCT CODE.
//
// A plain CPU restatement of the reference's exact k-mer counting path
// (jiehua1995/Kite v0.7.5): `kite count`, `kite dump` and `kite merge`
// for k <= 64 (u64 and u128 keys), in fast, balanced and compact modes (zstd
// through the system's libzstd.so.1).  It exists only so
// that tests/ and bench.py's CPU baseline can check and time the GPU path;
// nothing under kite_gb300/ links, imports or executes it.
//
// Every function names the reference file:line it restates.  Where the
// reference depends on thread scheduling (several count workers racing on
// the writer) the oracle reproduces the single-worker order, which is the
// only order in which the reference's `.kite` bytes are reproducible.
//
// Parity is pinned by the reference's own unit-test vectors
// (tests/golden/reference_vectors.json, exercised by tests/test_oracle.py).
//
// Build: `make -C oracle` (see oracle/Makefile) produces
//   oracle/_build/liboracle.so   (C API below, loaded by tests through ctypes)
//   oracle/_build/kite_oracle    (CLI: count / dump / merge / info)

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <dlfcn.h>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#if __has_include(<zlib.h>)
#include <zlib.h>
#define ORC_HAVE_ZLIB 1
#else
#define ORC_HAVE_ZLIB 0
#endif

typedef unsigned __int128 u128;

namespace orc {

static const size_t MIB = 1024ull * 1024ull;
static const size_t GIB = 1024ull * MIB;

struct Error : std::runtime_error {
  explicit Error(const std::string& m) : std::runtime_error(m) {}
};

// ---------------------------------------------------------------------------
// Base encoding: src/count/kmer.rs:2-13 (A/a=0, C/c=1, G/g=2, T/t=3, else 255)
// ---------------------------------------------------------------------------
static uint8_t g_base[256];
static bool g_base_init = [] {
  for (int i = 0; i < 256; ++i) g_base[i] = 255;
  g_base['A'] = g_base['a'] = 0;
  g_base['C'] = g_base['c'] = 1;
  g_base['G'] = g_base['g'] = 2;
  g_base['T'] = g_base['t'] = 3;
  return true;
}();

// ---------------------------------------------------------------------------
// Rolling k-mer iterators: KmerIter::next src/count/kmer.rs:241-267 (u64),
// KmerIter128::next src/count/kmer.rs:311-337 (u128).  A non-ACGT byte resets
// the window; canonical = min(fwd, revcomp) as integers.
// ---------------------------------------------------------------------------
template <class T, class F>
static void scan_kmers(const uint8_t* s, size_t n, unsigned k, bool canonical, F&& f) {
  const unsigned tbits = sizeof(T) * 8;
  const T mask = (2 * k == tbits) ? ~T(0) : ((T(1) << (2 * k)) - 1);
  const unsigned shift = 2 * (k - 1);
  T fwd = 0, rev = 0;
  uint32_t valid = 0;
  for (size_t i = 0; i < n; ++i) {
    uint8_t enc = g_base[s[i]];
    if (enc == 255) {
      fwd = 0;
      rev = 0;
      valid = 0;
      continue;
    }
    fwd = ((fwd << 2) | T(enc)) & mask;
    rev = (rev >> 2) | (T(enc ^ 3) << shift);
    valid += 1;
    if (valid >= k) f(canonical ? (fwd < rev ? fwd : rev) : fwd);
  }
}

// ---------------------------------------------------------------------------
// Partition (bucket) of a key: Fibonacci hash, src/count/kmer.rs:67-71 (u64),
// :111-116 (u128 XOR-folds hi^lo first); kiteops bucket_for_key :282-300.
// ---------------------------------------------------------------------------
static inline size_t bucket_of(uint64_t key, unsigned bits) {
  return (size_t)((key * 0x9E3779B97F4A7C15ull) >> (64 - bits));
}
static inline size_t bucket_of(u128 key, unsigned bits) {
  uint64_t lo = (uint64_t)key, hi = (uint64_t)(key >> 64);
  return bucket_of(lo ^ hi, bits);
}

// ---------------------------------------------------------------------------
// FASTQ parser: parse_sequences src/count/parser.rs:19-65.  Yields line 2 of
// every 4-line record (no trimming); a chunk not starting with '@' is an error
// which the count worker ignores (src/count/worker.rs:217).
// ---------------------------------------------------------------------------
template <class F>
static bool parse_sequences(const uint8_t* d, size_t len, F&& on_seq) {
  if (len == 0) return true;
  if (d[0] != '@') return false;
  int state = 0;  // 0 header, 1 seq, 2 plus, 3 qual
  size_t seq_start = 0;
  for (size_t i = 0; i < len; ++i) {
    if (d[i] != '\n') continue;
    switch (state) {
      case 0: state = 1; seq_start = i + 1; break;
      case 1:
        if (i > seq_start) on_seq(d + seq_start, i - seq_start);
        state = 2;
        break;
      case 2: state = 3; break;
      default: state = 0; break;
    }
  }
  if (state == 1 && seq_start < len) on_seq(d + seq_start, len - seq_start);
  return true;
}

// find_fastq_split_4lines: src/count/bgzf.rs:109-121
static size_t find_fastq_split_4lines(const uint8_t* d, size_t n) {
  size_t newlines = 0, last = 0;
  for (size_t i = 0; i < n; ++i)
    if (d[i] == '\n') {
      ++newlines;
      if (newlines % 4 == 0) last = i + 1;
    }
  return last;
}

// ---------------------------------------------------------------------------
// Input sniffing and chunked readers:
//   detect_compression src/count/reader.rs:22-51
//   PlainChunkedReader::next_chunk src/count/decompress.rs:104-138
//   GzipChunkedReader::next_chunk  src/count/decompress.rs:36-81 (multi-member)
// ---------------------------------------------------------------------------
enum Compression { PLAIN = 0, GZIP = 1, BGZF = 2 };

static Compression detect_compression(const std::string& path) {
  FILE* f = fopen(path.c_str(), "rb");
  if (!f) throw Error("failed to inspect input FASTQ compression.\nInput: " + path);
  uint8_t h[18];
  size_t n = fread(h, 1, 18, f);
  fclose(f);
  if (n < 2) return PLAIN;
  if (h[0] != 0x1f || h[1] != 0x8b) return PLAIN;
  if (n >= 18 && (h[3] & 0x04)) {
    size_t xlen = (size_t)h[10] | ((size_t)h[11] << 8);
    if (xlen >= 6 && h[12] == 0x42 && h[13] == 0x43) return BGZF;
  }
  return GZIP;
}

struct ByteSource {
  virtual ~ByteSource() {}
  // returns bytes read, 0 at EOF
  virtual size_t read(uint8_t* dst, size_t cap) = 0;
};

struct FileSource : ByteSource {
  FILE* f;
  explicit FileSource(const std::string& p) {
    f = fopen(p.c_str(), "rb");
    if (!f) throw Error("failed to open input FASTQ.\nInput: " + p);
  }
  ~FileSource() { if (f) fclose(f); }
  size_t read(uint8_t* dst, size_t cap) override { return fread(dst, 1, cap, f); }
};

#if ORC_HAVE_ZLIB
struct GzSource : ByteSource {
  gzFile g;
  explicit GzSource(const std::string& p) {
    g = gzopen(p.c_str(), "rb");
    if (!g) throw Error("failed to open input FASTQ.\nInput: " + p);
    gzbuffer(g, 1 << 20);
  }
  ~GzSource() { if (g) gzclose(g); }
  size_t read(uint8_t* dst, size_t cap) override {
    size_t total = 0;
    while (total < cap) {
      unsigned want = (unsigned)std::min<size_t>(cap - total, 1u << 30);
      int r = gzread(g, dst + total, want);
      if (r < 0) {
        int e = 0;
        throw Error(std::string("decompress_error: ") + gzerror(g, &e));
      }
      if (r == 0) break;
      total += (size_t)r;
    }
    return total;
  }
};
#endif

struct ChunkedReader {
  ByteSource* src;
  size_t chunk_size;
  std::vector<uint8_t> carry;
  ChunkedReader(ByteSource* s, size_t cs) : src(s), chunk_size(cs) {}
  bool next_chunk(std::vector<uint8_t>& chunk) {
    chunk.clear();
    chunk.insert(chunk.end(), carry.begin(), carry.end());
    carry.clear();
    size_t base = chunk.size();
    chunk.resize(base + chunk_size);
    size_t total = 0;
    while (total < chunk_size) {
      size_t r = src->read(chunk.data() + base + total, chunk_size - total);
      if (r == 0) break;
      total += r;
    }
    chunk.resize(base + total);
    if (chunk.empty()) return false;
    if (total < chunk_size) return true;
    size_t split = find_fastq_split_4lines(chunk.data(), chunk.size());
    if (split == 0 || split >= chunk.size()) return true;
    carry.assign(chunk.begin() + split, chunk.end());
    chunk.resize(split);
    return true;
  }
};

static ByteSource* open_source(const std::string& path, Compression c) {
  if (c == PLAIN) return new FileSource(path);
#if ORC_HAVE_ZLIB
  return new GzSource(path);  // gzread continues across gzip members
#else
  throw Error("gzip input needs zlib, which this binary is not compiled with");
#endif
}

// ---------------------------------------------------------------------------
// BGZF input:
//   is_bgzf_header / scan_bgzf_blocks  src/count/bgzf.rs:37-85
//   find_fastq_split_near              src/count/bgzf.rs:124-135
//   decompress_bgzf_parallel           src/count/bgzf.rs:149-258: blocks
//     inflated one by one here; the reference's batches and thread pool do
//     not move a chunk boundary, since it appends block by block and cuts
//     after every block
//   sample_bgzf_input                  src/count/mod.rs:1081-1123
// ---------------------------------------------------------------------------
static std::vector<uint8_t> read_whole_file(const std::string& path) {
  FILE* f = fopen(path.c_str(), "rb");
  if (!f) throw Error("failed to open input FASTQ.\nInput: " + path);
  std::vector<uint8_t> d;
  uint8_t buf[1 << 16];
  size_t r;
  while ((r = fread(buf, 1, sizeof buf, f)) > 0) d.insert(d.end(), buf, buf + r);
  fclose(f);
  return d;
}

static std::vector<std::pair<size_t, size_t>> scan_bgzf_blocks(const std::vector<uint8_t>& d) {
  std::vector<std::pair<size_t, size_t>> blocks;
  size_t pos = 0;
  while (pos + 18 <= d.size()) {
    const uint8_t* h = d.data() + pos;
    const bool hdr = h[0] == 0x1f && h[1] == 0x8b && (h[3] & 0x04) && h[12] == 0x42 && h[13] == 0x43 &&
                     h[14] == 0x02 && h[15] == 0x00;
    if (!hdr) throw Error("Non-BGZF data at offset " + std::to_string(pos) + " (expected gzip+BGZF header)");
    const size_t bsize = ((size_t)h[16] | ((size_t)h[17] << 8)) + 1;
    if (pos + bsize > d.size()) break;  // truncated final block: skipped
    blocks.push_back({pos, bsize});
    pos += bsize;
  }
  return blocks;
}

// One gzip member; on a decode error the bytes decoded so far are kept (the
// reference ignores read_to_end's error in the count path).  Returns false
// on that error.
static bool inflate_member(const uint8_t* raw, size_t n, std::vector<uint8_t>& out) {
  out.clear();
#if ORC_HAVE_ZLIB
  z_stream zs{};
  if (inflateInit2(&zs, 15 + 16) != Z_OK) return false;
  zs.next_in = const_cast<uint8_t*>(raw);
  zs.avail_in = (uInt)n;
  uint8_t buf[1 << 16];
  int r = Z_OK;
  while (r == Z_OK) {
    zs.next_out = buf;
    zs.avail_out = sizeof buf;
    r = inflate(&zs, Z_NO_FLUSH);
    out.insert(out.end(), buf, buf + (sizeof buf - zs.avail_out));
    if (r == Z_BUF_ERROR && zs.avail_in == 0) break;
  }
  inflateEnd(&zs);
  return r == Z_STREAM_END;
#else
  (void)raw;
  (void)n;
  throw Error("gzip input needs zlib, which this binary is not compiled with");
#endif
}

static size_t find_fastq_split_near(const uint8_t* d, size_t n, size_t target) {
  const size_t scan_end = std::min(target + 8192, n);
  const size_t b = find_fastq_split_4lines(d, scan_end);
  return b > 0 ? b : find_fastq_split_4lines(d, n);
}

// Chunks of a BGZF file; a scan error is reported like the reference's
// reader thread and yields no chunks.
static void bgzf_chunks(const std::string& path, size_t target, std::vector<std::vector<uint8_t>>& chunks) {
  const std::vector<uint8_t> d = read_whole_file(path);
  std::vector<std::pair<size_t, size_t>> blocks;
  try {
    blocks = scan_bgzf_blocks(d);
  } catch (const Error& e) {
    fprintf(stderr, "[kite count] bgzf_decompress_error: %s\n", e.what());
    return;
  }
  std::vector<uint8_t> carry, out;
  for (auto& b : blocks) {
    inflate_member(d.data() + b.first, b.second, out);
    if (out.empty()) continue;
    carry.insert(carry.end(), out.begin(), out.end());
    while (carry.size() >= target) {
      const size_t split = find_fastq_split_near(carry.data(), carry.size(), target);
      if (split == 0) break;
      chunks.emplace_back(carry.begin(), carry.begin() + split);
      carry.erase(carry.begin(), carry.begin() + split);
    }
  }
  if (!carry.empty()) chunks.push_back(carry);
}

static void read_all_chunks(const std::string& path, Compression c, size_t chunk_size,
                            std::vector<std::vector<uint8_t>>& store) {
  if (c == BGZF) {
    bgzf_chunks(path, chunk_size, store);
    return;
  }
  std::unique_ptr<ByteSource> src(open_source(path, c));
  ChunkedReader rd(src.get(), chunk_size);
  std::vector<uint8_t> chunk;
  while (rd.next_chunk(chunk)) store.push_back(chunk);
}

// ---------------------------------------------------------------------------
// Runtime memory spec: parse_memory_spec src/runtime.rs:6-54,
// resolve_memory_limit_bytes :56-71 (auto = 2/3 of MemAvailable).
// ---------------------------------------------------------------------------
static size_t parse_memory_spec(const std::string& spec) {
  bool digits = !spec.empty();
  for (char c : spec) digits = digits && (c >= '0' && c <= '9');
  auto bad = [&](const std::string& why) { return Error("invalid memory size '" + spec + "': " + why); };
  if (digits) {
    unsigned long long v = strtoull(spec.c_str(), nullptr, 10);
    if (v == 0) throw bad("value must be greater than zero");
    return (size_t)v;
  }
  if (spec.size() < 2) throw bad("expected formats like 512M, 64G, 1T, or raw bytes");
  char suf = spec.back();
  size_t mul = suf == 'M' ? MIB : suf == 'G' ? GIB : suf == 'T' ? 1024 * GIB : 0;
  if (!mul) throw bad("suffix must be M, G, or T");
  std::string num = spec.substr(0, spec.size() - 1);
  bool ok = !num.empty();
  for (char c : num) ok = ok && (c >= '0' && c <= '9');
  if (!ok) throw bad("numeric part must be a positive integer");
  unsigned long long v = strtoull(num.c_str(), nullptr, 10);
  if (v == 0) throw bad("value must be greater than zero");
  return (size_t)v * mul;
}

static size_t resolve_memory_limit_bytes(const std::string& spec) {
  if (!spec.empty()) return parse_memory_spec(spec);
  FILE* f = fopen("/proc/meminfo", "r");
  if (f) {
    char line[256];
    while (fgets(line, sizeof line, f)) {
      unsigned long long kib;
      if (sscanf(line, "MemAvailable: %llu", &kib) == 1) {
        fclose(f);
        size_t b = (size_t)kib * 1024;
        if (b * 2 / 3 > 0) return b * 2 / 3;
        break;
      }
    }
    fclose(f);
  }
  return 64 * GIB;
}

// ---------------------------------------------------------------------------
// Planner: derive_heuristic_plan src/count/mod.rs:624-864 and helpers
// :866-1016, sample_input :1018-1079.
// ---------------------------------------------------------------------------
struct Plan {
  size_t partitions, chunk_size_bytes, staging_bytes, worker_threads, local_flush_bytes,
      decomp_threads, writer_lanes;
  double avg_read_len;
};

static size_t round_up_pow2(size_t v) {
  size_t p = 1;
  while (p < std::max<size_t>(v, 1)) p <<= 1;
  return p;
}
static size_t floor_pow2(size_t v) {
  if (v <= 1) return 1;
  size_t p = 1;
  while ((p << 1) <= v) p <<= 1;
  return p;
}

static double sample_avg_read_len(const std::string& path, Compression c) {
  // sample_input: 8 MiB chunks until >= 200k reads or >= 32 MiB decompressed.
  uint64_t reads = 0, bases = 0;
  size_t decomp = 0;
  if (c == BGZF) {
    // sample_bgzf_input: block by block, complete records only; errors propagate
    const std::vector<uint8_t> d = read_whole_file(path);
    std::vector<uint8_t> carry, out;
    for (auto& b : scan_bgzf_blocks(d)) {
      if (!inflate_member(d.data() + b.first, b.second, out)) throw Error("invalid gzip data in a BGZF block");
      decomp += out.size();
      carry.insert(carry.end(), out.begin(), out.end());
      const size_t split = find_fastq_split_4lines(carry.data(), carry.size());
      if (split > 0) {
        parse_sequences(carry.data(), split, [&](const uint8_t*, size_t n) {
          reads++;
          bases += n;
        });
        carry.erase(carry.begin(), carry.begin() + split);
      }
      if (reads >= 200000 || decomp >= 32 * MIB) break;
    }
    return reads == 0 ? 150.0 : (double)bases / (double)reads;
  }
  std::unique_ptr<ByteSource> src(open_source(path, c));
  ChunkedReader rd(src.get(), 8 * MIB);
  std::vector<uint8_t> chunk;
  while (reads < 200000 && decomp < 32 * MIB) {
    if (!rd.next_chunk(chunk)) break;
    decomp += chunk.size();
    parse_sequences(chunk.data(), chunk.size(), [&](const uint8_t*, size_t n) {
      reads++;
      bases += n;
    });
  }
  return reads == 0 ? 150.0 : (double)bases / (double)reads;
}

static Plan derive_plan(size_t input_bytes, double avg_read_len, Compression comp, unsigned k,
                        size_t requested_partitions, size_t total_threads, size_t mem,
                        long buffer_mb, size_t chunk_kmers) {
  const bool u64keys = k <= 31;
  const size_t E = u64keys ? 1 : 2;
  size_t target_mb;  // target_partition_bytes_for :961-974
  size_t base_mb = u64keys ? 640 : 448;
  if (u64keys && k >= 22 && k <= 31) target_mb = 192;
  else if (k <= 21) target_mb = base_mb + 64;
  else if (k >= 52) target_mb = base_mb - 64;
  else target_mb = base_mb;
  size_t target_part = target_mb * MIB;
  size_t min_worker_budget = u64keys ? 1250 * MIB : 2 * GIB;  // :883-890
  min_worker_budget = std::min(min_worker_budget, std::max(mem / 2, 512 * MIB));

  size_t decomp_threads = 1;
  if (comp == BGZF) {
    size_t max_decomp = std::max<size_t>(total_threads / 2, 1);
    size_t div = k <= 31 ? 4 : k <= 51 ? 5 : k <= 75 ? 6 : 8;
    decomp_threads = std::min(std::max<size_t>(total_threads / div, 1), max_decomp);
  }
  size_t mmap_reserve = comp == BGZF ? input_bytes : 0;
  // estimate_untracked_reserve_bytes :866-881
  size_t untracked = mem / 6 + (total_threads + 3) * 8 * MIB + decomp_threads * 32 * MIB;
  untracked = std::min(std::max(untracked, 2 * GIB), 12 * GIB);
  untracked = std::min(untracked, mem / 3) + mmap_reserve;
  size_t workers = total_threads > decomp_threads + 1 ? total_threads - decomp_threads - 1 : 0;
  workers = std::max<size_t>(workers, 1);

  size_t partitions;
  const bool auto_p = requested_partitions == 0;
  if (!auto_p) {
    partitions = requested_partitions;
  } else {
    double expansion = std::min(std::max(avg_read_len / 10.0, 4.0), 24.0);
    size_t est = (size_t)((double)input_bytes * expansion * (double)E);
    size_t raw = std::max<size_t>((est + target_part - 1) / target_part, 1);
    size_t derived = std::min<size_t>(std::max<size_t>(round_up_pow2(raw), 256), 2048);
    // requested_buffer_mb.unwrap_or(8).max(1) (src/count/mod.rs:929): --buffer 0 plans with 1 MiB
    size_t plan_mb = buffer_mb >= 0 ? (size_t)std::max<long>(buffer_mb, 1) : 8;
    size_t per_part = plan_mb * MIB + workers * 5 * 1024;
    size_t capped = std::max<size_t>((mem / 4) / std::max<size_t>(per_part, 1), 256);
    capped = floor_pow2(capped);
    partitions = std::min<size_t>(std::max<size_t>(std::min(derived, capped), 256), 2048);
  }

  std::vector<size_t> cands;
  if (buffer_mb >= 0) {
    size_t req = std::max<long>(buffer_mb, 1);
    for (size_t v : {req, (size_t)16, (size_t)8, (size_t)4, (size_t)2, (size_t)1})
      if (v <= req) cands.push_back(v);
  } else {
    cands = {16, 8, 4, 2};
  }
  std::sort(cands.rbegin(), cands.rend());
  cands.erase(std::unique(cands.begin(), cands.end()), cands.end());

  size_t si = 0;
  for (;;) {
    size_t staging = cands[si] * MIB;
    size_t chunk;
    if (chunk_kmers)
      chunk = std::min(std::max(chunk_kmers * 2, 8 * MIB), 64 * MIB);
    else
      chunk = std::min(std::max(mem / (std::max<size_t>(workers, 1) * 96), 8 * MIB), 64 * MIB);
    size_t qbase = comp == PLAIN ? 8 : std::min<size_t>(std::max<size_t>(decomp_threads * 2, 8), 64);
    size_t qcap = std::min<size_t>(std::max<size_t>(mem / GIB, 8), 64);
    size_t queue = std::min(qbase, qcap);
    size_t decomp_budget = chunk * queue;
    size_t reserved = decomp_budget + partitions * staging + workers * 48 * MIB + untracked;
    size_t tracked = mem > untracked + decomp_budget ? mem - untracked - decomp_budget : 0;
    size_t worker_budget = (mem > reserved ? mem - reserved : 0) / std::max<size_t>(workers, 1);
    size_t minimum = std::max(chunk * 2, staging * 4);  // streaming_flush_target_bytes :976-988
    size_t local_flush = std::max(worker_budget * 45 / 100, minimum);
    if (reserved < mem && tracked > 0 && worker_budget >= min_worker_budget) {
      Plan p;
      p.partitions = partitions;
      p.chunk_size_bytes = chunk;
      p.staging_bytes = staging;
      p.worker_threads = workers;
      p.local_flush_bytes = local_flush;
      p.decomp_threads = decomp_threads;
      p.writer_lanes = std::min<size_t>(std::max<size_t>((workers + 7) / 8, 2), 6);
      p.avg_read_len = avg_read_len;
      return p;
    }
    if (si + 1 < cands.size()) { si++; continue; }
    if (workers > 1) { workers--; si = 0; continue; }
    if (auto_p && partitions > 256) { partitions /= 2; si = 0; continue; }
    throw Error("unable to derive count heuristic plan within memory budget " + std::to_string(mem) + " bytes");
  }
}

// ---------------------------------------------------------------------------
// Sorting (any correct sort gives the reference's order; this mirrors the
// MSD-then-leaf structure of radix_sort_u64_kmer src/count/sorter.rs:67-93
// for comparable CPU timing), RLE rle_compress_typed src/count/sorter.rs:514-530.
// ---------------------------------------------------------------------------
template <class T>
static void msd_sort(T* a, T* tmp, size_t n, int byte) {
  if (n <= 1024 || byte < 0) {
    std::sort(a, a + n);
    return;
  }
  size_t cnt[257] = {0};
  const unsigned sh = 8u * (unsigned)byte;
  for (size_t i = 0; i < n; ++i) cnt[(size_t)((a[i] >> sh) & 0xff) + 1]++;
  for (int i = 0; i < 256; ++i) cnt[i + 1] += cnt[i];
  size_t pos[256];
  memcpy(pos, cnt, sizeof pos);
  for (size_t i = 0; i < n; ++i) tmp[pos[(size_t)((a[i] >> sh) & 0xff)]++] = a[i];
  memcpy(a, tmp, n * sizeof(T));
  for (int b = 0; b < 256; ++b)
    if (cnt[b + 1] - cnt[b] > 1) msd_sort(a + cnt[b], tmp + cnt[b], cnt[b + 1] - cnt[b], byte - 1);
}

template <class T>
static void sort_keys(std::vector<T>& v, unsigned k, std::vector<T>& scratch) {
  if (v.size() < 2) return;
  int top = (int)std::min<unsigned>((2 * k + 7) / 8, sizeof(T)) - 1;
  scratch.resize(v.size());
  msd_sort(v.data(), scratch.data(), v.size(), top);
}

template <class T>
static void rle(const std::vector<T>& s, std::vector<T>& keys, std::vector<uint32_t>& counts) {
  keys.clear();
  counts.clear();
  if (s.empty()) return;
  T cur = s[0];
  uint32_t c = 1;
  for (size_t i = 1; i < s.size(); ++i) {
    if (s[i] == cur) {
      if (c != 0xffffffffu) c++;
    } else {
      keys.push_back(cur);
      counts.push_back(c);
      cur = s[i];
      c = 1;
    }
  }
  keys.push_back(cur);
  counts.push_back(c);
}

// ---------------------------------------------------------------------------
// DVLE / LEB128: write_varint_u64/u128 src/format/run_block.rs:9-35,
// read_varint :40-66, encode_dvle_u64/u128 :70-95.
// ---------------------------------------------------------------------------
template <class T>
static void put_varint(T v, std::vector<uint8_t>& out) {
  for (;;) {
    uint8_t b = (uint8_t)(v & 0x7f);
    v >>= 7;
    if (v == 0) {
      out.push_back(b);
      return;
    }
    out.push_back(b | 0x80);
  }
}

template <class T>
static size_t get_varint(const uint8_t* d, size_t n, size_t maxb, T& out) {
  T r = 0;
  unsigned sh = 0;
  for (size_t i = 0; i < n && i < maxb; ++i) {
    r |= (T)(d[i] & 0x7f) << sh;
    if (!(d[i] & 0x80)) {
      out = r;
      return i + 1;
    }
    sh += 7;
  }
  out = r;
  return std::min(n, maxb);
}

static void put_le(std::vector<uint8_t>& o, uint64_t v, int nbytes) {
  for (int i = 0; i < nbytes; ++i) o.push_back((uint8_t)(v >> (8 * i)));
}
static void put_le128(std::vector<uint8_t>& o, u128 v) {
  put_le(o, (uint64_t)v, 8);
  put_le(o, (uint64_t)(v >> 64), 8);
}
static uint64_t get_le(const uint8_t* p, int nbytes) {
  uint64_t v = 0;
  for (int i = 0; i < nbytes; ++i) v |= (uint64_t)p[i] << (8 * i);
  return v;
}
static u128 get_le128(const uint8_t* p) { return (u128)get_le(p, 8) | ((u128)get_le(p + 8, 8) << 64); }

// ---------------------------------------------------------------------------
// zstd (the zstd crate 0.13.3 / libzstd in the reference; here the system's
// libzstd.so.1 loaded at run time): bulk compress / decompress of one payload.
// ---------------------------------------------------------------------------
struct ZstdLib {
  size_t (*compress)(void*, size_t, const void*, size_t, int) = nullptr;
  size_t (*decompress)(void*, size_t, const void*, size_t) = nullptr;
  size_t (*bound)(size_t) = nullptr;
  unsigned (*is_error)(size_t) = nullptr;
};
static const ZstdLib& zstd_lib() {
  static ZstdLib z = [] {
    ZstdLib r;
    if (void* h = dlopen("libzstd.so.1", RTLD_NOW | RTLD_LOCAL)) {
      r.compress = (size_t(*)(void*, size_t, const void*, size_t, int))dlsym(h, "ZSTD_compress");
      r.decompress = (size_t(*)(void*, size_t, const void*, size_t))dlsym(h, "ZSTD_decompress");
      r.bound = (size_t(*)(size_t))dlsym(h, "ZSTD_compressBound");
      r.is_error = (unsigned (*)(size_t))dlsym(h, "ZSTD_isError");
    }
    if (!r.compress || !r.decompress || !r.bound || !r.is_error) throw std::runtime_error("libzstd.so.1 unavailable");
    return r;
  }();
  return z;
}

// zstd "if smaller" of one flushed bucket: CountWorker::flush_bucket
// src/count/worker.rs:340-374 with compression_level_for :484-501,
// min_compression_input_bytes :452-460, min_compression_savings_bytes :462-482.
// Returns true (and the compressed bytes in z) when the compressed payload is
// kept.
static bool zstd_if_smaller(const std::vector<uint8_t>& payload, size_t rows, unsigned k, int base_level,
                            std::vector<uint8_t>& z) {
  if (base_level <= 0) return false;
  const bool used_dvle = true;  // u64 / u128 keys always encode DVLE
  const size_t es = k <= 31 ? 12 : 20;
  const size_t pb = payload.size(), logical = rows * es;
  int level = base_level;
  if (used_dvle && es == 12 && k <= 31 && pb >= 1024 * 1024) level += 1;
  if (logical >= pb * 2 && pb >= 4 * 1024 * 1024) level += 1;
  level = std::min(level, 6);
  const size_t min_in = (es == 12 && k <= 31) ? 16 * 1024 : 32 * 1024;
  if (level <= 0 || pb < min_in) return false;
  const ZstdLib& zl = zstd_lib();
  z.resize(zl.bound(pb));
  const size_t got = zl.compress(z.data(), z.size(), payload.data(), pb, level);
  if (zl.is_error(got)) return false;
  z.resize(got);
  const size_t bias = std::min<size_t>((logical > pb ? logical - pb : 0) / 32, 24 * 1024);
  const size_t floor = std::max<size_t>(es == 12 ? 8 * 1024 : 16 * 1024, pb / 100);
  const size_t min_savings = floor > bias ? floor - bias : 0;
  return got + min_savings < pb;
}

template <class T>
static void encode_dvle(const T* keys, const uint32_t* counts, size_t n, std::vector<uint8_t>& out) {
  if (n == 0) return;
  if (sizeof(T) == 8) put_le(out, (uint64_t)keys[0], 8);
  else put_le128(out, (u128)keys[0]);
  put_le(out, counts[0], 4);
  for (size_t i = 1; i < n; ++i) {
    put_varint<T>(keys[i] - keys[i - 1], out);
    put_varint<uint64_t>(counts[i], out);
  }
}

// ---------------------------------------------------------------------------
// .kite KX2 format: KiteHeader::write_to src/format/header.rs:62-92,
// read_from :94-151; ChunkIndexEntry src/format/bucket_dir.rs:44-103 (128 B),
// PartitionEntry :6-40 (40 B), Kx2Footer :105-147 (24 B).
// ---------------------------------------------------------------------------
struct Header {
  uint8_t k = 0, canonical = 0;
  uint16_t version = 1, key_width = 64, codec_mask = 0;
  uint32_t partitions = 0, checksum = 0;
  uint64_t chunk_index_off = 0, partition_table_off = 0, footer_off = 0, total_chunks = 0, total_rows = 0;
  bool has_min = false, has_max = false;
  uint32_t min_count = 0, max_count = 0;
  size_t entry_size() const { return key_width == 64 ? 12 : key_width == 128 ? 20 : key_width == 256 ? 36 : 12; }
};

static void write_header(const Header& h, uint8_t* out128) {
  std::vector<uint8_t> o;
  o.insert(o.end(), {'K', 'X', '2', '!'});
  put_le(o, h.version, 2);
  o.push_back(h.k);
  o.push_back(h.canonical);
  put_le(o, h.partitions, 4);
  put_le(o, h.key_width, 2);
  put_le(o, h.codec_mask, 2);
  put_le(o, h.checksum, 4);
  put_le(o, h.chunk_index_off, 8);
  put_le(o, h.partition_table_off, 8);
  put_le(o, h.footer_off, 8);
  put_le(o, h.total_chunks, 8);
  put_le(o, h.total_rows, 8);
  uint8_t res[68] = {0};
  if (h.has_min || h.has_max) {
    memcpy(res, "KMT1", 4);
    uint32_t flags = (h.has_min ? 1u : 0u) | (h.has_max ? 2u : 0u);
    memcpy(res + 4, &flags, 4);
    uint32_t mn = h.has_min ? h.min_count : 0, mx = h.has_max ? h.max_count : 0;
    memcpy(res + 8, &mn, 4);
    memcpy(res + 12, &mx, 4);
  }
  o.insert(o.end(), res, res + 68);
  memcpy(out128, o.data(), 128);
}

static Header read_header(const uint8_t* p, size_t n) {
  if (n < 128) throw Error("file too small");
  if (memcmp(p, "KX2!", 4) != 0) throw Error("invalid magic: expected KITE");
  Header h;
  h.version = (uint16_t)get_le(p + 4, 2);
  if (h.version != 1) throw Error("unsupported version: " + std::to_string(h.version));
  h.k = p[6];
  h.canonical = p[7];
  h.partitions = (uint32_t)get_le(p + 8, 4);
  h.key_width = (uint16_t)get_le(p + 12, 2);
  h.codec_mask = (uint16_t)get_le(p + 14, 2);
  h.checksum = (uint32_t)get_le(p + 16, 4);
  h.chunk_index_off = get_le(p + 20, 8);
  h.partition_table_off = get_le(p + 28, 8);
  h.footer_off = get_le(p + 36, 8);
  h.total_chunks = get_le(p + 44, 8);
  h.total_rows = get_le(p + 52, 8);
  const uint8_t* r = p + 60;
  if (memcmp(r, "KMT1", 4) == 0) {
    uint32_t flags = (uint32_t)get_le(r + 4, 4);
    h.has_min = flags & 1;
    h.has_max = flags & 2;
    h.min_count = (uint32_t)get_le(r + 8, 4);
    h.max_count = (uint32_t)get_le(r + 12, 4);
  }
  return h;
}

struct ChunkMeta {
  uint64_t file_offset, row_count, encoded_bytes, raw_bytes;
  uint32_t codec;
  u128 kmin_lo, kmin_hi, kmax_lo, kmax_hi;
};

static void write_chunk_entry(std::vector<uint8_t>& o, uint32_t pid, const ChunkMeta& c) {
  put_le(o, pid, 4);
  put_le(o, c.codec, 4);
  put_le(o, c.file_offset, 8);
  put_le(o, c.encoded_bytes, 8);
  put_le(o, c.raw_bytes, 8);
  put_le(o, c.row_count, 8);
  put_le128(o, c.kmin_lo);
  put_le128(o, c.kmin_hi);
  put_le128(o, c.kmax_lo);
  put_le128(o, c.kmax_hi);
  for (int i = 0; i < 24; ++i) o.push_back(0);
}

// ---------------------------------------------------------------------------
// ConcurrentKiteWriter restated for a single appending thread:
//   create :76-146 (high watermark = staging*lanes*4, low = high/2),
//   flush_partition_locked :207-240, drain_one_partition :242-267 (largest
//   staged partition, ties to the lowest id), drain_excess_staging :269-283,
//   append_chunk :285-348, finalize :350-494.
// The file image is kept in memory: header + blobs in enqueue order + trailer.
// ---------------------------------------------------------------------------
struct Writer {
  struct Pending { uint64_t rel; ChunkMeta m; };
  struct Staging { std::vector<uint8_t> buf; std::vector<Pending> pending; std::vector<ChunkMeta> committed; };
  Header hdr;
  size_t staging_bytes, high, low;
  std::vector<Staging> parts;
  uint64_t next_offset = 128, staged = 0;
  std::vector<uint8_t> data;  // bytes after the header, in enqueue order
  bool keep_data = true;
  std::mutex mu;

  Writer(const Header& h, size_t staging, size_t lanes) : hdr(h), staging_bytes(staging) {
    high = std::max(staging * lanes * 4, staging);
    low = high / 2;
    parts.resize(h.partitions);
  }
  uint64_t enqueue(const uint8_t* p, size_t n) {
    uint64_t off = next_offset;
    next_offset += n;
    if (keep_data) data.insert(data.end(), p, p + n);
    return off;
  }
  void flush_partition(size_t pid) {
    Staging& s = parts[pid];
    if (s.buf.empty()) return;
    uint64_t off = enqueue(s.buf.data(), s.buf.size());
    staged -= s.buf.size();
    for (auto& pd : s.pending) {
      ChunkMeta m = pd.m;
      m.file_offset = off + pd.rel;
      s.committed.push_back(m);
    }
    s.pending.clear();
    s.buf.clear();
  }
  bool needs_runtime_drain() const { return staged >= high; }
  bool drain_one() {
    size_t best = SIZE_MAX, best_bytes = 0;
    for (size_t p = 0; p < parts.size(); ++p)
      if (parts[p].buf.size() > best_bytes) { best_bytes = parts[p].buf.size(); best = p; }
    if (best == SIZE_MAX) return false;
    flush_partition(best);
    return true;
  }
  void drain_excess() {
    int attempts = 0;
    while (staged > low && attempts < 4) {
      if (!drain_one()) break;
      attempts++;
    }
  }
  void append_chunk(size_t pid, uint32_t codec, uint64_t rows, uint64_t raw, u128 kmin_lo, u128 kmin_hi,
                    u128 kmax_lo, u128 kmax_hi, const uint8_t* d, size_t n) {
    std::lock_guard<std::mutex> g(mu);
    Staging& s = parts[pid];
    if (!s.buf.empty() && s.buf.size() + n > staging_bytes) flush_partition(pid);
    ChunkMeta m{0, rows, (uint64_t)n, raw, codec, kmin_lo, kmin_hi, kmax_lo, kmax_hi};
    if (n >= staging_bytes) {
      m.file_offset = enqueue(d, n);
      s.committed.push_back(m);
    } else {
      uint64_t rel = s.buf.size();
      s.buf.insert(s.buf.end(), d, d + n);
      s.pending.push_back({rel, m});
      staged += n;
      if (s.buf.size() >= staging_bytes) flush_partition(pid);
    }
    if (needs_runtime_drain()) drain_excess();
  }
  void worker_final_drain() {
    std::lock_guard<std::mutex> g(mu);
    while (needs_runtime_drain())
      if (!drain_one()) break;
  }
  // Returns the full file image (header + data + trailer).
  std::vector<uint8_t> finalize(uint64_t* total_chunks_out = nullptr, uint64_t* total_rows_out = nullptr) {
    std::vector<std::vector<ChunkMeta>> all(parts.size());
    for (size_t p = 0; p < parts.size(); ++p) {
      flush_partition(p);
      all[p] = parts[p].committed;
      std::sort(all[p].begin(), all[p].end(),
                [](const ChunkMeta& a, const ChunkMeta& b) { return a.file_offset < b.file_offset; });
    }
    uint64_t data_end = next_offset, total_chunks = 0, total_rows = 0;
    for (auto& v : all)
      for (auto& c : v) { total_chunks++; total_rows += c.row_count; }
    uint64_t cio = data_end, pto = cio + total_chunks * 128, fo = pto + parts.size() * 40;
    std::vector<uint8_t> trailer;
    for (size_t p = 0; p < all.size(); ++p)
      for (auto& c : all[p]) write_chunk_entry(trailer, (uint32_t)p, c);
    uint64_t first = 0;
    for (auto& v : all) {
      uint64_t rows = 0, bytes = 0, minoff = UINT64_MAX;
      for (auto& c : v) { rows += c.row_count; bytes += c.encoded_bytes; minoff = std::min(minoff, c.file_offset); }
      put_le(trailer, first, 8);
      put_le(trailer, v.size(), 8);
      put_le(trailer, rows, 8);
      put_le(trailer, v.empty() ? 0 : minoff, 8);
      put_le(trailer, bytes, 8);
      first += v.size();
    }
    put_le(trailer, total_chunks, 8);
    put_le(trailer, total_rows, 8);
    trailer.insert(trailer.end(), {'K', 'X', '2', 'F', 'O', 'O', 'T', '!'});
    Header h = hdr;
    h.chunk_index_off = cio;
    h.partition_table_off = pto;
    h.footer_off = fo;
    h.total_chunks = total_chunks;
    h.total_rows = total_rows;
    std::vector<uint8_t> file(128);
    write_header(h, file.data());
    file.insert(file.end(), data.begin(), data.end());
    file.insert(file.end(), trailer.begin(), trailer.end());
    if (total_chunks_out) *total_chunks_out = total_chunks;
    if (total_rows_out) *total_rows_out = total_rows;
    return file;
  }
};

// ---------------------------------------------------------------------------
// Count worker: CountWorker::process_chunk src/count/worker.rs:196-271,
// push_kmer :164-175 (64-entry write-combining slots only change when
// local_bytes grows), flush_all :284-294, flush_bucket :296-449 (fast mode:
// sort -> RLE -> DVLE, codec DVLE, raw_bytes = payload length).
// ---------------------------------------------------------------------------
template <class T>
struct Worker {
  unsigned k;
  bool canonical;
  unsigned bits;
  size_t partitions, flush_threshold;
  Writer* w;
  std::vector<std::vector<T>> buckets;
  std::vector<uint8_t> wc;  // write-combining fill per bucket (0..63)
  size_t local_bytes = 0;
  uint64_t reads = 0, bases = 0, kmers = 0;
  std::vector<T> scratch, keys;
  std::vector<uint32_t> counts;
  std::vector<uint8_t> payload;

  int zstd_level = 0;  // CountMode::zstd_level src/cli.rs:11-19 (fast 0, balanced 2, compact 5)
  std::vector<uint8_t> zbuf;

  Worker(unsigned k_, bool c, size_t P, size_t thr, Writer* wr)
      : k(k_), canonical(c), partitions(P), flush_threshold(thr), w(wr) {
    bits = 0;
    while ((size_t(1) << bits) < P) bits++;
    buckets.resize(P);
    wc.assign(P, 0);
  }
  void push(T key) {
    size_t b = bucket_of(key, bits);
    buckets[b].push_back(key);
    if (++wc[b] == 64) {
      wc[b] = 0;
      local_bytes += 64 * sizeof(T);
    }
  }
  void process_chunk(const uint8_t* d, size_t n) {
    parse_sequences(d, n, [&](const uint8_t* s, size_t len) {
      reads++;
      bases += len;
      scan_kmers<T>(s, len, k, canonical, [&](T key) {
        kmers++;
        push(key);
      });
    });
    if (local_bytes >= flush_threshold) {
      flush_all_buckets();
      if (w) {
        std::lock_guard<std::mutex> g(w->mu);
        if (w->needs_runtime_drain()) w->drain_excess();
      }
    }
  }
  void flush_all_buckets() {
    for (size_t b = 0; b < partitions; ++b)
      if (!buckets[b].empty()) flush_bucket(b);
    local_bytes = 0;
    std::fill(wc.begin(), wc.end(), 0);
  }
  void flush_bucket(size_t b) {
    sort_keys(buckets[b], k, scratch);
    rle(buckets[b], keys, counts);
    payload.clear();
    encode_dvle(keys.data(), counts.data(), keys.size(), payload);
    if (w) {
      if (zstd_if_smaller(payload, keys.size(), k, zstd_level, zbuf))
        w->append_chunk(b, 2 | 4, keys.size(), payload.size(), (u128)keys.front(), 0, (u128)keys.back(), 0,
                        zbuf.data(), zbuf.size());
      else
        w->append_chunk(b, 2, keys.size(), payload.size(), (u128)keys.front(), 0, (u128)keys.back(), 0,
                        payload.data(), payload.size());
    }
    buckets[b].clear();
  }
  void flush_all() {
    flush_all_buckets();
    if (w) w->worker_final_drain();
  }
};

struct CountStats {
  uint64_t reads = 0, bases = 0, kmers = 0, rows = 0, chunks = 0, payload_bytes = 0;
  double seconds = 0;
};

// Count an in-memory FASTQ buffer split into reader chunks; `workers` threads
// each own local buckets as in run_count_typed src/count/mod.rs:512-539.
template <class T>
static void count_chunks(const std::vector<std::pair<const uint8_t*, size_t>>& chunks,
                                         unsigned k, bool canonical, size_t P, size_t workers,
                                         size_t flush_threshold, Writer* writer, CountStats& st,
                                         int zstd_level = 0) {
  std::vector<std::unique_ptr<Worker<T>>> ws;
  for (size_t i = 0; i < workers; ++i) {
    ws.emplace_back(new Worker<T>(k, canonical, P, flush_threshold, writer));
    ws.back()->zstd_level = zstd_level;
  }
  std::atomic<size_t> next(0);
  auto run = [&](size_t wi) {
    for (;;) {
      size_t c = next.fetch_add(1);
      if (c >= chunks.size()) break;
      ws[wi]->process_chunk(chunks[c].first, chunks[c].second);
    }
    ws[wi]->flush_all();
  };
  if (workers == 1) {
    run(0);
  } else {
    std::vector<std::thread> th;
    for (size_t i = 0; i < workers; ++i) th.emplace_back(run, i);
    for (auto& t : th) t.join();
  }
  for (auto& w : ws) {
    st.reads += w->reads;
    st.bases += w->bases;
    st.kmers += w->kmers;
  }
}

// The payload of every partition as the single-worker count writes it (one
// flush per partition at flush_all, src/count/worker.rs:284-294: all of the
// partition's keys sorted, run-length reduced with saturating u32 counts and
// DVLE-encoded, flush_bucket :296-449), computed with `threads` threads:
// chunks are scanned in parallel into per-thread buckets, then partitions are
// sorted and encoded in parallel.  Same bytes as orc_count_kite's payloads,
// for inputs too large for one worker in a test or a benchmark's parity check.
struct PartOut {
  std::vector<uint8_t> payload;
  uint64_t rows = 0;
  u128 kmin = 0, kmax = 0;
};

template <class T>
static void count_parts(const std::vector<std::pair<const uint8_t*, size_t>>& chunks, unsigned k, bool canonical,
                        size_t P, size_t threads, std::vector<PartOut>& out, CountStats& st) {
  threads = std::max<size_t>(threads, 1);
  std::vector<std::unique_ptr<Worker<T>>> ws;
  for (size_t i = 0; i < threads; ++i) ws.emplace_back(new Worker<T>(k, canonical, P, SIZE_MAX, nullptr));
  std::atomic<size_t> next(0);
  auto scan = [&](size_t wi) {
    for (;;) {
      size_t c = next.fetch_add(1);
      if (c >= chunks.size()) break;
      ws[wi]->process_chunk(chunks[c].first, chunks[c].second);
    }
  };
  std::vector<std::thread> th;
  for (size_t i = 0; i < threads; ++i) th.emplace_back(scan, i);
  for (auto& t : th) t.join();
  th.clear();
  for (auto& w : ws) {
    st.reads += w->reads;
    st.bases += w->bases;
    st.kmers += w->kmers;
  }
  out.assign(P, PartOut());
  std::atomic<size_t> next_p(0);
  auto reduce = [&]() {
    std::vector<T> all, scratch, keys;
    std::vector<uint32_t> counts;
    for (;;) {
      size_t p = next_p.fetch_add(1);
      if (p >= P) break;
      size_t n = 0;
      for (auto& w : ws) n += w->buckets[p].size();
      if (n == 0) continue;
      all.clear();
      all.reserve(n);
      for (auto& w : ws) {
        all.insert(all.end(), w->buckets[p].begin(), w->buckets[p].end());
        std::vector<T>().swap(w->buckets[p]);
      }
      sort_keys(all, k, scratch);
      rle(all, keys, counts);
      PartOut& o = out[p];
      encode_dvle(keys.data(), counts.data(), keys.size(), o.payload);
      o.rows = keys.size();
      o.kmin = (u128)keys.front();
      o.kmax = (u128)keys.back();
    }
  };
  for (size_t i = 0; i < threads; ++i) th.emplace_back(reduce);
  for (auto& t : th) t.join();
}

// Split an in-memory FASTQ image into reader chunks the way the chunked
// readers do (fixed-size reads, cut after the last 4k-th newline, carry).
static std::vector<std::pair<const uint8_t*, size_t>> split_chunks(const uint8_t* d, size_t n, size_t chunk) {
  std::vector<std::pair<const uint8_t*, size_t>> out;
  size_t consumed = 0, carry = 0;
  for (;;) {
    size_t start = consumed - carry;
    size_t nw = std::min(chunk, n - consumed);
    consumed += nw;
    size_t len = carry + nw;
    if (len == 0) break;
    if (nw < chunk) {
      out.push_back({d + start, len});
      break;
    }
    size_t split = find_fastq_split_4lines(d + start, len);
    if (split == 0 || split >= len) {
      out.push_back({d + start, len});
      carry = 0;
    } else {
      out.push_back({d + start, split});
      carry = len - split;
    }
  }
  return out;
}

// ---------------------------------------------------------------------------
// Reader + dump: KiteReader::open src/dump/reader.rs:43-155,
// DvleRunIter/MmapRunIter src/dump/merge.rs:13-240, LoserTreeMerger
// src/dump/loser_tree.rs:35-176 (saturating u32 sums), stream_partition_slabs
// src/dump/merge.rs:282-428, decode_kmer_any src/dump/decoder.rs:27-50.
// ---------------------------------------------------------------------------
struct ChunkLoc { uint64_t off, len, raw, rows; uint32_t codec; };
struct Reader {
  std::vector<uint8_t> bytes;
  Header h;
  uint64_t total_chunks = 0;
  std::vector<std::vector<ChunkLoc>> parts;
  void open(const uint8_t* p, size_t n) {
    bytes.assign(p, p + n);
    if (n < 128 + 24) throw Error("file too small");
    h = read_header(p, n);
    size_t P = h.partitions;
    if (h.footer_off + 24 > n) throw Error("footer out of bounds");
    if (memcmp(p + h.footer_off + 16, "KX2FOOT!", 8) != 0) throw Error("invalid footer magic");
    total_chunks = get_le(p + h.footer_off, 8);
    if (h.partition_table_off + P * 40 > n) throw Error("partition table out of bounds");
    if (h.partition_table_off < h.chunk_index_off) throw Error("invalid chunk index offsets");
    size_t cb = h.partition_table_off - h.chunk_index_off;
    if (cb % 128) throw Error("chunk index size misaligned");
    size_t nchunks = cb / 128;
    parts.assign(P, {});
    for (size_t b = 0; b < P; ++b) {
      const uint8_t* e = p + h.partition_table_off + b * 40;
      uint64_t first = get_le(e, 8), cnt = get_le(e + 8, 8);
      if (first + cnt > nchunks) throw Error("partition " + std::to_string(b) + " chunk range out of bounds");
      for (uint64_t c = first; c < first + cnt; ++c) {
        const uint8_t* ce = p + h.chunk_index_off + c * 128;
        ChunkLoc l;
        l.codec = (uint32_t)get_le(ce + 4, 4);
        l.off = get_le(ce + 8, 8);
        l.len = get_le(ce + 16, 8);
        l.raw = get_le(ce + 24, 8);
        l.rows = get_le(ce + 32, 8);
        if (l.len == 0 || l.off + l.len > n) throw Error("partition " + std::to_string(b) + " chunk out of bounds");
        if (l.codec & ~7u) throw Error("partition " + std::to_string(b) + " chunk uses unsupported codec mask");
        if (l.codec & 4u) {
          // run_data_for_decode src/dump/reader.rs:162-186: the decoded
          // payload, appended after the file image
          const ZstdLib& zl = zstd_lib();
          const size_t at = bytes.size();
          bytes.resize(at + l.raw);
          const size_t got = zl.decompress(bytes.data() + at, l.raw, p + l.off, l.len);
          if (zl.is_error(got)) throw Error("zstd decompress failed");
          if (got != l.raw) throw Error("decoded payload size mismatch");
          l.off = at;
          l.len = l.raw;
          l.codec &= ~4u;
        }
        parts[b].push_back(l);
      }
    }
  }
};

// One segment stream (DVLE or RAW rows) of a chunk.
struct RunIter {
  const uint8_t* d;
  size_t len, pos = 0, remaining;
  u128 prev = 0;
  bool dvle, wide;
  size_t esize;
  bool next(u128& key, uint32_t& cnt) {
    if (remaining == 0) return false;
    remaining--;
    if (!dvle) {
      const uint8_t* p = d + pos;
      if (esize == 12) { key = get_le(p, 8); cnt = (uint32_t)get_le(p + 8, 4); }
      else { key = get_le128(p); cnt = (uint32_t)get_le(p + 16, 4); }
      pos += esize;
      return true;
    }
    if (pos == 0) {
      if (wide) { key = get_le128(d); cnt = (uint32_t)get_le(d + 16, 4); pos = 20; }
      else { key = get_le(d, 8); cnt = (uint32_t)get_le(d + 8, 4); pos = 12; }
      prev = key;
      return true;
    }
    u128 delta = 0;
    uint64_t c = 0;
    if (wide) pos += get_varint<u128>(d + pos, len - pos, 19, delta);
    else { uint64_t d64 = 0; pos += get_varint<uint64_t>(d + pos, len - pos, 10, d64); delta = d64; }
    pos += get_varint<uint64_t>(d + pos, len - pos, 10, c);
    key = prev + delta;
    prev = key;
    cnt = (uint32_t)c;
    return true;
  }
};

struct LoserTree {
  std::vector<RunIter> s;
  std::vector<bool> has;
  std::vector<u128> hk;
  std::vector<uint32_t> hc;
  std::vector<size_t> loser;
  size_t n = 0, nt = 1, winner = 0;
  explicit LoserTree(std::vector<RunIter> streams) : s(std::move(streams)) {
    n = s.size();
    if (n == 0) return;
    nt = 2;
    while (nt < n) nt <<= 1;
    has.assign(n, false);
    hk.assign(n, 0);
    hc.assign(n, 0);
    for (size_t i = 0; i < n; ++i) has[i] = s[i].next(hk[i], hc[i]);
    std::vector<size_t> w(2 * nt, n);
    for (size_t j = 0; j < n; ++j) w[nt + j] = j;
    loser.assign(nt, n);
    for (size_t t = nt - 1; t >= 1; --t) {
      size_t l = w[2 * t], r = w[2 * t + 1];
      if (key_of(l) <= key_of(r)) { loser[t] = r; w[t] = l; }
      else { loser[t] = l; w[t] = r; }
    }
    winner = w[1];
  }
  u128 key_of(size_t i) const { return (i >= n || !has[i]) ? ~(u128)0 : hk[i]; }
  void adjust(size_t leaf) {
    size_t cand = leaf;
    u128 ck = key_of(leaf);
    for (size_t t = (nt + leaf) >> 1; t >= 1; t >>= 1) {
      size_t sidx = loser[t];
      u128 sk = key_of(sidx);
      if (sk < ck) { loser[t] = cand; cand = sidx; ck = sk; }
    }
    winner = cand;
  }
  bool next_min(u128& key, uint32_t& total) {
    if (n == 0 || winner >= n || !has[winner]) return false;
    u128 mk = hk[winner];
    total = 0;
    for (;;) {
      size_t w = winner;
      if (w >= n || !has[w] || hk[w] != mk) break;
      uint32_t c = hc[w];
      total = (total > 0xffffffffu - c) ? 0xffffffffu : total + c;
      has[w] = s[w].next(hk[w], hc[w]);
      adjust(w);
    }
    key = mk;
    return true;
  }
};

static bool passes(uint64_t c, const Header& h) {
  if (h.has_min && c < h.min_count) return false;
  if (h.has_max && c > h.max_count) return false;
  return true;
}

static void decode_kmer(u128 key, unsigned k, char* out) {
  static const char dna[4] = {'A', 'C', 'G', 'T'};
  for (unsigned i = 0; i < k; ++i) out[i] = dna[(unsigned)(key >> (2 * (k - 1 - i))) & 3];
}

static RunIter make_iter(const Reader& r, const ChunkLoc& l) {
  RunIter it;
  it.d = r.bytes.data() + l.off;
  it.len = l.len;
  it.remaining = l.rows;
  it.dvle = (l.codec & 2u) != 0;
  it.wide = r.h.entry_size() == 20;
  it.esize = r.h.entry_size();
  return it;
}

static void dump_partition(const Reader& r, size_t p, std::string& out) {
  std::vector<RunIter> streams;
  for (auto& l : r.parts[p]) streams.push_back(make_iter(r, l));
  LoserTree lt(std::move(streams));
  u128 key;
  uint32_t cnt;
  char buf[80];
  char num[16];
  while (lt.next_min(key, cnt)) {
    if (!passes(cnt, r.h)) continue;
    decode_kmer(key, r.h.k, buf);
    out.append(buf, r.h.k);
    out.push_back('\t');
    int nn = snprintf(num, sizeof num, "%u", cnt);
    out.append(num, nn);
    out.push_back('\n');
  }
}

// ---------------------------------------------------------------------------
// Merge: load_partition_counts src/kiteops/mod.rs:433-473 (sort, u64
// saturating coalesce), apply_reader_filter_to_rows :103-108,
// merge_vectors_total :587-623 (u64 saturating), serialize_partition_chunk
// :804-859 (u32 overflow is an error), run_merge src/merge/mod.rs:22-191.
// ---------------------------------------------------------------------------
typedef std::pair<u128, uint64_t> Row;

static std::vector<Row> load_partition_counts(const Reader& r, size_t p) {
  std::vector<Row> rows;
  for (auto& l : r.parts[p]) {
    RunIter it = make_iter(r, l);
    u128 key;
    uint32_t c;
    while (it.next(key, c)) rows.push_back({key, c});
  }
  std::sort(rows.begin(), rows.end(), [](const Row& a, const Row& b) { return a.first < b.first; });
  std::vector<Row> merged;
  for (auto& rw : rows) {
    if (!merged.empty() && merged.back().first == rw.first) {
      uint64_t& t = merged.back().second;
      t = (t > UINT64_MAX - rw.second) ? UINT64_MAX : t + rw.second;
    } else {
      merged.push_back(rw);
    }
  }
  return merged;
}

static std::vector<Row> merge_vectors_total(const std::vector<std::vector<Row>>& v) {
  std::vector<Row> out;
  std::vector<size_t> idx(v.size(), 0);
  for (;;) {
    bool any = false;
    u128 mk = 0;
    for (size_t i = 0; i < v.size(); ++i)
      if (idx[i] < v[i].size() && (!any || v[i][idx[i]].first < mk)) { mk = v[i][idx[i]].first; any = true; }
    if (!any) break;
    uint64_t t = 0;
    for (size_t i = 0; i < v.size(); ++i)
      if (idx[i] < v[i].size() && v[i][idx[i]].first == mk) {
        uint64_t c = v[i][idx[i]].second;
        t = (t > UINT64_MAX - c) ? UINT64_MAX : t + c;
        idx[i]++;
      }
    out.push_back({mk, t});
  }
  return out;
}

static std::string u128_to_string(u128 v) {
  if (v == 0) return "0";
  std::string s;
  while (v) { s.push_back('0' + (int)(v % 10)); v /= 10; }
  std::reverse(s.begin(), s.end());
  return s;
}

// serialize_partition_chunk: returns false when rows is empty.
static bool serialize_partition_chunk(const std::vector<Row>& rows, uint16_t key_width, std::vector<uint8_t>& out) {
  out.clear();
  if (rows.empty()) return false;
  for (auto& r : rows)
    if (r.second > 0xffffffffull) throw Error("merged count exceeds u32 for key " + u128_to_string(r.first));
  std::vector<uint32_t> counts(rows.size());
  for (size_t i = 0; i < rows.size(); ++i) counts[i] = (uint32_t)rows[i].second;
  if (key_width == 64) {
    std::vector<uint64_t> keys(rows.size());
    for (size_t i = 0; i < rows.size(); ++i) keys[i] = (uint64_t)rows[i].first;
    encode_dvle(keys.data(), counts.data(), keys.size(), out);
  } else if (key_width == 128) {
    std::vector<u128> keys(rows.size());
    for (size_t i = 0; i < rows.size(); ++i) keys[i] = rows[i].first;
    encode_dvle(keys.data(), counts.data(), keys.size(), out);
  } else {
    throw Error("unsupported key_width=" + std::to_string(key_width));
  }
  return true;
}

static std::vector<uint8_t> read_file(const std::string& path) {
  FILE* f = fopen(path.c_str(), "rb");
  if (!f) throw Error("failed to open " + path);
  std::vector<uint8_t> v;
  uint8_t buf[1 << 16];
  size_t r;
  while ((r = fread(buf, 1, sizeof buf, f)) > 0) v.insert(v.end(), buf, buf + r);
  fclose(f);
  return v;
}

static void write_file(const std::string& path, const std::vector<uint8_t>& v) {
  FILE* f = fopen(path.c_str(), "wb");
  if (!f) throw Error("failed to create " + path);
  if (!v.empty() && fwrite(v.data(), 1, v.size(), f) != v.size()) { fclose(f); throw Error("write failed: " + path); }
  fclose(f);
}

static std::vector<uint8_t> merge_files(const std::vector<std::string>& paths, size_t lanes) {
  if (paths.empty()) throw Error("no input .kite files were provided.");
  std::vector<Reader> rs(paths.size());
  for (size_t i = 0; i < paths.size(); ++i) {
    auto b = read_file(paths[i]);
    rs[i].open(b.data(), b.size());
  }
  const Header& f = rs[0].h;
  for (size_t i = 1; i < rs.size(); ++i) {
    const Header& h = rs[i].h;
    if (h.k != f.k) throw Error("incompatible .kite inputs: k differs");
    if ((h.canonical != 0) != (f.canonical != 0)) throw Error("incompatible .kite inputs: canonical differs");
    if (h.partitions != f.partitions) throw Error("incompatible .kite inputs: partitions differ");
    if (h.key_width != f.key_width) throw Error("incompatible .kite inputs: key_width differs");
  }
  Header out;
  out.k = f.k;
  out.canonical = f.canonical != 0;
  out.partitions = f.partitions;
  out.key_width = f.key_width;
  out.codec_mask = 3;
  bool same_min = true, same_max = true;
  for (auto& r : rs) {
    same_min = same_min && r.h.has_min == f.has_min && (!f.has_min || r.h.min_count == f.min_count);
    same_max = same_max && r.h.has_max == f.has_max && (!f.has_max || r.h.max_count == f.max_count);
  }
  out.has_min = same_min && f.has_min;
  out.min_count = f.min_count;
  out.has_max = same_max && f.has_max;
  out.max_count = f.max_count;
  Writer w(out, 16 * MIB, lanes);
  std::vector<uint8_t> payload;
  for (size_t p = 0; p < f.partitions; ++p) {
    std::vector<std::vector<Row>> vecs;
    for (auto& r : rs) {
      auto rows = load_partition_counts(r, p);
      if (r.h.has_min || r.h.has_max) {
        std::vector<Row> kept;
        for (auto& x : rows)
          if (passes(x.second, r.h)) kept.push_back(x);
        rows.swap(kept);
      }
      vecs.push_back(std::move(rows));
    }
    auto merged = merge_vectors_total(vecs);
    if (serialize_partition_chunk(merged, out.key_width, payload))
      w.append_chunk(p, 2, merged.size(), payload.size(), merged.front().first, 0, merged.back().first, 0,
                     payload.data(), payload.size());
  }
  return w.finalize();
}

}  // namespace orc

// ===========================================================================
// C API (ctypes) — used by tests to pin the oracle against golden vectors and
// by bench.py for the CPU baseline.
// ===========================================================================
using namespace orc;

static thread_local std::string g_err;

// ---------------------------------------------------------------------------
// histo: run_histo src/histo/mod.rs:16-169 for one input: per partition
// load_partition_counts (u64 saturating sums), apply_reader_filter_to_rows
// (src/kiteops/mod.rs:103-108) on those sums, then count -> frequency.
// query: run_query src/query/mod.rs:15-96: encode_query_kmer
// (src/kiteops/mod.rs:302-348), bucket_for_key, load_partition_counts and a
// binary search; the header filter only labels the result.
// ---------------------------------------------------------------------------
static std::map<uint64_t, uint64_t> histo_of(const Reader& r) {
  std::map<uint64_t, uint64_t> h;
  for (size_t p = 0; p < r.h.partitions; ++p)
    for (auto& x : load_partition_counts(r, p))
      if (passes(x.second, r.h)) h[x.second] += 1;
  return h;
}

static uint64_t query_key(const Reader& r, u128 key, size_t* partition) {
  unsigned bits = 0;
  while ((1ull << bits) < r.h.partitions) ++bits;
  const size_t p = r.h.key_width == 64 ? bucket_of((uint64_t)key, bits) : bucket_of(key, bits);
  if (partition) *partition = p;
  const auto rows = load_partition_counts(r, p);
  auto it = std::lower_bound(rows.begin(), rows.end(), key, [](const Row& a, u128 k) { return a.first < k; });
  return it != rows.end() && it->first == key ? it->second : 0;
}

static u128 encode_query_kmer(const std::string& seq, const Header& h) {
  if (seq.size() != h.k)
    throw Error("query k-mer length " + std::to_string(seq.size()) + " does not match database k=" +
                std::to_string(h.k));
  for (char c : seq)
    if (!strchr("ACGTacgt", c) || c == 0) throw Error("query k-mer contains non-ACGT characters");
  u128 key = 0;
  size_t n = 0;
  if (h.key_width == 64)
    scan_kmers<uint64_t>((const uint8_t*)seq.data(), seq.size(), h.k, h.canonical != 0, [&](uint64_t x) {
      key = x;
      n++;
    });
  else
    scan_kmers<u128>((const uint8_t*)seq.data(), seq.size(), h.k, h.canonical != 0, [&](u128 x) {
      key = x;
      n++;
    });
  if (n != 1) throw Error("failed to encode query k-mer");
  return key;
}

extern "C" {

const char* orc_last_error() { return g_err.c_str(); }

// histo of one .kite image: bins ascending into counts / freqs (up to cap);
// returns the number of bins, -1 on error.
long long orc_histo_kite(const uint8_t* img, size_t n, uint64_t* counts, uint64_t* freqs, size_t cap) {
  try {
    Reader r;
    r.open(img, n);
    size_t i = 0;
    const auto h = histo_of(r);
    for (auto& kv : h) {
      if (i < cap) {
        counts[i] = kv.first;
        freqs[i] = kv.second;
      }
      ++i;
    }
    return (long long)h.size();
  } catch (const Error& e) {
    g_err = e.what();
    return -1;
  }
}

// u64 sums of encoded keys ((lo, hi) words each) in one .kite image, 0 when absent.
int orc_query_kite(const uint8_t* img, size_t n, const uint64_t* keys, size_t nq, uint64_t* out) {
  try {
    Reader r;
    r.open(img, n);
    for (size_t i = 0; i < nq; ++i) out[i] = query_key(r, ((u128)keys[2 * i + 1] << 64) | keys[2 * i], nullptr);
    return 0;
  } catch (const Error& e) {
    g_err = e.what();
    return -1;
  }
}

// Parse a FASTQ chunk: returns the number of sequence slices (start offset and
// length pairs written to out, up to cap), or -1 if the chunk is rejected.
long long orc_parse_sequences(const uint8_t* d, size_t n, uint64_t* starts, uint64_t* lens, size_t cap) {
  size_t cnt = 0;
  bool ok = parse_sequences(d, n, [&](const uint8_t* s, size_t len) {
    if (cnt < cap) { starts[cnt] = (uint64_t)(s - d); lens[cnt] = len; }
    cnt++;
  });
  return ok ? (long long)cnt : -1;
}

size_t orc_find_fastq_split(const uint8_t* d, size_t n) { return find_fastq_split_4lines(d, n); }

// Chunk lengths the reference's reader produces for a file (plain, gzip or
// BGZF): the number of chunks, up to cap lengths written; -1 on error.
int64_t orc_read_chunks(const char* path, size_t chunk_size, uint64_t* lens, size_t cap) {
  try {
    std::vector<std::vector<uint8_t>> store;
    read_all_chunks(path, detect_compression(path), chunk_size, store);
    for (size_t i = 0; i < store.size() && i < cap; ++i) lens[i] = store[i].size();
    return (int64_t)store.size();
  } catch (const Error& e) {
    g_err = e.what();
    return -1;
  }
}

// sample_input's mean read length for a file; < 0 on error.
double orc_sample_avg_read_len(const char* path) {
  try {
    return sample_avg_read_len(path, detect_compression(path));
  } catch (const Error& e) {
    g_err = e.what();
    return -1.0;
  }
}

// k-mers of one sequence; keys as (lo, hi) u64 pairs.  wide=1 uses the u128
// iterator (k <= 64), else the u64 iterator (k <= 32).
size_t orc_kmers(const uint8_t* s, size_t n, unsigned k, int canonical, int wide, uint64_t* out, size_t cap) {
  size_t c = 0;
  if (wide) {
    scan_kmers<u128>(s, n, k, canonical != 0, [&](u128 x) {
      if (c < cap) { out[2 * c] = (uint64_t)x; out[2 * c + 1] = (uint64_t)(x >> 64); }
      c++;
    });
  } else {
    scan_kmers<uint64_t>(s, n, k, canonical != 0, [&](uint64_t x) {
      if (c < cap) { out[2 * c] = x; out[2 * c + 1] = 0; }
      c++;
    });
  }
  return c;
}

size_t orc_bucket(uint64_t lo, uint64_t hi, int wide, unsigned bits) {
  return wide ? bucket_of(((u128)hi << 64) | lo, bits) : bucket_of(lo, bits);
}

size_t orc_rle_u64(const uint64_t* sorted, size_t n, uint64_t* keys, uint32_t* counts) {
  std::vector<uint64_t> s(sorted, sorted + n), k;
  std::vector<uint32_t> c;
  rle(s, k, c);
  std::copy(k.begin(), k.end(), keys);
  std::copy(c.begin(), c.end(), counts);
  return k.size();
}

size_t orc_sort_u64(uint64_t* v, size_t n, unsigned k) {
  std::vector<uint64_t> a(v, v + n), s;
  sort_keys(a, k, s);
  std::copy(a.begin(), a.end(), v);
  return n;
}

// DVLE-encode rows; keys as (lo, hi) pairs.  Returns bytes written (<= cap).
size_t orc_encode_dvle(const uint64_t* keys, const uint32_t* counts, size_t n, int wide, uint8_t* out, size_t cap) {
  std::vector<uint8_t> o;
  if (wide) {
    std::vector<u128> k(n);
    for (size_t i = 0; i < n; ++i) k[i] = ((u128)keys[2 * i + 1] << 64) | keys[2 * i];
    encode_dvle(k.data(), counts, n, o);
  } else {
    std::vector<uint64_t> k(n);
    for (size_t i = 0; i < n; ++i) k[i] = keys[2 * i];
    encode_dvle(k.data(), counts, n, o);
  }
  memcpy(out, o.data(), std::min(cap, o.size()));
  return o.size();
}

void orc_decode_kmer(uint64_t lo, uint64_t hi, unsigned k, char* out) {
  decode_kmer(((u128)hi << 64) | lo, k, out);
  out[k] = 0;
}

// Loser-tree merge of `ns` streams given as concatenated (key lo, count)
// arrays with per-stream lengths.  Returns number of merged rows.
size_t orc_loser_tree_u64(const uint64_t* keys, const uint32_t* counts, const size_t* lens, size_t ns,
                          uint64_t* out_keys, uint32_t* out_counts) {
  // Encode each stream as a RAW 12-byte run so the same iterator is used.
  std::vector<std::vector<uint8_t>> bufs(ns);
  std::vector<RunIter> its;
  size_t off = 0;
  for (size_t i = 0; i < ns; ++i) {
    for (size_t j = 0; j < lens[i]; ++j) { put_le(bufs[i], keys[off + j], 8); put_le(bufs[i], counts[off + j], 4); }
    off += lens[i];
    RunIter it;
    it.d = bufs[i].data(); it.len = bufs[i].size(); it.remaining = lens[i];
    it.dvle = false; it.wide = false; it.esize = 12;
    its.push_back(it);
  }
  LoserTree lt(std::move(its));
  u128 k; uint32_t c; size_t m = 0;
  while (lt.next_min(k, c)) { out_keys[m] = (uint64_t)k; out_counts[m] = c; m++; }
  return m;
}

// merge_vectors_total over u64 rows; returns merged row count.
size_t orc_merge_vectors_u64(const uint64_t* keys, const uint64_t* counts, const size_t* lens, size_t nv,
                             uint64_t* out_keys, uint64_t* out_counts) {
  std::vector<std::vector<Row>> v(nv);
  size_t off = 0;
  for (size_t i = 0; i < nv; ++i) {
    for (size_t j = 0; j < lens[i]; ++j) v[i].push_back({keys[off + j], counts[off + j]});
    off += lens[i];
  }
  auto m = merge_vectors_total(v);
  for (size_t i = 0; i < m.size(); ++i) { out_keys[i] = (uint64_t)m[i].first; out_counts[i] = m[i].second; }
  return m.size();
}

// serialize_partition_chunk over u64 rows: returns payload size, or -1 with
// orc_last_error() set on u32 overflow.
long long orc_serialize_u64(const uint64_t* keys, const uint64_t* counts, size_t n, uint8_t* out, size_t cap) {
  std::vector<Row> rows;
  for (size_t i = 0; i < n; ++i) rows.push_back({keys[i], counts[i]});
  std::vector<uint8_t> o;
  try {
    if (!serialize_partition_chunk(rows, 64, o)) return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
    return -1;
  }
  memcpy(out, o.data(), std::min(cap, o.size()));
  return (long long)o.size();
}

// 128-byte header image (header.rs write_to).
void orc_header_bytes(unsigned k, int canonical, unsigned partitions, unsigned key_width, unsigned codec_mask,
                      int has_min, unsigned min_count, int has_max, unsigned max_count, uint8_t* out128) {
  Header h;
  h.k = (uint8_t)k; h.canonical = canonical ? 1 : 0; h.partitions = partitions;
  h.key_width = (uint16_t)key_width; h.codec_mask = (uint16_t)codec_mask;
  h.has_min = has_min != 0; h.min_count = min_count; h.has_max = has_max != 0; h.max_count = max_count;
  write_header(h, out128);
}

// Parses a header image; writes [k, canonical, partitions, key_width,
// codec_mask, has_min, min, has_max, max] into out9.  Returns 0 or -1.
int orc_header_parse(const uint8_t* p, size_t n, uint64_t* out9) {
  try {
    Header h = read_header(p, n);
    uint64_t v[9] = {h.k, h.canonical, h.partitions, h.key_width, h.codec_mask,
                     h.has_min, h.min_count, h.has_max, h.max_count};
    memcpy(out9, v, sizeof v);
    return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
    return -1;
  }
}

// Counts an in-memory FASTQ image into per-partition DVLE payloads (no file),
// with `workers` threads: the CPU baseline unit of work.  stats7 receives
// [reads, bases, kmers, rows, chunks, payload_bytes, nanoseconds].
int orc_count_buffer(const uint8_t* d, size_t n, unsigned k, int canonical, size_t partitions, size_t workers,
                     size_t chunk_size, uint64_t* stats7) {
  try {
    auto t0 = std::chrono::steady_clock::now();
    auto chunks = split_chunks(d, n, chunk_size);
    Header h;
    h.k = (uint8_t)k; h.canonical = canonical != 0; h.partitions = (uint32_t)partitions;
    h.key_width = k <= 31 ? 64 : 128; h.codec_mask = 7;
    Writer w(h, 16 * MIB, 2);
    w.keep_data = false;
    CountStats st;
    if (k <= 31) count_chunks<uint64_t>(chunks, k, canonical != 0, partitions, workers, SIZE_MAX, &w, st);
    else count_chunks<u128>(chunks, k, canonical != 0, partitions, workers, SIZE_MAX, &w, st);
    uint64_t tc = 0, tr = 0;
    w.finalize(&tc, &tr);
    auto t1 = std::chrono::steady_clock::now();
    uint64_t v[7] = {st.reads, st.bases, st.kmers, tr, tc, w.next_offset - 128,
                     (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(t1 - t0).count()};
    memcpy(stats7, v, sizeof v);
    return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
    return -1;
  }
}

// Counts an in-memory FASTQ image with one worker (the reproducible layout)
// and returns the full .kite file image.  Returns the image size; the image
// is written to out only when it fits in cap.  -1 on error.
long long orc_count_kite(const uint8_t* d, size_t n, unsigned k, int canonical, size_t partitions,
                         size_t staging_bytes, size_t lanes, size_t chunk_size, int has_min, unsigned min_count,
                         int has_max, unsigned max_count, uint8_t* out, size_t cap, uint64_t* stats3) {
  try {
    auto chunks = split_chunks(d, n, chunk_size);
    Header h;
    h.k = (uint8_t)k; h.canonical = canonical != 0; h.partitions = (uint32_t)partitions;
    h.key_width = k <= 31 ? 64 : 128; h.codec_mask = 7;
    h.has_min = has_min != 0; h.min_count = min_count; h.has_max = has_max != 0; h.max_count = max_count;
    Writer w(h, staging_bytes, lanes);
    CountStats st;
    if (k <= 31) count_chunks<uint64_t>(chunks, k, canonical != 0, partitions, 1, SIZE_MAX, &w, st);
    else count_chunks<u128>(chunks, k, canonical != 0, partitions, 1, SIZE_MAX, &w, st);
    auto file = w.finalize();
    if (stats3) { stats3[0] = st.reads; stats3[1] = st.bases; stats3[2] = st.kmers; }
    if (file.size() <= cap) memcpy(out, file.data(), file.size());
    return (long long)file.size();
  } catch (const std::exception& e) {
    g_err = e.what();
    return -1;
  }
}

// Per-partition payloads of the single-worker count (count_parts above) with
// `threads` threads.  On success returns the total payload bytes, sets *out
// to a malloc'd buffer with the payloads in partition order (free it with
// orc_free) and fills meta[6 * P]: per partition rows, bytes, key_min (lo,
// hi), key_max (lo, hi); stats4 = reads, bases, k-mers, nanoseconds.
long long orc_count_parts(const uint8_t* d, size_t n, unsigned k, int canonical, size_t partitions, size_t threads,
                          size_t chunk_size, uint8_t** out, uint64_t* meta, uint64_t* stats4) {
  try {
    auto t0 = std::chrono::steady_clock::now();
    auto chunks = split_chunks(d, n, chunk_size);
    std::vector<PartOut> parts;
    CountStats st;
    if (k <= 31) count_parts<uint64_t>(chunks, k, canonical != 0, partitions, threads, parts, st);
    else count_parts<u128>(chunks, k, canonical != 0, partitions, threads, parts, st);
    size_t total = 0;
    for (auto& p : parts) total += p.payload.size();
    uint8_t* buf = static_cast<uint8_t*>(malloc(total ? total : 1));
    if (!buf) throw Error("out of memory");
    size_t off = 0;
    for (size_t p = 0; p < partitions; ++p) {
      const PartOut& o = parts[p];
      if (!o.payload.empty()) memcpy(buf + off, o.payload.data(), o.payload.size());
      off += o.payload.size();
      uint64_t* m = meta + 6 * p;
      m[0] = o.rows;
      m[1] = o.payload.size();
      m[2] = (uint64_t)o.kmin;
      m[3] = (uint64_t)(o.kmin >> 64);
      m[4] = (uint64_t)o.kmax;
      m[5] = (uint64_t)(o.kmax >> 64);
    }
    auto t1 = std::chrono::steady_clock::now();
    stats4[0] = st.reads;
    stats4[1] = st.bases;
    stats4[2] = st.kmers;
    stats4[3] = (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(t1 - t0).count();
    *out = buf;
    return (long long)total;
  } catch (const std::exception& e) {
    g_err = e.what();
    return -1;
  }
}

void orc_free(void* p) { free(p); }

// derive_heuristic_plan restated: out7 = [partitions, chunk_size_bytes,
// staging_bytes, worker_threads, local_flush_bytes, decomp_threads, lanes].
int orc_derive_plan(uint64_t input_bytes, double avg_read_len, int comp, unsigned k, uint64_t partitions,
                    uint64_t threads, uint64_t mem, long long buffer_mb, uint64_t chunk_kmers, uint64_t* out7) {
  try {
    Plan p = derive_plan(input_bytes, avg_read_len, (Compression)comp, k, partitions, threads, mem, (long)buffer_mb,
                         chunk_kmers);
    uint64_t v[7] = {p.partitions, p.chunk_size_bytes, p.staging_bytes, p.worker_threads, p.local_flush_bytes,
                     p.decomp_threads, p.writer_lanes};
    memcpy(out7, v, sizeof v);
    return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
    return -1;
  }
}

// parse_memory_spec restated: bytes or -1.
long long orc_parse_memory_spec(const char* spec) {
  try {
    return (long long)parse_memory_spec(spec);
  } catch (const std::exception& e) {
    g_err = e.what();
    return -1;
  }
}

// Dump (kite dump -o -) of a .kite image into out; returns bytes (written
// only when they fit), -1 on error.
long long orc_dump_kite(const uint8_t* img, size_t n, char* out, size_t cap) {
  try {
    Reader r;
    r.open(img, n);
    std::string s;
    for (size_t p = 0; p < r.h.partitions; ++p) dump_partition(r, p, s);
    if (s.size() <= cap) memcpy(out, s.data(), s.size());
    return (long long)s.size();
  } catch (const std::exception& e) {
    g_err = e.what();
    return -1;
  }
}

// Merge of .kite files by path (kite merge); writes the output image.
// The merge of n in-memory .kite images with `threads` threads working on
// partitions in turn (run_merge's rayon loop over partition batches,
// src/merge/mod.rs:117-151): per partition load_partition_counts of every
// input, the input's header filter, merge_vectors_total and
// serialize_partition_chunk, exactly as merge_files, without the writer.
// stats4 = rows in, rows out, payload bytes out, nanoseconds (from the
// images in memory to every payload made).  0 or -1.
int orc_merge_images(const uint8_t** imgs, const size_t* lens, size_t n, size_t threads, uint64_t* stats4) {
  try {
    std::vector<Reader> rs(n);
    for (size_t i = 0; i < n; ++i) rs[i].open(imgs[i], lens[i]);
    auto t0 = std::chrono::steady_clock::now();
    const size_t P = rs[0].h.partitions;
    std::atomic<size_t> next(0);
    std::atomic<uint64_t> rows_in(0), rows_out(0), bytes_out(0);
    std::atomic<int> failed(0);
    std::mutex emu;
    std::string err;
    auto work = [&]() {
      std::vector<uint8_t> payload;
      for (size_t p; (p = next.fetch_add(1)) < P;) {
        try {
          std::vector<std::vector<Row>> vecs;
          for (auto& r : rs) {
            auto rows = load_partition_counts(r, p);
            rows_in += rows.size();
            if (r.h.has_min || r.h.has_max) {
              std::vector<Row> kept;
              for (auto& x : rows)
                if (passes(x.second, r.h)) kept.push_back(x);
              rows.swap(kept);
            }
            vecs.push_back(std::move(rows));
          }
          auto merged = merge_vectors_total(vecs);
          if (serialize_partition_chunk(merged, rs[0].h.key_width, payload)) {
            rows_out += merged.size();
            bytes_out += payload.size();
          }
        } catch (const std::exception& e) {
          std::lock_guard<std::mutex> g(emu);
          err = e.what();
          failed = 1;
        }
      }
    };
    std::vector<std::thread> th;
    for (size_t t = 0; t < std::max<size_t>(threads, 1); ++t) th.emplace_back(work);
    for (auto& t : th) t.join();
    if (failed) throw Error(err);
    stats4[0] = rows_in;
    stats4[1] = rows_out;
    stats4[2] = bytes_out;
    stats4[3] = (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now() - t0)
                    .count();
    return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
    return -1;
  }
}

long long orc_merge_files(const char** paths, size_t n, size_t lanes, uint8_t* out, size_t cap) {
  try {
    std::vector<std::string> ps;
    for (size_t i = 0; i < n; ++i) ps.push_back(paths[i]);
    auto file = merge_files(ps, lanes);
    if (file.size() <= cap) memcpy(out, file.data(), file.size());
    return (long long)file.size();
  } catch (const std::exception& e) {
    g_err = e.what();
    return -1;
  }
}

}  // extern "C"

// ===========================================================================
// CLI (kite_oracle): count / dump / merge / info with the reference's flags.
// ===========================================================================
#ifdef ORC_MAIN
static void usage() {
  fprintf(stderr,
          "kite_oracle count -i IN -o OUT.kite [-k K] [--canonical true|false] [--min N] [--max N]\n"
          "                  [-t N] [--partitions N] [--chunk-kmers N] [--memory SPEC] [--buffer MB]\n"
          "                  [--workers N]   (default 1: the reproducible single-worker layout)\n"
          "kite_oracle dump -i IN.kite -o -|FILE\n"
          "kite_oracle merge -i A.kite B.kite ... -o OUT.kite [--lanes N]\n"
          "kite_oracle info -i IN.kite\n");
}

static bool parse_bool(const std::string& v) {
  if (v == "true") return true;
  if (v == "false") return false;
  throw Error("invalid value '" + v + "' for '--canonical <BOOL>'");
}

static int cmd_count(int argc, char** argv) {
  std::string in, out, mem;
  unsigned k = 21;
  bool canonical = false;
  bool has_min = false, has_max = false;
  uint32_t mn = 0, mx = 0;
  size_t threads = 0, partitions = 0, chunk_kmers = 0, workers_override = 1;
  long buffer_mb = -1;
  int zstd_level = 0;
  for (int i = 0; i < argc; ++i) {
    std::string a = argv[i];
    auto val = [&]() -> std::string {
      if (i + 1 >= argc) throw Error("missing value for " + a);
      return argv[++i];
    };
    if (a == "-i" || a == "--input") in = val();
    else if (a == "-o" || a == "--output") out = val();
    else if (a == "-k" || a == "--kmer") k = (unsigned)std::stoul(val());
    else if (a == "--canonical") canonical = parse_bool(val());
    else if (a == "--min") { has_min = true; mn = (uint32_t)std::stoul(val()); }
    else if (a == "--max") { has_max = true; mx = (uint32_t)std::stoul(val()); }
    else if (a == "-t" || a == "--threads") threads = std::stoul(val());
    else if (a == "--partitions") partitions = std::stoul(val());
    else if (a == "--chunk-kmers") chunk_kmers = std::stoul(val());
    else if (a == "--memory") mem = val();
    else if (a == "--buffer") buffer_mb = std::stol(val());
    else if (a == "--mode") {
      const std::string m = val();
      if (m == "fast") zstd_level = 0;
      else if (m == "balanced") zstd_level = 2;
      else if (m == "compact") zstd_level = 5;
      else throw Error("invalid --mode " + m);
    }
    else if (a == "--workers") workers_override = std::stoul(val());
    else throw Error("unknown argument " + a);
  }
  if (k < 1 || k > 64) throw Error("oracle supports k in 1..=64");
  if (partitions != 0 && (partitions & (partitions - 1))) throw Error("invalid partition count");
  if (partitions == 1) throw Error("partitions must be at least 2");
  if (has_min && has_max && mn > mx) throw Error("invalid count filter range");
  Compression comp = detect_compression(in);
  size_t total_threads = threads ? threads : std::max(1u, std::thread::hardware_concurrency());
  size_t memb = resolve_memory_limit_bytes(mem);
  FILE* f = fopen(in.c_str(), "rb");
  if (!f) throw Error("failed to open input FASTQ.\nInput: " + in);
  fseek(f, 0, SEEK_END);
  size_t input_bytes = (size_t)ftell(f);
  fclose(f);
  double avg = partitions == 0 ? sample_avg_read_len(in, comp) : 150.0;
  Plan plan = derive_plan(input_bytes, avg, comp, k, partitions, total_threads, memb, buffer_mb, chunk_kmers);
  size_t workers = std::max<size_t>(1, workers_override);
  Header h;
  h.k = (uint8_t)k; h.canonical = canonical; h.partitions = (uint32_t)plan.partitions;
  h.key_width = k <= 31 ? 64 : 128; h.codec_mask = 7;
  h.has_min = has_min; h.min_count = mn; h.has_max = has_max; h.max_count = mx;
  size_t lanes = std::min<size_t>(std::max<size_t>((workers + 7) / 8, 2), 6);
  Writer w(h, plan.staging_bytes, lanes);
  auto t0 = std::chrono::steady_clock::now();
  std::vector<std::vector<uint8_t>> store;
  read_all_chunks(in, comp, plan.chunk_size_bytes, store);
  std::vector<std::pair<const uint8_t*, size_t>> chunks;
  for (auto& c : store) chunks.push_back({c.data(), c.size()});
  CountStats st;
  if (k <= 31)
    count_chunks<uint64_t>(chunks, k, canonical, plan.partitions, workers, plan.local_flush_bytes, &w, st, zstd_level);
  else count_chunks<u128>(chunks, k, canonical, plan.partitions, workers, plan.local_flush_bytes, &w, st, zstd_level);
  uint64_t tc = 0, tr = 0;
  auto file = w.finalize(&tc, &tr);
  if (out != "/dev/null") write_file(out, file);
  double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  fprintf(stderr,
          "[kite count] summary reads=%llu bases=%llu kmers=%llu raw_rows_written=%llu chunks=%llu "
          "header_min=%s header_max=%s elapsed=%.3fs\n",
          (unsigned long long)st.reads, (unsigned long long)st.bases, (unsigned long long)st.kmers,
          (unsigned long long)tr, (unsigned long long)tc, has_min ? std::to_string(mn).c_str() : "none",
          has_max ? std::to_string(mx).c_str() : "none", el);
  fprintf(stderr, "[kite count] plan partitions=%zu chunk=%zu staging=%zu lanes=%zu\n", plan.partitions,
          plan.chunk_size_bytes, plan.staging_bytes, lanes);
  return 0;
}

static int cmd_dump(int argc, char** argv) {
  std::string in, out = "-";
  for (int i = 0; i < argc; ++i) {
    std::string a = argv[i];
    if ((a == "-i" || a == "--input") && i + 1 < argc) in = argv[++i];
    else if ((a == "-o" || a == "--output") && i + 1 < argc) out = argv[++i];
    else if ((a == "-t" || a == "--threads" || a == "--buffer") && i + 1 < argc) ++i;
    else throw Error("unknown argument " + a);
  }
  auto bytes = read_file(in);
  Reader r;
  r.open(bytes.data(), bytes.size());
  FILE* f = out == "-" ? stdout : fopen(out.c_str(), "wb");
  if (!f) throw Error("failed to create " + out);
  std::string buf;
  for (size_t p = 0; p < r.h.partitions; ++p) {
    buf.clear();
    dump_partition(r, p, buf);
    fwrite(buf.data(), 1, buf.size(), f);
  }
  if (f != stdout) fclose(f);
  else fflush(stdout);
  return 0;
}

static int cmd_merge(int argc, char** argv) {
  std::vector<std::string> ins;
  std::string out;
  size_t lanes = std::min<size_t>(std::max<size_t>((std::thread::hardware_concurrency() + 7) / 8, 2), 6);
  for (int i = 0; i < argc; ++i) {
    std::string a = argv[i];
    if (a == "-i" || a == "--input") {
      while (i + 1 < argc && argv[i + 1][0] != '-') ins.push_back(argv[++i]);
    } else if ((a == "-o" || a == "--output") && i + 1 < argc) out = argv[++i];
    else if ((a == "-t" || a == "--threads") && i + 1 < argc) ++i;
    else if (a == "--lanes" && i + 1 < argc) lanes = std::stoul(argv[++i]);
    else throw Error("unknown argument " + a);
  }
  auto file = merge_files(ins, lanes);
  write_file(out, file);
  return 0;
}

static std::string label_of(const std::string& path, size_t index) {
  std::string name = path.substr(path.find_last_of('/') == std::string::npos ? 0 : path.find_last_of('/') + 1);
  for (const char* suf : {".fastq.gz", ".fq.gz", ".fastq", ".fq", ".kite", ".tsv", ".txt", ".gz"}) {
    const size_t l = strlen(suf);
    if (name.size() >= l && name.compare(name.size() - l, l, suf) == 0) {
      name.resize(name.size() - l);
      break;
    }
  }
  return name.empty() ? "sample" + std::to_string(index + 1) : name;
}

static int cmd_histo(int argc, char** argv) {
  std::vector<std::string> ins, labels;
  std::string out;
  for (int i = 0; i < argc; ++i) {
    std::string a = argv[i];
    if (a == "-i" || a == "--input") {
      while (i + 1 < argc && argv[i + 1][0] != '-') ins.push_back(argv[++i]);
    } else if (a == "--label") {
      while (i + 1 < argc && argv[i + 1][0] != '-') labels.push_back(argv[++i]);
    } else if ((a == "-o" || a == "--output") && i + 1 < argc) out = argv[++i];
    else if ((a == "-t" || a == "--threads") && i + 1 < argc) ++i;
    else if (a == "-p" || a == "--progress" || a == "--test-mode") continue;
    else throw Error("unknown argument " + a);
  }
  if (labels.empty())
    for (size_t i = 0; i < ins.size(); ++i) labels.push_back(label_of(ins[i], i));
  std::vector<std::map<uint64_t, uint64_t>> hs;
  std::map<uint64_t, int> bins;
  for (auto& in : ins) {
    auto bytes = read_file(in);
    Reader r;
    r.open(bytes.data(), bytes.size());
    hs.push_back(histo_of(r));
    for (auto& kv : hs.back()) bins[kv.first] = 1;
  }
  std::string t = "count";
  for (auto& l : labels) t += "\t" + l;
  t += "\n";
  for (auto& b : bins) {
    t += std::to_string(b.first);
    for (auto& h : hs) {
      auto it = h.find(b.first);
      t += "\t" + std::to_string(it == h.end() ? 0 : it->second);
    }
    t += "\n";
  }
  std::vector<uint8_t> v(t.begin(), t.end());
  write_file(out, v);
  return 0;
}

static int cmd_query(int argc, char** argv) {
  std::string in, kmer;
  for (int i = 0; i < argc; ++i) {
    std::string a = argv[i];
    if ((a == "-i" || a == "--input") && i + 1 < argc) in = argv[++i];
    else if ((a == "-k" || a == "--kmer") && i + 1 < argc) kmer = argv[++i];
    else if (a == "--test-mode") continue;
    else throw Error("unknown argument " + a);
  }
  auto bytes = read_file(in);
  Reader r;
  r.open(bytes.data(), bytes.size());
  const u128 key = encode_query_kmer(kmer, r.h);
  size_t p = 0;
  const uint64_t c = query_key(r, key, &p);
  std::vector<char> ks(r.h.k + 1, 0);
  decode_kmer(key, r.h.k, ks.data());
  auto opt = [](bool has, uint32_t v) { return has ? std::to_string(v) : std::string("none"); };
  printf("Kite Query\n  Database:           %s\n  Query:              %s\n  Partition:          %zu\n"
         "  Count:              %llu\n  Header Min Count:   %s\n  Header Max Count:   %s\n  Header Filter:      %s\n",
         in.c_str(), ks.data(), p, (unsigned long long)c, opt(r.h.has_min, r.h.min_count).c_str(),
         opt(r.h.has_max, r.h.max_count).c_str(),
         c == 0 ? "not present" : (passes(c, r.h) ? "included" : "excluded from downstream analysis/output"));
  return 0;
}

static int cmd_info(int argc, char** argv) {
  std::string in;
  for (int i = 0; i < argc; ++i)
    if ((std::string(argv[i]) == "-i") && i + 1 < argc) in = argv[++i];
  auto bytes = read_file(in);
  Reader r;
  r.open(bytes.data(), bytes.size());
  printf("k=%u canonical=%u partitions=%u key_width=%u codec_mask=%u total_chunks=%llu total_rows=%llu\n", r.h.k,
         r.h.canonical, r.h.partitions, r.h.key_width, r.h.codec_mask, (unsigned long long)r.h.total_chunks,
         (unsigned long long)r.h.total_rows);
  return 0;
}

int main(int argc, char** argv) {
  if (argc < 2) { usage(); return 2; }
  std::string cmd = argv[1];
  try {
    if (cmd == "count") return cmd_count(argc - 2, argv + 2);
    if (cmd == "dump") return cmd_dump(argc - 2, argv + 2);
    if (cmd == "merge") return cmd_merge(argc - 2, argv + 2);
    if (cmd == "info") return cmd_info(argc - 2, argv + 2);
    if (cmd == "histo") return cmd_histo(argc - 2, argv + 2);
    if (cmd == "query") return cmd_query(argc - 2, argv + 2);
    usage();
    return 2;
  } catch (const std::exception& e) {
    fprintf(stderr, "Error: %s\n", e.what());
    return 1;
  }
}
#endif
