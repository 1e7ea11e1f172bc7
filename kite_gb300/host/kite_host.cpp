// libkite_host.so: .kite writer/reader, planner, FASTQ ingest, TSV dump and
// the synthetic-input generator.  See include/kite_host.h for the contract and
// the reference functions each part restates.
#include "kite_host.h"

#include <algorithm>
#include <atomic>
#include <cerrno>
#include <condition_variable>
#include <deque>
#include <dlfcn.h>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fcntl.h>
#include <memory>
#include <mutex>
#include <queue>
#include <string>
#include <sys/mman.h>
#include <sys/stat.h>
#include <thread>
#include <unistd.h>
#include <vector>

#if KITE_HAVE_ZLIB
#include <zlib.h>
#endif

typedef unsigned __int128 u128;

namespace {

constexpr uint64_t MiB = 1024ull * 1024ull;
constexpr uint64_t GiB = 1024ull * MiB;

thread_local std::string g_err;

int set_err(const std::string& m, int code = -1) {
  g_err = m;
  return code;
}

inline void le(std::vector<uint8_t>& o, uint64_t v, int n) {
  for (int i = 0; i < n; ++i) o.push_back((uint8_t)(v >> (8 * i)));
}
inline uint64_t rd(const uint8_t* p, int n) {
  uint64_t v = 0;
  for (int i = 0; i < n; ++i) v |= (uint64_t)p[i] << (8 * i);
  return v;
}

// zstd, loaded at run time from the system's libzstd.so.1 (the image ships the
// library without headers).  The few entry points used are declared here with
// their published prototypes.
struct Zstd {
  size_t (*compress)(void*, size_t, const void*, size_t, int) = nullptr;
  size_t (*decompress)(void*, size_t, const void*, size_t) = nullptr;
  size_t (*bound)(size_t) = nullptr;
  unsigned (*is_error)(size_t) = nullptr;
  bool ok = false;
};
const Zstd& zstd() {
  static const Zstd z = [] {
    Zstd r;
    void* h = dlopen("libzstd.so.1", RTLD_NOW | RTLD_LOCAL);
    if (!h) return r;
    r.compress = reinterpret_cast<size_t (*)(void*, size_t, const void*, size_t, int)>(dlsym(h, "ZSTD_compress"));
    r.decompress = reinterpret_cast<size_t (*)(void*, size_t, const void*, size_t)>(dlsym(h, "ZSTD_decompress"));
    r.bound = reinterpret_cast<size_t (*)(size_t)>(dlsym(h, "ZSTD_compressBound"));
    r.is_error = reinterpret_cast<unsigned (*)(size_t)>(dlsym(h, "ZSTD_isError"));
    r.ok = r.compress && r.decompress && r.bound && r.is_error;
    return r;
  }();
  return z;
}

// KiteHeader::write_to (src/format/header.rs:62-92): 128 bytes, LE.
void header_image(const kite_header_info& h, uint64_t cio, uint64_t pto, uint64_t fo, uint64_t tc, uint64_t tr,
                  uint8_t* out) {
  std::vector<uint8_t> o;
  o.reserve(128);
  o.insert(o.end(), {'K', 'X', '2', '!'});
  le(o, 1, 2);
  o.push_back((uint8_t)h.k);
  o.push_back(h.canonical ? 1 : 0);
  le(o, h.partitions, 4);
  le(o, h.key_width, 2);
  le(o, h.codec_mask, 2);
  le(o, 0, 4);
  le(o, cio, 8);
  le(o, pto, 8);
  le(o, fo, 8);
  le(o, tc, 8);
  le(o, tr, 8);
  uint8_t res[68] = {0};
  if (h.has_min || h.has_max) {
    memcpy(res, "KMT1", 4);
    uint32_t flags = (h.has_min ? 1u : 0u) | (h.has_max ? 2u : 0u);
    uint32_t mn = h.has_min ? h.min_count : 0, mx = h.has_max ? h.max_count : 0;
    memcpy(res + 4, &flags, 4);
    memcpy(res + 8, &mn, 4);
    memcpy(res + 12, &mx, 4);
  }
  o.insert(o.end(), res, res + 68);
  memcpy(out, o.data(), 128);
}

}  // namespace

// ============================================================================
// Writer: ConcurrentKiteWriter's layout for a single appending thread.  The
// byte layout follows from the order in which staged partitions are flushed:
// each flush takes the next file offset at once, and the bytes go out by
// positional writes, staged buffers on `write_lanes` threads (at most four)
// while appends go on, chunks of at least the staging size directly.
// ============================================================================
namespace {
int pwrite_all(int fd, const uint8_t* p, size_t n, uint64_t off) {
  while (n) {
    const ssize_t r = pwrite(fd, p, n, (off_t)off);
    if (r < 0) {
      if (errno == EINTR) continue;
      return -1;
    }
    p += r;
    n -= (size_t)r;
    off += (uint64_t)r;
  }
  return 0;
}
}  // namespace

struct kite_writer {
  struct Meta {
    uint64_t off, rows, enc, raw;
    uint32_t codec;
    uint64_t kmin[4], kmax[4];
  };
  struct Pending {
    uint64_t rel;
    Meta m;
  };
  struct Part {
    std::vector<uint8_t> buf;
    std::vector<Pending> pending;
    std::vector<Meta> committed;
  };
  kite_header_info h{};
  uint64_t staging = 0, high = 0, low = 0, next_off = 128, staged = 0;
  std::vector<Part> parts;
  // Emptied staging buffers, kept for the next partition that stages: a
  // partition usually stages one chunk per segment, so a buffer of its own
  // would take its page faults on every byte it ever holds, while the
  // buffers in use at once are bounded by the drain threshold.
  std::vector<std::vector<uint8_t>> spare;
  FILE* f = nullptr;
  int fd = -1;
  std::vector<uint8_t> image;  // in-memory mode
  bool in_memory = false;
  bool finalized = false;
  // write lanes (file mode): staged buffers queued with their offsets
  struct Job {
    std::vector<uint8_t> buf;
    uint64_t off;
  };
  std::vector<std::thread> lanes;
  std::mutex mu;
  std::condition_variable cv_job, cv_done;
  std::deque<Job> jobs;
  uint64_t queued = 0;  // bytes queued or being written
  bool stop = false;
  std::string lane_err;

  void lane_loop() {
    std::unique_lock<std::mutex> lk(mu);
    for (;;) {
      cv_job.wait(lk, [&] { return stop || !jobs.empty(); });
      if (jobs.empty()) return;
      Job j = std::move(jobs.front());
      jobs.pop_front();
      lk.unlock();
      const int r = pwrite_all(fd, j.buf.data(), j.buf.size(), j.off);
      const int e = errno;
      lk.lock();
      if (r && lane_err.empty()) lane_err = std::string("write failed: ") + strerror(e);
      queued -= j.buf.size();
      j.buf.clear();
      spare.push_back(std::move(j.buf));
      cv_done.notify_all();
    }
  }
  void start_lanes(uint64_t n) {
    for (uint64_t i = 0; i < n; ++i) lanes.emplace_back([this] { lane_loop(); });
  }
  void stop_lanes() {
    {
      std::lock_guard<std::mutex> lk(mu);
      stop = true;
    }
    cv_job.notify_all();
    for (auto& t : lanes) t.join();
    lanes.clear();
  }
  // every queued write done; the first write error, if any
  int wait_writes() {
    std::unique_lock<std::mutex> lk(mu);
    cv_done.wait(lk, [&] { return queued == 0; });
    return lane_err.empty() ? 0 : set_err(lane_err);
  }
  std::vector<uint8_t> take_buffer() {
    std::lock_guard<std::mutex> lk(mu);
    if (spare.empty()) return std::vector<uint8_t>();
    std::vector<uint8_t> b = std::move(spare.back());
    spare.pop_back();
    return b;
  }

  int put(const uint8_t* p, size_t n, uint64_t* off) {
    *off = next_off;
    next_off += n;
    if (in_memory) {
      image.insert(image.end(), p, p + n);
    } else if (n && pwrite_all(fd, p, n, *off)) {
      return set_err(std::string("write failed: ") + strerror(errno));
    }
    return 0;
  }
  int flush_part(size_t pid) {
    Part& s = parts[pid];
    if (s.buf.empty()) return 0;
    const uint64_t off = next_off;
    next_off += s.buf.size();
    staged -= s.buf.size();
    for (auto& pd : s.pending) {
      Meta m = pd.m;
      m.off = off + pd.rel;
      s.committed.push_back(m);
    }
    s.pending.clear();
    if (in_memory || lanes.empty()) {
      if (in_memory) image.insert(image.end(), s.buf.begin(), s.buf.end());
      else if (pwrite_all(fd, s.buf.data(), s.buf.size(), off))
        return set_err(std::string("write failed: ") + strerror(errno));
      s.buf.clear();
      std::lock_guard<std::mutex> lk(mu);
      spare.push_back(std::move(s.buf));
    } else {
      std::unique_lock<std::mutex> lk(mu);
      // bounded: no more than the drain threshold waits for the disk
      cv_done.wait(lk, [&] { return queued <= high; });
      if (!lane_err.empty()) return set_err(lane_err);
      queued += s.buf.size();
      jobs.push_back(Job{std::move(s.buf), off});
      lk.unlock();
      cv_job.notify_one();
    }
    s.buf = std::vector<uint8_t>();
    return 0;
  }
  bool needs_drain() const { return staged >= high; }
  int drain_one(bool* did) {
    size_t best = SIZE_MAX, bytes = 0;
    for (size_t p = 0; p < parts.size(); ++p)
      if (parts[p].buf.size() > bytes) {
        bytes = parts[p].buf.size();
        best = p;
      }
    *did = best != SIZE_MAX;
    return *did ? flush_part(best) : 0;
  }
  int drain_excess() {
    for (int attempts = 0; staged > low && attempts < 4; ++attempts) {
      bool did;
      if (drain_one(&did)) return -1;
      if (!did) break;
    }
    return 0;
  }
};

extern "C" {

const char* kite_host_last_error(void) { return g_err.c_str(); }

uint64_t kite_suggest_write_lanes(uint64_t workers) {
  return std::min<uint64_t>(std::max<uint64_t>((workers + 7) / 8, 2), 6);
}

kite_writer* kite_writer_open(const char* path, const kite_header_info* h, uint64_t staging_bytes,
                              uint64_t write_lanes) {
  if (!h || h->partitions == 0) {
    set_err("bad writer arguments");
    return nullptr;
  }
  auto* w = new kite_writer();
  w->h = *h;
  w->staging = staging_bytes;
  w->high = std::max<uint64_t>(staging_bytes * write_lanes * 4, staging_bytes);
  w->low = w->high / 2;
  w->parts.resize(h->partitions);
  uint8_t hdr[128];
  header_image(*h, 0, 0, 0, 0, 0, hdr);
  if (!path) {
    w->in_memory = true;
    w->image.assign(hdr, hdr + 128);
  } else {
    w->f = fopen(path, "wb+");
    if (!w->f) {
      set_err(std::string("failed to create ") + path + ": " + strerror(errno));
      delete w;
      return nullptr;
    }
    if (fwrite(hdr, 1, 128, w->f) != 128 || fflush(w->f)) {
      set_err("header write failed");
      fclose(w->f);
      delete w;
      return nullptr;
    }
    w->fd = fileno(w->f);
    w->start_lanes(std::max<uint64_t>(1, std::min<uint64_t>(write_lanes, 4)));
  }
  return w;
}

// append_chunk src/count/writer.rs:285-348
int kite_writer_append(kite_writer* w, const kite_chunk_meta* m, const uint8_t* data, size_t n) {
  if (!w || !m || m->partition_id >= w->parts.size()) return set_err("bad append");
  auto& s = w->parts[m->partition_id];
  if (!s.buf.empty() && s.buf.size() + n > w->staging)
    if (w->flush_part(m->partition_id)) return -1;
  kite_writer::Meta mm{};
  mm.rows = m->row_count;
  mm.enc = n;
  mm.raw = m->raw_bytes;
  mm.codec = m->codec;
  memcpy(mm.kmin, m->key_min_lo, 16);
  memcpy(mm.kmin + 2, m->key_min_hi, 16);
  memcpy(mm.kmax, m->key_max_lo, 16);
  memcpy(mm.kmax + 2, m->key_max_hi, 16);
  if (n >= w->staging) {
    if (w->put(data, n, &mm.off)) return -1;
    s.committed.push_back(mm);
  } else {
    kite_writer::Pending pd{s.buf.size(), mm};
    if (s.buf.capacity() == 0) {
      s.buf = w->take_buffer();
      if (s.buf.capacity() == 0) s.buf.reserve(w->staging);  // a staged partition never holds more
    }
    s.buf.insert(s.buf.end(), data, data + n);
    s.pending.push_back(pd);
    w->staged += n;
    if (s.buf.size() >= w->staging)
      if (w->flush_part(m->partition_id)) return -1;
  }
  if (w->needs_drain()) return w->drain_excess();
  return 0;
}

int kite_writer_emit(void* w, const kite_chunk_meta* meta, const uint8_t* data, size_t len) {
  return kite_writer_append(static_cast<kite_writer*>(w), meta, data, len) ? 1 : 0;
}

// CountWorker::flush_all's trailing loop (src/count/worker.rs:286-290)
int kite_writer_worker_drain(kite_writer* w) {
  while (w->needs_drain()) {
    bool did;
    if (w->drain_one(&did)) return -1;
    if (!did) break;
  }
  return 0;
}

// finalize src/count/writer.rs:350-494
int kite_writer_finalize(kite_writer* w, uint64_t* total_chunks, uint64_t* total_rows) {
  if (!w || w->finalized) return set_err("writer already finalized");
  std::vector<std::vector<kite_writer::Meta>> all(w->parts.size());
  for (size_t p = 0; p < w->parts.size(); ++p) {
    if (w->flush_part(p)) return -1;
    all[p] = w->parts[p].committed;
    std::sort(all[p].begin(), all[p].end(),
              [](const kite_writer::Meta& a, const kite_writer::Meta& b) { return a.off < b.off; });
  }
  if (!w->in_memory && w->wait_writes()) return -1;
  uint64_t data_end = w->next_off, tc = 0, tr = 0;
  for (auto& v : all)
    for (auto& c : v) {
      tc++;
      tr += c.rows;
    }
  const uint64_t cio = data_end, pto = cio + tc * 128, fo = pto + w->parts.size() * 40;
  std::vector<uint8_t> t;
  t.reserve(tc * 128 + w->parts.size() * 40 + 24);
  for (size_t p = 0; p < all.size(); ++p)
    for (auto& c : all[p]) {
      le(t, p, 4);
      le(t, c.codec, 4);
      le(t, c.off, 8);
      le(t, c.enc, 8);
      le(t, c.raw, 8);
      le(t, c.rows, 8);
      for (int i = 0; i < 4; ++i) le(t, c.kmin[i], 8);
      for (int i = 0; i < 4; ++i) le(t, c.kmax[i], 8);
      for (int i = 0; i < 24; ++i) t.push_back(0);
    }
  uint64_t first = 0;
  for (auto& v : all) {
    uint64_t rows = 0, bytes = 0, minoff = UINT64_MAX;
    for (auto& c : v) {
      rows += c.rows;
      bytes += c.enc;
      minoff = std::min(minoff, c.off);
    }
    le(t, first, 8);
    le(t, v.size(), 8);
    le(t, rows, 8);
    le(t, v.empty() ? 0 : minoff, 8);
    le(t, bytes, 8);
    first += v.size();
  }
  le(t, tc, 8);
  le(t, tr, 8);
  t.insert(t.end(), {'K', 'X', '2', 'F', 'O', 'O', 'T', '!'});
  uint8_t hdr[128];
  header_image(w->h, cio, pto, fo, tc, tr, hdr);
  if (w->in_memory) {
    w->image.insert(w->image.end(), t.begin(), t.end());
    memcpy(w->image.data(), hdr, 128);
  } else {
    if (pwrite_all(w->fd, t.data(), t.size(), data_end) || pwrite_all(w->fd, hdr, 128, 0))
      return set_err(std::string("finalize write failed: ") + strerror(errno));
    if (ftruncate(w->fd, (off_t)(fo + 24))) return set_err("set_len failed");
  }
  w->finalized = true;
  if (total_chunks) *total_chunks = tc;
  if (total_rows) *total_rows = tr;
  return 0;
}

const uint8_t* kite_writer_image(kite_writer* w, size_t* len) {
  if (!w || !w->in_memory) return nullptr;
  if (len) *len = w->image.size();
  return w->image.data();
}

void kite_writer_close(kite_writer* w) {
  if (!w) return;
  w->stop_lanes();  // the queued writes finish first
  if (w->f) fclose(w->f);
  delete w;
}

}  // extern "C"

// ============================================================================
// Reader
// ============================================================================
struct kite_reader {
  const uint8_t* data = nullptr;
  size_t len = 0;
  void* map = nullptr;
  std::vector<uint8_t> own;
  kite_header_info h{};
  uint64_t cio = 0, pto = 0, fo = 0, total_chunks = 0, total_rows = 0;
  std::vector<uint64_t> c_off, c_len, c_rows, c_raw, p_first, p_count;
  std::vector<uint32_t> c_codec;
  // payloads as the decoders read them: the file's bytes, or, when a chunk is
  // zstd-compressed, every payload copied into `dec` with those chunks
  // decompressed (run_data_for_decode src/dump/reader.rs:162-186)
  const uint8_t* d_base = nullptr;
  size_t d_len = 0;
  std::vector<uint64_t> d_off, d_size;
  std::vector<uint32_t> d_codec;
  std::vector<uint8_t> dec;
};

namespace {

// Payloads for the decoders: zero-copy unless some chunk is zstd-compressed.
int reader_decode(kite_reader* r) {
  const size_t nc = r->c_off.size();
  bool any = false;
  for (size_t c = 0; c < nc; ++c) any |= (r->c_codec[c] & 4u) != 0;
  r->d_codec = r->c_codec;
  if (!any) {
    r->d_base = r->data;
    r->d_len = r->len;
    r->d_off = r->c_off;
    r->d_size = r->c_len;
    return 0;
  }
  const Zstd& z = zstd();
  if (!z.ok) return set_err("zstd decompress failed: libzstd.so.1 is not available");
  uint64_t total = 0;
  for (size_t c = 0; c < nc; ++c) total += (r->c_codec[c] & 4u) ? r->c_raw[c] : r->c_len[c];
  r->dec.resize(total + 16);
  r->d_off.resize(nc);
  r->d_size.resize(nc);
  uint64_t at = 0;
  for (size_t c = 0; c < nc; ++c) {
    const uint8_t* src = r->data + r->c_off[c];
    r->d_off[c] = at;
    if (r->c_codec[c] & 4u) {
      const size_t got = z.decompress(r->dec.data() + at, r->c_raw[c], src, r->c_len[c]);
      if (z.is_error(got)) return set_err("zstd decompress failed: corrupt chunk " + std::to_string(c));
      if (got != r->c_raw[c])
        return set_err("decoded payload size mismatch: got " + std::to_string(got) + ", expected " +
                       std::to_string(r->c_raw[c]));
      r->d_size[c] = got;
      r->d_codec[c] &= ~4u;
    } else {
      memcpy(r->dec.data() + at, src, r->c_len[c]);
      r->d_size[c] = r->c_len[c];
    }
    at += r->d_size[c];
  }
  r->d_base = r->dec.data();
  r->d_len = at;
  return 0;
}

int reader_parse(kite_reader* r) {
  const uint8_t* p = r->data;
  const size_t n = r->len;
  if (n < 128 + 24) return set_err("file too small");
  if (memcmp(p, "KX2!", 4)) return set_err("invalid magic: expected KITE");
  if (rd(p + 4, 2) != 1) return set_err("unsupported version: " + std::to_string(rd(p + 4, 2)));
  r->h.k = p[6];
  r->h.canonical = p[7];
  r->h.partitions = (uint32_t)rd(p + 8, 4);
  r->h.key_width = (uint16_t)rd(p + 12, 2);
  r->h.codec_mask = (uint16_t)rd(p + 14, 2);
  r->cio = rd(p + 20, 8);
  r->pto = rd(p + 28, 8);
  r->fo = rd(p + 36, 8);
  r->total_rows = rd(p + 52, 8);
  if (!memcmp(p + 60, "KMT1", 4)) {
    uint32_t flags = (uint32_t)rd(p + 64, 4);
    r->h.has_min = (flags & 1) != 0;
    r->h.has_max = (flags & 2) != 0;
    r->h.min_count = (uint32_t)rd(p + 68, 4);
    r->h.max_count = (uint32_t)rd(p + 72, 4);
  }
  if (r->fo + 24 > n) return set_err("footer out of bounds");
  if (memcmp(p + r->fo + 16, "KX2FOOT!", 8)) return set_err("invalid footer magic");
  r->total_chunks = rd(p + r->fo, 8);
  const uint64_t P = r->h.partitions;
  if (r->pto + P * 40 > n) return set_err("partition table out of bounds");
  if (r->pto < r->cio) return set_err("invalid chunk index offsets");
  if ((r->pto - r->cio) % 128) return set_err("chunk index size misaligned");
  const uint64_t nc = (r->pto - r->cio) / 128;
  for (uint64_t c = 0; c < nc; ++c) {
    const uint8_t* e = p + r->cio + c * 128;
    r->c_codec.push_back((uint32_t)rd(e + 4, 4));
    r->c_off.push_back(rd(e + 8, 8));
    r->c_len.push_back(rd(e + 16, 8));
    r->c_raw.push_back(rd(e + 24, 8));
    r->c_rows.push_back(rd(e + 32, 8));
  }
  for (uint64_t b = 0; b < P; ++b) {
    const uint8_t* e = p + r->pto + b * 40;
    uint64_t first = rd(e, 8), cnt = rd(e + 8, 8);
    if (first + cnt > nc) return set_err("partition " + std::to_string(b) + " chunk range out of bounds");
    for (uint64_t c = first; c < first + cnt; ++c) {
      if (r->c_len[c] == 0 || r->c_off[c] + r->c_len[c] > n)
        return set_err("partition " + std::to_string(b) + " chunk out of bounds");
      if (r->c_codec[c] & ~7u) return set_err("partition " + std::to_string(b) + " chunk uses unsupported codec mask");
    }
    r->p_first.push_back(first);
    r->p_count.push_back(cnt);
  }
  return reader_decode(r);
}

}  // namespace

extern "C" {

kite_reader* kite_reader_open(const char* path) {
  int fd = open(path, O_RDONLY);
  if (fd < 0) {
    set_err(std::string("failed to open ") + path + ": " + strerror(errno));
    return nullptr;
  }
  struct stat st;
  fstat(fd, &st);
  auto* r = new kite_reader();
  r->len = (size_t)st.st_size;
  if (r->len) {
    r->map = mmap(nullptr, r->len, PROT_READ, MAP_PRIVATE, fd, 0);
    if (r->map == MAP_FAILED) {
      close(fd);
      set_err("mmap failed");
      delete r;
      return nullptr;
    }
    r->data = static_cast<const uint8_t*>(r->map);
  }
  close(fd);
  if (reader_parse(r)) {
    kite_reader_close(r);
    return nullptr;
  }
  return r;
}

kite_reader* kite_reader_open_image(const uint8_t* data, size_t len) {
  auto* r = new kite_reader();
  r->own.assign(data, data + len);
  r->data = r->own.data();
  r->len = len;
  if (reader_parse(r)) {
    delete r;
    return nullptr;
  }
  return r;
}

void kite_reader_close(kite_reader* r) {
  if (!r) return;
  if (r->map && r->map != MAP_FAILED) munmap(r->map, r->len);
  delete r;
}

int kite_reader_header(const kite_reader* r, kite_header_info* h, uint64_t* tc, uint64_t* tr) {
  if (!r) return -1;
  if (h) *h = r->h;
  if (tc) *tc = r->total_chunks;
  if (tr) *tr = r->total_rows;
  return 0;
}

int kite_reader_merge_input(const kite_reader* r, kite_gpu_merge_input* mi) {
  if (!r || !mi) return -1;
  mi->base = r->d_base;
  mi->base_len = r->d_len;
  mi->chunk_offset = r->d_off.data();
  mi->chunk_len = r->d_size.data();
  mi->chunk_rows = r->c_rows.data();
  mi->chunk_codec = r->d_codec.data();
  mi->part_first = r->p_first.data();
  mi->part_count = r->p_count.data();
  mi->has_min = r->h.has_min;
  mi->has_max = r->h.has_max;
  mi->min_count = r->h.min_count;
  mi->max_count = r->h.max_count;
  return 0;
}

int kite_count_passes_filter(uint64_t count, int has_min, uint32_t mn, int has_max, uint32_t mx) {
  if (has_min && count < mn) return 0;
  if (has_max && count > mx) return 0;
  return 1;
}

// Segment streams of one partition merged by key with saturating u32 sums
// (LoserTreeMerger src/dump/loser_tree.rs:141-175), header filter on the
// summed count, 2-bit -> ACGT MSB first (decode_kmer_any src/dump/decoder.rs:27-50).
int64_t kite_dump_partition(const kite_reader* r, uint32_t p, char** buf, size_t* cap, size_t* len) {
  if (!r || p >= r->h.partitions) return set_err("bad partition");
  const bool wide = r->h.key_width == 128;
  if (r->h.key_width != 64 && r->h.key_width != 128) return set_err("unsupported key width for dump");
  struct Stream {
    const uint8_t* d;
    size_t n, pos;
    uint64_t left;
    u128 prev;
    bool dvle;
    size_t es;
    bool next(u128& k, uint32_t& c) {
      if (!left) return false;
      left--;
      if (!dvle) {
        if (pos + es > n) return false;
        k = es == 12 ? (u128)rd(d + pos, 8) : ((u128)rd(d + pos + 8, 8) << 64) | rd(d + pos, 8);
        c = (uint32_t)rd(d + pos + es - 4, 4);
        pos += es;
        return true;
      }
      if (pos == 0) {
        const size_t kb = es - 4;
        if (n < es) return false;
        k = kb == 8 ? (u128)rd(d, 8) : ((u128)rd(d + 8, 8) << 64) | rd(d, 8);
        c = (uint32_t)rd(d + kb, 4);
        pos = es;
        prev = k;
        return true;
      }
      u128 delta = 0;
      unsigned sh = 0;
      for (size_t i = 0; pos < n && i < (es == 12 ? 10u : 19u); ++i) {
        uint8_t b = d[pos++];
        delta |= (u128)(b & 0x7f) << sh;
        sh += 7;
        if (!(b & 0x80)) break;
      }
      uint64_t cc = 0;
      sh = 0;
      for (size_t i = 0; pos < n && i < 10; ++i) {
        uint8_t b = d[pos++];
        cc |= (uint64_t)(b & 0x7f) << sh;
        sh += 7;
        if (!(b & 0x80)) break;
      }
      k = prev + delta;
      prev = k;
      c = (uint32_t)cc;
      return true;
    }
  };
  std::vector<Stream> ss;
  for (uint64_t c = r->p_first[p]; c < r->p_first[p] + r->p_count[p]; ++c) {
    ss.push_back(Stream{r->d_base + r->d_off[c], (size_t)r->d_size[c], 0, r->c_rows[c], 0,
                        (r->d_codec[c] & 2u) != 0, (size_t)(wide ? 20 : 12)});
  }
  struct Head {
    u128 k;
    uint32_t c;
    size_t s;
  };
  auto cmp = [](const Head& a, const Head& b) { return a.k != b.k ? a.k > b.k : a.s > b.s; };
  std::priority_queue<Head, std::vector<Head>, decltype(cmp)> pq(cmp);
  for (size_t i = 0; i < ss.size(); ++i) {
    Head h{0, 0, i};
    if (ss[i].next(h.k, h.c)) pq.push(h);
  }
  const unsigned k = (unsigned)r->h.k;
  static const char dna[4] = {'A', 'C', 'G', 'T'};
  size_t start = *len;
  while (!pq.empty()) {
    const u128 key = pq.top().k;
    uint32_t tot = 0;
    while (!pq.empty() && pq.top().k == key) {
      Head h = pq.top();
      pq.pop();
      tot = (tot > 0xffffffffu - h.c) ? 0xffffffffu : tot + h.c;
      if (ss[h.s].next(h.k, h.c)) pq.push(h);
    }
    if (!kite_count_passes_filter(tot, r->h.has_min, r->h.min_count, r->h.has_max, r->h.max_count)) continue;
    if (*len + k + 16 > *cap) {
      size_t nc = std::max<size_t>(*cap * 2, *len + k + (1 << 20));
      char* nb = static_cast<char*>(realloc(*buf, nc));
      if (!nb) return set_err("out of memory");
      *buf = nb;
      *cap = nc;
    }
    char* o = *buf + *len;
    for (unsigned i = 0; i < k; ++i) o[i] = dna[(unsigned)(key >> (2 * (k - 1 - i))) & 3];
    o[k] = '\t';
    int nn = snprintf(o + k + 1, 12, "%u", tot);
    o[k + 1 + nn] = '\n';
    *len += k + 2 + nn;
  }
  return (int64_t)(*len - start);
}

// ============================================================================
// zstd "if smaller" for count's balanced / compact modes
// (CountWorker::flush_bucket src/count/worker.rs:340-374, heuristics :452-501)
// ============================================================================
namespace {

size_t min_compression_input_bytes(int k, bool used_dvle, size_t entry_size) {
  if (entry_size == 12 && used_dvle && k <= 31) return 16 * 1024;
  if (entry_size == 20 && used_dvle) return 32 * 1024;
  if (entry_size == 36) return 64 * 1024;
  return 32 * 1024;
}

size_t min_compression_savings_bytes(size_t payload, size_t logical, bool used_dvle, size_t entry_size) {
  const size_t ratio_bias = (logical > payload ? logical - payload : 0) / 32;
  const size_t floor = (entry_size == 12 && used_dvle) ? 8 * 1024 : (entry_size == 20 && used_dvle) ? 16 * 1024
                                                                                                     : 32 * 1024;
  const size_t a = std::max(floor, payload / 100), b = std::min<size_t>(ratio_bias, 24 * 1024);
  return a > b ? a - b : 0;
}

int compression_level_for(int base, int k, size_t payload, size_t logical, bool used_dvle, size_t entry_size) {
  if (base <= 0) return 0;
  int level = base;
  if (used_dvle && entry_size == 12 && k <= 31 && payload >= 1024 * 1024) level += 1;
  if (logical >= payload * 2 && payload >= 4 * 1024 * 1024) level += 1;
  return std::min(level, 6);
}

}  // namespace

extern "C" {

int kite_zstd_available(void) { return zstd().ok ? 1 : 0; }

size_t kite_zstd_bound(size_t len) { return zstd().ok ? zstd().bound(len) : 0; }

int64_t kite_zstd_chunk(int k, int base_level, const kite_chunk_meta* meta, const uint8_t* payload, size_t len,
                        uint8_t* out, size_t cap) {
  if (!meta || (len && !payload)) return set_err("bad arguments");
  const bool used_dvle = (meta->codec & KITE_CODEC_DVLE) != 0;
  const size_t entry = k <= 31 ? 12 : k <= 64 ? 20 : 36;
  const size_t logical = (size_t)meta->row_count * entry;
  const int level = compression_level_for(base_level, k, len, logical, used_dvle, entry);
  if (level <= 0 || len < min_compression_input_bytes(k, used_dvle, entry)) return 0;
  const Zstd& z = zstd();
  if (!z.ok) return set_err("zstd compression needs libzstd.so.1, which is not available");
  if (cap < z.bound(len)) return set_err("zstd output buffer too small");
  const size_t got = z.compress(out, cap, payload, len, level);
  if (z.is_error(got)) return 0;  // the reference keeps the payload when compression fails
  const size_t min_savings = min_compression_savings_bytes(len, logical, used_dvle, entry);
  return got + min_savings < len ? (int64_t)got : 0;
}

}  // extern "C"

// ============================================================================
// Memory spec, planner
// ============================================================================
int64_t kite_parse_memory_spec(const char* spec) {
  const std::string s = spec ? spec : "";
  auto bad = [&](const std::string& why) { return set_err("invalid memory size '" + s + "': " + why); };
  bool digits = !s.empty() && std::all_of(s.begin(), s.end(), [](char c) { return c >= '0' && c <= '9'; });
  if (digits) {
    errno = 0;
    unsigned long long v = strtoull(s.c_str(), nullptr, 10);
    if (errno) return bad("expected formats like 512M, 64G, 1T, or raw bytes");
    if (v == 0) return bad("value must be greater than zero");
    return (int64_t)v;
  }
  if (s.size() < 2) return bad("expected formats like 512M, 64G, 1T, or raw bytes");
  const char suf = s.back();
  uint64_t mul = suf == 'M' ? MiB : suf == 'G' ? GiB : suf == 'T' ? 1024 * GiB : 0;
  if (!mul) return bad("suffix must be M, G, or T");
  const std::string num = s.substr(0, s.size() - 1);
  if (num.empty() || !std::all_of(num.begin(), num.end(), [](char c) { return c >= '0' && c <= '9'; }))
    return bad("numeric part must be a positive integer");
  unsigned long long v = strtoull(num.c_str(), nullptr, 10);
  if (v == 0) return bad("value must be greater than zero");
  if (v > (unsigned long long)INT64_MAX / mul) return set_err("memory size '" + s + "' exceeds supported range");
  return (int64_t)(v * mul);
}

// resolve_memory_limit_bytes src/runtime.rs:56-71: explicit spec, else 2/3 of
// MemAvailable, else physical memory minus headroom.
int64_t kite_resolve_memory_limit(const char* spec) {
  if (spec && *spec) return kite_parse_memory_spec(spec);
  FILE* f = fopen("/proc/meminfo", "r");
  if (f) {
    char line[256];
    while (fgets(line, sizeof line, f)) {
      unsigned long long kib;
      if (sscanf(line, "MemAvailable: %llu", &kib) == 1) {
        fclose(f);
        uint64_t v = (uint64_t)kib * 1024 * 2 / 3;
        if (v) return (int64_t)v;
        f = nullptr;
        break;
      }
    }
    if (f) fclose(f);
  }
  long pages = sysconf(_SC_PHYS_PAGES), ps = sysconf(_SC_PAGESIZE);
  if (pages <= 0 || ps <= 0) return set_err("sysconf(_SC_PHYS_PAGES/_SC_PAGESIZE) failed");
  uint64_t total = (uint64_t)pages * (uint64_t)ps;
  uint64_t head = std::min(std::max(total / 100, 512 * MiB), 2 * GiB);
  return (int64_t)(total - head);
}

int kite_derive_plan(uint64_t input_bytes, double avg_read_len, int comp, int k, uint64_t req_partitions,
                     uint64_t total_threads, uint64_t mem, int64_t buffer_mb, uint64_t chunk_kmers, kite_plan* out) {
  const bool u64keys = k <= 31;
  const uint64_t E = u64keys ? 1 : 2;
  // target_partition_bytes_for src/count/mod.rs:961-974
  const uint64_t base_mb = u64keys ? 640 : (k <= 64 ? 448 : 320);
  uint64_t tmb;
  if (u64keys && k >= 22) tmb = 192;
  else if (k <= 21) tmb = base_mb + 64;
  else if (k >= 52) tmb = base_mb - 64;
  else tmb = base_mb;
  const uint64_t target = tmb * MiB;
  // target_worker_budget_bytes :883-890
  uint64_t min_wb = u64keys ? 1250 * MiB : (k <= 64 ? 2 * GiB : 3 * GiB);
  min_wb = std::min(min_wb, std::max(mem / 2, 512 * MiB));
  uint64_t decomp = 1;
  if (comp == KITE_INPUT_BGZF) {
    uint64_t maxd = std::max<uint64_t>(total_threads / 2, 1);
    uint64_t div = k <= 31 ? 4 : k <= 51 ? 5 : k <= 75 ? 6 : 8;
    decomp = std::min(std::max<uint64_t>(total_threads / div, 1), maxd);
  }
  const uint64_t mmap_res = comp == KITE_INPUT_BGZF ? input_bytes : 0;
  uint64_t untracked = mem / 6 + (total_threads + 3) * 8 * MiB + decomp * 32 * MiB;
  untracked = std::min(std::max(untracked, 2 * GiB), 12 * GiB);
  untracked = std::min(untracked, mem / 3) + mmap_res;
  uint64_t workers = total_threads > decomp + 1 ? total_threads - decomp - 1 : 0;
  workers = std::max<uint64_t>(workers, 1);
  const bool auto_p = req_partitions == 0;
  uint64_t P = req_partitions;
  if (auto_p) {
    // derive_partition_count :998-1016 then memory_thread_capped_partitions :923-942
    double expansion = std::min(std::max(avg_read_len / 10.0, 4.0), 24.0);
    uint64_t est = (uint64_t)((double)input_bytes * expansion * (double)E);
    uint64_t raw = std::max<uint64_t>((est + target - 1) / target, 1);
    uint64_t rp = 1;
    while (rp < raw) rp <<= 1;
    uint64_t derived = std::min<uint64_t>(std::max<uint64_t>(rp, 256), 2048);
    uint64_t plan_mb = std::max<int64_t>(buffer_mb >= 0 ? buffer_mb : 8, 1);
    uint64_t per = plan_mb * MiB + workers * 5 * 1024;
    uint64_t capped = std::max<uint64_t>((mem / 4) / std::max<uint64_t>(per, 1), 256);
    uint64_t fp = 1;
    while ((fp << 1) <= capped) fp <<= 1;
    P = std::min<uint64_t>(std::max<uint64_t>(std::min(derived, fp), 256), 2048);
  }
  std::vector<uint64_t> cands;
  if (buffer_mb >= 0) {
    uint64_t req = std::max<int64_t>(buffer_mb, 1);
    for (uint64_t v : {req, (uint64_t)16, (uint64_t)8, (uint64_t)4, (uint64_t)2, (uint64_t)1})
      if (v <= req) cands.push_back(v);
  } else {
    cands = {16, 8, 4, 2};
  }
  std::sort(cands.rbegin(), cands.rend());
  cands.erase(std::unique(cands.begin(), cands.end()), cands.end());
  size_t si = 0;
  for (;;) {
    const uint64_t staging = cands[si] * MiB;
    uint64_t chunk = chunk_kmers ? std::min(std::max(chunk_kmers * 2, 8 * MiB), 64 * MiB)
                                 : std::min(std::max(mem / (workers * 96), 8 * MiB), 64 * MiB);
    uint64_t qbase = comp == KITE_INPUT_PLAIN ? 8 : std::min<uint64_t>(std::max<uint64_t>(decomp * 2, 8), 64);
    uint64_t queue = std::min(qbase, std::min<uint64_t>(std::max<uint64_t>(mem / GiB, 8), 64));
    uint64_t dbud = chunk * queue;
    uint64_t reserved = dbud + P * staging + workers * 48 * MiB + untracked;
    uint64_t tracked = mem > untracked + dbud ? mem - untracked - dbud : 0;
    uint64_t wb = (mem > reserved ? mem - reserved : 0) / workers;
    uint64_t lf = std::max(wb * 45 / 100, std::max(chunk * 2, staging * 4));
    if (reserved < mem && tracked > 0 && wb >= min_wb) {
      out->partitions = P;
      out->chunk_size_bytes = chunk;
      out->staging_bytes = staging;
      out->worker_threads = workers;
      out->local_flush_bytes = lf;
      out->decomp_threads = decomp;
      out->writer_lanes = kite_suggest_write_lanes(workers);
      out->queue_depth = queue;
      out->avg_read_len = avg_read_len;
      return 0;
    }
    if (si + 1 < cands.size()) {
      si++;
      continue;
    }
    if (workers > 1) {
      workers--;
      si = 0;
      continue;
    }
    if (auto_p && P > 256) {
      P /= 2;
      si = 0;
      continue;
    }
    return set_err("unable to derive count heuristic plan within memory budget " + std::to_string(mem) + " bytes");
  }
}

// ============================================================================
// Input: sniffing and chunked readers
// ============================================================================
int kite_detect_compression(const char* path) {
  FILE* f = fopen(path, "rb");
  if (!f) return set_err(std::string("failed to inspect input FASTQ compression.\nInput: ") + path);
  uint8_t h[18];
  size_t n = fread(h, 1, 18, f);
  fclose(f);
  if (n < 2 || h[0] != 0x1f || h[1] != 0x8b) return KITE_INPUT_PLAIN;
  if (n >= 18 && (h[3] & 0x04)) {
    size_t xlen = (size_t)h[10] | ((size_t)h[11] << 8);
    if (xlen >= 6 && h[12] == 0x42 && h[13] == 0x43) return KITE_INPUT_BGZF;
  }
  return KITE_INPUT_GZIP;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// BGZF (decompress_bgzf_parallel src/count/bgzf.rs:149-258): block headers
// scanned (scan_bgzf_blocks :54-85), batches of 8192 blocks inflated on a
// thread pool, output appended block by block in file order and cut by
// find_fastq_split_near (:124-135) whenever at least a chunk is held.
// ---------------------------------------------------------------------------
namespace {

constexpr size_t kBgzfBatch = 8192;

// Byte after the last 4k-th newline of d[0, n) (0 if none): find_fastq_split_4lines.
size_t split_4lines(const uint8_t* d, size_t n) {
  size_t nl = 0, last = 0;
  const uint8_t* p = d;
  const uint8_t* e = d + n;
  while (p < e) {
    const void* q = memchr(p, '\n', (size_t)(e - p));
    if (!q) break;
    p = static_cast<const uint8_t*>(q) + 1;
    if ((++nl & 3) == 0) last = (size_t)(p - d);
  }
  return last;
}

size_t split_near(const uint8_t* d, size_t n, size_t target) {
  const size_t b = split_4lines(d, std::min(target + 8192, n));
  return b > 0 ? b : split_4lines(d, n);
}

// Block (offset, size) pairs; false with the reference's message on data
// that is not a BGZF block.  A truncated final block is skipped.
bool scan_bgzf(const uint8_t* d, size_t n, std::vector<std::pair<size_t, size_t>>& blocks, std::string& err) {
  size_t pos = 0;
  while (pos + 18 <= n) {
    const uint8_t* h = d + pos;
    if (!(h[0] == 0x1f && h[1] == 0x8b && (h[3] & 0x04) && h[12] == 0x42 && h[13] == 0x43 && h[14] == 0x02 &&
          h[15] == 0x00)) {
      err = "Non-BGZF data at offset " + std::to_string(pos) + " (expected gzip+BGZF header)";
      return false;
    }
    const size_t bsize = ((size_t)h[16] | ((size_t)h[17] << 8)) + 1;
    if (pos + bsize > n) break;
    blocks.push_back({pos, bsize});
    pos += bsize;
  }
  return true;
}

// One gzip member into dst[0, cap): the bytes written, or ~0 when the member
// does not end exactly at cap bytes of output (a decode error, or an output
// size other than cap).
size_t inflate_member_into(const uint8_t* raw, size_t n, uint8_t* dst, size_t cap) {
#if KITE_HAVE_ZLIB
  z_stream zs{};
  if (inflateInit2(&zs, 15 + 16) != Z_OK) return ~(size_t)0;
  zs.next_in = const_cast<uint8_t*>(raw);
  zs.avail_in = (uInt)n;
  zs.next_out = dst;
  zs.avail_out = (uInt)cap;
  const int r = inflate(&zs, Z_FINISH);
  const size_t got = cap - zs.avail_out;
  inflateEnd(&zs);
  return r == Z_STREAM_END && got == cap ? got : ~(size_t)0;
#else
  (void)raw;
  (void)n;
  (void)dst;
  (void)cap;
  return ~(size_t)0;
#endif
}

// One gzip member into out; on a decode error the bytes decoded so far stay.
bool inflate_member(const uint8_t* raw, size_t n, std::vector<uint8_t>& out) {
  out.clear();
#if KITE_HAVE_ZLIB
  z_stream zs{};
  if (inflateInit2(&zs, 15 + 16) != Z_OK) return false;
  zs.next_in = const_cast<uint8_t*>(raw);
  zs.avail_in = (uInt)n;
  int r = Z_OK;
  while (r == Z_OK) {
    const size_t have = out.size();
    out.resize(have + 65536);
    zs.next_out = out.data() + have;
    zs.avail_out = 65536;
    r = inflate(&zs, Z_NO_FLUSH);
    out.resize(have + (65536 - zs.avail_out));
    if (r == Z_BUF_ERROR && zs.avail_in == 0) break;
  }
  inflateEnd(&zs);
  return r == Z_STREAM_END;
#else
  (void)raw;
  (void)n;
  return false;
#endif
}

// Mapped (or read) bytes of a whole file.
struct FileBytes {
  const uint8_t* p = nullptr;
  size_t n = 0;
  void* map = nullptr;
  std::vector<uint8_t> copy;
  bool open(const char* path) {
    const int fd = ::open(path, O_RDONLY);
    if (fd < 0) return false;
    struct stat st {};
    if (fstat(fd, &st) != 0) {
      ::close(fd);
      return false;
    }
    n = (size_t)st.st_size;
    if (n) {
      map = mmap(nullptr, n, PROT_READ, MAP_PRIVATE, fd, 0);
      if (map == MAP_FAILED) {
        map = nullptr;
        copy.resize(n);
        size_t got = 0;
        while (got < n) {
          const ssize_t r = ::read(fd, copy.data() + got, n - got);
          if (r <= 0) break;
          got += (size_t)r;
        }
        copy.resize(got);
        n = got;
        p = copy.data();
      } else {
        p = static_cast<const uint8_t*>(map);
      }
    }
    ::close(fd);
    return true;
  }
  void close() {
    if (map) munmap(map, n);
    map = nullptr;
    p = nullptr;
    n = 0;
    std::vector<uint8_t>().swap(copy);
  }
  ~FileBytes() { close(); }
};

// A gzip member header at i: magic, deflate, no reserved flag bits, an
// extra-flags byte deflate writes and a known OS byte.
bool gz_header_at(const uint8_t* p, size_t n, size_t i) {
  if (i + 10 > n || p[i] != 0x1f || p[i + 1] != 0x8b || p[i + 2] != 8 || (p[i + 3] & 0xe0)) return false;
  const uint8_t xfl = p[i + 8], os = p[i + 9];
  return (xfl == 0 || xfl == 2 || xfl == 4) && (os <= 13 || os == 255);
}

// Offsets of every position that looks like a gzip member header, ascending
// (scanned on several threads).
std::vector<size_t> gz_member_candidates(const uint8_t* p, size_t n) {
  const unsigned T = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  std::vector<std::vector<size_t>> part(T);
  std::vector<std::thread> th;
  for (unsigned t = 0; t < T; ++t)
    th.emplace_back([&, t]() {
      const size_t a = n * t / T, b = n * (t + 1) / T;
      for (size_t i = a; i < b;) {
        const void* q = memchr(p + i, 0x1f, b - i);
        if (!q) break;
        i = (size_t)(static_cast<const uint8_t*>(q) - p);
        if (gz_header_at(p, n, i)) part[t].push_back(i);
        ++i;
      }
    });
  for (auto& x : th) x.join();
  std::vector<size_t> all;
  for (auto& v : part) all.insert(all.end(), v.begin(), v.end());
  return all;
}

#if KITE_HAVE_ZLIB
// One complete gzip member from p[0, n) into out (at most cap bytes): true
// when it ends (CRC and size checked); *used = its compressed length.
bool inflate_whole_member(const uint8_t* p, size_t n, size_t hint, size_t cap, std::vector<uint8_t>& out,
                          size_t* used) {
  out.clear();
  z_stream zs{};
  if (inflateInit2(&zs, 15 + 16) != Z_OK) return false;
  out.resize(std::min(std::max<size_t>(hint, 1 << 20), cap));
  size_t fed = 0, have = 0;
  int r = Z_OK;
  while (r == Z_OK) {
    if (zs.avail_in == 0 && fed < n) {
      const size_t k = std::min<size_t>(n - fed, 1u << 30);
      zs.next_in = const_cast<uint8_t*>(p + fed);
      zs.avail_in = (uInt)k;
      fed += k;
    }
    if (have == out.size()) {
      if (out.size() >= cap) break;
      out.resize(std::min(cap, out.size() * 2));
    }
    const size_t room = std::min<size_t>(out.size() - have, 1u << 30);
    zs.next_out = out.data() + have;
    zs.avail_out = (uInt)room;
    r = inflate(&zs, Z_NO_FLUSH);
    have += room - zs.avail_out;
    if (r == Z_BUF_ERROR && zs.avail_in == 0 && fed >= n) break;
    if (r == Z_BUF_ERROR && zs.avail_out != 0) break;
    if (r == Z_BUF_ERROR) r = Z_OK;  // output room only
  }
  *used = (size_t)zs.total_in;
  inflateEnd(&zs);
  out.resize(have);
  return r == Z_STREAM_END;
}
#endif

}  // namespace

struct kite_input {
  FILE* f = nullptr;
#if KITE_HAVE_ZLIB
  gzFile gz = nullptr;
#endif
  uint64_t chunk = 0;
  std::vector<uint8_t> carry;
  bool eof = false;
  // BGZF: decompressed bytes of the current batch (after the uncut rest of
  // the previous one) in asm_buf, cut into chunks (offset, length)
  bool bgzf = false;
  FileBytes file;
  std::vector<std::pair<size_t, size_t>> blocks;
  size_t next_block = 0;
  unsigned threads = 1;
  std::vector<uint8_t> asm_buf;
  size_t asm_len = 0;   // valid bytes in asm_buf
  size_t asm_pos = 0;   // start of the uncut bytes
  std::deque<std::pair<size_t, size_t>> ready;
  std::string bgzf_err;
  // Batches are pipelined: while the chunks of one batch are handed out, the
  // next batch inflates on the pool into the other buffer (nxt_buf), after
  // room for the bytes the current batch leaves uncut.
  std::vector<uint8_t> nxt_buf;
  std::vector<size_t> nxt_off;  // block output ends in nxt_buf, nxt_off[0] = the room left in front
  size_t nxt_nb = 0;
  std::thread nxt_thread;
  bool nxt_pending = false;

  // Inflates blocks [first, first + nb) into buf after `room` bytes; off gets
  // every block's output end.  Each block inflates straight to its place (its
  // gzip ISIZE field gives its output size); a batch where a block does not
  // decode to exactly that size is assembled again block by block.
  void inflate_batch(size_t first, size_t nb, size_t room, std::vector<uint8_t>& buf, std::vector<size_t>& off) {
    off.assign(nb + 1, 0);
    off[0] = room;
    for (size_t i = 0; i < nb; ++i) {
      const auto& b = blocks[first + i];
      const uint8_t* t = file.p + b.first + b.second - 4;
      size_t isize = (size_t)t[0] | ((size_t)t[1] << 8) | ((size_t)t[2] << 16) | ((size_t)t[3] << 24);
      if (isize > 65536) isize = 65536;  // not a BGZF block size: the check below catches it
      off[i + 1] = off[i] + isize;
    }
    if (buf.size() < off[nb]) buf.resize(off[nb]);
    std::atomic<size_t> idx{0};
    std::atomic<bool> exact{true};
    auto work = [&]() {
      for (size_t i; (i = idx.fetch_add(1)) < nb;) {
        const auto& b = blocks[first + i];
        const size_t want = off[i + 1] - off[i];
        if (inflate_member_into(file.p + b.first, b.second, buf.data() + off[i], want) != want)
          exact.store(false);
      }
    };
    std::vector<std::thread> pool;
    try {
      for (unsigned t = 1; t < threads; ++t) pool.emplace_back(work);
    } catch (...) {
      // no more threads to be had: the ones running and this one finish the batch
    }
    work();
    for (auto& t : pool) t.join();
    if (!exact.load()) {
      // block by block: each block's actual output, partial on a decode error
      std::vector<uint8_t> o;
      size_t len = room;
      for (size_t i = 0; i < nb; ++i) {
        const auto& b = blocks[first + i];
        inflate_member(file.p + b.first, b.second, o);
        if (buf.size() < len + o.size()) buf.resize(len + o.size());
        if (!o.empty()) memcpy(buf.data() + len, o.data(), o.size());
        len += o.size();
        off[i + 1] = len;
      }
    }
  }
  // Starts the inflate of the batch after next_block, with `room` bytes left
  // in front of it for the current batch's uncut rest.
  void start_next(size_t room) {
    nxt_nb = std::min(kBgzfBatch, blocks.size() - next_block);
    if (nxt_nb == 0) return;
    const size_t first = next_block;
    nxt_pending = true;
    nxt_thread = std::thread([this, first, room]() { inflate_batch(first, nxt_nb, room, nxt_buf, nxt_off); });
  }
  void join_next() {
    if (nxt_pending) {
      nxt_thread.join();
      nxt_pending = false;
    }
  }
  // Called when every ready chunk has been handed out: takes the next batch
  // (inflated meanwhile), puts the uncut rest in front of it and cuts what it
  // can into ready chunks, as the reference does after every appended block;
  // after the last block the uncut rest is a chunk.
  void bgzf_fill() {
    const size_t rest = asm_len - asm_pos;
    if (!nxt_pending) start_next(rest);
    if (!nxt_pending) {
      if (rest) ready.push_back({asm_pos, rest});
      asm_pos = asm_len;
      eof = true;
      return;
    }
    join_next();
    // the batch was inflated after room for exactly this rest
    if (rest) memcpy(nxt_buf.data(), asm_buf.data() + asm_pos, rest);
    asm_buf.swap(nxt_buf);
    const size_t nb = nxt_nb;
    const std::vector<size_t> off = nxt_off;
    next_block += nb;
    asm_pos = 0;
    for (size_t i = 0; i < nb; ++i) {
      const size_t end = off[i + 1];
      if (end == off[i]) continue;
      while (end - asm_pos >= chunk) {
        const size_t split = split_near(asm_buf.data() + asm_pos, end - asm_pos, chunk);
        if (split == 0) break;
        ready.push_back({asm_pos, split});
        asm_pos += split;
      }
    }
    asm_len = off[nb];
    // the following batch inflates while these chunks are handed out
    start_next(asm_len - asm_pos);
  }
  ~kite_input() {
    join_next();
    gz_stop();
  }

  // Multi-member gzip: the members, chained from the file's start (each one
  // starts where the previous one's compressed bytes end), inflate on
  // `threads` threads up to that many ahead and are handed out in order.
  // Anything else (a member that does not decode, bytes after the last
  // member, one thread) goes to the serial reader, opened from the file's
  // start and skipping the bytes already handed out, so that the byte stream
  // and its errors are exactly the serial reader's.
  static constexpr size_t kGzMemberCap = 256u << 20;
  struct GzTask {
    std::thread th;
    bool ok = false;
    size_t used = 0;
    std::vector<uint8_t> out;
  };
  bool gzpar = false;
  std::string gz_path;
  std::vector<size_t> gz_cands;  // offsets that look like member headers
  size_t gz_next = 0;            // compressed offset of the next member of the chain
  size_t gz_launched = 0;        // candidates [0, gz_launched) have had a task
  uint64_t gz_delivered = 0;
  std::vector<uint8_t> gz_cur;
  size_t gz_cur_off = 0;
  std::deque<std::pair<size_t, std::unique_ptr<GzTask>>> gz_tasks;  // (candidate index, task), in order

  void gz_stop() {
    for (auto& t : gz_tasks)
      if (t.second->th.joinable()) t.second->th.join();
    gz_tasks.clear();
  }
  void gz_launch(size_t j) {
    const size_t c = gz_cands[j];
    // the member's output size, if the next candidate starts the next member
    const size_t e = j + 1 < gz_cands.size() ? gz_cands[j + 1] : file.n;
    const uint8_t* q = file.p + e - 4;
    const size_t hint = e >= c + 18 ? ((size_t)q[0] | ((size_t)q[1] << 8) | ((size_t)q[2] << 16) | ((size_t)q[3] << 24)) : 0;
    auto t = std::make_unique<GzTask>();
    GzTask* tp = t.get();
    tp->th = std::thread([this, c, hint, tp]() {
#if KITE_HAVE_ZLIB
      tp->ok = inflate_whole_member(file.p + c, file.n - c, hint, kGzMemberCap, tp->out, &tp->used);
#endif
    });
    gz_tasks.emplace_back(j, std::move(t));
  }
  // To the serial reader: from the file's start, the bytes already handed out skipped.
  void gz_fallback() {
    gzpar = false;
    gz_stop();
    std::vector<uint8_t>().swap(gz_cur);
    gz_cur_off = 0;
#if KITE_HAVE_ZLIB
    gz = gzopen(gz_path.c_str(), "rb");
    if (!gz) {
      g_err = "decompress_error: failed to reopen the input";
      return;
    }
    gzbuffer(gz, 1 << 20);
    std::vector<uint8_t> skip(1 << 20);
    for (uint64_t left = gz_delivered; left;) {
      const int r = gzread(gz, skip.data(), (unsigned)std::min<uint64_t>(left, skip.size()));
      if (r <= 0) break;
      left -= (uint64_t)r;
    }
#endif
  }
  // The next member's bytes into gz_cur; false at the chain's end, or when
  // the serial reader takes over (gzpar then false).
  bool gz_advance() {
    if (gz_next == file.n) return false;
    const auto it = std::lower_bound(gz_cands.begin(), gz_cands.end(), gz_next);
    if (threads <= 1 || it == gz_cands.end() || *it != gz_next) {
      gz_fallback();
      return false;
    }
    const size_t j = (size_t)(it - gz_cands.begin());
    // tasks for the candidates skipped (not member starts) are dropped
    while (!gz_tasks.empty() && gz_tasks.front().first < j) {
      gz_tasks.front().second->th.join();
      gz_tasks.pop_front();
    }
    gz_launched = std::max(gz_launched, j);
    while (gz_launched < gz_cands.size() && gz_launched < j + threads) gz_launch(gz_launched++);
    GzTask& t = *gz_tasks.front().second;
    t.th.join();
    if (!t.ok || t.used == 0) {
      gz_fallback();
      return false;
    }
    gz_cur.swap(t.out);
    gz_cur_off = 0;
    gz_next += t.used;
    gz_tasks.pop_front();
    return true;
  }
  size_t gz_read_par(uint8_t* dst, size_t want) {
    size_t total = 0;
    while (total < want) {
      if (gz_cur_off < gz_cur.size()) {
        const size_t m = std::min(want - total, gz_cur.size() - gz_cur_off);
        memcpy(dst + total, gz_cur.data() + gz_cur_off, m);
        gz_cur_off += m;
        total += m;
        gz_delivered += m;
        continue;
      }
      if (!gz_advance()) break;
    }
    return total;
  }
  size_t read_raw(uint8_t* dst, size_t want) {
    size_t total = 0;
#if KITE_HAVE_ZLIB
    if (gzpar) {
      total = gz_read_par(dst, want);
      if (gzpar || total == want) return total;  // the chain's end, or filled
    }
    if (gz) {
      while (total < want) {
        int r = gzread(gz, dst + total, (unsigned)std::min<size_t>(want - total, 1u << 30));
        if (r <= 0) {
          if (r < 0) {
            int e;
            g_err = std::string("decompress_error: ") + gzerror(gz, &e);
          }
          break;
        }
        total += (size_t)r;
      }
      return total;
    }
#endif
    while (total < want) {
      size_t r = fread(dst + total, 1, want - total, f);
      if (r == 0) break;
      total += r;
    }
    return total;
  }
};

extern "C" {

kite_input* kite_input_open(const char* path, uint64_t chunk_size) {
  int comp = kite_detect_compression(path);
  if (comp < 0) return nullptr;
  auto* in = new kite_input();
  in->chunk = chunk_size;
  if (comp == KITE_INPUT_BGZF) {
#if KITE_HAVE_ZLIB
    if (!in->file.open(path)) {
      set_err(std::string("failed to open input FASTQ.\nInput: ") + path);
      delete in;
      return nullptr;
    }
    in->bgzf = true;
    in->threads = std::max(1u, std::thread::hardware_concurrency() / 2);
    // a scan error is reported by the first read, as the reference's reader
    // thread reports it, and no chunk follows
    if (!scan_bgzf(in->file.p, in->file.n, in->blocks, in->bgzf_err)) in->blocks.clear();
    return in;
#else
    set_err("gzip input needs zlib, which this binary is not compiled with");
    delete in;
    return nullptr;
#endif
  }
  if (comp == KITE_INPUT_PLAIN) {
    in->f = fopen(path, "rb");
    if (!in->f) {
      set_err(std::string("failed to open input FASTQ.\nInput: ") + path);
      delete in;
      return nullptr;
    }
    setvbuf(in->f, nullptr, _IOFBF, 2 << 20);
  } else {
#if KITE_HAVE_ZLIB
    // several members: inflated in parallel (the serial reader stays for
    // one member and for anything the chain does not explain)
    if (in->file.open(path)) {
      in->gz_cands = gz_member_candidates(in->file.p, in->file.n);
      if (in->gz_cands.size() >= 2 && in->gz_cands[0] == 0) {
        in->gzpar = true;
        in->gz_path = path;
        in->threads = std::max(1u, std::thread::hardware_concurrency() / 2);
        return in;
      }
      std::vector<size_t>().swap(in->gz_cands);
    }
    in->file.close();
    in->gz = gzopen(path, "rb");
    if (!in->gz) {
      set_err(std::string("failed to open input FASTQ.\nInput: ") + path);
      delete in;
      return nullptr;
    }
    gzbuffer(in->gz, 1 << 20);
#else
    set_err("gzip input needs zlib, which this binary is not compiled with");
    delete in;
    return nullptr;
#endif
  }
  return in;
}

uint64_t kite_input_max_chunk(const kite_input* in) {
  // BGZF chunks may exceed the target by one block (64 KiB) and the cut window
  return in->chunk + std::max<uint64_t>(in->chunk, 1u << 17);
}

int kite_input_set_threads(kite_input* in, unsigned threads) {
  if (!in) return -1;
  in->threads = std::max(1u, threads);
  return 0;
}

// next_chunk: carry + chunk_size new bytes; on a full read cut after the last
// 4k-th newline and carry the rest (src/count/decompress.rs:36-81).
int64_t kite_input_next(kite_input* in, uint8_t* dst, size_t cap) {
  if (in->bgzf) {
    if (!in->bgzf_err.empty()) {
      fprintf(stderr, "[kite count] bgzf_decompress_error: %s\n", in->bgzf_err.c_str());
      in->bgzf_err.clear();
      in->eof = true;
      return 0;
    }
    while (in->ready.empty() && !in->eof) in->bgzf_fill();
    if (in->ready.empty()) return 0;
    const auto c = in->ready.front();
    if (c.second > cap) return set_err("input buffer too small");
    memcpy(dst, in->asm_buf.data() + c.first, c.second);
    in->ready.pop_front();
    return (int64_t)c.second;
  }
  const size_t c = in->carry.size();
  if (cap < c + in->chunk) return set_err("input buffer too small");
  if (c) memcpy(dst, in->carry.data(), c);
  in->carry.clear();
  const size_t got = in->eof ? 0 : in->read_raw(dst + c, in->chunk);
  if (!g_err.empty() && got < in->chunk && g_err.rfind("decompress_error", 0) == 0) {
    // the reference logs the error and stops reading (src/count/mod.rs:471-474)
    fprintf(stderr, "[kite count] %s\n", g_err.c_str());
    g_err.clear();
  }
  const size_t len = c + got;
  if (len == 0) return 0;
  if (got < in->chunk) {
    in->eof = true;
    return (int64_t)len;
  }
  const size_t last = split_4lines(dst, len);
  if (last == 0 || last >= len) return (int64_t)len;
  in->carry.assign(dst + last, dst + len);
  return (int64_t)last;
}

void kite_input_close(kite_input* in) {
  if (!in) return;
  if (in->f) fclose(in->f);
#if KITE_HAVE_ZLIB
  if (in->gz) gzclose(in->gz);
#endif
  delete in;
}

// sample_input src/count/mod.rs:1018-1079 (plain/gzip): 8 MiB chunks until
// >= 200,000 reads or >= 32 MiB decompressed; mean sequence-line length.
double kite_sample_avg_read_len(const char* path, int comp) {
  uint64_t reads = 0, bases = 0, decomp = 0;
  auto count_seqs = [&](const uint8_t* buf, size_t n) {
    if (n == 0 || buf[0] != '@') return;
    int state = 0;
    size_t seq_start = 0;
    for (size_t i = 0; i < n; ++i) {
      if (buf[i] != '\n') continue;
      if (state == 0) {
        state = 1;
        seq_start = i + 1;
      } else if (state == 1) {
        if (i > seq_start) {
          reads++;
          bases += i - seq_start;
        }
        state = 2;
      } else {
        state = state == 2 ? 3 : 0;
      }
    }
    if (state == 1 && seq_start < n) {
      reads++;
      bases += n - seq_start;
    }
  };
  if (comp == KITE_INPUT_BGZF) {
    // sample_bgzf_input src/count/mod.rs:1081-1123: block by block, complete
    // records only, until 200,000 reads or 32 MiB decompressed
    FileBytes fb;
    if (!fb.open(path)) return 150.0;
    std::vector<std::pair<size_t, size_t>> blocks;
    std::string err;
    if (!scan_bgzf(fb.p, fb.n, blocks, err)) return 150.0;
    std::vector<uint8_t> carry, out;
    for (const auto& b : blocks) {
      if (!inflate_member(fb.p + b.first, b.second, out)) break;
      decomp += out.size();
      carry.insert(carry.end(), out.begin(), out.end());
      const size_t split = split_4lines(carry.data(), carry.size());
      if (split > 0) {
        count_seqs(carry.data(), split);
        carry.erase(carry.begin(), carry.begin() + split);
      }
      if (reads >= 200000 || decomp >= 32 * MiB) break;
    }
    return reads == 0 ? 150.0 : (double)bases / (double)reads;
  }
  kite_input* in = kite_input_open(path, 8 * MiB);
  if (!in) return 150.0;
  std::vector<uint8_t> buf(16 * MiB + 64);
  while (reads < 200000 && decomp < 32 * MiB) {
    int64_t n = kite_input_next(in, buf.data(), buf.size());
    if (n <= 0) break;
    decomp += (uint64_t)n;
    count_seqs(buf.data(), (size_t)n);
  }
  kite_input_close(in);
  return reads ? (double)bases / (double)reads : 150.0;
}

// ============================================================================
// Synthetic reads
// ============================================================================
int64_t kite_synth_reads(const uint8_t* genome, uint64_t glen, uint64_t n_reads, uint32_t L, double sub_rate,
                         double n_rate, double rc_frac, uint64_t seed, uint64_t first_index, uint8_t* out,
                         uint64_t cap, int threads) {
  const uint64_t rec = 11 + 1 + L + 1 + 2 + L + 1;
  if (glen < L || n_reads * rec > cap) return set_err("synth: bad sizes");
  const int nt = std::max(1, threads);
  auto work = [&](uint64_t r0, uint64_t r1) {
    for (uint64_t r = r0; r < r1; ++r) {
      // splitmix64 stream per read: deterministic regardless of thread count
      uint64_t st = seed * 0x9E3779B97F4A7C15ull + (first_index + r) * 0xD1B54A32D192ED03ull;
      auto next = [&]() {
        uint64_t z = (st += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
      };
      auto unif = [&]() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); };
      uint8_t* o = out + r * rec;
      const uint64_t idx = first_index + r;
      o[0] = '@';
      o[1] = 'r';
      for (int d = 0; d < 9; ++d) {
        uint64_t p = 1;
        for (int e = 0; e < 8 - d; ++e) p *= 10;
        o[2 + d] = (uint8_t)('0' + (idx / p) % 10);
      }
      o[11] = '\n';
      const uint64_t start = next() % (glen - L + 1);
      const bool minus = unif() < rc_frac;
      uint8_t* s = o + 12;
      static const char dna[4] = {'A', 'C', 'G', 'T'};
      for (uint32_t i = 0; i < L; ++i) {
        uint8_t c = minus ? (uint8_t)(3 - genome[start + L - 1 - i]) : genome[start + i];
        if (sub_rate > 0 && unif() < sub_rate) c = (uint8_t)((c + 1 + next() % 3) & 3);
        s[i] = (uint8_t)dna[c];
        if (n_rate > 0 && unif() < n_rate) s[i] = 'N';
      }
      o[12 + L] = '\n';
      o[13 + L] = '+';
      o[14 + L] = '\n';
      memset(o + 15 + L, 'I', L);
      o[15 + 2 * L] = '\n';
    }
  };
  std::vector<std::thread> th;
  const uint64_t per = (n_reads + nt - 1) / nt;
  for (int t = 0; t < nt; ++t) {
    uint64_t a = t * per, b = std::min<uint64_t>(n_reads, a + per);
    if (a < b) th.emplace_back(work, a, b);
  }
  for (auto& x : th) x.join();
  return (int64_t)(n_reads * rec);
}

// Variable read lengths, uniform in [len_lo, len_hi] (drawn first from each
// read's own stream), records packed back to back; otherwise as
// kite_synth_reads.  Returns the bytes written, or -1.
int64_t kite_synth_reads_var(const uint8_t* genome, uint64_t glen, uint64_t n_reads, uint32_t len_lo, uint32_t len_hi,
                             double sub_rate, double n_rate, double rc_frac, uint64_t seed, uint64_t first_index,
                             uint8_t* out, uint64_t cap, int threads) {
  if (len_lo == 0 || len_hi < len_lo || glen < len_hi) return set_err("synth: bad sizes");
  auto stream = [seed](uint64_t idx) { return seed * 0x9E3779B97F4A7C15ull + idx * 0xD1B54A32D192ED03ull; };
  auto mix = [](uint64_t& st) {
    uint64_t z = (st += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  };
  const uint32_t span = len_hi - len_lo + 1;
  std::vector<uint64_t> off(n_reads + 1, 0);
  for (uint64_t r = 0; r < n_reads; ++r) {
    uint64_t st = stream(first_index + r);
    const uint32_t L = len_lo + (uint32_t)(mix(st) % span);
    off[r + 1] = off[r] + 2ull * L + 16;
  }
  if (off[n_reads] > cap) return set_err("synth: output buffer too small");
  const int nt = std::max(1, threads);
  auto work = [&](uint64_t r0, uint64_t r1) {
    static const char dna[4] = {'A', 'C', 'G', 'T'};
    for (uint64_t r = r0; r < r1; ++r) {
      uint64_t st = stream(first_index + r);
      const uint32_t L = len_lo + (uint32_t)(mix(st) % span);
      auto unif = [&]() { return (double)(mix(st) >> 11) * (1.0 / 9007199254740992.0); };
      uint8_t* o = out + off[r];
      const uint64_t idx = first_index + r;
      o[0] = '@';
      o[1] = 'r';
      for (int d = 0; d < 9; ++d) {
        uint64_t p = 1;
        for (int e = 0; e < 8 - d; ++e) p *= 10;
        o[2 + d] = (uint8_t)('0' + (idx / p) % 10);
      }
      o[11] = '\n';
      const uint64_t start = mix(st) % (glen - L + 1);
      const bool minus = unif() < rc_frac;
      uint8_t* sq = o + 12;
      for (uint32_t i = 0; i < L; ++i) {
        uint8_t c = minus ? (uint8_t)(3 - genome[start + L - 1 - i]) : genome[start + i];
        if (sub_rate > 0 && unif() < sub_rate) c = (uint8_t)((c + 1 + mix(st) % 3) & 3);
        sq[i] = (uint8_t)dna[c];
        if (n_rate > 0 && unif() < n_rate) sq[i] = 'N';
      }
      o[12 + L] = '\n';
      o[13 + L] = '+';
      o[14 + L] = '\n';
      memset(o + 15 + L, 'I', L);
      o[15 + 2 * L] = '\n';
    }
  };
  std::vector<std::thread> th;
  const uint64_t per = (n_reads + nt - 1) / nt;
  for (int t = 0; t < nt; ++t) {
    const uint64_t a = t * per, b = std::min<uint64_t>(n_reads, a + per);
    if (a < b) th.emplace_back(work, a, b);
  }
  for (auto& x : th) x.join();
  return (int64_t)off[n_reads];
}

}  // extern "C"
