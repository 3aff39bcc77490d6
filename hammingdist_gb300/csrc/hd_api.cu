// The C ABI (include/hammingdist_gb300.h): argument checks, error mapping,
// host<->device movement and the orchestration of the device stages.
#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cerrno>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <cstdio>
#include <cstdlib>
#include <limits>
#include <thread>

#include <nvtx3/nvToolsExt.h>

#include "hd_internal.cuh"

using hd::DevBuf;
using hd::Error;
using hd::fail;

namespace hd {

// ------------------------------------------------- large device buffers
namespace {
struct BigBlock {
  void *p;
  size_t size;        // bytes allocated
  int device;
  cudaEvent_t freed;  // recorded on the releasing stream at the release
};
struct BigCache {
  std::mutex mu;
  std::deque<BigBlock> released;             // oldest first
  std::map<void *, std::pair<size_t, int>> live;  // handed out: size, device
  std::map<int, size_t> cached;               // released bytes per device
  std::map<int, size_t> cap;                  // per device
};
BigCache &big_cache() {
  static BigCache *c = new BigCache();  // outlives the buffers that return to it
  return *c;
}
bool capturing(cudaStream_t s) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  return cudaStreamIsCapturing(s, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone;
}
// Frees the released blocks of `device` (all of them, or the oldest until
// its cached bytes are at most `keep`) on stream s after their release
// events. Called with the lock held.
void big_evict(BigCache &c, int device, size_t keep, cudaStream_t s) {
  for (auto it = c.released.begin(); it != c.released.end() && c.cached[device] > keep;) {
    if (it->device != device) {
      ++it;
      continue;
    }
    cudaStreamWaitEvent(s, it->freed, 0);
    cudaFreeAsync(it->p, s);
    cudaEventDestroy(it->freed);
    c.cached[device] -= it->size;
    it = c.released.erase(it);
  }
}
}  // namespace

void *big_alloc(size_t n, cudaStream_t s) {
  int dev = 0;
  HD_CUDA(cudaGetDevice(&dev));
  BigCache &c = big_cache();
  // a stream being captured into a graph allocates graph-owned memory, as before
  const bool cap = capturing(s);
  std::lock_guard<std::mutex> lk(c.mu);
  if (!cap) {
    auto best = c.released.end();
    for (auto it = c.released.begin(); it != c.released.end(); ++it)
      if (it->device == dev && it->size >= n && it->size - n <= n / 8 &&
          (best == c.released.end() || it->size < best->size))
        best = it;
    if (best != c.released.end()) {
      const BigBlock b = *best;
      c.released.erase(best);
      c.cached[dev] -= b.size;
      // the work that used the block before its release comes first
      const cudaError_t e = cudaStreamWaitEvent(s, b.freed, 0);
      cudaEventDestroy(b.freed);
      if (e != cudaSuccess) {
        cudaFreeAsync(b.p, s);
        HD_CUDA(e);
      }
      c.live[b.p] = {b.size, dev};
      return b.p;
    }
    // a request of another size: the released blocks go back to the pool,
    // which can split and reuse their memory. Kept for requests of other
    // sizes (calls on alignments of varying shapes), they made the pool map
    // new memory instead: 64 plain calls took 63.6 ms against 40.0.
    big_evict(c, dev, 0, s);
  }
  void *p = nullptr;
  cudaError_t e = cudaMallocAsync(&p, n, s);
  if (e == cudaErrorMemoryAllocation && !cap) {
    cudaGetLastError();
    big_evict(c, dev, 0, s);  // the released blocks first
    e = cudaMallocAsync(&p, n, s);
  }
  HD_CUDA(e);
  if (!cap) c.live[p] = {n, dev};
  return p;
}

void big_release(void *p, cudaStream_t s) {
  BigCache &c = big_cache();
  const bool cap = capturing(s);
  std::lock_guard<std::mutex> lk(c.mu);
  auto it = c.live.find(p);
  if (it == c.live.end()) {  // graph-owned memory
    cudaFreeAsync(p, s);
    return;
  }
  const size_t size = it->second.first;
  const int dev = it->second.second;
  c.live.erase(it);
  cudaEvent_t ev = nullptr;
  int cur = -1;
  cudaGetDevice(&cur);
  if (cur != dev) cudaSetDevice(dev);
  const bool kept = !cap && cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) == cudaSuccess &&
                    cudaEventRecord(ev, s) == cudaSuccess;
  if (!kept) {
    if (ev) cudaEventDestroy(ev);
    cudaGetLastError();
    cudaFreeAsync(p, s);
  } else {
    c.released.push_back({p, size, dev, ev});
    c.cached[dev] += size;
    auto cp = c.cap.find(dev);
    if (cp == c.cap.end()) {
      // at most 16 GB or 1/8 of the device's memory waits for reuse
      size_t free_b = 0, total_b = 0;
      cudaMemGetInfo(&free_b, &total_b);
      cp = c.cap.emplace(dev, std::min<size_t>(16ull << 30, total_b / 8)).first;
    }
    if (c.cached[dev] > cp->second) big_evict(c, dev, cp->second, s);
  }
  if (cur != dev && cur >= 0) cudaSetDevice(cur);
}

namespace {
cudaEvent_t trace_event(hd_ctx *ctx, size_t k) {
  while (ctx->trace.pool.size() <= k) {
    cudaEvent_t e;
    HD_CUDA(cudaEventCreate(&e));
    ctx->trace.pool.push_back(e);
  }
  return ctx->trace.pool[k];
}
}  // namespace

void upload_table(hd_ctx *ctx, void *d_dst, const void *host, size_t bytes, cudaStream_t s) {
  constexpr int kSlots = 8;
  constexpr size_t kSlotBytes = 1u << 20;
  if (bytes > kSlotBytes) {
    HD_CUDA(cudaMemcpyAsync(d_dst, host, bytes, cudaMemcpyHostToDevice, s));
    return;
  }
  struct Ring {
    uint8_t *mem = nullptr;
    cudaEvent_t ev[kSlots] = {};
    int next = 0;
  };
  static std::mutex mu;
  static std::map<int, Ring> rings;  // per device
  std::lock_guard<std::mutex> lk(mu);
  Ring &r = rings[ctx->device];
  if (!r.mem) {
    HD_CUDA(cudaHostAlloc(reinterpret_cast<void **>(&r.mem), kSlots * kSlotBytes, cudaHostAllocDefault));
    for (int k = 0; k < kSlots; ++k) HD_CUDA(cudaEventCreateWithFlags(&r.ev[k], cudaEventDisableTiming));
  }
  const int k = r.next;
  r.next = (k + 1) % kSlots;
  HD_CUDA(cudaEventSynchronize(r.ev[k]));  // the slot's previous copy has run
  uint8_t *slot = r.mem + (size_t)k * kSlotBytes;
  std::memcpy(slot, host, bytes);
  HD_CUDA(cudaMemcpyAsync(d_dst, slot, bytes, cudaMemcpyHostToDevice, s));
  HD_CUDA(cudaEventRecord(r.ev[k], s));
}

void trace_begin(hd_ctx *ctx, const char *call) {
  if (!ctx->trace.on) return;
  if (ctx->trace.call) nvtxRangePop();  // an earlier call ended by an error
  ctx->trace.call = call;
  ctx->trace.names.assign(1, nullptr);
  ctx->trace.at_names.clear();
  ctx->trace.host.clear();
  ctx->trace.t0 = std::chrono::steady_clock::now();
  HD_CUDA(cudaEventRecord(trace_event(ctx, 0), ctx->stream));
  nvtxRangePushA(call);
}

void trace_mark(hd_ctx *ctx, const char *phase) {
  if (!ctx->trace.on || !ctx->trace.call) return;
  const size_t k = ctx->trace.names.size();
  HD_CUDA(cudaEventRecord(trace_event(ctx, k), ctx->stream));
  ctx->trace.names.push_back(phase);
  nvtxMarkA(phase);
}

void trace_at(hd_ctx *ctx, const std::string &what, cudaStream_t s) {
  if (!ctx->trace.on || !ctx->trace.call) return;
  Trace &t = ctx->trace;
  const size_t k = t.at_names.size();
  while (t.at_pool.size() <= k) {
    cudaEvent_t e;
    HD_CUDA(cudaEventCreate(&e));
    t.at_pool.push_back(e);
  }
  HD_CUDA(cudaEventRecord(t.at_pool[k], s));
  t.at_names.push_back(what);
}

void trace_host(hd_ctx *ctx, const std::string &what) {
  if (!ctx->trace.on || !ctx->trace.call) return;
  ctx->trace.host.emplace_back(
      what, std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() -
                                                      ctx->trace.t0)
                .count());
}

void trace_end(hd_ctx *ctx) {
  if (!ctx->trace.on || !ctx->trace.call) return;
  nvtxRangePop();
  Trace &t = ctx->trace;
  std::string text = std::string(t.call) + ":";
  if (t.names.size() > 1) {
    HD_CUDA(cudaEventSynchronize(t.pool[t.names.size() - 1]));
    float total = 0;
    for (size_t k = 1; k < t.names.size(); ++k) {
      float ms = 0;
      HD_CUDA(cudaEventElapsedTime(&ms, t.pool[k - 1], t.pool[k]));
      total += ms;
      char buf[128];
      std::snprintf(buf, sizeof buf, " %s %.3f ms,", t.names[k], ms);
      text += buf;
    }
    char buf[64];
    std::snprintf(buf, sizeof buf, " stream time %.3f ms", total);
    text += buf;
  }
  for (size_t k = 0; k < t.at_names.size(); ++k) {
    float ms = 0;
    HD_CUDA(cudaEventSynchronize(t.at_pool[k]));
    HD_CUDA(cudaEventElapsedTime(&ms, t.pool[0], t.at_pool[k]));
    char buf[48];
    std::snprintf(buf, sizeof buf, " at %.3f ms", ms);
    text += (k ? ", " : "; ") + t.at_names[k] + buf;
  }
  for (size_t k = 0; k < t.host.size(); ++k) {
    char buf[48];
    std::snprintf(buf, sizeof buf, " at %.3f ms", t.host[k].second);
    text += (k ? ", host: " : "; host: ") + t.host[k].first + buf;
  }
  t.last = text;
  t.call = nullptr;
}

}  // namespace hd

namespace {

const char *kMsgEmpty = "Error: Empty sequence";
const char *kMsgLength = "Error: Sequences do not all have the same length";
const char *kMsgIncludeX = "use_gpu=True cannot be used if include_x=True, please set use_gpu=False";

template <class F>
int guard(hd_ctx *ctx, F &&f) {
  try {
    if (ctx) HD_CUDA(cudaSetDevice(ctx->device));
    f();
    return HD_OK;
  } catch (const Error &e) {
    if (ctx) ctx->err = e.msg;
    return e.code;
  } catch (const std::bad_alloc &) {
    if (ctx) ctx->err = "out of host memory";
    return HD_ERR_OOM;
  } catch (const std::exception &e) {
    if (ctx) ctx->err = e.what();
    return HD_ERR_CUDA;
  }
}

// safe_int_cast (include/hamming/hamming_impl.hh:37-45): above the dtype max
// saturates, otherwise static_cast (negative values wrap).
uint32_t clamp_max(int64_t max_distance, int dtype_bytes) {
  if (dtype_bytes == 4) {
    if (max_distance < 0) fail(HD_ERR_ARG, "max_distance must be >= 0 for 32-bit output");
    return max_distance > 0xffffffffll ? 0xffffffffu : (uint32_t)max_distance;
  }
  const uint32_t tmax = dtype_bytes == 1 ? 0xffu : 0xffffu;
  if (max_distance > (int64_t)tmax) return tmax;
  return (uint32_t)((uint64_t)max_distance & tmax);
}

void check_dtype(int dtype_bytes) {
  if (dtype_bytes != 1 && dtype_bytes != 2 && dtype_bytes != 4)
    fail(HD_ERR_ARG, "dtype_bytes must be 1, 2 or 4");
}

void check_status(hd_ctx *ctx) {
  int st = 0;
  HD_CUDA(cudaMemcpy(&st, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost));
  if (st == hd::kStatusTmaTimeout) {
    HD_CUDA(cudaMemset(ctx->d_status, 0, sizeof(int)));
    fail(HD_ERR_TIMEOUT, "a device wait for a TMA transfer ran out (pairwise kernel)");
  }
}

// Device copy of host (or pass-through of device) FASTA bytes; 16-byte aligned.
const uint8_t *stage_input(hd_ctx *ctx, const char *bytes, uint64_t n, int on_device) {
  if (on_device && (reinterpret_cast<uintptr_t>(bytes) & 15u) == 0)
    return reinterpret_cast<const uint8_t *>(bytes);
  ctx->file_tag.clear();
  if (ctx->file.bytes < n + 16) {
    ctx->file.release();
    ctx->file = DevBuf(hd::round_up(n + 16, 1 << 20), ctx->stream);
  }
  if (n)
    HD_CUDA(cudaMemcpyAsync(ctx->file.p, bytes, n,
                            on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                            ctx->stream));
  return ctx->file.as<uint8_t>();
}

std::string open_failed(const char *path) {
  return std::string("Error: Failed to open file '") + (path ? path : "") + "'";
}

// What identifies a file's contents for the device input cache: path, size,
// inode, device, and the modification and status-change times in ns.
std::string file_tag(const char *path, const struct stat &sb) {
  char buf[160];
  std::snprintf(buf, sizeof buf, "|%llu|%llu|%llu|%lld.%09ld|%lld.%09ld",
                (unsigned long long)sb.st_size, (unsigned long long)sb.st_ino,
                (unsigned long long)sb.st_dev, (long long)sb.st_mtim.tv_sec, sb.st_mtim.tv_nsec,
                (long long)sb.st_ctim.tv_sec, sb.st_ctim.tv_nsec);
  return std::string(path) + buf;
}

// Worker threads for a file read: pread into staging, or populating a
// mapping that is not all in the page cache (the workers then read it from
// storage), HAMMINGDIST_READ_THREADS, else 16; populating a mapping of a
// cached file, HAMMINGDIST_MAP_THREADS, else 1 (page-table updates from more
// threads contend and are slower: 598 MB took 3.4 ms to upload with 1, 4.0 ms
// with 16).
unsigned read_threads(bool cached_map) {
  const char *e = std::getenv(cached_map ? "HAMMINGDIST_MAP_THREADS" : "HAMMINGDIST_READ_THREADS");
  return e ? (unsigned)std::max(1, std::atoi(e)) : cached_map ? 1u : 16u;
}

// Fills the page-table entries of [p, p + len) in a read-only file mapping
// (p page aligned), reading from storage what is not cached, so that a copy
// from the mapping finds every page. False if the file cannot be read there
// (it shrank, or an I/O error).
bool populate(void *p, uint64_t len) {
  for (;;) {
    if (::madvise(p, (size_t)len, MADV_POPULATE_READ) == 0) return true;
    if (errno == EINTR || errno == EAGAIN) continue;
    if (errno != EINVAL) return false;
    // a kernel without MADV_POPULATE_READ: touch one byte per page
    const uint64_t page = (uint64_t)::sysconf(_SC_PAGESIZE);
    volatile const char *v = static_cast<const char *>(p);
    char sink = 0;
    for (uint64_t o = 0; o < len; o += page) sink ^= v[o];
    (void)sink;
    return true;
  }
}

// Whether every page of a mapping is in the page cache.
bool all_cached(void *map, size_t len) {
  const size_t page = (size_t)::sysconf(_SC_PAGESIZE);
  std::vector<unsigned char> v(hd::ceil_div(len, page));
  if (::mincore(map, len, v.data()) != 0) return false;
  for (unsigned char c : v)
    if (!(c & 1)) return false;
  return true;
}

// Background reader of a file into a device buffer. Worker threads take 8 MB
// parts in file order; one uploader thread copies the parts that are ready to
// the device, in file order, on ctx->up, and records an event after each.
//   mapped (ctx->map_files): the file is mapped read-only and a worker
//     populates a part's page-table entries (MADV_POPULATE_READ, which also
//     reads the part from storage if it is not cached); the copy then reads
//     the page cache directly, with no CPU copy.
//   staged: a worker preads a part into the context's pinned staging, which
//     is copied.
// host() holds the file's bytes [0, prefix_bytes()); wait_bytes(x) waits
// until it holds [0, x); stream_wait_bytes(s, x) makes stream s wait for the
// copies of [0, x) only, not for the copies queued after them. The destructor
// stops the threads, joins them, waits for the copies, unmaps and closes.
struct PartReader {
  hd_ctx *ctx;
  const char *path;
  uint64_t n;
  uint8_t *dev;
  static constexpr uint64_t kPart = 8ull << 20;
  static constexpr uint64_t kCopyParts = 8;  // parts per copy at most
  uint64_t parts;
  int fd = -1;
  void *map = nullptr;
  size_t map_len = 0;
  char *host_ = nullptr;  // the mapping, or pinned staging
  std::atomic<uint64_t> next{0};
  std::atomic<int> bad{0};  // 1 = read error, 2 = copy error, 3 = stopped
  std::mutex mu;
  std::condition_variable cv;
  std::vector<char> done;
  uint64_t prefix = 0;  // parts [0, prefix) on the host
  uint64_t queued = 0;  // parts [0, queued) copies queued on ctx->up, events recorded
  std::vector<std::thread> th;

  PartReader(hd_ctx *c, const char *p, uint64_t bytes, uint8_t *d)
      : ctx(c), path(p), n(bytes), dev(d), parts(hd::ceil_div(bytes, kPart)), done(parts, 0) {}
  ~PartReader() {
    fault(3);
    join();
    cudaStreamSynchronize(ctx->up);
    if (map) ::munmap(map, map_len);
    if (fd >= 0) ::close(fd);
  }
  const char *host() const { return host_; }

  void start() {
    fd = ::open(path, O_RDONLY);
    if (fd < 0) fail(HD_ERR_IO, open_failed(path));
    if (ctx->map_files && n) {
      const uint64_t page = (uint64_t)::sysconf(_SC_PAGESIZE);
      const size_t len = (size_t)hd::round_up(n, page);
      void *m = ::mmap(nullptr, len, PROT_READ, MAP_SHARED, fd, 0);
      if (m != MAP_FAILED) {
        map = m;
        map_len = len;
        host_ = static_cast<char *>(m);
      }
    }
    if (!host_) {
      if (n + 1 > ctx->pin_cap) {
        if (ctx->pin) cudaFreeHost(ctx->pin);
        ctx->pin = nullptr;
        ctx->pin_cap = 0;
        const size_t cap = (size_t)((n + 1) * 5 / 4 + (1 << 20));
        HD_CUDA(cudaHostAlloc(&ctx->pin, cap, cudaHostAllocDefault));
        ctx->pin_cap = cap;
      }
      host_ = static_cast<char *>(ctx->pin);
    }
    while (ctx->part_ev.size() < parts + 1) {
      cudaEvent_t e;
      HD_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
      ctx->part_ev.push_back(e);
    }
    // the device buffer is allocated (and earlier work on it ordered) on
    // ctx->stream: the copies on ctx->up come after that
    HD_CUDA(cudaEventRecord(ctx->part_ev[parts], ctx->stream));
    HD_CUDA(cudaStreamWaitEvent(ctx->up, ctx->part_ev[parts], 0));
    hd::trace_host(ctx, "file mapped");
    if (!parts) return;
    th.emplace_back([this] { upload(); });
    if (!map) {
      const unsigned nt = (unsigned)std::min<uint64_t>(read_threads(false), parts);
      for (unsigned t = 0; t < nt; ++t) th.emplace_back([this] { work(); });
      return;
    }
    // one worker starts on the first parts at once; whether the file is all
    // in the page cache (one populating thread, the pages only need mapping)
    // or not (many, which read from storage in parallel) is checked meanwhile:
    // the check takes about 0.35 ms for 598 MB
    th.emplace_back([this] { work(); });
    const bool cached_map = all_cached(map, map_len);
    hd::trace_host(ctx, "page cache checked");
    const unsigned nt = (unsigned)std::min<uint64_t>(read_threads(cached_map), parts);
    for (unsigned t = 1; t < nt; ++t) th.emplace_back([this] { work(); });
  }
  void join() {
    for (auto &x : th)
      if (x.joinable()) x.join();
  }
  bool read_part(uint64_t off, uint64_t len) {
    if (map) return populate(host_ + off, len);  // off: a multiple of 8 MB, page aligned
    uint64_t got = 0;
    while (got < len) {
      const ssize_t r = ::pread(fd, host_ + off + got, (size_t)(len - got), (off_t)(off + got));
      if (r <= 0) return false;
      got += (uint64_t)r;
    }
    return true;
  }
  void work() {
    for (;;) {
      const uint64_t k = next.fetch_add(1);
      if (k >= parts || bad.load()) return;
      const uint64_t off = k * kPart;
      if (!read_part(off, std::min(kPart, n - off))) {
        fault(1);
        return;
      }
      std::lock_guard<std::mutex> lk(mu);
      done[k] = 1;
      while (prefix < parts && done[prefix]) ++prefix;
      cv.notify_all();
    }
  }
  // the host prefix, in order, up to kCopyParts parts per copy
  void upload() {
    if (cudaSetDevice(ctx->device) != cudaSuccess) {
      fault(2);
      return;
    }
    for (uint64_t k = 0; k < parts;) {
      uint64_t e;
      {
        std::unique_lock<std::mutex> lk(mu);
        cv.wait(lk, [&] { return bad.load() || prefix > k; });
        if (bad.load()) return;
        e = std::min(prefix, k + kCopyParts);
      }
      const uint64_t off = k * kPart, len = std::min(e * kPart, n) - off;
      if (cudaMemcpyAsync(dev + off, host_ + off, len, cudaMemcpyHostToDevice, ctx->up) !=
          cudaSuccess) {
        fault(2);
        return;
      }
      for (uint64_t j = k; j < e; ++j)
        if (cudaEventRecord(ctx->part_ev[j], ctx->up) != cudaSuccess) {
          fault(2);
          return;
        }
      std::lock_guard<std::mutex> lk(mu);
      queued = k = e;
      cv.notify_all();
    }
  }
  void fault(int code) {
    std::lock_guard<std::mutex> lk(mu);
    if (!bad.load()) bad = code;
    cv.notify_all();
  }
  uint64_t prefix_bytes() {
    std::lock_guard<std::mutex> lk(mu);
    return std::min(n, prefix * kPart);
  }
  bool wait_bytes(uint64_t x) {
    std::unique_lock<std::mutex> lk(mu);
    cv.wait(lk, [&] { return bad.load() || std::min(n, prefix * kPart) >= std::min(x, n); });
    return !bad.load();
  }
  // stream s waits for the copies of bytes [0, x); false after an error
  bool stream_wait_bytes(cudaStream_t s, uint64_t x) {
    const uint64_t k = hd::ceil_div(std::min(x, n), kPart);
    if (k == 0) return !bad.load();
    {
      std::unique_lock<std::mutex> lk(mu);
      cv.wait(lk, [&] { return bad.load() || queued >= k; });
      if (bad.load()) return false;
    }
    return cudaStreamWaitEvent(s, ctx->part_ev[k - 1], 0) == cudaSuccess;
  }
  // waits for the whole file: ctx->stream then waits for every copy; throws
  // HD_ERR_IO after a read error, HD_ERR_CUDA after a copy error
  void finish() {
    const bool ok = stream_wait_bytes(ctx->stream, n);
    join();
    if (!ok || bad.load()) {
      if (bad.load() == 1) fail(HD_ERR_IO, open_failed(path));
      fail(HD_ERR_CUDA, "cudaMemcpyAsync of the FASTA file failed");
    }
  }
};

// Reads a FASTA file into the context's device input buffer with a
// PartReader: 8 MB parts are copied as they become ready, so the upload runs
// under the read. If the buffer already holds this file, unchanged, nothing
// is read or copied. Returns the device bytes; *nbytes = the file size.
const uint8_t *stage_file(hd_ctx *ctx, const char *path, uint64_t *nbytes) {
  struct stat sb;
  if (!path || ::stat(path, &sb) != 0 || !S_ISREG(sb.st_mode)) fail(HD_ERR_IO, open_failed(path));
  const uint64_t n = (uint64_t)sb.st_size;
  *nbytes = n;
  const std::string tag = file_tag(path, sb);
  if (!ctx->file_tag.empty() && ctx->file_tag == tag && ctx->file.bytes >= n + 16) {
    hd::trace_mark(ctx, "file already on the device");
    return ctx->file.as<uint8_t>();
  }
  ctx->file_tag.clear();
  if (ctx->file.bytes < n + 16) {
    ctx->file.release();
    ctx->file = DevBuf(hd::round_up(n + 16, 1 << 20), ctx->stream);
  }
  uint8_t *dev = ctx->file.as<uint8_t>();
  {
    PartReader rd(ctx, path, n, dev);
    rd.start();
    rd.finish();
  }
  ctx->file_tag = tag;
  return dev;
}

// The records of the FASTA file in the context's input buffer, parsed once
// per (file, record limit): a second call on the same unchanged file (e.g.
// fasta_reference_distances after from_fasta) reuses them.
hd::Records &file_records(hd_ctx *ctx, const uint8_t *d, uint64_t nbytes, uint64_t n_limit) {
  if (ctx->parsed && !ctx->file_tag.empty() && ctx->parsed_tag == ctx->file_tag &&
      ctx->parsed_limit == n_limit) {
    hd::trace_mark(ctx, "records already parsed");
    return *static_cast<hd::Records *>(ctx->parsed.get());
  }
  ctx->parsed.reset();
  auto rec = std::make_shared<hd::Records>(hd::parse_fasta(ctx, d, nbytes, n_limit));
  ctx->parsed = rec;
  ctx->parsed_tag = ctx->file_tag;
  ctx->parsed_limit = n_limit;
  return *rec;
}

// Writes one byte of every page of a large host output on up to 16 threads:
// the first touch of fresh pageable pages costs several ms per 100 MB on one
// thread, and pages already present (a recycled buffer) cost next to nothing.
// Called after the kernel is launched, so it runs while the GPU computes and
// the copy back then finds the pages present.
void prefault_host(void *p, uint64_t n) {
  const uint64_t kMin = 16ull << 20, kPart = 4ull << 20;
  if (n < kMin) return;
  static const uint64_t page = [] {
    const long v = sysconf(_SC_PAGESIZE);
    return (uint64_t)(v > 0 ? v : 4096);
  }();
  {
    // a recycled buffer has its pages already: then starting the threads
    // would cost more than the touches
    const uintptr_t a0 = reinterpret_cast<uintptr_t>(p) & ~(uintptr_t)(page - 1);
    const size_t len = reinterpret_cast<uintptr_t>(p) + n - a0;
    std::vector<unsigned char> v(hd::ceil_div(len, page));
    if (::mincore(reinterpret_cast<void *>(a0), len, v.data()) == 0 &&
        std::all_of(v.begin(), v.end(), [](unsigned char c) { return (c & 1) != 0; }))
      return;
  }
  const unsigned nt = (unsigned)std::min<uint64_t>(16, n / kPart);
  const uint64_t per = hd::round_up(hd::ceil_div(n, nt), page);
  std::vector<std::thread> th;
  for (unsigned t = 0; t < nt; ++t)
    th.emplace_back([=] {
      const uint64_t a = t * per, b = std::min(n, a + per);
      for (uint64_t off = a; off < b; off += page) static_cast<volatile char *>(p)[off] = 0;
    });
  for (auto &x : th) x.join();
}

uint64_t words_for(uint64_t L) { return hd::round_up(hd::ceil_div(L ? L : 1, 32), 8); }

// validate_data (src/hamming_impl.cc:80-91) + the include_x/use_gpu check
// (include/hamming/hamming_impl.hh:99-102) + dedupe + rule choice + pack.
hd_alignment *build_alignment(hd_ctx *ctx, hd::Records &rec, int remove_duplicates, int include_x,
                              int semantics) {
  if (rec.n == 0 || rec.len0 == 0) fail(HD_ERR_EMPTY, kMsgEmpty);
  if (!rec.all_equal) fail(HD_ERR_LENGTH, kMsgLength);
  if (semantics == HD_SEM_GPU && include_x) fail(HD_ERR_INCLUDE_X_GPU, kMsgIncludeX);
  if (semantics != HD_SEM_GPU && semantics != HD_SEM_CPU) fail(HD_ERR_ARG, "bad semantics");
  auto *aln = new hd_alignment();
  try {
    aln->ctx = ctx;
    aln->device = ctx->device;
    aln->n_input = rec.n;
    aln->length = rec.len0;
    aln->words = words_for(rec.len0);
    DevBuf rows;
    const uint64_t *d_rows = nullptr;
    if (remove_duplicates) {
      uint64_t nu = 0;
      rows = hd::dedupe(ctx, rec, &nu, aln->seqidx);
      d_rows = rows.as<uint64_t>();
      aln->n_rows = nu;
      hd::trace_mark(ctx, "dedupe");
    } else {
      aln->n_rows = rec.n;
    }
    int rule = HD_RULE_AND;
    if (semantics == HD_SEM_CPU) {
      if (include_x) {
        rule = HD_RULE_SPARSE_X;
      } else {
        // include/hamming/hamming_impl.hh:104-118: sparse when fewer than 0.5%
        // of all sites differ from the per-site consensus
        const uint64_t total = aln->n_rows * aln->length;
        const uint64_t same = hd::consensus_matches(ctx, rec, d_rows, aln->n_rows);
        const double frac = (double)(total - same) / (double)total;
        rule = frac < 0.005 ? HD_RULE_SPARSE : HD_RULE_AND;
        hd::trace_mark(ctx, "consensus");
      }
    }
    aln->rule = rule;
    aln->planes = hd::planes_of(rule);
    aln->groups = aln->planes > 4 ? 2 : 1;
    hd::pack_rows(ctx, rec, d_rows, aln);
    if (!aln->seqidx.empty()) {
      aln->d_seqidx = DevBuf(aln->seqidx.size() * 8, ctx->stream);
      HD_CUDA(cudaMemcpyAsync(aln->d_seqidx.p, aln->seqidx.data(), aln->seqidx.size() * 8,
                              cudaMemcpyHostToDevice, ctx->stream));
    }
    hd::trace_mark(ctx, "pack");
    HD_CUDA(cudaStreamSynchronize(ctx->stream));
  } catch (...) {
    delete aln;
    throw;
  }
  return aln;
}

// ---------------------------------------------------------------- file out
// Text output files, (re)created as the reference's writers do, written in
// order with write(). (A shared mapping of the file copied by 8 threads took
// 2.82 s for the 10 GB text of n=100,000 on ext4 with 64 KB pages, against
// 1.69 s for write(): page faults on the mapping cost more than one thread's
// copy saves.)
struct OutFile {
  int fd = -1;
  std::string path;
  explicit OutFile(const char *p) : path(p) {
    fd = ::open(p, O_WRONLY | O_CREAT | O_TRUNC, 0644);
    if (fd < 0) fail(HD_ERR_IO, "Error: Failed to open file '" + path + "'");
  }
  void write(const char *buf, uint64_t n) {
    while (n) {
      const ssize_t w = ::write(fd, buf, n > (1ull << 30) ? (1ull << 30) : n);
      if (w < 0) {
        if (errno == EINTR) continue;
        fail(HD_ERR_IO, "Error: Failed to write file '" + path + "'");
      }
      buf += w;
      n -= (uint64_t)w;
    }
  }
  ~OutFile() {
    if (fd >= 0) ::close(fd);
  }
};

// Pinned double buffer: the host writes one half while the device fills the
// other.
struct PinnedPair {
  char *buf[2] = {nullptr, nullptr};
  uint64_t cap = 0;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  explicit PinnedPair(uint64_t c) : cap(c) {
    for (int k = 0; k < 2; ++k) {
      HD_CUDA(cudaHostAlloc(reinterpret_cast<void **>(&buf[k]), c ? c : 1, cudaHostAllocDefault));
      HD_CUDA(cudaEventCreateWithFlags(&ev[k], cudaEventDisableTiming));
    }
  }
  ~PinnedPair() {
    for (int k = 0; k < 2; ++k) {
      if (buf[k]) cudaFreeHost(buf[k]);
      if (ev[k]) cudaEventDestroy(ev[k]);
    }
  }
};

uint64_t tri(uint64_t i) { return i * (i - 1) / 2; }

// Row ranges [r0, r1) whose lower-triangle entries stay under max_entries
// (at least one row each). If align is set, boundaries are multiples of it.
std::vector<std::pair<uint64_t, uint64_t>> row_chunks(uint64_t n, uint64_t max_entries,
                                                      uint64_t align) {
  std::vector<std::pair<uint64_t, uint64_t>> out;
  uint64_t r0 = 0;
  while (r0 < n) {
    uint64_t r1 = r0 + align;
    while (r1 < n && tri(std::min(r1 + align, n)) - tri(r0) <= max_entries) r1 += align;
    r1 = std::min(r1, n);
    out.emplace_back(r0, r1);
    r0 = r1;
  }
  return out;
}

constexpr uint64_t kTextChunkBytes = 256ull << 20;  // text per streamed chunk (bound)

// Streams lower-triangular text of rows [0, n) to `path`. `produce(r0, r1,
// d_lt)` leaves the entries of rows [r0, r1) in d_lt (lt index tri(r0) at
// d_lt[0]) on ctx->stream.
template <class Produce>
void stream_lt_text(hd_ctx *ctx, uint64_t n, int dtype_bytes, const char *path, uint64_t align,
                    Produce &&produce) {
  if (n < 2) return;  // no entries: the reference leaves the file untouched
  const uint64_t per = dtype_bytes == 1 ? 4 : dtype_bytes == 2 ? 6 : 11;
  const uint64_t max_entries = std::max<uint64_t>(kTextChunkBytes / per, 1);
  auto chunks = row_chunks(n, max_entries, align);
  uint64_t max_e = 0, max_text = 0;
  for (auto &c : chunks) {
    max_e = std::max(max_e, tri(c.second) - tri(std::max<uint64_t>(c.first, 1)));
    max_text = std::max(max_text, hd::lt_text_bound(c.first, c.second, dtype_bytes));
  }
  DevBuf d_lt((max_e + 1) * dtype_bytes, ctx->stream), d_text(max_text + 16, ctx->stream);
  PinnedPair pin(max_text + 16);
  OutFile f(path);
  uint64_t pending_bytes = 0;
  int pending = -1;
  for (size_t k = 0; k < chunks.size(); ++k) {
    const uint64_t r0 = chunks[k].first, r1 = chunks[k].second;
    produce(r0, r1, d_lt.p);
    // write the previous chunk while this one computes
    if (pending >= 0) {
      HD_CUDA(cudaEventSynchronize(pin.ev[pending]));
      f.write(pin.buf[pending], pending_bytes);
      pending = -1;
    }
    const uint64_t nb = hd::format_lt_rows(ctx, d_lt.p, dtype_bytes, tri(r0), r0, r1, d_text.as<char>());
    const int slot = (int)(k & 1);
    if (nb)
      HD_CUDA(cudaMemcpyAsync(pin.buf[slot], d_text.p, nb, cudaMemcpyDeviceToHost, ctx->stream));
    HD_CUDA(cudaEventRecord(pin.ev[slot], ctx->stream));
    pending = slot;
    pending_bytes = nb;
  }
  if (pending >= 0) {
    HD_CUDA(cudaEventSynchronize(pin.ev[pending]));
    f.write(pin.buf[pending], pending_bytes);
  }
  check_status(ctx);
}

// fasta_reference_distances (src/hamming.cc:104-141) over FASTA bytes already
// on the device: parse, one distance per record, copy to a malloc'd array.
// from_file: d is the context's input buffer holding a file (stage_file), so
// its parsed records may be reused
void reference_distances_of(hd_ctx *ctx, const uint8_t *d, uint64_t nbytes, const char *ref,
                            uint64_t ref_len, int include_x, uint32_t **out, uint64_t *n_out,
                            bool from_file) {
  hd::Records parsed;
  if (!from_file) parsed = hd::parse_fasta(ctx, d, nbytes, 0);
  const hd::Records &rec = from_file ? file_records(ctx, d, nbytes, 0) : parsed;
  hd::trace_mark(ctx, "parse");
  if (rec.max_len > ref_len)
    fail(HD_ERR_REF_LENGTH, "Error: a sequence is longer than the reference sequence");
  uint32_t *h = static_cast<uint32_t *>(std::malloc((rec.n ? rec.n : 1) * 4));
  if (!h) throw std::bad_alloc();
  try {
    if (rec.n) {
      DevBuf d_ref(ref_len + 16, ctx->stream), d_out(rec.n * 4, ctx->stream);
      if (ref_len)
        HD_CUDA(cudaMemcpyAsync(d_ref.p, ref, ref_len, cudaMemcpyHostToDevice, ctx->stream));
      // Records all of the reference's length, whose dense-rule rows a
      // from_fasta of this file left: without include_x the rule of
      // src/hamming.cc:128-136 counts a site exactly when the two codes share
      // no bit (a '-' shares bits with every symbol; equal symbols share
      // theirs; every other byte has code 0), so the distances are the rows'
      // dense distances to the packed reference
      const hd_alignment *rows = rec.rows.get();
      if (rows && !include_x && rec.all_equal && rec.len0 == ref_len && rows->length == ref_len &&
          rows->n_input == rec.n) {
        DevBuf d_rows(rows->n_rows * 4, ctx->stream);
        hd::query_rows_to_records(ctx, rows, d_ref.as<uint8_t>(), d_rows.as<uint32_t>(),
                                  rec.row_of.as<uint64_t>(), rec.n, d_out.as<uint32_t>());
        hd::trace_mark(ctx, "distances from the resident rows");
      } else {
        hd::reference_distances_device(ctx, rec, d_ref.as<uint8_t>(), include_x,
                                       d_out.as<uint32_t>());
        hd::trace_mark(ctx, "distances");
      }
      HD_CUDA(cudaMemcpyAsync(h, d_out.p, rec.n * 4, cudaMemcpyDeviceToHost, ctx->stream));
      hd::trace_mark(ctx, "copy to host");
      HD_CUDA(cudaStreamSynchronize(ctx->stream));
    }
    hd::trace_end(ctx);
  } catch (...) {
    std::free(h);
    throw;
  }
  *out = h;
  *n_out = rec.n;
}

// fasta_sequence_indices (src/hamming.cc:76-102) over FASTA bytes on the device.
void sequence_indices_of(hd_ctx *ctx, const uint8_t *d, uint64_t nbytes, uint64_t n_limit,
                         uint64_t **out, uint64_t *n_out, bool from_file) {
  hd::Records parsed;
  if (!from_file) parsed = hd::parse_fasta(ctx, d, nbytes, n_limit);
  const hd::Records &rec = from_file ? file_records(ctx, d, nbytes, n_limit) : parsed;
  std::vector<uint64_t> idx;
  uint64_t nu = 0;
  DevBuf rows = hd::dedupe(ctx, rec, &nu, idx);
  uint64_t *h = static_cast<uint64_t *>(std::malloc((idx.size() ? idx.size() : 1) * 8));
  if (!h) throw std::bad_alloc();
  if (!idx.empty()) std::memcpy(h, idx.data(), idx.size() * 8);
  *out = h;
  *n_out = idx.size();
}

}  // namespace

// =================================================================== ABI
extern "C" {

int hd_device_available(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n > 0 ? 1 : 0;
}

int hd_ctx_create(int device, hd_ctx **out) {
  if (!out) return HD_ERR_ARG;
  *out = nullptr;
  if (!hd_device_available()) return HD_ERR_NO_DEVICE;
  auto *ctx = new hd_ctx();
  ctx->device = device;
  int rc = guard(ctx, [&] {
    HD_CUDA(cudaSetDevice(device));
    HD_CUDA(cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device));
    HD_CUDA(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
    HD_CUDA(cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking));
    HD_CUDA(cudaStreamCreateWithFlags(&ctx->up, cudaStreamNonBlocking));
    // files are copied from their page-cache mapping where the device reads
    // pageable memory through the host's page tables (Grace: NVLink-C2C);
    // HAMMINGDIST_READ_MODE=pread keeps the pread + pinned staging order
    int host_pt = 0;
    HD_CUDA(cudaDeviceGetAttribute(&host_pt, cudaDevAttrPageableMemoryAccessUsesHostPageTables,
                                   device));
    ctx->map_files = host_pt == 1;
    if (const char *m = std::getenv("HAMMINGDIST_READ_MODE"))
      if (std::string(m) == "pread") ctx->map_files = 0;
    HD_CUDA(cudaEventCreate(&ctx->ev_start));
    HD_CUDA(cudaEventCreate(&ctx->ev_stop));
    HD_CUDA(cudaMalloc(&ctx->d_status, 64));
    HD_CUDA(cudaMemset(ctx->d_status, 0, 64));
    cudaMemPool_t pool;
    HD_CUDA(cudaDeviceGetDefaultMemPool(&pool, device));
    uint64_t thr = std::numeric_limits<uint64_t>::max();
    HD_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr));
    cudaDriverEntryPointQueryResult q;
    void *fn = nullptr;
    HD_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000,
                                             cudaEnableDefault, &q));
    if (!fn || q != cudaDriverEntryPointSuccess) fail(HD_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
    ctx->encode_tiled = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    if (const char *t = std::getenv("HAMMINGDIST_TRACE")) ctx->trace.on = t[0] && t[0] != '0';
    // default autotuner table: HAMMINGDIST_TUNING names a file saved by
    // hd_tune_save; it applies only if it was measured on this device kind
    if (const char *path = std::getenv("HAMMINGDIST_TUNING")) {
      cudaDeviceProp prop;
      HD_CUDA(cudaGetDeviceProperties(&prop, device));
      FILE *f = std::fopen(path, "rb");
      if (f) {
        char head[256] = {0};
        size_t got = std::fread(head, 1, sizeof(head) - 1, f);
        std::fclose(f);
        head[got] = 0;
        const std::string want = std::string("\"device\": \"") + prop.name + "\"";
        if (std::string(head).find(want) != std::string::npos) hd_tune_load(ctx, path);
      }
    }
  });
  if (rc != HD_OK) {
    hd_ctx_destroy(ctx);
    return rc;
  }
  *out = ctx;
  return HD_OK;
}

void hd_ctx_destroy(hd_ctx *ctx) {
  if (!ctx) return;
  for (hd_ctx *w : ctx->workers) hd_ctx_destroy(w);
  ctx->workers.clear();
  cudaSetDevice(ctx->device);
  ctx->parsed.reset();  // its buffers are freed on ctx->stream
  ctx->file.release();
  if (ctx->pin) cudaFreeHost(ctx->pin);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  if (ctx->d_status) cudaFree(ctx->d_status);
  if (ctx->ev_start) cudaEventDestroy(ctx->ev_start);
  if (ctx->ev_stop) cudaEventDestroy(ctx->ev_stop);
  for (cudaEvent_t e : ctx->trace.pool) cudaEventDestroy(e);
  if (ctx->up) cudaStreamSynchronize(ctx->up);
  for (cudaEvent_t e : ctx->part_ev) cudaEventDestroy(e);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  if (ctx->side) cudaStreamDestroy(ctx->side);
  if (ctx->up) cudaStreamDestroy(ctx->up);
  delete ctx;
}

const char *hd_last_error(const hd_ctx *ctx) { return ctx ? ctx->err.c_str() : ""; }

int hd_trace_enable(hd_ctx *ctx, int on) {
  if (!ctx) return HD_ERR_ARG;
  ctx->trace.on = on != 0;
  if (!ctx->trace.on) ctx->trace.last.clear();
  return HD_OK;
}

const char *hd_trace_last(const hd_ctx *ctx) { return ctx ? ctx->trace.last.c_str() : ""; }

uint64_t hd_ctx_kernel_launches(const hd_ctx *ctx) { return ctx ? ctx->launches : 0; }

int hd_host_alloc(hd_ctx *ctx, size_t bytes, void **out) {
  return guard(ctx, [&] {
    if (!out) fail(HD_ERR_ARG, "null output");
    *out = nullptr;
    HD_CUDA(cudaHostAlloc(out, bytes ? bytes : 1, cudaHostAllocDefault));
  });
}

void hd_host_free(hd_ctx *ctx, void *p) {
  if (ctx) cudaSetDevice(ctx->device);
  if (p) cudaFreeHost(p);
}

void hd_free(void *p) { std::free(p); }

void *hd_ctx_stream(const hd_ctx *ctx) { return ctx ? static_cast<void *>(ctx->stream) : nullptr; }

int hd_ctx_synchronize(hd_ctx *ctx) {
  return guard(ctx, [&] { HD_CUDA(cudaStreamSynchronize(ctx->stream)); });
}

int hd_alignment_from_fasta(hd_ctx *ctx, const char *fasta, uint64_t nbytes, int fasta_on_device,
                            int remove_duplicates, uint64_t n_limit, int include_x, int semantics,
                            hd_alignment **out) {
  if (!ctx || !out || (!fasta && nbytes)) return HD_ERR_ARG;
  *out = nullptr;
  return guard(ctx, [&] {
    hd::trace_begin(ctx, "hd_alignment_from_fasta");
    const uint8_t *d = stage_input(ctx, fasta, nbytes, fasta_on_device);
    hd::trace_mark(ctx, "upload");
    hd::Records rec = hd::parse_fasta(ctx, d, nbytes, n_limit);
    hd::trace_mark(ctx, "parse");
    *out = build_alignment(ctx, rec, remove_duplicates, include_x, semantics);
    hd::trace_end(ctx);
  });
}

int hd_alignment_from_fasta_file(hd_ctx *ctx, const char *path, int remove_duplicates,
                                 uint64_t n_limit, int include_x, int semantics,
                                 hd_alignment **out) {
  if (!ctx || !out || !path) return HD_ERR_ARG;
  *out = nullptr;
  return guard(ctx, [&] {
    hd::trace_begin(ctx, "hd_alignment_from_fasta_file");
    uint64_t nbytes = 0;
    const uint8_t *d = stage_file(ctx, path, &nbytes);
    hd::trace_mark(ctx, "read + upload");
    hd::Records &rec = file_records(ctx, d, nbytes, n_limit);
    hd::trace_mark(ctx, "parse");
    *out = build_alignment(ctx, rec, remove_duplicates, include_x, semantics);
    hd::trace_end(ctx);
  });
}

int hd_pairwise_lt_fasta_file(hd_ctx *ctx, const char *path, int remove_duplicates,
                              int dtype_bytes, int64_t max_distance, hd_output_fn out_fn,
                              void *user, hd_alignment **aln_out) {
  if (!ctx || !path || !out_fn || !aln_out) return HD_ERR_ARG;
  *aln_out = nullptr;
  return guard(ctx, [&] {
    check_dtype(dtype_bytes);
    const uint32_t md = clamp_max(max_distance, dtype_bytes);
    hd::trace_begin(ctx, "hd_pairwise_lt_fasta_file");
    struct stat sb;
    if (::stat(path, &sb) != 0 || !S_ISREG(sb.st_mode)) fail(HD_ERR_IO, open_failed(path));
    const uint64_t n = (uint64_t)sb.st_size;
    const std::string tag = file_tag(path, sb);
    // the whole matrix after the whole file: the file call + one pairwise call
    auto whole = [&] {
      hd_alignment *a = nullptr;
      uint64_t nbytes = 0;
      const uint8_t *d = stage_file(ctx, path, &nbytes);
      hd::trace_mark(ctx, "read + upload");
      hd::Records &rec = file_records(ctx, d, nbytes, 0);
      hd::trace_mark(ctx, "parse");
      a = build_alignment(ctx, rec, remove_duplicates, 0, HD_SEM_GPU);
      std::unique_ptr<hd_alignment> own(a);
      const uint64_t entries = a->n_rows < 2 ? 0 : tri(a->n_rows);
      void *host = out_fn(user, 0, a->n_rows, entries);
      if (!host && entries) fail(HD_ERR_ARG, "output callback returned no buffer");
      void *mirror = entries ? out_fn(user, HD_OUTPUT_MIRROR, a->n_rows, entries) : nullptr;
      if (entries) {
        DevBuf d_out(entries * dtype_bytes, ctx->stream);
        hd::pairwise_tiles(ctx, a, dtype_bytes, md, d_out.p, 0, 0,
                           (uint32_t)hd::ceil_div(a->n_rows, hd::kTile));
        hd::trace_mark(ctx, "pairwise");
        prefault_host(host, entries * dtype_bytes);
        HD_CUDA(cudaMemcpyAsync(host, d_out.p, entries * dtype_bytes, cudaMemcpyDeviceToHost,
                                ctx->stream));
        if (mirror) {
          prefault_host(mirror, entries * dtype_bytes);
          HD_CUDA(cudaMemcpyAsync(mirror, d_out.p, entries * dtype_bytes, cudaMemcpyDeviceToHost,
                                  ctx->stream));
        }
        HD_CUDA(cudaStreamSynchronize(ctx->stream));
        check_status(ctx);
      }
      *aln_out = own.release();
    };
    // small files (below 64 MB, or HAMMINGDIST_STREAM_MIN_BYTES), or a file
    // already on the device: nothing to overlap
    uint64_t min_bytes = 64ull << 20;
    if (const char *e = std::getenv("HAMMINGDIST_STREAM_MIN_BYTES"))
      min_bytes = std::strtoull(e, nullptr, 10);
    if (n < min_bytes || (!ctx->file_tag.empty() && ctx->file_tag == tag)) {
      whole();
      hd::trace_end(ctx);
      return;
    }
    ctx->file_tag.clear();
    ctx->parsed.reset();
    hd::trace_host(ctx, "earlier file released");
    if (ctx->file.bytes < n + 16) {
      ctx->file.release();
      ctx->file = DevBuf(hd::round_up(n + 16, 1 << 20), ctx->stream);
    }
    uint8_t *dev = ctx->file.as<uint8_t>();
    auto reader = std::make_unique<PartReader>(ctx, path, n, dev);
    reader->start();
    hd::trace_host(ctx, "readers started");
    const char *text = reader->host();
    hd::trace_mark(ctx, "setup");
    auto read_all = [&] {
      reader->finish();
      ctx->file_tag = tag;
    };
    // the first record header at or after pos (>= 1), 0 if none
    auto header_at = [&](uint64_t pos) -> uint64_t {
      for (;;) {
        if (!reader->wait_bytes(std::min(n, pos + PartReader::kPart))) return 0;
        const uint64_t avail = reader->prefix_bytes();
        for (; pos < avail; ++pos)
          if (text[pos] == '>' && text[pos - 1] == '\n') return pos;
        if (avail >= n) return 0;
      }
    };
    // The file is ingested in parts that end at the first record headers
    // after the given fractions of its bytes. After each part its new records
    // are deduplicated against the earlier ones (first occurrences keep their
    // order, so earlier unique rows keep their positions) and the new unique
    // rows are packed; the tile rows that are complete then run on the side
    // stream, with 16 SMs left for the next part's ingest. The last part's
    // tile rows run as two launches, split at 90% of the tile rows, so that
    // the copy of every finished range to the host overlaps the rest of the
    // distances.
    // part ends as fractions of the file (HAMMINGDIST_STREAM_SPLITS="f1,f2,...",
    // increasing, at most 3). At n=20,000 x L=29,903 the file-to-host step
    // (with the reference distances) took 7.17-7.21 ms with splits at 35% and
    // 65%, 7.28-7.37 at 30% and 60%, 7.53 at 40% and 70%, and 7.55-7.81 with
    // three splits (10-20%, 35-45%, 65-70%); without a split, 10.26 ms (with
    // older kernels). Each part's ingest costs launches and host round trips
    // whatever its size, so a few large parts do best.
    std::vector<double> ends = {0.35, 0.65};
    if (const char *e = std::getenv("HAMMINGDIST_STREAM_SPLITS")) {
      ends.clear();
      for (const char *q = e; *q && ends.size() < 3;) {
        char *endp = nullptr;
        const double f = std::strtod(q, &endp);
        if (endp == q) break;
        if (f > 0 && f < 1 && (ends.empty() || f > ends.back())) ends.push_back(f);
        q = *endp == ',' ? endp + 1 : endp;
      }
    }
    static const char *const kUp[] = {"part 1 uploaded", "part 2 uploaded", "part 3 uploaded",
                                      "part 4 uploaded"};
    static const char *const kParsed[] = {"part 1 parsed", "part 2 parsed", "part 3 parsed",
                                          "part 4 parsed"};
    static const char *const kPacked[] = {"part 1 deduplicated + packed", "part 2 deduplicated + packed",
                                          "part 3 deduplicated + packed", "part 4 deduplicated + packed"};
    struct Band {
      uint64_t row_lo = 0, row_hi = 0;  // rows whose entries it writes
      cudaEvent_t done = nullptr;
      hd_alignment view;
      hd::PairLaunchPlan plan;
    };
    std::vector<std::unique_ptr<Band>> bands;
    hd::Records all;
    DevBuf uniq, iota, d_lt, keep_planes;
    std::vector<uint64_t> seq;
    std::unique_ptr<hd_alignment> owner;
    // each part's new records only, while that resolves them (else the full
    // dedupe of the prefix, from then on)
    hd::IncDedupe inc;
    bool inc_ok = true;
    if (const char *e = std::getenv("HAMMINGDIST_STREAM_DEDUPE"))  // "full": the full path only
      inc_ok = std::string(e) != "full";
    // waits for every stream the call uses before any of the above is freed
    struct Sync {
      hd_ctx *c;
      std::vector<cudaEvent_t> ev;
      cudaEvent_t make() {
        cudaEvent_t e;
        HD_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        ev.push_back(e);
        return e;
      }
      ~Sync() {
        for (cudaStream_t s : {c->stream, c->side, c->up}) cudaStreamSynchronize(s);
        for (cudaEvent_t e : ev) cudaEventDestroy(e);
      }
    } sync{ctx, {}};
    auto fallback = [&] {  // the whole matrix after the whole file
      HD_CUDA(cudaStreamSynchronize(ctx->side));
      read_all();
      whole();
      hd::trace_end(ctx);
    };
    uint64_t L = 0, words = 0, R_max = 0, K = 0, B_prev = 0, tiles = 0;
    uint32_t T = 0, t_done = 0;
    bool use_mma = false;  // tensor-core engine: 128-row tiles
    // SMs left to the next part's ingest while a band runs
    // (HAMMINGDIST_STREAM_FREE_SMS, default 16)
    int free_sms = 16;
    if (const char *e = std::getenv("HAMMINGDIST_STREAM_FREE_SMS"))
      free_sms = std::min(std::max(0, std::atoi(e)), ctx->sm_count - 1);
    hd::TileConfig cfg;
    uint4 *g0 = nullptr;
    // tile rows [t_lo, t_hi) of the first `rows` unique rows on stream s
    auto launch = [&](uint32_t t_lo, uint32_t t_hi, uint64_t rows, cudaStream_t s, int sm_limit,
                      cudaEvent_t after) {
      auto b = std::make_unique<Band>();
      b->view.base = owner.get();
      b->view.n_rows = rows;
      b->view.length = L;
      b->view.words = words;
      b->view.device = ctx->device;
      b->row_lo = (uint64_t)t_lo * T;
      b->row_hi = std::min<uint64_t>((uint64_t)t_hi * T, rows);
      if (after) HD_CUDA(cudaStreamWaitEvent(s, after, 0));
      const std::string rows_text =
          "rows " + std::to_string(b->row_lo) + "-" + std::to_string(b->row_hi);
      hd::trace_at(ctx, rows_text + " start", s);
      ctx->last_pair_tiles = 0;
      // the tensor-core engine (its operand rows were expanded after the
      // pack, on ctx->stream), else the bit-plane engine
      if (!use_mma || !hd::pairwise_mma(ctx, &b->view, dtype_bytes, md, d_lt.p, 0, t_lo, t_hi, s,
                                        sm_limit)) {
        std::vector<hd::PairJobSpec> specs(1);
        specs[0].aln = &b->view;
        specs[0].dtype = dtype_bytes;
        specs[0].max_dist = md;
        specs[0].d_out = d_lt.p;
        specs[0].cfg = cfg;
        specs[0].tile_lo = t_lo;
        specs[0].tile_hi = t_hi;
        hd::prepare_pairwise_jobs(ctx, specs, s, &b->plan, sm_limit);
        hd::launch_pairwise_plan(ctx, b->plan, s);
      }
      tiles += ctx->last_pair_tiles;
      hd::trace_at(ctx, rows_text + " done", s);
      b->done = sync.make();
      HD_CUDA(cudaEventRecord(b->done, s));
      bands.push_back(std::move(b));
    };
    for (int c = 0;; ++c) {
      uint64_t B = n;
      if (c < (int)ends.size()) {
        B = header_at(std::max<uint64_t>(B_prev + 1, (uint64_t)(ends[c] * (double)n)));
        if (!B) {
          // no header in the rest (or a read error): the first part is the
          // whole file; later, the rest is the last part
          if (c == 0) return fallback();
          B = n;
        }
      }
      const bool last = B == n;
      if (last) read_all();  // throws on a read or copy error
      else if (!reader->stream_wait_bytes(ctx->stream, B)) read_all();
      hd::trace_mark(ctx, kUp[c]);
      // parse_fasta reads 16-byte vectors from a 16-byte aligned start: a
      // later part is parsed from B_prev rounded down. The bytes before B_prev
      // (up to 15) end the previous part; the records they hold or end (the
      // empty record before the first header, and any short record whose
      // header starts there) are the previous part's, and the parse leaves
      // them out.
      const uint64_t C = B_prev & ~15ull;
      hd::trace_host(ctx, "part " + std::to_string(c + 1) + " on the device");
      hd::Records rec = hd::parse_fasta(ctx, dev + C, B - C, 0, B_prev - C);
      hd::trace_host(ctx, "part " + std::to_string(c + 1) + " parsed");
      // multi-line records, or a first part the whole path reports on
      if (rec.gathered.p || (c == 0 && (rec.n == 0 || rec.len0 == 0 || !rec.all_equal)))
        return fallback();
      if (c == 0) all = std::move(rec);
      else all = hd::concat_records(ctx, all, rec, C, B);
      if (!all.all_equal) fail(HD_ERR_LENGTH, kMsgLength);
      hd::trace_mark(ctx, kParsed[c]);
      if (c == 0) {
        L = all.len0;
        words = words_for(L);
        // rows that can still come: a record of L sites takes at least L + 2
        // bytes (">\n" and the sites; the last one may lack its '\n')
        R_max = all.n + (n - B) / (L + 2) + 1;
        // the buffers are sized for R_max rows: the output for R_max (R_max -
        // 1) / 2 entries. Where that does not fit in half the free device
        // memory (short records, many of them duplicates), the plain order
        // runs: it sizes them for the unique rows
        {
          size_t free_b = 0, total_b = 0;
          HD_CUDA(cudaMemGetInfo(&free_b, &total_b));
          const double need = (double)(R_max < 2 ? 1 : tri(R_max)) * dtype_bytes +
                              2.0 * (double)R_max * (double)words * 16.0 +
                              (double)R_max * (double)words * (double)hd::kMmaOperandBytesPerWord;
          if (need > 0.5 * (double)free_b) return fallback();
        }
        owner = std::make_unique<hd_alignment>();
        owner->ctx = ctx;
        owner->device = ctx->device;
        owner->length = L;
        owner->words = words;
        owner->rule = HD_RULE_AND;
        owner->groups = 1;
        owner->planes = 4;
        owner->plane_buf[0] = DevBuf(R_max * words * 16, ctx->stream);
        g0 = owner->plane_buf[0].as<uint4>();
        // a second copy of the rows, written by the same packs, stays with
        // the file's records for the reference distances of the same file
        // (fasta_reference_distances after from_fasta)
        keep_planes = DevBuf(R_max * words * 16, ctx->stream);
        d_lt = DevBuf((R_max < 2 ? 1 : tri(R_max)) * dtype_bytes, ctx->stream);
        hd::trace_host(ctx, "row buffers allocated");
        if (!remove_duplicates) {
          std::vector<uint64_t> h(R_max);
          for (uint64_t i = 0; i < R_max; ++i) h[i] = i;
          iota = DevBuf(R_max * 8, ctx->stream);
          HD_CUDA(cudaMemcpyAsync(iota.p, h.data(), R_max * 8, cudaMemcpyHostToDevice, ctx->stream));
          HD_CUDA(cudaStreamSynchronize(ctx->stream));
        }
      }
      uint64_t Kc = all.n;
      const uint64_t *rows = iota.as<uint64_t>();
      if (remove_duplicates) {
        if (c == 0) inc.init(ctx, R_max);
        const bool added = inc_ok && inc.add(ctx, all);
        hd::trace_host(ctx, "part " + std::to_string(c + 1) + " deduplicated");
        if (added) {
          Kc = inc.n_unique;
          rows = inc.unique_rec.as<uint64_t>();
        } else {
          inc_ok = false;
          uniq = hd::dedupe(ctx, all, &Kc, seq);
          rows = uniq.as<uint64_t>();
        }
      }
      if (Kc > R_max || Kc < K) fail(HD_ERR_CUDA, "streamed ingest: inconsistent row counts");
      if (c == 0) {
        cfg = hd::tile_config_for(ctx, Kc * (n / std::max<uint64_t>(B, 1)), L, dtype_bytes);
        T = (uint32_t)cfg.tile;
        owner->n_rows = R_max;  // the eligibility test looks at the shape only
        use_mma = hd::mma_eligible(owner.get());
        owner->n_rows = 0;
        if (use_mma) {
          // bands count tile rows of 128; a band the tensor-core engine
          // declines (too few items) runs on the bit-plane engine with the
          // same 128-row tiles
          T = hd::kTile;
          cfg.tile = (int)hd::kTile;
          if (!hd::tile_config_valid(cfg.tile, cfg.stages)) cfg.stages = 3;
        }
      }
      hd::pack_rows_and(ctx, all, rows + K, Kc - K, L, words, g0 + K * words,
                        keep_planes.as<uint4>() + K * words);
      hd::trace_host(ctx, "part " + std::to_string(c + 1) + " packing queued");
      // the new rows' tensor-core operand, before the launches of any stream read it
      if (use_mma && Kc >= 2 && !hd::ensure_operand(ctx, owner.get(), Kc, ctx->stream, R_max)) {
        use_mma = false;
        T = (uint32_t)cfg.tile;
        if (t_done) fail(HD_ERR_OOM, "no memory for the tensor-core operand of a streamed call");
      }
      hd::trace_host(ctx, "part " + std::to_string(c + 1) + " operand queued");
      hd::trace_mark(ctx, kPacked[c]);
      K = Kc;
      if (!last) {
        const uint32_t t_end = (uint32_t)(K / T);
        if (t_end > t_done) {
          cudaEvent_t packed = sync.make();
          HD_CUDA(cudaEventRecord(packed, ctx->stream));
          launch(t_done, t_end, K, ctx->side, std::max(1, ctx->sm_count - free_sms), packed);
          t_done = t_end;
        }
        hd::trace_host(ctx, "part " + std::to_string(c + 1) + " queued");
        B_prev = B;
        continue;
      }
      const uint32_t t_end = K >= 2 ? (uint32_t)hd::ceil_div(K, T) : t_done;
      if (t_end > t_done) {
        const uint32_t t_split =
            std::max(t_done + 1, (uint32_t)std::ceil(0.9 * (double)t_end));
        // one after the other on the context's stream: launched on two
        // streams at once, the block scheduler sometimes gave the SMs to the
        // second launch's CTAs first, and the first launch (whose CTAs walk
        // fixed item lists) then ended up to 0.8 ms later
        launch(t_done, t_split < t_end ? t_split : t_end, K, ctx->stream, 0, nullptr);
        if (t_split < t_end) launch(t_split, t_end, K, ctx->stream, 0, nullptr);
      }
      break;
    }
    hd::trace_host(ctx, "launches queued");
    owner->n_rows = K;
    owner->n_input = all.n;
    // each record's row: on the device (the incremental dedupe's rowid,
    // copied to the host once the launches are done), or from the full dedupe
    // on the host
    const bool inc_rows = remove_duplicates && inc_ok;
    if (remove_duplicates) {
      owner->d_seqidx = DevBuf(all.n * 8, ctx->stream);
      if (inc_rows) {
        HD_CUDA(cudaMemcpyAsync(owner->d_seqidx.p, inc.rowid.p, all.n * 8, cudaMemcpyDeviceToDevice,
                                ctx->stream));
      } else {
        owner->seqidx = std::move(seq);
        HD_CUDA(cudaMemcpyAsync(owner->d_seqidx.p, owner->seqidx.data(), all.n * 8,
                                cudaMemcpyHostToDevice, ctx->stream));
      }
    }
    ctx->last_pair_tiles = tiles;
    // the second copy of the rows stays with the file's records, with each
    // record's row
    if (K && keep_planes.p) {
      auto keep = std::make_shared<hd_alignment>();
      keep->ctx = ctx;
      keep->device = ctx->device;
      keep->length = L;
      keep->words = words;
      keep->n_rows = K;
      keep->n_input = all.n;
      keep->plane_buf[0] = std::move(keep_planes);
      if (remove_duplicates) {
        all.row_of = DevBuf(all.n * 8, ctx->stream);
        if (inc_rows)
          HD_CUDA(cudaMemcpyAsync(all.row_of.p, inc.rowid.p, all.n * 8, cudaMemcpyDeviceToDevice,
                                  ctx->stream));
        else
          hd::upload_table(ctx, all.row_of.p, owner->seqidx.data(), all.n * 8, ctx->stream);
      }
      all.rows = std::move(keep);
    }
    // each finished range of rows is copied to the host on the upload stream
    // once its launch is done, while the later ones compute
    hd::trace_host(ctx, "rows kept");
    const uint64_t entries = K < 2 ? 0 : tri(K);
    void *host = out_fn(user, 0, K, entries);
    if (!host && entries) fail(HD_ERR_ARG, "output callback returned no buffer");
    void *mirror = entries ? out_fn(user, HD_OUTPUT_MIRROR, K, entries) : nullptr;
    hd::trace_host(ctx, "outputs");
    if (entries) {
      prefault_host(host, entries * dtype_bytes);  // while the kernels run
      if (mirror) prefault_host(mirror, entries * dtype_bytes);
      hd::trace_host(ctx, "outputs touched");
      for (const auto &b : bands) {
        const uint64_t e0 = tri(b->row_lo), e1 = tri(b->row_hi);
        if (e1 <= e0) continue;
        HD_CUDA(cudaStreamWaitEvent(ctx->up, b->done, 0));
        for (void *dst : {host, mirror})
          if (dst)
            HD_CUDA(cudaMemcpyAsync(static_cast<uint8_t *>(dst) + e0 * dtype_bytes,
                                    d_lt.as<uint8_t>() + e0 * dtype_bytes, (e1 - e0) * dtype_bytes,
                                    cudaMemcpyDeviceToHost, ctx->up));
        hd::trace_at(ctx, "rows " + std::to_string(b->row_lo) + "-" + std::to_string(b->row_hi) +
                              " copied",
                     ctx->up);
      }
      hd::trace_host(ctx, "copies queued");
    }
    if (ctx->trace.on) {
      // the context's stream waits for the distance launches, then for the
      // copies, so that the trace shows the two apart
      for (cudaStream_t s : {ctx->side}) {
        cudaEvent_t e = sync.make();
        HD_CUDA(cudaEventRecord(e, s));
        HD_CUDA(cudaStreamWaitEvent(ctx->stream, e, 0));
      }
      hd::trace_mark(ctx, "distances");
      cudaEvent_t e = sync.make();
      HD_CUDA(cudaEventRecord(e, ctx->up));
      HD_CUDA(cudaStreamWaitEvent(ctx->stream, e, 0));
      hd::trace_mark(ctx, "rest of the copy to host");
    }
    for (cudaStream_t s : {ctx->side, ctx->up, ctx->stream})
      HD_CUDA(cudaStreamSynchronize(s));
    check_status(ctx);
    if (inc_rows) inc.rows(ctx, owner->seqidx);
    // the file and its records stay for later calls on the same file
    ctx->parsed = std::make_shared<hd::Records>(std::move(all));
    ctx->parsed_tag = tag;
    ctx->parsed_limit = 0;
    *aln_out = owner.release();
    hd::trace_end(ctx);
  });
}

int hd_alignment_from_sequences(hd_ctx *ctx, const char *bytes, const uint64_t *offsets, uint64_t n,
                                int include_x, int semantics, hd_alignment **out) {
  if (!ctx || !out || (n && !offsets)) return HD_ERR_ARG;
  *out = nullptr;
  return guard(ctx, [&] {
    const uint64_t nbytes = n ? offsets[n] - offsets[0] : 0;
    const uint8_t *d = stage_input(ctx, bytes ? bytes + (n ? offsets[0] : 0) : bytes, nbytes, 0);
    hd::Records rec = hd::records_from_offsets(ctx, d, offsets, n);
    *out = build_alignment(ctx, rec, 0, include_x, semantics);
  });
}

int hd_alignment_info(const hd_alignment *aln, uint64_t *n_rows, uint64_t *length,
                      uint64_t *n_input, int *rule) {
  if (!aln) return HD_ERR_ARG;
  if (n_rows) *n_rows = aln->n_rows;
  if (length) *length = aln->length;
  if (n_input) *n_input = aln->n_input;
  if (rule) *rule = aln->rule;
  return HD_OK;
}

int hd_alignment_sequence_indices(const hd_alignment *aln, uint64_t *out) {
  if (!aln || !out) return HD_ERR_ARG;
  if (aln->seqidx.empty())
    for (uint64_t k = 0; k < aln->n_input; ++k) out[k] = k;
  else
    std::memcpy(out, aln->seqidx.data(), aln->seqidx.size() * 8);
  return HD_OK;
}

void hd_alignment_free(hd_alignment *aln) { delete aln; }

int hd_pairwise_lt(hd_ctx *ctx, const hd_alignment *aln, int dtype_bytes, int64_t max_distance,
                   void *out, int out_on_device) {
  if (!ctx || !aln) return HD_ERR_ARG;
  return guard(ctx, [&] {
    check_dtype(dtype_bytes);
    const uint32_t md = clamp_max(max_distance, dtype_bytes);
    const uint64_t n = aln->n_rows, entries = n < 2 ? 0 : tri(n);
    ctx->last_pair_ms = 0;
    ctx->last_pair_tiles = 0;
    HD_CUDA(cudaMemsetAsync(hd::mma_mac_counter(ctx), 0, 8, ctx->stream));
    if (!entries) return;
    if (!out) fail(HD_ERR_ARG, "null output");
    DevBuf tmp;
    void *d_out = out;
    if (!out_on_device) {
      tmp = DevBuf(entries * dtype_bytes, ctx->stream);
      d_out = tmp.p;
    }
    const uint32_t nb = (uint32_t)hd::ceil_div(n, hd::kTile);
    hd::trace_begin(ctx, "hd_pairwise_lt");
    // the tensor-core engine's operand and the launch plan (item lists,
    // tensor maps, job tables) first, so that the timing below is the
    // distance kernel's alone
    if (!aln->base && hd::mma_eligible(aln) && hd::ensure_operand(ctx, aln, n, ctx->stream))
      hd::trace_mark(ctx, "FP4 operand");
    hd::PairLaunchPlan plan;
    hd::plan_pairwise_tiles(ctx, aln, dtype_bytes, md, d_out, 0, 0, nb, &plan);
    HD_CUDA(cudaEventRecord(ctx->ev_start, ctx->stream));
    hd::launch_pairwise_plan(ctx, plan, ctx->stream);
    HD_CUDA(cudaEventRecord(ctx->ev_stop, ctx->stream));
    hd::trace_mark(ctx, "pairwise");
    if (!out_on_device) {
      prefault_host(out, entries * dtype_bytes);  // while the kernel runs
      HD_CUDA(cudaMemcpyAsync(out, d_out, entries * dtype_bytes, cudaMemcpyDeviceToHost, ctx->stream));
      hd::trace_mark(ctx, "copy to host");
    }
    HD_CUDA(cudaStreamSynchronize(ctx->stream));
    hd::trace_end(ctx);
    float ms = 0;
    HD_CUDA(cudaEventElapsedTime(&ms, ctx->ev_start, ctx->ev_stop));
    ctx->last_pair_ms = ms;
    check_status(ctx);
  });
}

int hd_pairwise_lt_to_file(hd_ctx *ctx, const hd_alignment *aln, int64_t max_distance,
                           const char *path) {
  if (!ctx || !aln || !path) return HD_ERR_ARG;
  return guard(ctx, [&] {
    // distances_cuda_to_lower_triangular: uint16, max above 65535 -> 65535
    const uint32_t md = clamp_max(max_distance, 2);
    stream_lt_text(ctx, aln->n_rows, 2, path, hd::kTile,
                   [&](uint64_t r0, uint64_t r1, void *d_lt) {
                     hd::pairwise_tiles(ctx, aln, 2, md, d_lt, tri(std::max<uint64_t>(r0, 1)),
                                        (uint32_t)(r0 / hd::kTile),
                                        (uint32_t)hd::ceil_div(r1, hd::kTile));
                   });
  });
}

int hd_write_full_matrix(hd_ctx *ctx, const void *lt, uint64_t entries, uint64_t nsamples,
                         int dtype_bytes, const char *path) {
  if (!ctx || !path || (!lt && entries)) return HD_ERR_ARG;
  return guard(ctx, [&] {
    check_dtype(dtype_bytes);
    OutFile f(path);
    if (!nsamples) return;
    DevBuf d_lt((entries ? entries : 1) * dtype_bytes, ctx->stream);
    if (entries)
      HD_CUDA(cudaMemcpyAsync(d_lt.p, lt, entries * dtype_bytes, cudaMemcpyHostToDevice,
                              ctx->stream));
    // rows per chunk: text of at most kTextChunkBytes (at least one row)
    const uint64_t row_bound = hd::full_text_bound(nsamples, 0, 1, dtype_bytes);
    const uint64_t rows_per = std::max<uint64_t>(1, kTextChunkBytes / row_bound);
    const uint64_t max_text = hd::full_text_bound(nsamples, 0, std::min(rows_per, nsamples),
                                                  dtype_bytes);
    DevBuf d_text(max_text + 16, ctx->stream);
    PinnedPair pin(max_text + 16);
    int pending = -1;
    uint64_t pending_bytes = 0;
    for (uint64_t r0 = 0, k = 0; r0 < nsamples; r0 += rows_per, ++k) {
      const uint64_t r1 = std::min(nsamples, r0 + rows_per);
      const uint64_t nb =
          hd::format_full_rows(ctx, d_lt.p, entries, dtype_bytes, nsamples, r0, r1, d_text.as<char>());
      // write the previous chunk while this one copies
      if (pending >= 0) {
        HD_CUDA(cudaEventSynchronize(pin.ev[pending]));
        f.write(pin.buf[pending], pending_bytes);
      }
      const int slot = (int)(k & 1);
      if (nb)
        HD_CUDA(cudaMemcpyAsync(pin.buf[slot], d_text.p, nb, cudaMemcpyDeviceToHost, ctx->stream));
      HD_CUDA(cudaEventRecord(pin.ev[slot], ctx->stream));
      pending = slot;
      pending_bytes = nb;
    }
    if (pending >= 0) {
      HD_CUDA(cudaEventSynchronize(pin.ev[pending]));
      f.write(pin.buf[pending], pending_bytes);
    }
  });
}

namespace {
// Copies parsed values to the caller's buffer from out_fn.
void deliver(hd_ctx *ctx, const hd::ParsedValues &pv, int dtype_bytes, hd_output_fn out_fn,
             void *user) {
  void *host = out_fn(user, 0, pv.nsamples, pv.entries);
  if (!host && pv.entries) fail(HD_ERR_ARG, "output callback returned no buffer");
  if (!pv.entries) return;
  const uint64_t bytes = pv.entries * dtype_bytes;
  prefault_host(host, bytes);
  HD_CUDA(cudaMemcpyAsync(host, pv.values.p, bytes, cudaMemcpyDeviceToHost, ctx->stream));
  HD_CUDA(cudaStreamSynchronize(ctx->stream));
}
}  // namespace

int hd_read_lower_triangular(hd_ctx *ctx, const char *path, int dtype_bytes, hd_output_fn out_fn,
                             void *user, uint64_t *entries, uint64_t *nsamples, int *parse_error) {
  if (!ctx || !path || !out_fn || (dtype_bytes != 1 && dtype_bytes != 2)) return HD_ERR_ARG;
  if (parse_error) *parse_error = 0;
  return guard(ctx, [&] {
    uint64_t nbytes = 0;
    const uint8_t *d = stage_file(ctx, path, &nbytes);
    hd::ParsedValues pv = hd::read_lower_triangular_device(ctx, d, nbytes, dtype_bytes);
    if (entries) *entries = pv.entries;
    if (nsamples) *nsamples = pv.nsamples;
    if (parse_error) *parse_error = pv.error;
    if (pv.error) fail(HD_ERR_PARSE, "stoi");
    deliver(ctx, pv, dtype_bytes, out_fn, user);
  });
}

int hd_read_csv(hd_ctx *ctx, const char *path, hd_output_fn out_fn, void *user, uint64_t *entries,
                uint64_t *nsamples, int *parse_error) {
  if (!ctx || !path || !out_fn) return HD_ERR_ARG;
  if (parse_error) *parse_error = 0;
  return guard(ctx, [&] {
    uint64_t nbytes = 0;
    const uint8_t *d = stage_file(ctx, path, &nbytes);
    hd::ParsedValues pv = hd::read_csv_device(ctx, d, nbytes);
    if (entries) *entries = pv.entries;
    if (nsamples) *nsamples = pv.nsamples;
    if (parse_error) *parse_error = pv.error;
    if (pv.error) fail(HD_ERR_PARSE, "stoi");
    deliver(ctx, pv, 1, out_fn, user);
  });
}

int hd_write_lower_triangular(hd_ctx *ctx, const void *lt, uint64_t nsamples, int dtype_bytes,
                              const char *path) {
  if (!ctx || !path || (!lt && nsamples > 1)) return HD_ERR_ARG;
  return guard(ctx, [&] {
    check_dtype(dtype_bytes);
    stream_lt_text(ctx, nsamples, dtype_bytes, path, 1, [&](uint64_t r0, uint64_t r1, void *d_lt) {
      const uint64_t e0 = tri(std::max<uint64_t>(r0, 1)), e1 = tri(r1);
      if (e1 > e0)
        HD_CUDA(cudaMemcpyAsync(d_lt, static_cast<const char *>(lt) + e0 * dtype_bytes,
                                (e1 - e0) * dtype_bytes, cudaMemcpyHostToDevice, ctx->stream));
    });
  });
}

int hd_write_sparse(hd_ctx *ctx, const void *lt, uint64_t nsamples, int dtype_bytes,
                    int64_t threshold, const char *path, uint64_t *n_lines) {
  if (!ctx || !path || (!lt && nsamples > 1)) return HD_ERR_ARG;
  return guard(ctx, [&] {
    check_dtype(dtype_bytes);
    OutFile f(path);  // the reference always (re)creates the file
    uint64_t lines_total = 0;
    if (nsamples >= 2) {
      // bytes per line <= 2 * digits(n) + digits(dtype max) + 3
      uint64_t dn = 1;
      for (uint64_t v = nsamples; v >= 10; v /= 10) ++dn;
      const uint64_t per = 2 * dn + (dtype_bytes == 1 ? 3 : dtype_bytes == 2 ? 5 : 10) + 3;
      const uint64_t max_entries = std::max<uint64_t>(kTextChunkBytes / per, 1);
      auto chunks = row_chunks(nsamples, max_entries, 1);
      uint64_t max_e = 0, max_rows = 0;
      for (auto &c : chunks) {
        max_e = std::max(max_e, tri(c.second) - tri(std::max<uint64_t>(c.first, 1)));
        max_rows = std::max(max_rows, c.second - c.first);
      }
      DevBuf d_lt((max_e + 1) * dtype_bytes, ctx->stream), d_text(max_e * per + 16, ctx->stream);
      DevBuf rb((max_rows + 1) * 8, ctx->stream), rl((max_rows + 1) * 8, ctx->stream),
          tot(8, ctx->stream);
      PinnedPair pin(max_e * per + 16);
      int pending = -1;
      uint64_t pending_bytes = 0;
      for (size_t k = 0; k < chunks.size(); ++k) {
        const uint64_t r0 = std::max<uint64_t>(chunks[k].first, 1), r1 = chunks[k].second;
        if (r1 <= r0) continue;
        const uint64_t e0 = tri(r0), e1 = tri(r1);
        HD_CUDA(cudaMemcpyAsync(d_lt.p, static_cast<const char *>(lt) + e0 * dtype_bytes,
                                (e1 - e0) * dtype_bytes, cudaMemcpyHostToDevice, ctx->stream));
        hd::sparse_row_sizes(ctx, d_lt.p, dtype_bytes, e0, r0, r1, threshold, rb.as<uint64_t>(),
                             rl.as<uint64_t>());
        if (pending >= 0) {
          HD_CUDA(cudaEventSynchronize(pin.ev[pending]));
          f.write(pin.buf[pending], pending_bytes);
          pending = -1;
        }
        uint64_t lines = 0;
        hd::scan_exclusive<uint64_t>(ctx, rl.as<uint64_t>(), rl.as<uint64_t>(), r1 - r0,
                                     tot.as<uint64_t>());
        HD_CUDA(cudaMemcpyAsync(&lines, tot.p, 8, cudaMemcpyDeviceToHost, ctx->stream));
        const uint64_t nb = hd::format_sparse_rows(ctx, d_lt.p, dtype_bytes, e0, r0, r1, threshold,
                                                   rb.as<uint64_t>(), d_text.as<char>());
        lines_total += lines;
        const int slot = (int)(k & 1);
        if (nb)
          HD_CUDA(cudaMemcpyAsync(pin.buf[slot], d_text.p, nb, cudaMemcpyDeviceToHost, ctx->stream));
        HD_CUDA(cudaEventRecord(pin.ev[slot], ctx->stream));
        pending = slot;
        pending_bytes = nb;
      }
      if (pending >= 0) {
        HD_CUDA(cudaEventSynchronize(pin.ev[pending]));
        f.write(pin.buf[pending], pending_bytes);
      }
    }
    if (n_lines) *n_lines = lines_total;
  });
}

int hd_reference_distances(hd_ctx *ctx, const char *ref, uint64_t ref_len, const char *fasta,
                           uint64_t nbytes, int include_x, uint32_t **out, uint64_t *n_out) {
  if (!ctx || !out || !n_out || (!ref && ref_len) || (!fasta && nbytes)) return HD_ERR_ARG;
  *out = nullptr;
  *n_out = 0;
  return guard(ctx, [&] {
    hd::trace_begin(ctx, "hd_reference_distances");
    const uint8_t *d = stage_input(ctx, fasta, nbytes, 0);
    hd::trace_mark(ctx, "upload");
    reference_distances_of(ctx, d, nbytes, ref, ref_len, include_x, out, n_out, false);
  });
}

int hd_reference_distances_file(hd_ctx *ctx, const char *ref, uint64_t ref_len, const char *path,
                                int include_x, uint32_t **out, uint64_t *n_out) {
  if (!ctx || !out || !n_out || (!ref && ref_len) || !path) return HD_ERR_ARG;
  *out = nullptr;
  *n_out = 0;
  return guard(ctx, [&] {
    hd::trace_begin(ctx, "hd_reference_distances_file");
    uint64_t nbytes = 0;
    const uint8_t *d = stage_file(ctx, path, &nbytes);
    hd::trace_mark(ctx, "read + upload");
    reference_distances_of(ctx, d, nbytes, ref, ref_len, include_x, out, n_out, true);
  });
}

int hd_alignment_reference_distances(hd_ctx *ctx, const hd_alignment *aln, const char *ref,
                                     uint64_t ref_len, int include_x, uint32_t *out) {
  if (!ctx || !aln || !ref || !out) return HD_ERR_ARG;
  return guard(ctx, [&] {
    if (include_x || aln->rule != HD_RULE_AND)
      fail(HD_ERR_ARG, "resident reference queries need an AND-rule alignment and include_x=False");
    if (ref_len != aln->length) fail(HD_ERR_LENGTH, kMsgLength);
    DevBuf d_ref(ref_len + 16, ctx->stream), d_rows(aln->n_rows * 4, ctx->stream);
    HD_CUDA(cudaMemcpyAsync(d_ref.p, ref, ref_len, cudaMemcpyHostToDevice, ctx->stream));
    hd::alignment_query_distances(ctx, aln, d_ref.as<uint8_t>(), d_rows.as<uint32_t>());
    std::vector<uint32_t> rows(aln->n_rows);
    HD_CUDA(cudaMemcpy(rows.data(), d_rows.p, aln->n_rows * 4, cudaMemcpyDeviceToHost));
    for (uint64_t k = 0; k < aln->n_input; ++k)
      out[k] = rows[aln->seqidx.empty() ? k : aln->seqidx[k]];
  });
}

int hd_fasta_sequence_indices(hd_ctx *ctx, const char *fasta, uint64_t nbytes, uint64_t n_limit,
                              uint64_t **out, uint64_t *n_out) {
  if (!ctx || !out || !n_out || (!fasta && nbytes)) return HD_ERR_ARG;
  *out = nullptr;
  *n_out = 0;
  return guard(ctx, [&] {
    const uint8_t *d = stage_input(ctx, fasta, nbytes, 0);
    sequence_indices_of(ctx, d, nbytes, n_limit, out, n_out, false);
  });
}

int hd_fasta_sequence_indices_file(hd_ctx *ctx, const char *path, uint64_t n_limit, uint64_t **out,
                                   uint64_t *n_out) {
  if (!ctx || !out || !n_out || !path) return HD_ERR_ARG;
  *out = nullptr;
  *n_out = 0;
  return guard(ctx, [&] {
    uint64_t nbytes = 0;
    const uint8_t *d = stage_file(ctx, path, &nbytes);
    sequence_indices_of(ctx, d, nbytes, n_limit, out, n_out, true);
  });
}

int hd_distance(hd_ctx *ctx, const char *s0, uint64_t l0, const char *s1, uint64_t l1,
                int include_x, uint32_t *out) {
  if (!ctx || !out || (!s0 && l0) || (!s1 && l1)) return HD_ERR_ARG;
  return guard(ctx, [&] {
    if (l0 != l1) fail(HD_ERR_LENGTH, kMsgLength);
    *out = 0;
    if (!l0) return;
    DevBuf d(2 * l0 + 32, ctx->stream), d_out(4, ctx->stream);
    HD_CUDA(cudaMemcpyAsync(d.p, s0, l0, cudaMemcpyHostToDevice, ctx->stream));
    HD_CUDA(cudaMemcpyAsync(d.as<char>() + l0 + 16, s1, l1, cudaMemcpyHostToDevice, ctx->stream));
    uint64_t offs[2] = {0, l1};
    hd::Records rec = hd::records_from_offsets(ctx, d.as<uint8_t>() + l0 + 16, offs, 1);
    hd::reference_distances_device(ctx, rec, d.as<uint8_t>(), include_x, d_out.as<uint32_t>());
    HD_CUDA(cudaMemcpyAsync(out, d_out.p, 4, cudaMemcpyDeviceToHost, ctx->stream));
    HD_CUDA(cudaStreamSynchronize(ctx->stream));
  });
}

int hd_measure_mma_peak(hd_ctx *ctx, double *fp4_flop_per_s) {
  if (!ctx || !fp4_flop_per_s) return HD_ERR_ARG;
  return guard(ctx, [&] {
    *fp4_flop_per_s = hd::measure_mma_peak(ctx);
    check_status(ctx);
  });
}

int hd_measure_int_peaks(hd_ctx *ctx, double *lop3_per_s, double *popc_per_s,
                         double *mix_pair_sites_per_s) {
  if (!ctx) return HD_ERR_ARG;
  return guard(ctx, [&] { hd::measure_int_peaks(ctx, lop3_per_s, popc_per_s, mix_pair_sites_per_s); });
}

int hd_last_pairwise_timing(const hd_ctx *ctx, double *ms, uint64_t *tiles) {
  if (!ctx) return HD_ERR_ARG;
  if (ms) *ms = ctx->last_pair_ms;
  if (tiles) *tiles = ctx->last_pair_tiles;
  return HD_OK;
}

int hd_last_pairwise_work(const hd_ctx *ctx, double *mma_macs) {
  if (!ctx || !mma_macs) return HD_ERR_ARG;
  unsigned long long m = 0;
  if (cudaMemcpy(&m, hd::mma_mac_counter(ctx), 8, cudaMemcpyDeviceToHost) != cudaSuccess)
    return HD_ERR_CUDA;
  *mma_macs = (double)m;
  return HD_OK;
}

// ------------------------------------------------------------------ batches
}  // extern "C"

struct hd_batch {
  hd_ctx *ctx = nullptr;
  struct Job {
    const hd_alignment *aln;
    int dtype;
    uint32_t max_dist;
    void *out;
    int out_on_device;
  };
  std::vector<Job> jobs;
  bool built = false;
  std::vector<DevBuf> staging;  // device outputs of host-output jobs
  hd::PairLaunchPlan plan;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  double last_ms = 0;
  uint64_t tiles = 0;
  void reset() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    exec = nullptr;
    graph = nullptr;
    plan = hd::PairLaunchPlan();
    staging.clear();
    built = false;
  }
  ~hd_batch() {
    if (ctx) cudaSetDevice(ctx->device);
    reset();
  }
};

extern "C" {

int hd_batch_create(hd_ctx *ctx, hd_batch **out) {
  if (!ctx || !out) return HD_ERR_ARG;
  *out = new hd_batch();
  (*out)->ctx = ctx;
  return HD_OK;
}

int hd_batch_add(hd_batch *b, const hd_alignment *aln, int dtype_bytes, int64_t max_distance,
                 void *out, int out_on_device) {
  if (!b || !aln) return HD_ERR_ARG;
  return guard(b->ctx, [&] {
    check_dtype(dtype_bytes);
    if (!out && aln->n_rows >= 2) fail(HD_ERR_ARG, "null output");
    b->jobs.push_back({aln, dtype_bytes, clamp_max(max_distance, dtype_bytes), out, out_on_device});
    b->reset();  // the graph is rebuilt on the next run
  });
}

int hd_batch_run(hd_batch *b) {
  if (!b) return HD_ERR_ARG;
  hd_ctx *ctx = b->ctx;
  return guard(ctx, [&] {
    cudaStream_t st = ctx->stream;
    if (!b->built) {
      std::vector<hd::PairJobSpec> specs;
      b->staging.clear();
      b->tiles = 0;
      for (auto &j : b->jobs) {
        const uint64_t n = j.aln->n_rows;
        if (n < 2) continue;
        hd::PairJobSpec s;
        s.aln = j.aln;
        s.dtype = j.dtype;
        s.max_dist = j.max_dist;
        if (j.out_on_device) {
          s.d_out = j.out;
        } else {
          b->staging.emplace_back(tri(n) * j.dtype, st);
          s.d_out = b->staging.back().p;
        }
        s.cfg = hd::tile_config_for(ctx, n, j.aln->length, j.dtype);
        s.tile_lo = 0;
        s.tile_hi = (uint32_t)hd::ceil_div(n, s.cfg.tile);
        specs.push_back(s);
      }
      b->plan = hd::PairLaunchPlan();
      hd::prepare_pairwise_jobs(ctx, specs, st, &b->plan);
      HD_CUDA(cudaStreamSynchronize(st));
      for (auto &L : b->plan.launches) b->tiles += L.tiles;
      // capture the counter resets + persistent launches once
      const uint64_t launches0 = ctx->launches;
      HD_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
      hd::launch_pairwise_plan(ctx, b->plan, st);
      HD_CUDA(cudaStreamEndCapture(st, &b->graph));
      ctx->launches = launches0;  // counted when the graph runs
      HD_CUDA(cudaGraphInstantiate(&b->exec, b->graph, 0));
      b->built = true;
    }
    HD_CUDA(cudaEventRecord(ctx->ev_start, st));
    HD_CUDA(cudaGraphLaunch(b->exec, st));
    ctx->launches += b->plan.launches.size();
    size_t k = 0;
    for (auto &j : b->jobs) {
      if (j.aln->n_rows < 2 || j.out_on_device) continue;
      HD_CUDA(cudaMemcpyAsync(j.out, b->staging[k].p, tri(j.aln->n_rows) * j.dtype,
                              cudaMemcpyDeviceToHost, st));
      ++k;
    }
    HD_CUDA(cudaEventRecord(ctx->ev_stop, st));
    HD_CUDA(cudaStreamSynchronize(st));
    float ms = 0;
    HD_CUDA(cudaEventElapsedTime(&ms, ctx->ev_start, ctx->ev_stop));
    b->last_ms = ms;
    check_status(ctx);
  });
}

int hd_batch_timing(const hd_batch *b, double *ms, uint64_t *launches, uint64_t *tiles) {
  if (!b) return HD_ERR_ARG;
  if (ms) *ms = b->last_ms;
  if (launches) *launches = b->plan.launches.size();
  if (tiles) *tiles = b->tiles;
  return HD_OK;
}

void hd_batch_free(hd_batch *b) { delete b; }

}  // extern "C"

namespace {

// Runs job(worker ctx, i) for i in [0, count) on up to max_workers worker
// contexts in parallel; stops at the first error and reports it (with the
// input index) as the context's error. Worker kernel launches are added to
// the parent's count.
template <class Job>
void run_on_workers(hd_ctx *ctx, uint64_t count, size_t max_workers, Job &&job) {
  const size_t nw = (size_t)std::min<uint64_t>(count, max_workers);
  while (ctx->workers.size() < nw) {
    hd_ctx *w = nullptr;
    int rc = hd_ctx_create(ctx->device, &w);
    if (rc != HD_OK) fail(rc, "could not create a worker context");
    ctx->workers.push_back(w);
  }
  std::vector<uint64_t> launches0;
  for (hd_ctx *w : ctx->workers) {
    w->tune = ctx->tune;
    launches0.push_back(w->launches);
  }
  std::atomic<uint64_t> next{0};
  std::atomic<int> first_rc{HD_OK};
  std::string first_msg;
  std::mutex mu;
  std::vector<std::thread> th;
  for (size_t t = 0; t < nw; ++t) {
    th.emplace_back([&, t] {
      hd_ctx *w = ctx->workers[t];
      for (uint64_t i = next++; i < count && first_rc.load() == HD_OK; i = next++) {
        int rc = job(w, i);
        if (rc != HD_OK) {
          std::lock_guard<std::mutex> lk(mu);
          if (first_rc.load() == HD_OK) {
            first_rc = rc;
            first_msg = std::string(hd_last_error(w)) + " (input " + std::to_string(i) + ")";
          }
        }
      }
    });
  }
  for (auto &x : th) x.join();
  for (size_t t = 0; t < ctx->workers.size() && t < launches0.size(); ++t)
    ctx->launches += ctx->workers[t]->launches - launches0[t];
  if (first_rc.load() != HD_OK) fail(first_rc.load(), first_msg);
}

// Reads `path` (n bytes) into dst.
int read_file_into(hd_ctx *w, const char *path, char *dst, uint64_t n) {
  return guard(w, [&] {
    int fd = ::open(path, O_RDONLY);
    if (fd < 0) fail(HD_ERR_IO, std::string("Error: Failed to open file '") + path + "'");
    uint64_t off = 0;
    while (off < n) {
      ssize_t r = ::pread(fd, dst + off, (size_t)std::min<uint64_t>(n - off, 1ull << 30), (off_t)off);
      if (r <= 0) {
        ::close(fd);
        fail(HD_ERR_IO, std::string("Error: Failed to open file '") + path + "'");
      }
      off += (uint64_t)r;
    }
    ::close(fd);
  });
}

}  // namespace

extern "C" {

int hd_alignments_from_fasta_many(hd_ctx *ctx, uint64_t count, const char *const *fasta,
                                  const uint64_t *nbytes, int remove_duplicates,
                                  uint64_t n_limit, int include_x, int semantics,
                                  hd_alignment **out) {
  if (!ctx || !out || (count && (!fasta || !nbytes))) return HD_ERR_ARG;
  for (uint64_t i = 0; i < count; ++i) out[i] = nullptr;
  int rc = guard(ctx, [&] {
    run_on_workers(ctx, count, 8, [&](hd_ctx *w, uint64_t i) {
      return hd_alignment_from_fasta(w, fasta[i], nbytes[i], 0, remove_duplicates, n_limit,
                                     include_x, semantics, &out[i]);
    });
  });
  if (rc != HD_OK)
    for (uint64_t i = 0; i < count; ++i) {
      hd_alignment_free(out[i]);
      out[i] = nullptr;
    }
  return rc;
}

int hd_alignments_from_fasta_files(hd_ctx *ctx, uint64_t count, const char *const *paths,
                                   int remove_duplicates, uint64_t n_limit, int include_x,
                                   int semantics, hd_alignment **out) {
  if (!ctx || !out || (count && !paths)) return HD_ERR_ARG;
  for (uint64_t i = 0; i < count; ++i) out[i] = nullptr;
  int rc = guard(ctx, [&] {
    // every file gets a slice of one pinned arena (grown once, then reused)
    std::vector<uint64_t> size(count), off(count + 1, 0);
    for (uint64_t i = 0; i < count; ++i) {
      struct stat sb;
      if (::stat(paths[i], &sb) != 0 || !S_ISREG(sb.st_mode))
        fail(HD_ERR_IO, std::string("Error: Failed to open file '") + paths[i] + "'");
      size[i] = (uint64_t)sb.st_size;
      off[i + 1] = off[i] + hd::round_up(size[i] + 1, 256);
    }
    if (off[count] > ctx->pin_cap) {
      if (ctx->pin) cudaFreeHost(ctx->pin);
      ctx->pin = nullptr;
      ctx->pin_cap = 0;
      const size_t cap = (size_t)(off[count] * 5 / 4 + (1 << 20));
      HD_CUDA(cudaHostAlloc(&ctx->pin, cap, cudaHostAllocDefault));
      ctx->pin_cap = cap;
    }
    char *arena = static_cast<char *>(ctx->pin);
    run_on_workers(ctx, count, 12, [&](hd_ctx *w, uint64_t i) {
      int r = read_file_into(w, paths[i], arena + off[i], size[i]);
      if (r != HD_OK) return r;
      return hd_alignment_from_fasta(w, arena + off[i], size[i], 0, remove_duplicates, n_limit,
                                     include_x, semantics, &out[i]);
    });
  });
  if (rc != HD_OK)
    for (uint64_t i = 0; i < count; ++i) {
      hd_alignment_free(out[i]);
      out[i] = nullptr;
    }
  return rc;
}


int hd_pairwise_lt_files(hd_ctx *ctx, uint64_t count, const char *const *paths,
                         int remove_duplicates, uint64_t n_limit, int include_x, int semantics,
                         const int *dtype_bytes, const int64_t *max_distance, hd_output_fn out_fn,
                         void *user, hd_alignment **alns) {
  if (!ctx || (count && (!paths || !dtype_bytes || !max_distance || !out_fn))) return HD_ERR_ARG;
  if (alns)
    for (uint64_t i = 0; i < count; ++i) alns[i] = nullptr;
  std::vector<hd_alignment *> A(count, nullptr);
  int rc = guard(ctx, [&] {
    std::vector<uint32_t> md(count);
    for (uint64_t i = 0; i < count; ++i) {
      check_dtype(dtype_bytes[i]);
      md[i] = clamp_max(max_distance[i], dtype_bytes[i]);
    }
    // Each file has a slice of an arena at off[i] (256-byte aligned).
    //   mapped (ctx->map_files): the files are mapped read-only; one thread
    //     populates them (16 if some pages are not cached) and one uploader
    //     copies each mapping into the device arena (ctx->file) on ctx->up in
    //     order, with an event per file; the workers ingest from the device.
    //     Every worker copying its own files from pageable memory, with many
    //     mappings populated at once, was slower (19.0 vs 17.2 ms for 64 files).
    //   staged: readers pread 8 MB parts into a pinned arena (grown once, then
    //     reused) and the workers copy their files from it.
    const bool mapped = ctx->map_files != 0;
    std::vector<uint64_t> size(count), off(count + 1, 0);
    for (uint64_t i = 0; i < count; ++i) {
      struct stat sb;
      if (!paths[i] || ::stat(paths[i], &sb) != 0 || !S_ISREG(sb.st_mode))
        fail(HD_ERR_IO, open_failed(paths[i]));
      size[i] = (uint64_t)sb.st_size;
      off[i + 1] = off[i] + hd::round_up(size[i] + 1, 256);
    }
    if (!mapped && off[count] > ctx->pin_cap) {
      if (ctx->pin) cudaFreeHost(ctx->pin);
      ctx->pin = nullptr;
      ctx->pin_cap = 0;
      const size_t cap = (size_t)(off[count] * 5 / 4 + (1 << 20));
      HD_CUDA(cudaHostAlloc(&ctx->pin, cap, cudaHostAllocDefault));
      ctx->pin_cap = cap;
    }
    ctx->file_tag.clear();
    ctx->parsed.reset();
    char *arena = static_cast<char *>(ctx->pin);
    uint8_t *d_arena = nullptr;
    if (mapped) {
      if (ctx->file.bytes < off[count] + 16) {
        ctx->file.release();
        ctx->file = DevBuf(hd::round_up(off[count] + 16, 1 << 20), ctx->stream);
      }
      d_arena = ctx->file.as<uint8_t>();
      while (ctx->part_ev.size() < count + 1) {
        cudaEvent_t e;
        HD_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        ctx->part_ev.push_back(e);
      }
      // the arena is allocated (and earlier work on it ordered) on ctx->stream
      HD_CUDA(cudaEventRecord(ctx->part_ev[count], ctx->stream));
      HD_CUDA(cudaStreamWaitEvent(ctx->up, ctx->part_ev[count], 0));
    }
    // host threads: readers copy from the page cache and ingest workers spin
    // while they wait for their streams, so together they stay within the
    // cores (half read, 3/8 ingest; 8 and 6 on 16 cores)
    const unsigned hw = std::max(4u, std::thread::hardware_concurrency());
    const size_t n_workers = (size_t)std::min<uint64_t>(count, std::min(12u, std::max(2u, hw * 3 / 8)));
    const unsigned max_readers = std::min(16u, std::max(2u, hw / 2));
    while (ctx->workers.size() < n_workers) {
      hd_ctx *w = nullptr;
      const int r = hd_ctx_create(ctx->device, &w);
      if (r != HD_OK) fail(r, "could not create a worker context");
      ctx->workers.push_back(w);
    }
    std::vector<uint64_t> launches0;
    for (hd_ctx *w : ctx->workers) {
      w->tune = ctx->tune;
      launches0.push_back(w->launches);
    }

    // timeline for the trace (host ms since the start of the call)
    const auto t_start = std::chrono::steady_clock::now();
    auto now_ms = [&] {
      return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start)
          .count();
    };
    double t_read_end = 0, t_ingest_end = 0;
    struct GroupLog {
      double launch, done;
      size_t jobs;
      uint64_t tiles;
    };
    std::vector<GroupLog> glog;
    // shared state of the pipeline
    std::mutex mu;
    std::condition_variable cv;
    std::vector<char> read_done(count, 0);
    std::deque<uint64_t> ready;  // ingested, not yet launched
    uint64_t ingested = 0;
    int err = HD_OK;
    std::string err_msg;
    auto set_err = [&](int code, const std::string &m) {
      std::lock_guard<std::mutex> lk(mu);
      if (err == HD_OK) {
        err = code;
        err_msg = m;
      }
      cv.notify_all();
    };
    auto failed = [&] {
      std::lock_guard<std::mutex> lk(mu);
      return err != HD_OK;
    };

    // largest files first: their matrices cost the most (~ rows^2), so their
    // kernels start early and the small ones fill in behind them
    std::vector<uint64_t> order(count);
    for (uint64_t i = 0; i < count; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(),
                     [&](uint64_t a, uint64_t b) { return size[a] > size[b]; });
    // readers: 8 MB parts of the files in that order, shared by all reader
    // threads, never waiting for the GPU; a file is read when its last part is
    struct Fds {  // closed on every way out
      std::vector<int> v;
      ~Fds() {
        for (int fd : v)
          if (fd >= 0) ::close(fd);
      }
    } fdset;
    fdset.v.assign(count, -1);
    std::vector<int> &fds = fdset.v;
    for (uint64_t i = 0; i < count; ++i) {
      fds[i] = ::open(paths[i], O_RDONLY);
      if (fds[i] < 0) fail(HD_ERR_IO, open_failed(paths[i]));
    }
    // the files' mappings. An unmapper thread ends each one once its copy is
    // done, while the GPU computes: unmapping 64 file mappings at the end
    // took ~3 ms. release() ends the rest, on every way out, once no copy
    // from them can still be queued.
    struct Maps {
      hd_ctx *ctx;
      std::vector<char *> at;  // file i's mapping (nullptr: empty file, or unmapped)
      std::vector<size_t> len;
      void unmap(uint64_t i) {
        if (at[i]) ::munmap(at[i], len[i]);
        at[i] = nullptr;
      }
      void release() {
        bool any = false;
        for (char *p : at) any = any || p;
        if (!any) return;
        cudaStreamSynchronize(ctx->up);
        for (uint64_t i = 0; i < at.size(); ++i) unmap(i);
      }
      ~Maps() { release(); }
    } maps{ctx, std::vector<char *>(count, nullptr), std::vector<size_t>(count, 0)};
    bool all_in_cache = true;
    if (mapped) {
      const uint64_t page = (uint64_t)::sysconf(_SC_PAGESIZE);
      for (uint64_t i = 0; i < count; ++i) {
        if (!size[i]) continue;
        const size_t len = (size_t)hd::round_up(size[i], page);
        void *m = ::mmap(nullptr, len, PROT_READ, MAP_SHARED, fds[i], 0);
        if (m == MAP_FAILED) fail(HD_ERR_IO, open_failed(paths[i]));
        maps.at[i] = static_cast<char *>(m);
        maps.len[i] = len;
        all_in_cache = all_in_cache && all_cached(m, len);
      }
    }
    struct Part {
      uint64_t file, off, len;
    };
    const uint64_t kPart = 8ull << 20;
    std::vector<Part> parts;
    std::vector<std::atomic<uint64_t>> parts_left(count);
    for (uint64_t q = 0; q < count; ++q) {
      const uint64_t i = order[q];
      uint64_t np = 0;
      for (uint64_t o = 0; o < size[i]; o += kPart, ++np) parts.push_back({i, o, std::min(kPart, size[i] - o)});
      if (size[i] == 0) {
        parts.push_back({i, 0, 0});
        np = 1;
      }
      parts_left[i] = np;
    }
    // mapped mode: mappers populate the files in order, the uploader copies
    // each one once it is populated; a file is read when its copy is queued
    std::vector<char> populated(count, 0);
    std::atomic<uint64_t> next_map{0};
    auto mapper = [&] {
      for (uint64_t q = next_map++; q < count && !failed(); q = next_map++) {
        const uint64_t i = order[q];
        if (size[i] && !populate(maps.at[i], size[i])) {
          set_err(HD_ERR_IO, open_failed(paths[i]));
          return;
        }
        std::lock_guard<std::mutex> lk(mu);
        populated[i] = 1;
        cv.notify_all();
      }
    };
    auto uploader = [&] {
      if (cudaSetDevice(ctx->device) != cudaSuccess) {
        set_err(HD_ERR_CUDA, "cudaSetDevice failed");
        return;
      }
      for (uint64_t q = 0; q < count; ++q) {
        const uint64_t i = order[q];
        {
          std::unique_lock<std::mutex> lk(mu);
          cv.wait(lk, [&] { return populated[i] || err != HD_OK; });
          if (err != HD_OK) return;
        }
        if ((size[i] && cudaMemcpyAsync(d_arena + off[i], maps.at[i], size[i],
                                        cudaMemcpyHostToDevice, ctx->up) != cudaSuccess) ||
            cudaEventRecord(ctx->part_ev[i], ctx->up) != cudaSuccess) {
          set_err(HD_ERR_CUDA, "cudaMemcpyAsync of a FASTA file failed");
          return;
        }
        std::lock_guard<std::mutex> lk(mu);
        read_done[i] = 1;
        t_read_end = std::max(t_read_end, now_ms());
        cv.notify_all();
      }
    };
    // file i's mapping ends once its copy has completed (the thread owns
    // maps.at[i] from then: the uploader has read it, no one else does)
    auto unmapper = [&] {
      if (cudaSetDevice(ctx->device) != cudaSuccess) return;  // release() unmaps
      for (uint64_t q = 0; q < count; ++q) {
        const uint64_t i = order[q];
        {
          std::unique_lock<std::mutex> lk(mu);
          cv.wait(lk, [&] { return read_done[i] || err != HD_OK; });
          if (err != HD_OK) return;
        }
        if (cudaEventSynchronize(ctx->part_ev[i]) != cudaSuccess) return;
        maps.unmap(i);
      }
    };
    std::atomic<uint64_t> next_part{0};
    auto reader = [&] {
      for (uint64_t k = next_part++; k < parts.size() && !failed(); k = next_part++) {
        const Part &pt = parts[k];
        bool ok = true;
        for (uint64_t o = 0; ok && o < pt.len;) {
          const ssize_t r = ::pread(fds[pt.file], arena + off[pt.file] + pt.off + o,
                                    (size_t)(pt.len - o), (off_t)(pt.off + o));
          if (r <= 0) ok = false;
          else o += (uint64_t)r;
        }
        if (!ok) {
          set_err(HD_ERR_IO, open_failed(paths[pt.file]));
          return;
        }
        if (parts_left[pt.file].fetch_sub(1) == 1) {
          std::lock_guard<std::mutex> lk(mu);
          read_done[pt.file] = 1;
          t_read_end = std::max(t_read_end, now_ms());
          cv.notify_all();
        }
      }
    };
    // ingest workers: each file once it is read, on the worker's own stream
    std::atomic<uint64_t> next_ingest{0};
    auto ingester = [&](hd_ctx *w) {
      for (uint64_t q = next_ingest++; q < count; q = next_ingest++) {
        const uint64_t i = order[q];
        {
          std::unique_lock<std::mutex> lk(mu);
          cv.wait(lk, [&] { return read_done[i] || err != HD_OK; });
          if (err != HD_OK) return;
        }
        hd_alignment *a = nullptr;
        int r;
        if (mapped) {  // from the device arena, after the file's copy
          r = cudaStreamWaitEvent(w->stream, ctx->part_ev[i], 0) == cudaSuccess ? HD_OK : HD_ERR_CUDA;
          if (r == HD_OK)
            r = hd_alignment_from_fasta(w, reinterpret_cast<const char *>(d_arena + off[i]),
                                        size[i], 1, remove_duplicates, n_limit, include_x,
                                        semantics, &a);
          else
            cudaGetLastError();
        } else {
          r = hd_alignment_from_fasta(w, arena + off[i], size[i], 0, remove_duplicates, n_limit,
                                      include_x, semantics, &a);
        }
        if (r != HD_OK) {
          set_err(r, std::string(hd_last_error(w)) + " (input " + std::to_string(i) + ")");
          return;
        }
        std::lock_guard<std::mutex> lk(mu);
        A[i] = a;
        ready.push_back(i);
        ++ingested;
        t_ingest_end = std::max(t_ingest_end, now_ms());
        cv.notify_all();
      }
    };

    // a launched group: its kernels' event, job tables and device outputs
    struct Group {
      size_t log = 0;  // index in glog
      cudaEvent_t done = nullptr;
      hd::PairLaunchPlan plan;
      std::vector<DevBuf> dev;
      std::vector<void *> host;
      std::vector<uint64_t> bytes;
    };
    std::deque<std::unique_ptr<Group>> to_copy;
    bool launcher_done = false;
    // completion: copies each finished group to its host outputs in order
    auto completer = [&] {
      if (cudaSetDevice(ctx->device) != cudaSuccess) {
        set_err(HD_ERR_CUDA, "cudaSetDevice failed");
        return;
      }
      for (;;) {
        std::unique_ptr<Group> g;
        {
          std::unique_lock<std::mutex> lk(mu);
          cv.wait(lk, [&] { return !to_copy.empty() || launcher_done; });
          if (to_copy.empty()) return;
          g = std::move(to_copy.front());
          to_copy.pop_front();
        }
        bool ok = cudaEventSynchronize(g->done) == cudaSuccess;
        {
          std::lock_guard<std::mutex> lk(mu);
          glog[g->log].done = now_ms();
        }
        for (size_t j = 0; ok && j < g->dev.size(); ++j) {
          prefault_host(g->host[j], g->bytes[j]);
          ok = cudaMemcpyAsync(g->host[j], g->dev[j].p, g->bytes[j], cudaMemcpyDeviceToHost,
                               ctx->side) == cudaSuccess &&
               cudaStreamSynchronize(ctx->side) == cudaSuccess;
        }
        cudaEventDestroy(g->done);
        if (!ok) set_err(HD_ERR_CUDA, "copying results to the host failed");
        // g's device buffers and job tables are freed here, after their last use
      }
    };

    // the launcher's own event, re-recorded after each group: the GPU is idle
    // when it has completed (the groups' events belong to the completer)
    cudaEvent_t last = nullptr;
    HD_CUDA(cudaEventCreateWithFlags(&last, cudaEventDisableTiming));
    std::vector<std::thread> threads;
    if (mapped) {
      const unsigned n_map = (unsigned)std::min<uint64_t>(count, all_in_cache ? 1 : max_readers);
      for (unsigned t = 0; t < n_map; ++t) threads.emplace_back(mapper);
      if (count) threads.emplace_back(uploader);
      if (count) threads.emplace_back(unmapper);
    } else {
      const unsigned n_readers = (unsigned)std::min<uint64_t>(parts.size(), max_readers);
      for (unsigned t = 0; t < n_readers; ++t) threads.emplace_back(reader);
    }
    for (size_t t = 0; t < n_workers; ++t) threads.emplace_back(ingester, ctx->workers[t]);
    std::thread completion(completer);

    // launcher (this thread): whenever the previous group's kernels are done,
    // every ingested alignment not yet computed goes into one persistent launch
    uint64_t launched = 0, tiles = 0;
    bool any = false;
    try {
      while (launched < count) {
        std::vector<uint64_t> take;
        {
          std::unique_lock<std::mutex> lk(mu);
          for (;;) {
            if (err != HD_OK) break;
            const bool idle = !any || cudaEventQuery(last) == cudaSuccess;
            if (!ready.empty() && (idle || ingested == count)) break;
            cv.wait_for(lk, std::chrono::microseconds(100));
          }
          if (err != HD_OK) break;
          take.assign(ready.begin(), ready.end());
          ready.clear();
        }
        auto g = std::make_unique<Group>();
        std::vector<hd::PairJobSpec> specs;
        for (uint64_t i : take) {
          const hd_alignment *a = A[i];
          const uint64_t entries = a->n_rows < 2 ? 0 : tri(a->n_rows);
          void *host = out_fn(user, i, a->n_rows, entries);
          if (!host && entries) fail(HD_ERR_ARG, "output callback returned no buffer");
          if (!entries) continue;
          g->dev.emplace_back(entries * dtype_bytes[i], ctx->stream);
          g->host.push_back(host);
          g->bytes.push_back(entries * dtype_bytes[i]);
          hd::PairJobSpec sp;
          sp.aln = a;
          sp.dtype = dtype_bytes[i];
          sp.max_dist = md[i];
          sp.d_out = g->dev.back().p;
          sp.out_base = 0;
          sp.cfg = hd::tile_config_for(ctx, a->n_rows, a->length, dtype_bytes[i]);
          sp.tile_lo = 0;
          sp.tile_hi = (uint32_t)hd::ceil_div(a->n_rows, sp.cfg.tile);
          specs.push_back(sp);
        }
        launched += take.size();
        uint64_t g_tiles = 0;
        if (!specs.empty()) {
          // while files are still being ingested, 16 SMs stay free for their
          // kernels (a persistent grid holds its SMs until it ends)
          bool pending;
          {
            std::lock_guard<std::mutex> lk(mu);
            pending = ingested < count;
          }
          hd::prepare_pairwise_jobs(ctx, specs, ctx->stream, &g->plan,
                                    pending ? std::max(1, ctx->sm_count - 16) : 0);
          hd::launch_pairwise_plan(ctx, g->plan, ctx->stream);
          for (auto &L : g->plan.launches) g_tiles += L.tiles;
          tiles += g_tiles;
        }
        {
          std::lock_guard<std::mutex> lk(mu);
          g->log = glog.size();
          glog.push_back({now_ms(), 0.0, specs.size(), g_tiles});
        }
        HD_CUDA(cudaEventCreateWithFlags(&g->done, cudaEventDisableTiming));
        HD_CUDA(cudaEventRecord(g->done, ctx->stream));
        HD_CUDA(cudaEventRecord(last, ctx->stream));
        any = true;
        std::lock_guard<std::mutex> lk(mu);
        to_copy.push_back(std::move(g));
        cv.notify_all();
      }
    } catch (const hd::Error &e) {
      set_err(e.code, e.msg);
    }
    for (auto &t : threads) t.join();
    {
      std::lock_guard<std::mutex> lk(mu);
      launcher_done = true;
      cv.notify_all();
    }
    completion.join();
    cudaEventDestroy(last);
    maps.release();
    const double t_unmapped = now_ms();
    for (size_t t = 0; t < ctx->workers.size() && t < launches0.size(); ++t)
      ctx->launches += ctx->workers[t]->launches - launches0[t];
    ctx->last_pair_tiles = tiles;
    if (err != HD_OK) fail(err, err_msg);
    HD_CUDA(cudaStreamSynchronize(ctx->stream));
    check_status(ctx);
    if (ctx->trace.on) {
      char buf[160];
      std::snprintf(buf, sizeof buf,
                    "hd_pairwise_lt_files: %llu files read by %.3f ms, ingested by %.3f ms, "
                    "%zu groups:",
                    (unsigned long long)count, t_read_end, t_ingest_end, glog.size());
      std::string text = buf;
      for (const auto &g : glog) {
        std::snprintf(buf, sizeof buf, " [%.3f-%.3f ms, %zu jobs, %llu tiles]", g.launch, g.done,
                      g.jobs, (unsigned long long)g.tiles);
        text += buf;
      }
      std::snprintf(buf, sizeof buf, ", files unmapped at %.3f ms, done at %.3f ms", t_unmapped,
                    now_ms());
      text += buf;
      ctx->trace.last = text;
    }
  });
  for (uint64_t i = 0; i < count; ++i) {
    if (rc == HD_OK && alns) alns[i] = A[i];
    else hd_alignment_free(A[i]);
  }
  return rc;
}

}  // extern "C"
