// The Python module: the reference's pybind11 API (python/hammingdist.cc:28-133)
// re-implemented over the libhd C ABI (include/hammingdist_gb300.h). Names,
// keyword arguments, defaults, return dtypes and error messages follow the
// reference; every distance is computed on the GPU.
//
// use_gpu keeps the reference's meaning for the RESULT: True gives the
// reference GPU's values (dense AND rule; include_x rejected), False gives
// the reference CPU's values (sparse rule when include_x or when fewer than
// 0.5% of sites differ from the consensus, else the dense rule). Both run on
// the GPU here.
#include <fcntl.h>
#include <pybind11/numpy.h>
#include <pybind11/pybind11.h>
#include <pybind11/stl.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
#include <sstream>
#include <stdexcept>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/hammingdist_gb300.h"

namespace py = pybind11;

namespace {

std::mutex g_mu;         // one context per process; calls are serialised
hd_ctx *g_ctx = nullptr;

hd_ctx *ctx() {
  if (!g_ctx) {
    int dev = 0;
    if (const char *e = std::getenv("HAMMINGDIST_DEVICE")) dev = std::atoi(e);
    int rc = hd_ctx_create(dev, &g_ctx);
    if (rc == HD_ERR_NO_DEVICE)
      throw std::runtime_error("hammingdist_gb300: no CUDA device available (this build has no CPU path)");
    if (rc != HD_OK) throw std::runtime_error("hammingdist_gb300: could not create a CUDA context");
  }
  return g_ctx;
}

void check(int rc) {
  if (rc != HD_OK) throw std::runtime_error(hd_last_error(g_ctx));
}

[[noreturn]] void open_failed(const std::string &f) {
  throw std::runtime_error("Error: Failed to open file '" + f + "'");
}

// Runs f(begin, end) over [0, n) bytes on up to 16 threads (4 MB or more each).
template <class F>
void split_parallel(size_t n, F &&f) {
  const size_t kMin = 4u << 20;
  const unsigned nt = (unsigned)std::max<size_t>(1, std::min<size_t>(16, n / kMin));
  if (nt == 1) {
    f(size_t(0), n);
    return;
  }
  const size_t per = (n + nt - 1) / nt;
  std::vector<std::thread> th;
  for (unsigned t = 0; t < nt; ++t)
    th.emplace_back([&, t] {
      const size_t a = t * per, b = std::min(n, a + per);
      if (a < b) f(a, b);
    });
  for (auto &x : th) x.join();
}

// memcpy of large results on up to 16 threads.
void copy_parallel(void *dst, const void *src, size_t n) {
  split_parallel(n, [&](size_t a, size_t b) {
    std::memcpy(static_cast<char *>(dst) + a, static_cast<const char *>(src) + a, b - a);
  });
}

// Large host results are recycled: a released result buffer keeps its pages
// mapped and present, so that the next result of a similar size is copied
// back without first-touch page faults (on a fresh 100 MB buffer they cost
// milliseconds). Buffers of 16 MB or more, at most 4 GB cached, reused for a
// request of at least half their size.
class ResultPool {
 public:
  static ResultPool &get() {
    static ResultPool *p = new ResultPool();  // outlives the arrays that return to it
    return *p;
  }
  void *take(size_t bytes) {
    if (bytes >= kMin) {
      std::lock_guard<std::mutex> lk(mu_);
      auto it = free_.lower_bound(bytes);
      if (it != free_.end() && it->first / 2 <= bytes) {
        void *p = it->second;
        cached_ -= it->first;
        size_[p] = it->first;
        free_.erase(it);
        return p;
      }
    }
    void *p = std::malloc(bytes ? bytes : 1);
    if (!p) throw std::bad_alloc();
    if (bytes >= kMin) {
      std::lock_guard<std::mutex> lk(mu_);
      size_[p] = bytes;
    }
    return p;
  }
  void give(void *p) {
    if (!p) return;
    std::lock_guard<std::mutex> lk(mu_);
    auto s = size_.find(p);
    if (s == size_.end()) {
      std::free(p);
      return;
    }
    const size_t bytes = s->second;
    size_.erase(s);
    free_.emplace(bytes, p);
    cached_ += bytes;
    while (cached_ > kCap && !free_.empty()) {  // drop the largest first
      auto last = std::prev(free_.end());
      cached_ -= last->first;
      std::free(last->second);
      free_.erase(last);
    }
  }

 private:
  static constexpr size_t kMin = 16u << 20, kCap = 4ull << 30;
  std::mutex mu_;
  std::multimap<size_t, void *> free_;     // size -> released buffer
  std::unordered_map<void *, size_t> size_;  // buffer in use -> its size
  size_t cached_ = 0;
};

// Allocator whose resize() leaves new elements uninitialised (result vectors
// are filled by the device copy), drawing large buffers from the ResultPool.
template <class T>
struct NoInitAlloc : std::allocator<T> {
  using value_type = T;
  template <class U>
  struct rebind {
    using other = NoInitAlloc<U>;
  };
  NoInitAlloc() = default;
  template <class U>
  NoInitAlloc(const NoInitAlloc<U> &) noexcept {}
  T *allocate(size_t n) { return static_cast<T *>(ResultPool::get().take(n * sizeof(T))); }
  void deallocate(T *p, size_t) noexcept { ResultPool::get().give(p); }
  template <class U>
  void construct(U *p) noexcept {
    ::new (static_cast<void *>(p)) U;
  }
  template <class U, class... A>
  void construct(U *p, A &&...a) {
    ::new (static_cast<void *>(p)) U(std::forward<A>(a)...);
  }
};
template <class T>
using HostVec = std::vector<T, NoInitAlloc<T>>;

struct Aln {
  hd_alignment *p = nullptr;
  ~Aln() { hd_alignment_free(p); }
};

void say(const std::string &s) { std::cout << "# hammingdist :: " << s << std::endl; }

// HAMMINGDIST_TRACE=1: the context traces its calls' phases (CUDA events on
// its stream); each traced call's line is printed after it, and host-side
// phases are timed here.
bool tracing() {
  static const bool on = [] {
    const char *t = std::getenv("HAMMINGDIST_TRACE");
    return t && t[0] && t[0] != '0';
  }();
  return on;
}
void say_trace() {
  if (tracing()) say(std::string("trace ") + hd_trace_last(g_ctx));
}
void say_host(const char *what, double ms) {
  if (tracing()) say(std::string("trace host: ") + what + " " + std::to_string(ms) + " ms");
}

double ms_since(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

// ------------------------------------------------------------------ DataSet
// include/hamming/hamming.hh:22-143: owns the lower triangle
// lt[i(i-1)/2 + j], i > j, and the sequence indices.
template <typename T>
struct DataSet {
  uint64_t nsamples = 0;
  HostVec<T> result;
  std::vector<uint64_t> sequence_indices;
  // A second copy of the result that the library wrote while the distances
  // ran (HD_OUTPUT_MIRROR). The first lt_array access hands it out as its
  // fresh array, and later accesses copy; shared by copies of the DataSet, so
  // only one of them can hand it out.
  struct FirstCopy {
    std::mutex mu;
    std::unique_ptr<HostVec<T>> buf;
  };
  std::shared_ptr<FirstCopy> first_copy;

  int at(const std::array<size_t, 2> &ij) const {
    size_t i = ij[0], j = ij[1];
    if (i < j) std::swap(i, j);
    if (i == j) return 0;
    return result.at(i * (i - 1) / 2 + j);
  }

  // hamming.hh:63-73 (full matrix, ", " separators): host formatting, not on
  // the device path
  // hamming.hh:63-73: the full matrix, formatted on the device
  void dump(const std::string &filename) const {
    std::lock_guard<std::mutex> lk(g_mu);
    hd_ctx *c = ctx();
    py::gil_scoped_release nogil;
    check(hd_write_full_matrix(c, result.data(), result.size(), nsamples, sizeof(T),
                               filename.c_str()));
  }

  void dump_lower_triangular(const std::string &filename) const {
    std::lock_guard<std::mutex> lk(g_mu);
    hd_ctx *c = ctx();
    py::gil_scoped_release nogil;
    check(hd_write_lower_triangular(c, result.data(), nsamples, sizeof(T), filename.c_str()));
  }

  void dump_sparse(const std::string &filename, int threshold) const {
    std::lock_guard<std::mutex> lk(g_mu);
    hd_ctx *c = ctx();
    py::gil_scoped_release nogil;
    check(hd_write_sparse(c, result.data(), nsamples, sizeof(T), threshold, filename.c_str(), nullptr));
  }

  // hamming.hh:116-127
  void dump_sequence_indices(const std::string &filename) const {
    std::ofstream s(filename);
    if (sequence_indices.empty()) {
      for (uint64_t i = 0; i < nsamples; ++i) s << i << "\n";
      return;
    }
    for (auto v : sequence_indices) s << v << "\n";
  }
};

namespace {

template <typename T>
DataSet<T> compute(hd_alignment *aln, int64_t max_distance, bool announce, const char *what,
                   std::chrono::steady_clock::time_point t0) {
  DataSet<T> ds;
  uint64_t n_rows = 0, L = 0, n_in = 0;
  int rule = 0;
  check(hd_alignment_info(aln, &n_rows, &L, &n_in, &rule));
  ds.nsamples = n_rows;
  const auto ta = std::chrono::steady_clock::now();
  // left uninitialised: hd_pairwise_lt touches the pages while the kernel runs
  ds.result.resize(n_rows < 2 ? 0 : n_rows * (n_rows - 1) / 2);
  say_host("result allocation", ms_since(ta));
  if (announce) {
    say(std::string("Using GPU (") + what +
        (rule == HD_RULE_AND ? ", dense distance rule)..." : ", sparse distance rule)..."));
    say("...pre-processing completed in " + std::to_string((long long)ms_since(t0)) + " ms...");
  }
  auto t1 = std::chrono::steady_clock::now();
  if (!ds.result.empty())
    check(hd_pairwise_lt(g_ctx, aln, sizeof(T), max_distance, ds.result.data(), 0));
  if (!ds.result.empty()) say_trace();
  if (announce)
    say("...distance calculation completed in " + std::to_string((long long)ms_since(t1)) + " ms.");
  return ds;
}

template <typename T>
DataSet<T> from_fasta(const std::string &filename, bool include_x, bool remove_duplicates,
                      size_t n, bool use_gpu, int max_distance) {
  std::lock_guard<std::mutex> lk(g_mu);
  hd_ctx *c = ctx();
  auto t0 = std::chrono::steady_clock::now();
  py::gil_scoped_release nogil;
  Aln a;
  if (use_gpu && !include_x && n == 0) {
    // one call: for large files the distances overlap the read
    DataSet<T> ds;
    hd_output_fn alloc = [](void *user, uint64_t index, uint64_t rows, uint64_t entries) -> void * {
      auto *d = static_cast<DataSet<T> *>(user);
      if (index == HD_OUTPUT_MIRROR) {
        // the first lt_array's copy, made while the distances run; not for
        // results above 2 GB, which would double the host memory held
        if (entries * sizeof(T) > (2ull << 30)) return nullptr;
        d->first_copy = std::make_shared<typename DataSet<T>::FirstCopy>();
        d->first_copy->buf = std::make_unique<HostVec<T>>();
        d->first_copy->buf->resize(entries);
        return d->first_copy->buf->data();
      }
      d->nsamples = rows;
      d->result.resize(entries);  // its pages are first touched while the kernels run
      return d->result.data();
    };
    say("Using GPU (use_gpu=True, dense distance rule)...");
    check(hd_pairwise_lt_fasta_file(c, filename.c_str(), remove_duplicates, sizeof(T), max_distance,
                                    alloc, &ds, &a.p));
    say_trace();
    say("...pre-processing and distance calculation completed in " +
        std::to_string((long long)ms_since(t0)) + " ms.");
    if (remove_duplicates) {
      uint64_t n_in = 0;
      check(hd_alignment_info(a.p, nullptr, nullptr, &n_in, nullptr));
      ds.sequence_indices.resize(n_in);
      check(hd_alignment_sequence_indices(a.p, ds.sequence_indices.data()));
    }
    return ds;
  }
  check(hd_alignment_from_fasta_file(c, filename.c_str(), remove_duplicates, n, include_x,
                                     use_gpu ? HD_SEM_GPU : HD_SEM_CPU, &a.p));
  say_trace();
  DataSet<T> ds = compute<T>(a.p, max_distance, true, use_gpu ? "use_gpu=True" : "use_gpu=False", t0);
  if (remove_duplicates) {
    uint64_t n_in = 0;
    check(hd_alignment_info(a.p, nullptr, nullptr, &n_in, nullptr));
    ds.sequence_indices.resize(n_in);
    check(hd_alignment_sequence_indices(a.p, ds.sequence_indices.data()));
  }
  return ds;
}

// from_fasta(use_gpu=True) for FASTA text already in device memory, with the
// lower triangle written to device memory: `fasta` and `out` are CUDA device
// pointers (e.g. tensor.data_ptr()), `out_bytes` the room at `out`. Parse,
// dedupe, pack and distances run on the device; optionally the distances of
// `reference_sequence` to every record (fasta_reference_distances,
// src/hamming.cc:104-141) come from the same resident rows. Returns a dict:
// nsamples, sequence_indices (uint64, empty without dedupe), kernel_ms (the
// distance launch's CUDA-event time) and reference_distances (uint32) when a
// reference was given. No reference counterpart: the reference reads files.
py::dict from_fasta_device(uintptr_t fasta, uint64_t nbytes, uintptr_t out, uint64_t out_bytes,
                           bool remove_duplicates, int max_distance, bool large,
                           py::object reference_sequence) {
  std::string ref;
  const bool want_ref = !reference_sequence.is_none();
  if (want_ref) ref = py::cast<std::string>(reference_sequence);
  std::lock_guard<std::mutex> lk(g_mu);
  hd_ctx *c = ctx();
  const int dtype = large ? 2 : 1;
  uint64_t n_rows = 0, n_in = 0;
  double kernel_ms = 0, mma_macs = 0;
  uint64_t tiles = 0;
  std::vector<uint64_t> idx;
  std::vector<uint32_t> rd;
  {
    py::gil_scoped_release nogil;
    Aln a;
    check(hd_alignment_from_fasta(c, reinterpret_cast<const char *>(fasta), nbytes, 1,
                                  remove_duplicates, 0, 0, HD_SEM_GPU, &a.p));
    check(hd_alignment_info(a.p, &n_rows, nullptr, &n_in, nullptr));
    const uint64_t entries = n_rows < 2 ? 0 : n_rows * (n_rows - 1) / 2;
    if (entries * dtype > out_bytes)
      throw std::invalid_argument("from_fasta_device: the output needs " +
                                  std::to_string(entries * dtype) + " bytes");
    if (entries) {
      check(hd_pairwise_lt(c, a.p, dtype, max_distance, reinterpret_cast<void *>(out), 1));
      hd_last_pairwise_timing(c, &kernel_ms, &tiles);
      hd_last_pairwise_work(c, &mma_macs);
    }
    if (remove_duplicates) {
      idx.resize(n_in);
      check(hd_alignment_sequence_indices(a.p, idx.data()));
    }
    if (want_ref) {
      rd.resize(n_in);
      check(hd_alignment_reference_distances(c, a.p, ref.data(), ref.size(), 0, rd.data()));
    }
  }
  py::dict r;
  r["nsamples"] = n_rows;
  r["sequence_indices"] = py::array_t<uint64_t>((py::ssize_t)idx.size(), idx.data());
  r["kernel_ms"] = kernel_ms;
  r["mma_macs"] = mma_macs;
  if (want_ref) r["reference_distances"] = py::array_t<uint32_t>((py::ssize_t)rd.size(), rd.data());
  return r;
}

DataSet<uint8_t> from_stringlist(const std::vector<std::string> &data, bool include_x, bool use_gpu,
                                 int max_distance) {
  std::lock_guard<std::mutex> lk(g_mu);
  hd_ctx *c = ctx();
  std::string cat;
  std::vector<uint64_t> offsets(data.size() + 1, 0);
  for (size_t k = 0; k < data.size(); ++k) {
    cat += data[k];
    offsets[k + 1] = cat.size();
  }
  py::gil_scoped_release nogil;
  Aln a;
  check(hd_alignment_from_sequences(c, cat.data(), offsets.data(), data.size(), include_x,
                                    use_gpu ? HD_SEM_GPU : HD_SEM_CPU, &a.p));
  return compute<uint8_t>(a.p, max_distance, false, "", std::chrono::steady_clock::now());
}

void from_fasta_to_lower_triangular(const std::string &in, const std::string &out,
                                    bool remove_duplicates, size_t n, bool use_gpu,
                                    int max_distance) {
  std::lock_guard<std::mutex> lk(g_mu);
  hd_ctx *c = ctx();
  auto t0 = std::chrono::steady_clock::now();
  if (use_gpu) say("Using GPU...");
  py::gil_scoped_release nogil;
  Aln a;
  check(hd_alignment_from_fasta_file(c, in.c_str(), remove_duplicates, n, 0, HD_SEM_GPU, &a.p));
  say_trace();
  say("...pre-processing completed in " + std::to_string((long long)ms_since(t0)) + " ms...");
  // src/hamming.cc:47-52: the reference computes this on the GPU only
  if (!use_gpu) throw std::runtime_error("from_fasta_to_lower_triangular is currently only available on GPU");
  auto t1 = std::chrono::steady_clock::now();
  check(hd_pairwise_lt_to_file(c, a.p, max_distance, out.c_str()));
  say("...distance calculation completed in " + std::to_string((long long)ms_since(t1)) + " ms.");
}

// Many FASTA files: concurrent ingest, then all matrices in one batch run
// (persistent kernel over every job's tiles, launches replayed from a CUDA
// graph). `large` / `max_distance` are one value or one per file; a large
// entry gives a DataSetLarge (uint16) like from_fasta_large. No reference
// counterpart: the reference computes one matrix per call.
py::list from_fasta_batch(const std::vector<std::string> &files, bool include_x,
                          bool remove_duplicates, size_t n, bool use_gpu, py::object max_distance,
                          py::object large) {
  const size_t k = files.size();
  std::vector<int> big(k, 0);
  std::vector<int64_t> md(k, 0);
  for (size_t i = 0; i < k; ++i) {
    big[i] = py::isinstance<py::sequence>(large) ? py::cast<bool>(large[py::int_(i)])
                                                 : py::cast<bool>(large);
    if (max_distance.is_none()) md[i] = big[i] ? 65535 : 255;
    else if (py::isinstance<py::sequence>(max_distance)) md[i] = py::cast<int>(max_distance[py::int_(i)]);
    else md[i] = py::cast<int>(max_distance);
  }
  std::lock_guard<std::mutex> lk(g_mu);
  hd_ctx *c = ctx();
  std::vector<const char *> paths(k);
  for (size_t i = 0; i < k; ++i) paths[i] = files[i].c_str();
  std::vector<hd_alignment *> alns(k, nullptr);
  std::vector<DataSet<uint8_t>> small(k);
  std::vector<DataSet<uint16_t>> wide(k);
  std::vector<int> dtype(k);
  for (size_t i = 0; i < k; ++i) dtype[i] = big[i] ? 2 : 1;
  struct Out {
    std::vector<int> *big;
    std::vector<DataSet<uint8_t>> *small;
    std::vector<DataSet<uint16_t>> *wide;
  } o{&big, &small, &wide};
  // sizes each result when its row count is known (distinct indices only)
  hd_output_fn alloc = [](void *user, uint64_t i, uint64_t rows, uint64_t entries) -> void * {
    Out *q = static_cast<Out *>(user);
    if ((*q->big)[i]) {
      auto &d = (*q->wide)[i];
      d.nsamples = rows;
      d.result.resize(entries);
      return d.result.data();
    }
    auto &d = (*q->small)[i];
    d.nsamples = rows;
    d.result.resize(entries);
    return d.result.data();
  };
  {
    py::gil_scoped_release nogil;
    auto t1 = std::chrono::steady_clock::now();
    check(hd_pairwise_lt_files(c, k, paths.data(), remove_duplicates, n, include_x,
                               use_gpu ? HD_SEM_GPU : HD_SEM_CPU, dtype.data(), md.data(), alloc, &o,
                               alns.data()));
    std::vector<Aln> own(k);
    for (size_t i = 0; i < k; ++i) own[i].p = alns[i];
    for (size_t i = 0; i < k; ++i) {
      if (!remove_duplicates) continue;
      uint64_t n_in = 0;
      check(hd_alignment_info(alns[i], nullptr, nullptr, &n_in, nullptr));
      auto &idx = big[i] ? wide[i].sequence_indices : small[i].sequence_indices;
      idx.resize(n_in);
      check(hd_alignment_sequence_indices(alns[i], idx.data()));
    }
    double pair_ms = 0;
    uint64_t tiles = 0;
    hd_last_pairwise_timing(c, &pair_ms, &tiles);
    say("batch of " + std::to_string(k) + " alignments: read, ingest and distances pipelined in " +
        std::to_string(ms_since(t1)) + " ms (" + std::to_string(tiles) + " tiles).");
    say_trace();
  }
  py::list out;
  for (size_t i = 0; i < k; ++i) {
    if (big[i]) out.append(py::cast(std::move(wide[i])));
    else out.append(py::cast(std::move(small[i])));
  }
  return out;
}

void autotune(const std::string &path) {
  std::lock_guard<std::mutex> lk(g_mu);
  hd_ctx *c = ctx();
  py::gil_scoped_release nogil;
  check(hd_autotune(c, 6));
  if (!path.empty()) check(hd_tune_save(c, path.c_str()));
}

void load_tuning(const std::string &path) {
  std::lock_guard<std::mutex> lk(g_mu);
  check(hd_tune_load(ctx(), path.c_str()));
}

uint32_t distance(const std::string &s0, const std::string &s1, bool include_x) {
  std::lock_guard<std::mutex> lk(g_mu);
  hd_ctx *c = ctx();
  uint32_t d = 0;
  check(hd_distance(c, s0.data(), s0.size(), s1.data(), s1.size(), include_x, &d));
  return d;
}

template <typename T>
py::array_t<T> owned_array(T *p, uint64_t n) {
  py::capsule cap(p, [](void *q) { hd_free(q); });
  return py::array_t<T>({(py::ssize_t)n}, {(py::ssize_t)sizeof(T)}, p, cap);
}

py::array_t<uint32_t> fasta_reference_distances(const std::string &ref, const std::string &fasta,
                                                bool include_x) {
  std::lock_guard<std::mutex> lk(g_mu);
  hd_ctx *c = ctx();
  uint32_t *out = nullptr;
  uint64_t n = 0;
  {
    py::gil_scoped_release nogil;
    check(hd_reference_distances_file(c, ref.data(), ref.size(), fasta.c_str(), include_x, &out, &n));
  }
  say_trace();
  return owned_array<uint32_t>(out, n);
}

py::array_t<uint64_t> fasta_sequence_indices(const std::string &fasta, size_t nlim) {
  std::lock_guard<std::mutex> lk(g_mu);
  hd_ctx *c = ctx();
  uint64_t *out = nullptr;
  uint64_t n = 0;
  {
    py::gil_scoped_release nogil;
    check(hd_fasta_sequence_indices_file(c, fasta.c_str(), nlim, &out, &n));
  }
  return owned_array<uint64_t>(out, n);
}

// Readers (hamming.hh:34-55, :152-166), parsed on the device. A field that
// std::stoi rejects raises the exception the reference raises there; a file
// that cannot be read gives an empty DataSet, as the reference's ifstream
// reads nothing from it.
[[noreturn]] void throw_parse(int kind) {
  if (kind == 2) throw std::out_of_range("stoi");
  throw std::invalid_argument("stoi");
}

template <typename T>
DataSet<T> read_result_file(const std::string &filename, bool csv) {
  std::lock_guard<std::mutex> lk(g_mu);
  hd_ctx *c = ctx();
  DataSet<T> ds;
  hd_output_fn alloc = [](void *user, uint64_t, uint64_t n, uint64_t entries) -> void * {
    auto *d = static_cast<DataSet<T> *>(user);
    d->nsamples = n;
    d->result.resize(entries);
    return d->result.data();
  };
  uint64_t entries = 0, n = 0;
  int kind = 0;
  int rc;
  {
    py::gil_scoped_release nogil;
    rc = csv ? hd_read_csv(c, filename.c_str(), alloc, &ds, &entries, &n, &kind)
             : hd_read_lower_triangular(c, filename.c_str(), sizeof(T), alloc, &ds, &entries, &n,
                                        &kind);
  }
  if (rc == HD_ERR_PARSE) throw_parse(kind);
  if (rc == HD_ERR_IO) {
    DataSet<T> empty;
    empty.nsamples = csv ? 0 : 1;  // no lines: 0 newlines / (round(sqrt(1)) + 1) / 2
    return empty;
  }
  check(rc);
  return ds;
}

template <typename T>
DataSet<T> from_lower_triangular(const std::string &filename) {
  return read_result_file<T>(filename, false);
}

DataSet<uint8_t> from_csv(const std::string &filename) {
  return read_result_file<uint8_t>(filename, true);
}

template <typename T>
void bind_dataset(py::module_ &m, const char *name, int default_threshold) {
  py::class_<DataSet<T>>(m, name)
      .def("dump", &DataSet<T>::dump, "Dump distances matrix in csv format")
      .def("dump_lower_triangular", &DataSet<T>::dump_lower_triangular,
           "Dump distances matrix in lower triangular format (comma-delimited, row-major)")
      .def("dump_sparse", &DataSet<T>::dump_sparse, py::arg("filename"),
           py::arg("threshold") = default_threshold,
           "Dump distances matrix in sparse format excluding any distances above threshold")
      .def("dump_sequence_indices", &DataSet<T>::dump_sequence_indices,
           "Dump row index in distances matrix for each input sequence")
      .def("__getitem__", &DataSet<T>::at)
      .def_readonly("_distances", &DataSet<T>::result)
      .def_property_readonly("lt_array", [](const DataSet<T> &self) {
        // a fresh copy on every access, as the reference's py::array(size, ptr);
        // the first access takes the copy written while the distances ran
        if (self.first_copy) {
          std::unique_ptr<HostVec<T>> b;
          {
            std::lock_guard<std::mutex> lk(self.first_copy->mu);
            b = std::move(self.first_copy->buf);
          }
          if (b && b->size() == self.result.size()) {
            HostVec<T> *raw = b.release();
            py::capsule owner(raw, [](void *p) { delete static_cast<HostVec<T> *>(p); });
            say_host("lt_array copy", 0.0);
            return py::array_t<T>((py::ssize_t)raw->size(), raw->data(), owner);
          }
        }
        py::array_t<T> a((py::ssize_t)self.result.size());
        const auto tc = std::chrono::steady_clock::now();
        copy_parallel(a.mutable_data(), self.result.data(), self.result.size() * sizeof(T));
        say_host("lt_array copy", ms_since(tc));
        return a;
      });
}

}  // namespace

PYBIND11_MODULE(_C, m) {
  m.doc() = "GB300 implementation of hammingdist's pairwise Hamming distances";
  bind_dataset<uint8_t>(m, "DataSet", 255);
  bind_dataset<uint16_t>(m, "DataSetLarge", 65535);
  m.def("from_stringlist", &from_stringlist, py::arg("data"), py::arg("include_x") = false,
        py::arg("use_gpu") = false, py::arg("max_distance") = std::numeric_limits<int>::max(),
        "Creates a dataset from a list of strings");
  m.def("from_csv", &from_csv,
        "Creates a dataset by reading already computed distances from csv (full matrix expected)");
  m.def("from_fasta", &from_fasta<uint8_t>, py::arg("filename"), py::arg("include_x") = false,
        py::arg("remove_duplicates") = false, py::arg("n") = 0, py::arg("use_gpu") = false,
        py::arg("max_distance") = 255,
        "Creates a dataset by reading from a fasta file (assuming all sequences have equal "
        "length). Maximum value of an element in the distances matrix: max_distance or 255, "
        "whichever is lower.");
  m.def("from_fasta_large", &from_fasta<uint16_t>, py::arg("filename"),
        py::arg("include_x") = false, py::arg("remove_duplicates") = false, py::arg("n") = 0,
        py::arg("use_gpu") = false, py::arg("max_distance") = 65535,
        "Creates a dataset by reading from a fasta file (assuming all sequences have equal "
        "length). Maximum value of an element in the distances matrix: max_distance or 65535, "
        "whichever is lower");
  m.def("from_fasta_to_lower_triangular", &from_fasta_to_lower_triangular,
        py::arg("fasta_filename"), py::arg("output_filename"), py::arg("remove_duplicates") = false,
        py::arg("n") = 0, py::arg("use_gpu") = true, py::arg("max_distance") = 65535,
        "Construct lower triangular distances matrix output file from the fasta file. Maximum "
        "value of an element in the distances matrix: max_distance or 65535, whichever is lower");
  m.def("from_lower_triangular", &from_lower_triangular<uint8_t>,
        "Creates a dataset by reading already computed distances from lower triangular format. "
        "Maximum value of an element in the distances matrix: 255.");
  m.def("from_lower_triangular_large", &from_lower_triangular<uint16_t>,
        "Creates a dataset by reading already computed distances from lower triangular format. "
        "Maximum value of an element in the distances matrix: 65535.");
  m.def("distance", &distance, py::arg("seq0"), py::arg("seq1"), py::arg("include_x") = false,
        "Calculate the distance between seq0 and seq1");
  m.def("fasta_reference_distances", &fasta_reference_distances, py::arg("reference_sequence"),
        py::arg("fasta_file"), py::arg("include_x") = false,
        "Calculates the distance of each sequence in the fasta file from the supplied reference "
        "sequence");
  m.def("fasta_sequence_indices", &fasta_sequence_indices, py::arg("fasta_file"), py::arg("n") = 0,
        "For each genome in the input fasta file the index of the corresponding row in the "
        "distances matrix which excludes duplicates");
  m.def("cuda_gpu_available", []() { return hd_device_available() != 0; },
        "True if a GPU that supports CUDA is available");
  m.def("from_fasta_batch", &from_fasta_batch, py::arg("filenames"), py::arg("include_x") = false,
        py::arg("remove_duplicates") = false, py::arg("n") = 0, py::arg("use_gpu") = true,
        py::arg("max_distance") = py::none(), py::arg("large") = false,
        "Distance matrices of several fasta files computed together on the GPU (one batch: "
        "concurrent ingest, one persistent kernel, launches replayed from a CUDA graph). "
        "Returns a list of DataSet (or DataSetLarge where `large`).");
  m.def("from_fasta_device", &from_fasta_device, py::arg("fasta_ptr"), py::arg("nbytes"),
        py::arg("out_ptr"), py::arg("out_bytes"), py::arg("remove_duplicates") = false,
        py::arg("max_distance") = 255, py::arg("large") = false,
        py::arg("reference_sequence") = py::none(),
        "from_fasta(use_gpu=True) on FASTA text already in device memory, the lower triangle "
        "written to device memory (uint8, or uint16 where `large`); optionally the reference "
        "distances of `reference_sequence` from the same resident rows. Returns a dict with "
        "nsamples, sequence_indices, kernel_ms and reference_distances.");
  m.def("autotune", &autotune, py::arg("path") = std::string(),
        "Times the pairwise kernel configurations on this GPU, keeps the fastest per "
        "(n, L, dtype) bucket and optionally saves the table as JSON");
  m.def("load_tuning", &load_tuning, py::arg("path"), "Loads a table saved by autotune");
  m.def("_kernel_launches", []() -> uint64_t {
    std::lock_guard<std::mutex> lk(g_mu);
    return g_ctx ? hd_ctx_kernel_launches(g_ctx) : 0;
  });
  // the module context's CUDA stream (cudaStream_t as an integer), on which
  // every call of this module runs: CUDA events recorded on it bracket calls
  m.def("_stream", []() -> uintptr_t {
    std::lock_guard<std::mutex> lk(g_mu);
    return reinterpret_cast<uintptr_t>(hd_ctx_stream(ctx()));
  });
}
