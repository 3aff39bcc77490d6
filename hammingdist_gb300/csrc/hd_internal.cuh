// Internal declarations shared by the libhd translation units: the context and
// alignment objects behind the C ABI, device buffers (the stream-ordered pool,
// large ones recycled by the library), a device-wide exclusive scan, and the
// PTX helpers (mbarrier, TMA) used by the pairwise kernel.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <cstdint>
#include <cstring>
#include <chrono>
#include <memory>
#include <string>
#include <utility>
#include <vector>

#include "../../include/hammingdist_gb300.h"

namespace hd {

// ---------------------------------------------------------------- errors
struct Error {
  int code;
  std::string msg;
};
[[noreturn]] inline void fail(int code, std::string msg) { throw Error{code, std::move(msg)}; }
inline void check_cuda(cudaError_t e, const char *what) {
  if (e != cudaSuccess) {
    if (e == cudaErrorMemoryAllocation) fail(HD_ERR_OOM, cudaGetErrorString(e));
    fail(HD_ERR_CUDA, std::string(cudaGetErrorString(e)) + " (" + what + ")");
  }
}
#define HD_CUDA(x) ::hd::check_cuda((x), #x)
#define HD_LAUNCHED(ctx)                                  \
  do {                                                    \
    ::hd::check_cuda(cudaGetLastError(), "kernel launch"); \
    (ctx)->launches++;                                     \
  } while (0)

// Status codes written by kernels into the context's device status word.
constexpr int kStatusOk = 0;
constexpr int kStatusTmaTimeout = 1;

inline uint64_t ceil_div(uint64_t a, uint64_t b) { return (a + b - 1) / b; }
inline uint64_t round_up(uint64_t a, uint64_t b) { return ceil_div(a, b) * b; }

// ------------------------------------------------------- device buffers
// Stream-ordered allocations from the device's default pool; the pool keeps
// freed memory (release threshold = max). Buffers of kBigBlock bytes or more
// are recycled by the library itself (big_alloc / big_release): a released
// one waits, with an event recorded on its stream at the release, for a
// later request of its size (up to 1/8 smaller), up to a cap per device. In
// steady-state calls of one shape, the pool's own large allocations took
// 0.7-2.5 ms of host time on some calls (about 1 ms per GB) and none on
// others, which left the GPU waiting for the next launch.
constexpr size_t kBigBlock = 32ull << 20;
void *big_alloc(size_t n, cudaStream_t s);
void big_release(void *p, cudaStream_t s);

struct DevBuf {
  void *p = nullptr;
  size_t bytes = 0;
  cudaStream_t s = nullptr;
  DevBuf() = default;
  DevBuf(size_t n, cudaStream_t stream) : bytes(n), s(stream) {
    if (n >= kBigBlock) p = big_alloc(n, stream);
    else if (n) HD_CUDA(cudaMallocAsync(&p, n, stream));
  }
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  DevBuf(DevBuf &&o) noexcept { *this = std::move(o); }
  DevBuf &operator=(DevBuf &&o) noexcept {
    if (this != &o) {
      release();
      p = o.p;
      bytes = o.bytes;
      s = o.s;
      o.p = nullptr;
      o.bytes = 0;
    }
    return *this;
  }
  ~DevBuf() { release(); }
  void release() {
    if (p) {
      if (bytes >= kBigBlock) big_release(p, s);
      else cudaFreeAsync(p, s);
    }
    p = nullptr;
    bytes = 0;
  }
  template <class T> T *as() const { return static_cast<T *>(p); }
};

}  // namespace hd

// -------------------------------------------------------------- objects
namespace hd {
// Per-call phase trace (off unless enabled): a CUDA event is recorded on the
// context's stream at each phase boundary and the durations are read once
// at the end of the call, so tracing adds no synchronisation inside a call.
// NVTX marks the call as a range and each boundary as a mark for profilers.
struct Trace {
  bool on = false;
  const char *call = nullptr;
  std::vector<cudaEvent_t> pool;
  std::vector<const char *> names;  // phase ending at event k (k >= 1)
  // points on other streams (trace_at): reported as times since the call began
  std::vector<cudaEvent_t> at_pool;
  std::vector<std::string> at_names;
  // host-side points (trace_host): milliseconds since the call began
  std::chrono::steady_clock::time_point t0;
  std::vector<std::pair<std::string, double>> host;
  std::string last;                 // text of the last traced call
};
// Kernel configuration of one matrix (autotuned per n, L and dtype bucket).
struct TileConfig {
  int tile = 128;    // bit-plane engine: tile edge (64 or 128 rows)
  int stages = 3;    // bit-plane engine: TMA staging depth
  int mma_band = 0;  // tensor-core engine: tile rows per L2 band (0: built-in)
  int mma_rows = 0;  // tensor-core engine: row tiles per item, 1 or 2 (0: built-in 2)
};
// The autotuner's table: a configuration per (n bucket, L bucket, dtype),
// and per L bucket the fewest single-row-tile items for which a launch goes
// to the tensor-core engine rather than the bit-plane engine.
struct TuneTable {
  std::vector<std::pair<uint32_t, TileConfig>> entries;
  uint64_t mma_min_items[4] = {0, 0, 0, 0};  // 0: built-in
};
}  // namespace hd

struct hd_ctx {
  int device = 0;
  int sm_count = 0;
  cudaStream_t stream = nullptr;  // compute
  cudaStream_t side = nullptr;    // copies that overlap compute
  std::string err;
  int *d_status = nullptr;        // kernel status word
  uint64_t launches = 0;
  cudaEvent_t ev_start = nullptr, ev_stop = nullptr;
  double last_pair_ms = 0.0;
  uint64_t last_pair_tiles = 0;
  PFN_cuTensorMapEncodeTiled_v12000 encode_tiled = nullptr;
  hd::DevBuf file;                // device copy of the last FASTA input
  // identity of the file whose bytes `file` holds (empty: none or other bytes)
  std::string file_tag;
  // records parsed from that file (an hd::Records), valid while parsed_tag ==
  // file_tag, for the record limit parsed_limit
  std::shared_ptr<void> parsed;
  std::string parsed_tag;
  uint64_t parsed_limit = 0;
  // autotuned kernel configurations
  hd::TuneTable tune;
  // engine choice for the autotuner's timings: -1 as configured, 0 the
  // bit-plane engine only, 1 the tensor-core engine at any launch size
  int engine_force = -1;
  // child contexts (own streams) for concurrent ingest of many inputs
  std::vector<hd_ctx *> workers;
  // pinned staging for file reads by this context (grows)
  void *pin = nullptr;
  size_t pin_cap = 0;
  // file reads: the copies into `file` run on `up`, with one event per 8 MB
  // part from part_ev (grows). map_files: the device reads pageable host
  // memory through the host's page tables, so a file's read-only mapping of
  // the page cache is copied directly (no CPU copy into `pin`).
  cudaStream_t up = nullptr;
  std::vector<cudaEvent_t> part_ev;
  int map_files = 0;
  hd::Trace trace;
};

namespace hd {
// Copies a launch table the planners built on the host to the device on
// stream s. A copy from pageable memory returns only once the stream has
// reached it (after the launches queued before it), which would hold the host
// back; tables up to 1 MB are staged in pinned memory instead (a ring of 8
// slots per device, kept for the life of the process, each reused once the
// copy it last staged has run), so the copy is queued like a launch. Larger
// tables go from pageable memory.
void upload_table(hd_ctx *ctx, void *d_dst, const void *host, size_t bytes, cudaStream_t s);

// tensor-core multiply-adds counted by the planning kernels (a 64-bit counter
// in the context's status block, after the status word)
inline unsigned long long *mma_mac_counter(const hd_ctx *ctx) {
  return reinterpret_cast<unsigned long long *>(reinterpret_cast<uint8_t *>(ctx->d_status) + 8);
}
}  // namespace hd

struct hd_alignment {
  hd_ctx *ctx = nullptr;  // creating context; may be destroyed before the alignment
  int device = 0;
  // a view (hd_alignment_view) borrows rows [row0, row0 + n_rows) of `base`
  const hd_alignment *base = nullptr;
  uint64_t row0 = 0;
  uint64_t n_input = 0;   // records read
  uint64_t n_rows = 0;    // rows after dedupe
  uint64_t length = 0;    // sites per row
  uint64_t words = 0;     // 32-site words per row, multiple of 8
  int rule = HD_RULE_AND;
  int groups = 1;         // plane groups of 4 planes (uint4 per word)
  int planes = 4;         // planes in use
  hd::DevBuf plane_buf[2];
  std::vector<uint64_t> seqidx;  // host, n_input entries (empty = identity)
  hd::DevBuf d_seqidx;           // device copy (serving / reference queries)
  // E2M1 (FP4) operand of the tensor-core engine (hd_mma.cu), rows [0, op_rows)
  // expanded so far out of op_cap; built on first use, freed with the
  // alignment
  mutable hd::DevBuf op;
  mutable uint64_t op_rows = 0, op_cap = 0;
  // per 256-site chunk of the operand (uint32 each): nonzero once an
  // expanded row has a '-' in it (the chunks whose dash products count)
  mutable hd::DevBuf op_dash;
  // Freed on the null stream: every API call has synchronised its own stream
  // before returning, so no queued work still reads these buffers, and the
  // creating context (and its streams) may already be gone.
  // device address of plane group g of this alignment (or view)
  const void *planes_ptr(int g) const {
    const hd_alignment *o = base ? base : this;
    return static_cast<const uint8_t *>(o->plane_buf[g].p) + row0 * words * 16;
  }
  ~hd_alignment() {
    cudaSetDevice(device);
    for (auto *b : {&plane_buf[0], &plane_buf[1], &d_seqidx, &op, &op_dash}) {
      b->s = nullptr;
      b->release();
    }
  }
};

namespace hd {

// --------------------------------------------------------- device scan
// Exclusive scan of n values (uint32 or uint64 input) into uint64 output;
// *d_total receives the sum. Three launches; any n.
constexpr int kScanThreads = 512;
constexpr int kScanItems = 8;
constexpr uint64_t kScanTile = (uint64_t)kScanThreads * kScanItems;

template <class T>
__device__ inline T warp_incl_scan(T v) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T u = __shfl_up_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) >= (unsigned)o) v += u;
  }
  return v;
}

template <class T>
__device__ inline T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide exclusive scan (blockDim.x multiple of 32, <= 1024).
template <class T>
__device__ inline T block_excl_scan(T v, T *warp_tmp /*[33]*/, T &total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  T inc = warp_incl_scan(v);
  if (lane == 31) warp_tmp[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    T w = lane < nw ? warp_tmp[lane] : T(0);
    T wi = warp_incl_scan(w);
    if (lane < nw) warp_tmp[lane] = wi - w;
    if (lane == nw - 1) warp_tmp[32] = wi;
  }
  __syncthreads();
  T res = warp_tmp[warp] + inc - v;
  total = warp_tmp[32];
  __syncthreads();
  return res;
}

template <class In>
__global__ void k_scan_reduce(const In *in, uint64_t n, uint64_t *block_sums) {
  __shared__ uint64_t tmp[33];
  uint64_t base = (uint64_t)blockIdx.x * kScanTile + (uint64_t)threadIdx.x * kScanItems;
  uint64_t s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k)
    if (base + k < n) s += (uint64_t)in[base + k];
  uint64_t tot;
  block_excl_scan<uint64_t>(s, tmp, tot);
  if (threadIdx.x == 0) block_sums[blockIdx.x] = tot;
}

// One block scans the block sums in place (exclusive) and writes the total.
template <class Dummy = void>
__global__ void k_scan_top(uint64_t *sums, uint64_t nb, uint64_t *d_total) {
  __shared__ uint64_t tmp[33];
  uint64_t carry = 0;
  for (uint64_t b0 = 0; b0 < nb; b0 += blockDim.x) {
    uint64_t i = b0 + threadIdx.x;
    uint64_t v = i < nb ? sums[i] : 0;
    uint64_t tot;
    uint64_t ex = block_excl_scan<uint64_t>(v, tmp, tot);
    if (i < nb) sums[i] = carry + ex;
    carry += tot;
  }
  if (threadIdx.x == 0 && d_total) *d_total = carry;
}

template <class In>
__global__ void k_scan_down(const In *in, uint64_t *out, uint64_t n, const uint64_t *block_off) {
  __shared__ uint64_t tmp[33];
  uint64_t base = (uint64_t)blockIdx.x * kScanTile + (uint64_t)threadIdx.x * kScanItems;
  uint64_t v[kScanItems];
  uint64_t s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    v[k] = base + k < n ? (uint64_t)in[base + k] : 0;
    s += v[k];
  }
  uint64_t tot;
  uint64_t off = block_excl_scan<uint64_t>(s, tmp, tot) + block_off[blockIdx.x];
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    if (base + k < n) out[base + k] = off;
    off += v[k];
  }
}

template <class In>
void scan_exclusive(hd_ctx *ctx, const In *in, uint64_t *out, uint64_t n, uint64_t *d_total) {
  uint64_t nb = ceil_div(n ? n : 1, kScanTile);
  DevBuf sums(nb * sizeof(uint64_t), ctx->stream);
  k_scan_reduce<In><<<(unsigned)nb, kScanThreads, 0, ctx->stream>>>(in, n, sums.as<uint64_t>());
  HD_LAUNCHED(ctx);
  k_scan_top<void><<<1, 1024, 0, ctx->stream>>>(sums.as<uint64_t>(), nb, d_total);
  HD_LAUNCHED(ctx);
  k_scan_down<In><<<(unsigned)nb, kScanThreads, 0, ctx->stream>>>(in, out, n, sums.as<uint64_t>());
  HD_LAUNCHED(ctx);
}

// ------------------------------------------------------- PTX helpers
__device__ inline uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ inline void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ inline void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ inline void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ inline bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ inline uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// Waits for the barrier phase with a wall-clock limit; false = gave up.
__device__ inline bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, uint64_t limit_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  for (;;) {
    if (mbar_try_wait(bar, parity)) return true;
    if (global_ns() - t0 > limit_ns) return false;
  }
}
// 2-D tiled TMA load (global -> shared), completion counted on `bar`.
__device__ inline void tma_load_2d(void *smem_dst, const CUtensorMap *map, int32_t x, int32_t y,
                                   uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(smem_dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}
__device__ inline void prefetch_tmap(const CUtensorMap *map) {
  asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}

// ------------------------------------------------- parsed FASTA records
// Records on the device: record r is rec_len[r] bytes at base + rec_start[r].
struct Records {
  uint64_t n = 0;          // records kept (after the n limit)
  uint64_t len0 = 0;       // length of record 0
  uint64_t max_len = 0;
  bool all_equal = true;
  const uint8_t *base = nullptr;
  uint64_t bytes = 0;         // readable bytes from base: [base, base + bytes)
  DevBuf rec_start, rec_len;  // uint64 [n]
  DevBuf gathered;            // concatenation when records span several lines
  // the dense-rule rows of these records, when the call that parsed them
  // built them (row_of[r]: device row of record r; none: row r): reference
  // distances of the same file read these instead of the records' bytes
  std::shared_ptr<hd_alignment> rows;
  DevBuf row_of;
};

// Character codes of the rules (bit p = bit plane p); '-' is all ones.
enum CodeTable { kCodesAnd = 0, kCodesSparse = 1, kCodesSparseX = 2, kNumCodeTables = 3 };
void code_table(int table, uint8_t out[256]);
inline int planes_of(int rule) { return rule == HD_RULE_AND ? 4 : rule == HD_RULE_SPARSE ? 5 : 6; }

// ----------------------------------------------------- stage launchers
// ingest.cu
// d_file must be 16-byte aligned (the newline scan reads 16-byte vectors)
// first > 0: the bytes before offset `first` (a '\n' precedes it, and a
// header starts there) end records parsed before, from an earlier part of the
// same file; the records up to that header are left out
Records parse_fasta(hd_ctx *ctx, const uint8_t *d_file, uint64_t nbytes, uint64_t n_limit,
                    uint64_t first = 0);
Records records_from_offsets(hd_ctx *ctx, const uint8_t *d_bytes, const uint64_t *h_offsets,
                             uint64_t n);
// Deduplicates: returns the unique records (first-occurrence order) as a list
// of record indices on the device and fills seqidx (host, n entries).
DevBuf dedupe(hd_ctx *ctx, const Records &rec, uint64_t *n_unique, std::vector<uint64_t> &seqidx);
// Duplicate removal over a growing record set (the parts of a streamed
// FASTA file): records [0, seen) are resolved, and add() hashes, inserts and
// verifies only the records after them. Earlier records hold the smaller
// indices, so they stay the first occurrences and their rows keep their
// numbers; unique_rec lists the unique rows' records (n_unique of them) and
// rowid (device) each record's row, which rows() copies to the host. A new
// record unlike the first record of its hash (a 64-bit collision), or more
// records than the capacity, makes add() return false: the caller runs the
// full dedupe.
struct IncDedupe {
  DevBuf hash, dup, rowid, unique_rec, list, next, flag, uidx, keys, mins, cnt;
  uint64_t cap = 0, T = 0, seen = 0, n_unique = 0;
  void init(hd_ctx *ctx, uint64_t capacity);
  bool add(hd_ctx *ctx, const Records &rec);
  void rows(hd_ctx *ctx, std::vector<uint64_t> &seqidx);  // records [0, seen)
};
// Sum over sites of the most frequent of A/C/G/T among the given rows.
uint64_t consensus_matches(hd_ctx *ctx, const Records &rec, const uint64_t *d_rows,
                           uint64_t n_rows);
// Packs rows (record ids d_rows, or identity if null) into bit planes.
void pack_rows(hd_ctx *ctx, const Records &rec, const uint64_t *d_rows, hd_alignment *aln);
// AND-rule planes of n_rows records (d_rows: record indices) into g0, and
// into g1 too unless it is null (n_rows x words uint4 each, already allocated)
void pack_rows_and(hd_ctx *ctx, const Records &rec, const uint64_t *d_rows, uint64_t n_rows,
                   uint64_t length, uint64_t words, uint4 *g0, uint4 *g1 = nullptr);
// records of a then b (b's starts shifted by b_off), one base; b parsed from
// bytes that follow a's in the same buffer
Records concat_records(hd_ctx *ctx, const Records &a, const Records &b, uint64_t b_off,
                       uint64_t bytes);
void reference_distances_device(hd_ctx *ctx, const Records &rec, const uint8_t *d_ref,
                                int include_x, uint32_t *d_out);
void alignment_query_distances(hd_ctx *ctx, const hd_alignment *aln, const uint8_t *d_query,
                               uint32_t *d_out_rows);
// the query's distance to every row (d_rows, n_rows entries), then per record
// r < n the distance of its row (row_of[r], or row r without row_of) into
// d_out; queued on the context's stream
void query_rows_to_records(hd_ctx *ctx, const hd_alignment *aln, const uint8_t *d_query,
                           uint32_t *d_rows, const uint64_t *row_of, uint64_t n, uint32_t *d_out);
// same without synchronising: q_planes holds the packed query until the caller syncs
void query_distances_async(hd_ctx *ctx, const hd_alignment *aln, const uint8_t *d_query,
                           uint32_t *d_out_rows, DevBuf &q_planes);

// pairwise.cu: tiles of rows [tile_lo*128, tile_hi*128) x all earlier columns
// into out (lt index out_base maps to out[0]).
void pairwise_tiles(hd_ctx *ctx, const hd_alignment *aln, int dtype_bytes, uint32_t max_dist,
                    void *d_out, uint64_t out_base, uint32_t tile_lo, uint32_t tile_hi);
constexpr uint32_t kTile = 128;
// columns of a tensor-core work item (the N of its MMAs)
constexpr uint32_t kMmaCols = 240;
// bytes of the tensor-core engine's E2M1 operand per 32-site word of a row
// of the dense AND rule (6 blocks of 16 bytes: 4 planes and 2 dash blocks)
constexpr uint32_t kMmaOperandBytesPerWord = 96;

// Kernel configuration of one job: tile edge (64 or 128 rows; 4 or 8 rows
// per thread) and TMA staging depth.
// One matrix (or a range of its tile rows, in units of cfg.tile) for the
// persistent engine.
struct PairJobSpec {
  const hd_alignment *aln = nullptr;
  int dtype = 1;
  uint32_t max_dist = 255;
  void *d_out = nullptr;
  uint64_t out_base = 0;
  uint32_t tile_lo = 0, tile_hi = 0;
  TileConfig cfg;
};
struct PairLaunchPlan {
  struct Launch {
    const void *fn = nullptr;  // kernel
    int smem = 0, tile = 0, stages = 0;
    uint64_t grid = 0, tiles = 0, jobs = 0;
    const void *d_jobs = nullptr;
    unsigned long long *d_counter = nullptr;
    bool mma = false;              // the tensor-core engine (hd_mma.cu): d_items holds
    const void *d_items = nullptr; // its work items, `tiles` of them
    bool queue = false;            // its CTAs draw items from d_counter (else round-robin)
  };
  std::vector<Launch> launches;
  std::vector<DevBuf> blocks;  // job tables + tensor maps + tile counters
};
void prepare_pairwise_jobs(hd_ctx *ctx, std::vector<PairJobSpec> &specs, cudaStream_t stream,
                           PairLaunchPlan *plan,
                           int sm_limit = 0);
void launch_pairwise_plan(hd_ctx *ctx, PairLaunchPlan &plan, cudaStream_t stream);
// pairwise_tiles in two steps: the plan (host work and the job-table upload
// on ctx->stream), then launch_pairwise_plan on ctx->stream
void plan_pairwise_tiles(hd_ctx *ctx, const hd_alignment *aln, int dtype_bytes, uint32_t max_dist,
                         void *d_out, uint64_t out_base, uint32_t tile_lo, uint32_t tile_hi,
                         PairLaunchPlan *plan);
void run_pairwise_jobs(hd_ctx *ctx, std::vector<PairJobSpec> &specs, cudaStream_t stream,
                       PairLaunchPlan *keep);
void make_tmap(hd_ctx *ctx, CUtensorMap *tm, const void *base, uint64_t words, uint64_t rows,
               uint32_t tile);
TileConfig default_tile_config(uint64_t n_rows, uint64_t length, int dtype_bytes);
bool tile_config_valid(int tile, int stages);
// tune.cu: the autotuned table (or the default) for (n, L, dtype)
TileConfig tile_config_for(hd_ctx *ctx, uint64_t n_rows, uint64_t length, int dtype_bytes);
// the tensor-core engine's minimum launch size (single-row-tile items) for
// rows of `length` sites: HAMMINGDIST_MMA_MIN_ITEMS, else the table, else
// the built-in value
uint64_t mma_min_items_for(hd_ctx *ctx, uint64_t length);
// mma.cu: the tensor-core engine's L2 band (tile rows) and row tiles per item
// for a configuration: HAMMINGDIST_MMA_BAND / HAMMINGDIST_MMA_ROWS, else the
// configuration's own, else the built-in 16 and 2
int mma_band_of(const TileConfig &c);
int mma_rows_of(const TileConfig &c);

// mma.cu: the tensor-core engine for every rule (4, 5 or 6 planes, with
// P L < 2^24; HAMMINGDIST_KERNEL=lop3 turns it off).
bool mma_eligible(const hd_alignment *aln);
// expands rows [op_rows, rows) of the alignment's planes into its E2M1
// operand on `stream` (room for cap_hint rows if it must grow); false if the
// operand cannot be allocated
bool ensure_operand(hd_ctx *ctx, const hd_alignment *aln, uint64_t rows, cudaStream_t stream,
                uint64_t cap_hint = 0);
// tile rows [tile_lo, tile_hi) (128 rows each) x all earlier columns into
// d_out (lt index out_base at d_out[0]) on `stream`; sm_limit > 0 caps the
// persistent grid. False when the alignment is not eligible (the caller
// runs the bit-plane engine).
bool pairwise_mma(hd_ctx *ctx, const hd_alignment *aln, int dtype_bytes, uint32_t max_dist,
                  void *d_out, uint64_t out_base, uint32_t tile_lo, uint32_t tile_hi,
                  cudaStream_t stream, int sm_limit);
// dense FP4 (kind::mxf4) MMA rate (FLOP/s) of this device from shared-memory operands
double measure_mma_peak(hd_ctx *ctx);
// One tensor-core launch for the specs it can take (dense AND rule, row
// range starting on a 128-row tile, operand memory available); taken[k] marks
// them. The plan keeps the launch's device block.
void prepare_mma_jobs(hd_ctx *ctx, const std::vector<PairJobSpec> &specs, cudaStream_t stream,
                      PairLaunchPlan *plan, int sm_limit, std::vector<char> &taken);
void launch_mma(hd_ctx *ctx, const PairLaunchPlan::Launch &L, cudaStream_t stream);

// format.cu: text of rows [i_lo, i_hi) of a lower triangle held on the
// device (lt index lt_base at d_lt[0]). Returns bytes written to d_text
// (capacity checked by the caller via the *_bound functions).
uint64_t lt_text_bound(uint64_t i_lo, uint64_t i_hi, int dtype_bytes);
// full n x n matrix text (DataSet::dump) of rows [i_lo, i_hi) from the whole
// device-resident triangle of `entries` values
uint64_t full_text_bound(uint64_t n, uint64_t i_lo, uint64_t i_hi, int dtype_bytes);
uint64_t format_full_rows(hd_ctx *ctx, const void *d_lt, uint64_t entries, int dtype_bytes,
                          uint64_t n, uint64_t i_lo, uint64_t i_hi, char *d_text);
// positions of every '\n' of a device buffer, in order (*m_nl of them)
DevBuf newline_positions(hd_ctx *ctx, const uint8_t *d, uint64_t nbytes, uint64_t *m_nl);
// result-file readers (hd_results.cu): see hd_read_lower_triangular / hd_read_csv
struct ParsedValues {
  uint64_t entries = 0;   // values produced
  uint64_t nsamples = 0;  // as the reference infers it
  int error = 0;          // 0, or 1 = a field without digits, 2 = a value outside int
  DevBuf values;          // entries x dtype bytes on the device
};
ParsedValues read_lower_triangular_device(hd_ctx *ctx, const uint8_t *d, uint64_t nbytes,
                                          int dtype_bytes);
ParsedValues read_csv_device(hd_ctx *ctx, const uint8_t *d, uint64_t nbytes);
uint64_t format_lt_rows(hd_ctx *ctx, const void *d_lt, int dtype_bytes, uint64_t lt_base,
                        uint64_t i_lo, uint64_t i_hi, char *d_text);
// Sparse lines of rows [i_lo, i_hi): counts text bytes per row into
// d_row_bytes (uint64 [i_hi-i_lo]) and lines into *n_lines.
void sparse_row_sizes(hd_ctx *ctx, const void *d_lt, int dtype_bytes, uint64_t lt_base,
                      uint64_t i_lo, uint64_t i_hi, int64_t threshold, uint64_t *d_row_bytes,
                      uint64_t *d_row_lines);
uint64_t format_sparse_rows(hd_ctx *ctx, const void *d_lt, int dtype_bytes, uint64_t lt_base,
                            uint64_t i_lo, uint64_t i_hi, int64_t threshold,
                            const uint64_t *d_row_bytes, char *d_text);

// peak.cu
void measure_int_peaks(hd_ctx *ctx, double *lop3, double *popc, double *mix);

// phase tracing of one API call (no-ops unless ctx->trace.on)
void trace_begin(hd_ctx *ctx, const char *call);
void trace_mark(hd_ctx *ctx, const char *phase);
// a point on stream s (e.g. a launch's end on a side stream), listed after the
// phases with its time since the call began
void trace_at(hd_ctx *ctx, const std::string &what, cudaStream_t s);
// a point of the host thread, listed with its time since the call began
void trace_host(hd_ctx *ctx, const std::string &what);
void trace_end(hd_ctx *ctx);

}  // namespace hd
