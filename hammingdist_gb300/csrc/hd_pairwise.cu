// The bit-plane pairwise lower-triangle engine, and the job planner both
// engines share.
//
// Replaces the reference's Dist<T> kernel and its chunked driver
// (src/distance_cuda.cu:9-202), which computes one lower-triangle entry per
// CTA from the nibble-packed rows with a shared-memory reduction and re-reads
// both rows from memory for every pair. prepare_pairwise_jobs first gives
// the tensor-core engine (hd_mma.cu) every job it can take; this engine
// computes the rest: launches too small to fill the SMs with the tensor-core
// engine's coarser items, and rows too long for its FP32 sums.
//
// One persistent kernel serves a single matrix and a batch of independent
// matrices alike: CTAs draw tiles from a device counter over a table of jobs
// (alignment, output, dtype, max_dist), biggest jobs first. A tile is a
// TILE x TILE block (I, J), J <= I, of one job's lower triangle:
//  * rows are bit planes: per 32-site word one uint32 per plane, 4 planes per
//    16-byte group (uint4); sites match when their codes share a plane bit
//    (the reference's "(a & b) nibble != 0", src/distance_cuda.cu:57-65, with
//    the codes of src/hamming_impl.cc:23-44);
//  * TMA (cp.async.bulk.tensor, 128-byte swizzle) stages 8 words (256 sites)
//    of the TILE A-rows and TILE B-rows per stage into shared memory, STAGES
//    deep, completion tracked by mbarriers with bounded waits;
//  * each of the 256 threads owns an R x R block of pairs (R = TILE / 16) and,
//    per word, counts matching sites as popc((a0&b0)|(a1&b1)|(a2&b2)|(a3&b3)):
//    four LOP3 and one POPC per 32 pair-sites; mismatches = sites - matches,
//    as every padded site matches;
//  * the epilogue saturates with min(count, max_dist) (safe_int_cast,
//    include/hamming/hamming_impl.hh:37-45), stages the tile in shared memory
//    and writes each row's contiguous lower-triangle span in the job's dtype.
#include <algorithm>
#include <mutex>

#include "hd_internal.cuh"

namespace hd {

constexpr int kThreads = 256;
constexpr int kKW = 8;                          // words per stage
constexpr uint64_t kWaitNs = 2000000000ull;     // TMA wait limit: 2 s
constexpr uint32_t kBand = 16;                  // tile rows per L2 band

struct PairJob {
  const CUtensorMap *tmap0;  // device copies of the job's tensor maps
  const CUtensorMap *tmap1;
  void *out;                 // device output; lt index out_base at out[0]
  unsigned long long out_base;
  unsigned long long tile_begin;  // first global tile index of the job
  uint32_t n, nk, max_dist, row_lo, row_hi;  // tile rows [row_lo, row_hi)
  uint32_t dtype;                            // 1, 2 or 4 bytes
};

template <int TILE, int STAGES, int G>
struct Cfg {
  static constexpr int R = TILE / 16;                    // rows (and columns) per thread
  static constexpr int box_bytes = TILE * kKW * 16;      // TILE rows x 128 B
  static constexpr int stage_bytes = G * 2 * box_bytes;
  static constexpr int smem_bytes = STAGES * stage_bytes + 1024;
  static constexpr int min_blocks = (TILE == 128 && G == 1 && STAGES <= 3) ? 2
                                    : (TILE == 64 ? 3 : 1);
};

__device__ __forceinline__ uint32_t mad_acc(uint32_t acc, uint32_t p, uint32_t one) {
  // acc + p * one as IMAD (FMA pipe): `one` is a kernel argument (always 1)
  // the compiler cannot fold, which keeps the add off the ALU pipe
  uint32_t d;
  asm("mad.lo.u32 %0, %1, %2, %3;" : "=r"(d) : "r"(p), "r"(one), "r"(acc));
  return d;
}

// x | (y & z) as one LOP3 (truth table 0xF8).
__device__ __forceinline__ uint32_t or_and(uint32_t x, uint32_t y, uint32_t z) {
  uint32_t d;
  asm("lop3.b32 %0, %1, %2, %3, 0xF8;" : "=r"(d) : "r"(x), "r"(y), "r"(z));
  return d;
}

__device__ inline uint32_t tri_root(uint64_t t) {
  uint32_t i = (uint32_t)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
  while ((uint64_t)(i + 1) * (i + 2) / 2 <= t) ++i;
  while ((uint64_t)i * (i + 1) / 2 > t) --i;
  return i;
}

// Tile (I, J) for row-major tile number t (t = I(I+1)/2 + J over all tile
// rows) within tile rows [row_lo, row_hi). Inside each band of kBand tile
// rows the order is column-major over the band's rectangle (J < I_lo) and
// row-major over its triangle, so the CTAs resident at one time share the
// band's A tiles and each B tile in L2.
__device__ inline void tile_of(uint64_t t, uint32_t row_lo, uint32_t row_hi, uint32_t &I,
                               uint32_t &J) {
  const uint32_t Ir = tri_root(t);
  const uint32_t I_lo = row_lo + (Ir - row_lo) / kBand * kBand;
  const uint32_t I_hi = min(I_lo + kBand, row_hi);
  const uint32_t h = I_hi - I_lo;
  const uint64_t u = t - (uint64_t)I_lo * (I_lo + 1) / 2;
  const uint64_t rect = (uint64_t)h * I_lo;
  if (u < rect) {
    J = (uint32_t)(u / h);
    I = I_lo + (uint32_t)(u % h);
  } else {
    const uint64_t v = u - rect;
    const uint32_t i = tri_root(v);
    I = I_lo + i;
    J = I_lo + (uint32_t)(v - (uint64_t)i * (i + 1) / 2);
  }
}

template <int TILE, typename T>
__device__ inline void store_tile(uint8_t *smem, const uint32_t (&acc)[TILE / 16][TILE / 16],
                                  uint32_t sites, uint32_t max_dist, uint32_t ty, uint32_t tx,
                                  const PairJob &job, uint32_t I, uint32_t J) {
  constexpr int R = TILE / 16;
  T *tile = reinterpret_cast<T *>(smem);
#pragma unroll
  for (int r = 0; r < R; ++r)
#pragma unroll
    for (int c = 0; c < R; ++c) {
      const uint32_t mism = sites - acc[r][c];
      tile[(ty + 16 * r) * TILE + tx + 16 * c] = (T)(mism < max_dist ? mism : max_dist);
    }
  __syncthreads();
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  T *out = static_cast<T *>(job.out);
  for (uint32_t rl = warp; rl < (uint32_t)TILE; rl += kThreads / 32) {
    const uint32_t i = I * TILE + rl;
    if (i >= job.n) break;
    const uint32_t ncols = (I == J) ? rl : (uint32_t)TILE;
    if (!ncols) continue;
    T *dst = out + ((uint64_t)i * (i - 1) / 2 + (uint64_t)J * TILE - job.out_base);
    for (uint32_t c = lane; c < ncols; c += 32) dst[c] = tile[rl * TILE + c];
  }
}

template <int TILE, int STAGES, int G, int P>
__global__ void __launch_bounds__(kThreads, Cfg<TILE, STAGES, G>::min_blocks)
    k_pairwise(const PairJob *__restrict__ jobs, uint32_t n_jobs, unsigned long long total_tiles,
               unsigned long long *counter, uint32_t one, int *status) {
  using C = Cfg<TILE, STAGES, G>;
  constexpr int R = C::R;
  constexpr uint32_t SB = C::stage_bytes;
  constexpr uint32_t BOX = C::box_bytes;
  extern __shared__ uint8_t smem_raw[];
  __shared__ __align__(8) uint64_t full[STAGES];
  __shared__ unsigned long long s_tile;
  __shared__ uint32_t s_job;
  uint8_t *smem =
      reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));

  const uint32_t tid = threadIdx.x;
  if (tid == 0) {
#pragma unroll
    for (int s = 0; s < STAGES; ++s) mbar_init(&full[s], 1);
    fence_mbar_init();
  }
  // thread (ty, tx) owns rows ty + 16 r and columns tx + 16 c of the tile;
  // with the 128-byte swizzle, 16-byte chunk w of smem row q sits at chunk
  // w ^ (q & 7), and q & 7 is ty & 7 (tx & 7) for all of a thread's rows.
  const uint32_t ty = tid >> 4, tx = tid & 15;
  const uint32_t a_off = ty * 128, b_off = tx * 128, a_sw = ty & 7, b_sw = tx & 7;
  uint32_t gk = 0;  // chunks this CTA has consumed, over all its tiles (mbarrier phases)

  for (;;) {
    if (tid == 0) {
      const unsigned long long g = atomicAdd(counter, 1ull);
      s_tile = g;
      if (g < total_tiles) {  // job of tile g: last job with tile_begin <= g
        uint32_t lo = 0, hi = n_jobs - 1;
        while (lo < hi) {
          const uint32_t mid = (lo + hi + 1) >> 1;
          if (jobs[mid].tile_begin <= g) lo = mid;
          else hi = mid - 1;
        }
        s_job = lo;
      }
    }
    __syncthreads();
    const unsigned long long g = s_tile;
    if (g >= total_tiles) break;
    const PairJob &job = jobs[s_job];
    const uint32_t nk = job.nk;
    uint32_t I, J;
    tile_of((uint64_t)job.row_lo * (job.row_lo + 1) / 2 + (g - job.tile_begin), job.row_lo,
            job.row_hi, I, J);

    auto issue = [&](uint32_t k, uint32_t kc) {  // chunk kc of this tile into stage k % STAGES
      const int s = k % STAGES;
      uint8_t *st = smem + s * SB;
      mbar_expect_tx(&full[s], SB);
      const int32_t x = (int32_t)(kc * 32);  // uint32 elements: 128 B per chunk
      tma_load_2d(st, job.tmap0, x, (int32_t)(I * TILE), &full[s]);
      tma_load_2d(st + BOX, job.tmap0, x, (int32_t)(J * TILE), &full[s]);
      if constexpr (G == 2) {
        tma_load_2d(st + 2 * BOX, job.tmap1, x, (int32_t)(I * TILE), &full[s]);
        tma_load_2d(st + 3 * BOX, job.tmap1, x, (int32_t)(J * TILE), &full[s]);
      }
    };
    if (tid == 0)
      for (uint32_t kc = 0; kc < (uint32_t)(STAGES - 1) && kc < nk; ++kc) issue(gk + kc, kc);

    uint32_t acc[R][R];
#pragma unroll
    for (int r = 0; r < R; ++r)
#pragma unroll
      for (int c = 0; c < R; ++c) acc[r][c] = 0;

    bool timed_out = false;
    for (uint32_t kc = 0; kc < nk; ++kc) {
      const uint32_t k = gk + kc;
      const int s = k % STAGES;
      if (tid == 0 && kc + STAGES - 1 < nk) issue(k + STAGES - 1, kc + STAGES - 1);
      if (!mbar_wait_bounded(&full[s], (k / STAGES) & 1u, kWaitNs)) timed_out = true;
      const uint8_t *A = smem + s * SB;
      const uint8_t *B = A + BOX;
#pragma unroll 1
      for (uint32_t w = 0; w < (uint32_t)kKW; ++w) {
        const uint32_t ca = (w ^ a_sw) << 4, cb = (w ^ b_sw) << 4;
        uint4 a[R];
#pragma unroll
        for (int r = 0; r < R; ++r)
          a[r] = *reinterpret_cast<const uint4 *>(A + a_off + r * (16 * 128) + ca);
        uint32_t a4[R], a5[R];
        if constexpr (G == 2) {
#pragma unroll
          for (int r = 0; r < R; ++r) {
            const uint8_t *p1 = A + 2 * BOX + a_off + r * (16 * 128) + ca;
            a4[r] = *reinterpret_cast<const uint32_t *>(p1);
            a5[r] = P == 6 ? *reinterpret_cast<const uint32_t *>(p1 + 4) : 0u;
          }
        }
#pragma unroll
        for (int c = 0; c < R; ++c) {
          const uint4 b = *reinterpret_cast<const uint4 *>(B + b_off + c * (16 * 128) + cb);
          uint32_t b4 = 0, b5 = 0;
          if constexpr (G == 2) {
            const uint8_t *q1 = B + 2 * BOX + b_off + c * (16 * 128) + cb;
            b4 = *reinterpret_cast<const uint32_t *>(q1);
            if (P == 6) b5 = *reinterpret_cast<const uint32_t *>(q1 + 4);
          }
#pragma unroll
          for (int r = 0; r < R; ++r) {
            uint32_t m = a[r].x & b.x;
            m = or_and(m, a[r].y, b.y);
            m = or_and(m, a[r].z, b.z);
            m = or_and(m, a[r].w, b.w);
            if constexpr (G == 2) {
              m = or_and(m, a4[r], b4);
              if (P == 6) m = or_and(m, a5[r], b5);
            }
            acc[r][c] = mad_acc(acc[r][c], __popc(m), one);
          }
        }
      }
      if (__syncthreads_or(timed_out)) {
        if (tid == 0) {
          atomicExch(status, kStatusTmaTimeout);
          // wait (bounded) for this CTA's copies still in flight, then leave
          for (uint32_t k2 = kc + 1; k2 < nk && k2 < kc + STAGES; ++k2)
            mbar_wait_bounded(&full[(gk + k2) % STAGES], ((gk + k2) / STAGES) & 1u, kWaitNs);
        }
        return;
      }
    }
    gk += nk;

    const uint32_t sites = nk * kKW * 32;
    if (job.dtype == 1)
      store_tile<TILE, uint8_t>(smem, acc, sites, job.max_dist, ty, tx, job, I, J);
    else if (job.dtype == 2)
      store_tile<TILE, uint16_t>(smem, acc, sites, job.max_dist, ty, tx, job, I, J);
    else
      store_tile<TILE, uint32_t>(smem, acc, sites, job.max_dist, ty, tx, job, I, J);
    __syncthreads();  // the next tile's loads reuse the staging memory
  }
}

// ------------------------------------------------------------------ host side
void make_tmap(hd_ctx *ctx, CUtensorMap *tm, const void *base, uint64_t words, uint64_t rows,
               uint32_t tile) {
  cuuint64_t dims[2] = {words * 4, rows};
  cuuint64_t strides[1] = {words * 16};
  cuuint32_t box[2] = {32, tile};
  cuuint32_t es[2] = {1, 1};
  CUresult r = ctx->encode_tiled(tm, CU_TENSOR_MAP_DATA_TYPE_UINT32, 2, const_cast<void *>(base),
                                 dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                 CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                 CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS)
    fail(HD_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
}

namespace {

using KernelFn = void (*)(const PairJob *, uint32_t, unsigned long long, unsigned long long *,
                          uint32_t, int *);

struct Variant {
  KernelFn fn;
  int smem;
  int tile;
  int stages;
  int groups;
  int planes;
};

template <int TILE, int STAGES, int G, int P>
Variant make_variant() {
  return {k_pairwise<TILE, STAGES, G, P>, Cfg<TILE, STAGES, G>::smem_bytes, TILE, STAGES, G, P};
}

const std::vector<Variant> &variants() {
  static const std::vector<Variant> v = {
      make_variant<128, 3, 1, 4>(), make_variant<128, 2, 1, 4>(), make_variant<128, 4, 1, 4>(),
      make_variant<64, 3, 1, 4>(),  make_variant<64, 4, 1, 4>(),  make_variant<128, 3, 2, 5>(),
      make_variant<128, 3, 2, 6>(), make_variant<64, 3, 2, 5>(),  make_variant<64, 3, 2, 6>(),
  };
  return v;
}

const Variant &find_variant(int tile, int stages, int planes) {
  for (const auto &v : variants())
    if (v.tile == tile && v.stages == stages && v.planes == planes) return v;
  // sparse-rule alignments are built in three stages only
  for (const auto &v : variants())
    if (v.tile == tile && v.planes == planes) return v;
  fail(HD_ERR_ARG, "no pairwise kernel variant for this configuration");
}

int resident_ctas(const Variant &v) {
  static std::mutex mu;
  static std::vector<std::pair<KernelFn, int>> cache;  // per variant
  std::lock_guard<std::mutex> lk(mu);
  for (auto &e : cache)
    if (e.first == v.fn) return e.second;
  HD_CUDA(cudaFuncSetAttribute(v.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, v.smem));
  int per_sm = 0;
  HD_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, v.fn, kThreads, v.smem));
  if (per_sm < 1) fail(HD_ERR_CUDA, "pairwise kernel does not fit on an SM");
  cache.emplace_back(v.fn, per_sm);
  return per_sm;
}

}  // namespace

TileConfig default_tile_config(uint64_t n_rows, uint64_t length, int dtype_bytes) {
  (void)length;
  (void)dtype_bytes;
  TileConfig c;
  c.tile = n_rows <= 384 ? 64 : 128;
  c.stages = 3;
  return c;
}

bool tile_config_valid(int tile, int stages) {
  for (const auto &v : variants())
    if (v.tile == tile && v.stages == stages && v.planes == 4) return true;
  return false;
}

// Groups the jobs by kernel variant and uploads one job table (+ tensor maps
// + tile counter) per group; the launches are recorded in the plan, and
// launch_pairwise_plan issues them. Outside a graph the two run back to back;
// a batch captures only the launch step and replays it.
void prepare_pairwise_jobs(hd_ctx *ctx, std::vector<PairJobSpec> &specs, cudaStream_t stream,
                           PairLaunchPlan *plan, int sm_limit) {
  // the dense AND rule goes to the tensor-core engine, one launch for all of it
  std::vector<char> taken;
  prepare_mma_jobs(ctx, specs, stream, plan, sm_limit, taken);
  struct Group {
    const Variant *v;
    std::vector<size_t> idx;
  };
  std::vector<Group> groups;
  for (size_t k = 0; k < specs.size(); ++k) {
    PairJobSpec &s = specs[k];
    if (taken[k] || s.aln->n_rows < 2 || s.tile_hi <= s.tile_lo) continue;
    if (s.aln->n_rows > 0xffffffffull) fail(HD_ERR_ARG, "too many rows");
    const Variant *v = &find_variant(s.cfg.tile, s.cfg.stages, s.aln->planes);
    s.cfg.tile = v->tile;
    s.cfg.stages = v->stages;
    auto it = std::find_if(groups.begin(), groups.end(), [&](const Group &g) { return g.v == v; });
    if (it == groups.end()) groups.push_back({v, {k}});
    else it->idx.push_back(k);
  }
  for (auto &grp : groups) {
    const Variant &v = *grp.v;
    auto cost = [&](size_t a) {
      const PairJobSpec &x = specs[a];
      return (double)x.aln->words *
             ((double)x.tile_hi * (x.tile_hi + 1) - (double)x.tile_lo * (x.tile_lo + 1));
    };
    // biggest jobs first: the long tiles start early and small ones fill the tail
    std::stable_sort(grp.idx.begin(), grp.idx.end(),
                     [&](size_t a, size_t b) { return cost(a) > cost(b); });
    const size_t nj = grp.idx.size();
    // one device block: [tensor maps (2 per job, 64-B aligned)][jobs][counter]
    const size_t tm_bytes = nj * 2 * sizeof(CUtensorMap);
    const size_t job_bytes = round_up(nj * sizeof(PairJob), 64);
    std::vector<uint8_t> host(tm_bytes + job_bytes + 64, 0);
    DevBuf dev(host.size(), stream);
    auto *tms = reinterpret_cast<CUtensorMap *>(host.data());
    auto *pj = reinterpret_cast<PairJob *>(host.data() + tm_bytes);
    const auto *d_tms = reinterpret_cast<const CUtensorMap *>(dev.p);
    unsigned long long tiles = 0;
    for (size_t q = 0; q < nj; ++q) {
      const PairJobSpec &s = specs[grp.idx[q]];
      const hd_alignment *a = s.aln;
      make_tmap(ctx, &tms[2 * q], a->planes_ptr(0), a->words, a->n_rows, v.tile);
      if (a->groups == 2) make_tmap(ctx, &tms[2 * q + 1], a->planes_ptr(1), a->words, a->n_rows, v.tile);
      else tms[2 * q + 1] = tms[2 * q];
      PairJob &j = pj[q];
      j.tmap0 = d_tms + 2 * q;
      j.tmap1 = d_tms + 2 * q + 1;
      j.out = s.d_out;
      j.out_base = s.out_base;
      j.tile_begin = tiles;
      j.n = (uint32_t)a->n_rows;
      j.nk = (uint32_t)(a->words / kKW);
      j.max_dist = s.max_dist;
      j.row_lo = s.tile_lo;
      j.row_hi = s.tile_hi;
      j.dtype = (uint32_t)s.dtype;
      tiles += (unsigned long long)s.tile_hi * (s.tile_hi + 1) / 2 -
               (unsigned long long)s.tile_lo * (s.tile_lo + 1) / 2;
    }
    // staged in pinned memory (pageable for a large table): `host` may go when this returns
    upload_table(ctx, dev.p, host.data(), host.size(), stream);
    PairLaunchPlan::Launch L;
    L.fn = reinterpret_cast<const void *>(v.fn);
    L.smem = v.smem;
    L.tile = v.tile;
    L.stages = v.stages;
    L.jobs = nj;
    L.tiles = tiles;
    L.d_jobs = dev.as<uint8_t>() + tm_bytes;
    L.d_counter = reinterpret_cast<unsigned long long *>(dev.as<uint8_t>() + tm_bytes + job_bytes);
    const int per_sm = resident_ctas(v);
    // sm_limit > 0 leaves the other SMs to kernels of other streams
    const int sms = sm_limit > 0 && sm_limit < ctx->sm_count ? sm_limit : ctx->sm_count;
    L.grid = std::min<uint64_t>(tiles, (uint64_t)per_sm * sms);
    plan->launches.push_back(L);
    plan->blocks.push_back(std::move(dev));
  }
}

void launch_pairwise_plan(hd_ctx *ctx, PairLaunchPlan &plan, cudaStream_t stream) {
  for (auto &L : plan.launches) {
    if (L.mma) {
      launch_mma(ctx, L, stream);
      continue;
    }
    HD_CUDA(cudaMemsetAsync(L.d_counter, 0, sizeof(unsigned long long), stream));
    const void *jobs = L.d_jobs;
    uint32_t nj = (uint32_t)L.jobs;
    unsigned long long tiles = L.tiles;
    unsigned long long *counter = L.d_counter;
    uint32_t one = 1;
    int *status = ctx->d_status;
    void *args[] = {&jobs, &nj, &tiles, &counter, &one, &status};
    HD_CUDA(cudaLaunchKernel(L.fn, dim3((unsigned)L.grid), dim3(kThreads), args, (size_t)L.smem,
                             stream));
    ctx->launches++;
    ctx->last_pair_tiles += L.tiles;
  }
}

void run_pairwise_jobs(hd_ctx *ctx, std::vector<PairJobSpec> &specs, cudaStream_t stream,
                       PairLaunchPlan *keep) {
  PairLaunchPlan plan;
  prepare_pairwise_jobs(ctx, specs, stream, &plan);
  launch_pairwise_plan(ctx, plan, stream);
  // without `keep` the job tables are released in stream order, after the kernels
  if (keep) *keep = std::move(plan);
}

void plan_pairwise_tiles(hd_ctx *ctx, const hd_alignment *aln, int dtype_bytes, uint32_t max_dist,
                         void *d_out, uint64_t out_base, uint32_t tile_lo, uint32_t tile_hi,
                         PairLaunchPlan *plan) {
  if (aln->n_rows < 2 || tile_hi <= tile_lo) return;
  std::vector<PairJobSpec> specs(1);
  PairJobSpec &s = specs[0];
  s.aln = aln;
  s.dtype = dtype_bytes;
  s.max_dist = max_dist;
  s.d_out = d_out;
  s.out_base = out_base;
  s.cfg = tile_config_for(ctx, aln->n_rows, aln->length, dtype_bytes);
  // callers give tile rows in units of kTile (128) rows
  const uint32_t scale = kTile / (uint32_t)s.cfg.tile;
  const uint32_t nb = (uint32_t)ceil_div(aln->n_rows, s.cfg.tile);
  s.tile_lo = tile_lo * scale;
  s.tile_hi = std::min(tile_hi * scale, nb);
  // the dense AND rule and the sparse rules go to the tensor cores
  // (hd_mma.cu) when the launch has enough items for them
  prepare_pairwise_jobs(ctx, specs, ctx->stream, plan);
}

void pairwise_tiles(hd_ctx *ctx, const hd_alignment *aln, int dtype_bytes, uint32_t max_dist,
                    void *d_out, uint64_t out_base, uint32_t tile_lo, uint32_t tile_hi) {
  PairLaunchPlan plan;
  plan_pairwise_tiles(ctx, aln, dtype_bytes, max_dist, d_out, out_base, tile_lo, tile_hi, &plan);
  // the plan's job tables are released in stream order, after the kernels
  launch_pairwise_plan(ctx, plan, ctx->stream);
}

}  // namespace hd
