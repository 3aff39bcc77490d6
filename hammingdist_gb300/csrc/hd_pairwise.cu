// The pairwise lower-triangle distance kernel.
//
// Replaces the reference's Dist<T> kernel and its chunked driver
// (src/distance_cuda.cu:9-202), which computes one lower-triangle entry per
// CTA from the nibble-packed rows with a shared-memory reduction and re-reads
// both rows from memory for every pair.
//
// Here a CTA computes a 128 x 128 tile (I, J), J <= I, of the lower triangle:
//  * rows are stored as bit planes: per 32-site word, one uint32 per plane,
//    4 planes per 16-byte group (uint4); sites match when their codes share a
//    plane bit (the reference's "(a & b) nibble != 0", src/distance_cuda.cu:
//    57-65, with the codes of src/hamming_impl.cc:23-44);
//  * TMA (cp.async.bulk.tensor, 128-byte swizzle) stages 8 words (256 sites)
//    of the 128 A-rows and the 128 B-rows per stage into shared memory, three
//    stages deep, completion tracked by mbarriers (bounded waits);
//  * each of the 256 threads owns an 8 x 8 block of pairs and, per word,
//    counts matching sites as popc((a0&b0)|(a1&b1)|(a2&b2)|(a3&b3)): four
//    LOP3 and one POPC per 32 pair-sites (mismatches = sites - matches, as
//    every padded site matches);
//  * the epilogue saturates with min(count, max_dist) (safe_int_cast,
//    include/hamming/hamming_impl.hh:37-45), stages the tile in shared memory
//    and writes each row's contiguous lower-triangle span.
#include "hd_internal.cuh"

namespace hd {

constexpr int kThreads = 256;
constexpr int kKW = 8;                              // words per stage
constexpr int kBoxBytes = kTile * kKW * 16;         // 128 rows x 128 B = 16 KB
constexpr uint64_t kWaitNs = 2000000000ull;         // TMA wait limit: 2 s

template <int G>
struct PairCfg {
  static constexpr int stages = 3;
  static constexpr int stage_bytes = G * 2 * kBoxBytes;
  static constexpr int smem_bytes = stages * stage_bytes + 1024;  // + 1024-B alignment slack
  static constexpr int min_blocks = G == 1 ? 2 : 1;
};

// acc + p * one, issued as IMAD on the FMA pipe: `one` is a kernel argument
// (always 1) that the compiler cannot fold, which keeps the accumulation off
// the ALU pipe that the LOP3s saturate.
__device__ __forceinline__ uint32_t mad_acc(uint32_t acc, uint32_t p, uint32_t one) {
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

constexpr uint32_t kBand = 16;  // tile rows per L2 band

// Tile of this CTA. Tiles are numbered row-major over the launch's tile rows
// [row_lo, row_hi); inside each band of kBand tile rows the order is
// column-major over the band's rectangle (J < I_lo) and row-major over its
// triangle, so the CTAs resident at one time share the band's A tiles and
// each B tile in L2.
__device__ inline void tile_of(uint64_t t, uint32_t row_lo, uint32_t row_hi, uint32_t &I,
                               uint32_t &J) {
  uint32_t Ir = (uint32_t)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
  while ((uint64_t)(Ir + 1) * (Ir + 2) / 2 <= t) ++Ir;
  while ((uint64_t)Ir * (Ir + 1) / 2 > t) --Ir;
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
    uint32_t i = (uint32_t)((sqrt(8.0 * (double)v + 1.0) - 1.0) * 0.5);
    while ((uint64_t)(i + 1) * (i + 2) / 2 <= v) ++i;
    while ((uint64_t)i * (i + 1) / 2 > v) --i;
    I = I_lo + i;
    J = I_lo + (uint32_t)(v - (uint64_t)i * (i + 1) / 2);
  }
}

template <int G, int P, typename OutT>
__global__ void __launch_bounds__(kThreads, PairCfg<G>::min_blocks)
    k_pairwise(const __grid_constant__ CUtensorMap tm0, const __grid_constant__ CUtensorMap tm1,
               uint32_t n, uint32_t nk, uint32_t max_dist, OutT *__restrict__ out,
               uint64_t out_base, uint64_t tile0, uint32_t row_lo, uint32_t row_hi, uint32_t one,
               int *status) {
  constexpr int S = PairCfg<G>::stages;
  constexpr uint32_t SB = PairCfg<G>::stage_bytes;
  extern __shared__ uint8_t smem_raw[];
  __shared__ __align__(8) uint64_t full[S];
  uint8_t *smem =
      reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));

  const uint32_t tid = threadIdx.x;
  uint32_t I, J;
  tile_of(tile0 + blockIdx.x, row_lo, row_hi, I, J);

  if (tid == 0) {
    prefetch_tmap(&tm0);
    if (G == 2) prefetch_tmap(&tm1);
#pragma unroll
    for (int s = 0; s < S; ++s) mbar_init(&full[s], 1);
    fence_mbar_init();
  }
  __syncthreads();

  auto issue = [&](uint32_t kc) {
    const int s = kc % S;
    uint8_t *st = smem + s * SB;
    mbar_expect_tx(&full[s], SB);
    const int32_t x = (int32_t)(kc * 32);  // uint32 elements: 128 B per chunk
    tma_load_2d(st, &tm0, x, (int32_t)(I * kTile), &full[s]);
    tma_load_2d(st + kBoxBytes, &tm0, x, (int32_t)(J * kTile), &full[s]);
    if constexpr (G == 2) {
      tma_load_2d(st + 2 * kBoxBytes, &tm1, x, (int32_t)(I * kTile), &full[s]);
      tma_load_2d(st + 3 * kBoxBytes, &tm1, x, (int32_t)(J * kTile), &full[s]);
    }
  };
  if (tid == 0)
    for (uint32_t kc = 0; kc < (uint32_t)(S - 1) && kc < nk; ++kc) issue(kc);

  // thread (ty, tx) owns rows ty + 16 r and columns tx + 16 c of the tile;
  // with the 128-byte swizzle, 16-byte chunk w of smem row q sits at chunk
  // w ^ (q & 7), and q & 7 is ty & 7 (tx & 7) for all of a thread's rows.
  const uint32_t ty = tid >> 4, tx = tid & 15;
  const uint32_t a_off = ty * 128, b_off = tx * 128, a_sw = ty & 7, b_sw = tx & 7;
  uint32_t acc[8][8];
#pragma unroll
  for (int r = 0; r < 8; ++r)
#pragma unroll
    for (int c = 0; c < 8; ++c) acc[r][c] = 0;

  bool timed_out = false;
  for (uint32_t kc = 0; kc < nk; ++kc) {
    const int s = kc % S;
    if (tid == 0 && kc + S - 1 < nk) issue(kc + S - 1);
    if (!mbar_wait_bounded(&full[s], (kc / S) & 1u, kWaitNs)) timed_out = true;
    const uint8_t *A = smem + s * SB;
    const uint8_t *B = A + kBoxBytes;
#pragma unroll 1
    for (uint32_t w = 0; w < (uint32_t)kKW; ++w) {
      const uint32_t ca = (w ^ a_sw) << 4, cb = (w ^ b_sw) << 4;
      uint4 a[8];
#pragma unroll
      for (int r = 0; r < 8; ++r)
        a[r] = *reinterpret_cast<const uint4 *>(A + a_off + r * (16 * 128) + ca);
      uint32_t a4[8], a5[8];
      if constexpr (G == 2) {
#pragma unroll
        for (int r = 0; r < 8; ++r) {
          const uint8_t *p1 = A + 2 * kBoxBytes + a_off + r * (16 * 128) + ca;
          a4[r] = *reinterpret_cast<const uint32_t *>(p1);
          a5[r] = P == 6 ? *reinterpret_cast<const uint32_t *>(p1 + 4) : 0u;
        }
      }
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        const uint4 b = *reinterpret_cast<const uint4 *>(B + b_off + c * (16 * 128) + cb);
        uint32_t b4 = 0, b5 = 0;
        if constexpr (G == 2) {
          const uint8_t *q1 = B + 2 * kBoxBytes + b_off + c * (16 * 128) + cb;
          b4 = *reinterpret_cast<const uint32_t *>(q1);
          if (P == 6) b5 = *reinterpret_cast<const uint32_t *>(q1 + 4);
        }
#pragma unroll
        for (int r = 0; r < 8; ++r) {
          // match bits: four LOP3 per word (one more per extra plane)
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
        for (uint32_t k2 = kc + 1; k2 < nk && k2 < kc + S; ++k2)
          mbar_wait_bounded(&full[k2 % S], (k2 / S) & 1u, kWaitNs);
      }
      return;
    }
  }

  // epilogue: mismatches = sites - matches; saturate, stage the tile, store
  // each row's contiguous span
  const uint32_t sites = nk * kKW * 32;
  OutT *tile = reinterpret_cast<OutT *>(smem);
#pragma unroll
  for (int r = 0; r < 8; ++r)
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      const uint32_t mism = sites - acc[r][c];  // every padded site matches
      const uint32_t v = mism < max_dist ? mism : max_dist;
      tile[(ty + 16 * r) * kTile + tx + 16 * c] = (OutT)v;
    }
  __syncthreads();
  const uint32_t warp = tid >> 5, lane = tid & 31;
  for (uint32_t rl = warp; rl < kTile; rl += kThreads / 32) {
    const uint32_t i = I * kTile + rl;
    if (i >= n) break;
    const uint32_t ncols = (I == J) ? rl : kTile;
    if (!ncols) continue;
    OutT *dst = out + ((uint64_t)i * (i - 1) / 2 + (uint64_t)J * kTile - out_base);
    for (uint32_t c = lane; c < ncols; c += 32) dst[c] = tile[rl * kTile + c];
  }
}

static void make_tmap(hd_ctx *ctx, CUtensorMap *tm, const void *base, uint64_t words,
                      uint64_t rows) {
  cuuint64_t dims[2] = {words * 4, rows};
  cuuint64_t strides[1] = {words * 16};
  cuuint32_t box[2] = {32, kTile};
  cuuint32_t es[2] = {1, 1};
  CUresult r = ctx->encode_tiled(tm, CU_TENSOR_MAP_DATA_TYPE_UINT32, 2, const_cast<void *>(base),
                                 dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                 CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                 CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) fail(HD_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
}

template <int G, int P, typename OutT>
static void launch(hd_ctx *ctx, const CUtensorMap &tm0, const CUtensorMap &tm1, uint32_t n,
                   uint32_t nk, uint32_t max_dist, void *d_out, uint64_t out_base,
                   uint32_t row_lo, uint32_t row_hi) {
  const uint64_t t0 = (uint64_t)row_lo * (row_lo + 1) / 2;
  const uint64_t t1 = (uint64_t)row_hi * (row_hi + 1) / 2;
  auto kern = k_pairwise<G, P, OutT>;
  static bool configured = false;  // per instantiation
  if (!configured) {
    HD_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 PairCfg<G>::smem_bytes));
    configured = true;
  }
  for (uint64_t t = t0; t < t1;) {
    uint64_t cnt = t1 - t < 0x7fffffffull ? t1 - t : 0x7fffffffull;
    kern<<<(unsigned)cnt, kThreads, PairCfg<G>::smem_bytes, ctx->stream>>>(
        tm0, tm1, n, nk, max_dist, static_cast<OutT *>(d_out), out_base, t, row_lo, row_hi, 1u,
        ctx->d_status);
    HD_LAUNCHED(ctx);
    t += cnt;
  }
}

template <int G, int P>
static void launch_dtype(hd_ctx *ctx, int dtype_bytes, const CUtensorMap &tm0,
                         const CUtensorMap &tm1, uint32_t n, uint32_t nk, uint32_t max_dist,
                         void *d_out, uint64_t out_base, uint32_t lo, uint32_t hi) {
  if (dtype_bytes == 1)
    launch<G, P, uint8_t>(ctx, tm0, tm1, n, nk, max_dist, d_out, out_base, lo, hi);
  else if (dtype_bytes == 2)
    launch<G, P, uint16_t>(ctx, tm0, tm1, n, nk, max_dist, d_out, out_base, lo, hi);
  else
    launch<G, P, uint32_t>(ctx, tm0, tm1, n, nk, max_dist, d_out, out_base, lo, hi);
}

void pairwise_tiles(hd_ctx *ctx, const hd_alignment *aln, int dtype_bytes, uint32_t max_dist,
                    void *d_out, uint64_t out_base, uint32_t tile_lo, uint32_t tile_hi) {
  if (aln->n_rows < 2 || tile_hi <= tile_lo) return;
  if (aln->n_rows > 0xffffffffull) fail(HD_ERR_ARG, "too many rows");
  const uint32_t n = (uint32_t)aln->n_rows;
  const uint32_t nk = (uint32_t)(aln->words / kKW);
  const uint64_t t0 = (uint64_t)tile_lo * (tile_lo + 1) / 2;
  const uint64_t t1 = (uint64_t)tile_hi * (tile_hi + 1) / 2;
  CUtensorMap tm0, tm1;
  make_tmap(ctx, &tm0, aln->plane_buf[0].p, aln->words, aln->n_rows);
  if (aln->groups == 2) make_tmap(ctx, &tm1, aln->plane_buf[1].p, aln->words, aln->n_rows);
  else tm1 = tm0;
  if (aln->planes == 4)
    launch_dtype<1, 4>(ctx, dtype_bytes, tm0, tm1, n, nk, max_dist, d_out, out_base, tile_lo, tile_hi);
  else if (aln->planes == 5)
    launch_dtype<2, 5>(ctx, dtype_bytes, tm0, tm1, n, nk, max_dist, d_out, out_base, tile_lo, tile_hi);
  else
    launch_dtype<2, 6>(ctx, dtype_bytes, tm0, tm1, n, nk, max_dist, d_out, out_base, tile_lo, tile_hi);
  ctx->last_pair_tiles += t1 - t0;
}

}  // namespace hd
