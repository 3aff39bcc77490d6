// Tensor-core lower-triangle distances (tcgen05, block-scaled FP4) for the
// dense AND rule and the sparse rules.
//
// Replaces the reference's Dist<T> kernel (src/distance_cuda.cu:9-202) and,
// for use_gpu=False, its CPU loops (include/hamming/hamming_impl.hh:120-175).
// A site pair matches when the two codes share a bit: the dense rule's
// 4-bit codes (src/distance_cuda.cu:57-65; src/hamming_impl.cc:23-44: A, C,
// G, T one-hot, '-' all four bits, every other byte 0) or the sparse rules'
// one-hot classes over P = 5 or 6 planes with '-' as all P bits
// (src/hamming_impl.cc:93-129).
//
// For those codes the match indicator is a bilinear form. With e(x) the P
// plane bits of x and d(x) = [x = '-'],
//   match(a, b) = <e(a), e(b)> - (P - 1) d(a) d(b):
// the plane dot product is 1 for equal symbols and for a symbol against '-',
// P for '-' against '-' (hence the -(P - 1)), and 0 otherwise. Summed over
// the sites of two rows this is one dot product of P + 1 values per site, the
// dash value being 1 on the row side and -(P - 1) on the column side. All
// values are 0, 1, -3 or -4, exact in E2M1 (FP4: 0, 0.5, 1, 1.5, 2, 3, 4, 6
// and their negatives); -5 (P = 6) is not, so there the column side's dash
// is -4 and -1 in two blocks, each paired with the row side's +1. The MMAs
// are kind::mxf4 with every UE8M0 scale factor 1.0 and FP32 accumulation,
// exact while P L < 2^24. mismatches = L - matches.
//
// K order: first the P plane blocks of every 256-site chunk (partial sums up
// to P L), then the dash products, only for the chunks where some row of the
// operand has a '-' (the expansion marks them): elsewhere every dash product
// is 0. On aligned genomes the '-' sit mostly in leading and trailing runs, so
// a row's P + 1 blocks per chunk shrink to about P.
//
// Operand (one buffer serves rows and columns): each row's bit planes are
// expanded to packed E2M1, two sites per byte, K-major: for every 256 sites,
// the P planes (1.0), the dash as 1.0 (read for rows) and the dash as -(P - 1)
// (read for columns; -4 and -1 for P = 6), 128 bytes each; sites past L are
// 0. An alignment caches its operand; a view of a resident alignment (a
// serving window) gets one of its own rows.
//
// One launch serves a job table of matrices. Persistent CTAs (320 threads,
// one per SM) walk a list of items: 240 columns J x one or two 128-row tiles
// I of one job, in bands of 16 tile rows, column-major within a band, so
// resident CTAs share operands in L2; the list ends with single-row-tile items
// so that every CTA gets the same work to within a row tile.
//  * warp 0 (one thread) issues TMA loads (128-byte swizzle) per stage of
//    one 128-byte K block (256 sites) of the item's 128 or 256 rows and 240
//    columns, 3 stages of 62 KB with full/empty mbarriers; warp 0 also
//    allocates and frees the TMEM;
//  * warp 1 (one thread) issues tcgen05.mma.cta_group::1.kind::mxf4
//    .block_scale (M=128, N=240, K=64), four per row tile per stage, into
//    TMEM (row tile h of the item at columns 256 h); the unit scale factors
//    sit in the columns the accumulators leave, 240-255 (rows) and 496-511
//    (columns), written once per CTA. Each stage's MMAs are
//    committed to its empty barrier, an item's last ones to `done`;
//  * warps 2-9, two per TMEM lane quarter, each read 32 rows x 128 or 112
//    columns of each accumulator (tcgen05.ld, 64, 32 or 16 columns at a time),
//    form min(L - matches, max_dist) (safe_int_cast,
//    include/hamming/hamming_impl.hh:37-45), turn each 32 x 32 chunk around
//    in a padded shared buffer and store it row by row, 32 consecutive
//    entries of the job's dtype per store; they then release the
//    accumulators (`tmem_free`) for the MMAs of the next item, whose first
//    stages the producer has already loaded. The MMAs wait for this, so the
//    epilogue's length is paid once per item.
// Every wait is bounded; on a timeout the CTA records it in the status word,
// waits (bounded) for its own copies and MMAs, frees its TMEM and returns.
#include <algorithm>
#include <cstdlib>
#include <mutex>
#include <string>
#include <vector>

#include "hd_internal.cuh"

namespace hd {
namespace {

constexpr int kEpiWarps = 8;      // two per TMEM lane quarter
constexpr int kMmaThreads = 64 + 32 * kEpiWarps;  // warp 0: TMA, warp 1: MMA, warps 2-9: epilogue
constexpr int kEpiThreads = 32 * kEpiWarps;
constexpr int kMmaStages = 3;
constexpr int kTM = 128, kTN = (int)kMmaCols;          // MMA tile: rows x columns (240)
constexpr uint32_t kEpiSplit = 128;                   // epilogue halves: [0, 128), [128, kTN)
// unit scale factors in the TMEM columns the two accumulators (columns
// [0, kTN) and [256, 256 + kTN)) leave: the rows' at kTN, the columns' at
// 256 + kTN, 16 columns each
constexpr uint32_t kSfColA = kTN, kSfColB = 256 + kTN;
constexpr uint32_t kSfWord = 0x7F7F7F7Fu;             // four UE8M0 scale factors of 2^0
constexpr uint32_t kHalfBytes = kTM * 128;            // one 128-byte K block of 128 rows
constexpr uint32_t kABytes = 2 * kHalfBytes;          // up to two row tiles
constexpr uint32_t kBBytes = kTN * 128;
constexpr uint32_t kStageBytes = kABytes + kBBytes;   // 62 KB, a multiple of 1 KB
constexpr uint32_t kEpiPitch = 33;                    // words per row of an epilogue chunk
constexpr uint32_t kEpiBytes = kEpiWarps * 32 * kEpiPitch * 4;  // 32 x 32 words per epilogue warp
constexpr int kMmaSmem = kMmaStages * kStageBytes + kEpiBytes + 1024;
static_assert(kStageBytes % 1024 == 0, "stages must stay 1 KB aligned for the 128-byte swizzle");
static_assert(kMmaSmem <= 232448, "dynamic shared memory above the per-block limit");
static_assert(kTN % 16 == 0 && kTN <= 240, "N of an M=128 MMA; 16 TMEM columns left for scales");
constexpr uint32_t kTmemCols = 512;                   // row tile h at columns 256 h
constexpr uint64_t kMmaWaitNs = 1000000000ull;        // 1 s
constexpr uint32_t kMmaBand = 16;  // tile rows per L2 band (HAMMINGDIST_MMA_BAND overrides)
constexpr int kItemRing = 4;                          // item indices handed to the consumers
constexpr uint32_t kNoItem = 0xFFFFFFFFu;             // end of this CTA's items
// 128-byte blocks per 256 sites of the operand: the P planes, the row side's
// dash and the column side's dash (two blocks for P = 6: -4 and -1)
__host__ __device__ constexpr uint32_t op_blocks(uint32_t planes) {
  return planes + (planes == 6 ? 3u : 2u);
}
// operand bytes per 32-site word: 16 bytes (32 sites of E2M1) per block
__host__ __device__ constexpr uint64_t row_bytes_per_word(uint32_t planes) {
  return (uint64_t)op_blocks(planes) * 16;
}
static_assert(row_bytes_per_word(4) == kMmaOperandBytesPerWord, "operand size of the AND rule");
// E2M1 codes: 1.0, and the column side's -(P - 1): -3 for P = 4, -4 else
// (then -1 for P = 6)
constexpr uint32_t kE2M1One = 0x2u, kE2M1Neg1 = 0xAu;
__device__ __forceinline__ uint32_t dash_neg(uint32_t planes) { return planes == 4 ? 0xDu : 0xEu; }
// instruction descriptor (block-scaled kinds): A and B E2M1 (1 at bits 7-9
// and 10-12), both K-major, N >> 3 at bits 17-22, scale factors UE8M0 (bit
// 23), M >> 4 at bits 24-28, scale factor ids 0, K = 64; D is FP32
__host__ __device__ constexpr uint32_t idesc_mxf4(uint32_t n) {
  return (1u << 7) | (1u << 10) | ((n >> 3) << 17) | (1u << 23) | ((uint32_t)(kTM >> 4) << 24);
}
constexpr uint32_t kIdesc = idesc_mxf4(kTN);

}  // namespace

// One matrix of a launch (device copy): its operand's tensor maps (boxes of
// 256 and 128 rows for the row side, kTN rows for the column side) and its
// output.
struct MmaJob {
  const CUtensorMap *tm256;
  const CUtensorMap *tm128;
  const CUtensorMap *tmb;
  void *out;                     // lt index out_base at out[0]
  unsigned long long out_base;
  uint32_t n, nkb, sites, max_dist, dtype;  // rows, K blocks per side, L, cap, 1/2/4 bytes
  uint32_t planes;                          // P
  uint32_t chunks;                          // 256-site chunks per row
  const uint32_t *dash_list;                // the chunks whose dash products count
  const uint32_t *dash_marks;               // per chunk: some row has a '-' in it
  unsigned long long pairs;                 // lower-triangle pairs of this launch
};

// One work item: kTN columns J x row tiles [I, I + halves) of job `job`.
struct MmaItem {
  uint32_t job;
  uint32_t I;       // first 128-row tile
  uint32_t J;       // kTN-column tile
  uint32_t halves;  // row tiles in the item: 1 or 2
};

namespace {

// 8 bits -> 8 nibbles (bit i -> the low bit of nibble i), times the E2M1
// code `v` (no carries: each nibble is 0 or 1 before the multiply)
__device__ __forceinline__ uint32_t nib8(uint32_t b, uint32_t v) {
  b = (b | (b << 12)) & 0x000F000Fu;
  b = (b | (b << 6)) & 0x03030303u;
  b = (b | (b << 3)) & 0x11111111u;
  return b * v;
}
// 32 sites (one plane word) -> 16 bytes of E2M1: site s in nibble s (byte
// s / 2, low nibble for even s), `v` where the bit is set, else 0
__device__ __forceinline__ void put16(uint8_t *dst, uint32_t w, uint32_t v) {
  *reinterpret_cast<uint4 *>(dst) =
      make_uint4(nib8(w & 0xFFu, v), nib8((w >> 8) & 0xFFu, v), nib8((w >> 16) & 0xFFu, v),
                 nib8(w >> 24, v));
}

// Rows [row_lo, row_hi) of a P-plane alignment (P = 4: the AND rule; 5, 6:
// the sparse rules, planes 4-5 in the second group) -> E2M1 operand rows.
// One thread per (row, 32-site word): 16 or 32 bytes read, 16 bytes written
// per block; eight consecutive words fill each 128-byte block of their 256
// sites. The dash is the AND of the P planes ('-' has every plane); a chunk
// of 256 sites where some row has a '-' is marked in dash_chunk.
__global__ void k_expand_op(const uint4 *__restrict__ g0, const uint4 *__restrict__ g1,
                            uint32_t planes, uint64_t words, uint64_t row_lo, uint64_t row_hi,
                            uint64_t L, uint8_t *__restrict__ x, uint32_t *dash_chunk) {
  const uint32_t nb = op_blocks(planes);  // 128-byte blocks per 256 sites
  // thread (x, y): word x of rows row_lo + y, row_lo + y + gridDim.y, ...
  const uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (w >= words) return;
  for (uint64_t r = row_lo + blockIdx.y; r < row_hi; r += gridDim.y) {
    const uint4 p = g0[r * words + w];
    const uint4 p1 = planes > 4 ? g1[r * words + w] : make_uint4(0u, 0u, 0u, 0u);
    const uint64_t s0 = w * 32;
    const uint32_t valid = s0 >= L ? 0u : (L - s0 >= 32 ? 0xffffffffu : ((1u << (L - s0)) - 1u));
    uint32_t dash = p.x & p.y & p.z & p.w & valid;
    if (planes > 4) dash &= p1.x;
    if (planes > 5) dash &= p1.y;
    uint8_t *blk = x + r * (words * row_bytes_per_word(planes)) + (w / 8) * (nb * 128) + (w % 8) * 16;
    put16(blk, p.x & valid, kE2M1One);
    put16(blk + 128, p.y & valid, kE2M1One);
    put16(blk + 256, p.z & valid, kE2M1One);
    put16(blk + 384, p.w & valid, kE2M1One);
    if (planes > 4) put16(blk + 512, p1.x & valid, kE2M1One);
    if (planes > 5) put16(blk + 640, p1.y & valid, kE2M1One);
    put16(blk + planes * 128, dash, kE2M1One);                // 1.0: the row side
    put16(blk + (planes + 1) * 128, dash, dash_neg(planes));  // the column side
    if (planes == 6) put16(blk + (planes + 2) * 128, dash, kE2M1Neg1);
    // the chunk holds a '-': its dash products count (every writer stores 1)
    if (dash && !dash_chunk[w / 8]) dash_chunk[w / 8] = 1u;
  }
}

// ------------------------------------------------------- tcgen05 helpers
// Shared-memory matrix descriptor, K-major, 128-byte swizzle: start address
// >> 4 (bits 0-13), leading byte offset 16 B (unused for this layout, bits
// 16-29), stride byte offset 1024 B between 8-row groups (bits 32-45),
// descriptor version 1 (bits 46-47), layout SWIZZLE_128B = 2 (bits 61-63).
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}
__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   smem_u32(dst)),
               "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tc_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// D (+)= A B^T over K = 64 E2M1 values, every block of 32 scaled by the UE8M0
// factors at TMEM addresses sfa and sfb
__device__ __forceinline__ void mma_f4(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc,
                                       uint32_t idesc, uint32_t accumulate, uint32_t sfa,
                                       uint32_t sfb) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::mxf4.block_scale.scale_vec::2X [%0], %1, %2, %3, [%5], "
      "[%6], p;\n\t}" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate), "r"(sfa), "r"(sfb)
      : "memory");
}
// The unit scale factors: this warp writes kSfWord to the NC TMEM columns
// from col0 in its lane quarter (lane base `t_lane`) and waits for the
// stores; the caller fences before the MMAs read them.
template <uint32_t NC>
__device__ __forceinline__ void write_unit_scales(uint32_t t_lane, uint32_t col0) {
#pragma unroll
  for (uint32_t c = col0; c < col0 + NC; c += 4)
    asm volatile("tcgen05.st.sync.aligned.32x32b.x4.b32 [%0], {%1, %2, %3, %4};" ::"r"(t_lane + c),
                 "r"(kSfWord), "r"(kSfWord), "r"(kSfWord), "r"(kSfWord)
                 : "memory");
  asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}
// arrives on `bar` once every earlier tcgen05.mma of this thread has completed
__device__ __forceinline__ void mma_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
// 32 lanes x 64 consecutive 32-bit columns: thread t gets row (lane base + t)
__device__ __forceinline__ void tmem_ld64(uint32_t taddr, uint32_t (&v)[64]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x64.b32 {"
      "%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16, %17, %18, "
      "%19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31, %32, %33, %34, %35, "
      "%36, %37, %38, %39, %40, %41, %42, %43, %44, %45, %46, %47, %48, %49, %50, %51, %52, "
      "%53, %54, %55, %56, %57, %58, %59, %60, %61, %62, %63 "
      "}, [%64];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
        "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
        "=r"(v[14]), "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]),
        "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]),
        "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31]),
        "=r"(v[32]), "=r"(v[33]), "=r"(v[34]), "=r"(v[35]), "=r"(v[36]), "=r"(v[37]),
        "=r"(v[38]), "=r"(v[39]), "=r"(v[40]), "=r"(v[41]), "=r"(v[42]), "=r"(v[43]),
        "=r"(v[44]), "=r"(v[45]), "=r"(v[46]), "=r"(v[47]), "=r"(v[48]), "=r"(v[49]),
        "=r"(v[50]), "=r"(v[51]), "=r"(v[52]), "=r"(v[53]), "=r"(v[54]), "=r"(v[55]),
        "=r"(v[56]), "=r"(v[57]), "=r"(v[58]), "=r"(v[59]), "=r"(v[60]), "=r"(v[61]),
        "=r"(v[62]), "=r"(v[63])
      : "r"(taddr)
      : "memory");
}
// 32 lanes x 32 consecutive 32-bit columns
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&v)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {"
      "%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16, %17, %18, "
      "%19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31 "
      "}, [%32];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
        "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
        "=r"(v[14]), "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]),
        "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]),
        "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
      : "r"(taddr)
      : "memory");
}
// 32 lanes x 16 consecutive 32-bit columns
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&v)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {"
      "%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15 "
      "}, [%16];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
        "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
        "=r"(v[14]), "=r"(v[15])
      : "r"(taddr)
      : "memory");
}
__device__ __forceinline__ void tmem_ld_wait() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// min(sites - matches, max_dist) of accumulator columns OFF .. OFF + W - 1
// (FP32 integers) into the warp's buffer, row `lane` at words 33 lane
template <int OFF, int N, int W = 32>
__device__ __forceinline__ void turn_chunk(uint32_t *buf, const uint32_t (&d)[N], uint32_t sites,
                                           uint32_t max_dist, uint32_t lane) {
  static_assert(OFF + W <= N, "columns outside the loaded registers");
#pragma unroll
  for (uint32_t j = 0; j < W; ++j) {
    const uint32_t mism = sites - (uint32_t)__uint_as_float(d[OFF + j]);
    buf[lane * kEpiPitch + j] = mism < max_dist ? mism : max_dist;
  }
}

// The buffered chunk of rows i0 .. i0 + rows - 1, columns j0 .. j0 + W - 1,
// row by row: lane l < W stores column j0 + l of row i0 + r, lower-triangle
// entry tri(i0 + r) + j0 + l = e0 + r i0 + r (r - 1) / 2, where it is below
// the diagonal (j0 + l < i0 + r). The row loop is unrolled so that several
// rows' loads and stores are in flight.
template <typename T, uint32_t W = 32>
__device__ __forceinline__ void store_chunk(T *out, unsigned long long e0, uint32_t i0,
                                            uint32_t rows, uint32_t j0, const uint32_t *buf,
                                            uint32_t lane) {
#pragma unroll 8
  for (uint32_t r = 0; r < 32; ++r)
    if (r < rows && lane < W && j0 + lane < i0 + r)
      out[e0 + (unsigned long long)r * i0 + r * (r - 1) / 2] = (T)buf[r * kEpiPitch + lane];
}

// One epilogue warp's share of an item: TMEM lanes of its quarter (rows
// 32 sub + lane of each row tile) x its columns [c_lo, c_hi), read 64
// columns at a time, then a last piece of 32 and one of 16 where the share
// leaves them (112 = 64 + 32 + 16).
template <typename T>
__device__ __forceinline__ void epilogue_share(const MmaItem &tl, const MmaJob &job,
                                               uint32_t t_lane, uint32_t c_lo, uint32_t c_hi,
                                               uint32_t sub, uint32_t lane, uint32_t *buf) {
  const uint32_t n = job.n, sites = job.sites, max_dist = job.max_dist;
  T *out = static_cast<T *>(job.out);
  for (uint32_t h = 0; h < tl.halves; ++h) {
    const uint32_t i0 = (tl.I + h) * kTM + sub * 32;  // output row of lane 0
    if (i0 >= n) continue;                           // warp-uniform
    const uint32_t rows = n - i0 < 32u ? n - i0 : 32u;
    const unsigned long long t0 = (unsigned long long)i0 * (i0 - 1) / 2 - job.out_base + lane;
#pragma unroll 1
    for (uint32_t c = c_lo; c < c_hi;) {
      const uint32_t j0 = tl.J * kTN + c;  // first column of this group
      if (j0 + 1 >= i0 + rows) break;      // no row reaches column j0 (warp-uniform)
      __syncwarp();
      if (c + 32 > c_hi) {  // a last piece of 16 columns
        uint32_t d[16];
        tmem_ld16(t_lane + 256u * h + c, d);
        tmem_ld_wait();
        turn_chunk<0, 16, 16>(buf, d, sites, max_dist, lane);
        __syncwarp();
        store_chunk<T, 16>(out, t0 + j0, i0, rows, j0, buf, lane);
        __syncwarp();
        break;
      }
      if (c + 64 > c_hi) {  // a piece of 32 columns
        uint32_t d[32];
        tmem_ld32(t_lane + 256u * h + c, d);
        tmem_ld_wait();
        turn_chunk<0>(buf, d, sites, max_dist, lane);
        __syncwarp();
        store_chunk<T>(out, t0 + j0, i0, rows, j0, buf, lane);
        __syncwarp();
        c += 32;
        continue;
      }
      uint32_t d[64];
      tmem_ld64(t_lane + 256u * h + c, d);
      tmem_ld_wait();
      turn_chunk<0>(buf, d, sites, max_dist, lane);
      __syncwarp();
      store_chunk<T>(out, t0 + j0, i0, rows, j0, buf, lane);
      __syncwarp();  // the buffer is rewritten next
      if (j0 + 33 >= i0 + rows) break;  // no row reaches column j0 + 32
      turn_chunk<32>(buf, d, sites, max_dist, lane);
      __syncwarp();
      store_chunk<T>(out, t0 + j0 + 32, i0, rows, j0 + 32, buf, lane);
      __syncwarp();
      c += 64;
    }
  }
}

__global__ void __launch_bounds__(kMmaThreads, 1)
    k_pairwise_mma(const MmaJob *__restrict__ jobs, const MmaItem *__restrict__ items,
                   uint32_t n_items, unsigned *__restrict__ counter, uint32_t queue,
                   int *status) {
  extern __shared__ uint8_t smem_raw[];
  __shared__ __align__(8) uint64_t full[kMmaStages], empty[kMmaStages], done, tmem_free, fin;
  __shared__ __align__(8) uint64_t item_full[kItemRing], item_empty[kItemRing];
  __shared__ uint32_t s_item[kItemRing];
  __shared__ uint32_t s_tmem;
  __shared__ int s_abort;
  uint8_t *smem =
      reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    for (int s = 0; s < kMmaStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int r = 0; r < kItemRing; ++r) {
      mbar_init(&item_full[r], 1);
      mbar_init(&item_empty[r], 1 + kEpiWarps);  // the MMA thread and each epilogue warp
    }
    mbar_init(&done, 1);
    mbar_init(&tmem_free, kEpiThreads);
    mbar_init(&fin, 1);
    fence_mbar_init();
    s_abort = 0;
  }
  if (warp == 0) {
    tmem_alloc(&s_tmem, kTmemCols);
    tmem_relinquish();
  }
  tc_before_sync();
  __syncthreads();
  tc_after_sync();
  const uint32_t tmem = s_tmem;
  // the unit scale factors, once per CTA: warps 2-5 cover the lane quarters
  if (warp >= 2 && warp < 6) {
    write_unit_scales<16>(tmem + (((warp & 3u) * 32) << 16), kSfColA);
    write_unit_scales<16>(tmem + (((warp & 3u) * 32) << 16), kSfColB);
  }
  tc_before_sync();
  __syncthreads();
  tc_after_sync();

  if (warp == 0) {
    if (lane == 0) {
      // producer: draws this CTA's items from the launch's queue (its first
      // item is blockIdx.x, later ones gridDim.x + an atomic count) or, with
      // `queue` 0, round-robin (blockIdx.x + k gridDim.x); hands each item's
      // index to the MMA and epilogue warps through the ring, then loads
      // every K block of the item
      uint32_t g = 0;  // K blocks issued (stage g % S, phase g / S)
      bool ok = true;
      for (uint32_t k = 0; ok; ++k) {
        const uint32_t r = k % kItemRing;
        if (k >= (uint32_t)kItemRing &&
            !mbar_wait_bounded(&item_empty[r], ((k / kItemRing) - 1) & 1u, kMmaWaitNs)) {
          ok = false;
          break;
        }
        uint32_t t = k == 0 ? blockIdx.x
                            : (queue ? gridDim.x + atomicAdd(counter, 1u) : blockIdx.x + k * gridDim.x);
        if (t >= n_items || *(volatile int *)&s_abort) t = kNoItem;
        *(volatile uint32_t *)&s_item[r] = t;
        mbar_arrive(&item_full[r]);  // releases the index to the waiting warps
        if (t == kNoItem) break;
        const MmaItem tl = items[t];
        const MmaJob &job = jobs[tl.job];
        const CUtensorMap *ta = tl.halves == 2 ? job.tm256 : job.tm128;
        prefetch_tmap(ta);
        prefetch_tmap(job.tmb);
        const int32_t ya = (int32_t)(tl.I * kTM), yb = (int32_t)(tl.J * kTN);
        const uint32_t bytes = kBBytes + tl.halves * kHalfBytes, nkb = job.nkb, P = job.planes;
        const uint32_t NB = op_blocks(P), plane_kb = P * job.chunks;
        for (uint32_t kb = 0; kb < nkb; ++kb) {
          const uint32_t s = g % kMmaStages;
          if ((g >= (uint32_t)kMmaStages &&
               !mbar_wait_bounded(&empty[s], ((g / kMmaStages) - 1) & 1u, kMmaWaitNs)) ||
              *(volatile int *)&s_abort) {
            ok = false;
            break;
          }
          // K block kb: first the P plane blocks of every 256-site chunk,
          // then the dash products of the chunks that hold a '-' (the rows'
          // +1 block against the columns' -(P - 1) block; for P = 6 the +1
          // block twice, against -4 and -1). Elsewhere the dash products are
          // all 0, so those blocks are left out.
          uint32_t blk_a, blk_b;
          if (kb < plane_kb) {
            blk_a = blk_b = NB * (kb / P) + kb % P;
          } else {
            const uint32_t j = kb - plane_kb, two = P == 6 ? 1u : 0u;
            const uint32_t c = job.dash_list[j >> two];
            blk_a = NB * c + P;
            blk_b = NB * c + P + 1 + (j & two);
          }
          const int32_t xa = (int32_t)(blk_a * 128), xb = (int32_t)(blk_b * 128);
          uint8_t *st = smem + s * kStageBytes;
          mbar_expect_tx(&full[s], bytes);
          tma_load_2d(st, ta, xa, ya, &full[s]);
          tma_load_2d(st + kABytes, job.tmb, xb, yb, &full[s]);
          ++g;
        }
      }
      if (!ok) {
        atomicExch(&s_abort, 1);
        atomicExch(status, kStatusTmaTimeout);
      }
      // the copies still in flight land before the CTA may leave
      for (uint32_t q = g > (uint32_t)kMmaStages ? g - kMmaStages : 0; q < g; ++q)
        mbar_wait_bounded(&full[q % kMmaStages], (q / kMmaStages) & 1u, kMmaWaitNs);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // MMA issuer
      uint32_t g = 0;
      bool ok = true;
      for (uint32_t it = 0; ok; ++it) {
        const uint32_t r = it % kItemRing;
        if (!mbar_wait_bounded(&item_full[r], (it / kItemRing) & 1u, 4 * kMmaWaitNs)) {
          ok = false;
          break;
        }
        const uint32_t t = *(volatile uint32_t *)&s_item[r];
        mbar_arrive(&item_empty[r]);
        if (t == kNoItem) break;
        const uint32_t halves = items[t].halves, nkb = jobs[items[t].job].nkb;
        // the epilogue has read the previous item's accumulators
        if (it > 0 && !mbar_wait_bounded(&tmem_free, (it - 1) & 1u, kMmaWaitNs)) {
          ok = false;
          break;
        }
        tc_after_sync();
        for (uint32_t kb = 0; kb < nkb; ++kb) {
          const uint32_t s = g % kMmaStages;
          if (!mbar_wait_bounded(&full[s], (g / kMmaStages) & 1u, kMmaWaitNs) ||
              *(volatile int *)&s_abort) {
            ok = false;
            break;
          }
          tc_after_sync();
          const uint32_t a0 = smem_u32(smem + s * kStageBytes);
          const uint64_t bd = sw128_desc(a0 + kABytes);
          for (uint32_t h = 0; h < halves; ++h) {
            const uint64_t ad = sw128_desc(a0 + h * kHalfBytes);
#pragma unroll
            for (uint32_t k = 0; k < 4; ++k)  // 32 bytes of K per MMA: +2 in 16-byte units
              mma_f4(tmem + 256u * h, ad + 2 * k, bd + 2 * k, kIdesc, (kb | k) ? 1u : 0u,
                     tmem + kSfColA, tmem + kSfColB);
          }
          mma_commit(&empty[s]);
          ++g;
        }
        if (!ok) break;
        mma_commit(&done);
      }
      if (!ok) {
        atomicExch(&s_abort, 1);
        atomicExch(status, kStatusTmaTimeout);
        mma_commit(&done);  // releases an epilogue waiting for this item
      }
      // every MMA of this thread has completed before TMEM is freed
      mma_commit(&fin);
      mbar_wait_bounded(&fin, 0, 4 * kMmaWaitNs);
    }
  } else {
    // epilogue warps 2 .. 2 + kEpiWarps - 1: warp w reads TMEM lanes
    // 32 (w % 4) .. + 31, which are rows 32 (w % 4) + lane of each row tile
    // of the item, in columns [0, 128) (w < 6) or [128, kTN) (w >= 6). Each
    // 32 x 32 chunk goes through the warp's padded shared buffer (row r at
    // words 33 r: conflict-free both ways), so that one store instruction
    // writes 32 consecutive entries of one row rather than one entry of 32
    // rows.
    const uint32_t sub = warp & 3u, c_lo = warp < 6 ? 0u : kEpiSplit, c_hi = warp < 6 ? kEpiSplit : (uint32_t)kTN;
    const uint32_t t_lane = tmem + ((sub * 32) << 16);
    uint32_t *buf = reinterpret_cast<uint32_t *>(smem + kMmaStages * kStageBytes) +
                    (warp - 2) * 32 * kEpiPitch;
    for (uint32_t it = 0;; ++it) {
      const uint32_t r = it % kItemRing;
      // lane 0 waits and reads the index; the warp takes its answer
      uint32_t t = kNoItem;
      bool got = true;
      if (lane == 0) {
        got = mbar_wait_bounded(&item_full[r], (it / kItemRing) & 1u, 4 * kMmaWaitNs);
        if (got) t = *(volatile uint32_t *)&s_item[r];
      }
      got = __shfl_sync(0xffffffffu, got ? 1u : 0u, 0) != 0;
      t = __shfl_sync(0xffffffffu, t, 0);
      if (got && lane == 0) mbar_arrive(&item_empty[r]);
      if (!got) {
        atomicExch(&s_abort, 1);
        atomicExch(status, kStatusTmaTimeout);
      }
      // one decision per warp: tcgen05.ld needs the whole warp
      if (__any_sync(0xffffffffu, t == kNoItem)) break;
      got = mbar_wait_bounded(&done, it & 1u, 4 * kMmaWaitNs);
      if (!got) {
        atomicExch(&s_abort, 1);
        atomicExch(status, kStatusTmaTimeout);
      }
      // one decision per warp: tcgen05.ld needs the whole warp
      if (__any_sync(0xffffffffu, !got || *(volatile int *)&s_abort)) break;
      tc_after_sync();
      const MmaItem tl = items[t];
      const MmaJob &job = jobs[tl.job];
      if (job.dtype == 1)
        epilogue_share<uint8_t>(tl, job, t_lane, c_lo, c_hi, sub, lane, buf);
      else if (job.dtype == 2)
        epilogue_share<uint16_t>(tl, job, t_lane, c_lo, c_hi, sub, lane, buf);
      else
        epilogue_share<uint32_t>(tl, job, t_lane, c_lo, c_hi, sub, lane, buf);
      // the accumulators may be overwritten
      tc_before_sync();
      mbar_arrive(&tmem_free);
    }
  }
  tc_before_sync();
  __syncthreads();
  tc_after_sync();
  if (warp == 0) {
    __syncwarp();
    tmem_dealloc(tmem, kTmemCols);
  }
}

// FP4 (kind::mxf4) MMA rate from shared memory alone (no loads): one CTA per
// SM (the shared-memory request keeps it alone) issues `rounds` x 4 MMAs of
// M=128, N=256, K=64 on a zeroed stage (the values do not change the rate),
// with unit scale factors in TMEM columns 256-287.
constexpr uint32_t kPeakN = 256, kPeakSf = 256;
__global__ void __launch_bounds__(128, 1) k_peak_mma(uint32_t rounds, int *status) {
  extern __shared__ uint8_t smem_raw[];
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t s_tmem;
  uint8_t *smem =
      reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  for (uint32_t k = threadIdx.x; k < (kABytes + kPeakN * 128) / 16; k += blockDim.x)
    reinterpret_cast<uint4 *>(smem)[k] = make_uint4(0, 0, 0, 0);
  // the generic-proxy writes above, before the tensor cores read them
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  if (threadIdx.x < 32) {
    tmem_alloc(&s_tmem, kTmemCols);
    tmem_relinquish();
  }
  tc_before_sync();
  __syncthreads();
  tc_after_sync();
  const uint32_t tmem = s_tmem;
  write_unit_scales<32>(tmem + (((threadIdx.x >> 5) * 32) << 16), kPeakSf);
  tc_before_sync();
  __syncthreads();
  tc_after_sync();
  if (threadIdx.x == 0) {
    const uint32_t a0 = smem_u32(smem);
    const uint64_t ad = sw128_desc(a0), bd = sw128_desc(a0 + kABytes);
    for (uint32_t r = 0; r < rounds; ++r)
#pragma unroll
      for (uint32_t k = 0; k < 4; ++k)
        mma_f4(tmem, ad + 2 * k, bd + 2 * k, idesc_mxf4(kPeakN), (r | k) ? 1u : 0u,
               tmem + kPeakSf, tmem + kPeakSf + 16);
    mma_commit(&bar);
    if (!mbar_wait_bounded(&bar, 0, 4 * kMmaWaitNs)) atomicExch(status, kStatusTmaTimeout);
  }
  tc_before_sync();
  __syncthreads();
  tc_after_sync();
  if (threadIdx.x < 32) {
    __syncwarp();
    tmem_dealloc(tmem, kTmemCols);
  }
}

// One warp per job: the ascending list of the chunks whose mark is set, and
// the job's K blocks (P per chunk, then one per listed chunk, two for P = 6);
// the job's multiply-adds (pairs x 256 values per K block) are added to
// *macs. A mark set concurrently by a later expansion (rows this launch does
// not read) only adds dash products of 0.
__global__ void k_dash_list(MmaJob *jobs, unsigned long long *macs) {
  MmaJob &job = jobs[blockIdx.x];
  const uint32_t lane = threadIdx.x;
  uint32_t *list = const_cast<uint32_t *>(job.dash_list);
  uint32_t n = 0;
  for (uint32_t c0 = 0; c0 < job.chunks; c0 += 32) {
    const uint32_t c = c0 + lane;
    const bool on = c < job.chunks && *(volatile const uint32_t *)&job.dash_marks[c] != 0u;
    const uint32_t bits = __ballot_sync(0xffffffffu, on);
    if (on) list[n + __popc(bits & ((1u << lane) - 1u))] = c;
    n += __popc(bits);
  }
  if (lane == 0) {
    job.nkb = job.planes * job.chunks + n * (job.planes == 6 ? 2u : 1u);
    atomicAdd(macs, job.pairs * 256ull * job.nkb);
  }
}

void set_smem_once() {
  static std::once_flag once;
  static cudaError_t err = cudaSuccess;
  std::call_once(once, [&] {
    err = cudaFuncSetAttribute(k_pairwise_mma, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               kMmaSmem);
  });
  HD_CUDA(err);
}

void make_tmap_u8(hd_ctx *ctx, CUtensorMap *tm, const void *base, uint64_t row_bytes,
                  uint64_t rows, uint32_t box_rows) {
  cuuint64_t dims[2] = {row_bytes, rows};
  cuuint64_t strides[1] = {row_bytes};
  cuuint32_t box[2] = {128, box_rows};
  cuuint32_t es[2] = {1, 1};
  CUresult r = ctx->encode_tiled(tm, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, const_cast<void *>(base),
                                 dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                 CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                 CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS)
    fail(HD_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
}

}  // namespace

int mma_band_of(const TileConfig &c) {
  if (const char *e = std::getenv("HAMMINGDIST_MMA_BAND")) return std::max(2, std::atoi(e)) & ~1;
  return c.mma_band > 0 ? std::max(2, c.mma_band) & ~1 : (int)kMmaBand;
}
int mma_rows_of(const TileConfig &c) {
  if (const char *e = std::getenv("HAMMINGDIST_MMA_ROWS")) return std::atoi(e) == 1 ? 1 : 2;
  return c.mma_rows == 1 ? 1 : 2;
}

bool mma_eligible(const hd_alignment *aln) {
  if (const char *e = std::getenv("HAMMINGDIST_KERNEL"))
    if (std::string(e) == "lop3") return false;
  // the AND rule (4 planes) or a sparse rule (5, 6 planes); FP32 sums of up
  // to P L are exact below 2^24
  const uint64_t P = (uint64_t)aln->planes;
  const bool shape = (P == 4 && aln->groups == 1) || ((P == 5 || P == 6) && aln->groups == 2);
  return shape && aln->length >= 1 && aln->length * P < (1ull << 24) && aln->n_rows >= 2 &&
         aln->n_rows < (1ull << 31);
}

bool ensure_operand(hd_ctx *ctx, const hd_alignment *aln, uint64_t rows, cudaStream_t stream,
                uint64_t cap_hint) {
  const hd_alignment *o = aln->base ? aln->base : aln;
  if (o->op_rows >= rows) return true;
  const uint32_t P = (uint32_t)o->planes;
  const uint64_t words = o->words, rb = words * row_bytes_per_word(P);
  if (rows > o->op_cap) {
    // room for the rows asked for, or for what the caller says will come
    const uint64_t plane_rows = o->plane_buf[0].bytes / (words * 16);
    const uint64_t cap = std::max(rows, std::min(cap_hint, plane_rows));
    DevBuf grown;
    try {
      grown = DevBuf(cap * rb, stream);
    } catch (const Error &e) {
      if (e.code != HD_ERR_OOM) throw;
      cudaGetLastError();
      return false;  // the bit-plane engine needs no extra memory
    }
    if (o->op_rows) {
      HD_CUDA(cudaMemcpyAsync(grown.p, o->op.p, o->op_rows * rb, cudaMemcpyDeviceToDevice, stream));
      // launches on the context's other streams may still read the old
      // operand: they finish before it is freed
      for (cudaStream_t st : {ctx->side, ctx->stream}) HD_CUDA(cudaStreamSynchronize(st));
    }
    o->op = std::move(grown);
    o->op_cap = cap;
  }
  if (!o->op_dash.p) {
    o->op_dash = DevBuf(words / 8 * 4, stream);
    HD_CUDA(cudaMemsetAsync(o->op_dash.p, 0, words / 8 * 4, stream));
  }
  const dim3 grid((unsigned)ceil_div(words, (uint64_t)256),
                  (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(rows - o->op_rows, 65535)));
  k_expand_op<<<grid, 256, 0, stream>>>(
      o->plane_buf[0].as<uint4>(), P > 4 ? o->plane_buf[1].as<uint4>() : nullptr, P, words,
      o->op_rows, rows, o->length, o->op.as<uint8_t>(), o->op_dash.as<uint32_t>());
  HD_LAUNCHED(ctx);
  o->op_rows = rows;
  return true;
}

double measure_mma_peak(hd_ctx *ctx) {
  static std::once_flag once;
  static cudaError_t err = cudaSuccess;
  std::call_once(once, [&] {
    err = cudaFuncSetAttribute(k_peak_mma, cudaFuncAttributeMaxDynamicSharedMemorySize, kMmaSmem);
  });
  HD_CUDA(err);
  const uint32_t rounds = 4096;
  k_peak_mma<<<ctx->sm_count, 128, kMmaSmem, ctx->stream>>>(256, ctx->d_status);  // warm-up
  HD_LAUNCHED(ctx);
  HD_CUDA(cudaEventRecord(ctx->ev_start, ctx->stream));
  k_peak_mma<<<ctx->sm_count, 128, kMmaSmem, ctx->stream>>>(rounds, ctx->d_status);
  HD_LAUNCHED(ctx);
  HD_CUDA(cudaEventRecord(ctx->ev_stop, ctx->stream));
  HD_CUDA(cudaStreamSynchronize(ctx->stream));
  float ms = 0;
  HD_CUDA(cudaEventElapsedTime(&ms, ctx->ev_start, ctx->ev_stop));
  const double flop = (double)ctx->sm_count * rounds * 4 * 2.0 * kTM * kPeakN * 64;
  return flop / (ms / 1e3);
}

// The E2M1 operand rows of a job: the alignment's own cache (an alignment, or
// a view at row 0 of a base whose cache already holds its rows: the streamed
// from_fasta), else the view's rows expanded into a buffer the plan keeps
// until the kernel has run (a serving window must not expand a large base).
// False if there is no memory for it.
bool operand_for(hd_ctx *ctx, const hd_alignment *a, cudaStream_t stream, PairLaunchPlan *plan,
                 const uint8_t *&op, const uint32_t *&dash) {
  const hd_alignment *o = a->base ? a->base : a;
  if (!a->base) {
    if (!ensure_operand(ctx, a, a->n_rows, stream)) return false;
    op = a->op.as<uint8_t>();
    dash = a->op_dash.as<uint32_t>();
    return true;
  }
  if (a->row0 == 0 && o->op.p && o->op_rows >= a->n_rows) {
    // the base's chunk marks cover its other rows too: a chunk marked for
    // them only adds dash products of 0
    op = o->op.as<uint8_t>();
    dash = o->op_dash.as<uint32_t>();
    return true;
  }
  const uint32_t P = (uint32_t)o->planes;
  const uint64_t rb = o->words * row_bytes_per_word(P), bytes = a->n_rows * rb;
  const uint64_t flag_bytes = o->words / 8 * 4;
  if (bytes > (8ull << 30)) return false;  // the bit-plane engine needs no extra memory
  DevBuf tmp;
  try {
    tmp = DevBuf(bytes + flag_bytes, stream);
  } catch (const Error &e) {
    if (e.code != HD_ERR_OOM) throw;
    cudaGetLastError();
    return false;
  }
  uint32_t *flags = reinterpret_cast<uint32_t *>(tmp.as<uint8_t>() + bytes);
  HD_CUDA(cudaMemsetAsync(flags, 0, flag_bytes, stream));
  const dim3 grid((unsigned)ceil_div(o->words, (uint64_t)256),
                  (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(a->n_rows, 65535)));
  k_expand_op<<<grid, 256, 0, stream>>>(
      static_cast<const uint4 *>(a->planes_ptr(0)),
      P > 4 ? static_cast<const uint4 *>(a->planes_ptr(1)) : nullptr, P, o->words, 0, a->n_rows,
      o->length, tmp.as<uint8_t>(), flags);
  HD_LAUNCHED(ctx);
  op = tmp.as<uint8_t>();
  dash = flags;
  plan->blocks.push_back(std::move(tmp));
  return true;
}

void prepare_mma_jobs(hd_ctx *ctx, const std::vector<PairJobSpec> &specs, cudaStream_t stream,
                      PairLaunchPlan *plan, int sm_limit, std::vector<char> &taken) {
  taken.assign(specs.size(), 0);
  std::vector<const uint8_t *> ops(specs.size(), nullptr);  // each job's operand rows
  std::vector<const uint32_t *> dash_marks(specs.size(), nullptr);  // and its chunk marks
  struct Job {
    size_t k;
    uint32_t t_lo, t_hi;
    double cost;
  };
  std::vector<Job> js;
  // A launch with few items leaves SMs idle: below a minimum of single row
  // tiles (128 x kTN) in all (mma_min_items_for, autotuned per row length),
  // the bit-plane engine's finer tiles finish first; a batch of small
  // matrices still goes here when together they are enough.
  if (ctx->engine_force == 0) return;
  uint64_t items_total = 0, max_len = 0;
  for (const PairJobSpec &sp : specs) {
    if (!mma_eligible(sp.aln) || sp.tile_hi <= sp.tile_lo) continue;
    max_len = std::max<uint64_t>(max_len, sp.aln->length);
    const uint64_t edge = sp.cfg.tile > 0 ? (uint64_t)sp.cfg.tile : kTile;
    const uint64_t lo = sp.tile_lo * edge / kTM;
    const uint64_t hi = ceil_div(std::min<uint64_t>(sp.tile_hi * edge, sp.aln->n_rows), kTM);
    for (uint64_t I = lo; I < hi; ++I) items_total += ((I + 1) * kTM - 2) / kTN + 1;
  }
  const uint64_t min_items = ctx->engine_force == 1 ? 0 : mma_min_items_for(ctx, max_len);
  if (items_total < min_items) return;
  for (size_t k = 0; k < specs.size(); ++k) {
    const PairJobSpec &sp = specs[k];
    const hd_alignment *a = sp.aln;
    if (!mma_eligible(a) || sp.tile_hi <= sp.tile_lo) continue;
    // the caller's tile rows are in units of its configuration's tile edge
    const uint64_t edge = sp.cfg.tile > 0 ? (uint64_t)sp.cfg.tile : kTile;
    const uint64_t row_lo = sp.tile_lo * edge, row_hi = std::min<uint64_t>(sp.tile_hi * edge, a->n_rows);
    if (row_lo % kTM || row_hi <= row_lo) continue;
    if (!operand_for(ctx, a, stream, plan, ops[k], dash_marks[k])) continue;
    const uint32_t lo = (uint32_t)(row_lo / kTM), hi = (uint32_t)ceil_div(row_hi, kTM);
    js.push_back({k, lo, hi, (double)a->words * ((double)hi * hi - (double)lo * lo)});
    taken[k] = 1;
  }
  if (js.empty()) return;
  // Each job's K blocks: the P plane blocks of every chunk, and the dash
  // products of the chunks its rows have a '-' in. The chunk list is built on
  // the device from the expansion's marks (k_dash_list, below), in stream
  // order after the operands; the host orders the jobs by the plane blocks.
  std::vector<uint32_t> kcost(specs.size(), 0);
  for (const Job &j : js) {
    const hd_alignment *o = specs[j.k].aln->base ? specs[j.k].aln->base : specs[j.k].aln;
    kcost[j.k] = (uint32_t)(o->planes * (o->words / 8));
  }
  // CTAs draw items from a queue in list order: the costliest items first
  // (an item's cost is its K length), biggest jobs first among equals, so
  // that the cheap items fill the tail
  std::stable_sort(js.begin(), js.end(), [&](const Job &a, const Job &b) {
    return kcost[a.k] != kcost[b.k] ? kcost[a.k] > kcost[b.k] : a.cost > b.cost;
  });
  // Items of each job: pairs of 128-row tiles (a single one where a range is
  // odd; single ones throughout with mma_rows 1) x kTN-column tiles up to the
  // last column any of their rows needs, in bands of mma_band tile rows,
  // column-major within a band.
  std::vector<MmaItem> list;
  for (uint32_t q = 0; q < (uint32_t)js.size(); ++q) {
    const TileConfig &cfg = specs[js[q].k].cfg;
    const uint32_t band = (uint32_t)mma_band_of(cfg), rows = (uint32_t)mma_rows_of(cfg);
    for (uint32_t b = js[q].t_lo; b < js[q].t_hi; b += band) {
      const uint32_t e = std::min(b + band, js[q].t_hi);
      const uint32_t j_end = (uint32_t)ceil_div((uint64_t)e * kTM - 1, kTN);
      for (uint32_t J = 0; J < j_end; ++J)
        for (uint32_t I = b; I < e; I += rows) {
          const uint32_t h = std::min(rows, e - I);
          // rows [128 I, 128 (I + h)) need columns < 128 (I + h) - 1; where
          // only the second row tile reaches column tile J, it goes alone
          if ((uint64_t)J * kTN >= (uint64_t)(I + h) * kTM - 1) continue;
          if (h == 2 && (uint64_t)J * kTN >= (uint64_t)(I + 1) * kTM - 1)
            list.push_back({q, I + 1, J, 1});
          else
            list.push_back({q, I, J, h});
        }
    }
  }
  // Work distribution. One matrix: every item costs the same, and the CTAs
  // take them round-robin, the last pairs split into single row tiles until
  // the count is a multiple of the grid, so that every CTA ends within one
  // row tile of the others. Several matrices (items of unequal length): the
  // CTAs draw items from a queue, and its last `grid` pairs are split, so
  // that the CTAs finish within about half an item of each other.
  // HAMMINGDIST_MMA_SCHEDULE=static|queue picks one for every launch. A
  // short list splits every pair to fill more SMs.
  const int sms = sm_limit > 0 && sm_limit < ctx->sm_count ? sm_limit : ctx->sm_count;
  bool queue = js.size() > 1;
  if (const char *e = std::getenv("HAMMINGDIST_MMA_SCHEDULE")) queue = std::string(e) == "queue";
  uint64_t pairs = 0;
  for (const MmaItem &m : list) pairs += m.halves == 2;
  const uint64_t grid_n = std::min<uint64_t>(list.size() + pairs, (uint64_t)sms);
  uint64_t split = list.size() < grid_n ? pairs
                   : queue ? std::min<uint64_t>(pairs, grid_n)
                           : (grid_n - list.size() % grid_n) % grid_n;
  std::vector<MmaItem> tail;
  for (size_t k = list.size(); k-- > 0 && split > 0;) {
    if (list[k].halves != 2) continue;
    tail.push_back({list[k].job, list[k].I + 1, list[k].J, 1});
    list[k].halves = 1;
    --split;
  }
  list.insert(list.end(), tail.rbegin(), tail.rend());
  // one device block: [tensor maps (3 per job)][jobs][items][queue counter]
  // [dash chunk lists]
  const size_t nj = js.size();
  const size_t tm_bytes = nj * 3 * sizeof(CUtensorMap);
  const size_t job_bytes = round_up(nj * sizeof(MmaJob), 64);
  const size_t item_bytes = round_up(list.size() * sizeof(MmaItem), 16);
  size_t dash_words = 0;
  for (const Job &j : js) {
    const hd_alignment *o = specs[j.k].aln->base ? specs[j.k].aln->base : specs[j.k].aln;
    dash_words += o->words / 8;
  }
  const size_t dash_at = tm_bytes + job_bytes + item_bytes + 16;
  std::vector<uint8_t> host(dash_at + dash_words * 4 + 4, 0);
  DevBuf dev(host.size(), stream);
  auto *tms = reinterpret_cast<CUtensorMap *>(host.data());
  auto *jobs = reinterpret_cast<MmaJob *>(host.data() + tm_bytes);
  const auto *d_tms = reinterpret_cast<const CUtensorMap *>(dev.p);
  size_t dash_off = 0;
  for (size_t q = 0; q < nj; ++q) {
    const PairJobSpec &sp = specs[js[q].k];
    const hd_alignment *a = sp.aln;
    const hd_alignment *o = a->base ? a->base : a;
    const uint64_t rb = o->words * row_bytes_per_word((uint32_t)o->planes);
    make_tmap_u8(ctx, &tms[3 * q], ops[js[q].k], rb, a->n_rows, 2 * kTM);
    make_tmap_u8(ctx, &tms[3 * q + 1], ops[js[q].k], rb, a->n_rows, kTM);
    make_tmap_u8(ctx, &tms[3 * q + 2], ops[js[q].k], rb, a->n_rows, kTN);
    MmaJob &m = jobs[q];
    m.tm256 = d_tms + 3 * q;
    m.tm128 = d_tms + 3 * q + 1;
    m.tmb = d_tms + 3 * q + 2;
    m.out = sp.d_out;
    m.out_base = sp.out_base;
    m.n = (uint32_t)a->n_rows;
    m.nkb = 0;  // set by k_dash_list
    m.chunks = (uint32_t)(o->words / 8);
    m.dash_list = reinterpret_cast<const uint32_t *>(static_cast<uint8_t *>(dev.p) + dash_at) + dash_off;
    m.dash_marks = dash_marks[js[q].k];
    dash_off += m.chunks;
    // the launch's lower-triangle pairs (for its multiply-add count)
    const uint64_t r_lo = (uint64_t)js[q].t_lo * kTM, r_hi = std::min<uint64_t>((uint64_t)js[q].t_hi * kTM, a->n_rows);
    m.pairs = r_hi * (r_hi - 1) / 2 - (r_lo ? r_lo * (r_lo - 1) / 2 : 0);
    m.planes = (uint32_t)o->planes;
    m.sites = (uint32_t)a->length;
    m.max_dist = sp.max_dist;
    m.dtype = (uint32_t)sp.dtype;
  }
  std::memcpy(host.data() + tm_bytes + job_bytes, list.data(), list.size() * sizeof(MmaItem));
  // staged in pinned memory (pageable for a large table): `host` may go when this returns
  upload_table(ctx, dev.p, host.data(), host.size(), stream);
  k_dash_list<<<(unsigned)nj, 32, 0, stream>>>(reinterpret_cast<MmaJob *>(dev.as<uint8_t>() + tm_bytes),
                                              mma_mac_counter(ctx));
  HD_LAUNCHED(ctx);
  PairLaunchPlan::Launch L;
  L.mma = true;
  L.fn = reinterpret_cast<const void *>(k_pairwise_mma);
  L.smem = kMmaSmem;
  L.tile = kTM;
  L.jobs = nj;
  L.tiles = list.size();
  L.grid = grid_n;
  L.d_jobs = dev.as<uint8_t>() + tm_bytes;
  L.d_items = dev.as<uint8_t>() + tm_bytes + job_bytes;
  L.d_counter = reinterpret_cast<unsigned long long *>(dev.as<uint8_t>() + tm_bytes + job_bytes +
                                                       item_bytes);
  L.queue = queue;
  plan->launches.push_back(L);
  plan->blocks.push_back(std::move(dev));
}

void launch_mma(hd_ctx *ctx, const PairLaunchPlan::Launch &L, cudaStream_t stream) {
  set_smem_once();
  // the item queue starts empty at every launch (also when a graph replays it)
  HD_CUDA(cudaMemsetAsync(L.d_counter, 0, sizeof(unsigned), stream));
  k_pairwise_mma<<<(unsigned)L.grid, kMmaThreads, kMmaSmem, stream>>>(
      static_cast<const MmaJob *>(L.d_jobs), static_cast<const MmaItem *>(L.d_items),
      (uint32_t)L.tiles, reinterpret_cast<unsigned *>(L.d_counter), L.queue ? 1u : 0u,
      ctx->d_status);
  HD_LAUNCHED(ctx);
  ctx->last_pair_tiles += L.tiles;
}

bool pairwise_mma(hd_ctx *ctx, const hd_alignment *aln, int dtype_bytes, uint32_t max_dist,
                  void *d_out, uint64_t out_base, uint32_t tile_lo, uint32_t tile_hi,
                  cudaStream_t stream, int sm_limit) {
  if (!mma_eligible(aln)) return false;
  std::vector<PairJobSpec> specs(1);
  PairJobSpec &sp = specs[0];
  sp.aln = aln;
  sp.dtype = dtype_bytes;
  sp.max_dist = max_dist;
  sp.d_out = d_out;
  sp.out_base = out_base;
  // the tensor-core settings of the whole matrix's bucket; row tiles of 128
  sp.cfg = tile_config_for(ctx, aln->n_rows, aln->length, dtype_bytes);
  sp.cfg.tile = kTM;
  sp.tile_lo = tile_lo;
  sp.tile_hi = std::min<uint32_t>(tile_hi, (uint32_t)ceil_div(aln->n_rows, kTM));
  if (sp.tile_hi <= sp.tile_lo) return true;
  PairLaunchPlan plan;
  std::vector<char> taken;
  prepare_mma_jobs(ctx, specs, stream, &plan, sm_limit, taken);
  if (!taken[0]) return false;
  for (const auto &L : plan.launches) launch_mma(ctx, L, stream);
  return true;  // the plan's device block is freed in stream order, after the kernel
}

}  // namespace hd
