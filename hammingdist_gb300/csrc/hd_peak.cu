// Integer-pipe peak rates of the device, used as the roofline denominator of
// the pairwise kernel (4 LOP3 + 1 POPC per 32 pair-sites). Each thread runs
// eight interleaved dependent chains; the chains feed each other so that no
// operand is loop-invariant and nothing can be folded. No reference
// counterpart (the reference publishes no device rates).
#include <algorithm>

#include "hd_internal.cuh"

namespace hd {

constexpr int kPeakThreads = 256;
constexpr int kPeakUnroll = 16;

__device__ __forceinline__ uint32_t lop3_xor3(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t d;
  asm volatile("lop3.b32 %0, %1, %2, %3, 0x96;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
  return d;
}
__device__ __forceinline__ uint32_t popc_asm(uint32_t a) {
  uint32_t d;
  asm volatile("popc.b32 %0, %1;" : "=r"(d) : "r"(a));
  return d;
}

__global__ void k_peak_lop3(uint32_t iters, uint32_t *sink) {
  uint32_t x[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) x[k] = threadIdx.x * 0x9e3779b9u + k * 0x85ebca6bu + blockIdx.x;
  for (uint32_t it = 0; it < iters; ++it) {
#pragma unroll
    for (int u = 0; u < kPeakUnroll; ++u)
#pragma unroll
      for (int k = 0; k < 8; ++k) x[k] = lop3_xor3(x[k], x[(k + 1) & 7], x[(k + 3) & 7]);
  }
  uint32_t v = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) v ^= x[k];
  if (v == 0x12345678u) sink[0] = v;  // keeps the chains alive
}

__global__ void k_peak_popc(uint32_t iters, uint32_t *sink) {
  uint32_t x[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) x[k] = threadIdx.x * 0x9e3779b9u + k * 0x85ebca6bu + blockIdx.x;
  for (uint32_t it = 0; it < iters; ++it) {
#pragma unroll
    for (int u = 0; u < kPeakUnroll; ++u)
#pragma unroll
      for (int k = 0; k < 8; ++k) x[k] = popc_asm(x[k]);
  }
  uint32_t v = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) v ^= x[k];
  if (v == 0x12345678u) sink[0] = v;
}

__device__ __forceinline__ uint32_t lop3_and(uint32_t a, uint32_t b) {
  uint32_t d;
  asm volatile("lop3.b32 %0, %1, %2, %1, 0x88;" : "=r"(d) : "r"(a), "r"(b));
  return d;
}
__device__ __forceinline__ uint32_t lop3_or_and(uint32_t x, uint32_t y, uint32_t z) {
  uint32_t d;
  asm volatile("lop3.b32 %0, %1, %2, %3, 0xF8;" : "=r"(d) : "r"(x), "r"(y), "r"(z));
  return d;
}
__device__ __forceinline__ uint32_t mad_asm(uint32_t acc, uint32_t p, uint32_t k) {
  uint32_t d;
  asm volatile("mad.lo.u32 %0, %1, %2, %3;" : "=r"(d) : "r"(p), "r"(k), "r"(acc));
  return d;
}

// The pairwise inner loop's instruction mix from registers alone: per word
// (32 pair-sites) one AND, three OR-AND LOP3s, a POPC and an IMAD
// accumulation; eight chains per thread, each word's operands taken from
// the other chains. Run at the pairwise kernel's occupancy (16 warps per SM),
// it gives the rate this mix reaches with no shared-memory loads, barriers
// or stores.
__global__ void k_peak_mix(uint32_t iters, uint32_t *sink) {
  uint32_t x[8], acc[8];
  const uint32_t c0 = threadIdx.x * 0x1234567u, c1 = blockIdx.x ^ 0x55aa55aau, c2 = c0 * 3u,
                 c3 = c1 + 7u;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    x[k] = threadIdx.x * 0x9e3779b9u + k * 0x85ebca6bu + blockIdx.x;
    acc[k] = 0;
  }
  const uint32_t one = (blockIdx.x >> 30) + 1u;  // 1, unknown to the compiler
  for (uint32_t it = 0; it < iters; ++it) {
#pragma unroll
    for (int u = 0; u < 8; ++u)
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        uint32_t m = lop3_and(x[k], c0);
        m = lop3_or_and(m, x[(k + 1) & 7], c1);
        m = lop3_or_and(m, x[(k + 2) & 7], c2);
        m = lop3_or_and(m, x[(k + 3) & 7], c3);
        acc[k] = mad_asm(acc[k], popc_asm(m), one);
        x[k] = m;
      }
  }
  uint32_t v = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) v ^= x[k] + acc[k];
  if (v == 0x12345678u) sink[0] = v;
}

static double time_kernel(hd_ctx *ctx, void (*kern)(uint32_t, uint32_t *), uint32_t iters,
                          uint32_t *sink, unsigned blocks) {
  cudaEvent_t a, b;
  HD_CUDA(cudaEventCreate(&a));
  HD_CUDA(cudaEventCreate(&b));
  kern<<<blocks, kPeakThreads, 0, ctx->stream>>>(iters / 8, sink);  // warm-up
  HD_LAUNCHED(ctx);
  HD_CUDA(cudaEventRecord(a, ctx->stream));
  kern<<<blocks, kPeakThreads, 0, ctx->stream>>>(iters, sink);
  HD_LAUNCHED(ctx);
  HD_CUDA(cudaEventRecord(b, ctx->stream));
  HD_CUDA(cudaEventSynchronize(b));
  float ms = 0;
  HD_CUDA(cudaEventElapsedTime(&ms, a, b));
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return ms * 1e-3;
}

void measure_int_peaks(hd_ctx *ctx, double *lop3, double *popc, double *mix) {
  DevBuf sink(64, ctx->stream);
  const unsigned blocks = (unsigned)ctx->sm_count * 8;  // 64 warps per SM
  const uint32_t iters = 256;  // ~0.5 ms per kernel at 64 LOP3 lanes/clk/SM
  const double ops = (double)blocks * kPeakThreads * iters * kPeakUnroll * 8;
  double t1 = time_kernel(ctx, k_peak_lop3, iters, sink.as<uint32_t>(), blocks);
  double t2 = time_kernel(ctx, k_peak_popc, iters / 4, sink.as<uint32_t>(), blocks);
  if (lop3) *lop3 = ops / t1;
  if (popc) *popc = ops / 4 / t2;
  // the mix at 16 warps per SM: words = blocks x threads x iters x 64
  const unsigned mix_blocks = (unsigned)ctx->sm_count * 2;
  const uint32_t mix_iters = 1024;
  const double t3 = time_kernel(ctx, k_peak_mix, mix_iters, sink.as<uint32_t>(), mix_blocks);
  if (mix) *mix = 32.0 * (double)mix_blocks * kPeakThreads * mix_iters * 64 / t3;
}

// Bounded-wait self-test: one thread initialises an mbarrier that nothing
// will ever arrive on and waits for it with the same bounded wait the
// pairwise kernel uses; when the limit runs out it records where it gave up
// and returns. Shows on the device that a stuck wait ends with a status the
// host can read and that the context stays usable. Nothing faults or hangs.
__global__ void k_wait_selftest(uint64_t limit_ns, int *status, unsigned long long *waited_ns) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x != 0) return;
  mbar_init(&bar, 1);
  fence_mbar_init();
  const uint64_t t0 = global_ns();
  const bool ok = mbar_wait_bounded(&bar, 0, limit_ns);
  *waited_ns = global_ns() - t0;
  *status = ok ? 0 : kStatusTmaTimeout;
}

}  // namespace hd

extern "C" int hd_selftest_wait_timeout(hd_ctx *ctx, uint64_t limit_ns, int *status,
                                        double *waited_ms) {
  if (!ctx || !status) return HD_ERR_ARG;
  try {
    HD_CUDA(cudaSetDevice(ctx->device));
    if (limit_ns > 1000000000ull) hd::fail(HD_ERR_ARG, "self-test limit above 1 s");
    hd::DevBuf out(16, ctx->stream);
    HD_CUDA(cudaMemsetAsync(out.p, 0xff, 16, ctx->stream));
    hd::k_wait_selftest<<<1, 32, 0, ctx->stream>>>(
        limit_ns, out.as<int>(), reinterpret_cast<unsigned long long *>(out.as<uint8_t>() + 8));
    HD_LAUNCHED(ctx);
    int host[4];
    HD_CUDA(cudaMemcpyAsync(host, out.p, 16, cudaMemcpyDeviceToHost, ctx->stream));
    HD_CUDA(cudaStreamSynchronize(ctx->stream));
    *status = host[0];
    unsigned long long ns;
    std::memcpy(&ns, host + 2, 8);
    if (waited_ms) *waited_ms = ns / 1e6;
    return HD_OK;
  } catch (const hd::Error &e) {
    ctx->err = e.msg;
    return e.code;
  }
}
