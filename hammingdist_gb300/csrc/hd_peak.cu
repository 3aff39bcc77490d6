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
  // pair-sites bound of the 4 LOP3 + 1 POPC mix when the two pipes overlap
  if (mix) *mix = std::min(8.0 * (ops / t1), 32.0 * (ops / 4 / t2));
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
