// Seeded synthetic FASTA written directly into device memory, for resident
// sets too large to generate on the host quickly (n up to 200,000 rows of
// L = 29,903 sites is 6 GB of text). The content follows the same model as
// hammingdist_gb300/synth.py: a root uniform over ACGT, per-site substitution
// with probability p (new base uniform over ACGT), internal N runs of 1-50
// sites (about n_rate per site), and leading/trailing '-' runs of 0..dash_max.
// Every byte is a pure function of (seed, record, site), so the host can
// rebuild any root or record (synth.device_root / synth.device_record).
// Records are ">s%09d\n" + L sites + "\n". No reference counterpart.
#include "hd_internal.cuh"

namespace hd {

__host__ __device__ inline uint64_t sx_mix(uint64_t x) {
  x ^= x >> 30;
  x *= 0xbf58476d1ce4e5b9ull;
  x ^= x >> 27;
  x *= 0x94d049bb133111ebull;
  x ^= x >> 31;
  return x;
}
// h(seed, a, b): the generator's random stream
__host__ __device__ inline uint64_t sx_hash(uint64_t seed, uint64_t a, uint64_t b) {
  return sx_mix(seed + a * 0x9e3779b97f4a7c15ull + b * 0xd1b54a32d192ed03ull);
}

constexpr int kSynthRuns = 32;       // candidate N runs per record
constexpr int kSynthHeader = 12;     // ">s" + 9 digits + "\n"
constexpr uint64_t kSynthChunk = 4096;

// grid: (record, chunk of 4096 bytes of the record)
__global__ void k_synth(uint64_t seed, uint64_t n, uint64_t L, uint64_t p_thr, uint32_t dash_max,
                        uint64_t run_thr, uint8_t *out) {
  __shared__ uint32_t run_lo[kSynthRuns], run_hi[kSynthRuns];
  __shared__ uint32_t lead, trail;
  const uint64_t rec_bytes = L + kSynthHeader + 1;
  const uint64_t chunks = (rec_bytes + kSynthChunk - 1) / kSynthChunk;
  const uint64_t r = blockIdx.x / chunks, c = blockIdx.x % chunks;
  if (r >= n) return;
  if (threadIdx.x < kSynthRuns) {
    const uint32_t j = threadIdx.x;
    const bool on = sx_hash(seed, r, 100 + j) < run_thr;
    const uint32_t st = (uint32_t)(sx_hash(seed, r, 200 + j) % L);
    const uint32_t len = 1 + (uint32_t)(sx_hash(seed, r, 300 + j) % 50);
    run_lo[j] = on ? st : 0;
    const uint64_t end = (uint64_t)st + len;
    run_hi[j] = on ? (uint32_t)(end < L ? end : L) : 0;
  }
  if (threadIdx.x == 0) {
    lead = (uint32_t)(sx_hash(seed, r, 1) % (dash_max + 1ull));
    trail = (uint32_t)(sx_hash(seed, r, 2) % (dash_max + 1ull));
  }
  __syncthreads();
  const char acgt[4] = {'A', 'C', 'G', 'T'};
  uint8_t *rec = out + r * rec_bytes;
  const uint64_t b0 = c * kSynthChunk, b1 = min(b0 + kSynthChunk, rec_bytes);
  for (uint64_t b = b0 + threadIdx.x; b < b1; b += blockDim.x) {
    uint8_t ch;
    if (b < kSynthHeader) {
      if (b == 0) ch = '>';
      else if (b == 1) ch = 's';
      else if (b == kSynthHeader - 1) ch = '\n';
      else {  // 9 digits of r, most significant first
        uint64_t v = r;
        for (uint64_t k = b; k < kSynthHeader - 2; ++k) v /= 10;
        ch = (uint8_t)('0' + v % 10);
      }
    } else if (b == rec_bytes - 1) {
      ch = '\n';
    } else {
      const uint64_t s = b - kSynthHeader;
      ch = acgt[sx_hash(seed, 0xffffffffull, s) & 3];  // root
      const uint64_t u = sx_hash(seed, r + 1, s);
      if (u < p_thr) ch = acgt[sx_hash(seed ^ 0x5bd1e995ull, r + 1, s) & 3];  // substitution
      for (int j = 0; j < kSynthRuns; ++j)
        if (s >= run_lo[j] && s < run_hi[j]) ch = 'N';
      if (s < lead || s >= L - trail) ch = '-';
    }
    rec[b] = ch;
  }
}

}  // namespace hd

extern "C" int hd_synthetic_fasta(hd_ctx *ctx, uint64_t n, uint64_t L, double p, uint64_t seed,
                                  uint32_t dash_max, double n_rate, void *d_out,
                                  uint64_t capacity, uint64_t *nbytes) {
  if (!ctx || !nbytes || L == 0) return HD_ERR_ARG;
  const uint64_t rec = L + hd::kSynthHeader + 1;
  *nbytes = n * rec;
  if (!d_out) return HD_OK;  // size query
  if (capacity < n * rec || n >= 1000000000ull || 2ull * dash_max >= L) {
    ctx->err = "hd_synthetic_fasta: bad size, buffer too small or dash runs too long";
    return HD_ERR_ARG;
  }
  try {
    HD_CUDA(cudaSetDevice(ctx->device));
    const double two64 = 18446744073709551616.0;
    const uint64_t p_thr = p <= 0 ? 0 : p >= 1 ? ~0ull : (uint64_t)(p * two64);
    const double run_p = n_rate * (double)L / hd::kSynthRuns;
    const uint64_t run_thr = run_p <= 0 ? 0 : run_p >= 1 ? ~0ull : (uint64_t)(run_p * two64);
    const uint64_t chunks = (rec + hd::kSynthChunk - 1) / hd::kSynthChunk;
    const uint64_t blocks = n * chunks;
    if (blocks > 0x7fffffffull) hd::fail(HD_ERR_ARG, "hd_synthetic_fasta: too large");
    if (blocks) {
      hd::k_synth<<<(unsigned)blocks, 256, 0, ctx->stream>>>(seed, n, L, p_thr, dash_max, run_thr,
                                                            static_cast<uint8_t *>(d_out));
      HD_LAUNCHED(ctx);
    }
    HD_CUDA(cudaStreamSynchronize(ctx->stream));
    return HD_OK;
  } catch (const hd::Error &e) {
    ctx->err = e.msg;
    return e.code;
  }
}
