// Device readers of the reference's result files.
//
// Replace from_lower_triangular<T> (include/hamming/hamming.hh:152-166) and
// from_csv / DataSet(filename) (hamming.hh:34-55, src/hamming.cc:23-25),
// which parse on the host with std::getline + std::istringstream + std::stoi.
// The file is split into lines by the device newline index; one warp walks a
// line 32 bytes at a time, finds its commas with a ballot, and the lane that
// holds a field's start parses that field with the rules of std::stoi.
//  - from_lower_triangular: every comma-separated field of every line (an
//    empty line or a trailing comma gives an empty field, which std::stoi
//    rejects), values through safe_int_cast<T>
//    (include/hamming/hamming_impl.hh:37-45: above the maximum saturates,
//    below 0 wraps).
//  - from_csv: nsamples = number of '\n'; line i gives its first i fields to
//    result[i(i-1)/2 + j] of nsamples(nsamples+1)/2 zero-initialised values;
//    when the line has fewer, std::getline leaves the last field in place, so
//    the missing fields repeat it; values are truncated to uint8.
// The first field std::stoi would reject, in file order, decides the error:
// no digits (std::invalid_argument) or a value outside int
// (std::out_of_range).
#include <climits>
#include <cmath>

#include "hd_internal.cuh"

namespace hd {

namespace {

// std::stoi on p[a..): C-locale whitespace, an optional sign, then digits up
// to the first non-digit. Returns 0 (value in *v), 1 (no digits) or 2
// (outside int). Bytes past `end` are not read. A field's own end needs no
// check: ',' stops every phase.
__device__ inline int dev_stoi(const uint8_t *p, uint64_t a, uint64_t end, int *v) {
  uint64_t k = a;
  while (k < end) {
    const uint8_t c = p[k];
    if (c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r') ++k;
    else break;
  }
  bool neg = false;
  if (k < end && (p[k] == '+' || p[k] == '-')) {
    neg = p[k] == '-';
    ++k;
  }
  const uint64_t d0 = k;
  long long acc = 0;
  while (k < end && p[k] >= '0' && p[k] <= '9') {
    if (acc < (1ll << 40)) acc = acc * 10 + (p[k] - '0');
    ++k;
  }
  if (k == d0) return 1;
  if (neg) acc = -acc;
  if (acc > INT_MAX || acc < INT_MIN) return 2;
  *v = (int)acc;
  return 0;
}

// safe_int_cast<T>(x): x above the maximum saturates, otherwise static_cast
template <typename T>
__device__ inline T safe_cast(int x) {
  const int mx = (int)(T)~(T)0;
  return x > mx ? (T)mx : (T)x;
}

// line k of M: [start, end)
__device__ inline void line_span(uint64_t k, const uint64_t *nl, uint64_t m_nl, uint64_t n,
                                 uint64_t &start, uint64_t &end) {
  start = k ? nl[k - 1] + 1 : 0;
  end = k < m_nl ? nl[k] : n;
}

// fields per line = commas + 1
__global__ void k_line_fields(const uint8_t *p, uint64_t n, const uint64_t *nl, uint64_t m_nl,
                              uint64_t M, uint64_t *cnt) {
  const int lane = threadIdx.x & 31;
  uint64_t wid = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  uint64_t nwarps = (gridDim.x * (uint64_t)blockDim.x) >> 5;
  for (uint64_t k = wid; k < M; k += nwarps) {
    uint64_t s, e;
    line_span(k, nl, m_nl, n, s, e);
    uint64_t c = 0;
    for (uint64_t x = s + lane; x < e; x += 32) c += p[x] == ',' ? 1u : 0u;
    c = warp_sum(c);
    if (lane == 0) cnt[k] = c + 1;
  }
}

__device__ inline void note_error(unsigned long long *err, uint64_t key, int kind) {
  atomicMin(err, (unsigned long long)((key << 2) | (uint64_t)kind));
}

// Calls f(field index in line, field start) for the fields of line [s, e)
// with index < limit, from the lane that sees the field's start; the warp
// stops after `limit` fields. Returns the line's number of fields seen (all
// of them when the line has fewer than `limit`).
template <class F>
__device__ inline uint64_t walk_fields(const uint8_t *p, uint64_t s, uint64_t e, uint64_t limit,
                                       int lane, F &&f) {
  if (limit == 0) return 0;
  if (lane == 0) f(0ull, s);
  uint64_t commas = 0;
  for (uint64_t x0 = s; x0 < e && commas + 1 < limit; x0 += 32) {
    const uint64_t x = x0 + lane;
    const bool comma = x < e && p[x] == ',';
    const uint32_t m = __ballot_sync(0xffffffffu, comma);
    const uint64_t idx = commas + 1 + __popc(m & ((1u << lane) - 1u));
    if (comma && idx < limit) f(idx, x + 1);
    commas += __popc(m);
  }
  return commas + 1;
}

template <typename T>
__global__ void k_lt_parse(const uint8_t *p, uint64_t n, const uint64_t *nl, uint64_t m_nl,
                           uint64_t M, const uint64_t *foff, T *out, unsigned long long *err) {
  const int lane = threadIdx.x & 31;
  uint64_t wid = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  uint64_t nwarps = (gridDim.x * (uint64_t)blockDim.x) >> 5;
  for (uint64_t k = wid; k < M; k += nwarps) {
    uint64_t s, e;
    line_span(k, nl, m_nl, n, s, e);
    const uint64_t base = foff[k];
    walk_fields(p, s, e, ~0ull, lane, [&](uint64_t j, uint64_t at) {
      int v = 0;
      const int r = dev_stoi(p, at, e, &v);
      if (r) note_error(err, base + j, r);
      out[base + j] = r ? (T)0 : safe_cast<T>(v);
    });
  }
}

__global__ void k_csv_parse(const uint8_t *p, uint64_t n, const uint64_t *nl, uint64_t m_nl,
                            uint64_t M, uint8_t *out, unsigned long long *err) {
  const int lane = threadIdx.x & 31;
  uint64_t wid = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  uint64_t nwarps = (gridDim.x * (uint64_t)blockDim.x) >> 5;
  for (uint64_t i = wid; i < M; i += nwarps) {
    if (i == 0) continue;  // line 0 gives no field
    uint64_t s, e;
    line_span(i, nl, m_nl, n, s, e);
    const uint64_t base = i * (i - 1) / 2;
    uint64_t last_start = s;  // start of the last field seen (uniform after the walk)
    const uint64_t seen = walk_fields(p, s, e, i, lane, [&](uint64_t j, uint64_t at) {
      int v = 0;
      const int r = dev_stoi(p, at, e, &v);
      if (r) note_error(err, base + j, r);
      out[base + j] = r ? (uint8_t)0 : (uint8_t)(unsigned)v;
    });
    if (seen >= i) continue;
    // fewer than i fields: fields seen..i-1 repeat the last one (field seen-1)
    unsigned long long mx = 0;
    for (uint64_t x = s + lane; x < e; x += 32)
      if (p[x] == ',') mx = x + 1;
    for (int o = 16; o; o >>= 1) {
      const unsigned long long y = __shfl_xor_sync(0xffffffffu, mx, o);
      mx = y > mx ? y : mx;
    }
    if (mx) last_start = mx;
    int v = 0;
    const int r = dev_stoi(p, last_start, e, &v);
    for (uint64_t j = seen + lane; j < i; j += 32) {
      if (r) note_error(err, base + j, r);
      out[base + j] = r ? (uint8_t)0 : (uint8_t)(unsigned)v;
    }
  }
}

unsigned line_grid(hd_ctx *ctx, uint64_t lines) {
  uint64_t g = ceil_div(lines * 32, 256);
  const uint64_t cap = (uint64_t)ctx->sm_count * 16;
  return (unsigned)(g < cap ? (g ? g : 1) : cap);
}

uint64_t lines_of(const uint8_t *d, uint64_t nbytes, uint64_t m_nl, cudaStream_t st) {
  // a last line without '\n' counts as a line (std::getline)
  if (!nbytes) return 0;
  uint8_t last = 0;
  HD_CUDA(cudaMemcpyAsync(&last, d + nbytes - 1, 1, cudaMemcpyDeviceToHost, st));
  HD_CUDA(cudaStreamSynchronize(st));
  return m_nl + (last != '\n' ? 1 : 0);
}

int decode_error(unsigned long long e) { return e == ~0ull ? 0 : (int)(e & 3ull); }

}  // namespace

ParsedValues read_lower_triangular_device(hd_ctx *ctx, const uint8_t *d, uint64_t nbytes,
                                          int dtype_bytes) {
  cudaStream_t st = ctx->stream;
  ParsedValues res;
  uint64_t m_nl = 0;
  DevBuf nl = newline_positions(ctx, d, nbytes, &m_nl);
  const uint64_t M = lines_of(d, nbytes, m_nl, st);
  if (M) {
    DevBuf cnt(M * 8, st), foff(M * 8, st), tot(8, st), err(8, st);
    const unsigned g = line_grid(ctx, M);
    k_line_fields<<<g, 256, 0, st>>>(d, nbytes, nl.as<uint64_t>(), m_nl, M, cnt.as<uint64_t>());
    HD_LAUNCHED(ctx);
    scan_exclusive<uint64_t>(ctx, cnt.as<uint64_t>(), foff.as<uint64_t>(), M, tot.as<uint64_t>());
    uint64_t F = 0;
    HD_CUDA(cudaMemcpyAsync(&F, tot.p, 8, cudaMemcpyDeviceToHost, st));
    HD_CUDA(cudaStreamSynchronize(st));
    res.entries = F;
    res.values = DevBuf((F ? F : 1) * dtype_bytes, st);
    HD_CUDA(cudaMemsetAsync(err.p, 0xff, 8, st));
    if (dtype_bytes == 1)
      k_lt_parse<uint8_t><<<g, 256, 0, st>>>(d, nbytes, nl.as<uint64_t>(), m_nl, M,
                                              foff.as<uint64_t>(), res.values.as<uint8_t>(),
                                              err.as<unsigned long long>());
    else
      k_lt_parse<uint16_t><<<g, 256, 0, st>>>(d, nbytes, nl.as<uint64_t>(), m_nl, M,
                                               foff.as<uint64_t>(), res.values.as<uint16_t>(),
                                               err.as<unsigned long long>());
    HD_LAUNCHED(ctx);
    unsigned long long e = 0;
    HD_CUDA(cudaMemcpyAsync(&e, err.p, 8, cudaMemcpyDeviceToHost, st));
    HD_CUDA(cudaStreamSynchronize(st));
    res.error = decode_error(e);
  } else {
    res.values = DevBuf(dtype_bytes, st);
  }
  // include/hamming/hamming.hh:18-20, 57-61
  res.nsamples = ((uint64_t)std::llround(std::sqrt((double)(8 * res.entries + 1))) + 1) / 2;
  return res;
}

ParsedValues read_csv_device(hd_ctx *ctx, const uint8_t *d, uint64_t nbytes) {
  cudaStream_t st = ctx->stream;
  ParsedValues res;
  uint64_t m_nl = 0;
  DevBuf nl = newline_positions(ctx, d, nbytes, &m_nl);
  const uint64_t M = lines_of(d, nbytes, m_nl, st);
  res.nsamples = m_nl;
  res.entries = m_nl * (m_nl + 1) / 2;
  res.values = DevBuf(res.entries ? res.entries : 1, st);
  if (res.entries) HD_CUDA(cudaMemsetAsync(res.values.p, 0, res.entries, st));
  if (M > 1) {
    DevBuf err(8, st);
    HD_CUDA(cudaMemsetAsync(err.p, 0xff, 8, st));
    k_csv_parse<<<line_grid(ctx, M), 256, 0, st>>>(d, nbytes, nl.as<uint64_t>(), m_nl, M,
                                                   res.values.as<uint8_t>(),
                                                   err.as<unsigned long long>());
    HD_LAUNCHED(ctx);
    unsigned long long e = 0;
    HD_CUDA(cudaMemcpyAsync(&e, err.p, 8, cudaMemcpyDeviceToHost, st));
    HD_CUDA(cudaStreamSynchronize(st));
    res.error = decode_error(e);
  }
  return res;
}

}  // namespace hd
