// Device-side text writers.
//
// Replaces lower_triangular_lines / partial_write_lower_triangular
// (include/hamming/hamming_utils.hh:19-104) and DataSet::dump_sparse
// (include/hamming/hamming.hh:79-114), which format on the CPU with fmt.
// One warp per row: the row's entries are contiguous in the lower triangle;
// per 32 entries each lane computes its text length, a warp prefix sum places
// it, and the lane writes its digits. Row starts come from a device scan of
// per-row text lengths.
#include <mutex>

#include "hd_internal.cuh"

namespace hd {

__device__ inline uint32_t ndig(uint32_t v) {
  return v < 10u ? 1 : v < 100u ? 2 : v < 1000u ? 3 : v < 10000u ? 4 : v < 100000u ? 5
       : v < 1000000u ? 6 : v < 10000000u ? 7 : v < 100000000u ? 8 : v < 1000000000u ? 9 : 10;
}

__device__ inline void put_dec(char *dst, uint32_t v, uint32_t nd) {
  for (int k = (int)nd - 1; k >= 0; --k) {
    dst[k] = (char)('0' + v % 10u);
    v /= 10u;
  }
}

__host__ __device__ inline uint64_t row_index(uint64_t i) { return i * (i - 1) / 2; }

// --------------------------------------------------- lower-triangular text
// Row i (i >= 1): "d(i,0),d(i,1),...,d(i,i-1)\n".
template <typename T>
__global__ void k_lt_len(const T *lt, uint64_t lt_base, uint64_t i_lo, uint64_t rows,
                         uint64_t *row_len) {
  const int lane = threadIdx.x & 31;
  uint64_t wid = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  uint64_t nwarps = (gridDim.x * (uint64_t)blockDim.x) >> 5;
  for (uint64_t q = wid; q < rows; q += nwarps) {
    const uint64_t i = i_lo + q;
    const T *rp = lt + (row_index(i) - lt_base);
    uint64_t len = 0;
    for (uint64_t j = lane; j < i; j += 32) len += ndig((uint32_t)rp[j]) + 1;
    len = warp_sum(len);
    if (lane == 0) row_len[q] = len;
  }
}

template <typename T>
__global__ void k_lt_write(const T *lt, uint64_t lt_base, uint64_t i_lo, uint64_t rows,
                           const uint64_t *row_off, char *text) {
  const int lane = threadIdx.x & 31;
  uint64_t wid = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  uint64_t nwarps = (gridDim.x * (uint64_t)blockDim.x) >> 5;
  for (uint64_t q = wid; q < rows; q += nwarps) {
    const uint64_t i = i_lo + q;
    const T *rp = lt + (row_index(i) - lt_base);
    uint64_t pos = row_off[q];
    for (uint64_t j0 = 0; j0 < i; j0 += 32) {
      const uint64_t j = j0 + lane;
      const bool on = j < i;
      const uint32_t v = on ? (uint32_t)rp[j] : 0u;
      const uint32_t nd = on ? ndig(v) : 0u;
      const uint32_t len = on ? nd + 1 : 0u;
      const uint32_t inc = warp_incl_scan(len);
      if (on) {
        char *dst = text + pos + inc - len;
        put_dec(dst, v, nd);
        dst[nd] = (j + 1 == i) ? '\n' : ',';
      }
      pos += __shfl_sync(0xffffffffu, inc, 31);
    }
  }
}

static unsigned warp_grid(hd_ctx *ctx, uint64_t rows) {
  uint64_t g = ceil_div(rows * 32, 256);
  uint64_t cap = (uint64_t)ctx->sm_count * 16;
  return (unsigned)(g < cap ? (g ? g : 1) : cap);
}

uint64_t lt_text_bound(uint64_t i_lo, uint64_t i_hi, int dtype_bytes) {
  if (i_lo < 1) i_lo = 1;
  if (i_hi <= i_lo) return 0;
  const uint64_t entries = row_index(i_hi) - row_index(i_lo);
  const uint64_t per = dtype_bytes == 1 ? 4 : dtype_bytes == 2 ? 6 : 11;
  return entries * per;
}

uint64_t format_lt_rows(hd_ctx *ctx, const void *d_lt, int dtype_bytes, uint64_t lt_base,
                        uint64_t i_lo, uint64_t i_hi, char *d_text) {
  if (i_lo < 1) i_lo = 1;
  if (i_hi <= i_lo) return 0;
  const uint64_t rows = i_hi - i_lo;
  cudaStream_t st = ctx->stream;
  DevBuf len(rows * 8, st), off(rows * 8, st), tot(8, st);
  const unsigned g = warp_grid(ctx, rows);
  if (dtype_bytes == 1)
    k_lt_len<uint8_t><<<g, 256, 0, st>>>((const uint8_t *)d_lt, lt_base, i_lo, rows, len.as<uint64_t>());
  else if (dtype_bytes == 2)
    k_lt_len<uint16_t><<<g, 256, 0, st>>>((const uint16_t *)d_lt, lt_base, i_lo, rows, len.as<uint64_t>());
  else
    k_lt_len<uint32_t><<<g, 256, 0, st>>>((const uint32_t *)d_lt, lt_base, i_lo, rows, len.as<uint64_t>());
  HD_LAUNCHED(ctx);
  scan_exclusive<uint64_t>(ctx, len.as<uint64_t>(), off.as<uint64_t>(), rows, tot.as<uint64_t>());
  if (dtype_bytes == 1)
    k_lt_write<uint8_t><<<g, 256, 0, st>>>((const uint8_t *)d_lt, lt_base, i_lo, rows, off.as<uint64_t>(), d_text);
  else if (dtype_bytes == 2)
    k_lt_write<uint16_t><<<g, 256, 0, st>>>((const uint16_t *)d_lt, lt_base, i_lo, rows, off.as<uint64_t>(), d_text);
  else
    k_lt_write<uint32_t><<<g, 256, 0, st>>>((const uint32_t *)d_lt, lt_base, i_lo, rows, off.as<uint64_t>(), d_text);
  HD_LAUNCHED(ctx);
  uint64_t total = 0;
  HD_CUDA(cudaMemcpyAsync(&total, tot.p, 8, cudaMemcpyDeviceToHost, st));
  HD_CUDA(cudaStreamSynchronize(st));
  return total;
}

// ------------------------------------------------------ full matrix text
// DataSet::dump (include/hamming/hamming.hh:63-73): row i of the n x n matrix,
// entries (*this)[{i, j}] (0 on the diagonal, lt[i(i-1)/2 + j] below it and
// lt[j(j-1)/2 + i] above it), ", " between entries, '\n' after the row. An
// index past the `entries` values read as 0 (a triangle whose size is not
// n(n-1)/2, where the reference reads out of bounds).
template <typename T>
__device__ inline uint32_t full_entry(const T *lt, uint64_t entries, uint64_t i, uint64_t j) {
  if (i == j) return 0u;
  const uint64_t k = i > j ? row_index(i) + j : row_index(j) + i;
  return k < entries ? (uint32_t)lt[k] : 0u;
}

template <typename T>
__global__ void k_full_len(const T *lt, uint64_t entries, uint64_t n, uint64_t i_lo, uint64_t rows,
                           uint64_t *row_len) {
  const int lane = threadIdx.x & 31;
  uint64_t wid = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  uint64_t nwarps = (gridDim.x * (uint64_t)blockDim.x) >> 5;
  for (uint64_t q = wid; q < rows; q += nwarps) {
    const uint64_t i = i_lo + q;
    uint64_t len = 0;
    for (uint64_t j = lane; j < n; j += 32) len += ndig(full_entry(lt, entries, i, j)) + 2;
    len = warp_sum(len);
    if (lane == 0) row_len[q] = len - 1;  // the last entry has "\n" instead of ", "
  }
}

template <typename T>
__global__ void k_full_write(const T *lt, uint64_t entries, uint64_t n, uint64_t i_lo, uint64_t rows,
                             const uint64_t *row_off, char *text) {
  const int lane = threadIdx.x & 31;
  uint64_t wid = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  uint64_t nwarps = (gridDim.x * (uint64_t)blockDim.x) >> 5;
  for (uint64_t q = wid; q < rows; q += nwarps) {
    const uint64_t i = i_lo + q;
    uint64_t pos = row_off[q];
    for (uint64_t j0 = 0; j0 < n; j0 += 32) {
      const uint64_t j = j0 + lane;
      const bool on = j < n;
      const bool last = j + 1 == n;
      const uint32_t v = on ? full_entry(lt, entries, i, j) : 0u;
      const uint32_t nd = on ? ndig(v) : 0u;
      const uint32_t len = on ? nd + (last ? 1u : 2u) : 0u;
      const uint32_t inc = warp_incl_scan(len);
      if (on) {
        char *dst = text + pos + inc - len;
        put_dec(dst, v, nd);
        if (last) {
          dst[nd] = '\n';
        } else {
          dst[nd] = ',';
          dst[nd + 1] = ' ';
        }
      }
      pos += __shfl_sync(0xffffffffu, inc, 31);
    }
  }
}

uint64_t full_text_bound(uint64_t n, uint64_t i_lo, uint64_t i_hi, int dtype_bytes) {
  if (i_hi <= i_lo) return 0;
  const uint64_t per = dtype_bytes == 1 ? 5 : dtype_bytes == 2 ? 7 : 12;  // digits + ", "
  return (i_hi - i_lo) * (n * per + 1);
}

uint64_t format_full_rows(hd_ctx *ctx, const void *d_lt, uint64_t entries, int dtype_bytes,
                          uint64_t n, uint64_t i_lo, uint64_t i_hi, char *d_text) {
  if (i_hi <= i_lo) return 0;
  const uint64_t rows = i_hi - i_lo;
  cudaStream_t st = ctx->stream;
  DevBuf len(rows * 8, st), off(rows * 8, st), tot(8, st);
  const unsigned g = warp_grid(ctx, rows);
  if (dtype_bytes == 1)
    k_full_len<uint8_t><<<g, 256, 0, st>>>((const uint8_t *)d_lt, entries, n, i_lo, rows, len.as<uint64_t>());
  else if (dtype_bytes == 2)
    k_full_len<uint16_t><<<g, 256, 0, st>>>((const uint16_t *)d_lt, entries, n, i_lo, rows, len.as<uint64_t>());
  else
    k_full_len<uint32_t><<<g, 256, 0, st>>>((const uint32_t *)d_lt, entries, n, i_lo, rows, len.as<uint64_t>());
  HD_LAUNCHED(ctx);
  scan_exclusive<uint64_t>(ctx, len.as<uint64_t>(), off.as<uint64_t>(), rows, tot.as<uint64_t>());
  if (dtype_bytes == 1)
    k_full_write<uint8_t><<<g, 256, 0, st>>>((const uint8_t *)d_lt, entries, n, i_lo, rows, off.as<uint64_t>(), d_text);
  else if (dtype_bytes == 2)
    k_full_write<uint16_t><<<g, 256, 0, st>>>((const uint16_t *)d_lt, entries, n, i_lo, rows, off.as<uint64_t>(), d_text);
  else
    k_full_write<uint32_t><<<g, 256, 0, st>>>((const uint32_t *)d_lt, entries, n, i_lo, rows, off.as<uint64_t>(), d_text);
  HD_LAUNCHED(ctx);
  uint64_t total = 0;
  HD_CUDA(cudaMemcpyAsync(&total, tot.p, 8, cudaMemcpyDeviceToHost, st));
  HD_CUDA(cudaStreamSynchronize(st));
  return total;
}

// ----------------------------------------------------------- sparse text
// Lines "i j d\n" for j < i with d <= threshold (integer compare, as the
// reference's `*d <= threshold`).
template <typename T>
__global__ void k_sp_len(const T *lt, uint64_t lt_base, uint64_t i_lo, uint64_t rows, int64_t thr,
                         uint64_t *row_bytes, uint64_t *row_lines) {
  const int lane = threadIdx.x & 31;
  uint64_t wid = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  uint64_t nwarps = (gridDim.x * (uint64_t)blockDim.x) >> 5;
  for (uint64_t q = wid; q < rows; q += nwarps) {
    const uint64_t i = i_lo + q;
    const T *rp = lt + (row_index(i) - lt_base);
    const uint32_t ndi = ndig((uint32_t)i);
    uint64_t bytes = 0, lines = 0;
    for (uint64_t j = lane; j < i; j += 32) {
      const uint32_t d = rp[j];
      if ((int64_t)d <= thr) {
        bytes += ndi + ndig((uint32_t)j) + ndig(d) + 3;
        ++lines;
      }
    }
    bytes = warp_sum(bytes);
    lines = warp_sum(lines);
    if (lane == 0) {
      row_bytes[q] = bytes;
      if (row_lines) row_lines[q] = lines;
    }
  }
}

template <typename T>
__global__ void k_sp_write(const T *lt, uint64_t lt_base, uint64_t i_lo, uint64_t rows, int64_t thr,
                           const uint64_t *row_off, char *text) {
  const int lane = threadIdx.x & 31;
  uint64_t wid = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  uint64_t nwarps = (gridDim.x * (uint64_t)blockDim.x) >> 5;
  for (uint64_t q = wid; q < rows; q += nwarps) {
    const uint64_t i = i_lo + q;
    const T *rp = lt + (row_index(i) - lt_base);
    const uint32_t ndi = ndig((uint32_t)i);
    uint64_t pos = row_off[q];
    for (uint64_t j0 = 0; j0 < i; j0 += 32) {
      const uint64_t j = j0 + lane;
      const uint32_t d = j < i ? (uint32_t)rp[j] : 0u;
      const bool on = j < i && (int64_t)d <= thr;
      const uint32_t ndj = ndig((uint32_t)j), ndd = ndig(d);
      const uint32_t len = on ? ndi + ndj + ndd + 3 : 0u;
      const uint32_t inc = warp_incl_scan(len);
      if (on) {
        char *dst = text + pos + inc - len;
        put_dec(dst, (uint32_t)i, ndi);
        dst[ndi] = ' ';
        put_dec(dst + ndi + 1, (uint32_t)j, ndj);
        dst[ndi + 1 + ndj] = ' ';
        put_dec(dst + ndi + ndj + 2, d, ndd);
        dst[ndi + ndj + ndd + 2] = '\n';
      }
      pos += __shfl_sync(0xffffffffu, inc, 31);
    }
  }
}

void sparse_row_sizes(hd_ctx *ctx, const void *d_lt, int dtype_bytes, uint64_t lt_base,
                      uint64_t i_lo, uint64_t i_hi, int64_t threshold, uint64_t *d_row_bytes,
                      uint64_t *d_row_lines) {
  if (i_lo < 1) i_lo = 1;
  if (i_hi <= i_lo) return;
  const uint64_t rows = i_hi - i_lo;
  const unsigned g = warp_grid(ctx, rows);
  cudaStream_t st = ctx->stream;
  if (dtype_bytes == 1)
    k_sp_len<uint8_t><<<g, 256, 0, st>>>((const uint8_t *)d_lt, lt_base, i_lo, rows, threshold, d_row_bytes, d_row_lines);
  else if (dtype_bytes == 2)
    k_sp_len<uint16_t><<<g, 256, 0, st>>>((const uint16_t *)d_lt, lt_base, i_lo, rows, threshold, d_row_bytes, d_row_lines);
  else
    k_sp_len<uint32_t><<<g, 256, 0, st>>>((const uint32_t *)d_lt, lt_base, i_lo, rows, threshold, d_row_bytes, d_row_lines);
  HD_LAUNCHED(ctx);
}

uint64_t format_sparse_rows(hd_ctx *ctx, const void *d_lt, int dtype_bytes, uint64_t lt_base,
                            uint64_t i_lo, uint64_t i_hi, int64_t threshold,
                            const uint64_t *d_row_bytes, char *d_text) {
  if (i_lo < 1) i_lo = 1;
  if (i_hi <= i_lo) return 0;
  const uint64_t rows = i_hi - i_lo;
  cudaStream_t st = ctx->stream;
  DevBuf off(rows * 8, st), tot(8, st);
  scan_exclusive<uint64_t>(ctx, d_row_bytes, off.as<uint64_t>(), rows, tot.as<uint64_t>());
  const unsigned g = warp_grid(ctx, rows);
  if (dtype_bytes == 1)
    k_sp_write<uint8_t><<<g, 256, 0, st>>>((const uint8_t *)d_lt, lt_base, i_lo, rows, threshold, off.as<uint64_t>(), d_text);
  else if (dtype_bytes == 2)
    k_sp_write<uint16_t><<<g, 256, 0, st>>>((const uint16_t *)d_lt, lt_base, i_lo, rows, threshold, off.as<uint64_t>(), d_text);
  else
    k_sp_write<uint32_t><<<g, 256, 0, st>>>((const uint32_t *)d_lt, lt_base, i_lo, rows, threshold, off.as<uint64_t>(), d_text);
  HD_LAUNCHED(ctx);
  uint64_t total = 0;
  HD_CUDA(cudaMemcpyAsync(&total, tot.p, 8, cudaMemcpyDeviceToHost, st));
  HD_CUDA(cudaStreamSynchronize(st));
  return total;
}

}  // namespace hd

// ===================================================== allocation-free text
// A variant of the lower-triangular formatter above for callers that must not
// allocate device memory: code that runs inside a host application whose
// device memory is fully owned by its own allocator or capped by a fixed
// budget, and latency-critical loops that cannot afford cudaMalloc/cudaFree
// (cudaFree synchronises the whole device). Its scratch (per-row text
// lengths, their offsets and the scan's block sums) lives in one file-scope
// device array of fixed size instead of pool allocations.
namespace {

constexpr uint64_t kNoAllocMaxRows = 262144;  // rows of text (nsamples - 1)
constexpr uint64_t kNoAllocMaxBlocks = (kNoAllocMaxRows + hd::kScanTile - 1) / hd::kScanTile;
constexpr uint64_t kNoAllocWords = 2 * kNoAllocMaxRows + kNoAllocMaxBlocks + 8;  // ~4.2 MB

// Held by every GPU that loads the library, until the process exits.
static __device__ __align__(256) uint64_t g_noalloc_scratch[kNoAllocWords];

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
uint64_t *g_noalloc_ptr[kNoAllocMaxDevices] = {};

// Device address of the scratch array on `device`, looked up once per device
// with that device current (in host code the array's name is only a host-side
// stand-in, not a device address).
uint64_t *noalloc_scratch(int device) {
  if (device < 0 || device >= kNoAllocMaxDevices)
    hd::fail(HD_ERR_ARG, "device ordinal out of range for the allocation-free formatter");
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[device]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess)
      hd::fail(HD_ERR_CUDA, std::string("cudaGetSymbolAddress failed: ") + cudaGetErrorString(e));
    g_noalloc_ptr[device] = static_cast<uint64_t *>(p);
  }
  return g_noalloc_ptr[device];
}

template <typename T>
uint64_t noalloc_text(hd_ctx *ctx, const T *d_lt, uint64_t nsamples, char *d_text,
                      uint64_t capacity, uint64_t *scratch) {
  using namespace hd;
  const uint64_t rows = nsamples - 1;  // text rows i = 1 .. nsamples-1
  uint64_t *row_len = scratch;
  uint64_t *row_off = scratch + kNoAllocMaxRows;
  uint64_t *sums = scratch + 2 * kNoAllocMaxRows;
  uint64_t *total = sums + kNoAllocMaxBlocks;
  const uint64_t nb = ceil_div(rows, kScanTile);
  const unsigned g = warp_grid(ctx, rows);
  cudaStream_t st = ctx->stream;
  // every scratch word read below is written earlier in this call, so nothing
  // has to be cleared between calls
  k_lt_len<T><<<g, 256, 0, st>>>(d_lt, 0, 1, rows, row_len);
  HD_LAUNCHED(ctx);
  k_scan_reduce<uint64_t><<<(unsigned)nb, kScanThreads, 0, st>>>(row_len, rows, sums);
  HD_LAUNCHED(ctx);
  k_scan_top<void><<<1, 1024, 0, st>>>(sums, nb, total);
  HD_LAUNCHED(ctx);
  k_scan_down<uint64_t><<<(unsigned)nb, kScanThreads, 0, st>>>(row_len, row_off, rows, sums);
  HD_LAUNCHED(ctx);
  uint64_t bytes = 0;
  HD_CUDA(cudaMemcpyAsync(&bytes, total, sizeof(bytes), cudaMemcpyDeviceToHost, st));
  HD_CUDA(cudaStreamSynchronize(st));
  if (bytes > capacity) return bytes;  // the caller reports the shortfall
  k_lt_write<T><<<g, 256, 0, st>>>(d_lt, 0, 1, rows, row_off, d_text);
  HD_LAUNCHED(ctx);
  HD_CUDA(cudaStreamSynchronize(st));
  return bytes;
}

}  // namespace

extern "C" int hd_lower_triangular_text_noalloc(hd_ctx *ctx, const void *d_lt, uint64_t nsamples,
                                                int dtype_bytes, char *d_text,
                                                uint64_t text_capacity, uint64_t *text_bytes) {
  if (!ctx || !text_bytes) return HD_ERR_ARG;
  *text_bytes = 0;
  try {
    HD_CUDA(cudaSetDevice(ctx->device));
    if (dtype_bytes != 1 && dtype_bytes != 2 && dtype_bytes != 4)
      hd::fail(HD_ERR_ARG, "dtype_bytes must be 1, 2 or 4");
    if (nsamples > kNoAllocMaxRows)
      hd::fail(HD_ERR_ARG, "hd_lower_triangular_text_noalloc: nsamples " + std::to_string(nsamples) +
                               " exceeds its fixed scratch limit of " +
                               std::to_string(kNoAllocMaxRows) + " rows");
    if (nsamples < 2) return HD_OK;  // no entries, no text
    if (!d_lt || (!d_text && text_capacity)) hd::fail(HD_ERR_ARG, "null buffer");
    uint64_t *scratch = noalloc_scratch(ctx->device);
    uint64_t need;
    if (dtype_bytes == 1)
      need = noalloc_text(ctx, static_cast<const uint8_t *>(d_lt), nsamples, d_text, text_capacity, scratch);
    else if (dtype_bytes == 2)
      need = noalloc_text(ctx, static_cast<const uint16_t *>(d_lt), nsamples, d_text, text_capacity, scratch);
    else
      need = noalloc_text(ctx, static_cast<const uint32_t *>(d_lt), nsamples, d_text, text_capacity, scratch);
    *text_bytes = need;
    if (need > text_capacity)
      hd::fail(HD_ERR_ARG, "text buffer too small: " + std::to_string(need) + " bytes needed");
    return HD_OK;
  } catch (const hd::Error &e) {
    ctx->err = e.msg;
    return e.code;
  }
}

