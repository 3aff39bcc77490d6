// Device FASTA ingest: newline index, record table, duplicate removal,
// consensus counts, bit-plane packing and reference distances.
//
// Replaces (ssciwr/hammingdist 1.4.0): read_fasta src/hamming_impl.cc:200-242,
// validate_data :80-91, to_dense_data/from_string :190-198/:244-267, the
// consensus of get_reference_expression :142-168 as used by the heuristic of
// include/hamming/hamming_impl.hh:104-118, and fasta_reference_distances /
// fasta_sequence_indices src/hamming.cc:76-141.
#include "hd_internal.cuh"

namespace hd {

// ------------------------------------------------------------ code tables
// Bit p of a code = membership in bit plane p. A pair of sites matches when
// their codes share a bit, so '-' (all ones) matches everything and a code of
// 0 matches nothing.
//  kCodesAnd:     the reference's 4-bit codes (src/hamming_impl.cc:23-44 with
//                 include_x = false): A C G T one-hot, '-' = 1111, else 0000.
//  kCodesSparse:  the sparse rule (src/hamming_impl.cc:93-129) with X invalid:
//                 codes differ and neither is '-' <=> no shared bit, with a
//                 fifth plane for the class of all invalid bytes.
//  kCodesSparseX: the same with X a symbol of its own (6 planes).
void code_table(int table, uint8_t out[256]) {
  for (int c = 0; c < 256; ++c) out[c] = 0;
  if (table == kCodesSparse)
    for (int c = 0; c < 256; ++c) out[c] = 0x10;
  if (table == kCodesSparseX)
    for (int c = 0; c < 256; ++c) out[c] = 0x20;
  out['A'] = 0x1;
  out['C'] = 0x2;
  out['G'] = 0x4;
  out['T'] = 0x8;
  if (table == kCodesAnd) out['-'] = 0x0f;
  if (table == kCodesSparse) out['-'] = 0x1f;
  if (table == kCodesSparseX) {
    out['X'] = 0x10;
    out['-'] = 0x3f;
  }
}

struct Table256 {
  uint8_t v[256];
};

// ------------------------------------------------------------ newline index
constexpr int kNlThreads = 256;
constexpr int kNlIters = 16;
constexpr uint64_t kNlWarpBytes = 32ull * 16 * kNlIters;                  // 8 KB
constexpr uint64_t kNlBlockBytes = kNlWarpBytes * (kNlThreads / 32);      // 64 KB

__device__ inline uint32_t nl_nibble(uint32_t w) {
  uint32_t e = __vcmpeq4(w, 0x0a0a0a0au) & 0x01010101u;
  return (e | (e >> 7) | (e >> 14) | (e >> 21)) & 0xfu;
}

// 16-bit mask of '\n' bytes in p[off, off+16).
__device__ inline uint32_t nl_mask16(const uint8_t *p, uint64_t off, uint64_t n) {
  if (off + 16 <= n) {
    uint4 v = __ldg(reinterpret_cast<const uint4 *>(p + off));
    return nl_nibble(v.x) | (nl_nibble(v.y) << 4) | (nl_nibble(v.z) << 8) | (nl_nibble(v.w) << 12);
  }
  uint32_t m = 0;
  for (int k = 0; k < 16; ++k)
    if (off + k < n && p[off + k] == '\n') m |= 1u << k;
  return m;
}

// Newlines per 64 KB block (counts) and per 8 KB warp span (warp_counts[w]).
// A span with one or two newlines also records their offsets in the span
// (warp_counts[W + 2 w] and [W + 2 w + 1], W = the launch's warps), so that
// the write pass need not read it again: a FASTA line is usually longer than
// a span. Each lane keeps the first two newlines of its own 16-byte slices,
// which it visits in increasing order; the span's first newline is the least
// of the lanes' first ones, and its second the least of the rest.
__global__ void k_nl_count(const uint8_t *p, uint64_t n, uint64_t *counts, uint32_t *warp_counts) {
  __shared__ uint64_t tmp[33];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint64_t base = blockIdx.x * kNlBlockBytes + warp * kNlWarpBytes + lane * 16;
  constexpr uint32_t kNone = 0xFFFFFFFFu;
  uint32_t c = 0, o0 = kNone, o1 = kNone;
#pragma unroll 4
  for (int it = 0; it < kNlIters; ++it) {
    const uint32_t m = nl_mask16(p, base + it * 512ull, n);
    if (m && c < 2) {
      const uint32_t rel = (uint32_t)it * 512u + (uint32_t)lane * 16u;
      const uint32_t a = rel + (uint32_t)(__ffs(m) - 1), m2 = m & (m - 1);
      if (c == 0) {
        o0 = a;
        if (m2) o1 = rel + (uint32_t)(__ffs(m2) - 1);
      } else {
        o1 = a;
      }
    }
    c += __popc(m);
  }
  const uint32_t cw = warp_sum(c);
  const uint32_t wid = blockIdx.x * (kNlThreads / 32) + warp;
  if (lane == 0) warp_counts[wid] = cw;
  if (cw >= 1 && cw <= 2) {  // warp-uniform
    const uint32_t q1 = __reduce_min_sync(0xffffffffu, o0);
    const uint32_t q2 = __reduce_min_sync(0xffffffffu, o0 == q1 ? o1 : o0);
    if (lane == 0) {
      uint32_t *pos = warp_counts + gridDim.x * (kNlThreads / 32) + 2ull * wid;
      pos[0] = q1;
      pos[1] = q2;
    }
  }
  uint64_t tot;
  block_excl_scan<uint64_t>((uint64_t)c, tmp, tot);
  if (threadIdx.x == 0) counts[blockIdx.x] = tot;
}

// Writes the positions of every '\n' in increasing order: each warp starts at
// its block's offset plus the counts of the block's earlier warps; a span
// with one or two newlines takes their offsets from the count pass, a span
// with more scans its lanes' counts where some lane holds a newline.
__global__ void k_nl_write(const uint8_t *p, uint64_t n, const uint64_t *block_off,
                           const uint32_t *warp_counts, uint64_t *nl) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint64_t wbase = blockIdx.x * kNlBlockBytes + warp * kNlWarpBytes;
  const uint32_t wid = blockIdx.x * (kNlThreads / 32) + warp;
  uint64_t off = block_off[blockIdx.x];
  for (int w = 0; w < warp; ++w) off += warp_counts[blockIdx.x * (kNlThreads / 32) + w];
  const uint32_t cw = warp_counts[wid];
  if (cw == 0) return;
  if (cw <= 2) {
    const uint32_t *pos = warp_counts + gridDim.x * (kNlThreads / 32) + 2ull * wid;
    if (lane < (int)cw) nl[off + lane] = wbase + pos[lane];
    return;
  }
  for (int it = 0; it < kNlIters; ++it) {
    uint64_t at = wbase + it * 512ull + lane * 16;
    uint32_t m = nl_mask16(p, at, n);
    if (!__any_sync(0xffffffffu, m != 0)) continue;
    uint32_t cnt = __popc(m);
    uint32_t inc = warp_incl_scan(cnt);
    uint64_t pos = off + inc - cnt;
    while (m) {
      int k = __ffs(m) - 1;
      nl[pos++] = at + k;
      m &= m - 1;
    }
    off += __shfl_sync(0xffffffffu, inc, 31);
  }
}

struct ParseSummary {
  unsigned long long m_nl;      // newlines
  unsigned long long lines;     // M
  unsigned long long R;         // records before the n limit
  unsigned long long Rk;        // records kept
  unsigned long long max_len;
  unsigned long long len0;
  unsigned long long skip;      // records left out at the start
  unsigned int unterminated;    // the last line has no '\n'
  unsigned int unequal;
  unsigned int multi;           // some record spans several non-empty lines
  unsigned int pad;
};

__global__ void k_nl_summary(const uint8_t *p, uint64_t n, const uint64_t *m_nl, ParseSummary *s) {
  s->m_nl = *m_nl;
  s->unterminated = (n > 0 && p[n - 1] != '\n') ? 1u : 0u;
  s->lines = *m_nl + s->unterminated;
}

__device__ inline void line_range(uint64_t k, const uint64_t *nl, uint64_t m_nl, uint64_t n,
                                  uint64_t &start, uint64_t &end) {
  start = k ? nl[k - 1] + 1 : 0;
  end = k < m_nl ? nl[k] : n;
}

// hdr[k] = line k (k >= 1) is a header: non-empty and starting with '>'.
__global__ void k_lines(const uint8_t *p, uint64_t n, const uint64_t *nl, uint64_t m_nl, uint64_t M,
                        uint32_t *hdr) {
  uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (k >= M) return;
  uint64_t s, e;
  line_range(k, nl, m_nl, n, s, e);
  hdr[k] = (k >= 1 && e > s && p[s] == '>') ? 1u : 0u;
}

// Number of records the getline loop of read_fasta produces
// (src/hamming_impl.cc:216-233): the first line is skipped; every later
// header closes a record; the loop ends when the stream reaches its end,
// which happens on reading an unterminated last line. first > 0: the bytes
// before `first` (which follows a '\n') belong to records parsed before,
// so the records up to the header that starts there are left out (s->skip:
// record 0 and those whose header line starts before `first`).
__global__ void k_rec_count(const uint64_t *H_total, const uint32_t *hdr, const uint64_t *H,
                            const uint64_t *nl, uint64_t first, uint64_t n_limit,
                            ParseSummary *s) {
  uint64_t M = s->lines, R;
  if (M == 0) R = 0;
  else if (M == 1) R = s->unterminated ? 0 : 1;
  else R = *H_total + 1 - ((hdr[M - 1] && s->unterminated) ? 1 : 0);
  s->R = R;
  uint64_t skip = 0;
  if (first) {
    // the line that starts at `first` follows the newline at first - 1
    uint64_t lo = 0, hi = s->m_nl;
    while (lo < hi) {
      const uint64_t mid = (lo + hi) / 2;
      if (nl[mid] < first - 1) lo = mid + 1;
      else hi = mid;
    }
    const uint64_t k0 = lo + 1;  // that line
    skip = k0 < M ? H[k0] + 1 : R;
  }
  s->skip = skip;
  const uint64_t after = R > skip ? R - skip : 0;
  s->Rk = (n_limit && n_limit < after) ? n_limit : after;
}

__global__ void k_records(const uint8_t *p, uint64_t n, const uint64_t *nl, uint64_t m_nl,
                          uint64_t M, const uint32_t *hdr, const uint64_t *H,
                          const ParseSummary *s, unsigned long long *rec_len,
                          unsigned int *rec_nseg, uint64_t *rec_start) {
  uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (k == 0 || k >= M || hdr[k]) return;
  uint64_t r = H[k];
  const uint64_t skip = s->skip;
  if (r < skip || r - skip >= s->Rk) return;
  r -= skip;
  uint64_t st, e;
  line_range(k, nl, m_nl, n, st, e);
  if (e == st) return;
  atomicAdd(&rec_len[r], (unsigned long long)(e - st));
  atomicAdd(&rec_nseg[r], 1u);
  rec_start[r] = st;
}

__global__ void k_validate(const unsigned long long *rec_len, const unsigned int *rec_nseg,
                           ParseSummary *s) {
  uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (r >= s->Rk) return;
  unsigned long long l = rec_len[r];
  if (r == 0) s->len0 = l;
  if (l != rec_len[0]) atomicOr(&s->unequal, 1u);
  if (rec_nseg[r] > 1) atomicOr(&s->multi, 1u);
  atomicMax(&s->max_len, l);
}

// Gather of multi-line records: masked line lengths, then line copies.
__global__ void k_seqline_len(const uint64_t *nl, uint64_t m_nl, uint64_t n, uint64_t M,
                              const uint32_t *hdr, const uint64_t *H, const ParseSummary *s,
                              uint64_t *len) {
  uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (k >= M) return;
  uint64_t st, e;
  line_range(k, nl, m_nl, n, st, e);
  const uint64_t skip = s->skip;
  len[k] = (k >= 1 && !hdr[k] && H[k] >= skip && H[k] - skip < s->Rk) ? e - st : 0;
}

__global__ void k_gather_lines(const uint8_t *p, const uint64_t *nl, uint64_t m_nl, uint64_t n,
                               uint64_t M, const uint64_t *len, const uint64_t *dst_off,
                               uint8_t *dst) {
  uint64_t wid = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  uint64_t nwarps = (gridDim.x * (uint64_t)blockDim.x) >> 5;
  for (uint64_t k = wid; k < M; k += nwarps) {
    uint64_t l = len[k];
    if (!l) continue;
    uint64_t st = k ? nl[k - 1] + 1 : 0;
    for (uint64_t i = lane; i < l; i += 32) dst[dst_off[k] + i] = p[st + i];
  }
}

static unsigned grid_for(uint64_t n, int threads) {
  uint64_t g = ceil_div(n ? n : 1, threads);
  return (unsigned)(g > 0x7fffffffull ? 0x7fffffffull : g);
}

DevBuf newline_positions(hd_ctx *ctx, const uint8_t *d, uint64_t nbytes, uint64_t *m_nl) {
  cudaStream_t st = ctx->stream;
  const uint64_t nblk = ceil_div(nbytes ? nbytes : 1, kNlBlockBytes);
  DevBuf counts(nblk * 8, st), offs(nblk * 8, st), total(8, st), wcounts(nblk * 12 * (kNlThreads / 32), st);
  k_nl_count<<<(unsigned)nblk, kNlThreads, 0, st>>>(d, nbytes, counts.as<uint64_t>(),
                                                     wcounts.as<uint32_t>());
  HD_LAUNCHED(ctx);
  scan_exclusive<uint64_t>(ctx, counts.as<uint64_t>(), offs.as<uint64_t>(), nblk,
                           total.as<uint64_t>());
  uint64_t h = 0;
  HD_CUDA(cudaMemcpyAsync(&h, total.p, 8, cudaMemcpyDeviceToHost, st));
  HD_CUDA(cudaStreamSynchronize(st));
  *m_nl = h;
  DevBuf nl((h + 1) * 8, st);
  if (h) {
    k_nl_write<<<(unsigned)nblk, kNlThreads, 0, st>>>(d, nbytes, offs.as<uint64_t>(),
                                                       wcounts.as<uint32_t>(), nl.as<uint64_t>());
    HD_LAUNCHED(ctx);
  }
  return nl;
}

Records parse_fasta(hd_ctx *ctx, const uint8_t *d_file, uint64_t nbytes, uint64_t n_limit,
                    uint64_t first) {
  cudaStream_t st = ctx->stream;
  Records rec;
  uint64_t nblk = ceil_div(nbytes ? nbytes : 1, kNlBlockBytes);
  DevBuf counts(nblk * 8, st), offs(nblk * 8, st), total(8, st), sumbuf(sizeof(ParseSummary), st);
  DevBuf wcounts(nblk * 12 * (kNlThreads / 32), st);
  ParseSummary *d_sum = sumbuf.as<ParseSummary>();
  HD_CUDA(cudaMemsetAsync(d_sum, 0, sizeof(ParseSummary), st));
  k_nl_count<<<(unsigned)nblk, kNlThreads, 0, st>>>(d_file, nbytes, counts.as<uint64_t>(),
                                                     wcounts.as<uint32_t>());
  HD_LAUNCHED(ctx);
  scan_exclusive<uint64_t>(ctx, counts.as<uint64_t>(), offs.as<uint64_t>(), nblk,
                           total.as<uint64_t>());
  k_nl_summary<<<1, 1, 0, st>>>(d_file, nbytes, total.as<uint64_t>(), d_sum);
  HD_LAUNCHED(ctx);
  ParseSummary hs;
  HD_CUDA(cudaMemcpyAsync(&hs, d_sum, sizeof(hs), cudaMemcpyDeviceToHost, st));
  HD_CUDA(cudaStreamSynchronize(st));
  const uint64_t m_nl = hs.m_nl, M = hs.lines;
  DevBuf nl((m_nl + 1) * 8, st);
  if (m_nl) {
    k_nl_write<<<(unsigned)nblk, kNlThreads, 0, st>>>(d_file, nbytes, offs.as<uint64_t>(),
                                                       wcounts.as<uint32_t>(), nl.as<uint64_t>());
    HD_LAUNCHED(ctx);
  }
  DevBuf hdr((M + 1) * 4, st), H((M + 1) * 8, st), htot(8, st);
  HD_CUDA(cudaMemsetAsync(htot.p, 0, 8, st));
  if (M) {
    k_lines<<<grid_for(M, 256), 256, 0, st>>>(d_file, nbytes, nl.as<uint64_t>(), m_nl, M,
                                              hdr.as<uint32_t>());
    HD_LAUNCHED(ctx);
    scan_exclusive<uint32_t>(ctx, hdr.as<uint32_t>(), H.as<uint64_t>(), M, htot.as<uint64_t>());
  }
  k_rec_count<<<1, 1, 0, st>>>(htot.as<uint64_t>(), hdr.as<uint32_t>(), H.as<uint64_t>(),
                               nl.as<uint64_t>(), first, n_limit, d_sum);
  HD_LAUNCHED(ctx);
  const uint64_t cap = M + 1;  // records <= lines
  rec.rec_len = DevBuf(cap * 8, st);
  rec.rec_start = DevBuf(cap * 8, st);
  DevBuf nseg(cap * 4, st);
  HD_CUDA(cudaMemsetAsync(rec.rec_len.p, 0, cap * 8, st));
  HD_CUDA(cudaMemsetAsync(rec.rec_start.p, 0, cap * 8, st));
  HD_CUDA(cudaMemsetAsync(nseg.p, 0, cap * 4, st));
  if (M) {
    k_records<<<grid_for(M, 256), 256, 0, st>>>(
        d_file, nbytes, nl.as<uint64_t>(), m_nl, M, hdr.as<uint32_t>(), H.as<uint64_t>(), d_sum,
        rec.rec_len.as<unsigned long long>(), nseg.as<unsigned int>(), rec.rec_start.as<uint64_t>());
    HD_LAUNCHED(ctx);
    k_validate<<<grid_for(cap, 256), 256, 0, st>>>(rec.rec_len.as<unsigned long long>(),
                                                   nseg.as<unsigned int>(), d_sum);
    HD_LAUNCHED(ctx);
  }
  HD_CUDA(cudaMemcpyAsync(&hs, d_sum, sizeof(hs), cudaMemcpyDeviceToHost, st));
  HD_CUDA(cudaStreamSynchronize(st));
  rec.n = hs.Rk;
  rec.len0 = hs.len0;
  rec.max_len = hs.max_len;
  rec.all_equal = hs.unequal == 0;
  rec.base = d_file;
  rec.bytes = nbytes;
  if (hs.multi) {
    // records spanning several lines: concatenate them into one buffer
    DevBuf len(M * 8, st), dst(M * 8, st), gtot(8, st);
    k_seqline_len<<<grid_for(M, 256), 256, 0, st>>>(nl.as<uint64_t>(), m_nl, nbytes, M,
                                                    hdr.as<uint32_t>(), H.as<uint64_t>(), d_sum,
                                                    len.as<uint64_t>());
    HD_LAUNCHED(ctx);
    scan_exclusive<uint64_t>(ctx, len.as<uint64_t>(), dst.as<uint64_t>(), M, gtot.as<uint64_t>());
    uint64_t total_bytes = 0;
    HD_CUDA(cudaMemcpyAsync(&total_bytes, gtot.p, 8, cudaMemcpyDeviceToHost, st));
    HD_CUDA(cudaStreamSynchronize(st));
    rec.gathered = DevBuf(total_bytes + 16, st);
    k_gather_lines<<<grid_for(M * 32, 256), 256, 0, st>>>(d_file, nl.as<uint64_t>(), m_nl, nbytes,
                                                          M, len.as<uint64_t>(),
                                                          dst.as<uint64_t>(),
                                                          rec.gathered.as<uint8_t>());
    HD_LAUNCHED(ctx);
    if (rec.n)
      scan_exclusive<uint64_t>(ctx, rec.rec_len.as<uint64_t>(), rec.rec_start.as<uint64_t>(),
                               rec.n, gtot.as<uint64_t>());
    rec.base = rec.gathered.as<uint8_t>();
    rec.bytes = total_bytes;
  }
  return rec;
}

Records records_from_offsets(hd_ctx *ctx, const uint8_t *d_bytes, const uint64_t *h_offsets,
                             uint64_t n) {
  Records rec;
  rec.n = n;
  rec.base = d_bytes;
  std::vector<uint64_t> start(n ? n : 1), len(n ? n : 1);
  for (uint64_t k = 0; k < n; ++k) {
    start[k] = h_offsets[k] - h_offsets[0];
    len[k] = h_offsets[k + 1] - h_offsets[k];
    rec.max_len = len[k] > rec.max_len ? len[k] : rec.max_len;
    if (len[k] != len[0]) rec.all_equal = false;
  }
  rec.len0 = n ? len[0] : 0;
  rec.bytes = n ? h_offsets[n] - h_offsets[0] : 0;
  rec.rec_start = DevBuf(start.size() * 8, ctx->stream);
  rec.rec_len = DevBuf(len.size() * 8, ctx->stream);
  HD_CUDA(cudaMemcpyAsync(rec.rec_start.p, start.data(), start.size() * 8, cudaMemcpyHostToDevice,
                          ctx->stream));
  HD_CUDA(cudaMemcpyAsync(rec.rec_len.p, len.data(), len.size() * 8, cudaMemcpyHostToDevice,
                          ctx->stream));
  HD_CUDA(cudaStreamSynchronize(ctx->stream));  // host vectors go out of scope
  return rec;
}

// ---------------------------------------------------------------- dedupe
__device__ inline uint64_t mix64(uint64_t x) {
  x ^= x >> 30;
  x *= 0xbf58476d1ce4e5b9ull;
  x ^= x >> 27;
  x *= 0x94d049bb133111ebull;
  x ^= x >> 31;
  return x;
}

constexpr unsigned long long kEmpty = ~0ull;
constexpr int kHashU = 2;     // 512-byte blocks per warp per step of k_hash and k_tab_cmp

// 16 bytes at the 16-byte aligned address x, bytes outside the readable
// range [lo, hi) read as 0 (byte loads only at the ends of the range).
__device__ inline uint4 load16_in(uint64_t x, uint64_t lo, uint64_t hi) {
  if (x >= lo && x + 16 <= hi) return *reinterpret_cast<const uint4 *>(x);
  uint32_t w[4] = {0u, 0u, 0u, 0u};
  for (int k = 0; k < 16; ++k)
    if (x + k >= lo && x + k < hi)
      w[k >> 2] |= (uint32_t)*reinterpret_cast<const uint8_t *>(x + k) << (8 * (k & 3));
  return make_uint4(w[0], w[1], w[2], w[3]);
}
__device__ inline uint32_t load4_in(uint64_t x, uint64_t lo, uint64_t hi) {
  if (x >= lo && x + 4 <= hi) return *reinterpret_cast<const uint32_t *>(x);
  uint32_t w = 0;
  for (int k = 0; k < 4; ++k)
    if (x + k >= lo && x + k < hi) w |= (uint32_t)*reinterpret_cast<const uint8_t *>(x + k) << (8 * k);
  return w;
}

// Hash of each record's bytes: a sum over its 8-byte groups (at record
// positions 8q; a short last group is zero-filled) of the 64-bit product of
// the group's two 4-byte halves, each XORed with a position-keyed 32-bit
// constant, then one 64-bit mix of the sum and the length (k_hash_fin).
// Different records rarely share a hash, and equal hashes are verified byte
// by byte, so a collision costs a verify round, never a wrong answer. The sum
// does not depend on the order of its terms, so a record is hashed in
// segments of kHashSeg bytes, one warp each, that add their partial sums to
// acc[r] (zeroed first): many warps per record keep enough loads in flight
// however few records there are. Block (x, y) takes records 8x .. 8x + 7
// (one per warp) from byte y kHashSeg on. A lane reads 16 aligned bytes per
// step (two 512-byte blocks per warp and step) and the next lane's first 8;
// the two groups starting in its 16 bytes start at byte d0 mod 8 of them (d0
// = the segment's start mod 16) and are realigned with funnel shifts. Index
// arithmetic within a segment is 32-bit, so that a 16-byte step costs about
// 40 instructions.
constexpr uint64_t kHashSeg = 4096;
constexpr int kHashWarps = 8;
__global__ void __launch_bounds__(32 * kHashWarps)
    k_hash(const uint8_t *base, uint64_t bytes, const uint64_t *rs, const uint64_t *rl, uint64_t R,
           unsigned long long *acc) {
  const int lane = threadIdx.x & 31;
  const uint64_t r = (uint64_t)blockIdx.x * kHashWarps + (threadIdx.x >> 5);
  if (r >= R) return;  // warp-uniform
  const uint64_t lo = reinterpret_cast<uint64_t>(base), hi = lo + bytes;
  const uint64_t len = rl[r];
  for (uint64_t s_lo = (uint64_t)blockIdx.y * kHashSeg; s_lo < len;
       s_lo += (uint64_t)gridDim.y * kHashSeg) {
    const uint32_t seg = (uint32_t)(len - s_lo < kHashSeg ? len - s_lo : kHashSeg);
    const uint64_t P = lo + rs[r] + s_lo;  // the record's byte s_lo
    const uint64_t A = P & ~15ull;
    const uint32_t d0 = (uint32_t)(P - A), h8 = d0 & 7u, sh = 8u * (d0 & 3u);
    const bool hi_word = h8 >= 4u;  // the groups start in the lane's second word
    const uint32_t span = d0 + seg, q0 = (uint32_t)(s_lo >> 3);
    uint64_t h = 0;
    for (uint32_t b0 = 0; b0 < span; b0 += 512 * kHashU) {
      uint4 v[kHashU];
      uint2 nx[kHashU];
#pragma unroll
      for (int k = 0; k < kHashU; ++k) {
        const uint32_t off = b0 + 512 * k + 16 * lane;
        v[k] = off < span ? load16_in(A + off, lo, hi) : make_uint4(0u, 0u, 0u, 0u);
        const uint32_t noff = b0 + 512 * k + 512;  // lane 31: the 8 bytes after its 16
        nx[k] = (lane == 31 && noff < span)
                    ? make_uint2(load4_in(A + noff, lo, hi), load4_in(A + noff + 4, lo, hi))
                    : make_uint2(0u, 0u);
      }
#pragma unroll
      for (int k = 0; k < kHashU; ++k) {
        uint32_t n0 = __shfl_down_sync(0xffffffffu, v[k].x, 1);
        uint32_t n1 = __shfl_down_sync(0xffffffffu, v[k].y, 1);
        if (lane == 31) {
          n0 = nx[k].x;
          n1 = nx[k].y;
        }
        // words from the one the first group starts in
        const uint32_t wd[5] = {hi_word ? v[k].y : v[k].x, hi_word ? v[k].z : v[k].y,
                                hi_word ? v[k].w : v[k].z, hi_word ? n0 : v[k].w,
                                hi_word ? n1 : n0};
        const int32_t t0 = (int32_t)(b0 + 512 * k + 16 * lane + h8) - (int32_t)d0;
#pragma unroll
        for (int g = 0; g < 2; ++g) {
          const int32_t t = t0 + 8 * g;  // the group's position in the segment
          uint32_t x = __funnelshift_r(wd[2 * g], wd[2 * g + 1], sh);
          uint32_t y = __funnelshift_r(wd[2 * g + 1], wd[2 * g + 2], sh);
          const uint32_t rem = (uint32_t)((int32_t)seg - t);  // > 0 where valid
          if (rem < 8u) {  // the record's last group: bytes from rem on are 0
            y = rem > 4u ? y & ((1u << (8u * (rem - 4u))) - 1u) : 0u;
            if (rem < 4u) x &= (1u << (8u * rem)) - 1u;
          }
          const uint32_t q = q0 + ((uint32_t)t >> 3);
          x ^= q * 0x9e3779b9u + 0x7f4a7c15u;
          y ^= q * 0x85ebca6bu + 0x165667b1u;
          if ((uint32_t)t < seg) h += (uint64_t)x * y;
        }
      }
    }
    h = warp_sum(h);
    if (lane == 0 && h) atomicAdd(&acc[r], (unsigned long long)h);
  }
}
// The record hashes from the sums k_hash left in h[r], in place.
__global__ void k_hash_fin(const uint64_t *rl, uint64_t R, unsigned long long *h) {
  const uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (r >= R) return;
  const uint64_t v = mix64(h[r] ^ (rl[r] * 0xd6e8feb86659fd93ull));
  h[r] = v == kEmpty ? v - 1 : v;
}
// Hashes of records [0, R) of rs/rl into out (R > 0).
void hash_records(hd_ctx *ctx, const Records &rec, const uint64_t *rs, const uint64_t *rl,
                  uint64_t R, uint64_t *out) {
  cudaStream_t st = ctx->stream;
  HD_CUDA(cudaMemsetAsync(out, 0, R * 8, st));
  unsigned long long *h = reinterpret_cast<unsigned long long *>(out);
  if (rec.max_len) {
    const uint64_t X = ceil_div(R, (uint64_t)kHashWarps), S = ceil_div(rec.max_len, kHashSeg);
    if (X > 0x7fffffffull) fail(HD_ERR_ARG, "too many records");
    // segments past 65,535 are taken by the warps' loop
    k_hash<<<dim3((unsigned)X, (unsigned)std::min<uint64_t>(S, 65535)), 32 * kHashWarps, 0, st>>>(
        rec.base, rec.bytes, rs, rl, R, h);
    HD_LAUNCHED(ctx);
  }
  k_hash_fin<<<grid_for(R, 256), 256, 0, st>>>(rl, R, h);
  HD_LAUNCHED(ctx);
}

__device__ inline uint64_t slot_of(uint64_t h, uint64_t mask) { return (h ^ (h >> 29)) & mask; }

__global__ void k_tab_insert(const uint64_t *hash, const uint64_t *list, uint64_t cnt,
                             unsigned long long *keys, unsigned long long *mins, uint64_t mask) {
  uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i >= cnt) return;
  uint64_t r = list ? list[i] : i;
  unsigned long long h = hash[r];
  uint64_t slot = slot_of(h, mask);
  for (;;) {
    unsigned long long prev = atomicCAS(&keys[slot], kEmpty, h);
    if (prev == kEmpty || prev == h) {
      atomicMin(&mins[slot], (unsigned long long)r);
      return;
    }
    slot = (slot + 1) & mask;
  }
}

// Each record against the lowest-index record of equal hash: equal bytes ->
// duplicate; different bytes (a hash collision) -> next round.
// Whether the len bytes (len < 2^31) at Pa and at Pb, both inside [lo, hi),
// are equal; called by a whole warp, same result in every lane. a is read
// with aligned 16-byte loads; b's bytes at the same relative positions come
// from b's aligned loads and the next lane's, shifted by d = (Pb - Pa) mod 16:
// whole words by a warp-uniform switch, the rest by funnel shifts. Offsets
// inside the span are 32-bit, and only the windows at its two ends mask
// bytes.
__device__ inline bool warp_equal(uint64_t Pa, uint64_t Pb, uint32_t len, uint64_t lo, uint64_t hi,
                                  int lane) {
  const uint64_t Aa = Pa & ~15ull;
  const uint32_t da = (uint32_t)(Pa - Aa);  // a's first byte in its first window
  const uint64_t Bs = Pb - da;              // b's byte at a's window start (may precede b)
  const uint64_t Ab = Bs & ~15ull;
  const uint32_t d = (uint32_t)(Bs - Ab), dw = d >> 2, sh = 8u * (d & 3u);
  const uint32_t span = da + len;                    // a's windows cover [0, span) from Aa
  const uint32_t b_end = (uint32_t)(Pb + len - Ab);  // b's bytes end there, from Ab
  for (uint32_t b0 = 0; b0 < span; b0 += 512 * kHashU) {
    uint32_t diff = 0;
#pragma unroll
    for (int k = 0; k < kHashU; ++k) {
      const uint32_t off = b0 + 512 * k + 16 * lane;
      const bool in = off < span;
      const uint4 va = in ? load16_in(Aa + off, lo, hi) : make_uint4(0u, 0u, 0u, 0u);
      const uint4 vb = off < b_end ? load16_in(Ab + off, lo, hi) : make_uint4(0u, 0u, 0u, 0u);
      uint4 vn;
      vn.x = __shfl_down_sync(0xffffffffu, vb.x, 1);
      vn.y = __shfl_down_sync(0xffffffffu, vb.y, 1);
      vn.z = __shfl_down_sync(0xffffffffu, vb.z, 1);
      vn.w = __shfl_down_sync(0xffffffffu, vb.w, 1);
      if (lane == 31)
        vn = (d && off + 16 < b_end) ? load16_in(Ab + off + 16, lo, hi) : make_uint4(0u, 0u, 0u, 0u);
      // words dw .. dw + 4 of b's 32 bytes (vb, vn)
      uint32_t w0, w1, w2, w3, w4;
      switch (dw) {  // warp-uniform
        case 0: w0 = vb.x; w1 = vb.y; w2 = vb.z; w3 = vb.w; w4 = vn.x; break;
        case 1: w0 = vb.y; w1 = vb.z; w2 = vb.w; w3 = vn.x; w4 = vn.y; break;
        case 2: w0 = vb.z; w1 = vb.w; w2 = vn.x; w3 = vn.y; w4 = vn.z; break;
        default: w0 = vb.w; w1 = vn.x; w2 = vn.y; w3 = vn.z; w4 = vn.w; break;
      }
      uint32_t x[4] = {va.x ^ __funnelshift_r(w0, w1, sh), va.y ^ __funnelshift_r(w1, w2, sh),
                       va.z ^ __funnelshift_r(w2, w3, sh), va.w ^ __funnelshift_r(w3, w4, sh)};
      if (!(off >= da && off + 16 <= span)) {
        // a window at an end of the span: only the bytes at positions
        // [0, len) from a's first byte count
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int32_t p = (int32_t)(off + 4 * j) - (int32_t)da;  // the word's first byte
          uint32_t m = in ? 0xffffffffu : 0u;
          if (p < 0) m &= p <= -4 ? 0u : (0xffffffffu << (8 * (uint32_t)(-p)));
          if (p + 4 > (int32_t)len)
            m &= p >= (int32_t)len ? 0u : (0xffffffffu >> (8 * (uint32_t)(p + 4 - (int32_t)len)));
          x[j] &= m;
        }
      }
      diff |= x[0] | x[1] | x[2] | x[3];
    }
    if (__any_sync(0xffffffffu, diff != 0)) return false;
  }
  return true;
}

// The verify step spread over segments: warp (i, seg) compares bytes
// [seg * seg_bytes, +seg_bytes) of list record i with the lowest-index record
// of its hash (rep_out[i]) and marks differs[i] on a difference; k_tab_resolve
// then files each record as unique, a duplicate of rep, or (a hash collision)
// a record for the next round. Many warps per record keep the loads in
// flight when there are few duplicates.
__global__ void k_tab_cmp(const uint8_t *base, uint64_t bytes, const uint64_t *rs,
                          const uint64_t *rl, const uint64_t *hash, const uint64_t *list,
                          uint64_t cnt, const unsigned long long *keys,
                          const unsigned long long *mins, uint64_t mask, uint64_t seg_bytes,
                          uint64_t segs, uint64_t *rep_out, uint32_t *differs) {
  const int lane = threadIdx.x & 31;
  const uint64_t wid = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  if (wid >= cnt * segs) return;
  const uint64_t i = wid / segs, seg = wid % segs;
  const uint64_t r = list ? list[i] : i;
  uint64_t rep = 0;
  if (lane == 0) {
    const unsigned long long h = hash[r];
    uint64_t slot = slot_of(h, mask);
    while (keys[slot] != h) slot = (slot + 1) & mask;
    rep = mins[slot];
    if (seg == 0) rep_out[i] = rep;
  }
  rep = __shfl_sync(0xffffffffu, rep, 0);
  if (rep == r) return;
  const uint64_t len = rl[r];
  if (len != rl[rep]) {
    if (seg == 0 && lane == 0) differs[i] = 1u;
    return;
  }
  const uint64_t o = seg * seg_bytes;
  if (o >= len) return;
  const uint64_t sl = len - o < seg_bytes ? len - o : seg_bytes;
  const uint64_t lo = reinterpret_cast<uint64_t>(base);
  const bool eq = warp_equal(lo + rs[r] + o, lo + rs[rep] + o, (uint32_t)sl, lo, lo + bytes, lane);
  if (!eq && lane == 0) differs[i] = 1u;
}

__global__ void k_tab_resolve(const uint64_t *list, uint64_t cnt, const uint64_t *rep_out,
                              const uint32_t *differs, uint64_t *dup, uint64_t *next,
                              unsigned long long *next_cnt) {
  const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i >= cnt) return;
  const uint64_t r = list ? list[i] : i, rep = rep_out[i];
  if (rep == r) {
    dup[r] = r;
  } else if (!differs[i]) {
    dup[r] = rep;
  } else {
    next[atomicAdd(next_cnt, 1ull)] = r;
  }
}

__global__ void k_unique_flags(const uint64_t *dup, uint64_t R, uint32_t *flag) {
  uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (r < R) flag[r] = dup[r] == r ? 1u : 0u;
}

__global__ void k_number(const uint64_t *dup, const uint64_t *uidx, uint64_t R, uint64_t *seqidx,
                         uint64_t *unique_rec) {
  uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (r >= R) return;
  seqidx[r] = uidx[dup[r]];
  if (dup[r] == r) unique_rec[uidx[r]] = r;
}

namespace {
// One verify round over `cnt` list records (k_tab_cmp + k_tab_resolve).
void verify_round(hd_ctx *ctx, const Records &rec, const uint64_t *hash, const uint64_t *list,
                  uint64_t cnt, const unsigned long long *keys, const unsigned long long *mins,
                  uint64_t mask, uint64_t *dup, uint64_t *next, unsigned long long *next_cnt) {
  if (!cnt) return;
  cudaStream_t st = ctx->stream;
  constexpr uint64_t kSeg = 4096;  // bytes compared per warp
  const uint64_t segs = ceil_div(rec.max_len ? rec.max_len : 1, kSeg);
  DevBuf rep(cnt * 8, st), differs(cnt * 4, st);
  HD_CUDA(cudaMemsetAsync(differs.p, 0, cnt * 4, st));
  k_tab_cmp<<<grid_for(cnt * segs * 32, 256), 256, 0, st>>>(
      rec.base, rec.bytes, rec.rec_start.as<uint64_t>(), rec.rec_len.as<uint64_t>(), hash, list, cnt,
      keys, mins, mask, kSeg, segs, rep.as<uint64_t>(), differs.as<uint32_t>());
  HD_LAUNCHED(ctx);
  k_tab_resolve<<<grid_for(cnt, 256), 256, 0, st>>>(list, cnt, rep.as<uint64_t>(),
                                                   differs.as<uint32_t>(), dup, next, next_cnt);
  HD_LAUNCHED(ctx);
}
}  // namespace

DevBuf dedupe(hd_ctx *ctx, const Records &rec, uint64_t *n_unique, std::vector<uint64_t> &seqidx) {
  cudaStream_t st = ctx->stream;
  const uint64_t R = rec.n;
  seqidx.assign(R, 0);
  DevBuf unique_rec((R ? R : 1) * 8, st);
  if (R == 0) {
    *n_unique = 0;
    return unique_rec;
  }
  uint64_t T = 64;
  while (T < 2 * R) T <<= 1;
  DevBuf hash(R * 8, st), dup(R * 8, st), keys(T * 8, st), mins(T * 8, st);
  DevBuf lists[2] = {DevBuf(R * 8, st), DevBuf(R * 8, st)};
  DevBuf cnt(8, st);
  hash_records(ctx, rec, rec.rec_start.as<uint64_t>(), rec.rec_len.as<uint64_t>(), R,
               hash.as<uint64_t>());
  uint64_t todo = R;
  const uint64_t *list = nullptr;
  for (int round = 0; todo; ++round) {
    uint64_t *next = lists[round & 1].as<uint64_t>();
    HD_CUDA(cudaMemsetAsync(keys.p, 0xff, T * 8, st));
    HD_CUDA(cudaMemsetAsync(mins.p, 0xff, T * 8, st));
    HD_CUDA(cudaMemsetAsync(cnt.p, 0, 8, st));
    k_tab_insert<<<grid_for(todo, 256), 256, 0, st>>>(hash.as<uint64_t>(), list, todo,
                                                      keys.as<unsigned long long>(),
                                                      mins.as<unsigned long long>(), T - 1);
    HD_LAUNCHED(ctx);
    verify_round(ctx, rec, hash.as<uint64_t>(), list, todo, keys.as<unsigned long long>(),
                 mins.as<unsigned long long>(), T - 1, dup.as<uint64_t>(), next,
                 cnt.as<unsigned long long>());
    uint64_t left = 0;
    HD_CUDA(cudaMemcpyAsync(&left, cnt.p, 8, cudaMemcpyDeviceToHost, st));
    HD_CUDA(cudaStreamSynchronize(st));
    if (left >= todo) fail(HD_ERR_CUDA, "duplicate removal made no progress");
    todo = left;
    list = next;
  }
  DevBuf flag(R * 4, st), uidx(R * 8, st), tot(8, st), d_seqidx(R * 8, st);
  k_unique_flags<<<grid_for(R, 256), 256, 0, st>>>(dup.as<uint64_t>(), R, flag.as<uint32_t>());
  HD_LAUNCHED(ctx);
  scan_exclusive<uint32_t>(ctx, flag.as<uint32_t>(), uidx.as<uint64_t>(), R, tot.as<uint64_t>());
  k_number<<<grid_for(R, 256), 256, 0, st>>>(dup.as<uint64_t>(), uidx.as<uint64_t>(), R,
                                             d_seqidx.as<uint64_t>(), unique_rec.as<uint64_t>());
  HD_LAUNCHED(ctx);
  HD_CUDA(cudaMemcpyAsync(n_unique, tot.p, 8, cudaMemcpyDeviceToHost, st));
  HD_CUDA(cudaMemcpyAsync(seqidx.data(), d_seqidx.p, R * 8, cudaMemcpyDeviceToHost, st));
  HD_CUDA(cudaStreamSynchronize(st));
  return unique_rec;
}

// ------------------------------------------- incremental duplicate removal
__global__ void k_iota(uint64_t *out, uint64_t start, uint64_t n) {
  const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i < n) out[i] = start + i;
}
__global__ void k_inc_flags(const uint64_t *dup, uint64_t r0, uint64_t m, uint32_t *flag) {
  const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i < m) flag[i] = dup[r0 + i] == r0 + i ? 1u : 0u;
}
// new unique record r0 + i gets row k0 + uidx[i]
__global__ void k_inc_number(const uint64_t *dup, const uint64_t *uidx, uint64_t r0, uint64_t m,
                             uint64_t k0, uint64_t *rowid, uint64_t *unique_rec) {
  const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i >= m || dup[r0 + i] != r0 + i) return;
  rowid[r0 + i] = k0 + uidx[i];
  unique_rec[k0 + uidx[i]] = r0 + i;
}
// a new duplicate gets the row of its first occurrence (earlier, or new and
// numbered by k_inc_number)
__global__ void k_inc_link(const uint64_t *dup, uint64_t r0, uint64_t m, uint64_t *rowid) {
  const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i < m && dup[r0 + i] != r0 + i) rowid[r0 + i] = rowid[dup[r0 + i]];
}

void IncDedupe::init(hd_ctx *ctx, uint64_t capacity) {
  cudaStream_t st = ctx->stream;
  cap = capacity ? capacity : 1;
  T = 64;
  while (T < 2 * cap) T <<= 1;
  hash = DevBuf(cap * 8, st);
  dup = DevBuf(cap * 8, st);
  rowid = DevBuf(cap * 8, st);
  unique_rec = DevBuf(cap * 8, st);
  list = DevBuf(cap * 8, st);
  next = DevBuf(cap * 8, st);
  flag = DevBuf(cap * 4, st);
  uidx = DevBuf(cap * 8, st);
  keys = DevBuf(T * 8, st);
  mins = DevBuf(T * 8, st);
  cnt = DevBuf(16, st);
  HD_CUDA(cudaMemsetAsync(keys.p, 0xff, T * 8, st));
  HD_CUDA(cudaMemsetAsync(mins.p, 0xff, T * 8, st));
  seen = 0;
  n_unique = 0;
}

bool IncDedupe::add(hd_ctx *ctx, const Records &rec) {
  cudaStream_t st = ctx->stream;
  const uint64_t r0 = seen, m = rec.n - seen;
  if (rec.n < seen || rec.n > cap) return false;
  if (m == 0) return true;
  uint64_t *hp = hash.as<uint64_t>(), *lp = list.as<uint64_t>();
  hash_records(ctx, rec, rec.rec_start.as<uint64_t>() + r0, rec.rec_len.as<uint64_t>() + r0, m,
               hp + r0);
  k_iota<<<grid_for(m, 256), 256, 0, st>>>(lp, r0, m);
  HD_LAUNCHED(ctx);
  // earlier records hold the smaller indices: they stay each hash's minimum
  k_tab_insert<<<grid_for(m, 256), 256, 0, st>>>(hp, lp, m, keys.as<unsigned long long>(),
                                                 mins.as<unsigned long long>(), T - 1);
  HD_LAUNCHED(ctx);
  HD_CUDA(cudaMemsetAsync(cnt.p, 0, 16, st));
  verify_round(ctx, rec, hp, lp, m, keys.as<unsigned long long>(), mins.as<unsigned long long>(),
               T - 1, dup.as<uint64_t>(), next.as<uint64_t>(), cnt.as<unsigned long long>());
  k_inc_flags<<<grid_for(m, 256), 256, 0, st>>>(dup.as<uint64_t>(), r0, m, flag.as<uint32_t>());
  HD_LAUNCHED(ctx);
  scan_exclusive<uint32_t>(ctx, flag.as<uint32_t>(), uidx.as<uint64_t>(), m,
                           cnt.as<uint64_t>() + 1);
  uint64_t h[2] = {0, 0};  // unresolved records, new unique rows
  HD_CUDA(cudaMemcpyAsync(h, cnt.p, 16, cudaMemcpyDeviceToHost, st));
  HD_CUDA(cudaStreamSynchronize(st));
  // a new record unlike the first record of its hash: the full dedupe decides
  if (h[0]) return false;
  k_inc_number<<<grid_for(m, 256), 256, 0, st>>>(dup.as<uint64_t>(), uidx.as<uint64_t>(), r0, m,
                                                 n_unique, rowid.as<uint64_t>(),
                                                 unique_rec.as<uint64_t>());
  HD_LAUNCHED(ctx);
  k_inc_link<<<grid_for(m, 256), 256, 0, st>>>(dup.as<uint64_t>(), r0, m, rowid.as<uint64_t>());
  HD_LAUNCHED(ctx);
  n_unique += h[1];
  seen = rec.n;
  return true;
}

void IncDedupe::rows(hd_ctx *ctx, std::vector<uint64_t> &seqidx) {
  seqidx.resize(seen);
  if (!seen) return;
  HD_CUDA(cudaMemcpyAsync(seqidx.data(), rowid.p, seen * 8, cudaMemcpyDeviceToHost, ctx->stream));
  HD_CUDA(cudaStreamSynchronize(ctx->stream));
}

// -------------------------------------------------------------- consensus
constexpr int kColRows = 128;

__global__ void k_colcount(const uint8_t *base, const uint64_t *rs, const uint64_t *rows,
                           uint64_t n_rows, uint64_t L, unsigned int *counts) {
  uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (s >= L) return;
  uint64_t u0 = (uint64_t)blockIdx.y * kColRows;
  uint64_t u1 = u0 + kColRows < n_rows ? u0 + kColRows : n_rows;
  unsigned a = 0, c = 0, g = 0, t = 0;
  for (uint64_t u = u0; u < u1; ++u) {
    uint64_t r = rows ? rows[u] : u;
    uint8_t ch = base[rs[r] + s];
    a += ch == 'A';
    c += ch == 'C';
    g += ch == 'G';
    t += ch == 'T';
  }
  if (a) atomicAdd(&counts[4 * s + 0], a);
  if (c) atomicAdd(&counts[4 * s + 1], c);
  if (g) atomicAdd(&counts[4 * s + 2], g);
  if (t) atomicAdd(&counts[4 * s + 3], t);
}

__global__ void k_colmax_sum(const unsigned int *counts, uint64_t L, unsigned long long *sum) {
  __shared__ uint64_t tmp[33];
  uint64_t v = 0;
  for (uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s < L;
       s += (uint64_t)gridDim.x * blockDim.x) {
    unsigned m = max(max(counts[4 * s], counts[4 * s + 1]), max(counts[4 * s + 2], counts[4 * s + 3]));
    v += m;
  }
  uint64_t tot;
  block_excl_scan<uint64_t>(v, tmp, tot);
  if (threadIdx.x == 0) atomicAdd(sum, (unsigned long long)tot);
}

uint64_t consensus_matches(hd_ctx *ctx, const Records &rec, const uint64_t *d_rows,
                           uint64_t n_rows) {
  cudaStream_t st = ctx->stream;
  const uint64_t L = rec.len0;
  if (!L || !n_rows) return 0;
  DevBuf counts(L * 16, st), sum(8, st);
  HD_CUDA(cudaMemsetAsync(counts.p, 0, L * 16, st));
  HD_CUDA(cudaMemsetAsync(sum.p, 0, 8, st));
  uint64_t chunks = ceil_div(n_rows, kColRows);
  for (uint64_t c0 = 0; c0 < chunks; c0 += 65535) {
    uint64_t cn = chunks - c0 < 65535 ? chunks - c0 : 65535;
    dim3 grid((unsigned)ceil_div(L, 256), (unsigned)cn);
    const uint64_t *rows = d_rows ? d_rows + c0 * kColRows : nullptr;
    // without a row list the rows are records [c0*kColRows, ...): shift the starts
    const uint64_t *rs = rec.rec_start.as<uint64_t>() + (d_rows ? 0 : c0 * kColRows);
    k_colcount<<<grid, 256, 0, st>>>(rec.base, rs, rows, n_rows - c0 * kColRows, L,
                                     counts.as<unsigned int>());
    HD_LAUNCHED(ctx);
  }
  k_colmax_sum<<<(unsigned)(ctx->sm_count * 4), 256, 0, st>>>(counts.as<unsigned int>(), L,
                                                             sum.as<unsigned long long>());
  HD_LAUNCHED(ctx);
  uint64_t h = 0;
  HD_CUDA(cudaMemcpyAsync(&h, sum.p, 8, cudaMemcpyDeviceToHost, st));
  HD_CUDA(cudaStreamSynchronize(st));
  return h;
}

// ------------------------------------------------------------------- pack
// Packing: a warp job is kPackCPG chunks of 32 words (1024 sites each) of
// one row. Per chunk the warp reads the 1024 bytes with coalesced byte loads
// (all issued before use), stages their codes in shared memory, and lane i
// then builds word i from its 32 consecutive codes: for plane p, the p bits
// of 4 codes (one per byte) are gathered into 4 bits by one multiply
// ((v & 0x01010101) * 0x01020408 moves bit 8j to bit 24 + j). Sites past L
// get the '-' code, which matches everything, so padding never counts (the
// reference pads with '-' too, src/hamming_impl.cc:256-264).
constexpr int kPackThreads = 256;
constexpr int kPackCPG = 4;
template <int P>
__global__ void __launch_bounds__(kPackThreads)
    k_pack(const uint8_t *base, const uint64_t *rs, const uint64_t *rows, uint64_t n_rows,
           uint64_t L, uint64_t words, Table256 table, uint4 *g0, uint4 *g1) {
  __shared__ uint8_t tbl[256];
  __shared__ __align__(16) uint8_t stage[kPackThreads / 32][1024 + 16];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) tbl[i] = table.v[i];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  uint8_t *sw = stage[threadIdx.x >> 5];
  const uint64_t chunks = (words + 31) / 32;
  const uint64_t groups = (chunks + kPackCPG - 1) / kPackCPG;
  uint64_t wid = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  uint64_t nwarps = (gridDim.x * (uint64_t)blockDim.x) >> 5;
  for (uint64_t job = wid; job < n_rows * groups; job += nwarps) {
    const uint64_t u = job / groups;
    const uint64_t q0 = (job - u * groups) * kPackCPG;
    const uint64_t r = rows ? rows[u] : u;
    const uint8_t *src = base + rs[r];
    for (uint64_t q = q0; q < q0 + kPackCPG && q < chunks; ++q) {
      const uint8_t *cs = src + q * 1024;
      const int64_t rem64 = (int64_t)L - (int64_t)(q * 1024);
      const int rem = rem64 <= 0 ? 0 : (rem64 >= 1024 ? 1024 : (int)rem64);
      uint8_t ch[32];
#pragma unroll
      for (int i = 0; i < 32; ++i) {
        const int s = i * 32 + lane;
        ch[i] = s < rem ? cs[s] : (uint8_t)'-';
      }
#pragma unroll
      for (int i = 0; i < 32; ++i) sw[i * 32 + lane] = tbl[ch[i]];
      __syncwarp();
      const uint4 c0 = *reinterpret_cast<const uint4 *>(sw + lane * 32);
      const uint4 c1 = *reinterpret_cast<const uint4 *>(sw + lane * 32 + 16);
      __syncwarp();  // the next chunk overwrites the staging
      const uint32_t cw[8] = {c0.x, c0.y, c0.z, c0.w, c1.x, c1.y, c1.z, c1.w};
      uint32_t x[6] = {0u, 0u, 0u, 0u, 0u, 0u};
#pragma unroll
      for (int p = 0; p < P; ++p) {
        uint32_t acc = 0;
#pragma unroll
        for (int k = 0; k < 8; ++k)
          acc |= ((((cw[k] >> p) & 0x01010101u) * 0x01020408u) >> 24 & 0xFu) << (4 * k);
        x[p] = acc;
      }
      const uint64_t w = q * 32 + lane;
      if (w < words) {
        g0[u * words + w] = make_uint4(x[0], x[1], x[2], x[3]);
        if (P > 4) g1[u * words + w] = make_uint4(x[4], x[5], 0u, 0u);
      }
    }
  }
}

// AND-rule packer: a warp job is one 1024-site chunk of one row, and lane l
// builds its 32-site word l from the chunk's bytes [32 l, 32 l + 32), read as
// aligned 16-byte vectors (two of its own and the next lane's first;
// realigned by the row's offset mod 16 with funnel shifts). A 256-entry table
// in shared memory gives each byte its code (A, C, G, T one-hot, '-' 1111,
// every other byte 0, as in src/hamming_impl.cc:23-44) with plane p's bit at
// bit 8 p. Summed with weights 1, 2, 4, 8 over 4 sites, and 16 for the next 4,
// byte p of the sum holds plane p's bits of 8 sites; four such sums give each
// plane word by byte permutes. Sites past L get the '-' code.
__global__ void __launch_bounds__(256)
    k_pack_and(const uint8_t *base, uint64_t bytes, const uint64_t *rs, const uint64_t *rows,
               uint64_t n_rows, uint64_t L, uint64_t words, uint4 *g0, uint4 *g1) {
  __shared__ uint32_t spread[256];
  {
    const uint32_t b = threadIdx.x;  // the block has 256 threads
    const uint32_t c = b == 'A' ? 1u : b == 'C' ? 2u : b == 'G' ? 4u : b == 'T' ? 8u : b == '-' ? 15u : 0u;
    spread[b] = (c & 1u) | ((c & 2u) << 7) | ((c & 4u) << 14) | ((c & 8u) << 21);
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const uint64_t lo = reinterpret_cast<uint64_t>(base), hi = lo + bytes;
  const uint64_t chunks = (words + 31) / 32;
  const uint64_t wid = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nwarps = (gridDim.x * (uint64_t)blockDim.x) >> 5;
  for (uint64_t job = wid; job < n_rows * chunks; job += nwarps) {
    const uint64_t u = job / chunks, q = job - u * chunks;
    const uint64_t r = rows ? rows[u] : u;
    const uint64_t P0 = lo + rs[r] + q * 1024;  // the chunk's first byte
    const uint64_t A = P0 & ~15ull;
    const uint32_t d = (uint32_t)(P0 - A), dw = d >> 2, db = d & 3u;
    const int64_t rem64 = (int64_t)L - (int64_t)(q * 1024);
    const uint32_t rem = rem64 <= 0 ? 0u : (rem64 >= 1024 ? 1024u : (uint32_t)rem64);
    const uint64_t la = A + 32ull * lane;
    uint32_t w[12];
    {
      const uint4 v0 = rem ? load16_in(la, lo, hi) : make_uint4(0u, 0u, 0u, 0u);
      const uint4 v1 = rem ? load16_in(la + 16, lo, hi) : make_uint4(0u, 0u, 0u, 0u);
      uint4 v2;
      v2.x = __shfl_down_sync(0xffffffffu, v0.x, 1);
      v2.y = __shfl_down_sync(0xffffffffu, v0.y, 1);
      v2.z = __shfl_down_sync(0xffffffffu, v0.z, 1);
      v2.w = __shfl_down_sync(0xffffffffu, v0.w, 1);
      if (lane == 31) v2 = (rem && d) ? load16_in(la + 32, lo, hi) : make_uint4(0u, 0u, 0u, 0u);
      w[0] = v0.x; w[1] = v0.y; w[2] = v0.z; w[3] = v0.w;
      w[4] = v1.x; w[5] = v1.y; w[6] = v1.z; w[7] = v1.w;
      w[8] = v2.x; w[9] = v2.y; w[10] = v2.z; w[11] = v2.w;
    }
    // the 36 bytes from byte 4 dw (dw is the same in the whole warp)
    uint32_t x[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) x[k] = w[k];
    if (dw == 1) {
#pragma unroll
      for (int k = 0; k < 9; ++k) x[k] = w[k + 1];
    } else if (dw == 2) {
#pragma unroll
      for (int k = 0; k < 9; ++k) x[k] = w[k + 2];
    } else if (dw == 3) {
#pragma unroll
      for (int k = 0; k < 9; ++k) x[k] = w[k + 3];
    }
    const uint32_t s0 = 32u * lane;  // chunk-relative site of this lane's first byte
    uint32_t pair[4];  // byte p: plane p's bits of sites 8 m .. 8 m + 7
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      uint32_t e2 = 0;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int k = 2 * m + h;
        uint32_t y = __funnelshift_r(x[k], x[k + 1], 8 * db);
        const uint32_t sk = s0 + 4 * k;
        if (sk + 4 > rem) {  // past the row's end: '-'
          const uint32_t keep = sk >= rem ? 0u : (0xFFFFFFFFu >> (8 * (sk + 4 - rem)));
          y = (y & keep) | (0x2D2D2D2Du & ~keep);
        }
        const uint32_t e = spread[y & 0xFFu] + 2u * spread[(y >> 8) & 0xFFu] +
                           4u * spread[(y >> 16) & 0xFFu] + 8u * spread[y >> 24];
        e2 += e << (4 * h);
      }
      pair[m] = e2;
    }
    uint32_t pl[4];
#pragma unroll
    for (int p = 0; p < 4; ++p) {
      const uint32_t lo2 = __byte_perm(pair[0], pair[1], (uint32_t)p | ((uint32_t)(4 + p) << 4));
      const uint32_t hi2 = __byte_perm(pair[2], pair[3], (uint32_t)p | ((uint32_t)(4 + p) << 4));
      pl[p] = __byte_perm(lo2, hi2, 0x5410u);
    }
    const uint64_t wi = q * 32 + lane;
    if (wi < words) {
      const uint4 v = make_uint4(pl[0], pl[1], pl[2], pl[3]);
      g0[u * words + wi] = v;
      if (g1) g1[u * words + wi] = v;
    }
  }
}

void pack_rows_and(hd_ctx *ctx, const Records &rec, const uint64_t *d_rows, uint64_t n_rows,
                   uint64_t length, uint64_t words, uint4 *g0, uint4 *g1) {
  if (!n_rows) return;
  const uint64_t jobs = n_rows * ((words + 31) / 32);
  k_pack_and<<<grid_for(jobs * 32, 256), 256, 0, ctx->stream>>>(
      rec.base, rec.bytes, rec.rec_start.as<uint64_t>(), d_rows, n_rows, length, words, g0, g1);
  HD_LAUNCHED(ctx);
}

__global__ void k_concat_starts(const uint64_t *a, uint64_t na, const uint64_t *b, uint64_t nb,
                                uint64_t b_off, uint64_t *out) {
  const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i < na) out[i] = a[i];
  else if (i < na + nb) out[i] = b[i - na] + b_off;
}

Records concat_records(hd_ctx *ctx, const Records &a, const Records &b, uint64_t b_off,
                       uint64_t bytes) {
  cudaStream_t st = ctx->stream;
  Records r;
  r.n = a.n + b.n;
  r.len0 = a.n ? a.len0 : b.len0;
  r.max_len = a.max_len > b.max_len ? a.max_len : b.max_len;
  r.all_equal = a.all_equal && b.all_equal && (!a.n || !b.n || a.len0 == b.len0);
  r.base = a.base;
  r.bytes = bytes;
  r.rec_start = DevBuf((r.n ? r.n : 1) * 8, st);
  r.rec_len = DevBuf((r.n ? r.n : 1) * 8, st);
  if (r.n) {
    k_concat_starts<<<grid_for(r.n, 256), 256, 0, st>>>(a.rec_start.as<uint64_t>(), a.n,
                                                        b.rec_start.as<uint64_t>(), b.n, b_off,
                                                        r.rec_start.as<uint64_t>());
    HD_LAUNCHED(ctx);
    if (a.n)
      HD_CUDA(cudaMemcpyAsync(r.rec_len.p, a.rec_len.p, a.n * 8, cudaMemcpyDeviceToDevice, st));
    if (b.n)
      HD_CUDA(cudaMemcpyAsync(r.rec_len.as<uint64_t>() + a.n, b.rec_len.p, b.n * 8,
                              cudaMemcpyDeviceToDevice, st));
  }
  return r;
}

void pack_rows(hd_ctx *ctx, const Records &rec, const uint64_t *d_rows, hd_alignment *aln) {
  Table256 t;
  int table = aln->rule == HD_RULE_AND ? kCodesAnd
              : aln->rule == HD_RULE_SPARSE ? kCodesSparse : kCodesSparseX;
  code_table(table, t.v);
  const uint64_t bytes = aln->n_rows * aln->words * 16;
  aln->plane_buf[0] = DevBuf(bytes ? bytes : 16, ctx->stream);
  if (aln->groups > 1) aln->plane_buf[1] = DevBuf(bytes ? bytes : 16, ctx->stream);
  if (!aln->n_rows) return;
  const uint64_t jobs = aln->n_rows * hd::ceil_div((aln->words + 31) / 32, (uint64_t)kPackCPG);
  unsigned grid = grid_for(jobs * 32, kPackThreads);
  uint4 *g0 = aln->plane_buf[0].as<uint4>(), *g1 = aln->plane_buf[1].as<uint4>();
  const uint64_t *rs = rec.rec_start.as<uint64_t>();
  if (aln->planes == 4)
    k_pack_and<<<grid_for(aln->n_rows * ((aln->words + 31) / 32) * 32, 256), 256, 0, ctx->stream>>>(
        rec.base, rec.bytes, rs, d_rows, aln->n_rows, aln->length, aln->words, g0, nullptr);
  else if (aln->planes == 5)
    k_pack<5><<<grid, kPackThreads, 0, ctx->stream>>>(rec.base, rs, d_rows, aln->n_rows, aln->length,
                                             aln->words, t, g0, g1);
  else
    k_pack<6><<<grid, kPackThreads, 0, ctx->stream>>>(rec.base, rs, d_rows, aln->n_rows, aln->length,
                                             aln->words, t, g0, g1);
  HD_LAUNCHED(ctx);
}

// ----------------------------------------------------- reference distances
// Rule of src/hamming.cc:128-136: a site counts when the reference codes of
// the two bytes share no bit, or when the bytes differ and neither is '-'.
// 4-bit site codes of four bytes, as the reference's distance lookup
// classifies them: A 1, C 2, G 4, T 8, '-' 15, X 3 (with include_x), any
// other byte 0. The six symbols differ in their low three bits (X 0, A 1,
// C 3, T 4, '-' 5, G 7), which pick each byte's code from code_lo:code_hi
// and the symbol it must equal from a second table (both with __byte_perm).
constexpr uint32_t kSymLo = 0x43004158u, kSymHi = 0x47002D54u;  // X A . C / T - . G
__device__ __forceinline__ uint32_t site_codes(uint32_t w, uint32_t code_lo, uint32_t code_hi) {
  const uint32_t sel =
      (w & 0x7u) | ((w >> 4) & 0x70u) | ((w >> 8) & 0x700u) | ((w >> 12) & 0x7000u);
  const uint32_t z = w ^ __byte_perm(kSymLo, kSymHi, sel);
  const uint32_t eq = ~(((z & 0x7F7F7F7Fu) + 0x7F7F7F7Fu) | z) & 0x80808080u;  // 0x80: equal
  return __byte_perm(code_lo, code_hi, sel) & ((eq >> 7) * 0xFFu);
}
// Sites of four bytes that count, among those flagged (0x80) in `valid`: a
// pair counts if its codes share no bit, or if the bytes differ and neither
// is '-' (src/hamming.cc:104-141 through the distance lookup).
__device__ __forceinline__ uint32_t count_sites(uint32_t a, uint32_t ca, uint32_t b, uint32_t cb,
                                               uint32_t valid) {
  const uint32_t share = ((ca & cb) + 0x7F7F7F7Fu) & 0x80808080u;  // codes <= 15: no carry
  const uint32_t z = a ^ b;
  const uint32_t differ = (((z & 0x7F7F7F7Fu) + 0x7F7F7F7Fu) | z) & 0x80808080u;
  const uint32_t dash = (((ca >> 2) & (ca >> 3)) | ((cb >> 2) & (cb >> 3))) & 0x01010101u;
  return __popc((~share | (differ & ~(dash << 7))) & valid & 0x80808080u);
}

// Block (x, y) compares records 8x .. 8x + 7 (one per warp) over sites
// [y kRefSeg, (y + 1) kRefSeg) and adds each count to out[r], which starts at
// 0, so that short and long records spread evenly over the SMs. The block
// first copies that stretch of the reference, and its site codes, to shared
// memory. Lane l takes 16 consecutive sites per step: the reference's from
// shared memory, the record's from aligned 16-byte loads of its own and the
// next lane's, realigned with funnel shifts, and classifies and compares
// them four at a time, two steps per iteration with both steps' loads
// issued first. 20,000 records of 29,903 sites take 0.39 ms (one step per
// iteration: 0.41 ms; two shared-memory lookups per site: 0.53 ms).
constexpr uint64_t kRefSeg = 4096;
constexpr int kRefWarps = 8;
__global__ void __launch_bounds__(32 * kRefWarps)
    k_refdist(const uint8_t *base, uint64_t bytes, const uint64_t *rs, const uint64_t *rl,
              uint64_t R, uint64_t max_len, const uint8_t *ref, uint32_t code_lo,
              uint32_t code_hi, uint32_t *out) {
  __shared__ uint4 rsm[kRefSeg / 16], csm[kRefSeg / 16];
  const int lane = threadIdx.x & 31;
  const uint64_t r = (uint64_t)blockIdx.x * kRefWarps + (threadIdx.x >> 5);
  const uint64_t len = r < R ? rl[r] : 0;
  const uint64_t lo = reinterpret_cast<uint64_t>(base), hi = lo + bytes;
  const uint64_t S = (max_len + kRefSeg - 1) / kRefSeg;
  for (uint64_t y = blockIdx.y; y < S; y += gridDim.y) {  // block-uniform
    const uint64_t s_lo = y * kRefSeg;                     // < max_len
    // the reference is 16-byte aligned with 16 readable bytes past max_len
    const uint64_t avail = max_len - s_lo < kRefSeg ? max_len - s_lo : kRefSeg;
    const uint4 *rg = reinterpret_cast<const uint4 *>(ref + s_lo);
    __syncthreads();  // no warp still reads the previous stretch
    for (uint64_t i = threadIdx.x; i < (avail + 15) / 16; i += blockDim.x) {
      const uint4 v = rg[i];
      rsm[i] = v;
      csm[i] = make_uint4(site_codes(v.x, code_lo, code_hi), site_codes(v.y, code_lo, code_hi),
                          site_codes(v.z, code_lo, code_hi), site_codes(v.w, code_lo, code_hi));
    }
    __syncthreads();
    if (s_lo >= len) continue;  // warp-uniform (also r >= R)
    const uint64_t seg = len - s_lo < kRefSeg ? len - s_lo : kRefSeg;
    const uint64_t P = lo + rs[r] + s_lo;  // the record's site s_lo
    const uint64_t A = P & ~15ull, end = P + seg;
    const uint32_t d = (uint32_t)(P - A), dw = d >> 2, db = d & 3;
    uint32_t cnt = 0;
    // two 512-site steps per iteration: both steps' loads are issued first
    for (uint64_t o0 = 0; o0 < seg; o0 += 1024) {  // warp-uniform
      uint4 va[2], vx[2];
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const uint64_t o = o0 + 512 * u + 16 * (uint64_t)lane;
        va[u] = A + o < end ? load16_in(A + o, lo, hi) : make_uint4(0u, 0u, 0u, 0u);
        // lane 31: the 16 bytes after its own, which no lane holds
        vx[u] = (lane == 31 && d && A + o + 16 < end) ? load16_in(A + o + 16, lo, hi)
                                                      : make_uint4(0u, 0u, 0u, 0u);
      }
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const uint64_t o = o0 + 512 * u + 16 * (uint64_t)lane;
        uint4 vn;
        vn.x = __shfl_down_sync(0xffffffffu, va[u].x, 1);
        vn.y = __shfl_down_sync(0xffffffffu, va[u].y, 1);
        vn.z = __shfl_down_sync(0xffffffffu, va[u].z, 1);
        vn.w = __shfl_down_sync(0xffffffffu, va[u].w, 1);
        if (lane == 31) vn = vx[u];
        if (o >= seg) continue;
        const uint4 vr = rsm[o >> 4], vc = csm[o >> 4];
        const uint32_t bw[8] = {va[u].x, va[u].y, va[u].z, va[u].w, vn.x, vn.y, vn.z, vn.w};
        const uint32_t rw[4] = {vr.x, vr.y, vr.z, vr.w}, cw[4] = {vc.x, vc.y, vc.z, vc.w};
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          uint32_t blo = bw[j], bhi = bw[j + 1];
#pragma unroll
          for (int t = 1; t < 4; ++t)
            if (dw == (uint32_t)t) {
              blo = bw[j + t];
              bhi = bw[j + t + 1];
            }
          const uint32_t aw = __funnelshift_r(blo, bhi, 8 * db);  // record sites o + 4j ..
          const uint64_t rem = seg - o;                           // >= 1
          const uint32_t valid = rem >= (uint64_t)(4 * j + 4) ? 0x80808080u
                                 : rem <= (uint64_t)(4 * j) ? 0u
                                   : 0x80808080u & ((1u << (8 * (uint32_t)(rem - 4 * j))) - 1u);
          cnt += count_sites(aw, site_codes(aw, code_lo, code_hi), rw[j], cw[j], valid);
        }
      }
    }
    cnt = warp_sum(cnt);
    if (lane == 0 && cnt) atomicAdd(&out[r], cnt);
  }
}

void reference_distances_device(hd_ctx *ctx, const Records &rec, const uint8_t *d_ref,
                                int include_x, uint32_t *d_out) {
  if (!rec.n) return;
  // codes by the low three bits of the symbol: X, A, -, C / T, -, -, G
  const uint32_t code_lo = (include_x ? 3u : 0u) | (1u << 8) | (2u << 24);
  const uint32_t code_hi = 8u | (15u << 8) | (4u << 24);
  HD_CUDA(cudaMemsetAsync(d_out, 0, rec.n * sizeof(uint32_t), ctx->stream));
  if (!rec.max_len) return;
  const uint64_t S = ceil_div(rec.max_len, kRefSeg), X = ceil_div(rec.n, (uint64_t)kRefWarps);
  if (X > 0x7fffffffull) fail(HD_ERR_ARG, "too many records");
  // stretches past 65,535 are taken by the blocks' loop
  k_refdist<<<dim3((unsigned)X, (unsigned)std::min<uint64_t>(S, 65535)), 32 * kRefWarps, 0,
              ctx->stream>>>(rec.base, rec.bytes, rec.rec_start.as<uint64_t>(),
                             rec.rec_len.as<uint64_t>(), rec.n, rec.max_len, d_ref, code_lo,
                             code_hi, d_out);
  HD_LAUNCHED(ctx);
}

// Query row (packed with the alignment's AND codes) against every row.
__global__ void k_query(const uint4 *g0, uint64_t words, uint64_t n_rows, const uint4 *q,
                        uint32_t *out) {
  const int lane = threadIdx.x & 31;
  uint64_t wid = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  uint64_t nwarps = (gridDim.x * (uint64_t)blockDim.x) >> 5;
  for (uint64_t u = wid; u < n_rows; u += nwarps) {
    const uint4 *row = g0 + u * words;
    uint32_t cnt = 0;
    for (uint64_t w = lane; w < words; w += 32) {
      uint4 a = row[w], b = q[w];
      cnt += __popc(~((a.x & b.x) | (a.y & b.y) | (a.z & b.z) | (a.w & b.w)));
    }
    cnt = warp_sum(cnt);
    if (lane == 0) out[u] = cnt;
  }
}

void query_distances_async(hd_ctx *ctx, const hd_alignment *aln, const uint8_t *d_query,
                           uint32_t *d_out_rows, DevBuf &q_planes) {
  // pack the query with the alignment's AND codes (one row), then one warp per row
  Table256 t;
  code_table(kCodesAnd, t.v);
  q_planes = DevBuf(aln->words * 16, ctx->stream);
  DevBuf rs(8, ctx->stream);  // record start 0, freed after the kernels in stream order
  HD_CUDA(cudaMemsetAsync(rs.p, 0, 8, ctx->stream));
  k_pack<4><<<grid_for(hd::ceil_div((aln->words + 31) / 32, (uint64_t)kPackCPG) * 32, kPackThreads),
              kPackThreads, 0, ctx->stream>>>(
      d_query, rs.as<uint64_t>(), nullptr, 1, aln->length, aln->words, t, q_planes.as<uint4>(),
      nullptr);
  HD_LAUNCHED(ctx);
  k_query<<<grid_for(aln->n_rows * 32, 256), 256, 0, ctx->stream>>>(
      static_cast<const uint4 *>(aln->planes_ptr(0)), aln->words, aln->n_rows,
      q_planes.as<uint4>(), d_out_rows);
  HD_LAUNCHED(ctx);
}

// out[r] = the distance of record r's row
__global__ void k_gather_rows(const uint32_t *row_dist, const uint64_t *row_of, uint64_t n,
                              uint32_t *out) {
  const uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (r < n) out[r] = row_dist[row_of ? row_of[r] : r];
}

void query_rows_to_records(hd_ctx *ctx, const hd_alignment *aln, const uint8_t *d_query,
                           uint32_t *d_rows, const uint64_t *row_of, uint64_t n, uint32_t *d_out) {
  DevBuf q;  // freed after the kernels in stream order
  query_distances_async(ctx, aln, d_query, d_rows, q);
  k_gather_rows<<<grid_for(n, 256), 256, 0, ctx->stream>>>(d_rows, row_of, n, d_out);
  HD_LAUNCHED(ctx);
}

void alignment_query_distances(hd_ctx *ctx, const hd_alignment *aln, const uint8_t *d_query,
                               uint32_t *d_out_rows) {
  DevBuf q;
  query_distances_async(ctx, aln, d_query, d_out_rows, q);
  HD_CUDA(cudaStreamSynchronize(ctx->stream));
}

}  // namespace hd
