// Autotuner for the pairwise engine: picks the tile edge (64 or 128 rows,
// i.e. 4 or 8 rows per thread) and the TMA staging depth per
// (n bucket, L bucket, output dtype). Each candidate is timed with the GPU
// filled: a batch of copies of a synthetic packed alignment of the bucket's
// representative size, so the figure is throughput per pair-site as the
// batched and served paths see it. The table can be saved to and loaded from
// a small JSON file; HAMMINGDIST_TILE=<tile>x<stages> overrides it.
// No reference counterpart (the reference has one kernel shape).
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <sstream>

#include "hd_internal.cuh"

namespace hd {

namespace {

const uint64_t kNEdges[] = {96, 192, 384, 768, 1536, 4096};  // n buckets 0..6
const uint64_t kNRep[] = {64, 160, 320, 640, 1280, 3072, 8192};
const uint64_t kLEdges[] = {2048, 8192, 16384};               // L buckets 0..3
const uint64_t kLRep[] = {1000, 5000, 12000, 29903};

int n_bucket(uint64_t n) {
  int b = 0;
  while (b < 6 && n > kNEdges[b]) ++b;
  return b;
}
int l_bucket(uint64_t L) {
  int b = 0;
  while (b < 3 && L > kLEdges[b]) ++b;
  return b;
}
uint32_t key_of(int nb, int lb, int dtype) { return (uint32_t)(nb * 100 + lb * 10 + dtype); }

bool env_override(TileConfig &c) {
  const char *e = std::getenv("HAMMINGDIST_TILE");
  int t = 0, s = 0;
  if (!e || std::sscanf(e, "%dx%d", &t, &s) != 2 || !tile_config_valid(t, s)) return false;
  c.tile = t;
  c.stages = s;
  return true;
}

__global__ void k_random_planes(uint4 *p, uint64_t n_words, uint64_t seed) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n_words;
       i += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t x = (i + 1) * 0x9e3779b97f4a7c15ull ^ seed;
    x ^= x >> 31;
    x *= 0xbf58476d1ce4e5b9ull;
    x ^= x >> 29;
    const uint32_t lo = (uint32_t)x, hi = (uint32_t)(x >> 32);
    // one-hot-like planes: every bit set in exactly one plane
    const uint32_t s0 = lo & hi, s1 = lo & ~hi, s2 = ~lo & hi, s3 = ~(lo | hi);
    p[i] = make_uint4(s0, s1, s2, s3);
  }
}

double time_config(hd_ctx *ctx, const hd_alignment &a, int copies, int dtype, TileConfig tc,
                   DevBuf &out) {
  std::vector<PairJobSpec> specs(copies);
  const uint64_t pairs = a.n_rows * (a.n_rows - 1) / 2;
  const uint32_t nb = (uint32_t)ceil_div(a.n_rows, tc.tile);
  for (int k = 0; k < copies; ++k) {
    PairJobSpec &s = specs[k];
    s.aln = &a;
    s.dtype = dtype;
    s.max_dist = 0xffffffffu;
    s.d_out = out.as<uint8_t>() + (uint64_t)k * pairs * dtype;
    s.tile_lo = 0;
    s.tile_hi = nb;
    s.cfg = tc;
  }
  cudaEvent_t e0, e1;
  HD_CUDA(cudaEventCreate(&e0));
  HD_CUDA(cudaEventCreate(&e1));
  double best = 1e30;
  for (int rep = 0; rep < 3; ++rep) {
    std::vector<PairJobSpec> sp = specs;
    HD_CUDA(cudaEventRecord(e0, ctx->stream));
    run_pairwise_jobs(ctx, sp, ctx->stream, nullptr);
    HD_CUDA(cudaEventRecord(e1, ctx->stream));
    HD_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    HD_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    if (rep > 0 && ms < best) best = ms;  // first run warms up
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return best;
}

}  // namespace

TileConfig tile_config_for(hd_ctx *ctx, uint64_t n_rows, uint64_t length, int dtype_bytes) {
  TileConfig c;
  if (env_override(c)) return c;
  const uint32_t key = key_of(n_bucket(n_rows), l_bucket(length), dtype_bytes == 1 ? 1 : 2);
  for (const auto &e : ctx->tune)
    if (e.first == key) return {e.second.first, e.second.second};
  return default_tile_config(n_rows, length, dtype_bytes);
}

}  // namespace hd

using hd::DevBuf;

namespace {
template <class F>
int tune_guard(hd_ctx *ctx, F &&f) {
  try {
    HD_CUDA(cudaSetDevice(ctx->device));
    f();
    return HD_OK;
  } catch (const hd::Error &e) {
    ctx->err = e.msg;
    return e.code;
  } catch (const std::exception &e) {
    ctx->err = e.what();
    return HD_ERR_CUDA;
  }
}
}  // namespace

extern "C" int hd_autotune(hd_ctx *ctx, uint64_t max_n_bucket) {
  if (!ctx) return HD_ERR_ARG;
  return tune_guard(ctx, [&] {
    const hd::TileConfig cands[] = {{128, 3}, {128, 2}, {128, 4}, {64, 3}, {64, 4}};
    const int nbmax = (int)std::min<uint64_t>(max_n_bucket, 6);
    ctx->tune.clear();
    for (int nb = 0; nb <= nbmax; ++nb) {
      for (int lb = 0; lb < 4; ++lb) {
        hd_alignment a;
        a.ctx = ctx;
        a.device = ctx->device;
        a.n_rows = hd::kNRep[nb];
        a.length = hd::kLRep[lb];
        a.words = hd::round_up(hd::ceil_div(a.length, 32), 8);
        a.rule = HD_RULE_AND;
        a.groups = 1;
        a.planes = 4;
        a.plane_buf[0] = DevBuf(a.n_rows * a.words * 16, ctx->stream);
        hd::k_random_planes<<<ctx->sm_count * 4, 256, 0, ctx->stream>>>(
            a.plane_buf[0].as<uint4>(), a.n_rows * a.words, 1234 + nb * 10 + lb);
        HD_LAUNCHED(ctx);
        // enough copies to fill every SM a few times over at the 128-row tile
        const uint64_t tiles128 = hd::ceil_div(a.n_rows, 128) * (hd::ceil_div(a.n_rows, 128) + 1) / 2;
        const int copies = (int)std::max<uint64_t>(1, std::min<uint64_t>(256, 4ull * ctx->sm_count / tiles128 + 1));
        const uint64_t pairs = a.n_rows * (a.n_rows - 1) / 2;
        for (int dtype : {1, 2}) {
          DevBuf out(pairs * dtype * copies + 64, ctx->stream);
          double best = 1e30;
          hd::TileConfig pick = hd::default_tile_config(a.n_rows, a.length, dtype);
          for (const auto &c : cands) {
            const double ms = hd::time_config(ctx, a, copies, dtype, c, out);
            if (ms < best) {
              best = ms;
              pick = c;
            }
          }
          ctx->tune.push_back({hd::key_of(nb, lb, dtype), {pick.tile, pick.stages}});
        }
      }
    }
    HD_CUDA(cudaStreamSynchronize(ctx->stream));
  });
}

extern "C" int hd_tune_lookup(hd_ctx *ctx, uint64_t n_rows, uint64_t length, int dtype_bytes,
                              int *tile, int *stages) {
  if (!ctx || !tile || !stages) return HD_ERR_ARG;
  hd::TileConfig c = hd::tile_config_for(ctx, n_rows, length, dtype_bytes);
  *tile = c.tile;
  *stages = c.stages;
  return HD_OK;
}

extern "C" int hd_tune_save(hd_ctx *ctx, const char *path) {
  if (!ctx || !path) return HD_ERR_ARG;
  return tune_guard(ctx, [&] {
    cudaDeviceProp prop;
    HD_CUDA(cudaGetDeviceProperties(&prop, ctx->device));
    std::ofstream f(path);
    if (!f) hd::fail(HD_ERR_IO, std::string("Error: Failed to open file '") + path + "'");
    f << "{\"device\": \"" << prop.name << "\", \"sm_count\": " << ctx->sm_count
      << ", \"entries\": [";
    for (size_t k = 0; k < ctx->tune.size(); ++k) {
      const uint32_t key = ctx->tune[k].first;
      f << (k ? ", " : "") << "{\"n_bucket\": " << key / 100 << ", \"L_bucket\": " << key / 10 % 10
        << ", \"dtype\": " << key % 10 << ", \"tile\": " << ctx->tune[k].second.first
        << ", \"stages\": " << ctx->tune[k].second.second << "}";
    }
    f << "]}\n";
  });
}

extern "C" int hd_tune_load(hd_ctx *ctx, const char *path) {
  if (!ctx || !path) return HD_ERR_ARG;
  return tune_guard(ctx, [&] {
    std::ifstream f(path);
    if (!f) hd::fail(HD_ERR_IO, std::string("Error: Failed to open file '") + path + "'");
    std::stringstream ss;
    ss << f.rdbuf();
    const std::string s = ss.str();
    std::vector<std::pair<uint32_t, std::pair<int, int>>> table;
    // one entry per object holding "n_bucket"; whitespace between tokens is free
    auto field = [&](const char *name, size_t from, size_t to, int &v) {
      const std::string key = std::string("\"") + name + "\"";
      size_t p = s.find(key, from);
      if (p == std::string::npos || p >= to) return false;
      p = s.find(':', p + key.size());
      if (p == std::string::npos || p >= to) return false;
      v = std::atoi(s.c_str() + p + 1);
      return true;
    };
    size_t pos = 0;
    while ((pos = s.find("\"n_bucket\"", pos)) != std::string::npos) {
      const size_t begin = s.rfind('{', pos);
      const size_t end = s.find('}', pos);
      int nb, lb, dt, tile, st;
      if (begin == std::string::npos || end == std::string::npos || !field("n_bucket", begin, end, nb) ||
          !field("L_bucket", begin, end, lb) || !field("dtype", begin, end, dt) ||
          !field("tile", begin, end, tile) || !field("stages", begin, end, st) ||
          !hd::tile_config_valid(tile, st))
        hd::fail(HD_ERR_ARG, std::string("malformed tuning file '") + path + "'");
      table.push_back({hd::key_of(nb, lb, dt), {tile, st}});
      pos = end;
    }
    ctx->tune = table;
  });
}
