// Autotuner for the two distance engines, per (n bucket, L bucket, output
// dtype):
//  * the bit-plane engine's tile edge (64 or 128 rows, i.e. 4 or 8 rows per
//    thread) and TMA staging depth;
//  * the tensor-core engine's L2 band (tile rows per band) and item shape
//    (one or two 128-row tiles per item);
// and per L bucket the launch size (single-row-tile items) from which a
// matrix launched alone goes to the tensor-core engine rather than the
// bit-plane engine. The configurations are timed with the GPU filled (a batch
// of copies of a synthetic packed alignment of the bucket's representative
// size), so the figure is throughput per pair-site as the batched and served
// paths see it; the launch-size threshold is timed on single matrices. The
// table can be saved to and loaded from a small JSON file;
// HAMMINGDIST_TILE=<tile>x<stages>, HAMMINGDIST_MMA_BAND=<rows>,
// HAMMINGDIST_MMA_ROWS=<1|2> and HAMMINGDIST_MMA_MIN_ITEMS=<items> override it.
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
// single-row-tile items of the tensor-core engine for one matrix of n rows
uint64_t mma_items_of(uint64_t n) {
  uint64_t items = 0;
  for (uint64_t I = 0; I < ceil_div(n, (uint64_t)kTile); ++I)
    items += ((I + 1) * kTile - 2) / kMmaCols + 1;
  return items;
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

// Best of four timed runs (after a warm-up run) of the launches of `copies`
// matrices of the alignment in one launch plan, with engine choice `engine`
// (-1 as configured, 0 bit-plane only, 1 tensor cores).
double time_config(hd_ctx *ctx, const hd_alignment &a, int copies, int dtype, TileConfig tc,
                   DevBuf &out, int engine = 0) {
  struct Restore {
    hd_ctx *c;
    int e;
    ~Restore() { c->engine_force = e; }
  } restore{ctx, ctx->engine_force};
  ctx->engine_force = engine;
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
  for (int rep = 0; rep < 5; ++rep) {
    // the launches alone: planning (tables, operands) happens before
    std::vector<PairJobSpec> sp = specs;
    PairLaunchPlan plan;
    prepare_pairwise_jobs(ctx, sp, ctx->stream, &plan);
    HD_CUDA(cudaEventRecord(e0, ctx->stream));
    launch_pairwise_plan(ctx, plan, ctx->stream);
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
  TileConfig c = default_tile_config(n_rows, length, dtype_bytes);
  const uint32_t key = key_of(n_bucket(n_rows), l_bucket(length), dtype_bytes == 1 ? 1 : 2);
  for (const auto &e : ctx->tune.entries)
    if (e.first == key) c = e.second;
  env_override(c);
  return c;
}

uint64_t mma_min_items_for(hd_ctx *ctx, uint64_t length) {
  if (const char *e = std::getenv("HAMMINGDIST_MMA_MIN_ITEMS")) return (uint64_t)std::max(0, std::atoi(e));
  const uint64_t t = ctx->tune.mma_min_items[l_bucket(length)];
  return t ? t : 48;
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

namespace {
// a synthetic packed alignment of n rows x L sites (random one-hot planes)
void make_synthetic(hd_ctx *ctx, hd_alignment &a, uint64_t n, uint64_t L, uint64_t seed) {
  a.ctx = ctx;
  a.device = ctx->device;
  a.n_rows = n;
  a.n_input = n;
  a.length = L;
  a.words = hd::round_up(hd::ceil_div(a.length, 32), 8);
  a.rule = HD_RULE_AND;
  a.groups = 1;
  a.planes = 4;
  a.plane_buf[0] = DevBuf(a.n_rows * a.words * 16, ctx->stream);
  hd::k_random_planes<<<ctx->sm_count * 4, 256, 0, ctx->stream>>>(a.plane_buf[0].as<uint4>(),
                                                                   a.n_rows * a.words, seed);
  HD_LAUNCHED(ctx);
}
}  // namespace

extern "C" int hd_autotune(hd_ctx *ctx, uint64_t max_n_bucket) {
  if (!ctx) return HD_ERR_ARG;
  return tune_guard(ctx, [&] {
    const hd::TileConfig cands[] = {{128, 3}, {128, 2}, {128, 4}, {64, 3}, {64, 4}};
    // tensor-core engine: (band, row tiles per item)
    const int mma_cands[][2] = {{16, 2}, {8, 2}, {32, 2}, {16, 1}};
    const int nbmax = (int)std::min<uint64_t>(max_n_bucket, 6);
    hd::TuneTable table;
    for (int nb = 0; nb <= nbmax; ++nb) {
      for (int lb = 0; lb < 4; ++lb) {
        hd_alignment a;
        make_synthetic(ctx, a, hd::kNRep[nb], hd::kLRep[lb], 1234 + nb * 10 + lb);
        // enough copies to fill every SM a few times over at the 128-row tile
        const uint64_t tiles128 = hd::ceil_div(a.n_rows, 128) * (hd::ceil_div(a.n_rows, 128) + 1) / 2;
        const int copies = (int)std::max<uint64_t>(1, std::min<uint64_t>(256, 4ull * ctx->sm_count / tiles128 + 1));
        const uint64_t pairs = a.n_rows * (a.n_rows - 1) / 2;
        for (int dtype : {1, 2}) {
          DevBuf out(pairs * dtype * copies + 64, ctx->stream);
          double best = 1e30;
          hd::TileConfig pick = hd::default_tile_config(a.n_rows, a.length, dtype);
          for (const auto &c : cands) {
            const double ms = hd::time_config(ctx, a, copies, dtype, c, out, 0);
            if (ms < best) {
              best = ms;
              pick.tile = c.tile;
              pick.stages = c.stages;
            }
          }
          double best_mma = 1e30;
          for (const auto &m : mma_cands) {
            hd::TileConfig c = pick;
            c.mma_band = m[0];
            c.mma_rows = m[1];
            const double ms = hd::time_config(ctx, a, copies, dtype, c, out, 1);
            if (ms < best_mma) {
              best_mma = ms;
              pick.mma_band = m[0];
              pick.mma_rows = m[1];
            }
          }
          table.entries.push_back({hd::key_of(nb, lb, dtype), pick});
        }
      }
    }
    // launch-size threshold per L bucket: single matrices of growing n, each
    // on both engines with the bucket's configuration; the threshold is the
    // item count of the smallest n from which the tensor cores win for every
    // larger n measured
    const uint64_t ns[] = {128, 256, 384, 512, 768, 1024, 1536, 2048, 3072};
    for (int lb = 0; lb < 4; ++lb) {
      uint64_t threshold = 0;  // none found: keep the built-in value
      bool mma_wins_above = true;
      for (int k = (int)(sizeof(ns) / sizeof(ns[0])) - 1; k >= 0; --k) {
        hd_alignment a;
        make_synthetic(ctx, a, ns[k], hd::kLRep[lb], 77 + k * 10 + lb);
        const uint64_t pairs = a.n_rows * (a.n_rows - 1) / 2;
        DevBuf out(pairs + 64, ctx->stream);
        hd::TileConfig c = hd::default_tile_config(a.n_rows, a.length, 1);
        const uint32_t key = hd::key_of(hd::n_bucket(a.n_rows), lb, 1);
        for (const auto &e : table.entries)
          if (e.first == key) c = e.second;
        const double t_lop3 = hd::time_config(ctx, a, 1, 1, c, out, 0);
        const double t_mma = hd::time_config(ctx, a, 1, 1, c, out, 1);
        mma_wins_above = mma_wins_above && t_mma < t_lop3;
        if (mma_wins_above) threshold = hd::mma_items_of(ns[k]);
      }
      table.mma_min_items[lb] = threshold ? threshold : 0;
    }
    ctx->tune = table;
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

extern "C" int hd_tune_lookup_mma(hd_ctx *ctx, uint64_t n_rows, uint64_t length, int dtype_bytes,
                                  int *band, int *rows, uint64_t *min_items) {
  if (!ctx || !band || !rows || !min_items) return HD_ERR_ARG;
  hd::TileConfig c = hd::tile_config_for(ctx, n_rows, length, dtype_bytes);
  *band = hd::mma_band_of(c);
  *rows = hd::mma_rows_of(c);
  *min_items = hd::mma_min_items_for(ctx, length);
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
      << ", \"mma_min_items\": [";
    for (int lb = 0; lb < 4; ++lb) f << (lb ? ", " : "") << ctx->tune.mma_min_items[lb];
    f << "], \"entries\": [";
    for (size_t k = 0; k < ctx->tune.entries.size(); ++k) {
      const uint32_t key = ctx->tune.entries[k].first;
      const hd::TileConfig &c = ctx->tune.entries[k].second;
      f << (k ? ",\n  " : "\n  ") << "{\"n_bucket\": " << key / 100 << ", \"L_bucket\": "
        << key / 10 % 10 << ", \"dtype\": " << key % 10 << ", \"tile\": " << c.tile
        << ", \"stages\": " << c.stages << ", \"mma_band\": " << c.mma_band
        << ", \"mma_rows\": " << c.mma_rows << "}";
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
    hd::TuneTable table;
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
      int nb, lb, dt, tile, st, band = 0, rows = 0;
      if (begin == std::string::npos || end == std::string::npos || !field("n_bucket", begin, end, nb) ||
          !field("L_bucket", begin, end, lb) || !field("dtype", begin, end, dt) ||
          !field("tile", begin, end, tile) || !field("stages", begin, end, st) ||
          !hd::tile_config_valid(tile, st))
        hd::fail(HD_ERR_ARG, std::string("malformed tuning file '") + path + "'");
      // the tensor-core fields are optional (0: built-in)
      field("mma_band", begin, end, band);
      field("mma_rows", begin, end, rows);
      if (band < 0 || band > 1024 || rows < 0 || rows > 2)
        hd::fail(HD_ERR_ARG, std::string("malformed tuning file '") + path + "'");
      hd::TileConfig c;
      c.tile = tile;
      c.stages = st;
      c.mma_band = band;
      c.mma_rows = rows;
      table.entries.push_back({hd::key_of(nb, lb, dt), c});
      pos = end;
    }
    // optional "mma_min_items": [four values, one per L bucket]
    const size_t mi = s.find("\"mma_min_items\"");
    const size_t open_b = mi == std::string::npos ? mi : s.find('[', mi);
    const size_t close_b = open_b == std::string::npos ? open_b : s.find(']', open_b);
    if (close_b != std::string::npos) {
      size_t q = open_b + 1;
      for (int lb = 0; lb < 4 && q < close_b; ++lb) {
        table.mma_min_items[lb] = (uint64_t)std::strtoull(s.c_str() + q, nullptr, 10);
        const size_t comma = s.find(',', q);
        if (comma == std::string::npos || comma > close_b) break;
        q = comma + 1;
      }
    }
    ctx->tune = table;
  });
}
