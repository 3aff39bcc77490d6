// Serving: packed alignments stay resident in HBM and requests are folded
// into the persistent pairwise engine as they arrive. No reference
// counterpart (the reference computes one matrix per call).
//
// Requests:
//  * reference query  : distances of a query sequence to every record of a
//                       resident alignment (fasta_reference_distances rule,
//                       src/hamming.cc:128-136; uint32 per input record);
//  * pairwise matrix  : the lower triangle of a window of n rows of a resident
//                       alignment (uint8/uint16, max_distance clamped as
//                       safe_int_cast, include/hamming/hamming_impl.hh:37-45);
//  * sparse dump      : the "i j d" lines with d <= threshold of a window's
//                       lower triangle (DataSet::dump_sparse,
//                       include/hamming/hamming.hh:79-114).
//
// Scheduling (continuous batching): a launcher thread admits queued requests
// in arrival order while the device output bytes they need fit in the
// budget, folds all admitted requests into one wave (one persistent kernel
// over every matrix's tiles + the query kernels) and launches it on a free
// worker stream; up to `max_waves` waves are on the device at once, so a
// wave launched while earlier ones run fills the SMs their CTAs release. A
// completion thread finalises waves in launch order (copies results back,
// formats sparse text on the device), releases their bytes and wakes
// waiters. All waits are host-side and bounded by the caller's timeout.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>

#include "hd_internal.cuh"

using hd::DevBuf;

namespace {

using Clock = std::chrono::steady_clock;
enum Kind { kRef = 0, kPair = 1, kSparse = 2 };
constexpr size_t kMaxPerWave = 512;

struct Req {
  uint64_t id = 0;
  int kind = kRef;
  uint32_t aln = 0;
  const hd_alignment *a = nullptr;  // resolved under the lock at submission
  uint64_t r0 = 0, n = 0;
  int dtype = 1;
  uint32_t max_dist = 255;
  int64_t thr = 0;
  std::string query;
  Clock::time_point t_submit, t_admit, t_done;
  int status = 1;  // 1 pending, 0 done, < 0 error code; written under the lock only
  std::string err;
  int outcome = 1;  // status computed by the completion thread, published under the lock
  std::vector<uint8_t> result;
  uint64_t count = 0;
  uint64_t out_bytes = 0;  // device bytes reserved at admission
  // in flight
  DevBuf d_out, d_query, q_planes;
  std::unique_ptr<hd_alignment> view;
};

struct Wave {
  hd_ctx *w = nullptr;  // worker context: its own stream
  std::vector<Req *> reqs;
  hd::PairLaunchPlan plan;
  cudaEvent_t done = nullptr;
  uint64_t reserved = 0;
  std::string launch_err;
  int launch_rc = HD_OK;
};

uint64_t tri(uint64_t n) { return n < 2 ? 0 : n * (n - 1) / 2; }

}  // namespace

struct hd_server {
  hd_ctx *ctx = nullptr;
  uint64_t budget = 0, in_use = 0;
  std::vector<const hd_alignment *> resident;
  std::mutex mu;
  std::condition_variable cv;
  std::deque<Req *> pending;
  std::unordered_map<uint64_t, std::unique_ptr<Req>> reqs;
  uint64_t next_id = 1;
  std::deque<std::unique_ptr<Wave>> inflight;
  std::vector<hd_ctx *> workers, free_slots;
  std::thread launcher, completer;
  bool stop = false;
  uint64_t waves = 0, completed = 0, max_inflight = 0;

  bool head_fits() const {
    return !pending.empty() &&
           (inflight.empty() || in_use + pending.front()->out_bytes <= budget);
  }
  void launch_loop();
  void complete_loop();
  void launch_wave(Wave &wv);
  void finalize_wave(Wave &wv);
};

void hd_server::launch_loop() {
  std::unique_lock<std::mutex> lk(mu);
  for (;;) {
    cv.wait(lk, [&] { return stop || (!free_slots.empty() && head_fits()); });
    if (stop) return;
    auto wv = std::make_unique<Wave>();
    wv->w = free_slots.back();
    free_slots.pop_back();
    while (!pending.empty() && wv->reqs.size() < kMaxPerWave) {
      Req *r = pending.front();
      const bool alone = inflight.empty() && wv->reqs.empty();
      if (!alone && in_use + r->out_bytes > budget) break;
      pending.pop_front();
      in_use += r->out_bytes;
      wv->reserved += r->out_bytes;
      r->t_admit = Clock::now();
      wv->reqs.push_back(r);
    }
    lk.unlock();
    launch_wave(*wv);
    lk.lock();
    ++waves;
    inflight.push_back(std::move(wv));
    max_inflight = std::max<uint64_t>(max_inflight, inflight.size());
    cv.notify_all();
  }
}

void hd_server::launch_wave(Wave &wv) {
  hd_ctx *w = wv.w;
  try {
    HD_CUDA(cudaSetDevice(w->device));
    if (!wv.done) HD_CUDA(cudaEventCreateWithFlags(&wv.done, cudaEventDisableTiming));
    std::vector<hd::PairJobSpec> specs;
    for (Req *r : wv.reqs) {
      const hd_alignment *a = r->a;
      if (r->kind == kRef) {
        r->d_query = DevBuf(r->query.size() + 16, w->stream);
        HD_CUDA(cudaMemcpyAsync(r->d_query.p, r->query.data(), r->query.size(),
                                cudaMemcpyHostToDevice, w->stream));
        r->d_out = DevBuf(a->n_rows * 4 + 16, w->stream);
        hd::query_distances_async(w, a, r->d_query.as<uint8_t>(), r->d_out.as<uint32_t>(),
                                  r->q_planes);
        continue;
      }
      auto v = std::make_unique<hd_alignment>();
      v->ctx = w;
      v->device = w->device;
      v->base = a->base ? a->base : a;
      v->row0 = a->row0 + r->r0;
      v->n_rows = r->n;
      v->n_input = r->n;
      v->length = a->length;
      v->words = a->words;
      v->rule = a->rule;
      v->groups = a->groups;
      v->planes = a->planes;
      const int dt = r->kind == kPair ? r->dtype : 1;
      r->d_out = DevBuf(std::max<uint64_t>(tri(r->n) * dt, 16), w->stream);
      hd::PairJobSpec s;
      s.aln = v.get();
      s.dtype = dt;
      s.max_dist = r->kind == kPair ? r->max_dist : 255;
      s.d_out = r->d_out.p;
      s.cfg = hd::tile_config_for(w, r->n, a->length, dt);
      s.tile_lo = 0;
      s.tile_hi = (uint32_t)hd::ceil_div(r->n, (uint64_t)s.cfg.tile);
      specs.push_back(s);
      r->view = std::move(v);
    }
    if (!specs.empty()) hd::run_pairwise_jobs(w, specs, w->stream, &wv.plan);
  } catch (const hd::Error &e) {
    wv.launch_rc = e.code;
    wv.launch_err = e.msg;
  }
  cudaEventRecord(wv.done, w->stream);
}

void hd_server::finalize_wave(Wave &wv) {
  hd_ctx *w = wv.w;
  cudaSetDevice(w->device);
  cudaEventSynchronize(wv.done);
  int st = 0;
  cudaMemcpy(&st, w->d_status, sizeof(int), cudaMemcpyDeviceToHost);
  if (st) {
    cudaMemset(w->d_status, 0, sizeof(int));
    if (wv.launch_rc == HD_OK) {
      wv.launch_rc = HD_ERR_TIMEOUT;
      wv.launch_err = "a device wait for a TMA transfer ran out (pairwise kernel)";
    }
  }
  cudaError_t ce = cudaGetLastError();
  if (ce != cudaSuccess && wv.launch_rc == HD_OK) {
    wv.launch_rc = HD_ERR_CUDA;
    wv.launch_err = cudaGetErrorString(ce);
  }
  // results go to fields no waiter reads before `status` is published
  for (Req *r : wv.reqs) {
    if (wv.launch_rc != HD_OK) {
      r->outcome = wv.launch_rc;
      r->err = wv.launch_err;
      continue;
    }
    try {
      const hd_alignment *a = r->a;
      if (r->kind == kRef) {
        std::vector<uint32_t> rows(a->n_rows);
        HD_CUDA(cudaMemcpy(rows.data(), r->d_out.p, a->n_rows * 4, cudaMemcpyDeviceToHost));
        const uint64_t n_in = a->seqidx.empty() ? a->n_rows : a->n_input;
        r->result.resize(n_in * 4);
        auto *out = reinterpret_cast<uint32_t *>(r->result.data());
        for (uint64_t k = 0; k < n_in; ++k) out[k] = rows[a->seqidx.empty() ? k : a->seqidx[k]];
        r->count = n_in;
      } else if (r->kind == kPair) {
        r->result.resize(tri(r->n) * r->dtype);
        if (!r->result.empty())
          HD_CUDA(cudaMemcpy(r->result.data(), r->d_out.p, r->result.size(), cudaMemcpyDeviceToHost));
        r->count = tri(r->n);
      } else {
        const uint64_t n = r->n;
        if (n >= 2) {
          DevBuf rb((n + 1) * 8, w->stream), rl((n + 1) * 8, w->stream), tot(8, w->stream);
          hd::sparse_row_sizes(w, r->d_out.p, 1, 0, 1, n, r->thr, rb.as<uint64_t>(),
                               rl.as<uint64_t>());
          hd::scan_exclusive<uint64_t>(w, rl.as<uint64_t>(), rl.as<uint64_t>(), n - 1,
                                       tot.as<uint64_t>());
          uint64_t lines = 0;
          HD_CUDA(cudaMemcpyAsync(&lines, tot.p, 8, cudaMemcpyDeviceToHost, w->stream));
          // the text size is the sum of the row byte counts (scanned on a copy;
          // format_sparse_rows scans the counts again to place the rows)
          DevBuf scratch((n + 1) * 8, w->stream), text_tot(8, w->stream);
          HD_CUDA(cudaMemcpyAsync(scratch.p, rb.p, (n - 1) * 8, cudaMemcpyDeviceToDevice, w->stream));
          hd::scan_exclusive<uint64_t>(w, scratch.as<uint64_t>(), scratch.as<uint64_t>(), n - 1,
                                       text_tot.as<uint64_t>());
          uint64_t text = 0;
          HD_CUDA(cudaMemcpyAsync(&text, text_tot.p, 8, cudaMemcpyDeviceToHost, w->stream));
          HD_CUDA(cudaStreamSynchronize(w->stream));
          DevBuf d_text(text + 16, w->stream);
          const uint64_t nb = hd::format_sparse_rows(w, r->d_out.p, 1, 0, 1, n, r->thr,
                                                     rb.as<uint64_t>(), d_text.as<char>());
          r->result.resize(nb);
          if (nb) HD_CUDA(cudaMemcpy(r->result.data(), d_text.p, nb, cudaMemcpyDeviceToHost));
          r->count = lines;
        }
      }
      r->outcome = 0;
    } catch (const hd::Error &e) {
      r->outcome = e.code;
      r->err = e.msg;
    }
  }
  for (Req *r : wv.reqs) {
    r->d_out.release();
    r->d_query.release();
    r->q_planes.release();
  }
  wv.plan = hd::PairLaunchPlan();
  cudaStreamSynchronize(w->stream);
  for (Req *r : wv.reqs) r->view.reset();
}

void hd_server::complete_loop() {
  std::unique_lock<std::mutex> lk(mu);
  for (;;) {
    cv.wait(lk, [&] { return !inflight.empty() || (stop && inflight.empty()); });
    if (inflight.empty()) return;  // stopping
    Wave *wv = inflight.front().get();
    lk.unlock();
    finalize_wave(*wv);
    lk.lock();
    const auto now = Clock::now();
    for (Req *r : wv->reqs) {  // publish: waiters may now read and release r
      r->t_done = now;
      r->status = r->outcome;
      ++completed;
    }
    in_use -= wv->reserved;
    if (wv->done) cudaEventDestroy(wv->done);
    free_slots.push_back(wv->w);
    inflight.pop_front();
    cv.notify_all();
  }
}

namespace {
template <class F>
int srv_guard(hd_server *s, F &&f) {
  try {
    f();
    return HD_OK;
  } catch (const hd::Error &e) {
    if (s && s->ctx) s->ctx->err = e.msg;
    return e.code;
  }
}

uint64_t submit(hd_server *s, std::unique_ptr<Req> r) {
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->stop) hd::fail(HD_ERR_STATE, "server stopped");
  r->id = s->next_id++;
  r->t_submit = Clock::now();
  Req *p = r.get();
  s->reqs.emplace(p->id, std::move(r));
  s->pending.push_back(p);
  s->cv.notify_all();
  return p->id;
}

const hd_alignment *resident_of(hd_server *s, uint32_t id) {
  std::lock_guard<std::mutex> lk(s->mu);
  if (id >= s->resident.size()) hd::fail(HD_ERR_ARG, "unknown resident alignment");
  return s->resident[id];
}

void check_window(const hd_alignment *a, uint64_t r0, uint64_t n) {
  if (r0 > a->n_rows || n > a->n_rows - r0) hd::fail(HD_ERR_ARG, "row window out of range");
}
}  // namespace

extern "C" {

int hd_server_create(hd_ctx *ctx, uint64_t output_budget_bytes, int max_waves, hd_server **out) {
  if (!ctx || !out || max_waves < 1) return HD_ERR_ARG;
  *out = nullptr;
  auto *s = new hd_server();
  s->ctx = ctx;
  s->budget = output_budget_bytes;
  for (int k = 0; k < max_waves; ++k) {
    hd_ctx *w = nullptr;
    int rc = hd_ctx_create(ctx->device, &w);
    if (rc != HD_OK) {
      for (hd_ctx *x : s->workers) hd_ctx_destroy(x);
      delete s;
      return rc;
    }
    w->tune = ctx->tune;
    s->workers.push_back(w);
    s->free_slots.push_back(w);
  }
  s->launcher = std::thread([s] { s->launch_loop(); });
  s->completer = std::thread([s] { s->complete_loop(); });
  *out = s;
  return HD_OK;
}

int hd_server_add_alignment(hd_server *s, const hd_alignment *aln, uint32_t *id) {
  if (!s || !aln || !id) return HD_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  s->resident.push_back(aln);
  *id = (uint32_t)(s->resident.size() - 1);
  return HD_OK;
}

int hd_server_submit_reference(hd_server *s, uint32_t aln_id, const char *query, uint64_t len,
                               uint64_t *ticket) {
  if (!s || !query || !ticket) return HD_ERR_ARG;
  return srv_guard(s, [&] {
    const hd_alignment *a = resident_of(s, aln_id);
    if (a->rule != HD_RULE_AND)
      hd::fail(HD_ERR_ARG, "reference queries need an AND-rule alignment");
    if (len != a->length) hd::fail(HD_ERR_LENGTH, "Error: Sequences do not all have the same length");
    auto r = std::make_unique<Req>();
    r->kind = kRef;
    r->aln = aln_id;
    r->a = a;
    r->query.assign(query, len);
    r->out_bytes = a->n_rows * 4;
    *ticket = submit(s, std::move(r));
  });
}

int hd_server_submit_pairwise(hd_server *s, uint32_t aln_id, uint64_t row0, uint64_t n_rows,
                              int dtype_bytes, int64_t max_distance, uint64_t *ticket) {
  if (!s || !ticket) return HD_ERR_ARG;
  return srv_guard(s, [&] {
    const hd_alignment *a = resident_of(s, aln_id);
    check_window(a, row0, n_rows);
    if (dtype_bytes != 1 && dtype_bytes != 2) hd::fail(HD_ERR_ARG, "dtype_bytes must be 1 or 2");
    const uint32_t tmax = dtype_bytes == 1 ? 0xffu : 0xffffu;
    auto r = std::make_unique<Req>();
    r->kind = kPair;
    r->aln = aln_id;
    r->a = a;
    r->r0 = row0;
    r->n = n_rows;
    r->dtype = dtype_bytes;
    r->max_dist = max_distance > (int64_t)tmax ? tmax : (uint32_t)((uint64_t)max_distance & tmax);
    r->out_bytes = tri(n_rows) * dtype_bytes;
    *ticket = submit(s, std::move(r));
  });
}

int hd_server_submit_sparse(hd_server *s, uint32_t aln_id, uint64_t row0, uint64_t n_rows,
                            int64_t threshold, uint64_t *ticket) {
  if (!s || !ticket) return HD_ERR_ARG;
  return srv_guard(s, [&] {
    const hd_alignment *a = resident_of(s, aln_id);
    check_window(a, row0, n_rows);
    if (threshold >= 255) hd::fail(HD_ERR_ARG, "sparse requests take a threshold below 255");
    auto r = std::make_unique<Req>();
    r->kind = kSparse;
    r->aln = aln_id;
    r->a = a;
    r->r0 = row0;
    r->n = n_rows;
    r->thr = threshold;
    r->out_bytes = tri(n_rows);
    *ticket = submit(s, std::move(r));
  });
}

int hd_server_wait(hd_server *s, uint64_t ticket, double timeout_s) {
  if (!s) return HD_ERR_ARG;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) {
    s->ctx->err = "unknown ticket";
    return HD_ERR_ARG;
  }
  Req *r = it->second.get();
  const bool ok = s->cv.wait_for(lk, std::chrono::duration<double>(timeout_s),
                                 [&] { return r->status != 1; });
  if (!ok) {
    s->ctx->err = "request not finished within the timeout";
    return HD_ERR_TIMEOUT;
  }
  if (r->status < 0) {
    s->ctx->err = r->err;
    return r->status;
  }
  return HD_OK;
}

int hd_server_result(hd_server *s, uint64_t ticket, const void **data, uint64_t *bytes,
                     uint64_t *count, double *latency_ms, double *queue_ms) {
  if (!s) return HD_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end() || it->second->status != 0) {
    s->ctx->err = "no finished result for this ticket";
    return HD_ERR_STATE;
  }
  Req *r = it->second.get();
  if (data) *data = r->result.data();
  if (bytes) *bytes = r->result.size();
  if (count) *count = r->count;
  if (latency_ms)
    *latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
  if (queue_ms)
    *queue_ms = std::chrono::duration<double, std::milli>(r->t_admit - r->t_submit).count();
  return HD_OK;
}

int hd_server_cancel(hd_server *s, uint64_t ticket) {
  if (!s) return HD_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return HD_ERR_ARG;
  Req *r = it->second.get();
  auto q = std::find(s->pending.begin(), s->pending.end(), r);
  if (q == s->pending.end()) {
    s->ctx->err = "request already admitted";
    return HD_ERR_STATE;
  }
  s->pending.erase(q);
  r->status = HD_ERR_STATE;
  r->err = "request cancelled";
  s->cv.notify_all();
  return HD_OK;
}

int hd_server_release(hd_server *s, uint64_t ticket) {
  if (!s) return HD_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end() || it->second->status == 1) return HD_ERR_STATE;
  s->reqs.erase(it);
  return HD_OK;
}

int hd_server_stats(hd_server *s, uint64_t *waves, uint64_t *completed, uint64_t *max_inflight,
                    uint64_t *bytes_in_use) {
  if (!s) return HD_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  if (waves) *waves = s->waves;
  if (completed) *completed = s->completed;
  if (max_inflight) *max_inflight = s->max_inflight;
  if (bytes_in_use) *bytes_in_use = s->in_use;
  return HD_OK;
}

void hd_server_free(hd_server *s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
    for (Req *r : s->pending) {
      r->status = HD_ERR_STATE;
      r->err = "server stopped";
    }
    s->pending.clear();
    s->cv.notify_all();
  }
  s->launcher.join();
  s->completer.join();  // drains the waves already on the device
  for (hd_ctx *w : s->workers) hd_ctx_destroy(w);
  delete s;
}

int hd_alignment_view(const hd_alignment *base, uint64_t row0, uint64_t n_rows,
                      hd_alignment **out) {
  if (!base || !out) return HD_ERR_ARG;
  if (row0 > base->n_rows || n_rows > base->n_rows - row0) return HD_ERR_ARG;
  auto *v = new hd_alignment();
  v->ctx = base->ctx;
  v->device = base->device;
  v->base = base->base ? base->base : base;
  v->row0 = base->row0 + row0;
  v->n_rows = n_rows;
  v->n_input = n_rows;
  v->length = base->length;
  v->words = base->words;
  v->rule = base->rule;
  v->groups = base->groups;
  v->planes = base->planes;
  *out = v;
  return HD_OK;
}

}  // extern "C"
