// Serving: continuous batching of reconstruction requests on one GPU.
//
// Requests wait in an arrival-order queue and are admitted while the sum of
// the admitted requests' device footprints stays within the byte budget.
// Admitted requests keep all their state on the device (projections,
// per-axis iterates, MACE state) until they retire.  Every step runs one
// SIRT iteration of every admitted request through the persistent batched
// kernels (one launch per phase over all of them), so a request's latency
// is its own iteration count times the step time of the mix it shares the
// GPU with, and new requests join at the next step instead of waiting for a
// whole batch to drain.  The schedule of one request (WBP init, n_outer x
// (n_inner SIRT iterations, MACE step)) is the one mtr_reconstruct runs.
#include <algorithm>
#include <deque>
#include <memory>
#include <new>
#include <vector>

#include "mtr_internal.h"
#include "mtr_runtime.h"

using namespace mtr;

namespace {

struct Request {
  long long id = 0;
  mtr_request q{};
  std::vector<mtr_axis> axes;
  long long footprint = 0;
  long long voxel_updates = 0;
  mtr_recon* r = nullptr;
  int it = 0, j = 0;      // outer iteration, SIRT iteration within it
  bool finished = false;  // its last MACE step is enqueued
};

}  // namespace

struct mtr_server {
  mtr_context* ctx = nullptr;
  long long budget = 0;
  int precision = MTR_PREC_FP32;
  std::deque<std::unique_ptr<Request>> queue;
  std::vector<std::unique_ptr<Request>> active;
  SirtTables tables;
  bool dirty = true;
  DevBuf err;
  long long next_id = 1;
  mtr_server_stats st{};
  ~mtr_server() {
    for (auto& a : active)
      if (a->r) mtr_recon_destroy(a->r);
  }
};

namespace {

mtr_status retire(mtr_server* s, int max_done, long long* done_ids, int* n_done) {
  for (size_t i = 0; i < s->active.size();) {
    Request& a = *s->active[i];
    if (!a.finished || *n_done >= max_done) {
      ++i;
      continue;
    }
    mtr_status rs = mtr_recon_download(a.r, a.q.out, MTR_MEM_HOST);
    if (rs != MTR_OK) return rs;
    mtr_recon_destroy(a.r);
    a.r = nullptr;
    s->st.bytes_in_use -= a.footprint;
    s->st.completed += 1;
    s->st.voxel_updates += a.voxel_updates;
    done_ids[(*n_done)++] = a.id;
    s->active.erase(s->active.begin() + (long)i);
  }
  return MTR_OK;
}

mtr_status admit(mtr_server* s) {
  while (!s->queue.empty() && s->st.bytes_in_use + s->queue.front()->footprint <= s->budget) {
    std::unique_ptr<Request> a = std::move(s->queue.front());
    s->queue.pop_front();
    mtr_params p{};
    p.iter_times = a->q.iter_times;
    p.sirt_inner = a->q.sirt_inner;
    p.sirt_step = a->q.sirt_step;
    p.mace_step = a->q.mace_step;
    p.precision = s->precision;
    p.flags = 0;
    mtr_status rs = mtr_recon_create(s->ctx, a->q.n_axes, a->axes.data(), a->q.vol, &p, MTR_MEM_HOST, &a->r);
    if (rs != MTR_OK) {
      s->queue.push_front(std::move(a));  // stays first in line
      return rs;
    }
    a->footprint = std::max(a->footprint, a->r->bytes);
    s->st.bytes_in_use += a->footprint;
    s->st.peak_bytes = std::max(s->st.peak_bytes, s->st.bytes_in_use);
    rs = recon_enqueue_init(a->r);
    if (rs != MTR_OK) return rs;
    if (a->q.iter_times == 0 || a->q.sirt_inner == 0) a->finished = true;  // the WBP sum is the result
    s->active.push_back(std::move(a));
    s->dirty = true;
  }
  return MTR_OK;
}

}  // namespace

extern "C" {

mtr_status mtr_server_create(mtr_context* ctx, long long budget_bytes, int precision, mtr_server** out) {
  if (!ctx || !out || budget_bytes <= 0) return set_error(ctx, MTR_ERR_INVALID_ARGUMENT, "invalid argument");
  if (precision < MTR_PREC_FP32 || precision > MTR_PREC_MIXED_FP16)
    return set_error(ctx, MTR_ERR_INVALID_ARGUMENT, "unknown precision");
  *out = nullptr;
  DeviceGuard g(ctx->device);
  std::unique_ptr<mtr_server> s(new (std::nothrow) mtr_server());
  if (!s) return set_error(ctx, MTR_ERR_OUT_OF_MEMORY, "host allocation");
  s->ctx = ctx;
  s->budget = budget_bytes;
  s->precision = precision;
  s->st.budget_bytes = budget_bytes;
  MTR_CK(ctx, s->err.alloc(sizeof(int)));
  MTR_CK(ctx, cudaMemsetAsync(s->err.p, 0, sizeof(int), ctx->stream));
  *out = s.release();
  return MTR_OK;
}

mtr_status mtr_server_submit(mtr_server* s, const mtr_request* req, long long* id) {
  if (!s || !req || !id) return MTR_ERR_INVALID_ARGUMENT;
  mtr_context* ctx = s->ctx;
  if (req->n_axes <= 0 || req->n_axes > MTR_MAX_AXES || !req->axes || !req->out)
    return set_error(ctx, MTR_ERR_INVALID_ARGUMENT, "request needs 1..MTR_MAX_AXES axes and an output buffer");
  if (req->iter_times < 0 || req->sirt_inner < 0)
    return set_error(ctx, MTR_ERR_INVALID_ARGUMENT, "negative iteration count");
  mtr_status rs = check_volume(ctx, req->vol);
  if (rs != MTR_OK) return rs;
  std::vector<mtr_projection_size> prjs;
  for (int k = 0; k < req->n_axes; ++k) {
    rs = check_axis(ctx, req->axes[k]);
    if (rs != MTR_OK) return rs;
    prjs.push_back(req->axes[k].prj);
  }
  std::unique_ptr<Request> a(new (std::nothrow) Request());
  if (!a) return set_error(ctx, MTR_ERR_OUT_OF_MEMORY, "host allocation");
  rs = mtr_estimate_footprint(req->n_axes, prjs.data(), req->vol, s->precision, &a->footprint);
  if (rs != MTR_OK) return rs;
  if (a->footprint > s->budget)
    return set_error(ctx, MTR_ERR_CAPACITY, "request footprint exceeds the server budget");
  a->q = *req;
  a->axes.assign(req->axes, req->axes + req->n_axes);
  a->q.axes = nullptr;
  a->voxel_updates = (long long)req->vol.X * req->vol.Y * req->vol.Z * req->n_axes * req->iter_times * req->sirt_inner;
  a->id = s->next_id++;
  *id = a->id;
  s->queue.push_back(std::move(a));
  s->st.submitted += 1;
  return MTR_OK;
}

mtr_status mtr_server_step(mtr_server* s, int max_done, long long* done_ids, int* n_done) {
  if (!s || !n_done || (max_done > 0 && !done_ids)) return MTR_ERR_INVALID_ARGUMENT;
  *n_done = 0;
  mtr_context* ctx = s->ctx;
  DeviceGuard g(ctx->device);
  MTR_CK(ctx, cudaStreamSynchronize(ctx->stream));
  int flag = 0;
  MTR_CK(ctx, cudaMemcpy(&flag, s->err.p, sizeof(int), cudaMemcpyDeviceToHost));
  if (flag) return set_error(ctx, MTR_ERR_TIMEOUT, "a batched kernel gave up on a bounded wait");
  mtr_status rs = retire(s, max_done, done_ids, n_done);
  if (rs != MTR_OK) return rs;
  rs = admit(s);
  if (rs != MTR_OK && !(rs == MTR_ERR_OUT_OF_MEMORY && !s->active.empty())) return rs;
  std::vector<mtr_recon*> sirt;
  for (auto& a : s->active)
    if (!a->finished) sirt.push_back(a->r);
  if (s->dirty) {
    rs = build_sirt_tables(ctx, sirt, s->precision, s->tables);
    if (rs != MTR_OK) return rs;
    s->dirty = false;
  }
  if (!sirt.empty()) {
    rs = enqueue_sirt_iteration(ctx, s->tables, s->err.as<int>());
    if (rs != MTR_OK) return rs;
    for (auto& a : s->active) {
      if (a->finished) continue;
      if (++a->j < a->q.sirt_inner) continue;
      a->j = 0;
      rs = recon_enqueue_mace(a->r, a->it);
      if (rs != MTR_OK) return rs;
      if (++a->it == a->q.iter_times) {
        a->finished = true;
        s->dirty = true;
      }
    }
    s->st.steps += 1;
  }
  s->st.queued = (long long)s->queue.size();
  s->st.active = (long long)s->active.size();
  return MTR_OK;
}

mtr_status mtr_server_stats_get(const mtr_server* s, mtr_server_stats* st) {
  if (!s || !st) return MTR_ERR_INVALID_ARGUMENT;
  *st = s->st;
  st->queued = (long long)s->queue.size();
  st->active = (long long)s->active.size();
  return MTR_OK;
}

mtr_status mtr_server_destroy(mtr_server* s) {
  if (!s) return MTR_OK;
  DeviceGuard g(s->ctx->device);
  cudaStreamSynchronize(s->ctx->stream);
  delete s;
  return MTR_OK;
}

}  // extern "C"
