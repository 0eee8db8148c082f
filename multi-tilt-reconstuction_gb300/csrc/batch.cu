// Batched reconstruction of many tilt series of uneven size and axis count.
//
// Each instance is an mtr_recon (its own buffers, WBP init and MACE state).
// The SIRT phases of all instances run together: per phase ONE persistent
// launch whose CTAs (a grid sized to the GPU's resident capacity) take the
// items of a work list covering the small axes of every instance:
//   forward splat   item = (axis, brick)            fwd_batch_kernel
//   residual        item = (axis, 64 Ki pixels)     residual_batch_kernel
//   back-projection item = (axis, brick)            bp_batch_kernel
//   MACE consensus  item = (instance, 64 Ki voxels) mace_batch_kernel
// so small instances no longer leave SMs idle.  An axis with enough bricks to
// fill the GPU for kOwnWaves waves, an axis tuned to patch tiles, and an axis
// whose window fits no TMA box keep their own launches instead (arguments in
// the constant bank, which the persistent kernels have to stage through
// shared memory): each such axis' forward -> residual -> back-projection
// chain runs on a side stream, concurrent with the persistent launches.  A
// work list is a descriptor table in cost order plus the prefix sum of the
// descriptors' item counts; a CTA finds its descriptor by binary search.
// Each axis keeps the brick depth, lane layout and tensor maps it was tuned
// to.  The whole schedule (WBP init of every instance, n_outer x n_inner SIRT
// phases, MACE steps) is captured once into a CUDA graph and replayed.
#include <algorithm>
#include <memory>
#include <new>
#include <numeric>
#include <vector>

#include "mtr_internal.h"
#include "mtr_runtime.h"

using namespace mtr;

namespace {

int copy_kind_of(int precision) {
  return precision == MTR_PREC_MIXED_BF16 ? 1 : precision == MTR_PREC_MIXED_FP16 ? 2 : 0;
}

constexpr int kOwnWaves = 4;

int forward_ctas_per_sm(int ck, size_t smem) {
  if (ck == 1) return forward_batch_ctas_per_sm<__nv_bfloat16>(smem);
  if (ck == 2) return forward_batch_ctas_per_sm<__half>(smem);
  return forward_batch_ctas_per_sm<float>(smem);
}

// Copy a host table to a device buffer that only grows.
template <typename T>
mtr_status upload_grow(mtr_context* ctx, DevBuf& buf, const std::vector<T>& v) {
  if (v.empty()) return MTR_OK;
  const size_t n = sizeof(T) * v.size();
  if (buf.bytes < n) MTR_CK(ctx, buf.alloc(n + n / 2));
  MTR_CK(ctx, cudaMemcpyAsync(buf.p, v.data(), n, cudaMemcpyHostToDevice, ctx->stream));
  return MTR_OK;
}

// Reorder descriptors by decreasing per-item cost; returns the prefix sum of
// the item counts in the new order (n + 1 entries).
template <typename D>
std::vector<long long> order_by_cost(std::vector<D>& descs, const std::vector<long long>& counts,
                                     const std::vector<long long>& cost) {
  std::vector<int> idx(descs.size());
  std::iota(idx.begin(), idx.end(), 0);
  std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return cost[a] > cost[b]; });
  std::vector<D> d2;
  std::vector<long long> first(1, 0);
  for (int i : idx) {
    d2.push_back(descs[i]);
    first.push_back(first.back() + counts[i]);
  }
  descs.swap(d2);
  return first;
}

}  // namespace

mtr_status mtr::build_sirt_tables(mtr_context* ctx, const std::vector<mtr_recon*>& recs, int precision,
                                  SirtTables& t) {
  const int ck = copy_kind_of(precision);
  t.copy_kind = ck;
  t.own.clear();
  t.bp_smem = t.fwd_smem = 0;
  std::vector<CUtensorMap> maps;
  std::vector<BpBatchDesc> bpd;
  std::vector<FwdBatchDesc> fwd;
  std::vector<ResBatchDesc> resd;
  std::vector<long long> bp_count, fwd_count, res_count, bp_cost, fwd_cost, res_cost;
  std::vector<int> bp_map, fwd_map;  // index of each descriptor's tensor map in `maps`
  for (mtr_recon* r : recs) {
    if (copy_kind_of(r->p.precision) != ck) return set_error(ctx, MTR_ERR_INVALID_ARGUMENT, "mixed precisions");
    const VolDev& v = r->vol;
    for (int k = 0; k < r->K; ++k) {
      AxisState& a = r->ax[k];
      // brick depth, lane axis, windows and tensor maps as tuned for this axis
      const BpPlan& bp = a.plan;
      const FwdPlan& fp = a.fplan;
      const int bgx = (v.NX + (bp.lanes == 1 ? 8 : 32) - 1) / (bp.lanes == 1 ? 8 : 32);
      const int bgy = (v.NY + (bp.lanes == 1 ? 32 : 8) - 1) / (bp.lanes == 1 ? 32 : 8);
      const int fgx = (v.NX + (fp.lanes == 1 ? 8 : 32) - 1) / (fp.lanes == 1 ? 8 : 32);
      const int fgy = (v.NY + (fp.lanes == 1 ? 32 : 8) - 1) / (fp.lanes == 1 ? 32 : 8);
      // the persistent kernels take lines along X or Y over FP32 windows,
      // depths up to 16, of small axes
      const bool bp_ok = a.tma && !tma_disabled() && bp.lanes != 2 && !bp.pairs && bp.nz <= 16 &&
                         (long long)bgx * bgy * ((v.NZ + bp.nz - 1) / bp.nz) <
                             (long long)kOwnWaves * ctx->num_sms * backproject_batch_ctas_per_sm(bp.smem);
      const bool fwd_ok = a.ftma && !tma_disabled() && fp.lanes != 2 &&
                          (long long)fgx * fgy * ((v.NZ + fp.nz - 1) / fp.nz) <
                              (long long)kOwnWaves * ctx->num_sms * forward_ctas_per_sm(ck, fp.smem);
      if (!bp_ok || !fwd_ok) {  // the whole SIRT chain of this axis runs on its own launches
        t.own.push_back({r, k});
        continue;
      }
      resd.push_back(ResBatchDesc{a.b.p, a.s.as<float>(), a.cf.as<float>(), a.r.as<float>(), a.np});
      res_count.push_back((a.np + kBatchChunk - 1) / kBatchChunk);
      res_cost.push_back(1);
      const int j = (int)maps.size() / 2;
      maps.push_back(a.map_r);
      maps.push_back(a.map_s);
      {
        BpBatchDesc d{};
        d.ax = a.dev();
        d.vol = v;
        d.WX = bp.WX; d.WY = bp.WY; d.align = bp.align;
        const int BX = bp.lanes == 1 ? 8 : 32, BY = bp.lanes == 1 ? 32 : 8;
        d.gx = (v.NX + BX - 1) / BX;
        d.gy = (v.NY + BY - 1) / BY;
        d.lane_y = bp.lanes == 1; d.bz0 = bp.bz0; d.nz = bp.nz;
        d.step = r->p.sirt_step;
        d.vol_out = a.x.as<float>();
        d.cbp = a.cbp.as<float>();
        d.vol_copy = a.xcopy.p;
        d.copy_kind = ck;
        d.map = nullptr;  // set after the maps are uploaded
        bpd.push_back(d);
        bp_map.push_back(2 * j);
        bp_count.push_back((long long)d.gx * d.gy * ((v.NZ + d.nz - 1) / d.nz));
        bp_cost.push_back((long long)a.A * d.nz);
        t.bp_smem = std::max(t.bp_smem, bp.smem);
      }
      {
        FwdBatchDesc d{};
        d.ax = a.dev();
        d.vol = v;
        d.WX = fp.WX; d.WY = fp.WY; d.mass_shift = fp.mass_shift;
        const int BX = fp.lanes == 1 ? 8 : 32, BY = fp.lanes == 1 ? 32 : 8;
        d.gx = (v.NX + BX - 1) / BX;
        d.gy = (v.NY + BY - 1) / BY;
        d.lane_y = fp.lanes == 1; d.bz0 = fp.bz0; d.nz = fp.nz;
        d.x = ck ? a.xcopy.p : a.x.p;
        d.map = nullptr;
        fwd.push_back(d);
        fwd_map.push_back(2 * j + 1);
        fwd_count.push_back((long long)d.gx * d.gy * ((v.NZ + d.nz - 1) / d.nz));
        fwd_cost.push_back((long long)a.A * d.nz);
        t.fwd_smem = std::max(t.fwd_smem, fp.smem);
      }
    }
  }
  mtr_status s = upload_grow(ctx, t.maps, maps);
  if (s != MTR_OK) return s;
  const CUtensorMap* base = t.maps.as<CUtensorMap>();
  for (size_t q = 0; q < bpd.size(); ++q) bpd[q].map = base + bp_map[q];
  for (size_t q = 0; q < fwd.size(); ++q) fwd[q].map = base + fwd_map[q];
  const std::vector<long long> bpf = order_by_cost(bpd, bp_count, bp_cost);
  const std::vector<long long> fwf = order_by_cost(fwd, fwd_count, fwd_cost);
  const std::vector<long long> ref = order_by_cost(resd, res_count, res_cost);
  t.n_bp_desc = (int)bpd.size();
  t.n_fwd_desc = (int)fwd.size();
  t.n_res_desc = (int)resd.size();
  t.n_bp = bpf.back();
  t.n_fwd = fwf.back();
  t.n_res = ref.back();
  if ((s = upload_grow(ctx, t.bp_descs, bpd)) != MTR_OK || (s = upload_grow(ctx, t.fwd_descs, fwd)) != MTR_OK ||
      (s = upload_grow(ctx, t.res_descs, resd)) != MTR_OK || (s = upload_grow(ctx, t.bp_first, bpf)) != MTR_OK ||
      (s = upload_grow(ctx, t.fwd_first, fwf)) != MTR_OK || (s = upload_grow(ctx, t.res_first, ref)) != MTR_OK)
    return s;
  const int sms = ctx->num_sms;
  t.bp_grid = t.n_bp ? (int)std::min<long long>(t.n_bp, (long long)sms * backproject_batch_ctas_per_sm(t.bp_smem)) : 0;
  t.fwd_grid = t.n_fwd ? (int)std::min<long long>(t.n_fwd, (long long)sms * forward_ctas_per_sm(ck, t.fwd_smem)) : 0;
  t.ew_grid = sms * 8;
  // the host tables are released on return: wait for their copies
  MTR_CK(ctx, cudaStreamSynchronize(ctx->stream));
  return MTR_OK;
}

mtr_status mtr::enqueue_sirt_iteration(mtr_context* ctx, const SirtTables& t, int* err) {
  cudaStream_t st = ctx->stream;
  // Own-launch axes: each axis' forward -> residual -> back-projection chain
  // on a side stream (round-robin over up to kSides), concurrent with the
  // persistent launches on the context stream; all joined at the end.
  // Serial when per-kernel profiling is on.
  constexpr int kSides = 8;
  const bool par = !t.own.empty() && !ctx->profiling;
  const int sides = par ? std::min<int>(kSides, (int)t.own.size()) : 0;
  ForkJoin fj(ctx);  // joined back to the context stream on every exit path
  if (par) {
    const mtr_status s = fj.fork(sides);
    if (s != MTR_OK) return s;
  }
  for (size_t i = 0; i < t.own.size(); ++i) {
    if (par) fj.use((int)(i % (size_t)sides));
    mtr_status s = recon_enqueue_forward(t.own[i].first, t.own[i].second);
    if (s == MTR_OK) s = recon_enqueue_residual(t.own[i].first, t.own[i].second);
    if (s == MTR_OK) s = recon_enqueue_sirt_bp(t.own[i].first, t.own[i].second);
    fj.use(-1);
    if (s != MTR_OK) return s;
  }
  {
    ProfScope ps(ctx, MTR_KERNEL_FORWARD);
    if (t.n_fwd > 0) {
      const FwdBatchDesc* d = t.fwd_descs.as<FwdBatchDesc>();
      const long long* f = t.fwd_first.as<long long>();
      cudaError_t e;
      if (t.copy_kind == 1)
        e = launch_forward_batch<__nv_bfloat16>(d, f, t.n_fwd_desc, t.n_fwd, t.fwd_smem, t.fwd_grid, st);
      else if (t.copy_kind == 2)
        e = launch_forward_batch<__half>(d, f, t.n_fwd_desc, t.n_fwd, t.fwd_smem, t.fwd_grid, st);
      else
        e = launch_forward_batch<float>(d, f, t.n_fwd_desc, t.n_fwd, t.fwd_smem, t.fwd_grid, st);
      g_launches.fetch_add(1);
      if (e != cudaSuccess) return cuda_error(ctx, e, "batched forward");
    }
  }
  if (t.n_res > 0) {
    ProfScope ps(ctx, MTR_KERNEL_RESIDUAL);
    launch_residual_batch(t.res_descs.as<ResBatchDesc>(), t.res_first.as<long long>(), t.n_res_desc, t.n_res,
                          t.copy_kind != 0, t.ew_grid, st);
    MTR_CK_LAUNCH(ctx, "batched residual");
  }
  {
    ProfScope ps(ctx, MTR_KERNEL_BACKPROJECT);
    if (t.n_bp > 0) {
      cudaError_t e = launch_backproject_batch(t.bp_descs.as<BpBatchDesc>(), t.bp_first.as<long long>(), t.n_bp_desc,
                                               t.n_bp, t.bp_smem, t.bp_grid, err, st);
      g_launches.fetch_add(1);
      if (e != cudaSuccess) return cuda_error(ctx, e, "batched back-projection");
    }
  }
  return MTR_OK;  // (fj joins the side streams)
}

struct mtr_batch {
  mtr_context* ctx = nullptr;
  mtr_params p{};
  std::vector<mtr_recon*> rec;
  SirtTables sirt;
  DevBuf mace_descs, mace_first;
  int n_mace_desc = 0;
  long long n_mace = 0;
  DevBuf err;
  cudaGraphExec_t graph = nullptr;
  long long graph_nodes = 0;
  long long voxel_updates = 0;
  ~mtr_batch() {
    if (graph) cudaGraphExecDestroy(graph);
    for (mtr_recon* r : rec) mtr_recon_destroy(r);
  }
};

namespace {

mtr_status build_mace_table(mtr_batch* b) {
  mtr_context* ctx = b->ctx;
  const int ck = copy_kind_of(b->p.precision);
  std::vector<MaceBatchDesc> maced;
  std::vector<long long> count, cost;
  for (mtr_recon* r : b->rec) {
    MaceBatchDesc md{};
    md.K = r->K;
    md.w_half = ck != 0;  // mixed precision keeps the MACE states as FP16 deviations
    for (int k = 0; k < r->K; ++k) {
      md.w[k] = r->ax[k].w.p;
      md.x[k] = r->ax[k].x.as<float>();
      md.xc[k] = r->ax[k].xcopy.p;
    }
    md.wavg = r->wavg.as<float>();
    md.n = r->nv;
    md.rho = r->p.mace_step;
    md.copy_kind = ck;
    maced.push_back(md);
    count.push_back((r->nv + kBatchChunk - 1) / kBatchChunk);
    cost.push_back(r->K);
  }
  const std::vector<long long> first = order_by_cost(maced, count, cost);
  b->n_mace_desc = (int)maced.size();
  b->n_mace = first.back();
  mtr_status s = upload_grow(ctx, b->mace_descs, maced);
  if (s == MTR_OK) s = upload_grow(ctx, b->mace_first, first);
  if (s != MTR_OK) return s;
  MTR_CK(ctx, cudaStreamSynchronize(ctx->stream));
  return MTR_OK;
}

mtr_status enqueue_batch(mtr_batch* b) {
  mtr_context* ctx = b->ctx;
  cudaStream_t st = ctx->stream;
  MTR_CK(ctx, cudaMemsetAsync(b->err.p, 0, sizeof(int), st));
  // WBP initialisation of every instance: independent arrays, so the
  // instances go round-robin onto up to 8 side streams forked from the
  // context stream and joined back (serial when per-kernel profiling is on).
  constexpr int kSides = 8;
  const bool par = b->rec.size() > 1 && !ctx->profiling;
  const int sides = par ? std::min<int>(kSides, (int)b->rec.size()) : 0;
  {
    ForkJoin fj(ctx);  // joined back to the context stream on every exit path
    if (par) {
      const mtr_status s = fj.fork(sides);
      if (s != MTR_OK) return s;
    }
    for (size_t i = 0; i < b->rec.size(); ++i) {
      if (par) fj.use((int)(i % (size_t)sides));
      const mtr_status s = recon_enqueue_init(b->rec[i]);
      fj.use(-1);
      if (s != MTR_OK) return s;
    }
  }
  for (int it = 0; it < b->p.iter_times; ++it) {
    for (int j = 0; j < b->p.sirt_inner; ++j) {
      mtr_status s = enqueue_sirt_iteration(ctx, b->sirt, b->err.as<int>());
      if (s != MTR_OK) return s;
    }
    ProfScope ps(ctx, MTR_KERNEL_MACE);
    launch_mace_batch(b->mace_descs.as<MaceBatchDesc>(), b->mace_first.as<long long>(), b->n_mace_desc, b->n_mace,
                      ctx->num_sms * 8, st);
    MTR_CK_LAUNCH(ctx, "batched mace");
  }
  return MTR_OK;
}

}  // namespace

extern "C" {

mtr_status mtr_batch_create(mtr_context* ctx, int n, const mtr_instance* inst, const mtr_params* params, int mem_kind,
                            mtr_batch** out) {
  if (!ctx || !inst || !params || !out || n <= 0) return set_error(ctx, MTR_ERR_INVALID_ARGUMENT, "invalid argument");
  *out = nullptr;
  // The batch API has no upload call: every axis of every instance must bring
  // its projections.
  for (int i = 0; i < n; ++i) {
    if (!inst[i].axes || inst[i].n_axes <= 0 || inst[i].n_axes > MTR_MAX_AXES)
      return set_error(ctx, MTR_ERR_INVALID_ARGUMENT, "instance: null axes or axis count out of range");
    for (int k = 0; k < inst[i].n_axes; ++k) {
      const mtr_status sa = check_axis(ctx, inst[i].axes[k], true);
      if (sa != MTR_OK) return sa;
    }
  }
  DeviceGuard g(ctx->device);
  std::unique_ptr<mtr_batch> b(new (std::nothrow) mtr_batch());
  if (!b) return set_error(ctx, MTR_ERR_OUT_OF_MEMORY, "host allocation");
  b->ctx = ctx;
  b->p = *params;
  mtr_params rp = *params;
  rp.flags = params->flags & MTR_FLAG_HOST_VOLUMES;  // the batch captures its own graph; no norm records
  for (int i = 0; i < n; ++i) {
    mtr_recon* r = nullptr;
    mtr_status s = mtr_recon_create(ctx, inst[i].n_axes, inst[i].axes, inst[i].vol, &rp, mem_kind, &r);
    if (s != MTR_OK) return s;
    b->rec.push_back(r);
    b->voxel_updates += r->nv * r->K * (long long)params->iter_times * params->sirt_inner;
  }
  MTR_CK(ctx, b->err.alloc(sizeof(int)));
  mtr_status s = build_sirt_tables(ctx, b->rec, params->precision, b->sirt);
  if (s == MTR_OK) s = build_mace_table(b.get());
  if (s != MTR_OK) return s;
  *out = b.release();
  return MTR_OK;
}

mtr_status mtr_batch_run(mtr_batch* b) {
  if (!b) return MTR_ERR_INVALID_ARGUMENT;
  mtr_context* ctx = b->ctx;
  DeviceGuard g(ctx->device);
  if (!(b->p.flags & MTR_FLAG_GRAPH)) return enqueue_batch(b);
  if (!b->graph) {
    cudaGraph_t graph = nullptr;
    MTR_CK(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    const long long before = g_launches.load();
    mtr_status s = enqueue_batch(b);
    const long long nodes = g_launches.load() - before;
    g_launches.fetch_sub(nodes);
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &graph);
    if (s != MTR_OK) {
      if (graph) cudaGraphDestroy(graph);
      return s;
    }
    if (e != cudaSuccess) return cuda_error(ctx, e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&b->graph, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
      b->graph = nullptr;
      return cuda_error(ctx, e, "cudaGraphInstantiate");
    }
    b->graph_nodes = nodes;
  }
  MTR_CK(ctx, cudaGraphLaunch(b->graph, ctx->stream));
  g_launches.fetch_add(b->graph_nodes);
  return MTR_OK;
}

mtr_status mtr_batch_download(mtr_batch* b, int i, float* out, int mem_kind) {
  if (!b || i < 0 || i >= (int)b->rec.size()) return MTR_ERR_INVALID_ARGUMENT;
  mtr_status s = mtr_recon_download(b->rec[i], out, mem_kind);
  if (s != MTR_OK || mem_kind == MTR_MEM_DEVICE) return s;
  int flag = 0;
  MTR_CK(b->ctx, cudaMemcpy(&flag, b->err.p, sizeof(int), cudaMemcpyDeviceToHost));
  if (flag) return set_error(b->ctx, MTR_ERR_TIMEOUT, "a batched kernel gave up on a bounded wait");
  return MTR_OK;
}

mtr_status mtr_batch_info(const mtr_batch* b, long long* voxel_updates_per_run, long long* device_bytes,
                          long long* work_items) {
  if (!b) return MTR_ERR_INVALID_ARGUMENT;
  if (voxel_updates_per_run) *voxel_updates_per_run = b->voxel_updates;
  if (device_bytes) {
    long long t = 0;
    for (const mtr_recon* r : b->rec) t += r->bytes;
    *device_bytes = t;
  }
  if (work_items) {
    work_items[0] = b->sirt.n_fwd;
    work_items[1] = b->sirt.n_res;
    work_items[2] = b->sirt.n_bp;
    work_items[3] = b->n_mace;
    work_items[4] = (long long)b->sirt.own.size();
  }
  return MTR_OK;
}

mtr_status mtr_batch_destroy(mtr_batch* b) {
  if (!b) return MTR_OK;
  DeviceGuard g(b->ctx->device);
  cudaStreamSynchronize(b->ctx->stream);
  delete b;
  return MTR_OK;
}

}  // extern "C"
