// Batched reconstruction of many tilt series of uneven size and axis count.
//
// Each instance is an mtr_recon (its own buffers, WBP init and MACE state).
// The SIRT phases of all instances run together: per phase ONE persistent
// launch whose CTAs (a grid sized to the GPU's resident capacity) loop over a
// cost-ordered work list covering every instance and axis:
//   forward splat   item = (axis, brick)          fwd_batch_kernel
//   residual        item = (axis, 64 Ki pixels)   residual_batch_kernel
//   back-projection item = (axis, brick)          bp_batch_kernel
//   MACE consensus  item = (instance, 64 Ki voxels) mace_batch_kernel
// so small instances no longer leave SMs idle.  The whole schedule (WBP init
// of every instance, n_outer x n_inner SIRT phases, MACE steps) is captured
// once into a CUDA graph and replayed.  An axis whose detector window does
// not fit a TMA box falls back to its own plain kernels inside the same
// phase.  Work lists and tensor maps live in device memory, built once.
#include <algorithm>
#include <memory>
#include <new>
#include <numeric>
#include <vector>

#include "mtr_internal.h"
#include "mtr_runtime.h"

using namespace mtr;

struct mtr_batch {
  mtr_context* ctx = nullptr;
  mtr_params p{};
  std::vector<mtr_recon*> rec;
  DevBuf maps;  // CUtensorMap per batched axis: [2j] residual (bp), [2j+1] ray sums (fwd)
  DevBuf bp_descs, fwd_descs, res_descs, mace_descs;
  DevBuf bp_items, fwd_items, res_items, mace_items;
  long long n_bp = 0, n_fwd = 0, n_res = 0, n_mace = 0;
  size_t bp_smem = 0, fwd_smem = 0;
  int bp_grid = 0, fwd_grid = 0, ew_grid = 0;
  std::vector<std::pair<int, int>> bp_fallback, fwd_fallback;  // (instance, axis) run with their own kernels
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

int copy_kind_of(int precision) {
  return precision == MTR_PREC_MIXED_BF16 ? 1 : precision == MTR_PREC_MIXED_FP16 ? 2 : 0;
}

template <typename T>
mtr_status upload(mtr_context* ctx, DevBuf& buf, const std::vector<T>& v) {
  if (v.empty()) return MTR_OK;
  MTR_CK(ctx, buf.alloc(sizeof(T) * v.size()));
  MTR_CK(ctx, cudaMemcpyAsync(buf.p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, ctx->stream));
  return MTR_OK;
}

// Items of all axes, ordered by decreasing per-item cost (angle count).
std::vector<int2> order_items(const std::vector<long long>& counts, const std::vector<int>& cost) {
  std::vector<int> idx(counts.size());
  std::iota(idx.begin(), idx.end(), 0);
  std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return cost[a] > cost[b]; });
  std::vector<int2> items;
  for (int d : idx)
    for (long long i = 0; i < counts[d]; ++i) items.push_back(make_int2(d, (int)i));
  return items;
}

mtr_status build_work(mtr_batch* b) {
  mtr_context* ctx = b->ctx;
  const int ck = copy_kind_of(b->p.precision);
  std::vector<CUtensorMap> maps;
  std::vector<BpBatchDesc> bpd;
  std::vector<FwdBatchDesc> fwd;
  std::vector<ResBatchDesc> resd;
  std::vector<MaceBatchDesc> maced;
  std::vector<long long> bp_count, fwd_count, res_count, mace_count;
  std::vector<int> bp_cost, fwd_cost, res_cost, mace_cost;
  std::vector<int> bp_map, fwd_map;  // index of each descriptor's tensor map in `maps`
  for (size_t i = 0; i < b->rec.size(); ++i) {
    mtr_recon* r = b->rec[i];
    const VolDev& v = r->vol;
    MaceBatchDesc md{};
    md.K = r->K;
    for (int k = 0; k < r->K; ++k) {
      AxisState& a = r->ax[k];
      md.w[k] = a.w.as<float>();
      md.x[k] = a.x.as<float>();
      md.xc[k] = a.xcopy.p;
      resd.push_back(ResBatchDesc{a.b.p, a.s.as<float>(), a.cf.as<float>(), a.r.as<float>(), a.np});
      res_count.push_back((a.np + kBatchChunk - 1) / kBatchChunk);
      res_cost.push_back(1);
      // back-projection at the batch depth, lane axis as tuned for this axis
      const int bp_lane = a.tma ? (a.plan.lane_y ? 1 : 0) : -1;
      BpPlan bp = plan_backproject(a.hxc, a.hyc, a.A, false, kBatchBpNZ, bp_lane);
      CUtensorMap mr{}, ms{};
      const bool bp_ok = !tma_disabled() && bp.ok &&
                         encode_tensor_map_3d(&mr, a.r.p, false, a.PX, a.pitch, a.PY, a.A, bp.WX, bp.WY);
      const int fwd_lane = a.ftma ? (a.fplan.lane_y ? 1 : 0) : -1;
      FwdPlan fp = plan_forward(a.hxc, a.hyc, a.A, a.PX, a.PY, a.pitch, kBatchFwdNZ, fwd_lane);
      const bool fwd_ok = !tma_disabled() && fp.ok && fp.nz == kBatchFwdNZ &&
                          encode_tensor_map_3d(&ms, a.s.p, false, a.pitch, a.pitch, a.PY, a.A, fp.WX, fp.WY);
      const int j = (int)maps.size() / 2;
      maps.push_back(mr);
      maps.push_back(ms);
      if (bp_ok) {
        BpBatchDesc d{};
        d.ax = a.dev();
        d.vol = v;
        d.WX = bp.WX; d.WY = bp.WY; d.align = bp.align;
        const int BX = bp.lane_y ? 8 : 32, BY = bp.lane_y ? 32 : 8;
        d.gx = (v.NX + BX - 1) / BX;
        d.gy = (v.NY + BY - 1) / BY;
        d.lane_y = bp.lane_y; d.bz0 = bp.bz0;
        d.step = b->p.sirt_step;
        d.vol_out = a.x.as<float>();
        d.cbp = a.cbp.as<float>();
        d.vol_copy = a.xcopy.p;
        d.copy_kind = ck;
        d.map = nullptr;  // set after the maps are uploaded
        bpd.push_back(d);
        bp_map.push_back(2 * j);
        bp_count.push_back((long long)d.gx * d.gy * ((v.NZ + kBatchBpNZ - 1) / kBatchBpNZ));
        bp_cost.push_back(a.A);
        b->bp_smem = std::max(b->bp_smem, bp.smem);
      } else {
        b->bp_fallback.push_back({(int)i, k});
      }
      if (fwd_ok) {
        FwdBatchDesc d{};
        d.ax = a.dev();
        d.vol = v;
        d.WX = fp.WX; d.WY = fp.WY; d.mass_shift = fp.mass_shift;
        const int BX = fp.lane_y ? 8 : 32, BY = fp.lane_y ? 32 : 8;
        d.gx = (v.NX + BX - 1) / BX;
        d.gy = (v.NY + BY - 1) / BY;
        d.lane_y = fp.lane_y; d.bz0 = fp.bz0;
        d.x = ck ? a.xcopy.p : a.x.p;
        d.map = nullptr;
        fwd.push_back(d);
        fwd_map.push_back(2 * j + 1);
        fwd_count.push_back((long long)d.gx * d.gy * ((v.NZ + kBatchFwdNZ - 1) / kBatchFwdNZ));
        fwd_cost.push_back(a.A);
        b->fwd_smem = std::max(b->fwd_smem, fp.smem);
      } else {
        b->fwd_fallback.push_back({(int)i, k});
      }
    }
    md.wavg = r->wavg.as<float>();
    md.n = r->nv;
    md.rho = b->p.mace_step;
    md.copy_kind = ck;
    maced.push_back(md);
    mace_count.push_back((r->nv + kBatchChunk - 1) / kBatchChunk);
    mace_cost.push_back(r->K);
  }
  mtr_status s = upload(ctx, b->maps, maps);
  if (s != MTR_OK) return s;
  const CUtensorMap* base = b->maps.as<CUtensorMap>();
  for (size_t q = 0; q < bpd.size(); ++q) bpd[q].map = base + bp_map[q];
  for (size_t q = 0; q < fwd.size(); ++q) fwd[q].map = base + fwd_map[q];
  const std::vector<int2> bpi = order_items(bp_count, bp_cost), fwi = order_items(fwd_count, fwd_cost);
  const std::vector<int2> rei = order_items(res_count, res_cost), mai = order_items(mace_count, mace_cost);
  b->n_bp = (long long)bpi.size();
  b->n_fwd = (long long)fwi.size();
  b->n_res = (long long)rei.size();
  b->n_mace = (long long)mai.size();
  if ((s = upload(ctx, b->bp_descs, bpd)) != MTR_OK || (s = upload(ctx, b->fwd_descs, fwd)) != MTR_OK ||
      (s = upload(ctx, b->res_descs, resd)) != MTR_OK || (s = upload(ctx, b->mace_descs, maced)) != MTR_OK ||
      (s = upload(ctx, b->bp_items, bpi)) != MTR_OK || (s = upload(ctx, b->fwd_items, fwi)) != MTR_OK ||
      (s = upload(ctx, b->res_items, rei)) != MTR_OK || (s = upload(ctx, b->mace_items, mai)) != MTR_OK)
    return s;
  const int sms = ctx->num_sms;
  b->bp_grid = (int)std::min<long long>(b->n_bp, (long long)sms * backproject_batch_ctas_per_sm(b->bp_smem));
  int fwd_per_sm = 1;
  if (ck == 1) fwd_per_sm = forward_batch_ctas_per_sm<__nv_bfloat16>(b->fwd_smem);
  else if (ck == 2) fwd_per_sm = forward_batch_ctas_per_sm<__half>(b->fwd_smem);
  else fwd_per_sm = forward_batch_ctas_per_sm<float>(b->fwd_smem);
  b->fwd_grid = (int)std::min<long long>(b->n_fwd, (long long)sms * fwd_per_sm);
  b->ew_grid = sms * 8;
  MTR_CK(ctx, cudaStreamSynchronize(ctx->stream));
  return MTR_OK;
}

mtr_status enqueue_batch(mtr_batch* b) {
  mtr_context* ctx = b->ctx;
  cudaStream_t st = ctx->stream;
  const int ck = copy_kind_of(b->p.precision);
  MTR_CK(ctx, cudaMemsetAsync(b->err.p, 0, sizeof(int), st));
  for (mtr_recon* r : b->rec) {
    mtr_status s = recon_enqueue_init(r);
    if (s != MTR_OK) return s;
  }
  for (int it = 0; it < b->p.iter_times; ++it) {
    for (int j = 0; j < b->p.sirt_inner; ++j) {
      {
        ProfScope ps(ctx, MTR_KERNEL_FORWARD);
        if (b->n_fwd > 0) {
          cudaError_t e;
          if (ck == 1)
            e = launch_forward_batch<__nv_bfloat16>(b->fwd_descs.as<FwdBatchDesc>(), b->fwd_items.as<int2>(),
                                                    b->n_fwd, b->fwd_smem, b->fwd_grid, st);
          else if (ck == 2)
            e = launch_forward_batch<__half>(b->fwd_descs.as<FwdBatchDesc>(), b->fwd_items.as<int2>(), b->n_fwd,
                                             b->fwd_smem, b->fwd_grid, st);
          else
            e = launch_forward_batch<float>(b->fwd_descs.as<FwdBatchDesc>(), b->fwd_items.as<int2>(), b->n_fwd,
                                            b->fwd_smem, b->fwd_grid, st);
          g_launches.fetch_add(1);
          if (e != cudaSuccess) return cuda_error(ctx, e, "batched forward");
        }
      }
      for (auto& f : b->fwd_fallback) {
        mtr_status s = recon_enqueue_forward(b->rec[f.first], f.second);
        if (s != MTR_OK) return s;
      }
      {
        ProfScope ps(ctx, MTR_KERNEL_RESIDUAL);
        launch_residual_batch(b->res_descs.as<ResBatchDesc>(), b->res_items.as<int2>(), b->n_res, ck != 0,
                              b->ew_grid, st);
        MTR_CK_LAUNCH(ctx, "batched residual");
      }
      {
        ProfScope ps(ctx, MTR_KERNEL_BACKPROJECT);
        if (b->n_bp > 0) {
          cudaError_t e = launch_backproject_batch(b->bp_descs.as<BpBatchDesc>(), b->bp_items.as<int2>(), b->n_bp,
                                                   b->bp_smem, b->bp_grid, b->err.as<int>(), st);
          g_launches.fetch_add(1);
          if (e != cudaSuccess) return cuda_error(ctx, e, "batched back-projection");
        }
      }
      for (auto& f : b->bp_fallback) {
        mtr_status s = recon_enqueue_sirt_bp(b->rec[f.first], f.second);
        if (s != MTR_OK) return s;
      }
    }
    ProfScope ps(ctx, MTR_KERNEL_MACE);
    launch_mace_batch(b->mace_descs.as<MaceBatchDesc>(), b->mace_items.as<int2>(), b->n_mace, b->ew_grid, st);
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
  DeviceGuard g(ctx->device);
  std::unique_ptr<mtr_batch> b(new (std::nothrow) mtr_batch());
  if (!b) return set_error(ctx, MTR_ERR_OUT_OF_MEMORY, "host allocation");
  b->ctx = ctx;
  b->p = *params;
  mtr_params rp = *params;
  rp.flags = 0;  // the batch captures its own graph; no norm records
  for (int i = 0; i < n; ++i) {
    mtr_recon* r = nullptr;
    mtr_status s = mtr_recon_create(ctx, inst[i].n_axes, inst[i].axes, inst[i].vol, &rp, mem_kind, &r);
    if (s != MTR_OK) return s;
    b->rec.push_back(r);
    b->voxel_updates += r->nv * r->K * (long long)params->iter_times * params->sirt_inner;
  }
  MTR_CK(ctx, b->err.alloc(sizeof(int)));
  mtr_status s = build_work(b.get());
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
    work_items[0] = b->n_fwd;
    work_items[1] = b->n_res;
    work_items[2] = b->n_bp;
    work_items[3] = b->n_mace;
    work_items[4] = (long long)(b->fwd_fallback.size() + b->bp_fallback.size());
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
