// Device-resident multi-axis reconstruction (WBP init -> SIRT -> MACE) and the
// C ABI entry points that replace the reference's host functions.
//
// Reference flow being replaced (one MPI rank per GPU, host round trips):
//   ComputeInitialModel + Gatherv/Reduce  (FunctionOnGPU.cu:138-179, MultiAxis.cpp:172-200)
//   reconstructModel                      (MultiAxis.cpp:40-71)
//     initialZdata, Scatterv, runSIRTOnGPU, Gatherv, runMaceOnCPU, Reduce/Bcast
// Here every array stays in HBM for the whole run; each SIRT iteration is
// three launches per axis (forward splat, residual, back-projection update)
// and each MACE iteration ends with one fused launch over all axes.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include "mtr_internal.h"
#include "mtr_runtime.h"

using namespace mtr;

mtr_recon::~mtr_recon() {
  if (graph) cudaGraphExecDestroy(graph);
}

namespace {

int copy_kind_of(int precision) {
  if (precision == MTR_PREC_MIXED_BF16) return 1;
  if (precision == MTR_PREC_MIXED_FP16) return 2;
  return 0;
}

bool mixed(int precision) { return precision != MTR_PREC_FP32; }

// Bytes of the residual array of an axis: room for the FP32 residual and for
// its pair form (8 bytes per pixel plus one column), whichever the axis' back-
// projection reads.
long long residual_bytes(int PX, int PY, int A) {
  return std::max((long long)projection_pitch(PX) * PY * A * 4, (long long)pair_pitch(PX) * PY * A * 8);
}

// Bytes per voxel of an axis' MACE state w_k: FP32, or in mixed precision its
// FP16 deviation from the FP32 consensus (it changes once per outer
// iteration; the SIRT iterate x_k, which accumulates an update every
// iteration, stays FP32).
long long state_bytes(int precision) { return mixed(precision) ? 2 : 4; }

long long axis_bytes(long long np, long long r_bytes, long long nv, int precision) {
  const long long pe = mixed(precision) ? 2 : 4;
  long long b = 0;
  b += np * pe;       // b
  b += np * 4;        // s
  b += np * 4;        // cf
  b += r_bytes;       // r (FP32 values in every mode: the back-projection reads them per tap)
  b += nv * 4 * 2;    // cbp, x
  b += nv * state_bytes(precision);   // w
  if (mixed(precision)) b += nv * 2;  // xcopy
  return b;
}

// w_k = v (FP32 on the device): copied, or in mixed precision stored as
// fp16(v - w_avg) against the consensus already in r->wavg.
mtr_status set_state(mtr_recon* r, AxisState& a, const float* v, cudaStream_t st) {
  if (!mixed(r->p.precision)) {
    MTR_CK(r->ctx, cudaMemcpyAsync(a.w.p, v, (size_t)r->nv * 4, cudaMemcpyDefault, st));
    return MTR_OK;
  }
  launch_state_dev(v, r->wavg.as<float>(), a.w.as<__half>(), r->nv, st);
  MTR_CK_LAUNCH(r->ctx, "state copy");
  return MTR_OK;
}

// FP32 value of axis k's state into `out` (device or mapped memory).
mtr_status state_value(mtr_recon* r, int k, float* out, cudaStream_t st) {
  if (!mixed(r->p.precision)) {
    MTR_CK(r->ctx, cudaMemcpyAsync(out, r->ax[k].w.p, (size_t)r->nv * 4, cudaMemcpyDefault, st));
    return MTR_OK;
  }
  launch_state_value(r->ax[k].w.as<__half>(), r->wavg.as<float>(), out, r->nv, st);
  MTR_CK_LAUNCH(r->ctx, "state value");
  return MTR_OK;
}

mtr_status check_params(mtr_context* ctx, const mtr_params& p) {
  if (p.iter_times < 0 || p.sirt_inner < 0) return set_error(ctx, MTR_ERR_INVALID_ARGUMENT, "negative iteration count");
  if (p.precision < MTR_PREC_FP32 || p.precision > MTR_PREC_MIXED_FP16)
    return set_error(ctx, MTR_ERR_INVALID_ARGUMENT, "unknown precision");
  if (!std::isfinite(p.sirt_step) || !std::isfinite(p.mace_step))
    return set_error(ctx, MTR_ERR_INVALID_ARGUMENT, "non-finite step");
  return MTR_OK;
}

// Projections [A][PY][PX] (caller layout) -> device [A][PY][pitch], padding zero.
mtr_status upload_projections(mtr_recon* r, int k, const float* data, int mem_kind) {
  mtr_context* ctx = r->ctx;
  AxisState& a = r->ax[k];
  const size_t fbytes = (size_t)a.np * sizeof(float);
  const cudaMemcpyKind kind = mem_kind == MTR_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  float* dst = mixed(r->p.precision) ? a.s.as<float>() : a.b.as<float>();
  if (a.pitch != a.PX) MTR_CK(ctx, cudaMemsetAsync(dst, 0, fbytes, ctx->stream));
  MTR_CK(ctx, cudaMemcpy2DAsync(dst, (size_t)a.pitch * 4, data, (size_t)a.PX * 4, (size_t)a.PX * 4,
                                (size_t)a.PY * a.A, kind, ctx->stream));
  if (!mixed(r->p.precision)) return MTR_OK;
  // Mixed: staged as float in the forward accumulator, converted to fp16.
  launch_convert_copy(a.s.as<float>(), a.b.p, 2, a.np, ctx->stream);
  MTR_CK_LAUNCH(ctx, "convert projections");
  MTR_CK(ctx, cudaMemsetAsync(a.s.p, 0, fbytes, ctx->stream));
  return MTR_OK;
}

// FP16 projections [A][PY][PX] (caller layout).  Mixed precision stores
// projections as FP16: they go straight into b.  The FP32 path stages them in
// the forward accumulator and widens them into b.
mtr_status upload_projections_half(mtr_recon* r, int k, const void* data, int mem_kind) {
  mtr_context* ctx = r->ctx;
  AxisState& a = r->ax[k];
  const cudaMemcpyKind kind = mem_kind == MTR_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  __half* dst = mixed(r->p.precision) ? a.b.as<__half>() : a.s.as<__half>();
  if (a.pitch != a.PX) MTR_CK(ctx, cudaMemsetAsync(dst, 0, (size_t)a.np * sizeof(__half), ctx->stream));
  MTR_CK(ctx, cudaMemcpy2DAsync(dst, (size_t)a.pitch * sizeof(__half), data, (size_t)a.PX * sizeof(__half),
                                (size_t)a.PX * sizeof(__half), (size_t)a.PY * a.A, kind, ctx->stream));
  if (mixed(r->p.precision)) return MTR_OK;
  launch_widen(a.s.as<__half>(), a.b.as<float>(), a.np, ctx->stream);
  MTR_CK_LAUNCH(ctx, "widen projections");
  MTR_CK(ctx, cudaMemsetAsync(a.s.p, 0, (size_t)a.np * 4, ctx->stream));
  return MTR_OK;
}

// Geometry-only arrays: forward row sums cf = A 1.  (cbp is produced by WBP.)
mtr_status enqueue_geometry(mtr_recon* r) {
  mtr_context* ctx = r->ctx;
  const VolDev& v = r->vol;
  for (auto& a : r->ax) {
    MTR_CK(ctx, cudaMemsetAsync(a.cf.p, 0, (size_t)a.np * 4, ctx->stream));
    ProfScope ps(ctx, MTR_KERNEL_OTHER);
    if (a.ftma) {
      cudaError_t e = launch_forward_tma<float>(a.map_cf, a.fplan, a.dev(), v, nullptr, v.Zs, v.Zs + v.NZ,
                                                r->err.as<int>(), ctx->stream);
      g_launches.fetch_add(1);
      if (e != cudaSuccess) return cuda_error(ctx, e, "forward row sums (tma)");
      continue;
    }
    launch_forward<float>(a.dev(), v, nullptr, a.cf.as<float>(), v.Zs, v.Zs + v.NZ, ctx->stream);
    MTR_CK_LAUNCH(ctx, "forward row sums");
  }
  return MTR_OK;
}

VolSpan whole_volume(const mtr_recon* r, AxisState& a) {
  return VolSpan{r->vol.Zs, r->vol.Zs + r->vol.NZ, a.x.as<float>(), a.cbp.as<float>(), a.xcopy.p};
}

mtr_status enqueue_forward(mtr_recon* r, AxisState& a, const VolSpan& sp) {
  mtr_context* ctx = r->ctx;
  const VolDev& v = r->vol;
  const int z0 = sp.z0, z1 = sp.z1;
  ProfScope ps(ctx, MTR_KERNEL_FORWARD);
  if (a.ftma) {
    cudaError_t e;
    switch (copy_kind_of(r->p.precision)) {
      case 1: e = launch_forward_tma<__nv_bfloat16>(a.map_s, a.fplan, a.dev(), v,
                                                     static_cast<const __nv_bfloat16*>(sp.xcopy), z0, z1,
                                                     r->err.as<int>(), ctx->stream); break;
      case 2: e = launch_forward_tma<__half>(a.map_s, a.fplan, a.dev(), v, static_cast<const __half*>(sp.xcopy), z0,
                                              z1, r->err.as<int>(), ctx->stream); break;
      default: e = launch_forward_tma<float>(a.map_s, a.fplan, a.dev(), v, sp.x, z0, z1, r->err.as<int>(),
                                              ctx->stream); break;
    }
    g_launches.fetch_add(1);
    if (e != cudaSuccess) return cuda_error(ctx, e, "forward splat (tma)");
    return MTR_OK;
  }
  switch (copy_kind_of(r->p.precision)) {
    case 1: launch_forward<__nv_bfloat16>(a.dev(), v, static_cast<const __nv_bfloat16*>(sp.xcopy), a.s.as<float>(),
                                          z0, z1, ctx->stream); break;
    case 2: launch_forward<__half>(a.dev(), v, static_cast<const __half*>(sp.xcopy), a.s.as<float>(), z0, z1,
                                   ctx->stream); break;
    default: launch_forward<float>(a.dev(), v, sp.x, a.s.as<float>(), z0, z1, ctx->stream); break;
  }
  MTR_CK_LAUNCH(ctx, "forward splat");
  return MTR_OK;
}
mtr_status enqueue_forward(mtr_recon* r, AxisState& a) { return enqueue_forward(r, a, whole_volume(r, a)); }

mtr_status enqueue_residual(mtr_recon* r, AxisState& a, double* norm) {
  mtr_context* ctx = r->ctx;
  ProfScope ps(ctx, MTR_KERNEL_RESIDUAL);
  const long long rows = (long long)a.A * a.PY;
  if (a.tma && a.plan.pairs) {  // this axis' windowed update reads (value, next - value) pairs
    if (mixed(r->p.precision))
      launch_residual_pairs<__half>(rows, a.pitch, a.pitch2, a.b.as<__half>(), a.s.as<float>(), a.cf.as<float>(),
                                    a.r.as<float>(), a.plan.half ? 2 : a.plan.planar ? 1 : 0, norm, ctx->stream);
    else
      launch_residual_pairs<float>(rows, a.pitch, a.pitch2, a.b.as<float>(), a.s.as<float>(), a.cf.as<float>(),
                                   a.r.as<float>(), a.plan.planar ? 1 : 0, norm, ctx->stream);
  } else if (mixed(r->p.precision)) {
    launch_residual<__half, float>(a.np, a.b.as<__half>(), a.s.as<float>(), a.cf.as<float>(), a.r.as<float>(), norm,
                                   ctx->stream);
  } else {
    launch_residual<float, float>(a.np, a.b.as<float>(), a.s.as<float>(), a.cf.as<float>(), a.r.as<float>(), norm,
                                  ctx->stream);
  }
  MTR_CK_LAUNCH(ctx, "residual");
  return MTR_OK;
}

// Mixed precision: the windowed WBP gathers FP32 windows, so the FP16
// projections are first widened into r (free until the first residual).
mtr_status enqueue_widen_for_wbp(mtr_recon* r, AxisState& a) {
  if (!(a.tma_b && mixed(r->p.precision))) return MTR_OK;
  launch_widen(a.b.as<__half>(), a.r.as<float>(), a.np, r->ctx->stream);
  MTR_CK_LAUNCH(r->ctx, "widen projections");
  return MTR_OK;
}

// mode 0: WBP (x = s/c, cbp = c); mode 1: SIRT update from the residual.
// widen: for the windowed mixed-precision WBP, widen the projections first
// (a caller that runs several WBP spans of one axis widens them once).
mtr_status enqueue_bp(mtr_recon* r, AxisState& a, int mode, const VolSpan& sp, bool widen = true) {
  mtr_context* ctx = r->ctx;
  const VolDev& v = r->vol;
  const int z0 = sp.z0, z1 = sp.z1;
  const int ck = copy_kind_of(r->p.precision);
  ProfScope ps(ctx, mode == 0 ? MTR_KERNEL_WBP : MTR_KERNEL_BACKPROJECT);
  // WBP reads the projections (fp16 when mixed), SIRT reads the FP32 residual.
  const bool half_img = mode == 0 && mixed(r->p.precision);
  if (mode == 0 ? a.tma_b : a.tma) {
    if (half_img && widen) {
      mtr_status s = enqueue_widen_for_wbp(r, a);
      if (s != MTR_OK) return s;
    }
    cudaError_t e = launch_backproject_tma<float>(mode == 0 ? a.map_b : a.map_r, mode == 0 ? a.plan_b : a.plan,
                                                  a.dev(), v, mode, r->p.sirt_step, sp.x, sp.cbp, sp.xcopy, ck, z0,
                                                  z1, r->err.as<int>(), ctx->stream);
    g_launches.fetch_add(1);
    if (e != cudaSuccess) return cuda_error(ctx, e, "tma back-projection");
    return MTR_OK;
  }
  if (half_img) {
    launch_backproject<__half>(a.dev(), v, a.b.as<__half>(), mode, r->p.sirt_step, sp.x, sp.cbp, sp.xcopy, ck, z0,
                               z1, ctx->stream);
  } else if (mixed(r->p.precision)) {
    launch_backproject<float>(a.dev(), v, a.r.as<float>(), mode, r->p.sirt_step, sp.x, sp.cbp, sp.xcopy, ck, z0, z1,
                              ctx->stream);
  } else {
    const float* img = mode == 0 ? a.b.as<float>() : a.r.as<float>();
    launch_backproject<float>(a.dev(), v, img, mode, r->p.sirt_step, sp.x, sp.cbp, nullptr, 0, z0, z1, ctx->stream);
  }
  MTR_CK_LAUNCH(ctx, mode == 0 ? "wbp" : "sirt back-projection");
  return MTR_OK;
}
mtr_status enqueue_bp(mtr_recon* r, AxisState& a, int mode) { return enqueue_bp(r, a, mode, whole_volume(r, a)); }

}  // namespace

// WBP init: w_avg = sum of per-axis WBPs, w_k = z_k = w_avg (and the
// forward-read copies), norms and change records reset.
mtr_status mtr::recon_enqueue_init(mtr_recon* r) {
  if (r->slabs) return stream_enqueue_init(r);
  mtr_context* ctx = r->ctx;
  const long long nv = r->nv;
  const size_t vbytes = (size_t)nv * 4;
  const int ck = copy_kind_of(r->p.precision);
  float* wavg = r->wavg.as<float>();
  MTR_CK(ctx, cudaMemsetAsync(r->err.p, 0, sizeof(int), ctx->stream));
  // Initial model: sum over axes of each axis' WBP (MultiAxis.cpp:181-200).
  MTR_CK(ctx, cudaMemsetAsync(wavg, 0, vbytes, ctx->stream));
  for (auto& a : r->ax) {
    mtr_status s = enqueue_bp(r, a, 0);
    if (s != MTR_OK) return s;
    ProfScope ps(ctx, MTR_KERNEL_OTHER);
    launch_axpy_acc(wavg, a.x.as<float>(), nv, ctx->stream);
    MTR_CK_LAUNCH(ctx, "initial model sum");
  }
  // w_k = w_avg (in mixed precision a zero deviation); first z_k = 2 w_avg - w_k = w_avg.
  for (auto& a : r->ax) {
    if (mixed(r->p.precision)) {
      MTR_CK(ctx, cudaMemsetAsync(a.w.p, 0, (size_t)nv * 2, ctx->stream));
    } else {
      mtr_status s = set_state(r, a, wavg, ctx->stream);
      if (s != MTR_OK) return s;
    }
    MTR_CK(ctx, cudaMemcpyAsync(a.x.p, wavg, vbytes, cudaMemcpyDefault, ctx->stream));
    if (ck) {
      ProfScope ps(ctx, MTR_KERNEL_OTHER);
      launch_convert_copy(a.x.as<float>(), a.xcopy.p, ck, nv, ctx->stream);
      MTR_CK_LAUNCH(ctx, "volume copy");
    }
  }
  const int K = r->K, ni = r->p.sirt_inner, no = r->p.iter_times;
  double* norms = r->norms.as<double>();
  double* dch = r->dchange.as<double>();
  if (norms) MTR_CK(ctx, cudaMemsetAsync(norms, 0, sizeof(double) * (size_t)no * K * ni, ctx->stream));
  if (dch) MTR_CK(ctx, cudaMemsetAsync(dch, 0, sizeof(double) * 2 * (size_t)std::max(1, no), ctx->stream));
  return MTR_OK;
}

mtr_status mtr::recon_enqueue_forward_span(mtr_recon* r, int k, const VolSpan& sp) {
  return enqueue_forward(r, r->ax[k], sp);
}
mtr_status mtr::recon_enqueue_bp_span(mtr_recon* r, int k, int mode, const VolSpan& sp, bool widen) {
  return enqueue_bp(r, r->ax[k], mode, sp, widen);
}
mtr_status mtr::recon_enqueue_widen(mtr_recon* r, int k) { return enqueue_widen_for_wbp(r, r->ax[k]); }
mtr_status mtr::recon_enqueue_residual_norm(mtr_recon* r, int k, double* norm) {
  return enqueue_residual(r, r->ax[k], norm);
}
double* mtr::recon_norm_slot(mtr_recon* r, int it, int k, int j) {
  double* norms = r->norms.as<double>();
  if (!norms || it >= r->p.iter_times) return nullptr;
  return norms + ((long long)it * r->K + k) * r->p.sirt_inner + j;
}
double* mtr::recon_change_slot(mtr_recon* r, int it) {
  double* dch = r->dchange.as<double>();
  return r->record_changes && dch && it < r->p.iter_times ? dch + 2 * it : nullptr;
}
int mtr::recon_copy_kind(const mtr_recon* r) { return copy_kind_of(r->p.precision); }
mtr_status mtr::recon_enqueue_wbp(mtr_recon* r, int k) { return enqueue_bp(r, r->ax[k], 0); }
mtr_status mtr::recon_enqueue_forward(mtr_recon* r, int k) { return enqueue_forward(r, r->ax[k]); }
mtr_status mtr::recon_enqueue_residual(mtr_recon* r, int k) { return enqueue_residual(r, r->ax[k], nullptr); }
mtr_status mtr::recon_enqueue_sirt_bp(mtr_recon* r, int k) { return enqueue_bp(r, r->ax[k], 1); }

namespace {

// The n_inner SIRT iterations of one axis in outer iteration `it`.
mtr_status enqueue_axis_chain(mtr_recon* r, int k, int it) {
  const int K = r->K, ni = r->p.sirt_inner, no = r->p.iter_times;
  double* norms = r->norms.as<double>();
  AxisState& a = r->ax[k];
  for (int j = 0; j < ni; ++j) {
    mtr_status s = enqueue_forward(r, a);
    if (s != MTR_OK) return s;
    s = enqueue_residual(r, a, norms && it < no ? norms + ((long long)it * K + k) * ni + j : nullptr);
    if (s != MTR_OK) return s;
    s = enqueue_bp(r, a, 1);
    if (s != MTR_OK) return s;
  }
  return MTR_OK;
}

// Axes run their SIRT chains concurrently (each on a side stream, forked
// from and joined back to the context stream) unless MTR_SERIAL_AXES=1 or
// per-kernel profiling is on (concurrent kernels would share their event
// intervals).  The chains touch disjoint buffers until the MACE step.
bool concurrent_axes(const mtr_recon* r) {
  const char* e = std::getenv("MTR_SERIAL_AXES");
  return r->K > 1 && !r->ctx->profiling && !(e && e[0] == '1');
}

// MACE outer iterations [first, first + count): n_inner SIRT iterations of
// every axis, then the MACE step.
mtr_status enqueue_outer(mtr_recon* r, int first, int count) {
  if (r->slabs) return stream_enqueue_outer(r, first, count);
  mtr_context* ctx = r->ctx;
  const int K = r->K;
  const bool par = concurrent_axes(r);
  for (int it = first; it < first + count; ++it) {
    if (!par) {
      for (int k = 0; k < K; ++k) {
        mtr_status s = enqueue_axis_chain(r, k, it);
        if (s != MTR_OK) return s;
      }
    } else {
      ForkJoin fj(ctx);  // every axis' chain on its own side stream, joined on any exit
      mtr_status s = fj.fork(K);
      for (int k = 0; s == MTR_OK && k < K; ++k) {
        fj.use(k);
        s = enqueue_axis_chain(r, k, it);
      }
      if (s != MTR_OK) return s;
    }
    mtr_status st = recon_enqueue_mace(r, it);
    if (st != MTR_OK) return st;
  }
  return MTR_OK;
}

// WBP init, then the MACE loop.
mtr_status enqueue_run(mtr_recon* r) {
  mtr_status st = recon_enqueue_init(r);
  if (st != MTR_OK) return st;
  return enqueue_outer(r, 0, r->p.iter_times);
}

// Checkpoint file: header, then w_avg and w_k of every axis (float32, x fastest).
struct CkptHeader {
  char magic[8];  // "MTRCKPT1"
  int32_t version, K, X, Y, Z, outer_done, precision;
  int64_t reserved;
};
constexpr char kCkptMagic[8] = {'M', 'T', 'R', 'C', 'K', 'P', 'T', '1'};

}  // namespace

// MACE step `it` of a reconstruction (one fused launch over its K axes).
mtr_status mtr::recon_enqueue_mace(mtr_recon* r, int it) {
  mtr_context* ctx = r->ctx;
  const int K = r->K;
  void* ws[MTR_MAX_AXES];
  float* xs[MTR_MAX_AXES];
  void* xcs[MTR_MAX_AXES];
  for (int k = 0; k < K; ++k) {
    ws[k] = r->ax[k].w.p;
    xs[k] = r->ax[k].x.as<float>();
    xcs[k] = r->ax[k].xcopy.p;
  }
  {
    ProfScope ps(ctx, MTR_KERNEL_MACE);
    // the FP64 convergence sums cost five of the step's FP64 operations per
    // voxel: only when a record is kept
    launch_mace(K, ws, mixed(r->p.precision) ? 1 : 0, xs, r->wavg.as<float>(), r->nv, r->p.mace_step, xcs,
                copy_kind_of(r->p.precision), recon_change_slot(r, it), ctx->stream);
  }
  MTR_CK_LAUNCH(ctx, "mace");
  return MTR_OK;
}

extern "C" {

mtr_status mtr_estimate_footprint(int n_axes, const mtr_projection_size* prjs, mtr_volume_size vol, int precision,
                                  long long* bytes) {
  if (!bytes || n_axes <= 0 || !prjs) return MTR_ERR_INVALID_ARGUMENT;
  const long long nv = (long long)vol.X * vol.Y * vol.Z;
  long long b = nv * 4;  // wavg
  for (int k = 0; k < n_axes; ++k) {
    const long long np = (long long)projection_pitch(prjs[k].X) * prjs[k].Y * prjs[k].AngN;
    b += axis_bytes(np, residual_bytes(prjs[k].X, prjs[k].Y, prjs[k].AngN), nv, precision) + 64LL * prjs[k].AngN;
  }
  *bytes = b;
  return MTR_OK;
}

mtr_status mtr_recon_create(mtr_context* ctx, int n_axes, const mtr_axis* axes, mtr_volume_size vol,
                            const mtr_params* params, int mem_kind, mtr_recon** out) {
  if (!ctx || !out || !axes || !params) return set_error(ctx, MTR_ERR_INVALID_ARGUMENT, "null argument");
  *out = nullptr;
  if (n_axes <= 0 || n_axes > MTR_MAX_AXES) return set_error(ctx, MTR_ERR_INVALID_ARGUMENT, "axis count out of range");
  if (mem_kind != MTR_MEM_HOST && mem_kind != MTR_MEM_DEVICE)
    return set_error(ctx, MTR_ERR_INVALID_ARGUMENT, "unknown memory kind");
  mtr_status s = check_volume(ctx, vol);
  if (s != MTR_OK) return s;
  s = check_params(ctx, *params);
  if (s != MTR_OK) return s;
  for (int k = 0; k < n_axes; ++k) {
    s = check_axis(ctx, axes[k], false);  // null data: uploaded later
    if (s != MTR_OK) return s;
  }
  DeviceGuard g(ctx->device);
  std::unique_ptr<mtr_recon> r(new (std::nothrow) mtr_recon());
  if (!r) return set_error(ctx, MTR_ERR_OUT_OF_MEMORY, "host allocation");
  // On a failed create, the work already enqueued on the arrays ends before
  // they go back to the pool (this guard is destroyed before `r`).
  struct SyncOnFailure {
    mtr_context* c;
    const std::unique_ptr<mtr_recon>& r;
    ~SyncOnFailure() {
      if (r) cudaStreamSynchronize(c->stream);
    }
  } sync_on_failure{ctx, r};
  r->ctx = ctx;
  r->vs = vol;
  r->vol = VolDev{vol.Xstart, vol.Ystart, vol.Zstart, vol.X, vol.Y, vol.Z};
  r->p = *params;
  r->K = n_axes;
  r->nv = (long long)vol.X * vol.Y * vol.Z;
  r->record_changes = (params->flags & MTR_FLAG_RECORD_CHANGES) != 0;
  r->ax.resize(n_axes);
  const bool mx = mixed(params->precision);
  const size_t vb = (size_t)r->nv * 4;
  // volume arrays in mapped host memory (MTR_FLAG_HOST_VOLUMES) or in HBM
  // (streamed slabs keep them in host memory too, and a device working set)
  const bool streamed = (params->flags & MTR_FLAG_STREAM_SLABS) != 0;
  const bool hv = streamed || (params->flags & MTR_FLAG_HOST_VOLUMES) != 0;
  MTR_CK(ctx, r->wavg.alloc_where(vb, hv, ctx));
  MTR_CK(ctx, r->err.alloc_pooled(sizeof(int), ctx));
  if (streamed) {
    s = stream_setup(r.get());
    if (s != MTR_OK) return s;
    r->bytes += r->slabs->device_bytes;
  }
  MTR_CK(ctx, cudaMemsetAsync(r->err.p, 0, sizeof(int), ctx->stream));
  r->bytes += hv ? 0 : vb;
  for (int k = 0; k < n_axes; ++k) {
    AxisState& a = r->ax[k];
    a.PX = axes[k].prj.X;
    a.PY = axes[k].prj.Y;
    a.A = axes[k].prj.AngN;
    a.pitch = projection_pitch(a.PX);
    a.np = (long long)a.pitch * a.PY * a.A;
    a.hxc.assign(axes[k].x_coef, axes[k].x_coef + 4 * a.A);
    a.hyc.assign(axes[k].y_coef, axes[k].y_coef + 4 * a.A);
    const size_t pe = mx ? 2 : 4;
    MTR_CK(ctx, a.xc.alloc_pooled(sizeof(double) * 4 * a.A, ctx));
    MTR_CK(ctx, a.yc.alloc_pooled(sizeof(double) * 4 * a.A, ctx));
    MTR_CK(ctx, a.b.alloc_pooled((size_t)a.np * pe, ctx));
    MTR_CK(ctx, a.s.alloc_pooled((size_t)a.np * 4, ctx));
    MTR_CK(ctx, a.cf.alloc_pooled((size_t)a.np * 4, ctx));
    a.pitch2 = pair_pitch(a.PX);
    const long long rb = residual_bytes(a.PX, a.PY, a.A);
    MTR_CK(ctx, a.r.alloc_pooled((size_t)rb, ctx));
    MTR_CK(ctx, a.cbp.alloc_where(vb, hv, ctx));
    MTR_CK(ctx, a.w.alloc_where((size_t)(r->nv * state_bytes(params->precision)), hv, ctx));
    MTR_CK(ctx, a.x.alloc_where(vb, hv, ctx));
    if (mx) MTR_CK(ctx, a.xcopy.alloc_where((size_t)r->nv * 2, hv, ctx));
    r->bytes += axis_bytes(a.np, rb, hv ? 0 : r->nv, params->precision) + 64LL * a.A;  // device bytes
    MTR_CK(ctx, cudaMemcpyAsync(a.xc.p, axes[k].x_coef, sizeof(double) * 4 * a.A, cudaMemcpyHostToDevice, ctx->stream));
    MTR_CK(ctx, cudaMemcpyAsync(a.yc.p, axes[k].y_coef, sizeof(double) * 4 * a.A, cudaMemcpyHostToDevice, ctx->stream));
    MTR_CK(ctx, cudaMemsetAsync(a.s.p, 0, (size_t)a.np * 4, ctx->stream));
    MTR_CK(ctx, cudaMemsetAsync(a.r.p, 0, (size_t)rb, ctx->stream));
    if (axes[k].prj_data) {
      s = upload_projections(r.get(), k, axes[k].prj_data, mem_kind);
      if (s != MTR_OK) return s;
    } else {  // zero until mtr_recon_upload / mtr_recon_upload_half
      MTR_CK(ctx, cudaMemsetAsync(a.b.p, 0, (size_t)a.np * pe, ctx->stream));
    }
    // TMA kernels where the window geometry fits (else the plain kernels run).
    if (!tma_disabled()) {
      // WBP over b; with FP16 projections over their FP32 widening in r (r is
      // free until the first residual), so the WBP gathers FP32 like SIRT.
      // SIRT back-projection over the FP32 residual and the forward splat: tuned depths
      if (streamed) {  // candidates over one slab, in the slot arrays the run uses
        VolDev tv = r->vol;
        tv.NZ = r->slabs->depth;
        tune_axis(ctx, a, tv, params->precision, r->slabs->x[0].as<float>(), r->slabs->cbp[0].as<float>(),
                  r->slabs->xc[0].p, r->err.as<int>());
      } else {
        // (x and cbp: FP32 volume arrays the WBP init writes afterwards)
        tune_axis(ctx, a, r->vol, params->precision, a.x.as<float>(), a.cbp.as<float>(), a.xcopy.p,
                  r->err.as<int>());
      }
      // The WBP gathers the same windows as the SIRT update: the lane layout
      // tuned for it (lines or 8x4 patches), at depth 16 where the tuned depth
      // is 16 or more, else 8.
      a.plan_b = plan_backproject(a.hxc, a.hyc, a.A, 0, a.plan.ok && a.plan.nz >= 16 ? 16 : 8,
                                  a.plan.ok ? a.plan.lanes : -1);
      a.tma_b = a.plan_b.ok && encode_tensor_map_3d(&a.map_b, mx ? a.r.p : a.b.p, false, a.PX, a.pitch, a.PY, a.A,
                                                    a.plan_b.WX, a.plan_b.WY);
    }
  }
  if (params->flags & MTR_FLAG_RECORD_NORMS) {
    const size_t n = (size_t)std::max(1, params->iter_times) * n_axes * std::max(1, params->sirt_inner);
    MTR_CK(ctx, r->norms.alloc_pooled(sizeof(double) * n, ctx));
  }
  // convergence record: FP64 sum (w_avg change)^2 and sum w_avg^2 per outer iteration
  MTR_CK(ctx, r->dchange.alloc_pooled(sizeof(double) * 2 * std::max(1, params->iter_times), ctx));
  MTR_CK(ctx, cudaMemsetAsync(r->dchange.p, 0, sizeof(double) * 2 * std::max(1, params->iter_times), ctx->stream));
  s = enqueue_geometry(r.get());
  if (s != MTR_OK) return s;
  r->geometry_ready = true;
  // Host staging buffers passed in may be freed after return: finish the copies.
  MTR_CK(ctx, cudaStreamSynchronize(ctx->stream));
  *out = r.release();
  return MTR_OK;
}

mtr_status mtr_recon_upload(mtr_recon* r, int axis, const float* prj_data, int mem_kind) {
  if (!r || !prj_data || axis < 0 || axis >= r->K) return MTR_ERR_INVALID_ARGUMENT;
  DeviceGuard g(r->ctx->device);
  return upload_projections(r, axis, prj_data, mem_kind);
}

mtr_status mtr_recon_upload_half(mtr_recon* r, int axis, const void* prj_f16, int mem_kind) {
  if (!r || !prj_f16 || axis < 0 || axis >= r->K) return MTR_ERR_INVALID_ARGUMENT;
  if (mem_kind != MTR_MEM_HOST && mem_kind != MTR_MEM_DEVICE)
    return set_error(r->ctx, MTR_ERR_INVALID_ARGUMENT, "unknown memory kind");
  DeviceGuard g(r->ctx->device);
  return upload_projections_half(r, axis, prj_f16, mem_kind);
}

mtr_status mtr_recon_init(mtr_recon* r) {
  if (!r) return MTR_ERR_INVALID_ARGUMENT;
  DeviceGuard g(r->ctx->device);
  r->outer_done = 0;
  return recon_enqueue_init(r);
}

mtr_status mtr_recon_run_outer(mtr_recon* r, int first, int count) {
  if (!r || first < 0 || count < 0) return MTR_ERR_INVALID_ARGUMENT;
  DeviceGuard g(r->ctx->device);
  mtr_status s = enqueue_outer(r, first, count);
  if (s == MTR_OK) r->outer_done = first + count;
  return s;
}

mtr_status mtr_recon_save(mtr_recon* r, const char* path) {
  if (!r || !path) return MTR_ERR_INVALID_ARGUMENT;
  mtr_context* ctx = r->ctx;
  DeviceGuard g(ctx->device);
  const size_t vb = (size_t)r->nv * 4;
  std::vector<float> host((size_t)r->nv);
  CkptHeader h{};
  std::memcpy(h.magic, kCkptMagic, 8);
  h.version = 1;
  h.K = r->K;
  h.X = r->vs.X;
  h.Y = r->vs.Y;
  h.Z = r->vs.Z;
  h.outer_done = r->outer_done;
  h.precision = r->p.precision;
  DevBuf tmp;  // FP32 value of an FP16 deviation state (mixed precision)
  if (mixed(r->p.precision)) MTR_CK(ctx, tmp.alloc_pooled(vb, ctx));
  FILE* f = std::fopen(path, "wb");
  if (!f) return set_error(ctx, MTR_ERR_IO, std::string("cannot create ") + path);
  bool ok = std::fwrite(&h, sizeof h, 1, f) == 1;
  for (int k = -1; ok && k < r->K; ++k) {
    const void* src = k < 0 ? r->wavg.p : r->ax[k].w.p;
    if (k >= 0 && tmp.p) {  // the file holds FP32 states in every precision
      const mtr_status ss = state_value(r, k, tmp.as<float>(), ctx->stream);
      if (ss != MTR_OK) {
        std::fclose(f);
        return ss;
      }
      src = tmp.p;
    }
    cudaError_t e = cudaMemcpyAsync(host.data(), src, vb, cudaMemcpyDefault, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) {
      std::fclose(f);
      return cuda_error(ctx, e, "checkpoint download");
    }
    ok = std::fwrite(host.data(), 4, (size_t)r->nv, f) == (size_t)r->nv;
  }
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) return set_error(ctx, MTR_ERR_IO, std::string("cannot write ") + path);
  return mtr_recon_check(r);
}

mtr_status mtr_recon_load(mtr_recon* r, const char* path, int* outer_done) {
  if (!r || !path) return MTR_ERR_INVALID_ARGUMENT;
  mtr_context* ctx = r->ctx;
  DeviceGuard g(ctx->device);
  FILE* f = std::fopen(path, "rb");
  if (!f) return set_error(ctx, MTR_ERR_IO, std::string("cannot open ") + path);
  CkptHeader h{};
  if (std::fread(&h, sizeof h, 1, f) != 1 || std::memcmp(h.magic, kCkptMagic, 8) != 0 || h.version != 1) {
    std::fclose(f);
    return set_error(ctx, MTR_ERR_FORMAT, "not a checkpoint file");
  }
  if (h.K != r->K || h.X != r->vs.X || h.Y != r->vs.Y || h.Z != r->vs.Z || h.outer_done < 0) {
    std::fclose(f);
    return set_error(ctx, MTR_ERR_INVALID_ARGUMENT, "checkpoint of another volume or axis count");
  }
  // the WBP init computes the back-projection weight sums the SIRT update
  // reads; its volumes are then replaced by the saved state
  mtr_status s = recon_enqueue_init(r);
  if (s != MTR_OK) {
    std::fclose(f);
    return s;
  }
  const size_t vb = (size_t)r->nv * 4;
  std::vector<float> host((size_t)r->nv);
  DevBuf tmp;  // FP32 staging of a state that is stored FP16 (mixed precision)
  if (mixed(r->p.precision)) {
    const cudaError_t e = tmp.alloc_pooled(vb, ctx);
    if (e != cudaSuccess) {
      std::fclose(f);
      return cuda_error(ctx, e, "checkpoint staging");
    }
  }
  for (int k = -1; k < r->K; ++k) {
    if (std::fread(host.data(), 4, (size_t)r->nv, f) != (size_t)r->nv) {
      std::fclose(f);
      return set_error(ctx, MTR_ERR_FORMAT, "truncated checkpoint");
    }
    void* dst = k < 0 ? r->wavg.p : (tmp.p ? tmp.p : r->ax[k].w.p);
    cudaError_t e = cudaMemcpyAsync(dst, host.data(), vb, cudaMemcpyDefault, ctx->stream);
    if (e == cudaSuccess && k >= 0 && tmp.p) {
      const mtr_status ss = set_state(r, r->ax[k], tmp.as<float>(), ctx->stream);
      if (ss != MTR_OK) {
        std::fclose(f);
        return ss;
      }
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);  // host buffer is reused
    if (e != cudaSuccess) {
      std::fclose(f);
      return cuda_error(ctx, e, "checkpoint upload");
    }
  }
  std::fclose(f);
  // next SIRT start z_k = 2 w_avg - w_k (as the MACE step leaves it) and its copy
  const int ck = copy_kind_of(r->p.precision);
  for (auto& a : r->ax) {
    if (mixed(r->p.precision))
      launch_initial_z_half(a.w.as<__half>(), r->wavg.as<float>(), a.x.as<float>(), r->nv, ctx->stream);
    else
      launch_initial_z(a.w.as<float>(), r->wavg.as<float>(), a.x.as<float>(), r->nv, ctx->stream);
    MTR_CK_LAUNCH(ctx, "resume z");
    if (ck) {
      launch_convert_copy(a.x.as<float>(), a.xcopy.p, ck, r->nv, ctx->stream);
      MTR_CK_LAUNCH(ctx, "resume copy");
    }
  }
  r->outer_done = h.outer_done;
  if (outer_done) *outer_done = h.outer_done;
  // a streamed run copies these host arrays in on its own streams
  return r->slabs ? stream_join(r) : MTR_OK;
}

mtr_status mtr_recon_run(mtr_recon* r) {
  if (!r) return MTR_ERR_INVALID_ARGUMENT;
  mtr_context* ctx = r->ctx;
  DeviceGuard g(ctx->device);
  r->outer_done = r->p.iter_times;
  // (a streamed run waits on copies between its streams: not captured; with
  // per-kernel profiling on, the launches run one by one between their events)
  if (!(r->p.flags & MTR_FLAG_GRAPH) || r->slabs || ctx->profiling) return enqueue_run(r);
  if (!r->graph) {
    cudaGraph_t graph = nullptr;
    MTR_CK(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    const long long before = g_launches.load();
    mtr_status s = enqueue_run(r);
    const long long nodes = g_launches.load() - before;
    g_launches.fetch_sub(nodes);
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &graph);
    if (s != MTR_OK) {
      if (graph) cudaGraphDestroy(graph);
      return s;
    }
    if (e != cudaSuccess) return cuda_error(ctx, e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&r->graph, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
      r->graph = nullptr;
      return cuda_error(ctx, e, "cudaGraphInstantiate");
    }
    r->graph_nodes = nodes;
  }
  MTR_CK(ctx, cudaGraphLaunch(r->graph, ctx->stream));
  g_launches.fetch_add(r->graph_nodes);
  return MTR_OK;
}

mtr_status mtr_recon_download(mtr_recon* r, float* out, int mem_kind) {
  if (!r || !out) return MTR_ERR_INVALID_ARGUMENT;
  mtr_context* ctx = r->ctx;
  DeviceGuard g(ctx->device);
  // (volume arrays may be mapped host memory: let unified addressing pick the direction)
  const cudaMemcpyKind kind = cudaMemcpyDefault;
  MTR_CK(ctx, cudaMemcpyAsync(out, r->wavg.p, (size_t)r->nv * 4, kind, ctx->stream));
  if (mem_kind != MTR_MEM_DEVICE) {
    MTR_CK(ctx, cudaStreamSynchronize(ctx->stream));
    return mtr_recon_check(r);
  }
  return MTR_OK;
}

mtr_status mtr_recon_check(mtr_recon* r) {
  if (!r) return MTR_ERR_INVALID_ARGUMENT;
  mtr_context* ctx = r->ctx;
  DeviceGuard g(ctx->device);
  int flag = 0;
  MTR_CK(ctx, cudaMemcpyAsync(&flag, r->err.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  MTR_CK(ctx, cudaStreamSynchronize(ctx->stream));
  if (flag != 0)
    return set_error(ctx, MTR_ERR_TIMEOUT,
                     "a kernel gave up on a bounded wait or a window bound (code " + std::to_string(flag) + ")");
  return MTR_OK;
}

mtr_status mtr_recon_download_axes(mtr_recon* r, float* out, int mem_kind) {
  if (!r || !out) return MTR_ERR_INVALID_ARGUMENT;
  mtr_context* ctx = r->ctx;
  DeviceGuard g(ctx->device);
  // (volume arrays may be mapped host memory: let unified addressing pick the direction)
  const cudaMemcpyKind kind = cudaMemcpyDefault;
  if (!mixed(r->p.precision)) {
    for (int k = 0; k < r->K; ++k)
      MTR_CK(ctx, cudaMemcpyAsync(out + (size_t)k * r->nv, r->ax[k].w.p, (size_t)r->nv * 4, kind, ctx->stream));
  } else if (mem_kind == MTR_MEM_DEVICE) {  // FP32 values of the FP16 deviations straight into the caller's array
    for (int k = 0; k < r->K; ++k) {
      const mtr_status s = state_value(r, k, out + (size_t)k * r->nv, ctx->stream);
      if (s != MTR_OK) return s;
    }
  } else {
    DevBuf tmp;
    MTR_CK(ctx, tmp.alloc_pooled((size_t)r->nv * 4, ctx));
    for (int k = 0; k < r->K; ++k) {
      const mtr_status s = state_value(r, k, tmp.as<float>(), ctx->stream);
      if (s != MTR_OK) return s;
      MTR_CK(ctx, cudaMemcpyAsync(out + (size_t)k * r->nv, tmp.p, (size_t)r->nv * 4, kind, ctx->stream));
    }
    MTR_CK(ctx, cudaStreamSynchronize(ctx->stream));
  }
  if (mem_kind != MTR_MEM_DEVICE) MTR_CK(ctx, cudaStreamSynchronize(ctx->stream));
  return MTR_OK;
}

mtr_status mtr_recon_norms(mtr_recon* r, double* out, long long n) {
  if (!r || !out) return MTR_ERR_INVALID_ARGUMENT;
  if (!r->norms.p) return set_error(r->ctx, MTR_ERR_INVALID_ARGUMENT, "norms not recorded (MTR_FLAG_RECORD_NORMS)");
  const long long have = (long long)r->p.iter_times * r->K * r->p.sirt_inner;
  if (n > have) n = have;
  DeviceGuard g(r->ctx->device);
  MTR_CK(r->ctx, cudaMemcpyAsync(out, r->norms.p, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, r->ctx->stream));
  MTR_CK(r->ctx, cudaStreamSynchronize(r->ctx->stream));
  return MTR_OK;
}

mtr_status mtr_recon_changes(mtr_recon* r, double* out, int n) {
  if (!r || !out || n < 0) return MTR_ERR_INVALID_ARGUMENT;
  if (!r->record_changes)
    return set_error(r->ctx, MTR_ERR_INVALID_ARGUMENT, "convergence record not kept (MTR_FLAG_RECORD_CHANGES)");
  n = std::min(n, std::max(1, r->p.iter_times));
  DeviceGuard g(r->ctx->device);
  std::vector<double> raw(2 * (size_t)n);
  MTR_CK(r->ctx, cudaMemcpyAsync(raw.data(), r->dchange.p, sizeof(double) * raw.size(), cudaMemcpyDeviceToHost,
                                 r->ctx->stream));
  MTR_CK(r->ctx, cudaStreamSynchronize(r->ctx->stream));
  for (int i = 0; i < n; ++i) out[i] = raw[2 * i + 1] > 0.0 ? std::sqrt(raw[2 * i] / raw[2 * i + 1]) : 0.0;
  return MTR_OK;
}

mtr_status mtr_recon_run_until(mtr_recon* r, int first, double tol, int* outer_done) {
  if (!r || first < 0 || !(tol >= 0.0)) return MTR_ERR_INVALID_ARGUMENT;
  DeviceGuard g(r->ctx->device);
  r->record_changes = true;  // the stopping rule reads the record
  int it = first;
  while (it < r->p.iter_times) {
    mtr_status s = enqueue_outer(r, it, 1);
    if (s != MTR_OK) return s;
    ++it;
    r->outer_done = it;
    std::vector<double> all((size_t)it);
    s = mtr_recon_changes(r, all.data(), it);  // synchronises
    if (s != MTR_OK) return s;
    if (all[(size_t)it - 1] < tol) break;
  }
  if (outer_done) *outer_done = it;
  return mtr_recon_check(r);
}

mtr_status mtr_recon_footprint(const mtr_recon* r, long long* bytes) {
  if (!r || !bytes) return MTR_ERR_INVALID_ARGUMENT;
  *bytes = r->bytes;
  return MTR_OK;
}

mtr_status mtr_recon_describe(const mtr_recon* r, char* buf, int cap) {
  if (!r || !buf || cap <= 0) return MTR_ERR_INVALID_ARGUMENT;
  std::string s = "[";
  for (size_t k = 0; k < r->ax.size(); ++k) {
    const AxisState& a = r->ax[k];
    char t[512];
    std::snprintf(t, sizeof(t),
                  "%s{\"axis\":%zu,\"back_projection\":{\"tma\":%s,\"depth\":%d,\"window\":[%d,%d],\"lanes\":\"%s\","
                  "\"window_format\":\"%s\"},"
                  "\"forward\":{\"tma\":%s,\"depth\":%d,\"window\":[%d,%d],\"lanes\":\"%s\",\"y_has_z\":%s}}",
                  k ? "," : "", k, a.tma ? "true" : "false", a.plan.nz, a.plan.WX, a.plan.WY,
                  a.plan.lanes == 1 ? "y" : a.plan.lanes == 2 ? "patch" : "x",
                  a.plan.half ? "fp16 pairs" : a.plan.planar ? "planar pairs" : a.plan.pairs ? "pairs" : "fp32",
                  a.ftma ? "true" : "false", a.fplan.nz, a.fplan.WX, a.fplan.WY,
                  a.fplan.lanes == 1 ? "y" : a.fplan.lanes == 2 ? "patch" : "x", a.fplan.bz0 ? "false" : "true");
    s += t;
  }
  s += "]";
  std::snprintf(buf, (size_t)cap, "%s", s.c_str());
  return MTR_OK;
}

mtr_status mtr_recon_destroy(mtr_recon* r) {
  if (!r) return MTR_OK;
  DeviceGuard g(r->ctx->device);
  // The arrays return to the context's pool without a further wait, so every
  // stream that used them must be done: the whole device, as cudaFree would
  // have waited (the context stream may have been changed since the run).
  cudaDeviceSynchronize();
  delete r;
  return MTR_OK;
}

// ---- Reference-shaped entry points (host buffers in and out) --------------

mtr_status mtr_reconstruct(mtr_context* ctx, int n_axes, const mtr_axis* axes, mtr_volume_size vol,
                           const mtr_params* params, float* out_volume) {
  if (!ctx || !out_volume || !axes) return set_error(ctx, MTR_ERR_INVALID_ARGUMENT, "null argument");
  if (n_axes <= 0 || n_axes > MTR_MAX_AXES) return set_error(ctx, MTR_ERR_INVALID_ARGUMENT, "axis count out of range");
  // This entry point has no later upload: every axis must bring its projections.
  for (int k = 0; k < n_axes; ++k) {
    const mtr_status sa = check_axis(ctx, axes[k], true);
    if (sa != MTR_OK) return sa;
  }
  mtr_recon* r = nullptr;
  mtr_status s = mtr_recon_create(ctx, n_axes, axes, vol, params, MTR_MEM_HOST, &r);
  if (s != MTR_OK) return s;
  s = mtr_recon_run(r);
  if (s == MTR_OK) s = mtr_recon_download(r, out_volume, MTR_MEM_HOST);
  mtr_recon_destroy(r);
  return s;
}

}  // extern "C"
