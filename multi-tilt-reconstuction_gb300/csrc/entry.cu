// Single-axis entry points with the reference's host-buffer contract:
// mtr_wbp (ComputeInitialModel), mtr_sirt (runSIRTOnGPU), mtr_initial_z
// (initialZdata) and mtr_update_w (runMaceOnGPU / runMaceOnCPU).
// Like the reference they upload, compute and download per call; unlike it
// they keep the whole SIRT loop on the device (no per-iteration host
// residual, no MPI) and return a status instead of exiting.  mtr_wbp and
// mtr_sirt run on a one-axis reconstruction object over the slab, so they use
// the autotuned, TMA-windowed projectors and the context's memory pool.
#include "mtr_internal.h"
#include "mtr_runtime.h"

using namespace mtr;

namespace {

mtr_status check_slab(mtr_context* ctx, const mtr_volume_size& vol, int z0, int z1) {
  if (z0 < vol.Zstart || z1 > vol.Zend || z0 >= z1)
    return set_error(ctx, MTR_ERR_INVALID_ARGUMENT, "slab [slice_start, slice_end) outside the volume or empty");
  return MTR_OK;
}

// A one-axis FP32 reconstruction object whose volume frame is the Z-slab
// [z0, z1) of vol: the same arrays (from the context's pool), autotuned tiles
// and kernels as mtr_recon_create, so the reference-shaped calls run the
// TMA-windowed projectors wherever the windows fit.  Destroyed with the
// object, which waits for the work that used its arrays.
struct SlabRecon {
  mtr_recon* r = nullptr;
  mtr_status create(mtr_context* ctx, const mtr_axis& axis, const mtr_volume_size& vol, int z0, int z1, int n_inner,
                    float step) {
    mtr_volume_size sv = vol;
    sv.Zstart = z0;
    sv.Zend = z1;
    sv.Z = z1 - z0;
    mtr_params p;
    mtr_params_default(&p);
    p.iter_times = 1;
    p.sirt_inner = n_inner;
    p.sirt_step = step;
    p.precision = MTR_PREC_FP32;
    p.flags = 0;
    return mtr_recon_create(ctx, 1, &axis, sv, &p, MTR_MEM_HOST, &r);
  }
  ~SlabRecon() { mtr_recon_destroy(r); }
};

}  // namespace

extern "C" {

mtr_status mtr_wbp(mtr_context* ctx, const mtr_axis* axis, mtr_volume_size vol, int slice_start, int slice_end,
                   float* slab_out) {
  if (!ctx || !axis || !slab_out) return set_error(ctx, MTR_ERR_INVALID_ARGUMENT, "null argument");
  mtr_status s = check_volume(ctx, vol);
  if (s == MTR_OK) s = check_axis(ctx, *axis);
  if (s == MTR_OK) s = check_slab(ctx, vol, slice_start, slice_end);
  if (s != MTR_OK) return s;
  DeviceGuard g(ctx->device);
  SlabRecon sr;
  s = sr.create(ctx, *axis, vol, slice_start, slice_end, 0, 0.f);
  if (s != MTR_OK) return s;
  mtr_recon* r = sr.r;
  s = recon_enqueue_wbp(r, 0);  // x = s/c, cbp = c over the slab
  if (s != MTR_OK) return s;
  MTR_CK(ctx, cudaMemcpyAsync(slab_out, r->ax[0].x.p, (size_t)r->nv * 4, cudaMemcpyDeviceToHost, ctx->stream));
  MTR_CK(ctx, cudaStreamSynchronize(ctx->stream));
  return mtr_recon_check(r);
}

mtr_status mtr_sirt(mtr_context* ctx, const mtr_axis* axis, mtr_volume_size vol, int slice_start, int slice_end,
                    int n_inner, float sirt_step, float* slab_inout) {
  if (!ctx || !axis || !slab_inout) return set_error(ctx, MTR_ERR_INVALID_ARGUMENT, "null argument");
  if (n_inner < 0) return set_error(ctx, MTR_ERR_INVALID_ARGUMENT, "negative iteration count");
  mtr_status s = check_volume(ctx, vol);
  if (s == MTR_OK) s = check_axis(ctx, *axis);
  if (s == MTR_OK) s = check_slab(ctx, vol, slice_start, slice_end);
  if (s != MTR_OK) return s;
  DeviceGuard g(ctx->device);
  SlabRecon sr;
  s = sr.create(ctx, *axis, vol, slice_start, slice_end, n_inner, sirt_step);
  if (s != MTR_OK) return s;
  mtr_recon* r = sr.r;
  // The WBP pass yields the back-projection weight sums C = A^T 1 of the slab
  // (geometry only; the reference recomputes its sums every call and every
  // iteration, FunctionOnGPU.cu:218-232); its volume is then replaced by the
  // caller's slab.
  s = recon_enqueue_wbp(r, 0);
  if (s != MTR_OK) return s;
  MTR_CK(ctx, cudaMemcpyAsync(r->ax[0].x.p, slab_inout, (size_t)r->nv * 4, cudaMemcpyHostToDevice, ctx->stream));
  for (int it = 0; it < n_inner; ++it) {
    if ((s = recon_enqueue_forward(r, 0)) != MTR_OK) return s;
    if ((s = recon_enqueue_residual(r, 0)) != MTR_OK) return s;
    if ((s = recon_enqueue_sirt_bp(r, 0)) != MTR_OK) return s;
  }
  MTR_CK(ctx, cudaMemcpyAsync(slab_inout, r->ax[0].x.p, (size_t)r->nv * 4, cudaMemcpyDeviceToHost, ctx->stream));
  MTR_CK(ctx, cudaStreamSynchronize(ctx->stream));
  return mtr_recon_check(r);
}

static mtr_status elementwise(mtr_context* ctx, mtr_volume_size vol, const float* a, const float* b, float* io,
                              int op, float step) {
  if (!ctx || !a || !b || !io) return set_error(ctx, MTR_ERR_INVALID_ARGUMENT, "null argument");
  mtr_status s = check_volume(ctx, vol);
  if (s != MTR_OK) return s;
  DeviceGuard g(ctx->device);
  const long long n = (long long)vol.X * vol.Y * vol.Z;
  DevBuf da, db, dio;
  MTR_CK(ctx, da.alloc((size_t)n * 4));
  MTR_CK(ctx, db.alloc((size_t)n * 4));
  MTR_CK(ctx, dio.alloc((size_t)n * 4));
  MTR_CK(ctx, cudaMemcpyAsync(da.p, a, (size_t)n * 4, cudaMemcpyHostToDevice, ctx->stream));
  MTR_CK(ctx, cudaMemcpyAsync(db.p, b, (size_t)n * 4, cudaMemcpyHostToDevice, ctx->stream));
  if (op == 0) {
    launch_initial_z(da.as<float>(), db.as<float>(), dio.as<float>(), n, ctx->stream);
  } else {
    MTR_CK(ctx, cudaMemcpyAsync(dio.p, io, (size_t)n * 4, cudaMemcpyHostToDevice, ctx->stream));
    launch_update_w(da.as<float>(), db.as<float>(), dio.as<float>(), n, step, ctx->stream);
  }
  MTR_CK_LAUNCH(ctx, op == 0 ? "initial z" : "update w");
  MTR_CK(ctx, cudaMemcpyAsync(io, dio.p, (size_t)n * 4, cudaMemcpyDeviceToHost, ctx->stream));
  MTR_CK(ctx, cudaStreamSynchronize(ctx->stream));
  return MTR_OK;
}

mtr_status mtr_initial_z(mtr_context* ctx, mtr_volume_size vol, const float* w, const float* w_avg, float* z) {
  return elementwise(ctx, vol, w, w_avg, z, 0, 0.f);
}

mtr_status mtr_update_w(mtr_context* ctx, mtr_volume_size vol, const float* v, const float* z, float* w, float step) {
  return elementwise(ctx, vol, v, z, w, 1, step);
}

}  // extern "C"
