// Single-axis entry points with the reference's host-buffer contract:
// mtr_wbp (ComputeInitialModel), mtr_sirt (runSIRTOnGPU), mtr_initial_z
// (initialZdata) and mtr_update_w (runMaceOnGPU / runMaceOnCPU).
// Like the reference they upload, compute and download per call; unlike it
// they keep the whole SIRT loop on the device (no per-iteration host
// residual, no MPI) and return a status instead of exiting.
#include "mtr_internal.h"
#include "mtr_runtime.h"

using namespace mtr;

namespace {

mtr_status check_slab(mtr_context* ctx, const mtr_volume_size& vol, int z0, int z1) {
  if (z0 < vol.Zstart || z1 > vol.Zend || z0 >= z1)
    return set_error(ctx, MTR_ERR_INVALID_ARGUMENT, "slab [slice_start, slice_end) outside the volume or empty");
  return MTR_OK;
}

struct AxisUpload {
  DevBuf xc, yc, b;
  AxisDev dev;
};

mtr_status upload_axis(mtr_context* ctx, const mtr_axis& a, AxisUpload& u) {
  const long long np = (long long)a.prj.X * a.prj.Y * a.prj.AngN;
  MTR_CK(ctx, u.xc.alloc(sizeof(double) * 4 * a.prj.AngN));
  MTR_CK(ctx, u.yc.alloc(sizeof(double) * 4 * a.prj.AngN));
  MTR_CK(ctx, u.b.alloc((size_t)np * 4));
  MTR_CK(ctx, cudaMemcpyAsync(u.xc.p, a.x_coef, sizeof(double) * 4 * a.prj.AngN, cudaMemcpyHostToDevice, ctx->stream));
  MTR_CK(ctx, cudaMemcpyAsync(u.yc.p, a.y_coef, sizeof(double) * 4 * a.prj.AngN, cudaMemcpyHostToDevice, ctx->stream));
  MTR_CK(ctx, cudaMemcpyAsync(u.b.p, a.prj_data, (size_t)np * 4, cudaMemcpyHostToDevice, ctx->stream));
  u.dev = AxisDev{a.prj.X, a.prj.Y, a.prj.AngN, u.xc.as<double>(), u.yc.as<double>(), a.prj.X};
  return MTR_OK;
}

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
  AxisUpload u;
  s = upload_axis(ctx, *axis, u);
  if (s != MTR_OK) return s;
  const long long ns = (long long)vol.X * vol.Y * (slice_end - slice_start);
  DevBuf x, cbp;
  MTR_CK(ctx, x.alloc((size_t)ns * 4));
  MTR_CK(ctx, cbp.alloc((size_t)ns * 4));
  const VolDev v{vol.Xstart, vol.Ystart, slice_start, vol.X, vol.Y, slice_end - slice_start};
  launch_backproject<float>(u.dev, v, u.b.as<float>(), 0, 0.f, x.as<float>(), cbp.as<float>(), nullptr, 0,
                            slice_start, slice_end, ctx->stream);
  MTR_CK_LAUNCH(ctx, "wbp");
  MTR_CK(ctx, cudaMemcpyAsync(slab_out, x.p, (size_t)ns * 4, cudaMemcpyDeviceToHost, ctx->stream));
  MTR_CK(ctx, cudaStreamSynchronize(ctx->stream));
  return MTR_OK;
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
  AxisUpload u;
  s = upload_axis(ctx, *axis, u);
  if (s != MTR_OK) return s;
  const long long np = (long long)axis->prj.X * axis->prj.Y * axis->prj.AngN;
  const long long ns = (long long)vol.X * vol.Y * (slice_end - slice_start);
  DevBuf x, cbp, sbuf, cf, r;
  MTR_CK(ctx, x.alloc((size_t)ns * 4));
  MTR_CK(ctx, cbp.alloc((size_t)ns * 4));
  MTR_CK(ctx, sbuf.alloc((size_t)np * 4));
  MTR_CK(ctx, cf.alloc((size_t)np * 4));
  MTR_CK(ctx, r.alloc((size_t)np * 4));
  MTR_CK(ctx, cudaMemcpyAsync(x.p, slab_inout, (size_t)ns * 4, cudaMemcpyHostToDevice, ctx->stream));
  MTR_CK(ctx, cudaMemsetAsync(sbuf.p, 0, (size_t)np * 4, ctx->stream));
  MTR_CK(ctx, cudaMemsetAsync(cf.p, 0, (size_t)np * 4, ctx->stream));
  const VolDev v{vol.Xstart, vol.Ystart, slice_start, vol.X, vol.Y, slice_end - slice_start};
  // Geometry-only sums, once (the reference recomputes c every iteration).
  launch_forward<float>(u.dev, v, nullptr, cf.as<float>(), slice_start, slice_end, ctx->stream);
  MTR_CK_LAUNCH(ctx, "forward row sums");
  launch_backproject<float>(u.dev, v, u.b.as<float>(), 2, 0.f, nullptr, cbp.as<float>(), nullptr, 0, slice_start,
                            slice_end, ctx->stream);
  MTR_CK_LAUNCH(ctx, "back-projection weight sums");
  for (int it = 0; it < n_inner; ++it) {
    launch_forward<float>(u.dev, v, x.as<float>(), sbuf.as<float>(), slice_start, slice_end, ctx->stream);
    MTR_CK_LAUNCH(ctx, "forward splat");
    launch_residual<float, float>(np, u.b.as<float>(), sbuf.as<float>(), cf.as<float>(), r.as<float>(), nullptr,
                                  ctx->stream);
    MTR_CK_LAUNCH(ctx, "residual");
    launch_backproject<float>(u.dev, v, r.as<float>(), 1, sirt_step, x.as<float>(), cbp.as<float>(), nullptr, 0,
                              slice_start, slice_end, ctx->stream);
    MTR_CK_LAUNCH(ctx, "sirt back-projection");
  }
  MTR_CK(ctx, cudaMemcpyAsync(slab_inout, x.p, (size_t)ns * 4, cudaMemcpyDeviceToHost, ctx->stream));
  MTR_CK(ctx, cudaStreamSynchronize(ctx->stream));
  return MTR_OK;
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
