// mtr_sirt_noalloc: SIRT iterations of one tilt axis that allocate no device
// memory.
//
// Who needs it: callers that cannot call cudaMalloc at the point where they
// reconstruct.  cudaMalloc/cudaFree synchronise the whole device and may
// fail under memory pressure, so a stage of a real-time pipeline, code that
// runs between other work on a stream it must not stall, or a host program
// whose device memory is owned by another allocator (a framework's caching
// allocator, a fixed arena) cannot afford them.  mtr_sirt allocates its
// working arrays per call; this entry point uses a fixed device array
// compiled into the library instead, and the caller passes inputs and
// outputs as device pointers it already owns.
//
// The scratch array holds the per-call working arrays (ray sums, row sums,
// residual, back-projection weight sums): 3*AngN*Y*X + X*Y*(z1-z0) floats,
// at most MTR_NOALLOC_SCRATCH_FLOATS.  Every GPU that loads libmtr keeps it
// for the life of the process.  Every call shares the same array and it keeps
// the last call's contents; this entry point clears what must start at zero.
// Calls that overlap on the GPU (two streams, or two host threads) race on
// the array: issue them one after another on one stream.
//
// The first call on a device looks up the array's device address (with that
// device current) and caches it; make that first call before any stream
// capture.
#include <mutex>

#include "mtr_internal.h"
#include "mtr_runtime.h"

using namespace mtr;

namespace {

static __device__ __align__(256) float g_noalloc_scratch[MTR_NOALLOC_SCRATCH_FLOATS];

constexpr int kMaxDevices = 64;
float* g_scratch_ptr[kMaxDevices] = {};
std::mutex g_scratch_mu;

// Device address of the scratch array on the current device (set-up once per
// device; the host-side symbol is only a handle, never a device address).
cudaError_t scratch_on_device(int dev, float** out) {
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_ptr[dev] = static_cast<float*>(p);
  }
  *out = g_scratch_ptr[dev];
  return cudaSuccess;
}

}  // namespace

extern "C" mtr_status mtr_sirt_noalloc(mtr_context* ctx, mtr_projection_size prj, const double* x_coef_dev,
                                       const double* y_coef_dev, const float* prj_dev, mtr_volume_size vol,
                                       int slice_start, int slice_end, int n_inner, float sirt_step,
                                       float* slab_dev) {
  if (!ctx || !x_coef_dev || !y_coef_dev || !prj_dev || !slab_dev)
    return set_error(ctx, MTR_ERR_INVALID_ARGUMENT, "null argument");
  if (prj.X <= 0 || prj.Y <= 0 || prj.AngN <= 0 || prj.AngN > kMaxAngles || n_inner < 0)
    return set_error(ctx, MTR_ERR_INVALID_ARGUMENT, "projection size or iteration count out of range");
  mtr_status s = check_volume(ctx, vol);
  if (s != MTR_OK) return s;
  if (slice_start < vol.Zstart || slice_end > vol.Zend || slice_start >= slice_end)
    return set_error(ctx, MTR_ERR_INVALID_ARGUMENT, "slab [slice_start, slice_end) outside the volume or empty");
  const long long np = (long long)prj.X * prj.Y * prj.AngN;
  const long long ns = (long long)vol.X * vol.Y * (slice_end - slice_start);
  if (3 * np + ns > (long long)MTR_NOALLOC_SCRATCH_FLOATS)
    return set_error(ctx, MTR_ERR_CAPACITY,
                     "mtr_sirt_noalloc: 3*AngN*Y*X + X*Y*(slice_end-slice_start) = " + std::to_string(3 * np + ns) +
                         " floats exceeds the fixed scratch of " + std::to_string((long long)MTR_NOALLOC_SCRATCH_FLOATS) +
                         " floats; use mtr_sirt");
  DeviceGuard g(ctx->device);
  float* scratch = nullptr;
  cudaError_t e = scratch_on_device(ctx->device, &scratch);
  if (e != cudaSuccess) return cuda_error(ctx, e, "cudaGetSymbolAddress(scratch)");
  float* sbuf = scratch;       // ray sums, zero at the start of every forward pass
  float* cf = sbuf + np;       // row sums A 1
  float* r = cf + np;          // residual
  float* cbp = r + np;         // back-projection weight sums A^T 1 over the slab
  cudaStream_t st = ctx->stream;
  MTR_CK(ctx, cudaMemsetAsync(sbuf, 0, sizeof(float) * 2 * np, st));  // s and cf start at zero
  const AxisDev ax{prj.X, prj.Y, prj.AngN, x_coef_dev, y_coef_dev, prj.X};
  const VolDev v{vol.Xstart, vol.Ystart, slice_start, vol.X, vol.Y, slice_end - slice_start};
  launch_forward<float>(ax, v, nullptr, cf, slice_start, slice_end, st);
  MTR_CK_LAUNCH(ctx, "noalloc row sums");
  launch_backproject<float>(ax, v, prj_dev, 2, 0.f, nullptr, cbp, nullptr, 0, slice_start, slice_end, st);
  MTR_CK_LAUNCH(ctx, "noalloc weight sums");
  for (int it = 0; it < n_inner; ++it) {
    launch_forward<float>(ax, v, slab_dev, sbuf, slice_start, slice_end, st);
    MTR_CK_LAUNCH(ctx, "noalloc forward");
    launch_residual<float, float>(np, prj_dev, sbuf, cf, r, nullptr, st);  // also re-zeroes s
    MTR_CK_LAUNCH(ctx, "noalloc residual");
    launch_backproject<float>(ax, v, r, 1, sirt_step, slab_dev, cbp, nullptr, 0, slice_start, slice_end, st);
    MTR_CK_LAUNCH(ctx, "noalloc back-projection");
  }
  return MTR_OK;
}
