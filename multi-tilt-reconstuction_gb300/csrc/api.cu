// C ABI of libmtr: context, device-resident reconstruction objects and the
// entry points that replace the reference's FunctionOnGPU.cuh:41-44 and the
// MACE driver of MultiAxis.cpp.  No entry point prints or exits; errors come
// back as mtr_status with a message in the context.
#include <atomic>
#include <cmath>
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

// ---------------------------------------------------------------------------
// Context
// ---------------------------------------------------------------------------

std::atomic<long long> mtr::g_launches{0};
std::atomic<long long> mtr::g_windowed_launches{0};

namespace {

const char* kStatusNames[] = {"ok",          "invalid argument", "CUDA error",   "out of device memory",
                              "I/O error",   "format error",     "unsupported",  "no CUDA device",
                              "timed out",   "not ready",        "over capacity"};

}  // namespace

mtr_status mtr::set_error(mtr_context* ctx, mtr_status s, const std::string& msg) {
  if (ctx) ctx->last_error = msg;
  return s;
}

mtr_status mtr::cuda_error(mtr_context* ctx, cudaError_t e, const char* what) {
  std::string m = std::string(what) + ": " + cudaGetErrorString(e);
  cudaGetLastError();  // clear a sticky-free error so the context stays usable
  if (e == cudaErrorMemoryAllocation) return set_error(ctx, MTR_ERR_OUT_OF_MEMORY, m);
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return set_error(ctx, MTR_ERR_NO_DEVICE, m);
  return set_error(ctx, MTR_ERR_CUDA, m);
}

extern "C" {

int mtr_abi_version(void) { return MTR_ABI_VERSION; }

const char* mtr_status_string(mtr_status s) {
  const int i = (int)s;
  if (i < 0 || i >= (int)(sizeof(kStatusNames) / sizeof(kStatusNames[0]))) return "unknown status";
  return kStatusNames[i];
}

const char* mtr_context_last_error(const mtr_context* ctx) { return ctx ? ctx->last_error.c_str() : ""; }

void mtr_params_default(mtr_params* p) {
  if (!p) return;
  p->iter_times = 5;
  p->sirt_inner = MTR_DEFAULT_SIRT_INNER;
  p->sirt_step = 0.5f;
  p->mace_step = 0.7f;
  p->precision = MTR_PREC_FP32;
  p->flags = 0;
  p->slab_depth = 0;
}

mtr_status mtr_context_create(int device, mtr_context** out) {
  if (!out) return MTR_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    cudaGetLastError();
    return MTR_ERR_NO_DEVICE;
  }
  if (device < 0) {
    if (cudaGetDevice(&device) != cudaSuccess) return MTR_ERR_NO_DEVICE;
  }
  if (device >= n) return MTR_ERR_INVALID_ARGUMENT;
  std::unique_ptr<mtr_context> ctx(new (std::nothrow) mtr_context());
  if (!ctx) return MTR_ERR_OUT_OF_MEMORY;
  ctx->device = device;
  DeviceGuard g(device);
  e = cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) return cuda_error(nullptr, e, "cudaStreamCreate");
  ctx->stream = ctx->own_stream;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) == cudaSuccess) {
    ctx->num_sms = prop.multiProcessorCount;
    ctx->cc_major = prop.major;
    ctx->cc_minor = prop.minor;
  }
  *out = ctx.release();
  return MTR_OK;
}

mtr_status mtr_context_destroy(mtr_context* ctx) {
  if (!ctx) return MTR_OK;
  {
    DeviceGuard g(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    for (auto& r : ctx->prof_pending) {
      cudaEventDestroy(r.a);
      cudaEventDestroy(r.b);
    }
    for (cudaEvent_t e : ctx->event_pool) cudaEventDestroy(e);
    for (cudaStream_t s : ctx->side_streams) {
      cudaStreamSynchronize(s);
      cudaStreamDestroy(s);
    }
    for (cudaEvent_t e : ctx->sync_events) cudaEventDestroy(e);
    if (ctx->own_stream) cudaStreamSynchronize(ctx->own_stream);
    // (a pool with arrays still allocated is released when they are freed)
    if (ctx->pool) cudaMemPoolDestroy(ctx->pool);
    if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
  }
  delete ctx;
  return MTR_OK;
}

mtr_status mtr_context_trim(mtr_context* ctx) {
  if (!ctx) return MTR_ERR_INVALID_ARGUMENT;
  DeviceGuard g(ctx->device);
  if (!ctx->pool) return MTR_OK;
  cudaError_t e = cudaStreamSynchronize(ctx->own_stream);
  if (e != cudaSuccess) return cuda_error(ctx, e, "cudaStreamSynchronize");
  e = cudaMemPoolTrimTo(ctx->pool, 0);
  if (e != cudaSuccess) return cuda_error(ctx, e, "cudaMemPoolTrimTo");
  return MTR_OK;
}

mtr_status mtr_context_set_stream(mtr_context* ctx, void* cuda_stream) {
  if (!ctx) return MTR_ERR_INVALID_ARGUMENT;
  ctx->stream = cuda_stream ? (cudaStream_t)cuda_stream : ctx->own_stream;
  return MTR_OK;
}

mtr_status mtr_context_synchronize(mtr_context* ctx) {
  if (!ctx) return MTR_ERR_INVALID_ARGUMENT;
  DeviceGuard g(ctx->device);
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_error(ctx, e, "cudaStreamSynchronize");
  return MTR_OK;
}

mtr_status mtr_context_launch_count(const mtr_context* ctx, long long* out) {
  if (!out) return MTR_ERR_INVALID_ARGUMENT;
  (void)ctx;
  *out = g_launches.load();
  return MTR_OK;
}

mtr_status mtr_set_wait_limit(long long polls) {
  set_pipeline_wait_limit(polls);
  return MTR_OK;
}

mtr_status mtr_context_windowed_launch_count(const mtr_context* ctx, long long* out) {
  if (!out) return MTR_ERR_INVALID_ARGUMENT;
  (void)ctx;
  *out = g_windowed_launches.load();
  return MTR_OK;
}

mtr_status mtr_context_set_profiling(mtr_context* ctx, int enable) {
  if (!ctx) return MTR_ERR_INVALID_ARGUMENT;
  ctx->profiling = enable != 0;
  return MTR_OK;
}

mtr_status mtr_context_profile(mtr_context* ctx, int kernel_class, long long* launches, double* total_ms) {
  if (!ctx || kernel_class < 0 || kernel_class >= MTR_KERNEL_CLASSES) return MTR_ERR_INVALID_ARGUMENT;
  DeviceGuard g(ctx->device);
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_error(ctx, e, "cudaStreamSynchronize");
  for (auto& r : ctx->prof_pending) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess) {
      ctx->prof_ms[r.kind] += ms;
      ctx->prof_count[r.kind] += 1;
    }
    ctx->event_pool.push_back(r.a);
    ctx->event_pool.push_back(r.b);
  }
  ctx->prof_pending.clear();
  if (launches) *launches = ctx->prof_count[kernel_class];
  if (total_ms) *total_ms = ctx->prof_ms[kernel_class];
  return MTR_OK;
}

mtr_status mtr_context_profile_reset(mtr_context* ctx) {
  if (!ctx) return MTR_ERR_INVALID_ARGUMENT;
  mtr_context_profile(ctx, 0, nullptr, nullptr);
  for (int i = 0; i < MTR_KERNEL_CLASSES; ++i) {
    ctx->prof_count[i] = 0;
    ctx->prof_ms[i] = 0.0;
  }
  return MTR_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Validation helpers
// ---------------------------------------------------------------------------

bool mtr::tma_disabled() {
  const char* e = std::getenv("MTR_DISABLE_TMA");
  return e && e[0] == '1';
}

mtr_status mtr::check_volume(mtr_context* ctx, const mtr_volume_size& v) {
  if (v.X != v.Xend - v.Xstart || v.Y != v.Yend - v.Ystart || v.Z != v.Zend - v.Zstart)
    return set_error(ctx, MTR_ERR_INVALID_ARGUMENT, "volume size: X/Y/Z must equal end - start");
  if (v.X <= 0 || v.Y <= 0 || v.Z <= 0) return set_error(ctx, MTR_ERR_INVALID_ARGUMENT, "volume size: empty volume");
  if ((long long)v.X * v.Y * v.Z > (1LL << 40)) return set_error(ctx, MTR_ERR_INVALID_ARGUMENT, "volume too large");
  return MTR_OK;
}

mtr_status mtr::check_axis(mtr_context* ctx, const mtr_axis& a, bool data_required) {
  if (a.prj.X <= 0 || a.prj.Y <= 0 || a.prj.AngN <= 0)
    return set_error(ctx, MTR_ERR_INVALID_ARGUMENT, "projection size: X, Y and AngN must be positive");
  if (a.prj.AngN > kMaxAngles) return set_error(ctx, MTR_ERR_UNSUPPORTED, "more angles than supported");
  if (!a.x_coef || !a.y_coef || (data_required && !a.prj_data))
    return set_error(ctx, MTR_ERR_INVALID_ARGUMENT, "axis: null coefficient or data pointer");
  for (int i = 0; i < 4 * a.prj.AngN; ++i)
    if (!std::isfinite(a.x_coef[i]) || !std::isfinite(a.y_coef[i]))
      return set_error(ctx, MTR_ERR_INVALID_ARGUMENT, "axis: non-finite projection coefficient");
  return MTR_OK;
}
