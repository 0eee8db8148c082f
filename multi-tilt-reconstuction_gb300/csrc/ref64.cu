// All-FP64 reconstruction on the GPU: the error reference for the FP32 and
// mixed-precision paths at full benchmark sizes, where the CPU FP64 oracle
// would take hours.  Every quantity is double: the affine map per voxel and
// angle (as the reference's computeWeight, FunctionOnGPU.cu:12-25), the
// bilinear weights, the splat (double atomics) and gather sums, the residual
// and the MACE state.  It is validated against the CPU FP64 oracle.
// Throughput is not a goal here (GB300's FP64 rate is a small fraction of
// its FP32 rate).
#include <cmath>
#include <vector>

#include "mtr_internal.h"
#include "mtr_runtime.h"

using namespace mtr;

namespace {

struct Tap64 {
  int ix, iy;
  double dx, dy;
};

__device__ __forceinline__ Tap64 map64(const double* xc, const double* yc, int a, int X, int Y, int Z) {
  const double* cx = xc + 4 * a;
  const double* cy = yc + 4 * a;
  const double x = cx[0] + cx[1] * X + cx[2] * Y + cx[3] * Z - 1.0;
  const double y = cy[0] + cy[1] * X + cy[2] * Y + cy[3] * Z - 1.0;
  Tap64 t;
  const double fx = floor(fmin(fmax(x, -1.0e9), 1.0e9)), fy = floor(fmin(fmax(y, -1.0e9), 1.0e9));
  t.ix = (int)fx;
  t.iy = (int)fy;
  t.dx = x - fx;
  t.dy = y - fy;
  return t;
}

// mode 0: WBP (out = s/c, cbp = c); mode 1: SIRT update (out += step*s/cbp)
__global__ void bp64_kernel(AxisDev ax, VolDev vol, const double* __restrict__ img, int mode, double step,
                            double* __restrict__ out, double* __restrict__ cbp) {
  const long long n = (long long)vol.NX * vol.NY * vol.NZ;
  const long long plane = (long long)ax.PX * ax.PY;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int X = vol.Xs + (int)(i % vol.NX);
    const int Y = vol.Ys + (int)((i / vol.NX) % vol.NY);
    const int Z = vol.Zs + (int)(i / ((long long)vol.NX * vol.NY));
    double s = 0.0, c = 0.0;
    for (int a = 0; a < ax.A; ++a) {
      const Tap64 t = map64(ax.xc, ax.yc, a, X, Y, Z);
      const double* im = img + plane * a;
      const double w[4] = {(1 - t.dx) * (1 - t.dy), t.dx * (1 - t.dy), (1 - t.dx) * t.dy, t.dx * t.dy};
      const int xs[4] = {t.ix, t.ix + 1, t.ix, t.ix + 1};
      const int ys[4] = {t.iy, t.iy, t.iy + 1, t.iy + 1};
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        if ((unsigned)xs[q] < (unsigned)ax.PX && (unsigned)ys[q] < (unsigned)ax.PY) {
          s += w[q] * im[xs[q] + (long long)ys[q] * ax.PX];
          c += w[q];
        }
      }
    }
    if (mode == 0) {
      out[i] = c != 0.0 ? s / c : 0.0;
      cbp[i] = c;
    } else if (cbp[i] != 0.0) {
      out[i] += step * (s / cbp[i]);
    }
  }
}

__global__ void fwd64_kernel(AxisDev ax, VolDev vol, const double* __restrict__ x, double* __restrict__ s) {
  const long long n = (long long)vol.NX * vol.NY * vol.NZ;
  const long long plane = (long long)ax.PX * ax.PY;
  const long long total = n * ax.A;
  for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < total;
       j += (long long)gridDim.x * blockDim.x) {
    const long long i = j % n;
    const int a = (int)(j / n);
    const int X = vol.Xs + (int)(i % vol.NX);
    const int Y = vol.Ys + (int)((i / vol.NX) % vol.NY);
    const int Z = vol.Zs + (int)(i / ((long long)vol.NX * vol.NY));
    const double v = x ? x[i] : 1.0;
    const Tap64 t = map64(ax.xc, ax.yc, a, X, Y, Z);
    double* sp = s + plane * a;
    const double w[4] = {(1 - t.dx) * (1 - t.dy), t.dx * (1 - t.dy), (1 - t.dx) * t.dy, t.dx * t.dy};
    const int xs[4] = {t.ix, t.ix + 1, t.ix, t.ix + 1};
    const int ys[4] = {t.iy, t.iy, t.iy + 1, t.iy + 1};
#pragma unroll
    for (int q = 0; q < 4; ++q)
      if ((unsigned)xs[q] < (unsigned)ax.PX && (unsigned)ys[q] < (unsigned)ax.PY)
        atomicAdd(sp + xs[q] + (long long)ys[q] * ax.PX, w[q] * v);
  }
}

__global__ void residual64_kernel(long long n, const double* __restrict__ b, double* __restrict__ s,
                                  const double* __restrict__ c, double* __restrict__ r) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    double sv = s[i];
    if (c[i] != 0.0) sv /= c[i];
    r[i] = b[i] - sv;
    s[i] = 0.0;
  }
}

__global__ void f2d_kernel(const float* __restrict__ a, double* __restrict__ b, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    b[i] = a[i];
}

__global__ void add64_kernel(double* __restrict__ a, const double* __restrict__ b, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    a[i] += b[i];
}

constexpr int kMaxK = MTR_MAX_AXES;
struct Mace64Ptrs {
  double* w[kMaxK];
  double* x[kMaxK];
};

__global__ void mace64_kernel(int K, Mace64Ptrs P, double* __restrict__ wavg, long long n, double rho) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double wa = wavg[i];
    double sum = 0.0;
    for (int k = 0; k < K; ++k) {
      const double wk = P.w[k][i];
      const double zk = 2.0 * wa - wk;
      const double nw = rho * (2.0 * P.x[k][i] - zk) + (1.0 - rho) * wk;
      P.w[k][i] = nw;
      sum += nw;
    }
    const double na = sum / K;
    wavg[i] = na;
    for (int k = 0; k < K; ++k) P.x[k][i] = 2.0 * na - P.w[k][i];
  }
}

unsigned grid_for(long long n) {
  long long b = (n + 255) / 256;
  const long long cap = (long long)device_sm_count() * 16;
  if (b > cap) b = cap;
  return (unsigned)(b < 1 ? 1 : b);
}

}  // namespace

extern "C" mtr_status mtr_reconstruct_fp64(mtr_context* ctx, int n_axes, const mtr_axis* axes, mtr_volume_size vol,
                                           const mtr_params* params, double* out_volume, int mem_kind) {
  if (!ctx || !axes || !params || !out_volume || n_axes <= 0 || n_axes > MTR_MAX_AXES)
    return set_error(ctx, MTR_ERR_INVALID_ARGUMENT, "invalid argument");
  mtr_status st = check_volume(ctx, vol);
  if (st != MTR_OK) return st;
  for (int k = 0; k < n_axes; ++k)
    if ((st = check_axis(ctx, axes[k])) != MTR_OK) return st;
  DeviceGuard g(ctx->device);
  cudaStream_t s = ctx->stream;
  const long long nv = (long long)vol.X * vol.Y * vol.Z;
  const VolDev v{vol.Xstart, vol.Ystart, vol.Zstart, vol.X, vol.Y, vol.Z};
  struct Ax {
    DevBuf xc, yc, b, sb, cf, r, cbp, w, x;
    AxisDev dev;
    long long np;
  };
  std::vector<Ax> ax(n_axes);
  DevBuf wavg, tmp;
  MTR_CK(ctx, wavg.alloc(nv * 8));
  MTR_CK(ctx, tmp.alloc(nv * 8));
  for (int k = 0; k < n_axes; ++k) {
    Ax& a = ax[k];
    const mtr_axis& in = axes[k];
    a.np = (long long)in.prj.X * in.prj.Y * in.prj.AngN;
    MTR_CK(ctx, a.xc.alloc(sizeof(double) * 4 * in.prj.AngN));
    MTR_CK(ctx, a.yc.alloc(sizeof(double) * 4 * in.prj.AngN));
    MTR_CK(ctx, a.b.alloc(a.np * 8));
    MTR_CK(ctx, a.sb.alloc(a.np * 8));
    MTR_CK(ctx, a.cf.alloc(a.np * 8));
    MTR_CK(ctx, a.r.alloc(a.np * 8));
    MTR_CK(ctx, a.cbp.alloc(nv * 8));
    MTR_CK(ctx, a.w.alloc(nv * 8));
    MTR_CK(ctx, a.x.alloc(nv * 8));
    MTR_CK(ctx, cudaMemcpyAsync(a.xc.p, in.x_coef, sizeof(double) * 4 * in.prj.AngN, cudaMemcpyHostToDevice, s));
    MTR_CK(ctx, cudaMemcpyAsync(a.yc.p, in.y_coef, sizeof(double) * 4 * in.prj.AngN, cudaMemcpyHostToDevice, s));
    // stage the float projections in r, widen to double in b
    MTR_CK(ctx, cudaMemcpyAsync(a.r.p, in.prj_data, a.np * 4,
                                mem_kind == MTR_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
    f2d_kernel<<<grid_for(a.np), 256, 0, s>>>(a.r.as<float>(), a.b.as<double>(), a.np);
    MTR_CK_LAUNCH(ctx, "widen projections");
    a.dev = AxisDev{in.prj.X, in.prj.Y, in.prj.AngN, a.xc.as<double>(), a.yc.as<double>(), in.prj.X};
    MTR_CK(ctx, cudaMemsetAsync(a.sb.p, 0, a.np * 8, s));
    MTR_CK(ctx, cudaMemsetAsync(a.cf.p, 0, a.np * 8, s));
    fwd64_kernel<<<grid_for(nv * in.prj.AngN), 256, 0, s>>>(a.dev, v, nullptr, a.cf.as<double>());
    MTR_CK_LAUNCH(ctx, "fp64 row sums");
  }
  MTR_CK(ctx, cudaMemsetAsync(wavg.p, 0, nv * 8, s));
  for (auto& a : ax) {
    bp64_kernel<<<grid_for(nv), 256, 0, s>>>(a.dev, v, a.b.as<double>(), 0, 0.0, tmp.as<double>(),
                                             a.cbp.as<double>());
    MTR_CK_LAUNCH(ctx, "fp64 wbp");
    add64_kernel<<<grid_for(nv), 256, 0, s>>>(wavg.as<double>(), tmp.as<double>(), nv);
    MTR_CK_LAUNCH(ctx, "fp64 sum");
  }
  Mace64Ptrs P{};
  for (int k = 0; k < n_axes; ++k) {
    MTR_CK(ctx, cudaMemcpyAsync(ax[k].w.p, wavg.p, nv * 8, cudaMemcpyDeviceToDevice, s));
    MTR_CK(ctx, cudaMemcpyAsync(ax[k].x.p, wavg.p, nv * 8, cudaMemcpyDeviceToDevice, s));
    P.w[k] = ax[k].w.as<double>();
    P.x[k] = ax[k].x.as<double>();
  }
  for (int it = 0; it < params->iter_times; ++it) {
    for (auto& a : ax) {
      for (int j = 0; j < params->sirt_inner; ++j) {
        fwd64_kernel<<<grid_for(nv * a.dev.A), 256, 0, s>>>(a.dev, v, a.x.as<double>(), a.sb.as<double>());
        MTR_CK_LAUNCH(ctx, "fp64 forward");
        residual64_kernel<<<grid_for(a.np), 256, 0, s>>>(a.np, a.b.as<double>(), a.sb.as<double>(),
                                                         a.cf.as<double>(), a.r.as<double>());
        MTR_CK_LAUNCH(ctx, "fp64 residual");
        bp64_kernel<<<grid_for(nv), 256, 0, s>>>(a.dev, v, a.r.as<double>(), 1, (double)params->sirt_step,
                                                 a.x.as<double>(), a.cbp.as<double>());
        MTR_CK_LAUNCH(ctx, "fp64 back-projection");
      }
    }
    mace64_kernel<<<grid_for(nv), 256, 0, s>>>(n_axes, P, wavg.as<double>(), nv, (double)params->mace_step);
    MTR_CK_LAUNCH(ctx, "fp64 mace");
  }
  MTR_CK(ctx, cudaMemcpyAsync(out_volume, wavg.p, nv * 8,
                              mem_kind == MTR_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, s));
  MTR_CK(ctx, cudaStreamSynchronize(s));
  return MTR_OK;
}
