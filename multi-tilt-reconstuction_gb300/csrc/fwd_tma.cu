// Forward projection (bilinear splat) with shared-memory detector windows
// and TMA bulk reduce-add (sm_103a).
//
// The reference adds every voxel's four bilinear weights into the projection
// with global float atomics (FunctionOnGPU.cu:27-52, 316-333): eight atomics
// per voxel and angle, contending along every ray.  Here one CTA owns a
// brick of BX x BY x NZ voxels, held in registers for the whole launch.  For
// each angle it splats the brick into a private detector window in shared
// memory (shared-memory atomics, no global traffic), then one thread flushes
// the window to the ray-sum array with a single 3-D tiled
// cp.reduce.async.bulk.tensor add (the L2 performs the reduction on whole
// sectors).  Two window stages alternate so the flush of angle a overlaps
// the splat of angle a+1.
//
// Windows are clamped inside the detector (TMA reduces must not start at a
// negative coordinate), so a window tap is on the detector iff it lies in the
// window; taps off the detector are dropped as in the reference.
#include "mtr_internal.h"
#include "tma.cuh"

namespace mtr {
namespace {

constexpr int kWarps = 8;
constexpr int kThreads = kWarps * 32;
constexpr float kMagic = 12582912.0f;
constexpr int kMagicBits = 0x4B400000;

struct FwdConst {
  float xf, a1, a2, a3;
  float yf, b1, b2, b3;
  int lxm, lym;  // window-local integer base minus the magic bits
  int ox, oy;    // window origin (clamped inside the detector, ox aligned)
  int wlx;       // valid window columns (window part left of the detector's right edge)
  int pad[3];
};

struct FwdArgs {
  AxisDev ax;
  VolDev vol;
  int z0, z1;
  int WX, WY;
  const void* x;   // volume (nullptr: ones)
  int* err;
};

__device__ __forceinline__ int magic_int(float integral) { return __float_as_int(__fadd_rn(integral, kMagic)); }
__device__ __forceinline__ int floor_div(int a, int b) { return (a >= 0) ? a / b : -((-a + b - 1) / b); }

template <typename VT> __device__ __forceinline__ float ldv(const void* p, long long i);
template <> __device__ __forceinline__ float ldv<float>(const void* p, long long i) {
  return __ldg(static_cast<const float*>(p) + i);
}
template <> __device__ __forceinline__ float ldv<__nv_bfloat16>(const void* p, long long i) {
  return __bfloat162float(__ldg(static_cast<const __nv_bfloat16*>(p) + i));
}
template <> __device__ __forceinline__ float ldv<__half>(const void* p, long long i) {
  return __half2float(__ldg(static_cast<const __half*>(p) + i));
}

template <typename VT, bool LANE_Y, bool BZ0, int NZ>
__global__ void __launch_bounds__(kThreads)
fwd_tma_kernel(const __grid_constant__ CUtensorMap smap, const FwdArgs P) {
  constexpr int BX = LANE_Y ? kWarps : 32;
  constexpr int BY = LANE_Y ? 32 : kWarps;
  extern __shared__ __align__(128) unsigned char smem[];
  const int A = P.ax.A;
  FwdConst* kc = reinterpret_cast<FwdConst*>(smem);
  const size_t kc_bytes = ((size_t)A * sizeof(FwdConst) + 127) & ~(size_t)127;
  const int WX = P.WX, WY = P.WY;
  const int win_elems = WX * WY;
  const size_t stage_bytes = ((size_t)win_elems * 4 + 127) & ~(size_t)127;
  float* win0 = reinterpret_cast<float*>(smem + kc_bytes);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int X0 = P.vol.Xs + blockIdx.x * BX;
  const int Y0 = P.vol.Ys + blockIdx.y * BY;
  const int Z0 = P.z0 + blockIdx.z * NZ;
  const int PX = P.ax.PX, PY = P.ax.PY;

  for (int a = tid; a < A; a += kThreads) {
    const double* cx = P.ax.xc + 4 * a;
    const double* cy = P.ax.yc + 4 * a;
    const double xb = cx[0] + cx[1] * X0 + cx[2] * Y0 + cx[3] * Z0 - 1.0;
    const double yb = cy[0] + cy[1] * X0 + cy[2] * Y0 + cy[3] * Z0 - 1.0;
    const double fxb = floor(fmin(fmax(xb, -1.0e9), 1.0e9)), fyb = floor(fmin(fmax(yb, -1.0e9), 1.0e9));
    FwdConst k;
    k.xf = (float)(xb - fxb);
    k.yf = (float)(yb - fyb);
    k.a1 = (float)cx[1]; k.a2 = (float)cx[2]; k.a3 = (float)cx[3];
    k.b1 = (float)cy[1]; k.b2 = (float)cy[2]; k.b3 = (float)cy[3];
    const int xi = (int)fxb, yi = (int)fyb;
    const float xmin = k.xf + fminf(0.f, k.a1 * (BX - 1)) + fminf(0.f, k.a2 * (BY - 1)) + fminf(0.f, k.a3 * (NZ - 1));
    const float ymin = k.yf + fminf(0.f, k.b1 * (BX - 1)) + fminf(0.f, k.b2 * (BY - 1)) + fminf(0.f, k.b3 * (NZ - 1));
    int ox = floor_div(xi + (int)floorf(xmin) - 1, 4) * 4;
    int oy = yi + (int)floorf(ymin) - 1;
    // clamp inside [0, pitch - WX] x [0, PY - WY]; the host guarantees both ranges exist
    ox = min(max(ox, 0), P.ax.pitch - WX);
    oy = min(max(oy, 0), PY - WY);
    k.ox = ox;
    k.oy = oy;
    k.lxm = xi - ox - kMagicBits;
    k.lym = yi - oy - kMagicBits;
    k.wlx = min(WX, PX - ox);
    kc[a] = k;
  }

  // own voxels, loaded once (coalesced along lanes)
  const int tx = LANE_Y ? warp : lane;
  const int ty = LANE_Y ? lane : warp;
  const bool active = (X0 + tx < P.vol.Xs + P.vol.NX) && (Y0 + ty < P.vol.Ys + P.vol.NY);
  float v[NZ];
  {
    const long long sx = P.vol.NX, sxy = (long long)P.vol.NX * P.vol.NY;
    const long long base = (long long)(X0 + tx - P.vol.Xs) + (long long)(Y0 + ty - P.vol.Ys) * sx;
#pragma unroll
    for (int z = 0; z < NZ; ++z) {
      const int zz = Z0 + z;
      v[z] = 0.f;
      if (active && zz < P.z1) v[z] = P.x ? ldv<VT>(P.x, base + (long long)(zz - P.z0) * sxy) : 1.f;
    }
  }
  __syncthreads();
  if (tid == 0) prefetch_tensormap(&smap);

  bool bad = false;
  for (int a = 0; a < A; ++a) {
    const int st = a & 1;
    float* w = reinterpret_cast<float*>(reinterpret_cast<unsigned char*>(win0) + st * stage_bytes);
    // the bulk reduce that last read this stage (angle a-2) must be done reading
    if (tid == 0 && a >= 2) bulk_wait_read<1>();
    __syncthreads();
    for (int i = tid * 4; i < win_elems; i += kThreads * 4) {
      if (i + 3 < win_elems) *reinterpret_cast<float4*>(w + i) = make_float4(0.f, 0.f, 0.f, 0.f);
      else
        for (int j = i; j < win_elems; ++j) w[j] = 0.f;
    }
    __syncthreads();
    const FwdConst k = kc[a];
    if (active) {
      const float xr = fmaf(k.a2, (float)ty, fmaf(k.a1, (float)tx, k.xf));
      const float yr = fmaf(k.b2, (float)ty, fmaf(k.b1, (float)tx, k.yf));
      float wy0 = 0.f, wy1 = 0.f;
      int rowi = 0;
      bool y0ok = false, y1ok = false;
      if (BZ0) {
        const float fly = floorf(yr);
        const float fy = yr - fly;
        rowi = magic_int(fly) + k.lym;
        wy0 = 1.f - fy;
        wy1 = fy;
        y0ok = (unsigned)rowi < (unsigned)WY;
        y1ok = (unsigned)(rowi + 1) < (unsigned)WY;
      }
#pragma unroll
      for (int z = 0; z < NZ; ++z) {
        if (!BZ0) {
          const float y = fmaf(k.b3, (float)z, yr);
          const float fly = floorf(y);
          const float fy = y - fly;
          rowi = magic_int(fly) + k.lym;
          wy0 = 1.f - fy;
          wy1 = fy;
          y0ok = (unsigned)rowi < (unsigned)WY;
          y1ok = (unsigned)(rowi + 1) < (unsigned)WY;
        }
        const float x = fmaf(k.a3, (float)z, xr);
        const float flx = floorf(x);
        const float fx = x - flx;
        const int ix = magic_int(flx) + k.lxm;
        const bool x0ok = (unsigned)ix < (unsigned)k.wlx;
        const bool x1ok = (unsigned)(ix + 1) < (unsigned)k.wlx;
        const float g0 = wy0 * v[z], g1 = wy1 * v[z];
        float* r0 = w + (rowi * WX + ix);
        if (y0ok) {
          if (x0ok) atomicAdd(r0, g0 - fx * g0);
          if (x1ok) atomicAdd(r0 + 1, fx * g0);
        }
        if (y1ok) {
          if (x0ok) atomicAdd(r0 + WX, g1 - fx * g1);
          if (x1ok) atomicAdd(r0 + WX + 1, fx * g1);
        }
      }
    }
    fence_proxy_async_smem();
    __syncthreads();
    if (tid == 0) {
      tma_reduce_add_3d(&smap, w, k.ox, k.oy, a);
      bulk_commit();
    }
  }
  if (tid == 0) bulk_wait_all();
  if (bad && P.err) atomicExch(P.err, 6);
}

template <typename VT, bool LY, bool BZ>
cudaError_t launch_one(const CUtensorMap& map, const FwdArgs& P, size_t smem, cudaStream_t st) {
  constexpr int NZ = 16;
  auto kern = fwd_tma_kernel<VT, LY, BZ, NZ>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const int BX = LY ? kWarps : 32, BY = LY ? 32 : kWarps;
  const dim3 grid((P.vol.NX + BX - 1) / BX, (P.vol.NY + BY - 1) / BY, (P.z1 - P.z0 + NZ - 1) / NZ);
  kern<<<grid, kThreads, smem, st>>>(map, P);
  return cudaGetLastError();
}

}  // namespace

FwdPlan plan_forward(const std::vector<double>& xc, const std::vector<double>& yc, int A, int PX, int PY, int pitch) {
  FwdPlan p;
  double sx = 0, sy = 0;
  bool bz0 = true;
  for (int a = 0; a < A; ++a) {
    sx += std::fabs(xc[4 * a + 1]) - std::fabs(yc[4 * a + 1]);
    sy += std::fabs(xc[4 * a + 2]) - std::fabs(yc[4 * a + 2]);
    if (yc[4 * a + 3] != 0.0) bz0 = false;
  }
  p.lane_y = sy > sx;
  p.bz0 = bz0;
  const int BX = p.lane_y ? kWarps : 32, BY = p.lane_y ? 32 : kWarps, BZ = 16;
  double ex = 0, ey = 0;
  for (int a = 0; a < A; ++a) {
    ex = std::max(ex, std::fabs(xc[4 * a + 1]) * (BX - 1) + std::fabs(xc[4 * a + 2]) * (BY - 1) +
                          std::fabs(xc[4 * a + 3]) * (BZ - 1));
    ey = std::max(ey, std::fabs(yc[4 * a + 1]) * (BX - 1) + std::fabs(yc[4 * a + 2]) * (BY - 1) +
                          std::fabs(yc[4 * a + 3]) * (BZ - 1));
  }
  p.WX = ((int)std::ceil(ex) + 4 + 4 + 3) / 4 * 4;
  p.WY = (int)std::ceil(ey) + 4;
  const size_t stage = (((size_t)p.WX * p.WY * 4) + 127) & ~(size_t)127;
  p.smem = ((((size_t)A * sizeof(FwdConst)) + 127) & ~(size_t)127) + 2 * stage;
  p.ok = p.WX <= 256 && p.WY <= 256 && p.WX <= pitch && p.WY <= PY && p.smem <= 200 * 1024;
  (void)PX;
  return p;
}

template <typename VT>
cudaError_t launch_forward_tma(const CUtensorMap& smap, const FwdPlan& plan, const AxisDev& ax, const VolDev& vol,
                               const VT* x, int z0, int z1, int* err, cudaStream_t st) {
  FwdArgs P{ax, vol, z0, z1, plan.WX, plan.WY, x, err};
  if (!plan.lane_y && plan.bz0) return launch_one<VT, false, true>(smap, P, plan.smem, st);
  if (!plan.lane_y && !plan.bz0) return launch_one<VT, false, false>(smap, P, plan.smem, st);
  if (plan.lane_y && plan.bz0) return launch_one<VT, true, true>(smap, P, plan.smem, st);
  return launch_one<VT, true, false>(smap, P, plan.smem, st);
}

template cudaError_t launch_forward_tma<float>(const CUtensorMap&, const FwdPlan&, const AxisDev&, const VolDev&,
                                               const float*, int, int, int*, cudaStream_t);
template cudaError_t launch_forward_tma<__nv_bfloat16>(const CUtensorMap&, const FwdPlan&, const AxisDev&,
                                                       const VolDev&, const __nv_bfloat16*, int, int, int*,
                                                       cudaStream_t);
template cudaError_t launch_forward_tma<__half>(const CUtensorMap&, const FwdPlan&, const AxisDev&, const VolDev&,
                                                const __half*, int, int, int*, cudaStream_t);

}  // namespace mtr
