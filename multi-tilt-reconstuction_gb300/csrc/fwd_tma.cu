// Forward projection (bilinear splat) with shared-memory detector windows
// and TMA bulk reduce-add (sm_103a).
//
// The reference adds every voxel's four bilinear weights into the projection
// with global float atomics (FunctionOnGPU.cu:27-52, 316-333): eight atomics
// per voxel and angle, contending along every ray.  Here one CTA owns a
// brick of BX x BY x NZ voxels, held in registers for the whole launch.  For
// each of its angles it splats the brick into a private detector window in
// shared memory, then one thread flushes the window into the ray-sum array
// with a single 3-D tiled cp.reduce.async.bulk.tensor add (the L2 reduces
// whole sectors).  Two window stages alternate so the flush of one angle
// overlaps the splat of the next.
//
// Window accumulation is fixed point: shared-memory float atomicAdd is not a
// single native operation on this part, integer adds are.  Each CTA scales
// its voxels by a power of two S with S * max|v| < 2^b, b <= 21, so every tap
// weight*value rounds to an integer below 2^21 (rounded with the 1.5*2^23
// trick, no float->int conversion) with an absolute error of at most
// 2^-(b+1) * max|v|.  The host bounds the weight one pixel can receive from
// one brick by 2^mass_shift (lattice points in the preimage of a 2x2-pixel
// square, times the brick depth) and b = min(21, 30 - mass_shift) keeps every
// window sum below 2^30.  Before the flush the window is converted back to
// float and divided by S (exact: S is a power of two).
//
// Windows are clamped inside the detector (TMA reduces must not start at a
// negative coordinate), so a tap is on the detector iff it lies in the valid
// part of the window; taps off the detector are dropped as in the reference.
#include "mtr_internal.h"
#include "tma.cuh"

namespace mtr {
namespace {

constexpr int kWarps = 8;
constexpr int kThreads = kWarps * 32;
constexpr int kNZ = 16;
constexpr float kMagic = 12582912.0f;  // 1.5 * 2^23
constexpr int kMagicBits = 0x4B400000;

struct FwdConst {
  float xf, a1, a2, a3;
  float yf, b1, b2, b3;
  int lxm, lym;  // window-local integer base minus the magic bits
  int ox, oy;    // window origin (clamped inside the detector, ox aligned)
  int wlx;       // valid window columns (left of the detector's right edge)
  int pad[3];
};

struct FwdArgs {
  AxisDev ax;
  VolDev vol;
  int z0, z1;
  int WX, WY;
  int groups;      // angle groups (grid.z = z-blocks * groups)
  int max_angles;  // angles per group (shared-memory constants sized for it)
  int mass_shift;  // log2 bound of one pixel's total weight from one brick
  const void* x;   // volume (nullptr: ones)
  int* err;
};

__device__ __forceinline__ int magic_int(float integral) { return __float_as_int(__fadd_rn(integral, kMagic)); }
__device__ __forceinline__ int floor_div(int a, int b) { return (a >= 0) ? a / b : -((-a + b - 1) / b); }
// round(w * v) for |w*v| < 2^22, as an integer, without a conversion instruction
__device__ __forceinline__ int fixq(float w, float v) { return __float_as_int(fmaf(w, v, kMagic)) - kMagicBits; }

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

template <typename VT, bool LANE_Y, bool BZ0>
__global__ void __launch_bounds__(kThreads)
fwd_tma_kernel(const __grid_constant__ CUtensorMap smap, const FwdArgs P) {
  constexpr int NZ = kNZ;
  constexpr int BX = LANE_Y ? kWarps : 32;
  constexpr int BY = LANE_Y ? 32 : kWarps;
  extern __shared__ __align__(128) unsigned char smem[];
  FwdConst* kc = reinterpret_cast<FwdConst*>(smem);
  const size_t kc_bytes = ((size_t)P.max_angles * sizeof(FwdConst) + 127) & ~(size_t)127;
  const int WX = P.WX, WY = P.WY;
  const int win_elems = WX * WY;
  const size_t stage_bytes = ((size_t)win_elems * 4 + 127) & ~(size_t)127;
  unsigned char* win0 = smem + kc_bytes + 128;
  float* red = reinterpret_cast<float*>(smem + kc_bytes);  // 32 floats for the block max

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int zb = blockIdx.z / P.groups, g = blockIdx.z % P.groups;
  const int A = P.ax.A;
  const int a_begin = (int)((long long)A * g / P.groups), a_end = (int)((long long)A * (g + 1) / P.groups);
  const int na = a_end - a_begin;
  const int X0 = P.vol.Xs + blockIdx.x * BX;
  const int Y0 = P.vol.Ys + blockIdx.y * BY;
  const int Z0 = P.z0 + zb * NZ;
  const int PX = P.ax.PX, PY = P.ax.PY;

  for (int j = tid; j < na; j += kThreads) {
    const int a = a_begin + j;
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
    // clamp inside [0, pitch - WX] x [0, PY - WY]; the host checked both ranges exist
    ox = min(max(ox, 0), P.ax.pitch - WX);
    oy = min(max(oy, 0), PY - WY);
    k.ox = ox;
    k.oy = oy;
    k.lxm = xi - ox - kMagicBits;
    k.lym = yi - oy - kMagicBits;
    k.wlx = min(WX, PX - ox);
    kc[j] = k;
  }

  // own voxels, loaded once (coalesced along lanes), and the brick's max |v|
  const int tx = LANE_Y ? warp : lane;
  const int ty = LANE_Y ? lane : warp;
  const bool active = (X0 + tx < P.vol.Xs + P.vol.NX) && (Y0 + ty < P.vol.Ys + P.vol.NY);
  float v[NZ];
  float vmax = 0.f;
  {
    const long long sx = P.vol.NX, sxy = (long long)P.vol.NX * P.vol.NY;
    const long long base = (long long)(X0 + tx - P.vol.Xs) + (long long)(Y0 + ty - P.vol.Ys) * sx;
#pragma unroll
    for (int z = 0; z < NZ; ++z) {
      const int zz = Z0 + z;
      v[z] = 0.f;
      if (active && zz < P.z1) v[z] = P.x ? ldv<VT>(P.x, base + (long long)(zz - P.z0) * sxy) : 1.f;
      vmax = fmaxf(vmax, fabsf(v[z]));
    }
  }
  for (int o = 16; o > 0; o >>= 1) vmax = fmaxf(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
  if (lane == 0) red[warp] = vmax;
  __syncthreads();
  vmax = red[0];
  for (int w = 1; w < kWarps; ++w) vmax = fmaxf(vmax, red[w]);
  // S = 2^(b-e) with vmax < 2^e: every |w*v*S| < 2^b <= 2^21 (magic rounding
  // range) and a pixel's window sum < 2^(b + mass_shift) <= 2^30 (no overflow)
  int e2 = 0;
  if (vmax > 0.f && isfinite(vmax)) frexpf(vmax, &e2);
  const int bits = min(21, 30 - P.mass_shift);
  const int sexp = max(-120, min(120, bits - e2));
  const float S = ldexpf(1.f, sexp), invS = ldexpf(1.f, -sexp);
#pragma unroll
  for (int z = 0; z < NZ; ++z) v[z] *= S;
  if (tid == 0) prefetch_tensormap(&smap);

  for (int j = 0; j < na; ++j) {
    const int a = a_begin + j;
    const int st = j & 1;
    int* wi = reinterpret_cast<int*>(win0 + st * stage_bytes);
    float* wf = reinterpret_cast<float*>(wi);
    // the bulk reduce that last read this stage (two angles ago) must be done reading
    if (tid == 0 && j >= 2) bulk_wait_read<1>();
    __syncthreads();
    for (int i = tid * 4; i < win_elems; i += kThreads * 4) {
      if (i + 3 < win_elems) *reinterpret_cast<int4*>(wi + i) = make_int4(0, 0, 0, 0);
      else
        for (int q = i; q < win_elems; ++q) wi[q] = 0;
    }
    __syncthreads();
    const FwdConst k = kc[j];
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
        const float wx0 = 1.f - fx;
        int* r0 = wi + (rowi * WX + ix);
        if (y0ok) {
          if (x0ok) atomicAdd(r0, fixq(wx0, g0));
          if (x1ok) atomicAdd(r0 + 1, fixq(fx, g0));
        }
        if (y1ok) {
          if (x0ok) atomicAdd(r0 + WX, fixq(wx0, g1));
          if (x1ok) atomicAdd(r0 + WX + 1, fixq(fx, g1));
        }
      }
    }
    __syncthreads();
    // fixed point -> float (exact power-of-two scale), in place
    for (int i = tid; i < win_elems; i += kThreads) wf[i] = (float)wi[i] * invS;
    fence_proxy_async_smem();
    __syncthreads();
    if (tid == 0) {
      tma_reduce_add_3d(&smap, wf, k.ox, k.oy, a);
      bulk_commit();
    }
  }
  if (tid == 0) bulk_wait_all();
}

template <typename VT, bool LY, bool BZ>
cudaError_t launch_one(const CUtensorMap& map, FwdArgs P, size_t smem, int num_sms, cudaStream_t st) {
  auto kern = fwd_tma_kernel<VT, LY, BZ>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const int BX = LY ? kWarps : 32, BY = LY ? 32 : kWarps;
  const long long bricks = (long long)((P.vol.NX + BX - 1) / BX) * ((P.vol.NY + BY - 1) / BY) *
                           ((P.z1 - P.z0 + kNZ - 1) / kNZ);
  // split the angles over several CTAs when there are too few bricks to fill the GPU
  const long long target = (long long)num_sms * 8;
  int groups = (int)std::min<long long>((target + bricks - 1) / bricks, (long long)P.ax.A);
  if (groups < 1) groups = 1;
  P.groups = groups;
  P.max_angles = (P.ax.A + groups - 1) / groups;
  const dim3 grid((P.vol.NX + BX - 1) / BX, (P.vol.NY + BY - 1) / BY, ((P.z1 - P.z0 + kNZ - 1) / kNZ) * groups);
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
  const int BX = p.lane_y ? kWarps : 32, BY = p.lane_y ? 32 : kWarps, BZ = kNZ;
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
  // constants for up to A angles (one group) + block-max scratch + 2 stages
  p.smem = ((((size_t)A * sizeof(FwdConst)) + 127) & ~(size_t)127) + 128 + 2 * stage;
  // Weight a pixel can receive from one brick: per Z plane at most the number
  // of voxels whose taps reach it, i.e. lattice points in the preimage of a
  // 2x2-pixel square under the in-plane map J (bounding box of J^-1 [-1,1]^2).
  double count = 0;
  bool singular = false;
  for (int a = 0; a < A; ++a) {
    const double j00 = xc[4 * a + 1], j01 = xc[4 * a + 2], j10 = yc[4 * a + 1], j11 = yc[4 * a + 2];
    const double det = j00 * j11 - j01 * j10;
    if (std::fabs(det) < 1e-3) { singular = true; break; }
    const double wx = 2.0 * (std::fabs(j11) + std::fabs(j01)) / std::fabs(det);
    const double wy = 2.0 * (std::fabs(j10) + std::fabs(j00)) / std::fabs(det);
    count = std::max(count, (wx + 1.0) * (wy + 1.0));
  }
  p.mass_shift = (int)std::ceil(std::log2(std::max(1.0, count * BZ)));
  p.ok = !singular && p.mass_shift <= 16 && p.WX <= 256 && p.WY <= 256 && p.WX <= pitch && p.WY <= PY &&
         p.smem <= 200 * 1024;
  (void)PX;
  return p;
}

template <typename VT>
cudaError_t launch_forward_tma(const CUtensorMap& smap, const FwdPlan& plan, const AxisDev& ax, const VolDev& vol,
                               const VT* x, int z0, int z1, int* err, cudaStream_t st) {
  int dev = 0, sms = 152;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  FwdArgs P{ax, vol, z0, z1, plan.WX, plan.WY, 1, ax.A, plan.mass_shift, x, err};
  if (!plan.lane_y && plan.bz0) return launch_one<VT, false, true>(smap, P, plan.smem, sms, st);
  if (!plan.lane_y && !plan.bz0) return launch_one<VT, false, false>(smap, P, plan.smem, sms, st);
  if (plan.lane_y && plan.bz0) return launch_one<VT, true, true>(smap, P, plan.smem, sms, st);
  return launch_one<VT, true, false>(smap, P, plan.smem, sms, st);
}

template cudaError_t launch_forward_tma<float>(const CUtensorMap&, const FwdPlan&, const AxisDev&, const VolDev&,
                                               const float*, int, int, int*, cudaStream_t);
template cudaError_t launch_forward_tma<__nv_bfloat16>(const CUtensorMap&, const FwdPlan&, const AxisDev&,
                                                       const VolDev&, const __nv_bfloat16*, int, int, int*,
                                                       cudaStream_t);
template cudaError_t launch_forward_tma<__half>(const CUtensorMap&, const FwdPlan&, const AxisDev&, const VolDev&,
                                                const __half*, int, int, int*, cudaStream_t);

}  // namespace mtr
