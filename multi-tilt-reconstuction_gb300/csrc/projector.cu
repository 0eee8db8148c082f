// Bilinear projector kernels for the multi-axis SIRT path (sm_103a).
//
// Geometry (the reference's computeWeight, FunctionOnGPU.cu:12-25): voxel
// (X,Y,Z) lands on detector coordinate
//     x = a0 + a1 X + a2 Y + a3 Z - 1,   y = b0 + b1 X + b2 Y + b3 Z - 1
// and touches the four pixels (ix,iy), (ix+1,iy), (ix,iy+1), (ix+1,iy+1),
// ix = floor(x), with bilinear weights (1-dx)(1-dy), dx(1-dy), (1-dx)dy,
// dx dy.  Taps outside the detector are dropped (FunctionOnGPU.cu:27-79).
//
// Coordinates: the reference evaluates the map in FP64 per voxel and angle.
// Here each CTA evaluates it once per angle in FP64 at its base voxel, splits
// the result into an integer part and a float fraction in [0,1), and each
// thread adds float slope * (small offset) to the fraction.  The float part
// stays below ~100 in magnitude, so the tap position carries ~1e-5 px of
// error however large the detector is, and the inner loop is pure FP32.
#include <cstdint>
#include <type_traits>

#include "mtr_internal.h"

namespace mtr {
namespace {

// Split-precision affine map of one angle relative to a CTA base voxel.
struct AngleConst {
  float xf, a1, a2, a3;
  float yf, b1, b2, b3;
  int xi, yi;
};

__device__ __forceinline__ int clamp_int_base(double v) {
  // Keep the integer base far from int overflow when it is added to small
  // offsets; anything this far off the detector is dropped by the tap tests.
  v = fmin(fmax(v, -1.0e9), 1.0e9);
  return (int)v;
}

__device__ __forceinline__ void make_angle_const(const double* __restrict__ xc, const double* __restrict__ yc,
                                                 int a, int X0, int Y0, int Z0, AngleConst& k) {
  const double* cx = xc + 4 * a;
  const double* cy = yc + 4 * a;
  const double xb = cx[0] + cx[1] * X0 + cx[2] * Y0 + cx[3] * Z0 - 1.0;
  const double yb = cy[0] + cy[1] * X0 + cy[2] * Y0 + cy[3] * Z0 - 1.0;
  const double fxb = floor(xb), fyb = floor(yb);
  k.xi = clamp_int_base(fxb);
  k.yi = clamp_int_base(fyb);
  k.xf = (float)(xb - fxb);
  k.yf = (float)(yb - fyb);
  k.a1 = (float)cx[1]; k.a2 = (float)cx[2]; k.a3 = (float)cx[3];
  k.b1 = (float)cy[1]; k.b2 = (float)cy[2]; k.b3 = (float)cy[3];
}

template <typename T> __device__ __forceinline__ float ld_f(const T* p);
template <> __device__ __forceinline__ float ld_f<float>(const float* p) { return __ldg(p); }
template <> __device__ __forceinline__ float ld_f<__half>(const __half* p) { return __half2float(__ldg(p)); }
template <> __device__ __forceinline__ float ld_f<__nv_bfloat16>(const __nv_bfloat16* p) {
  return __bfloat162float(__ldg(p));
}

template <typename T> __device__ __forceinline__ T from_f(float v);
template <> __device__ __forceinline__ float from_f<float>(float v) { return v; }
template <> __device__ __forceinline__ __half from_f<__half>(float v) { return __float2half_rn(v); }
template <> __device__ __forceinline__ __nv_bfloat16 from_f<__nv_bfloat16>(float v) { return __float2bfloat16_rn(v); }

constexpr int kTX = 32;  // CTA tile in X (one warp row)
constexpr int kTY = 8;   // CTA tile in Y
constexpr int kZR = 8;   // voxels per thread along Z

// Back-projection gather over all angles.
//   MODE 0 (WBP, FunctionOnGPU.cu:82-109): vol_out = s/c (0 where c == 0), cbp = c.
//   MODE 1 (SIRT, FunctionOnGPU.cu:111-135): vol_out += step * s/cbp where cbp != 0.
//   MODE 2: cbp = c only.
// copy_kind 1/2 additionally writes the updated voxel as bf16/f16 to vol_copy.
template <typename PT, int MODE>
__global__ void __launch_bounds__(kTX * kTY)
bp_gather_kernel(AxisDev ax, VolDev vol, const PT* __restrict__ img, float step, float* __restrict__ vol_out,
                 float* __restrict__ cbp, void* __restrict__ vol_copy, int copy_kind, int z0, int z1) {
  extern __shared__ AngleConst sk[];
  const int tid = threadIdx.x + threadIdx.y * kTX;
  const int X0 = vol.Xs + blockIdx.x * kTX;
  const int Y0 = vol.Ys + blockIdx.y * kTY;
  const int Z0 = z0 + blockIdx.z * kZR;
  for (int a = tid; a < ax.A; a += kTX * kTY) make_angle_const(ax.xc, ax.yc, a, X0, Y0, Z0, sk[a]);
  __syncthreads();

  const int tx = threadIdx.x, ty = threadIdx.y;
  if (X0 + tx >= vol.Xs + vol.NX || Y0 + ty >= vol.Ys + vol.NY) return;
  const int PX = ax.PX, PY = ax.PY, RP = ax.pitch;
  const long long plane = (long long)RP * PY;

  float s[kZR], c[kZR];
#pragma unroll
  for (int z = 0; z < kZR; ++z) { s[z] = 0.f; c[z] = 0.f; }

  for (int a = 0; a < ax.A; ++a) {
    const AngleConst k = sk[a];
    const float xr = fmaf(k.a2, (float)ty, fmaf(k.a1, (float)tx, k.xf));
    const float yr = fmaf(k.b2, (float)ty, fmaf(k.b1, (float)tx, k.yf));
    const PT* im = img + plane * a;
#pragma unroll
    for (int z = 0; z < kZR; ++z) {
      const float x = fmaf(k.a3, (float)z, xr);
      const float y = fmaf(k.b3, (float)z, yr);
      const float flx = floorf(x), fly = floorf(y);
      const float fx = x - flx, fy = y - fly;
      const int ix = k.xi + (int)flx, iy = k.yi + (int)fly;
      const bool x0 = (unsigned)ix < (unsigned)PX, x1 = (unsigned)(ix + 1) < (unsigned)PX;
      const bool y0 = (unsigned)iy < (unsigned)PY, y1 = (unsigned)(iy + 1) < (unsigned)PY;
      if (MODE != 2) {
        const PT* row0 = im + (long long)iy * RP + ix;
        const PT* row1 = row0 + RP;
        const float p00 = (x0 && y0) ? ld_f(row0) : 0.f;
        const float p10 = (x1 && y0) ? ld_f(row0 + 1) : 0.f;
        const float p01 = (x0 && y1) ? ld_f(row1) : 0.f;
        const float p11 = (x1 && y1) ? ld_f(row1 + 1) : 0.f;
        const float r0 = fmaf(fx, p10 - p00, p00);
        const float r1 = fmaf(fx, p11 - p01, p01);
        s[z] += fmaf(fy, r1 - r0, r0);
      }
      if (MODE != 1) {
        const float cx = (x0 ? 1.f - fx : 0.f) + (x1 ? fx : 0.f);
        const float cy = (y0 ? 1.f - fy : 0.f) + (y1 ? fy : 0.f);
        c[z] = fmaf(cx, cy, c[z]);
      }
    }
  }

  const long long sx = vol.NX, sxy = (long long)vol.NX * vol.NY;
  const long long base = (long long)(X0 + tx - vol.Xs) + (long long)(Y0 + ty - vol.Ys) * sx;
#pragma unroll
  for (int z = 0; z < kZR; ++z) {
    const int zz = Z0 + z;
    if (zz >= z1) break;
    const long long vi = base + (long long)(zz - z0) * sxy;
    float out;
    if (MODE == 0) {
      out = (c[z] != 0.f) ? s[z] / c[z] : 0.f;
      vol_out[vi] = out;
      cbp[vi] = c[z];
    } else if (MODE == 1) {
      const float cv = cbp[vi];
      out = vol_out[vi];
      if (cv != 0.f) {
        out = fmaf(step, s[z] / cv, out);
        vol_out[vi] = out;
      }
    } else {
      cbp[vi] = c[z];
      continue;
    }
    if (copy_kind == 1) static_cast<__nv_bfloat16*>(vol_copy)[vi] = __float2bfloat16_rn(out);
    else if (copy_kind == 2) static_cast<__half*>(vol_copy)[vi] = __float2half_rn(out);
  }
}

// Voxel-driven bilinear splat (FunctionOnGPU.cu:27-52, 316-333) into s.
// x == nullptr splats ones (row sums c = A 1).
template <typename VT>
__global__ void __launch_bounds__(kTX * kTY)
fwd_splat_kernel(AxisDev ax, VolDev vol, const VT* __restrict__ x, float* __restrict__ s, int z0, int z1) {
  extern __shared__ AngleConst sk[];
  const int tid = threadIdx.x + threadIdx.y * kTX;
  const int X0 = vol.Xs + blockIdx.x * kTX;
  const int Y0 = vol.Ys + blockIdx.y * kTY;
  const int Z0 = z0 + blockIdx.z * kZR;
  for (int a = tid; a < ax.A; a += kTX * kTY) make_angle_const(ax.xc, ax.yc, a, X0, Y0, Z0, sk[a]);
  __syncthreads();

  const int tx = threadIdx.x, ty = threadIdx.y;
  if (X0 + tx >= vol.Xs + vol.NX || Y0 + ty >= vol.Ys + vol.NY) return;
  const int PX = ax.PX, PY = ax.PY, RP = ax.pitch;
  const long long plane = (long long)RP * PY;

  const long long sx = vol.NX, sxy = (long long)vol.NX * vol.NY;
  const long long base = (long long)(X0 + tx - vol.Xs) + (long long)(Y0 + ty - vol.Ys) * sx;
  float v[kZR];
#pragma unroll
  for (int z = 0; z < kZR; ++z) {
    const int zz = Z0 + z;
    v[z] = 0.f;
    if (zz < z1) v[z] = x ? ld_f(x + base + (long long)(zz - z0) * sxy) : 1.f;
  }

  for (int a = 0; a < ax.A; ++a) {
    const AngleConst k = sk[a];
    const float xr = fmaf(k.a2, (float)ty, fmaf(k.a1, (float)tx, k.xf));
    const float yr = fmaf(k.b2, (float)ty, fmaf(k.b1, (float)tx, k.yf));
    float* sp = s + plane * a;
#pragma unroll
    for (int z = 0; z < kZR; ++z) {
      if (Z0 + z >= z1) break;
      const float xx = fmaf(k.a3, (float)z, xr);
      const float yy = fmaf(k.b3, (float)z, yr);
      const float flx = floorf(xx), fly = floorf(yy);
      const float fx = xx - flx, fy = yy - fly;
      const int ix = k.xi + (int)flx, iy = k.yi + (int)fly;
      const bool x0 = (unsigned)ix < (unsigned)PX, x1 = (unsigned)(ix + 1) < (unsigned)PX;
      const bool y0 = (unsigned)iy < (unsigned)PY, y1 = (unsigned)(iy + 1) < (unsigned)PY;
      const float g0 = (1.f - fy) * v[z], g1 = fy * v[z];
      float* row0 = sp + (long long)iy * RP + ix;
      if (x0 && y0) atomicAdd(row0, (1.f - fx) * g0);
      if (x1 && y0) atomicAdd(row0 + 1, fx * g0);
      if (x0 && y1) atomicAdd(row0 + RP, (1.f - fx) * g1);
      if (x1 && y1) atomicAdd(row0 + RP + 1, fx * g1);
    }
  }
}

// Residual (FunctionOnGPU.cu:228-236): r = b - s/c where c != 0, else b;
// resets s to zero for the next forward pass; FP64 sum of r^2.
// Four consecutive projection values as floats (16-byte / 8-byte vector loads).
__device__ __forceinline__ void ld4(const float* p, float (&v)[4]) {
  const float4 t = __ldg(reinterpret_cast<const float4*>(p));
  v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
}
__device__ __forceinline__ void ld4(const __half* p, float (&v)[4]) {
  const uint2 t = __ldg(reinterpret_cast<const uint2*>(p));
  const float2 lo = __half22float2(*reinterpret_cast<const __half2*>(&t.x));
  const float2 hi = __half22float2(*reinterpret_cast<const __half2*>(&t.y));
  v[0] = lo.x; v[1] = lo.y; v[2] = hi.x; v[3] = hi.y;
}

// r = b - s/c for 4 consecutive pixels (c == 0: r = b - s, the reference's
// residual loop, FunctionOnGPU.cu:228-236), s reset to zero for the next
// forward pass; returns the sum of the four r^2 (FP32, added into FP64).
template <typename BT>
__device__ __forceinline__ float residual4(const BT* b, float* s, const float* c, float* r) {
  float bv[4];
  ld4(b, bv);
  const float4 sv = *reinterpret_cast<const float4*>(s);
  const float4 cv = __ldg(reinterpret_cast<const float4*>(c));
  float4 rv;
  rv.x = bv[0] - (cv.x != 0.f ? sv.x / cv.x : sv.x);
  rv.y = bv[1] - (cv.y != 0.f ? sv.y / cv.y : sv.y);
  rv.z = bv[2] - (cv.z != 0.f ? sv.z / cv.z : sv.z);
  rv.w = bv[3] - (cv.w != 0.f ? sv.w / cv.w : sv.w);
  *reinterpret_cast<float4*>(r) = rv;
  *reinterpret_cast<float4*>(s) = make_float4(0.f, 0.f, 0.f, 0.f);
  return rv.x * rv.x + rv.y * rv.y + rv.z * rv.z + rv.w * rv.w;
}

// r = b - s/c (c != 0), else b - s (FunctionOnGPU.cu:228-236); also
// resets s to zero for the next forward pass.  NORM: FP64 sum of r^2 (the
// FP64 pipe is slow, so it is only accumulated when a norm is recorded).
// Pixels [0, 4*n4) four per thread and step (the host passes n4 = 0 unless
// every array is 16-byte aligned), the rest one per thread.
template <typename BT, bool NORM>
__global__ void __launch_bounds__(256)
residual_kernel(long long n, long long n4, const BT* __restrict__ b, float* __restrict__ s,
                const float* __restrict__ c, float* __restrict__ r, double* __restrict__ norm2) {
  double acc = 0.0;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n4; q += stride) {
    const float sq = residual4(b + 4 * q, s + 4 * q, c + 4 * q, r + 4 * q);
    if (NORM) acc += (double)sq;
  }
  for (long long i = 4 * n4 + blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += stride) {
    float sv = s[i];
    const float cv = c[i];
    if (cv != 0.f) sv = sv / cv;
    const float rv = ld_f(b + i) - sv;
    r[i] = rv;
    s[i] = 0.f;
    if (NORM) acc += (double)(rv * rv);
  }
  if (NORM) {
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    __shared__ double red[8];
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
      atomicAdd(norm2, t);
    }
  }
}

// Residual of one detector row in pair form, for the windowed SIRT update:
// pair column c = (r[c-1], r[c] - r[c-1]), r[-1] = 0 and r = 0 at and beyond
// the detector's right edge (the zero padding of b, s and c gives r = 0 there
// by itself); a back-projection tap at pixel ix reads pair column ix + 1.  The
// calling warp's lane l takes columns [c0 + 4l, c0 + 4l + 4) of each 128-column
// chunk; r[c-1] of a lane's first column comes from the lane below (lane 0:
// the last column of the previous chunk).  s is reset to zero.  Returns the
// lane's sum of r^2.
// FORM 1: the row's pairs are written as two planes of pitch2 floats, the
// values and then the differences (out is the row's first float); FORM 2:
// as FP16 pairs, one 32-bit word each (out is the row's first word).
template <typename BT, int FORM>
__device__ __forceinline__ float residual_pair_row(const BT* __restrict__ br, float* __restrict__ sr,
                                                   const float* __restrict__ cr, float* __restrict__ out, int pitch,
                                                   int pitch2, int lane) {
  float carry = 0.f, sq = 0.f;
  for (int c0 = 0; c0 < pitch2; c0 += 128) {
    const int col = c0 + 4 * lane;
    float r4[4] = {0.f, 0.f, 0.f, 0.f};
    if (col < pitch) {  // pitch is a multiple of 8: the four columns are all in the row
      float bv[4];
      ld4(br + col, bv);
      const float4 sv = *reinterpret_cast<const float4*>(sr + col);
      const float4 cv = __ldg(reinterpret_cast<const float4*>(cr + col));
      r4[0] = bv[0] - (cv.x != 0.f ? sv.x / cv.x : sv.x);
      r4[1] = bv[1] - (cv.y != 0.f ? sv.y / cv.y : sv.y);
      r4[2] = bv[2] - (cv.z != 0.f ? sv.z / cv.z : sv.z);
      r4[3] = bv[3] - (cv.w != 0.f ? sv.w / cv.w : sv.w);
      *reinterpret_cast<float4*>(sr + col) = make_float4(0.f, 0.f, 0.f, 0.f);
      sq += r4[0] * r4[0] + r4[1] * r4[1] + r4[2] * r4[2] + r4[3] * r4[3];
    }
    float prev = __shfl_up_sync(0xffffffffu, r4[3], 1);
    if (lane == 0) prev = carry;
    carry = __shfl_sync(0xffffffffu, r4[3], 31);
    if (col < pitch2) {  // pitch2 is a multiple of 4: four pairs, 32 bytes (16 in FP16)
      if constexpr (FORM == 2) {
        __half2 h[4];
        h[0] = __floats2half2_rn(prev, r4[0] - prev);
        h[1] = __floats2half2_rn(r4[0], r4[1] - r4[0]);
        h[2] = __floats2half2_rn(r4[1], r4[2] - r4[1]);
        h[3] = __floats2half2_rn(r4[2], r4[3] - r4[2]);
        *reinterpret_cast<uint4*>(out + col) = *reinterpret_cast<const uint4*>(h);
      } else if constexpr (FORM == 1) {
        *reinterpret_cast<float4*>(out + col) = make_float4(prev, r4[0], r4[1], r4[2]);
        *reinterpret_cast<float4*>(out + pitch2 + col) =
            make_float4(r4[0] - prev, r4[1] - r4[0], r4[2] - r4[1], r4[3] - r4[2]);
      } else {
        float4* o = reinterpret_cast<float4*>(out + 2 * col);
        o[0] = make_float4(prev, r4[0] - prev, r4[0], r4[1] - r4[0]);
        o[1] = make_float4(r4[1], r4[2] - r4[1], r4[2], r4[3] - r4[2]);
      }
    }
  }
  return sq;
}

// One warp per detector row (rows = AngN * PY); FP64 norm when NORM.
template <typename BT, bool NORM, int FORM>
__global__ void __launch_bounds__(256)
residual_pairs_kernel(long long rows, int pitch, int pitch2, const BT* __restrict__ b, float* __restrict__ s,
                      const float* __restrict__ c, float* __restrict__ rp, double* __restrict__ norm2) {
  const int lane = threadIdx.x & 31;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  double acc = 0.0;
  for (long long row = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5; row < rows; row += nwarps) {
    const float sq = residual_pair_row<BT, FORM>(b + row * pitch, s + row * pitch, c + row * pitch,
                                                 rp + row * (FORM == 2 ? 1 : 2) * pitch2, pitch, pitch2, lane);
    if (NORM) acc += (double)sq;
  }
  if (NORM) {
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    __shared__ double red[8];
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
      atomicAdd(norm2, t);
    }
  }
}

// Residual over many axes: item = (descriptor, chunk of kBatchChunk pixels).
template <bool HALF_B>
__global__ void __launch_bounds__(256)
residual_batch_kernel(const ResBatchDesc* __restrict__ descs, const long long* __restrict__ first, int n_desc,
                      long long n_items) {
  for (long long it = blockIdx.x; it < n_items; it += gridDim.x) {
    const int2 item = work_item(first, n_desc, it);
    const ResBatchDesc& D = descs[item.x];
    const long long i0 = (long long)item.y * kBatchChunk;
    const long long i1 = min(D.n, i0 + kBatchChunk);  // both multiples of 8 (row pitch)
    for (long long i = i0 + 4 * threadIdx.x; i < i1; i += 4 * blockDim.x) {
      if (HALF_B) residual4(static_cast<const __half*>(D.b) + i, D.s + i, D.cf + i, D.r + i);
      else residual4(static_cast<const float*>(D.b) + i, D.s + i, D.cf + i, D.r + i);
    }
  }
}

dim3 vol_grid(const VolDev& vol, int z0, int z1) {
  return dim3((vol.NX + kTX - 1) / kTX, (vol.NY + kTY - 1) / kTY, (z1 - z0 + kZR - 1) / kZR);
}

}  // namespace

template <typename PT>
void launch_backproject(const AxisDev& ax, const VolDev& vol, const PT* img, int mode, float step,
                        float* vol_out, float* cbp, void* vol_copy, int copy_kind, int z0, int z1,
                        cudaStream_t st) {
  const dim3 grid = vol_grid(vol, z0, z1), block(kTX, kTY);
  const size_t smem = sizeof(AngleConst) * ax.A;
  if (mode == 0)
    bp_gather_kernel<PT, 0><<<grid, block, smem, st>>>(ax, vol, img, step, vol_out, cbp, vol_copy, copy_kind, z0, z1);
  else if (mode == 1)
    bp_gather_kernel<PT, 1><<<grid, block, smem, st>>>(ax, vol, img, step, vol_out, cbp, vol_copy, copy_kind, z0, z1);
  else
    bp_gather_kernel<PT, 2><<<grid, block, smem, st>>>(ax, vol, img, step, vol_out, cbp, vol_copy, copy_kind, z0, z1);
}

template <typename VT>
void launch_forward(const AxisDev& ax, const VolDev& vol, const VT* x, float* s, int z0, int z1, cudaStream_t st) {
  const dim3 grid = vol_grid(vol, z0, z1), block(kTX, kTY);
  const size_t smem = sizeof(AngleConst) * ax.A;
  fwd_splat_kernel<VT><<<grid, block, smem, st>>>(ax, vol, x, s, z0, z1);
}

template <typename BT, typename RT>
void launch_residual(long long n, const BT* b, float* s, const float* c, RT* r, double* norm2, cudaStream_t st) {
  long long blocks = (n / 4 + 255) / 256;
  const long long cap = (long long)device_sm_count() * 16;
  if (blocks > cap) blocks = cap;  // grid-stride loops cover the rest
  if (blocks < 1) blocks = 1;
  static_assert(std::is_same<RT, float>::value, "the residual is FP32");
  // vector loads need 16-byte aligned arrays (caller-owned buffers may not be)
  const bool aligned = ((reinterpret_cast<uintptr_t>(b) | reinterpret_cast<uintptr_t>(s) |
                         reinterpret_cast<uintptr_t>(c) | reinterpret_cast<uintptr_t>(r)) & 15) == 0;
  const long long n4 = aligned ? n / 4 : 0;
  if (norm2) residual_kernel<BT, true><<<(unsigned)blocks, 256, 0, st>>>(n, n4, b, s, c, r, norm2);
  else residual_kernel<BT, false><<<(unsigned)blocks, 256, 0, st>>>(n, n4, b, s, c, r, nullptr);
}

void launch_residual_batch(const ResBatchDesc* descs, const long long* first, int n_desc, long long n_items, int half_b,
                           int grid, cudaStream_t st) {
  if (half_b) residual_batch_kernel<true><<<grid, 256, 0, st>>>(descs, first, n_desc, n_items);
  else residual_batch_kernel<false><<<grid, 256, 0, st>>>(descs, first, n_desc, n_items);
}

template <typename BT>
void launch_residual_pairs(long long rows, int pitch, int pitch2, const BT* b, float* s, const float* c, float* rp,
                           int form, double* norm2, cudaStream_t st) {
  long long blocks = (rows + 7) / 8;  // 8 warps per block, one row per warp
  const long long cap = (long long)device_sm_count() * 16;
  if (blocks > cap) blocks = cap;  // grid-stride over the rest
  if (blocks < 1) blocks = 1;
  const unsigned g = (unsigned)blocks;
  if (form == 2) {
    if (norm2) residual_pairs_kernel<BT, true, 2><<<g, 256, 0, st>>>(rows, pitch, pitch2, b, s, c, rp, norm2);
    else residual_pairs_kernel<BT, false, 2><<<g, 256, 0, st>>>(rows, pitch, pitch2, b, s, c, rp, nullptr);
  } else if (form == 1) {
    if (norm2) residual_pairs_kernel<BT, true, 1><<<g, 256, 0, st>>>(rows, pitch, pitch2, b, s, c, rp, norm2);
    else residual_pairs_kernel<BT, false, 1><<<g, 256, 0, st>>>(rows, pitch, pitch2, b, s, c, rp, nullptr);
  } else {
    if (norm2) residual_pairs_kernel<BT, true, 0><<<g, 256, 0, st>>>(rows, pitch, pitch2, b, s, c, rp, norm2);
    else residual_pairs_kernel<BT, false, 0><<<g, 256, 0, st>>>(rows, pitch, pitch2, b, s, c, rp, nullptr);
  }
}

template void launch_residual_pairs<float>(long long, int, int, const float*, float*, const float*, float*, int,
                                           double*, cudaStream_t);
template void launch_residual_pairs<__half>(long long, int, int, const __half*, float*, const float*, float*, int,
                                            double*, cudaStream_t);

template void launch_backproject<float>(const AxisDev&, const VolDev&, const float*, int, float, float*, float*,
                                        void*, int, int, int, cudaStream_t);
template void launch_backproject<__half>(const AxisDev&, const VolDev&, const __half*, int, float, float*, float*,
                                         void*, int, int, int, cudaStream_t);
template void launch_forward<float>(const AxisDev&, const VolDev&, const float*, float*, int, int, cudaStream_t);
template void launch_forward<__nv_bfloat16>(const AxisDev&, const VolDev&, const __nv_bfloat16*, float*, int, int,
                                            cudaStream_t);
template void launch_forward<__half>(const AxisDev&, const VolDev&, const __half*, float*, int, int, cudaStream_t);
template void launch_residual<float, float>(long long, const float*, float*, const float*, float*, double*,
                                            cudaStream_t);
template void launch_residual<__half, float>(long long, const __half*, float*, const float*, float*, double*,
                                             cudaStream_t);

}  // namespace mtr
