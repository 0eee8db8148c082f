// Device side of the TMA-windowed back-projection (bp_tma.cu, bp_pairs.cu):
// the brick routine, its kernel and the templated launch helpers.  Included by
// the two translation units that instantiate the FP32-window and the
// residual-pair variants, so that they compile in parallel.
#pragma once

#include <algorithm>
#include <atomic>
#include <type_traits>

#include "mtr_internal.h"
#include "tma.cuh"

namespace mtr {

// Arguments of one windowed back-projection launch (shared by both units).
struct BpArgs {
  AxisDev ax;
  VolDev vol;
  int z0, z1;
  int WX, WY;       // window box (elements)
  int align;        // TMA x alignment (elements)
  int mode;         // 0 WBP, 1 SIRT
  float step;
  float* vol_out;
  float* cbp;
  void* vol_copy;
  int copy_kind;
  int* err;
  unsigned wait_iters;  // polls of a pipeline wait before it gives up
};

// The SIRT update over residual-pair windows (bp_pairs.cu).
cudaError_t launch_backproject_tma_pairs(const CUtensorMap& map, const BpPlan& plan, const BpArgs& P,
                                         cudaStream_t st);

namespace {

constexpr int NST = 4;             // pipeline stages
constexpr int kConsumerWarps = 8;  // 256 consumer threads
constexpr int kThreads = (kConsumerWarps + 1) * 32;
// Polls of the pipeline waits (producer on a free stage, consumers on a
// loaded window) before they give up are a launch argument, so that a test
// can make them give up at once.  The drain of the producer's own copies in
// flight always has the full bound: a CTA never exits with a copy pending.
constexpr uint32_t kDrainIters = 1u << 24;
constexpr float kMagic = 12582912.0f;  // 1.5 * 2^23: x + kMagic holds round(x) in its low bits
constexpr int kMagicBits = 0x4B400000;

struct WinConst {
  float xf, a1, a2, a3;  // x map relative to the CTA base voxel (fractional base)
  float yf, b1, b2, b3;
  int lxm, lym;          // window-local integer base minus the magic bits
  int ox, oy;            // window origin on the detector (ox aligned for TMA)
};

template <typename PT> __device__ __forceinline__ float to_f(PT v);
template <> __device__ __forceinline__ float to_f<float>(float v) { return v; }

__device__ __forceinline__ int floor_div(int a, int b) { return (a >= 0) ? a / b : -((-a + b - 1) / b); }

__device__ __forceinline__ int magic_int(float integral) { return __float_as_int(__fadd_rn(integral, kMagic)); }

// Shared-memory loads at a 32-bit shared address plus a constant byte offset:
// the column gathers step their tap address in this form (one 32-bit add per
// pixel crossed) instead of a generic pointer.  Volatile keeps them after the
// pipeline's mbarrier waits.
template <int OFF> __device__ __forceinline__ float lds_f32(uint32_t a) {
  float v;
  asm volatile("ld.shared.f32 %0, [%1+%2];" : "=f"(v) : "r"(a), "n"(OFF));
  return v;
}
template <int OFF> __device__ __forceinline__ float2 lds_f32x2(uint32_t a) {
  float2 v;
  asm volatile("ld.shared.v2.f32 {%0, %1}, [%2+%3];" : "=f"(v.x), "=f"(v.y) : "r"(a), "n"(OFF));
  return v;
}
template <int OFF> __device__ __forceinline__ float2 lds_h2_widened(uint32_t a) {
  __half2 h;
  asm volatile("ld.shared.b32 %0, [%1+%2];" : "=r"(*reinterpret_cast<unsigned*>(&h)) : "r"(a), "n"(OFF));
  return __half22float2(h);
}

// Gather of one voxel column (fixed X, Y; y-map without a Z term) from
// detector rows `row0` and `row0 + WX`, adding into s[0..NZ).  x advances by
// |a3| < 1 per voxel, so the fraction is stepped by one add and the tap
// address by a predicated increment instead of a floor per voxel.  ASC walks
// z upwards (a3 >= 0), else downwards, so that x never decreases.  Rounding
// of the stepped fraction stays below 4e-6 px over 32 voxels; the caller
// leaves one pixel of window slack for it.
template <bool ASC, int NZ, typename PT>
__device__ __forceinline__ void bp_column(float (&s)[NZ], const PT* row0, int WX, float xr, float a3, int lxm,
                                          float wy0, float wy1) {
  constexpr int zf = ASC ? 0 : NZ - 1;
  const float x = fmaf(a3, (float)zf, xr);
  const float flx = floorf(x);
  float fx = x - flx;
  const float step = fabsf(a3);
  static_assert(sizeof(PT) == 4, "FP32 windows");
  uint32_t p = smem_u32(row0) + 4u * (uint32_t)(magic_int(flx) + lxm);
  const uint32_t dr = 4u * (uint32_t)WX;
#pragma unroll
  for (int i = 0; i < NZ; ++i) {
    const int z = ASC ? i : NZ - 1 - i;
    if (i > 0) {
      fx += step;
      const bool adv = fx >= 1.f;
      fx = adv ? fx - 1.f : fx;
      p += adv ? 4u : 0u;
    }
    const float p00 = lds_f32<0>(p), p10 = lds_f32<4>(p);
    const float p01 = lds_f32<0>(p + dr), p11 = lds_f32<4>(p + dr);
    const float r0 = fmaf(fx, p10 - p00, p00);
    const float r1 = fmaf(fx, p11 - p01, p01);
    s[z] = fmaf(wy0, r0, s[z]);
    s[z] = fmaf(wy1, r1, s[z]);
  }
}

// The same column gather from a row pre-blended by the warp: b[i] holds the
// y-interpolated detector value at window column i, so a voxel needs 2 taps.
template <bool ASC, int NZ>
__device__ __forceinline__ void bp_column_blended(float (&s)[NZ], const float* b, float xr, float a3, int lxm) {
  constexpr int zf = ASC ? 0 : NZ - 1;
  const float x = fmaf(a3, (float)zf, xr);
  const float flx = floorf(x);
  float fx = x - flx;
  const float step = fabsf(a3);
  uint32_t p = smem_u32(b) + 4u * (uint32_t)(magic_int(flx) + lxm);
#pragma unroll
  for (int i = 0; i < NZ; ++i) {
    const int z = ASC ? i : NZ - 1 - i;
    if (i > 0) {
      fx += step;
      const bool adv = fx >= 1.f;
      fx = adv ? fx - 1.f : fx;
      p += adv ? 4u : 0u;
    }
    const float p0 = lds_f32<0>(p), p1 = lds_f32<4>(p);
    s[z] += fmaf(fx, p1 - p0, p0);
  }
}

// The SIRT update's windows hold (value, next value - value) pairs of the
// residual (residual_pairs_kernel): a tap pair of one detector row is one
// 8-byte load and its x interpolation one FFMA.
template <bool ASC, int NZ>
__device__ __forceinline__ void bp_column(float (&s)[NZ], const float2* row0, int WX, float xr, float a3, int lxm,
                                          float wy0, float wy1) {
  constexpr int zf = ASC ? 0 : NZ - 1;
  const float x = fmaf(a3, (float)zf, xr);
  const float flx = floorf(x);
  float fx = x - flx;
  const float step = fabsf(a3);
  uint32_t p = smem_u32(row0) + 8u * (uint32_t)(magic_int(flx) + lxm);
  const uint32_t dr = 8u * (uint32_t)WX;
#pragma unroll
  for (int i = 0; i < NZ; ++i) {
    const int z = ASC ? i : NZ - 1 - i;
    if (i > 0) {
      fx += step;
      const bool adv = fx >= 1.f;
      fx = adv ? fx - 1.f : fx;
      p += adv ? 8u : 0u;
    }
    const float2 q0 = lds_f32x2<0>(p), q1 = lds_f32x2<0>(p + dr);
    s[z] = fmaf(wy0, fmaf(fx, q0.y, q0.x), s[z]);
    s[z] = fmaf(wy1, fmaf(fx, q1.y, q1.x), s[z]);
  }
}

// The same from planar pair windows: a detector row's values, then its
// differences, WX floats each, so a voxel's row r reads p[0] and p[WX] and
// row r + 1 reads p[2 WX] and p[3 WX] (four 4-byte loads, two FFMAs).
template <bool ASC, int NZ>
__device__ __forceinline__ void bp_column_planar(float (&s)[NZ], const float* row0, int WX, float xr, float a3,
                                                 int lxm, float wy0, float wy1) {
  constexpr int zf = ASC ? 0 : NZ - 1;
  const float x = fmaf(a3, (float)zf, xr);
  const float flx = floorf(x);
  float fx = x - flx;
  const float step = fabsf(a3);
  uint32_t p = smem_u32(row0) + 4u * (uint32_t)(magic_int(flx) + lxm);
  const uint32_t d1 = 4u * (uint32_t)WX, d2 = 2u * d1, d3 = 3u * d1;
#pragma unroll
  for (int i = 0; i < NZ; ++i) {
    const int z = ASC ? i : NZ - 1 - i;
    if (i > 0) {
      fx += step;
      const bool adv = fx >= 1.f;
      fx = adv ? fx - 1.f : fx;
      p += adv ? 4u : 0u;
    }
    s[z] = fmaf(wy0, fmaf(fx, lds_f32<0>(p + d1), lds_f32<0>(p)), s[z]);
    s[z] = fmaf(wy1, fmaf(fx, lds_f32<0>(p + d3), lds_f32<0>(p + d2)), s[z]);
  }
}

// The same from FP16 pair windows (mixed precision): a detector row's tap
// pair is one 4-byte load of (value, next - value) in FP16, widened to FP32
// before the interpolation.  Half the shared-memory bytes of the FP32 formats.
template <bool ASC, int NZ>
__device__ __forceinline__ void bp_column_half(float (&s)[NZ], const __half2* row0, int WX, float xr, float a3,
                                               int lxm, float wy0, float wy1) {
  constexpr int zf = ASC ? 0 : NZ - 1;
  const float x = fmaf(a3, (float)zf, xr);
  const float flx = floorf(x);
  float fx = x - flx;
  const float step = fabsf(a3);
  uint32_t p = smem_u32(row0) + 4u * (uint32_t)(magic_int(flx) + lxm);
  const uint32_t dr = 4u * (uint32_t)WX;
#pragma unroll
  for (int i = 0; i < NZ; ++i) {
    const int z = ASC ? i : NZ - 1 - i;
    if (i > 0) {
      fx += step;
      const bool adv = fx >= 1.f;
      fx = adv ? fx - 1.f : fx;
      p += adv ? 4u : 0u;
    }
    const float2 q0 = lds_h2_widened<0>(p), q1 = lds_h2_widened<0>(p + dr);
    s[z] = fmaf(wy0, fmaf(fx, q0.y, q0.x), s[z]);
    s[z] = fmaf(wy1, fmaf(fx, q1.y, q1.x), s[z]);
  }
}

template <bool ASC, int NZ>
__device__ __forceinline__ void bp_column_blended(float (&s)[NZ], const float2* b, float xr, float a3, int lxm) {
  constexpr int zf = ASC ? 0 : NZ - 1;
  const float x = fmaf(a3, (float)zf, xr);
  const float flx = floorf(x);
  float fx = x - flx;
  const float step = fabsf(a3);
  uint32_t p = smem_u32(b) + 8u * (uint32_t)(magic_int(flx) + lxm);
#pragma unroll
  for (int i = 0; i < NZ; ++i) {
    const int z = ASC ? i : NZ - 1 - i;
    if (i > 0) {
      fx += step;
      const bool adv = fx >= 1.f;
      fx = adv ? fx - 1.f : fx;
      p += adv ? 8u : 0u;
    }
    const float2 q = lds_f32x2<0>(p);
    s[z] += fmaf(fx, q.y, q.x);
  }
}

// One brick (bx, by, bz) of one axis.  LANES: 0 = each warp a line of 32
// voxels along X (brick 32x8), 1 = a line along Y (brick 8x32, used when the
// detector x follows Y), 2 = an 8x4 patch (brick 32x8: on oblique axes the
// taps of a line fall on a diagonal of the window that maps several lanes to
// one shared-memory bank; a patch keeps them compact).  `smem` is the CTA's
// dynamic shared memory; `reinit` re-initialises the mbarriers of a CTA that
// already ran a brick.  PF (pair format, with PAIR): 0 interleaved FP32
// pairs; 1 planar FP32 pairs, each detector row as two FP32 rows, its values
// and then its differences; 2 FP16 pairs (value, next - value) in 32 bits.
template <typename PT, int MODE, bool PAIR, int LANES, bool BZ0, int NZ, int PF = 0>
__device__ __forceinline__ void bp_brick(const CUtensorMap* tmap, const BpArgs& P, int bx, int by, int bz,
                                         unsigned char* smem, bool reinit) {
  constexpr int BX = LANES == 1 ? kConsumerWarps : 32;
  constexpr int BY = LANES == 1 ? 32 : kConsumerWarps;
  // The SIRT update's windows hold residual pairs (value, next - value), one
  // per pixel, from a pair array whose column c is pixel c - 1; the WBP's
  // windows hold the projections.
  static_assert(!PAIR || MODE == 1, "residual pairs feed the SIRT update only");
  constexpr bool PLANAR = PAIR && PF == 1, HALF = PAIR && PF == 2;
  static_assert(!PLANAR || BZ0, "planar windows are a pair format, for y-maps without a Z term");
  using WT = typename std::conditional<
      PLANAR, float,
      typename std::conditional<HALF, __half2, typename std::conditional<PAIR, float2, PT>::type>::type>::type;
  using BT = typename std::conditional<PAIR, float2, float>::type;  // blended-row element
  uint64_t* full = reinterpret_cast<uint64_t*>(smem);
  uint64_t* empty = full + NST;
  WinConst* kc = reinterpret_cast<WinConst*>(smem + 128);
  const int A = P.ax.A;
  const size_t kc_bytes = ((size_t)A * sizeof(WinConst) + 127) & ~(size_t)127;
  const int win_elems = P.WX * P.WY * (PLANAR ? 2 : 1);
  const size_t stage_bytes = (((size_t)win_elems * sizeof(WT)) + 127) & ~(size_t)127;
  WT* win0 = reinterpret_cast<WT*>(smem + 128 + kc_bytes);
  // per-warp blended row (uniform-row angles)
  BT* blend = reinterpret_cast<BT*>(smem + 128 + kc_bytes + NST * stage_bytes) + (threadIdx.x >> 5) * P.WX;

  const int tid = threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31;
  const int X0 = P.vol.Xs + bx * BX;
  const int Y0 = P.vol.Ys + by * BY;
  const int Z0 = P.z0 + bz * NZ;

  if (tid == 0) {
    for (int s = 0; s < NST; ++s) {
      if (reinit) {
        mbar_inval(&full[s]);
        mbar_inval(&empty[s]);
      }
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], kConsumerWarps);
    }
    mbar_fence_init();
  }
  // Per-angle constants: FP64 map at the base voxel, split into int + float.
  for (int a = tid; a < A; a += kThreads) {
    const double* cx = P.ax.xc + 4 * a;
    const double* cy = P.ax.yc + 4 * a;
    const double xb = cx[0] + cx[1] * X0 + cx[2] * Y0 + cx[3] * Z0 - 1.0;
    const double yb = cy[0] + cy[1] * X0 + cy[2] * Y0 + cy[3] * Z0 - 1.0;
    const double fxb = floor(fmin(fmax(xb, -1.0e9), 1.0e9)), fyb = floor(fmin(fmax(yb, -1.0e9), 1.0e9));
    WinConst k;
    k.xf = (float)(xb - fxb);
    k.yf = (float)(yb - fyb);
    k.a1 = (float)cx[1]; k.a2 = (float)cx[2]; k.a3 = (float)cx[3];
    k.b1 = (float)cy[1]; k.b2 = (float)cy[2]; k.b3 = (float)cy[3];
    const int xi = (int)fxb, yi = (int)fyb;
    const float xmin = k.xf + fminf(0.f, k.a1 * (BX - 1)) + fminf(0.f, k.a2 * (BY - 1)) + fminf(0.f, k.a3 * (NZ - 1));
    const float ymin = k.yf + fminf(0.f, k.b1 * (BX - 1)) + fminf(0.f, k.b2 * (BY - 1)) + fminf(0.f, k.b3 * (NZ - 1));
    // leftmost tap pixel xi + floor(xmin) - 1; for pairs the window's first
    // pair column (pixel + 1) is rounded down to an even one (TMA alignment)
    const int ox = PAIR ? floor_div(xi + (int)floorf(xmin), P.align) * P.align - 1
                        : floor_div(xi + (int)floorf(xmin) - 1, P.align) * P.align;
    const int oy = yi + (int)floorf(ymin) - 1;
    k.ox = ox;
    k.oy = oy;
    k.lxm = xi - ox - kMagicBits;
    k.lym = yi - oy - kMagicBits;
    kc[a] = k;
  }
  __syncthreads();

  if (warp == kConsumerWarps) {
    // ---------------- producer warp: one elected lane issues the TMA loads
    if (lane == 0) {
      prefetch_tensormap(tmap);
      const uint32_t bytes = (uint32_t)(win_elems * sizeof(WT));
      int issued = 0;  // angles whose window load has been issued
      for (int a = 0; a < A; ++a) {
        const int s = a % NST;
        const int n = a / NST;
        if (n > 0 && !mbar_wait_bounded(&empty[s], (uint32_t)((n - 1) & 1), P.wait_iters)) {
          atomicExch(P.err, 2);
          break;
        }
        WT* dst = reinterpret_cast<WT*>(reinterpret_cast<unsigned char*>(win0) + s * stage_bytes);
        mbar_arrive_expect_tx(&full[s], bytes);
        // interleaved pair arrays are mapped as FP32 pairs: x = 2 * (first pair
        // column), a multiple of 4; planar ones as two FP32 rows per detector row
        tma_load_3d(dst, tmap, (PLANAR || HALF) ? kc[a].ox + 1 : PAIR ? 2 * (kc[a].ox + 1) : kc[a].ox,
                    PLANAR ? 2 * kc[a].oy : kc[a].oy, a, &full[s]);
        issued = a + 1;
      }
      // Drain: the last load issued into each stage must land before exit
      // (earlier ones into that stage completed before it could be reissued).
      for (int s = 0; s < NST && s < issued; ++s) {
        const int n_last = (issued - 1 - s) / NST;
        if (!mbar_wait_bounded(&full[s], (uint32_t)(n_last & 1), kDrainIters)) atomicExch(P.err, 3);
      }
    }
    return;
  }

  // ---------------- consumer warps
  const int tx = LANES == 0 ? lane : LANES == 1 ? warp : (warp & 3) * 8 + (lane & 7);
  const int ty = LANES == 0 ? warp : LANES == 1 ? lane : (warp >> 2) * 4 + (lane >> 3);
  const bool active = (X0 + tx < P.vol.Xs + P.vol.NX) && (Y0 + ty < P.vol.Ys + P.vol.NY);
  const int WX = P.WX;
  // a tap at window column ix reads columns ix and ix + 1 (one pair column with pairs)
  const unsigned lim_x = (unsigned)(PAIR ? WX : WX - 1), lim_y = (unsigned)(P.WY - 1);
  float s[NZ], c[NZ];
#pragma unroll
  for (int z = 0; z < NZ; ++z) { s[z] = 0.f; c[z] = 0.f; }
  bool bad = false;
  int n_inside = 0;  // WBP: angles whose taps of this column all lie on the detector

  for (int a = 0; a < A; ++a) {
    const int st = a % NST;
    // every lane of the warp takes the same branch (the warp syncs below)
    if (!__all_sync(0xffffffffu, mbar_wait_bounded(&full[st], (uint32_t)((a / NST) & 1), P.wait_iters))) {
      if (lane == 0) atomicExch(P.err, 4);
      break;
    }
    const WT* w = reinterpret_cast<const WT*>(reinterpret_cast<const unsigned char*>(win0) + st * stage_bytes);
    const WinConst k = kc[a];
    const float xr = fmaf(k.a2, (float)ty, fmaf(k.a1, (float)tx, k.xf));
    float yr = fmaf(k.b2, (float)ty, fmaf(k.b1, (float)tx, k.yf));
    // Uniform rows: the detector y does not move along the lanes (|slope| * 31
    // below 1e-6 px), so every lane of the warp reads the same two rows with
    // the same weights; the warp blends them once per angle.
    const bool uni = BZ0 && LANES != 2 && fabsf(LANES == 1 ? k.b2 : k.b1) < 3e-8f;
    bool blended = false;
    if (uni) {
      yr = __shfl_sync(0xffffffffu, yr, 0);
      const float fly = floorf(yr);
      const float fy = yr - fly;
      const int rowi = magic_int(fly) + k.lym;
      if ((unsigned)rowi < lim_y) {
        const WT* row0 = w + rowi * WX * (PLANAR ? 2 : 1);
        for (int i = lane; i < WX; i += 32) {
          if constexpr (PLANAR) {
            const float v0 = row0[i], d0 = row0[i + WX], v1 = row0[i + 2 * WX], d1 = row0[i + 3 * WX];
            blend[i] = make_float2(fmaf(fy, v1 - v0, v0), fmaf(fy, d1 - d0, d0));
          } else if constexpr (HALF) {
            const float2 q0 = __half22float2(row0[i]), q1 = __half22float2(row0[i + WX]);
            blend[i] = make_float2(fmaf(fy, q1.x - q0.x, q0.x), fmaf(fy, q1.y - q0.y, q0.y));
          } else if constexpr (PAIR) {
            const float2 q0 = row0[i], q1 = row0[i + WX];
            blend[i] = make_float2(fmaf(fy, q1.x - q0.x, q0.x), fmaf(fy, q1.y - q0.y, q0.y));
          } else {
            const float r0 = to_f(row0[i]);
            blend[i] = fmaf(fy, to_f(row0[i + WX]) - r0, r0);
          }
        }
        blended = true;
      }
      __syncwarp();
    }
    bool done = !active;
    if (active && BZ0 && fabsf(k.a3) < 0.999f) {
      // x is affine in z: the column's end voxels bound every tap index, so
      // the window bound is checked once per column instead of per voxel; the
      // stepped tap may run one pixel past the exact last one.
      const float fly = floorf(yr);
      const float fy = yr - fly;
      const int rowi = magic_int(fly) + k.lym;
      const int ixa = magic_int(floorf(xr)) + k.lxm;
      const int ixb = magic_int(floorf(fmaf(k.a3, (float)(NZ - 1), xr))) + k.lxm;
      bool inside = (unsigned)rowi < lim_y && (unsigned)min(ixa, ixb) < lim_x && (unsigned)(max(ixa, ixb) + 1) < lim_x;
      if (MODE == 0) {
        // WBP also sums the in-detector weights: when both rows and every tap
        // column of the voxel column lie on the detector, each voxel's four
        // weights sum to one and the angle adds exactly 1 to its weight sum.
        const int iy = rowi + k.oy, ix_lo = min(ixa, ixb) + k.ox, ix_hi = max(ixa, ixb) + 1 + k.ox;
        inside = inside && iy >= 0 && iy + 1 < P.ax.PY && ix_lo >= 0 && ix_hi < P.ax.PX;
      }
      if (inside) {
        if (blended) {
          if (k.a3 >= 0.f) bp_column_blended<true, NZ>(s, blend, xr, k.a3, k.lxm);
          else bp_column_blended<false, NZ>(s, blend, xr, k.a3, k.lxm);
        } else if constexpr (PLANAR) {
          const float* row0 = w + rowi * 2 * WX;
          if (k.a3 >= 0.f) bp_column_planar<true, NZ>(s, row0, WX, xr, k.a3, k.lxm, 1.f - fy, fy);
          else bp_column_planar<false, NZ>(s, row0, WX, xr, k.a3, k.lxm, 1.f - fy, fy);
        } else if constexpr (HALF) {
          const __half2* row0 = w + rowi * WX;
          if (k.a3 >= 0.f) bp_column_half<true, NZ>(s, row0, WX, xr, k.a3, k.lxm, 1.f - fy, fy);
          else bp_column_half<false, NZ>(s, row0, WX, xr, k.a3, k.lxm, 1.f - fy, fy);
        } else {
          const WT* row0 = w + rowi * WX;
          if (k.a3 >= 0.f) bp_column<true, NZ>(s, row0, WX, xr, k.a3, k.lxm, 1.f - fy, fy);
          else bp_column<false, NZ>(s, row0, WX, xr, k.a3, k.lxm, 1.f - fy, fy);
        }
        if (MODE == 0) ++n_inside;
        done = true;
      }
    }
    if (!done) {
      // y part (per column when the map has no Z term)
      float fy = 0.f, wy0 = 0.f, wy1 = 0.f, cy = 0.f;
      int rowi = 0;
      if (BZ0) {
        const float fly = floorf(yr);
        fy = yr - fly;
        rowi = magic_int(fly) + k.lym;
        if ((unsigned)rowi >= lim_y) bad = true;
        wy0 = 1.f - fy;
        wy1 = fy;
        if (MODE == 0) {
          const int iya = rowi + k.oy;
          cy = ((unsigned)iya < (unsigned)P.ax.PY ? wy0 : 0.f) + ((unsigned)(iya + 1) < (unsigned)P.ax.PY ? wy1 : 0.f);
        }
      }
#pragma unroll
      for (int z = 0; z < NZ; ++z) {
        if (!BZ0) {
          const float y = fmaf(k.b3, (float)z, yr);
          const float fly = floorf(y);
          fy = y - fly;
          rowi = magic_int(fly) + k.lym;
          if ((unsigned)rowi >= lim_y) bad = true;
          wy0 = 1.f - fy;
          wy1 = fy;
          if (MODE == 0) {
            const int iya = rowi + k.oy;
            cy = ((unsigned)iya < (unsigned)P.ax.PY ? wy0 : 0.f) +
                 ((unsigned)(iya + 1) < (unsigned)P.ax.PY ? wy1 : 0.f);
          }
        }
        const float x = fmaf(k.a3, (float)z, xr);
        const float flx = floorf(x);
        const float fx = x - flx;
        const int ix = magic_int(flx) + k.lxm;
        if ((unsigned)ix >= lim_x) bad = true;
        const int i0 = bad ? 0 : ix + rowi * WX * (PLANAR ? 2 : 1);  // never index outside the window
        float r0, r1;
        if constexpr (PLANAR) {
          r0 = fmaf(fx, w[i0 + WX], w[i0]);
          r1 = fmaf(fx, w[i0 + 3 * WX], w[i0 + 2 * WX]);
        } else if constexpr (HALF) {
          const float2 q0 = __half22float2(w[i0]), q1 = __half22float2(w[i0 + WX]);
          r0 = fmaf(fx, q0.y, q0.x);
          r1 = fmaf(fx, q1.y, q1.x);
        } else if constexpr (PAIR) {
          const float2 q0 = w[i0], q1 = w[i0 + WX];
          r0 = fmaf(fx, q0.y, q0.x);
          r1 = fmaf(fx, q1.y, q1.x);
        } else {
          const float p00 = to_f(w[i0]), p10 = to_f(w[i0 + 1]);
          const float p01 = to_f(w[i0 + WX]), p11 = to_f(w[i0 + WX + 1]);
          r0 = fmaf(fx, p10 - p00, p00);
          r1 = fmaf(fx, p11 - p01, p01);
        }
        s[z] = fmaf(wy0, r0, s[z]);
        s[z] = fmaf(wy1, r1, s[z]);
        if (MODE == 0) {
          const int ixa = ix + k.ox;
          const float cx = ((unsigned)ixa < (unsigned)P.ax.PX ? 1.f - fx : 0.f) +
                           ((unsigned)(ixa + 1) < (unsigned)P.ax.PX ? fx : 0.f);
          c[z] = fmaf(cx, cy, c[z]);
        }
      }
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[st]);
  }
  if (bad) atomicExch(P.err, 5);
  if (!active) return;
  if (MODE == 0) {
#pragma unroll
    for (int z = 0; z < NZ; ++z) c[z] += (float)n_inside;
  }

  const long long sx = P.vol.NX, sxy = (long long)P.vol.NX * P.vol.NY;
  const long long base = (long long)(X0 + tx - P.vol.Xs) + (long long)(Y0 + ty - P.vol.Ys) * sx;
#pragma unroll
  for (int z = 0; z < NZ; ++z) {
    const int zz = Z0 + z;
    if (zz >= P.z1) break;
    const long long vi = base + (long long)(zz - P.z0) * sxy;
    float out;
    if (MODE == 0) {
      out = (c[z] != 0.f) ? s[z] / c[z] : 0.f;
      P.vol_out[vi] = out;
      P.cbp[vi] = c[z];
    } else {
      const float cv = P.cbp[vi];
      out = P.vol_out[vi];
      if (cv != 0.f) {
        out = fmaf(P.step, s[z] / cv, out);
        P.vol_out[vi] = out;
      }
    }
    if (P.copy_kind == 1) static_cast<__nv_bfloat16*>(P.vol_copy)[vi] = __float2bfloat16_rn(out);
    else if (P.copy_kind == 2) static_cast<__half*>(P.vol_copy)[vi] = __float2half_rn(out);
  }
}

// One CTA per brick of one axis.  The grid runs x fastest, then z, then y:
// bricks of the same rows at all depths run together, so the detector rows
// they read stay in L2 instead of being re-read from DRAM once per z layer.
template <typename PT, int MODE, bool PAIR, int LANES, bool BZ0, int NZ, int PF = 0>
// (FP32 pair windows take twice the shared memory: 4 CTAs per SM below depth 32;
// at depth 32 the 32 accumulators fit the 56 registers of 4 CTAs per SM)
__global__ void __launch_bounds__(kThreads, MODE == 1 ? (NZ >= 32 ? 4 : (PAIR && PF != 2 ? 4 : 5)) : 4)
bp_tma_kernel(const __grid_constant__ CUtensorMap tmap, const BpArgs P) {
  extern __shared__ __align__(128) unsigned char smem[];
  bp_brick<PT, MODE, PAIR, LANES, BZ0, NZ, PF>(&tmap, P, blockIdx.x, blockIdx.z, blockIdx.y, smem, false);
}

template <typename PT, int MODE, bool PAIR, int LANES, bool BZ0, int NZ, int PF = 0>
cudaError_t launch_one(const CUtensorMap& map, const BpArgs& P, size_t smem, cudaStream_t st) {
  auto kern = bp_tma_kernel<PT, MODE, PAIR, LANES, BZ0, NZ, PF>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const int BX = LANES == 1 ? kConsumerWarps : 32, BY = LANES == 1 ? 32 : kConsumerWarps;
  const dim3 grid((P.vol.NX + BX - 1) / BX, (P.z1 - P.z0 + NZ - 1) / NZ, (P.vol.NY + BY - 1) / BY);
  kern<<<grid, kThreads, smem, st>>>(map, P);
  const cudaError_t le = cudaGetLastError();
  if (le == cudaSuccess) g_windowed_launches.fetch_add(1, std::memory_order_relaxed);
  return le;
}

template <typename PT, int MODE, bool PAIR, int LANES, bool BZ0, int PF = 0>
cudaError_t launch_nz(const CUtensorMap& map, const BpArgs& P, const BpPlan& plan, cudaStream_t st) {
  // WBP: depth 16 or 8 (it runs once per reconstruction).  SIRT: the tuned depth.
  if constexpr (MODE == 0) {
    if (plan.nz == 16) return launch_one<PT, 0, PAIR, LANES, BZ0, 16>(map, P, plan.smem, st);
    return launch_one<PT, 0, PAIR, LANES, BZ0, 8>(map, P, plan.smem, st);
  } else {
    if (plan.nz == 8) return launch_one<PT, MODE, PAIR, LANES, BZ0, 8, PF>(map, P, plan.smem, st);
    if (plan.nz == 4) return launch_one<PT, MODE, PAIR, LANES, BZ0, 4, PF>(map, P, plan.smem, st);
    if (plan.nz == 16) return launch_one<PT, MODE, PAIR, LANES, BZ0, 16, PF>(map, P, plan.smem, st);
    if (plan.nz == 32) return launch_one<PT, MODE, PAIR, LANES, BZ0, 32, PF>(map, P, plan.smem, st);
    return cudaErrorInvalidValue;
  }
}

}  // namespace
}  // namespace mtr
