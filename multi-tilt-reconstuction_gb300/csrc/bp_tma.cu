// Back-projection gather with TMA-staged projection windows (sm_103a).
//
// One CTA owns a brick of BX x BY x BZ voxels.  For every angle the brick's
// footprint on the detector is a small window (<= 256 x 256 px); a producer
// warp streams these windows into a ring of NST shared-memory stages with
// 3-D tiled cp.async.bulk.tensor loads (one box per angle; pixels outside
// the detector are zero-filled by the TMA unit, which is exactly the
// reference's "drop taps outside the detector" for the numerator).  Eight
// consumer warps gather the four bilinear taps of every voxel from shared
// memory and accumulate over all angles in registers.
//
// Arithmetic per voxel and angle: one FFMA for the coordinate, FRND.FLOOR +
// FADD for the fraction, an integer add to index the window (the float floor
// is turned into an int by adding 1.5*2^23 and reading the bits, so no
// float->int conversion runs in the loop), four LDS and six FFMA/FADD for the
// interpolation.  When the y-map does not depend on Z (every synthetic and
// single-axis TXBR geometry), the y-part is computed once per voxel column.
//
// All mbarrier waits are bounded; a wait that gives up sets *err and the CTA
// drains its own in-flight copies (bounded) before returning.
#include <algorithm>
#include <atomic>
#include <type_traits>

#include "mtr_internal.h"
#include "tma.cuh"

namespace mtr {
namespace {

constexpr int NST = 4;             // pipeline stages
constexpr int kConsumerWarps = 8;  // 256 consumer threads
constexpr int kThreads = (kConsumerWarps + 1) * 32;
// Polls of the pipeline waits (producer on a free stage, consumers on a
// loaded window) before they give up; a launch argument, so that a test can
// make them give up at once.  The drain of the producer's own copies in
// flight always has the full bound: a CTA never exits with a copy pending.
constexpr uint32_t kDrainIters = 1u << 24;
std::atomic<unsigned> g_wait_iters{1u << 24};
constexpr float kMagic = 12582912.0f;  // 1.5 * 2^23: x + kMagic holds round(x) in its low bits
constexpr int kMagicBits = 0x4B400000;

struct WinConst {
  float xf, a1, a2, a3;  // x map relative to the CTA base voxel (fractional base)
  float yf, b1, b2, b3;
  int lxm, lym;          // window-local integer base minus the magic bits
  int ox, oy;            // window origin on the detector (ox aligned for TMA)
};

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

template <typename PT> __device__ __forceinline__ float to_f(PT v);
template <> __device__ __forceinline__ float to_f<float>(float v) { return v; }

__device__ __forceinline__ int floor_div(int a, int b) { return (a >= 0) ? a / b : -((-a + b - 1) / b); }

__device__ __forceinline__ int magic_int(float integral) { return __float_as_int(__fadd_rn(integral, kMagic)); }

// Gather of one voxel column (fixed X, Y; y-map without a Z term) from
// detector rows `row0` and `row0 + WX`, adding into s[0..NZ).  x advances by
// |a3| < 1 per voxel, so the fraction is stepped by one add and the tap
// pointer by a predicated increment instead of a floor per voxel.  ASC walks
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
  const PT* p = row0 + (magic_int(flx) + lxm);
#pragma unroll
  for (int i = 0; i < NZ; ++i) {
    const int z = ASC ? i : NZ - 1 - i;
    if (i > 0) {
      fx += step;
      const bool adv = fx >= 1.f;
      fx = adv ? fx - 1.f : fx;
      p += adv ? 1 : 0;
    }
    const float p00 = to_f(p[0]), p10 = to_f(p[1]);
    const float p01 = to_f(p[WX]), p11 = to_f(p[WX + 1]);
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
  const float* p = b + (magic_int(flx) + lxm);
#pragma unroll
  for (int i = 0; i < NZ; ++i) {
    const int z = ASC ? i : NZ - 1 - i;
    if (i > 0) {
      fx += step;
      const bool adv = fx >= 1.f;
      fx = adv ? fx - 1.f : fx;
      p += adv ? 1 : 0;
    }
    const float p0 = p[0], p1 = p[1];
    s[z] += fmaf(fx, p1 - p0, p0);
  }
}

// One brick (bx, by, bz) of one axis.  LANES: 0 = each warp a line of 32
// voxels along X (brick 32x8), 1 = a line along Y (brick 8x32, used when the
// detector x follows Y), 2 = an 8x4 patch (brick 32x8: on oblique axes the
// taps of a line fall on a diagonal of the window that maps several lanes to
// one shared-memory bank; a patch keeps them compact).  `smem` is the CTA's
// dynamic shared memory; `reinit` re-initialises the mbarriers of a CTA that
// already ran a brick.
template <typename PT, int MODE, int LANES, bool BZ0, int NZ>
__device__ __forceinline__ void bp_brick(const CUtensorMap* tmap, const BpArgs& P, int bx, int by, int bz,
                                         unsigned char* smem, bool reinit) {
  constexpr int BX = LANES == 1 ? kConsumerWarps : 32;
  constexpr int BY = LANES == 1 ? 32 : kConsumerWarps;
  uint64_t* full = reinterpret_cast<uint64_t*>(smem);
  uint64_t* empty = full + NST;
  WinConst* kc = reinterpret_cast<WinConst*>(smem + 128);
  const int A = P.ax.A;
  const size_t kc_bytes = ((size_t)A * sizeof(WinConst) + 127) & ~(size_t)127;
  const int win_elems = P.WX * P.WY;
  const size_t stage_bytes = (((size_t)win_elems * sizeof(PT)) + 127) & ~(size_t)127;
  PT* win0 = reinterpret_cast<PT*>(smem + 128 + kc_bytes);
  // per-warp blended row (uniform-row angles)
  float* blend = reinterpret_cast<float*>(smem + 128 + kc_bytes + NST * stage_bytes) + (threadIdx.x >> 5) * P.WX;

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
    const int ox = floor_div(xi + (int)floorf(xmin) - 1, P.align) * P.align;
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
      const uint32_t bytes = (uint32_t)(win_elems * sizeof(PT));
      int issued = 0;  // angles whose window load has been issued
      for (int a = 0; a < A; ++a) {
        const int s = a % NST;
        const int n = a / NST;
        if (n > 0 && !mbar_wait_bounded(&empty[s], (uint32_t)((n - 1) & 1), P.wait_iters)) {
          atomicExch(P.err, 2);
          break;
        }
        PT* dst = reinterpret_cast<PT*>(reinterpret_cast<unsigned char*>(win0) + s * stage_bytes);
        mbar_arrive_expect_tx(&full[s], bytes);
        tma_load_3d(dst, tmap, kc[a].ox, kc[a].oy, a, &full[s]);
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
  const unsigned lim_x = (unsigned)(WX - 1), lim_y = (unsigned)(P.WY - 1);
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
    const PT* w = reinterpret_cast<const PT*>(reinterpret_cast<const unsigned char*>(win0) + st * stage_bytes);
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
        const PT* row0 = w + rowi * WX;
        for (int i = lane; i < WX; i += 32) {
          const float r0 = to_f(row0[i]);
          blend[i] = fmaf(fy, to_f(row0[i + WX]) - r0, r0);
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
        } else {
          const PT* row0 = w + rowi * WX;
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
        const int i0 = bad ? 0 : ix + rowi * WX;  // never index outside the window
        const float p00 = to_f(w[i0]), p10 = to_f(w[i0 + 1]);
        const float p01 = to_f(w[i0 + WX]), p11 = to_f(w[i0 + WX + 1]);
        const float r0 = fmaf(fx, p10 - p00, p00);
        const float r1 = fmaf(fx, p11 - p01, p01);
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
template <typename PT, int MODE, int LANES, bool BZ0, int NZ>
__global__ void __launch_bounds__(kThreads, MODE == 1 ? (NZ >= 32 ? 3 : 5) : 4)
bp_tma_kernel(const __grid_constant__ CUtensorMap tmap, const BpArgs P) {
  extern __shared__ __align__(128) unsigned char smem[];
  bp_brick<PT, MODE, LANES, BZ0, NZ>(&tmap, P, blockIdx.x, blockIdx.z, blockIdx.y, smem, false);
}

template <typename PT, int MODE, int LANES, bool BZ0, int NZ>
cudaError_t launch_one(const CUtensorMap& map, const BpArgs& P, size_t smem, cudaStream_t st) {
  auto kern = bp_tma_kernel<PT, MODE, LANES, BZ0, NZ>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const int BX = LANES == 1 ? kConsumerWarps : 32, BY = LANES == 1 ? 32 : kConsumerWarps;
  const dim3 grid((P.vol.NX + BX - 1) / BX, (P.z1 - P.z0 + NZ - 1) / NZ, (P.vol.NY + BY - 1) / BY);
  kern<<<grid, kThreads, smem, st>>>(map, P);
  const cudaError_t le = cudaGetLastError();
  if (le == cudaSuccess) g_windowed_launches.fetch_add(1, std::memory_order_relaxed);
  return le;
}

template <typename PT, int MODE, int LANES, bool BZ0>
cudaError_t launch_nz(const CUtensorMap& map, const BpArgs& P, const BpPlan& plan, cudaStream_t st) {
  // WBP: depth 16 or 8 (it runs once per reconstruction).  SIRT: the tuned depth.
  if constexpr (MODE == 0) {
    if (plan.nz == 16) return launch_one<PT, 0, LANES, BZ0, 16>(map, P, plan.smem, st);
    return launch_one<PT, 0, LANES, BZ0, 8>(map, P, plan.smem, st);
  } else {
    if (plan.nz == 8) return launch_one<PT, MODE, LANES, BZ0, 8>(map, P, plan.smem, st);
    if (plan.nz == 4) return launch_one<PT, MODE, LANES, BZ0, 4>(map, P, plan.smem, st);
    if (plan.nz == 16) return launch_one<PT, MODE, LANES, BZ0, 16>(map, P, plan.smem, st);
    if (plan.nz == 32) return launch_one<PT, MODE, LANES, BZ0, 32>(map, P, plan.smem, st);
    return cudaErrorInvalidValue;
  }
}

}  // namespace

const int kBpDepths[4] = {4, 8, 16, 32};

namespace {

// Persistent SIRT back-projection over the bricks of many axes: each CTA
// takes items blockIdx.x, blockIdx.x + gridDim.x, ...; items are ordered by
// cost (most angles first) so the tail is short.  Between items every warp
// (producer included) meets at a barrier, then the mbarriers are
// re-initialised for the next brick.

template <int NZ>
__device__ __forceinline__ void bp_batch_item(const CUtensorMap* map, const BpArgs& P, const int* b,
                                              unsigned char* smem, bool reinit) {
  switch (b[4]) {  // lines along X or Y (axes tuned to patches keep their own launches)
    case 0: bp_brick<float, 1, 0, false, NZ>(map, P, b[0], b[1], b[2], smem, reinit); break;
    case 1: bp_brick<float, 1, 0, true, NZ>(map, P, b[0], b[1], b[2], smem, reinit); break;
    case 2: bp_brick<float, 1, 1, false, NZ>(map, P, b[0], b[1], b[2], smem, reinit); break;
    default: bp_brick<float, 1, 1, true, NZ>(map, P, b[0], b[1], b[2], smem, reinit); break;
  }
}

__global__ void __launch_bounds__(kThreads, 5)
bp_batch_kernel(const BpBatchDesc* __restrict__ descs, const long long* __restrict__ first, int n_desc,
                long long n_items, int* err, unsigned wait_iters) {
  extern __shared__ __align__(128) unsigned char smem[];
  // The item's arguments are staged in shared memory: read from there (like
  // the constant bank of a single launch) they cost no registers.
  __shared__ BpArgs sP;
  __shared__ const CUtensorMap* sMap;
  __shared__ int sB[5];  // brick x, y, z, depth, lane_y * 2 + bz0
  for (long long it = blockIdx.x; it < n_items; it += gridDim.x) {
    __syncthreads();
    if (threadIdx.x == 0) {
      const int2 item = work_item(first, n_desc, it);
      const BpBatchDesc& D = descs[item.x];
      sP = BpArgs{D.ax, D.vol, D.vol.Zs, D.vol.Zs + D.vol.NZ, D.WX, D.WY, D.align, 1, D.step, D.vol_out,
                  const_cast<float*>(D.cbp), D.vol_copy, D.copy_kind, err, wait_iters};
      sMap = D.map;
      const int gz = (D.vol.NZ + D.nz - 1) / D.nz;  // x fastest, then z, then y (as bp_tma_kernel)
      sB[0] = item.y % D.gx;
      sB[2] = (item.y / D.gx) % gz;
      sB[1] = item.y / (D.gx * gz);
      sB[3] = D.nz;
      sB[4] = D.lane_y * 2 + D.bz0;
    }
    __syncthreads();
    const bool reinit = it != blockIdx.x;
    if (sB[3] == 4) bp_batch_item<4>(sMap, sP, sB, smem, reinit);
    else if (sB[3] == 16) bp_batch_item<16>(sMap, sP, sB, smem, reinit);
    else bp_batch_item<8>(sMap, sP, sB, smem, reinit);
  }
}

}  // namespace

int backproject_batch_ctas_per_sm(size_t smem) {
  int n = 0;
  if (cudaFuncSetAttribute(bp_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, bp_batch_kernel, kThreads, smem) != cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  return n > 0 ? n : 1;
}

cudaError_t launch_backproject_batch(const BpBatchDesc* descs, const long long* first, int n_desc, long long n_items,
                                     size_t smem, int grid, int* err, cudaStream_t st) {
  cudaError_t e = cudaFuncSetAttribute(bp_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  bp_batch_kernel<<<grid, kThreads, smem, st>>>(descs, first, n_desc, n_items, err,
                                                 g_wait_iters.load(std::memory_order_relaxed));
  const cudaError_t le = cudaGetLastError();
  if (le == cudaSuccess) g_windowed_launches.fetch_add(1, std::memory_order_relaxed);
  return le;
}

void set_pipeline_wait_limit(long long polls) {
  g_wait_iters.store(polls < 0 ? (1u << 24) : (unsigned)std::min<long long>(polls, 0xffffffffLL),
                     std::memory_order_relaxed);
}

// Mean number of shared-memory wavefronts per tap load of one warp for a
// window row pitch WX: for a sample of angles, base fractions and depths the
// 32 lanes' tap addresses are laid out and, per tap, the largest number of
// distinct addresses that share a bank is counted (1 = conflict-free).
double window_bank_cost(const std::vector<double>& xc, const std::vector<double>& yc, int A, int lanes, int nz,
                        int WX) {
  const int na = std::min(A, 16);
  double total = 0;
  int n = 0;
  int cnt[32];
  int seen[32][32];
  for (int s = 0; s < na; ++s) {
    const int a = (int)((long long)s * A / na);
    const double a1 = xc[4 * a + 1], a2 = xc[4 * a + 2], a3 = xc[4 * a + 3];
    const double b1 = yc[4 * a + 1], b2 = yc[4 * a + 2], b3 = yc[4 * a + 3];
    for (int f = 0; f < 9; ++f) {
      const double xf = 0.1 + 0.35 * (f % 3), yf = 0.1 + 0.35 * (f / 3);
      for (int z = 0; z < nz; z += std::max(1, nz / 2)) {
        int r[32], c[32];
        for (int l = 0; l < 32; ++l) {
          const int tx = lanes == 0 ? l : lanes == 1 ? 0 : (l & 7);
          const int ty = lanes == 0 ? 0 : lanes == 1 ? l : (l >> 3);
          r[l] = (int)std::floor(yf + b1 * tx + b2 * ty + b3 * z + 64);
          c[l] = (int)std::floor(xf + a1 * tx + a2 * ty + a3 * z + 64);
        }
        for (int t = 0; t < 4; ++t) {
          std::fill(cnt, cnt + 32, 0);
          int worst = 0;
          for (int l = 0; l < 32; ++l) {
            const int addr = (r[l] + (t >> 1)) * WX + c[l] + (t & 1);
            const int bank = addr & 31;
            bool dup = false;
            for (int q = 0; q < cnt[bank]; ++q) dup = dup || seen[bank][q] == addr;
            if (!dup) seen[bank][cnt[bank]++] = addr;
            worst = std::max(worst, cnt[bank]);
          }
          total += worst;
          ++n;
        }
      }
    }
  }
  return n ? total / n : 1.0;
}

namespace {

// Window box for a brick of depth nz over all angles of an axis.
BpPlan plan_backproject_uncached(const std::vector<double>& xc, const std::vector<double>& yc, int A, bool half,
                                 int nz, int lane) {
  BpPlan p;
  p.align = half ? 8 : 4;
  p.nz = nz;
  // Choose the lane axis so that consecutive lanes step along detector x.
  double sx = 0, sy = 0;
  bool bz0 = true;
  for (int a = 0; a < A; ++a) {
    sx += std::fabs(xc[4 * a + 1]) - std::fabs(yc[4 * a + 1]);
    sy += std::fabs(xc[4 * a + 2]) - std::fabs(yc[4 * a + 2]);
    if (yc[4 * a + 3] != 0.0) bz0 = false;
  }
  // lane: -1 heuristic (lines along X or Y), 0 lines along X, 1 along Y, 2 patches
  p.lanes = lane < 0 ? (sy > sx ? 1 : 0) : std::min(lane, 2);
  p.bz0 = bz0;
  const int BX = p.lanes == 1 ? kConsumerWarps : 32, BY = p.lanes == 1 ? 32 : kConsumerWarps, BZ = nz;
  double ex = 0, ey = 0;
  for (int a = 0; a < A; ++a) {
    ex = std::max(ex, std::fabs(xc[4 * a + 1]) * (BX - 1) + std::fabs(xc[4 * a + 2]) * (BY - 1) +
                          std::fabs(xc[4 * a + 3]) * (BZ - 1));
    ey = std::max(ey, std::fabs(yc[4 * a + 1]) * (BX - 1) + std::fabs(yc[4 * a + 2]) * (BY - 1) +
                          std::fabs(yc[4 * a + 3]) * (BZ - 1));
  }
  // taps span [floor(min)-1, floor(max)+1], origin rounded down to the alignment
  const int wx = (int)std::ceil(ex) + 4 + p.align;
  const int wx_min = (wx + p.align - 1) / p.align * p.align;
  p.WY = (int)std::ceil(ey) + 4;
  auto smem_for = [&](int WX) {
    const size_t stage = (((size_t)WX * p.WY * (half ? 2 : 4)) + 127) & ~(size_t)127;
    return 128 + ((((size_t)A * sizeof(WinConst)) + 127) & ~(size_t)127) + NST * stage +
           (((size_t)kConsumerWarps * WX * sizeof(float) + 127) & ~(size_t)127);  // per-warp blended rows
  };
  // Row pitch (= box width): the smallest one whose tap loads have the fewest
  // bank conflicts, among widths that keep 5 CTAs per SM.  A wider box only
  // loads more of the (zero-filled or unused) detector columns.
  // A tap's bank is (row * WX + column) mod 32, and two lanes of a warp can
  // share an address only on the same row (their columns differ by less than
  // wx_min), so the cost depends on WX mod 32 alone: each residue is
  // simulated once.
  p.WX = wx_min;
  double best = 1e30;
  double cost_of[32];
  bool known[32] = {};
  for (int WX = wx_min; WX <= std::min(256, wx_min + 16 * p.align); WX += p.align) {
    if (WX > wx_min && smem_for(WX) > (size_t)(228 * 1024 / 5 - 1024)) break;
    if (!known[WX & 31]) {
      cost_of[WX & 31] = window_bank_cost(xc, yc, A, p.lanes, nz, WX);
      known[WX & 31] = true;
    }
    const double c = cost_of[WX & 31];
    if (c < best - 1e-9) {
      best = c;
      p.WX = WX;
    }
  }
  p.ok = p.WX <= 256 && p.WY <= 256 && (nz == 4 || nz == 8 || nz == 16 || nz == 32);
  p.smem = smem_for(p.WX);
  if (p.smem > 227 * 1024) p.ok = false;
  return p;
}

PlanMemo<BpPlan> g_bp_plans;

}  // namespace

BpPlan plan_backproject(const std::vector<double>& xc, const std::vector<double>& yc, int A, bool half, int nz,
                        int lane) {
  return g_bp_plans.get(plan_key(xc, yc, A, {half ? 1 : 0, nz, lane}),
                        [&] { return plan_backproject_uncached(xc, yc, A, half, nz, lane); });
}

template <typename PT>
cudaError_t launch_backproject_tma(const CUtensorMap& map, const BpPlan& plan, const AxisDev& ax, const VolDev& vol,
                                   int mode, float step, float* vol_out, float* cbp, void* vol_copy, int copy_kind,
                                   int z0, int z1, int* err, cudaStream_t st) {
  BpArgs P{ax,        vol,      z0,       z1,   plan.WX, plan.WY, plan.align,
           mode,      step,     vol_out,  cbp,  vol_copy, copy_kind, err,
           g_wait_iters.load(std::memory_order_relaxed)};
  if (mode == 0) {
    if (plan.lanes == 2) return plan.bz0 ? launch_nz<PT, 0, 2, true>(map, P, plan, st)
                                         : launch_nz<PT, 0, 2, false>(map, P, plan, st);
    if (plan.lanes == 1) return plan.bz0 ? launch_nz<PT, 0, 1, true>(map, P, plan, st)
                                         : launch_nz<PT, 0, 1, false>(map, P, plan, st);
    return plan.bz0 ? launch_nz<PT, 0, 0, true>(map, P, plan, st) : launch_nz<PT, 0, 0, false>(map, P, plan, st);
  }
  if constexpr (std::is_same<PT, float>::value) {
    if (plan.lanes == 2) return plan.bz0 ? launch_nz<PT, 1, 2, true>(map, P, plan, st)
                                         : launch_nz<PT, 1, 2, false>(map, P, plan, st);
    if (plan.lanes == 1) return plan.bz0 ? launch_nz<PT, 1, 1, true>(map, P, plan, st)
                                         : launch_nz<PT, 1, 1, false>(map, P, plan, st);
    return plan.bz0 ? launch_nz<PT, 1, 0, true>(map, P, plan, st) : launch_nz<PT, 1, 0, false>(map, P, plan, st);
  }
  return cudaErrorInvalidValue;  // the SIRT update reads the FP32 residual only
}

template cudaError_t launch_backproject_tma<float>(const CUtensorMap&, const BpPlan&, const AxisDev&, const VolDev&,
                                                   int, float, float*, float*, void*, int, int, int, int*,
                                                   cudaStream_t);

// ---- host: tensor-map encoding via the driver entry point -------------------
namespace {
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
    else
      cudaGetLastError();
  }
  return fn;
}
}  // namespace

bool encode_tensor_map_3d(CUtensorMap* map, const void* base, bool half, int width, int pitch, int height, int depth,
                          int bw, int bh) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) return false;
  const int es = half ? 2 : 4;
  if (((uintptr_t)base & 15) || ((size_t)pitch * es) % 16 || (bw * es) % 16 || bw > 256 || bh > 256) return false;
  cuuint64_t dims[3] = {(cuuint64_t)width, (cuuint64_t)height, (cuuint64_t)depth};
  cuuint64_t strides[2] = {(cuuint64_t)pitch * es, (cuuint64_t)pitch * es * height};
  cuuint32_t box[3] = {(cuuint32_t)bw, (cuuint32_t)bh, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = fn(map, half ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3,
                  const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

}  // namespace mtr
