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
// whole sectors).  Three window stages rotate: the flush of one angle
// overlaps the splat of the next, and the stage after it is zeroed during the
// conversion pass, so an angle costs two block barriers.
//
// Window accumulation is fixed point: shared-memory float atomicAdd is not a
// single native operation on this part, integer adds are.  Each CTA scales
// its voxels by a power of two S with S * max|v| < 2^b, b <= 21 - log2(depth),
// so every added value (a tap, or a column's merged run of at most depth
// voxels) rounds to an integer below 2^21 (rounded with the 1.5*2^23 trick,
// no float->int conversion) with an absolute error of at most
// 2^-(b+1) * max|v|.  The host bounds the weight one pixel can receive from
// one brick by 2^mass_shift (lattice points in the preimage of a 2x2-pixel
// square, times the brick depth) and b <= 30 - mass_shift keeps every window
// sum below 2^30.  Before the flush the window is converted back to float and
// divided by S (exact: S is a power of two).
//
// When the y-map has no Z term, a voxel column's y weights are common to the
// column and its x advances by |a3| < 1 per voxel: the column walk merges
// the column's 1-D splat in registers and adds one value per pixel it leaves
// (2-16x fewer shared-memory adds than four per voxel, depending on the tilt),
// in branch-free chunks where the slope allows, with red.shared adds on 32-bit
// shared addresses; bricks at the detector edge check each add against the
// window.  The per-tap path remains for z-dependent y-maps and slopes >= 0.999.
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
constexpr int kStages = 3;  // window stages in flight (splat, flush, next)
constexpr float kMagic = 12582912.0f;  // 1.5 * 2^23
constexpr int kMagicBits = 0x4B400000;

struct FwdConst {
  float xf, a1, a2, a3;
  float yf, b1, b2, b3;
  int lxm, lym;  // window-local integer base minus the magic bits
  int ox, oy;    // window origin (clamped inside the detector, ox aligned)
  int wlx;       // valid window columns (left of the detector's right edge)
  int interior;  // window not clamped and inside the detector: every tap is valid
  int pad[2];
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
// Zeroes a window stage (16-byte aligned) with all threads of the block.
__device__ __forceinline__ void zero_window(int* w, int n) {
  for (int i = threadIdx.x * 4; i < n; i += kThreads * 4) {
    if (i + 3 < n) *reinterpret_cast<int4*>(w + i) = make_int4(0, 0, 0, 0);
    else
      for (int q = i; q < n; ++q) w[q] = 0;
  }
}
__device__ __forceinline__ int floor_div(int a, int b) { return (a >= 0) ? a / b : -((-a + b - 1) / b); }
// round(w * v) for |w*v| < 2^22, as an integer, without a conversion instruction
__device__ __forceinline__ int fixq(float w, float v) { return __float_as_int(fmaf(w, v, kMagic)) - kMagicBits; }
// Integer add to the shared-memory word at 32-bit shared address `addr`
// (no value returned; the column walks keep their addresses in this form).
__device__ __forceinline__ void red_shared(uint32_t addr, int v) {
  asm volatile("red.shared.add.s32 [%0], %1;" ::"r"(addr), "r"(v) : "memory");
}

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

// Streaming splat of one voxel column (fixed X, Y; y-map without a Z term):
// its detector y (rows and weights wy0 / wy1) is common to the column and
// its detector x moves by |a3| < 1 per voxel, so consecutive voxels reach at
// most one new pixel.  The column's 1-D splat is accumulated in registers and
// a pixel is emitted (one integer add per detector row) only once the column
// has left it.  ROW: the warp's lanes share their rows and weights, so the
// unsplit values go into the warp's row buffer `row` (one add per pixel; the
// warp splits the row afterwards), else into detector rows `row` and
// `row + WX`.
//
// The walk always runs z upwards.  Where a3 < 0 it runs in the mirrored
// coordinate u = -x, which grows by |a3| per voxel: a voxel at u with
// fraction f splats (1 - f, f) onto mirrored pixels (p, p + 1), which are the
// original pixels (-p, -p - 1) with the original splat's weights, so the
// emissions go to window column (xi - ox) - p.  One code path serves both
// slope signs (half the unrolled code of a walk per sign).
//
// L > 1 (slope below 1 / L): a chunk of L voxels crosses at most one pixel
// boundary, so it accumulates without a branch and the column emits at most
// once per chunk; branching per voxel made the warp run the emission on
// almost every voxel (its lanes cross at different voxels).  S is the weight
// not yet emitted (pixels p and p + 1), a1 its part on p + 1.  Inside a chunk
// the fraction runs on past 1: a voxel beyond the crossing (fraction f in
// [1, 2)) is first added as if it were not (1 - f on p, f on p + 1) and C
// collects (f - 1) v, which moves it to its true pixels (2 - f on p + 1,
// f - 1 on p + 2) when the chunk ends.
//
// CHK: the brick's window is clamped at the detector edge (or reaches past
// it), so some of the column's pixels are off the detector: each emission
// checks its window column against the valid columns (span = 4 * valid
// columns, in bytes) and each detector row against the window (y0ok, y1ok),
// and drops what falls outside, as the reference drops off-detector taps.
template <int NZ, int L, bool ROW, bool CHK>
__device__ __forceinline__ void stream_column(uint32_t row, int WX, const float (&v)[NZ], float xr, float a3, int lxm,
                                              float wy0, float wy1, uint32_t span, bool y0ok, bool y1ok) {
  const int dir = a3 >= 0.f ? 1 : -1;
  const float u = a3 >= 0.f ? xr : -xr;
  const float flu = floorf(u);
  float fx = u - flu;
  const float step = fabsf(a3);
  // window column of pixel p: (xi - ox) + dir * p, with xi - ox = lxm + kMagicBits;
  // `at` is the shared address of the current pixel, `dstep` the next pixel's offset
  uint32_t at = row + 4u * (uint32_t)((lxm + kMagicBits) + dir * (magic_int(flu) - kMagicBits));
  const uint32_t dstep = dir > 0 ? 4u : 0xFFFFFFFCu, drow = 4u * (uint32_t)WX;
  auto emit = [&](uint32_t q, float e) {
    if (ROW) {
      red_shared(q, fixq(1.f, e));
    } else if (CHK) {
      const bool xok = q - row < span;  // (a column left of the window wraps to a large offset)
      if (xok && y0ok) red_shared(q, fixq(wy0, e));
      if (xok && y1ok) red_shared(q + drow, fixq(wy1, e));
    } else {
      red_shared(q, fixq(wy0, e));
      red_shared(q + drow, fixq(wy1, e));
    }
  };
  if constexpr (L == 1) {
    float acc0 = (1.f - fx) * v[0], acc1 = fx * v[0];
#pragma unroll
    for (int z = 1; z < NZ; ++z) {
      // the fraction is stepped (rounding < 4e-6 px over 32 voxels; the window
      // keeps one pixel of slack past the last exact tap on either side)
      fx += step;
      if (fx >= 1.f) {  // the column left the pixel at `at`
        fx -= 1.f;
        emit(at, acc0);
        acc0 = acc1;
        acc1 = 0.f;
        at += dstep;
      }
      acc0 = fmaf(1.f - fx, v[z], acc0);
      acc1 = fmaf(fx, v[z], acc1);
    }
    emit(at, acc0);
    emit(at + dstep, acc1);
  } else {
    float S = v[0], a1 = fx * v[0];
#pragma unroll
    for (int z0 = 1; z0 < NZ; z0 += L) {
      float C = 0.f;
#pragma unroll
      for (int j = 0; j < L; ++j) {
        if (z0 + j < NZ) {
          fx += step;
          S += v[z0 + j];
          a1 = fmaf(fx, v[z0 + j], a1);
          C = fmaf(__saturatef(fx - 1.f), v[z0 + j], C);  // f - 1 < 1: saturation is max(f - 1, 0)
        }
      }
      if (fx >= 1.f) {  // the chunk left the pixel at `at`
        emit(at, (S - a1) + C);
        S = a1 - C;
        a1 = C;
        fx -= 1.f;
        at += dstep;
      }
    }
    emit(at, S - a1);
    emit(at + dstep, a1);
  }
}

// stream_column with the longest chunk the slope allows (the bounds leave
// room for the stepped fraction's rounding: a chunk's fraction stays below 2).
template <int NZ, bool ROW, bool CHK>
__device__ __forceinline__ void splat_column(uint32_t row, int WX, const float (&v)[NZ], float xr, float a3, int lxm,
                                             float wy0, float wy1, uint32_t span = 0, bool y0ok = true,
                                             bool y1ok = true) {
  const float st = fabsf(a3);
  if (st < 0.2499f) stream_column<NZ, 4, ROW, CHK>(row, WX, v, xr, a3, lxm, wy0, wy1, span, y0ok, y1ok);
  else if (st < 0.4999f) stream_column<NZ, 2, ROW, CHK>(row, WX, v, xr, a3, lxm, wy0, wy1, span, y0ok, y1ok);
  else stream_column<NZ, 1, ROW, CHK>(row, WX, v, xr, a3, lxm, wy0, wy1, span, y0ok, y1ok);
}

// One brick (bx, by, zb) and angle group g of one axis; `smem` is the CTA's
// dynamic shared memory.  On return every bulk reduce it issued is complete.
template <typename VT, int LANES, bool BZ0, int NZ>
__device__ __forceinline__ void fwd_brick(const CUtensorMap* smap, const FwdArgs& P, int bx, int by, int zb, int g,
                                          unsigned char* smem) {
  constexpr int BX = LANES == 1 ? kWarps : 32;
  constexpr int BY = LANES == 1 ? 32 : kWarps;
  FwdConst* kc = reinterpret_cast<FwdConst*>(smem);
  const size_t kc_bytes = ((size_t)P.max_angles * sizeof(FwdConst) + 127) & ~(size_t)127;
  const int WX = P.WX, WY = P.WY;
  const int win_elems = WX * WY;
  const size_t stage_bytes = ((size_t)win_elems * 4 + 127) & ~(size_t)127;
  unsigned char* win0 = smem + kc_bytes + 128;
  float* red = reinterpret_cast<float*>(smem + kc_bytes);  // 32 floats for the block max
  // per-warp row buffers of the uniform-row angles (kept zero between uses)
  int* urow = reinterpret_cast<int*>(win0 + kStages * stage_bytes) + (threadIdx.x >> 5) * WX;
  for (int i = threadIdx.x & 31; i < WX; i += 32) urow[i] = 0;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int A = P.ax.A;
  const int a_begin = (int)((long long)A * g / P.groups), a_end = (int)((long long)A * (g + 1) / P.groups);
  const int na = a_end - a_begin;
  const int X0 = P.vol.Xs + bx * BX;
  const int Y0 = P.vol.Ys + by * BY;
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
    const int ox0 = floor_div(xi + (int)floorf(xmin) - 1, 4) * 4;
    const int oy0 = yi + (int)floorf(ymin) - 1;
    // clamp inside [0, pitch - WX] x [0, PY - WY]; the host checked both ranges exist
    const int ox = min(max(ox0, 0), P.ax.pitch - WX);
    const int oy = min(max(oy0, 0), PY - WY);
    k.ox = ox;
    k.oy = oy;
    k.lxm = xi - ox - kMagicBits;
    k.lym = yi - oy - kMagicBits;
    k.wlx = min(WX, PX - ox);
    // An unclamped window holds the whole footprint; inside the detector every tap is kept.
    k.interior = (ox == ox0 && oy == oy0 && ox + WX <= PX) ? 1 : 0;
    kc[j] = k;
  }

  // own voxels, loaded once (coalesced along lanes), and the brick's max |v|
  // LANES: 0 each warp a line along X, 1 a line along Y, 2 an 8x4 patch
  const int tx = LANES == 0 ? lane : LANES == 1 ? warp : (warp & 3) * 8 + (lane & 7);
  const int ty = LANES == 0 ? warp : LANES == 1 ? lane : (warp >> 2) * 4 + (lane >> 3);
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
  zero_window(reinterpret_cast<int*>(win0), win_elems);  // the first angle's stage
  __syncthreads();
  vmax = red[0];
  for (int w = 1; w < kWarps; ++w) vmax = fmaxf(vmax, red[w]);
  // S = 2^(b-e) with vmax < 2^e, so |v*S| < 2^b.  One emitted value merges at
  // most NZ voxels of weight <= 1 each: |emission| < 2^(b + log2 NZ) <= 2^21,
  // the range of the magic rounding.  A pixel's window sum stays below
  // 2^(b + mass_shift) <= 2^30 (no int overflow).
  int e2 = 0;
  if (vmax > 0.f && isfinite(vmax)) frexpf(vmax, &e2);
  constexpr int kLog2NZ = NZ >= 32 ? 5 : NZ >= 16 ? 4 : 3;
  const int bits = min(21 - kLog2NZ, 30 - P.mass_shift);
  const int sexp = max(-120, min(120, bits - e2));
  const float S = ldexpf(1.f, sexp), invS = ldexpf(1.f, -sexp);
#pragma unroll
  for (int z = 0; z < NZ; ++z) v[z] *= S;
  if (tid == 0) prefetch_tensormap(smap);

  // Three window stages: angle j splats into stage j % 3 (zeroed while angle
  // j - 1 was flushed), then converts it while zeroing the stage of angle
  // j + 1, whose last reader (the bulk reduce of angle j - 2) has finished.
  // Two block barriers per angle.
  for (int j = 0; j < na; ++j) {
    const int a = a_begin + j;
    const int st = j % kStages;
    int* wi = reinterpret_cast<int*>(win0 + st * stage_bytes);
    float* wf = reinterpret_cast<float*>(wi);
    const FwdConst k = kc[j];
    // Uniform rows: the detector y does not move along the lanes (|slope| * 31
    // below 1e-6 px), so the lanes of a warp share their two rows and weights.
    if (BZ0 && LANES != 2 && k.interior && fabsf(k.a3) < 0.999f && fabsf(LANES == 1 ? k.b2 : k.b1) < 3e-8f) {
      const float xr = fmaf(k.a2, (float)ty, fmaf(k.a1, (float)tx, k.xf));
      const float yr = __shfl_sync(0xffffffffu, fmaf(k.b2, (float)ty, fmaf(k.b1, (float)tx, k.yf)), 0);
      if (active) splat_column<NZ, true, false>(smem_u32(urow), WX, v, xr, k.a3, k.lxm, 1.f, 0.f);
      __syncwarp();
      // split the warp's row into the two detector rows (values up to 2^30:
      // rounded with a conversion, the magic-number rounding needs < 2^22)
      const float fly = floorf(yr);
      const float fy = yr - fly;
      int* rowp = wi + (magic_int(fly) + k.lym) * WX;
      for (int i = lane; i < WX; i += 32) {
        const int q = urow[i];
        if (q != 0) {
          const float uf = (float)q;
          red_shared(smem_u32(rowp + i), __float2int_rn((1.f - fy) * uf));
          red_shared(smem_u32(rowp + WX + i), __float2int_rn(fy * uf));
          urow[i] = 0;
        }
      }
    } else if (active && BZ0 && fabsf(k.a3) < 0.999f) {
      // stream the column; at an interior window every tap lands in the
      // window and on the detector, elsewhere each emission is checked
      const float xr = fmaf(k.a2, (float)ty, fmaf(k.a1, (float)tx, k.xf));
      const float yr = fmaf(k.b2, (float)ty, fmaf(k.b1, (float)tx, k.yf));
      const float fly = floorf(yr);
      const float fy = yr - fly;
      const int rowi = magic_int(fly) + k.lym;
      const uint32_t rowa = smem_u32(wi) + 4u * (uint32_t)(rowi * WX);
      if (k.interior)
        splat_column<NZ, false, false>(rowa, WX, v, xr, k.a3, k.lxm, 1.f - fy, fy);
      else
        splat_column<NZ, false, true>(rowa, WX, v, xr, k.a3, k.lxm, 1.f - fy, fy, 4u * (uint32_t)k.wlx,
                                      (unsigned)rowi < (unsigned)WY, (unsigned)(rowi + 1) < (unsigned)WY);
    } else if (active && BZ0 && k.interior) {
      // every tap lands in the window and on the detector: no per-tap tests
      const float xr = fmaf(k.a2, (float)ty, fmaf(k.a1, (float)tx, k.xf));
      const float yr = fmaf(k.b2, (float)ty, fmaf(k.b1, (float)tx, k.yf));
      const float fly = floorf(yr);
      const float fy = yr - fly;
      const int rowi = magic_int(fly) + k.lym;
      const float wy0 = 1.f - fy, wy1 = fy;
      int* rowp = wi + rowi * WX;
#pragma unroll
      for (int z = 0; z < NZ; ++z) {
        const float x = fmaf(k.a3, (float)z, xr);
        const float flx = floorf(x);
        const float fx = x - flx;
        int* r0 = rowp + (magic_int(flx) + k.lxm);
        const float g0 = wy0 * v[z], g1 = wy1 * v[z];
        const float wx0 = 1.f - fx;
        const uint32_t a0 = smem_u32(r0), a1 = a0 + 4u * (uint32_t)WX;
        red_shared(a0, fixq(wx0, g0));
        red_shared(a0 + 4u, fixq(fx, g0));
        red_shared(a1, fixq(wx0, g1));
        red_shared(a1 + 4u, fixq(fx, g1));
      }
    } else if (active) {
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
          if (x0ok) red_shared(smem_u32(r0), fixq(wx0, g0));
          if (x1ok) red_shared(smem_u32(r0 + 1), fixq(fx, g0));
        }
        if (y1ok) {
          if (x0ok) red_shared(smem_u32(r0 + WX), fixq(wx0, g1));
          if (x1ok) red_shared(smem_u32(r0 + WX + 1), fixq(fx, g1));
        }
      }
    }
    // the bulk reduce of angle j - 2 (the next stage's last reader) must be done reading
    if (tid == 0 && j >= 2) bulk_wait_read<1>();
    __syncthreads();
    // fixed point -> float (exact power-of-two scale), in place, 16 bytes a step
    for (int i = tid * 4; i < win_elems; i += kThreads * 4) {
      if (i + 3 < win_elems) {
        const int4 q = *reinterpret_cast<const int4*>(wi + i);
        *reinterpret_cast<float4*>(wf + i) =
            make_float4((float)q.x * invS, (float)q.y * invS, (float)q.z * invS, (float)q.w * invS);
      } else {
        for (int e = i; e < win_elems; ++e) wf[e] = (float)wi[e] * invS;
      }
    }
    if (j + 1 < na) zero_window(reinterpret_cast<int*>(win0 + ((j + 1) % kStages) * stage_bytes), win_elems);
    fence_proxy_async_smem();
    __syncthreads();
    if (tid == 0) {
      tma_reduce_add_3d(smap, wf, k.ox, k.oy, a);
      bulk_commit();
    }
  }
  if (tid == 0) bulk_wait_all();
}

// One CTA per (brick, angle group) of one axis.
template <typename VT, int LANES, bool BZ0, int NZ>
__global__ void __launch_bounds__(kThreads)
fwd_tma_kernel(const __grid_constant__ CUtensorMap smap, const FwdArgs P) {
  extern __shared__ __align__(128) unsigned char smem[];
  fwd_brick<VT, LANES, BZ0, NZ>(&smap, P, blockIdx.x, blockIdx.y, blockIdx.z / P.groups, blockIdx.z % P.groups,
                                 smem);
}

template <typename VT, int LY, bool BZ, int NZ>
cudaError_t launch_one(const CUtensorMap& map, FwdArgs P, size_t smem, int num_sms, cudaStream_t st) {
  auto kern = fwd_tma_kernel<VT, LY, BZ, NZ>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const int BX = LY == 1 ? kWarps : 32, BY = LY == 1 ? 32 : kWarps;
  const long long bricks = (long long)((P.vol.NX + BX - 1) / BX) * ((P.vol.NY + BY - 1) / BY) *
                           ((P.z1 - P.z0 + NZ - 1) / NZ);
  // split the angles over several CTAs when there are too few bricks to fill the GPU
  const long long target = (long long)num_sms * 8;
  int groups = (int)std::min<long long>((target + bricks - 1) / bricks, (long long)P.ax.A);
  if (groups < 1) groups = 1;
  P.groups = groups;
  P.max_angles = (P.ax.A + groups - 1) / groups;
  const dim3 grid((P.vol.NX + BX - 1) / BX, (P.vol.NY + BY - 1) / BY, ((P.z1 - P.z0 + NZ - 1) / NZ) * groups);
  kern<<<grid, kThreads, smem, st>>>(map, P);
  const cudaError_t le = cudaGetLastError();
  if (le == cudaSuccess) g_windowed_launches.fetch_add(1, std::memory_order_relaxed);
  return le;
}

// Z-dependent y-maps take the per-tap path and use one depth.
template <typename VT, int LY, bool BZ>
cudaError_t launch_nz(const CUtensorMap& map, const FwdArgs& P, const FwdPlan& plan, int sms, cudaStream_t st) {
  if constexpr (!BZ) {
    return launch_one<VT, LY, false, 16>(map, P, plan.smem, sms, st);
  } else {
    if (plan.nz == 16) return launch_one<VT, LY, true, 16>(map, P, plan.smem, sms, st);
    if (plan.nz == 8) return launch_one<VT, LY, true, 8>(map, P, plan.smem, sms, st);
    if (plan.nz == 32) return launch_one<VT, LY, true, 32>(map, P, plan.smem, sms, st);
    return cudaErrorInvalidValue;
  }
}

}  // namespace

const int kFwdDepths[3] = {8, 16, 32};

namespace {

// Persistent forward splat over the bricks of many axes (one angle group per
// brick): each CTA takes items blockIdx.x, blockIdx.x + gridDim.x, ...; every
// brick ends with its bulk reduces complete, so the next one reuses the
// shared-memory windows after a barrier.
template <typename VT, int NZ>
__device__ __forceinline__ void fwd_batch_item(const CUtensorMap* map, const FwdArgs& P, const int* b,
                                               unsigned char* smem) {
  if (b[4] == 3) fwd_brick<VT, 1, true, NZ>(map, P, b[0], b[1], b[2], 0, smem);
  else fwd_brick<VT, 0, true, NZ>(map, P, b[0], b[1], b[2], 0, smem);
}

template <typename VT>
__global__ void __launch_bounds__(kThreads)
fwd_batch_kernel(const FwdBatchDesc* __restrict__ descs, const long long* __restrict__ first, int n_desc,
                 long long n_items) {
  extern __shared__ __align__(128) unsigned char smem[];
  // The item's arguments are staged in shared memory (no registers held).
  __shared__ FwdArgs sP;
  __shared__ const CUtensorMap* sMap;
  __shared__ int sB[5];  // brick x, y, z, depth, lane_y * 2 + bz0
  for (long long it = blockIdx.x; it < n_items; it += gridDim.x) {
    __syncthreads();
    if (threadIdx.x == 0) {
      const int2 item = work_item(first, n_desc, it);
      const FwdBatchDesc& D = descs[item.x];
      sP = FwdArgs{D.ax, D.vol, D.vol.Zs, D.vol.Zs + D.vol.NZ, D.WX, D.WY, 1, D.ax.A, D.mass_shift, D.x, nullptr};
      sMap = D.map;
      sB[0] = item.y % D.gx;
      sB[1] = (item.y / D.gx) % D.gy;
      sB[2] = item.y / (D.gx * D.gy);
      sB[3] = D.nz;
      sB[4] = D.lane_y * 2 + D.bz0;
    }
    __syncthreads();
    switch (sB[4]) {
      case 0: fwd_brick<VT, 0, false, 16>(sMap, sP, sB[0], sB[1], sB[2], 0, smem); break;  // z-dependent y-map
      case 2: fwd_brick<VT, 1, false, 16>(sMap, sP, sB[0], sB[1], sB[2], 0, smem); break;
      default:
        if (sB[3] == 8) fwd_batch_item<VT, 8>(sMap, sP, sB, smem);
        else if (sB[3] == 32) fwd_batch_item<VT, 32>(sMap, sP, sB, smem);
        else fwd_batch_item<VT, 16>(sMap, sP, sB, smem);
    }
  }
}

}  // namespace

template <typename VT>
int forward_batch_ctas_per_sm(size_t smem) {
  int n = 0;
  if (cudaFuncSetAttribute(fwd_batch_kernel<VT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
          cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fwd_batch_kernel<VT>, kThreads, smem) != cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  return n > 0 ? n : 1;
}

template <typename VT>
cudaError_t launch_forward_batch(const FwdBatchDesc* descs, const long long* first, int n_desc, long long n_items,
                                 size_t smem, int grid, cudaStream_t st) {
  cudaError_t e = cudaFuncSetAttribute(fwd_batch_kernel<VT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  fwd_batch_kernel<VT><<<grid, kThreads, smem, st>>>(descs, first, n_desc, n_items);
  const cudaError_t le = cudaGetLastError();
  if (le == cudaSuccess) g_windowed_launches.fetch_add(1, std::memory_order_relaxed);
  return le;
}

template int forward_batch_ctas_per_sm<float>(size_t);
template int forward_batch_ctas_per_sm<__nv_bfloat16>(size_t);
template int forward_batch_ctas_per_sm<__half>(size_t);
template cudaError_t launch_forward_batch<float>(const FwdBatchDesc*, const long long*, int, long long, size_t,
                                                  int, cudaStream_t);
template cudaError_t launch_forward_batch<__nv_bfloat16>(const FwdBatchDesc*, const long long*, int, long long,
                                                          size_t, int, cudaStream_t);
template cudaError_t launch_forward_batch<__half>(const FwdBatchDesc*, const long long*, int, long long, size_t,
                                                   int, cudaStream_t);

namespace {

FwdPlan plan_forward_uncached(const std::vector<double>& xc, const std::vector<double>& yc, int A, int PX, int PY,
                              int pitch, int nz, int lane) {
  FwdPlan p;
  double sx = 0, sy = 0;
  bool bz0 = true;
  for (int a = 0; a < A; ++a) {
    sx += std::fabs(xc[4 * a + 1]) - std::fabs(yc[4 * a + 1]);
    sy += std::fabs(xc[4 * a + 2]) - std::fabs(yc[4 * a + 2]);
    if (yc[4 * a + 3] != 0.0) bz0 = false;
  }
  // lane: -1 heuristic (lines along X or Y), 0 lines along X, 1 along Y, 2 8x4 patches
  p.lanes = lane < 0 ? (sy > sx ? 1 : 0) : std::min(lane, 2);
  p.bz0 = bz0;
  p.nz = bz0 ? nz : 16;  // Z-dependent y-maps use one depth
  const int BX = p.lanes == 1 ? kWarps : 32, BY = p.lanes == 1 ? 32 : kWarps, BZ = p.nz;
  double ex = 0, ey = 0;
  for (int a = 0; a < A; ++a) {
    ex = std::max(ex, std::fabs(xc[4 * a + 1]) * (BX - 1) + std::fabs(xc[4 * a + 2]) * (BY - 1) +
                          std::fabs(xc[4 * a + 3]) * (BZ - 1));
    ey = std::max(ey, std::fabs(yc[4 * a + 1]) * (BX - 1) + std::fabs(yc[4 * a + 2]) * (BY - 1) +
                          std::fabs(yc[4 * a + 3]) * (BZ - 1));
  }
  const int wx_min = ((int)std::ceil(ex) + 4 + 4 + 3) / 4 * 4;
  p.WY = (int)std::ceil(ey) + 4;
  auto smem_for = [&](int WX) {
    const size_t stage = (((size_t)WX * p.WY * 4) + 127) & ~(size_t)127;
    // constants for up to A angles (one group) + block-max scratch + window
    // stages + per-warp row buffers of the uniform-row angles
    return ((((size_t)A * sizeof(FwdConst)) + 127) & ~(size_t)127) + 128 + kStages * stage +
           (size_t)kWarps * WX * sizeof(int);
  };
  // Row pitch (= box width) with the fewest shared-memory bank conflicts of
  // the warp's splat atomics, searched over a few widths only: a wider window
  // leaves the interior fast path at more bricks near the detector edge.
  p.WX = wx_min;
  double best = 1e30;
  for (int WX = wx_min; WX <= std::min(std::min(256, pitch), wx_min + 16); WX += 4) {
    if (WX > wx_min && smem_for(WX) > (size_t)(228 * 1024 / 4 - 1024)) break;
    const double c = window_bank_cost(xc, yc, A, p.lanes, p.nz, WX);
    if (c < best - 1e-9) {
      best = c;
      p.WX = WX;
    }
  }
  p.smem = smem_for(p.WX);
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
         p.smem <= 200 * 1024 && (p.nz == 8 || p.nz == 16 || p.nz == 32);
  (void)PX;
  return p;
}

PlanMemo<FwdPlan> g_fwd_plans;

}  // namespace

FwdPlan plan_forward(const std::vector<double>& xc, const std::vector<double>& yc, int A, int PX, int PY, int pitch,
                     int nz, int lane) {
  return g_fwd_plans.get(plan_key(xc, yc, A, {PX, PY, pitch, nz, lane}),
                         [&] { return plan_forward_uncached(xc, yc, A, PX, PY, pitch, nz, lane); });
}

template <typename VT>
cudaError_t launch_forward_tma(const CUtensorMap& smap, const FwdPlan& plan, const AxisDev& ax, const VolDev& vol,
                               const VT* x, int z0, int z1, int* err, cudaStream_t st) {
  const int sms = device_sm_count();
  FwdArgs P{ax, vol, z0, z1, plan.WX, plan.WY, 1, ax.A, plan.mass_shift, x, err};
  if (plan.lanes == 2) return plan.bz0 ? launch_nz<VT, 2, true>(smap, P, plan, sms, st)
                                       : launch_nz<VT, 2, false>(smap, P, plan, sms, st);
  if (plan.lanes == 1) return plan.bz0 ? launch_nz<VT, 1, true>(smap, P, plan, sms, st)
                                       : launch_nz<VT, 1, false>(smap, P, plan, sms, st);
  return plan.bz0 ? launch_nz<VT, 0, true>(smap, P, plan, sms, st) : launch_nz<VT, 0, false>(smap, P, plan, sms, st);
}

template cudaError_t launch_forward_tma<float>(const CUtensorMap&, const FwdPlan&, const AxisDev&, const VolDev&,
                                               const float*, int, int, int*, cudaStream_t);
template cudaError_t launch_forward_tma<__nv_bfloat16>(const CUtensorMap&, const FwdPlan&, const AxisDev&,
                                                       const VolDev&, const __nv_bfloat16*, int, int, int*,
                                                       cudaStream_t);
template cudaError_t launch_forward_tma<__half>(const CUtensorMap&, const FwdPlan&, const AxisDev&, const VolDev&,
                                                const __half*, int, int, int*, cudaStream_t);

}  // namespace mtr
