// Internal declarations shared by the CUDA translation units of libmtr.
#pragma once

#include <atomic>
#include <cuda.h>
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cuda_bf16.h>
#include <cstdint>
#include <initializer_list>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/mtr.h"

namespace mtr {

// Process-wide count of launches of the TMA-windowed projector kernels (the
// back-projection gather and the forward splat that stage detector windows in
// shared memory), single and persistent, counted when they are issued.
extern std::atomic<long long> g_windowed_launches;

// Maximum number of projection angles per tilt axis handled by one launch.
// The per-angle constants of a CTA live in shared memory (10 words/angle).
constexpr int kMaxAngles = 1024;

// Storage precision of one reconstruction (see mtr_precision in mtr.h).
enum class Prec : int { F32 = 0, MIXED_BF16 = 1, MIXED_F16 = 2 };

// Geometry of one tilt axis as the kernels see it: detector size, angle
// count and the 4+4 affine coefficients per angle in double (the reference's
// TXBR maps, FunctionOnGPU.cu:16-18: x = a0 + a1 X + a2 Y + a3 Z - 1).
struct AxisDev {
  int PX, PY, A;
  const double* xc;  // [A*4]
  const double* yc;  // [A*4]
  int pitch;         // row pitch of projection-space arrays, elements (>= PX)
};

// Row pitch used for device projection-space arrays: a multiple of 8
// elements so that rows start on 16-byte boundaries for fp16 and fp32 (TMA).
inline int projection_pitch(int px) { return (px + 7) / 8 * 8; }

// Volume frame (absolute voxel coordinates, end-exclusive), identical to the
// reference's VolumeSize (MrcFileIOBaseFunction.h:50-63).
struct VolDev {
  int Xs, Ys, Zs;  // start coordinates
  int NX, NY, NZ;  // extents
};

// Projection-space arrays of one axis in HBM: [A][PY][PX], x fastest.
// Volume arrays: [NZ][NY][NX], x fastest (the MRC output order).

// ---- kernels (projector.cu) ---------------------------------------------
// Back-projection gather.  mode 0: WBP (out = s/c, also writes c to cbp);
// mode 1: SIRT update (vol += step * s / cbp where cbp != 0).
template <typename PT>
void launch_backproject(const AxisDev& ax, const VolDev& vol, const PT* img, int mode, float step,
                        float* vol_out, float* cbp, void* vol_copy, int copy_kind, int z0, int z1,
                        cudaStream_t st);

// Forward splat: s[A][PY][PX] += A x over voxels z in [z0,z1) (s must be zeroed
// by the caller).  VT is the volume storage type read (float, bf16, half), or
// nullptr volume = all ones (computes the row sums c = A 1).
template <typename VT>
void launch_forward(const AxisDev& ax, const VolDev& vol, const VT* x, float* s, int z0, int z1,
                    cudaStream_t st);

// Residual: r = b - s/c (c != 0) else b; s <- 0; accumulate sum r^2 (FP64).
template <typename BT, typename RT>
void launch_residual(long long n, const BT* b, float* s, const float* c, RT* r, double* norm2,
                     cudaStream_t st);

// Exact key of a planner call: its integer arguments and the raw bytes of the
// 4*A coefficients of both maps.
inline std::string plan_key(const std::vector<double>& xc, const std::vector<double>& yc, int A,
                            std::initializer_list<int> args) {
  std::string k;
  k.reserve(args.size() * sizeof(int) + 8 * (size_t)A * sizeof(double));
  for (int v : args) k.append(reinterpret_cast<const char*>(&v), sizeof(int));
  k.append(reinterpret_cast<const char*>(xc.data()), 4 * (size_t)A * sizeof(double));
  k.append(reinterpret_cast<const char*>(yc.data()), 4 * (size_t)A * sizeof(double));
  return k;
}

// Process-wide memo of planner results.  A plan depends only on the planner's
// arguments, and planning simulates the warps' shared-memory bank pattern for
// every candidate row pitch (milliseconds per call), which every
// reconstruction of an already-seen geometry would otherwise repeat.
template <typename Plan>
struct PlanMemo {
  std::mutex mu;
  std::unordered_map<std::string, Plan> map;
  template <typename F>
  Plan get(std::string key, F&& compute) {
    {
      std::lock_guard<std::mutex> lock(mu);
      auto it = map.find(key);
      if (it != map.end()) return it->second;
    }
    const Plan p = compute();
    std::lock_guard<std::mutex> lock(mu);
    if (map.size() >= 1024) map.clear();  // keys are 64 bytes per angle
    map.emplace(std::move(key), p);
    return p;
  }
};

// ---- TMA-staged back-projection (bp_tma.cu) -------------------------------
// Window geometry of one axis for the brick shape used by the TMA kernel.
struct BpPlan {
  bool ok = false;     // window fits the TMA box and shared-memory limits
  int lanes = 0;       // warp layout: 0 lines along X, 1 lines along Y, 2 8x4 patches
  bool bz0 = false;    // y map independent of Z for every angle
  int WX = 0, WY = 0;  // window box (elements)
  int align = 4;       // TMA x alignment (elements)
  int nz = 8;          // brick depth (voxels per thread along Z): 4, 8 or 16
  bool pairs = false;  // windows of residual pairs (SIRT update) rather than FP32 projections (WBP)
  bool planar = false; // pairs as two FP32 planes per row (values, differences) instead of interleaved
  bool half = false;   // pairs as FP16 (value, difference) in 32 bits (mixed precision)
  size_t smem = 0;     // dynamic shared memory per CTA
};
extern const int kBpDepths[4];  // candidate brick depths of the SIRT back-projection
// Mean shared-memory wavefronts per tap access of one warp (1 = no bank
// conflict) for a detector window of row pitch WX, simulated on the host for
// a sample of the axis' angles; lanes: 0 lines along X, 1 along Y, 2 8x4 patches.
double window_bank_cost(const std::vector<double>& xc, const std::vector<double>& yc, int A, int lanes, int nz,
                        int WX, bool pairs = false);
// lane: -1 picks lines along the larger x-map slope, 0 = lines along X,
// 1 = lines along Y, 2 = 8x4 patches.
// pairs: windows of residual pairs for the SIRT update (false: FP32 windows
// of the projections for the WBP).
// fmt: 0 FP32 windows, 1 interleaved residual pairs, 2 planar residual pairs,
// 3 FP16 residual pairs (mixed precision).
BpPlan plan_backproject(const std::vector<double>& xc, const std::vector<double>& yc, int A, int fmt, int nz,
                        int lane = -1);
// Row pitch (pairs) of the residual pair array of a detector PX pixels wide:
// pair column c holds (r[c-1], r[c] - r[c-1]) for c in [0, PX], zero beyond,
// padded to a multiple of 4 pairs (32-byte rows).
inline int pair_pitch(int px) { return (px + 1 + 3) / 4 * 4; }
// Residual in pair form: r = b - s/c (c != 0, else b - s) per detector row
// (`rows` rows of `pitch` elements), written as pitch2 pairs per row:
// form 0 interleaved FP32 (value, difference), 1 planar (the row's values,
// then its differences), 2 FP16 (value, difference) in 32 bits; s reset to
// zero; norm2: FP64 sum of r^2 (or null).
template <typename BT>
void launch_residual_pairs(long long rows, int pitch, int pitch2, const BT* b, float* s, const float* c, float* rp,
                           int form, double* norm2, cudaStream_t st);
template <typename PT>
cudaError_t launch_backproject_tma(const CUtensorMap& map, const BpPlan& plan, const AxisDev& ax,
                                   const VolDev& vol, int mode, float step, float* vol_out, float* cbp,
                                   void* vol_copy, int copy_kind, int z0, int z1, int* err, cudaStream_t st);

// Polls a pipeline wait of the windowed back-projection makes before it
// gives up and flags the launch (negative: the default, 2^24); read at launch.
void set_pipeline_wait_limit(long long polls);

// 3-D tiled tensor map over [depth][height][pitch] fp32/fp16 elements with
// logical width `width`, box (bw, bh, 1), zero fill (bp_tma.cu).
bool encode_tensor_map_3d(CUtensorMap* map, const void* base, bool half, int width, int pitch, int height, int depth,
                          int bw, int bh);

// ---- windowed forward splat with TMA reduce (fwd_tma.cu) --------------------
struct FwdPlan {
  bool ok = false;
  int lanes = 0;       // warp layout: 0 lines along X, 1 lines along Y, 2 8x4 patches
  bool bz0 = false;
  int WX = 0, WY = 0;
  int mass_shift = 0;  // log2 bound of a pixel's weight from one brick
  int nz = 16;         // brick depth: 8, 16 or 32
  size_t smem = 0;
};
extern const int kFwdDepths[3];  // candidate brick depths of the forward splat
FwdPlan plan_forward(const std::vector<double>& xc, const std::vector<double>& yc, int A, int PX, int PY, int pitch,
                     int nz, int lane = -1);
template <typename VT>
cudaError_t launch_forward_tma(const CUtensorMap& smap, const FwdPlan& plan, const AxisDev& ax, const VolDev& vol,
                               const VT* x, int z0, int z1, int* err, cudaStream_t st);

// ---- persistent batched launches over many axes (batch.cu) -----------------
// One descriptor per (instance, axis); one work item per brick, (descriptor,
// brick index).  The kernels' CTAs loop over items (a grid sized to the GPU).
struct BpBatchDesc {
  AxisDev ax;
  VolDev vol;
  int WX, WY, align;
  int gx, gy;            // brick grid in X and Y
  int lane_y, bz0, nz;   // lane axis, z-independent y-map, brick depth (4, 8 or 16)
  float step;
  float* vol_out;        // SIRT iterate (updated in place)
  const float* cbp;      // back-projection weight sums
  void* vol_copy;        // bf16/f16 copy (mixed) or null
  int copy_kind;
  const CUtensorMap* map;  // device address of the residual's tensor map
};
struct FwdBatchDesc {
  AxisDev ax;
  VolDev vol;
  int WX, WY, mass_shift;
  int gx, gy;
  int lane_y, bz0, nz;   // brick depth 8, 16 or 32 (16 when the y-map depends on z)
  const void* x;         // volume read by the splat (float / bf16 / f16)
  const CUtensorMap* map;  // device address of the ray-sum tensor map
};
struct ResBatchDesc {
  const void* b;         // projections (float or half)
  float* s;
  const float* cf;
  float* r;
  long long n;
};
struct MaceBatchDesc {
  int K;
  void* w[MTR_MAX_AXES];  // MACE states: FP32, or FP16 deviations from wavg when w_half
  int w_half;
  float* x[MTR_MAX_AXES];
  void* xc[MTR_MAX_AXES];
  float* wavg;
  long long n;
  float rho;
  int copy_kind;
};
constexpr int kBatchChunk = 1 << 16;  // elements per residual / MACE work item

// Work list of a persistent kernel: descriptor d owns the items
// [first[d], first[d+1]) (first[n] = total); descriptors are stored in the
// order their items should be taken (most costly first).
#ifdef __CUDACC__
__device__ __forceinline__ int2 work_item(const long long* __restrict__ first, int n, long long it) {
  int lo = 0, hi = n - 1;  // the last descriptor with first[d] <= it
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (first[mid] <= it) lo = mid;
    else hi = mid - 1;
  }
  return make_int2(lo, (int)(it - first[lo]));
}
#endif

// Each descriptor carries the brick depth and lane axis its axis was tuned to.
cudaError_t launch_backproject_batch(const BpBatchDesc* descs, const long long* first, int n_desc, long long n_items,
                                     size_t smem, int grid, int* err, cudaStream_t st);
template <typename VT>
cudaError_t launch_forward_batch(const FwdBatchDesc* descs, const long long* first, int n_desc, long long n_items,
                                 size_t smem, int grid, cudaStream_t st);
int backproject_batch_ctas_per_sm(size_t smem);
template <typename VT>
int forward_batch_ctas_per_sm(size_t smem);
void launch_residual_batch(const ResBatchDesc* descs, const long long* first, int n_desc, long long n_items, int half_b,
                           int grid, cudaStream_t st);
void launch_mace_batch(const MaceBatchDesc* descs, const long long* first, int n_desc, long long n_items, int grid,
                       cudaStream_t st);

// ---- elementwise / MACE (mace.cu) ----------------------------------------
// Streaming multiprocessors of the current device (queried once per device).
int device_sm_count();
void launch_fill(float* p, long long n, float v, cudaStream_t st);
void launch_axpy_acc(float* dst, const float* src, long long n, cudaStream_t st);  // dst += src
// Fused MACE step over K axes (see mace.cu).  w: the K states, FP32 or
// (w_half) FP16 deviations from wavg; dchange null: no convergence record.
void launch_mace(int K, void* const* w, int w_half, float* const* x, float* wavg, long long n, float rho,
                 void* const* x_copy, int copy_kind, double* dchange, cudaStream_t st);
void launch_initial_z(const float* w, const float* wavg, float* z, long long n, cudaStream_t st);
// Mixed precision keeps each MACE state as the FP16 deviation d = w - w_avg
// from the FP32 consensus.  z = 2 w_avg - (w_avg + d):
void launch_initial_z_half(const __half* d, const float* wavg, float* z, long long n, cudaStream_t st);
// d = fp16(w - w_avg), and back: w = w_avg + d
void launch_state_dev(const float* w, const float* wavg, __half* d, long long n, cudaStream_t st);
void launch_state_value(const __half* d, const float* wavg, float* w, long long n, cudaStream_t st);
void launch_update_w(const float* v, const float* z, float* w, long long n, float step, cudaStream_t st);
void launch_convert_copy(const float* src, void* dst, int copy_kind, long long n, cudaStream_t st);
// dst[i] = (float)src[i]: FP16 projections widened for the FP32 WBP kernel.
void launch_widen(const __half* src, float* dst, long long n, cudaStream_t st);

}  // namespace mtr
