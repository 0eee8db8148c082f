// Internal declarations shared by the CUDA translation units of libmtr.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cuda_bf16.h>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/mtr.h"

namespace mtr {

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

// ---- TMA-staged back-projection (bp_tma.cu) -------------------------------
// Window geometry of one axis for the brick shape used by the TMA kernel.
struct BpPlan {
  bool ok = false;     // window fits the TMA box and shared-memory limits
  bool lane_y = false; // lanes walk Y (detector x follows volume Y)
  bool bz0 = false;    // y map independent of Z for every angle
  int WX = 0, WY = 0;  // window box (elements)
  int align = 4;       // TMA x alignment (elements)
  size_t smem = 0;     // dynamic shared memory per CTA
};
BpPlan plan_backproject(const std::vector<double>& xc, const std::vector<double>& yc, int A, bool half);
template <typename PT>
cudaError_t launch_backproject_tma(const CUtensorMap& map, const BpPlan& plan, const AxisDev& ax,
                                   const VolDev& vol, int mode, float step, float* vol_out, float* cbp,
                                   void* vol_copy, int copy_kind, int z0, int z1, int* err, cudaStream_t st);

// 3-D tiled tensor map over [depth][height][pitch] fp32/fp16 elements with
// logical width `width`, box (bw, bh, 1), zero fill (bp_tma.cu).
bool encode_tensor_map_3d(CUtensorMap* map, const void* base, bool half, int width, int pitch, int height, int depth,
                          int bw, int bh);

// ---- windowed forward splat with TMA reduce (fwd_tma.cu) --------------------
struct FwdPlan {
  bool ok = false;
  bool lane_y = false;
  bool bz0 = false;
  int WX = 0, WY = 0;
  int mass_shift = 0;  // log2 bound of a pixel's weight from one brick
  size_t smem = 0;
};
FwdPlan plan_forward(const std::vector<double>& xc, const std::vector<double>& yc, int A, int PX, int PY, int pitch);
template <typename VT>
cudaError_t launch_forward_tma(const CUtensorMap& smap, const FwdPlan& plan, const AxisDev& ax, const VolDev& vol,
                               const VT* x, int z0, int z1, int* err, cudaStream_t st);

// ---- elementwise / MACE (mace.cu) ----------------------------------------
void launch_fill(float* p, long long n, float v, cudaStream_t st);
void launch_axpy_acc(float* dst, const float* src, long long n, cudaStream_t st);  // dst += src
// Fused MACE step over K axes (see mace.cu).
void launch_mace(int K, float* const* w, float* const* x, float* wavg, long long n, float rho,
                 void* const* x_copy, int copy_kind, double* dchange, cudaStream_t st);
void launch_initial_z(const float* w, const float* wavg, float* z, long long n, cudaStream_t st);
void launch_update_w(const float* v, const float* z, float* w, long long n, float step, cudaStream_t st);
void launch_convert_copy(const float* src, void* dst, int copy_kind, long long n, cudaStream_t st);

}  // namespace mtr
