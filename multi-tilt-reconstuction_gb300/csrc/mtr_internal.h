// Internal declarations shared by the CUDA translation units of libmtr.
#pragma once

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
};

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
