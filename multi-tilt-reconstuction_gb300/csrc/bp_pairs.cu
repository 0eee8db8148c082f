// The SIRT back-projection update over windows of residual pairs.
//
// The residual of such an axis is written as (value, next value - value)
// pairs, one per detector pixel (residual_pairs_kernel), so a voxel's two
// taps of one detector row are one 8-byte shared-memory load and their x
// interpolation one FFMA (the FP32-window kernel needs two loads, a
// subtraction and an FFMA).  Twice the window bytes: the tuner keeps this
// layout for an axis only where it measures faster (on lines of lanes that
// share detector rows it saves a third of the instructions; on oblique axes
// the 8-byte loads of a warp conflict in the shared-memory banks).  Planar
// pair windows hold a detector row as two FP32 rows, its values and then its
// differences: four 4-byte loads per voxel, with the FP32 window's bank
// pattern, but still one FFMA per row.  FP16 pair windows (mixed precision)
// hold each pair in 32 bits: one 4-byte load per row, the FP32 window's bytes
// halved and its bank pattern kept.  Separate from bp_tma.cu so that the
// two sets of instantiations compile in parallel.
#include "bp_brick.cuh"

namespace mtr {

cudaError_t launch_backproject_tma_pairs(const CUtensorMap& map, const BpPlan& plan, const BpArgs& P,
                                         cudaStream_t st) {
  if (plan.planar) {  // (planned for y-maps without a Z term only)
    if (!plan.bz0) return cudaErrorInvalidValue;
    if (plan.lanes == 2) return launch_nz<float, 1, true, 2, true, 1>(map, P, plan, st);
    if (plan.lanes == 1) return launch_nz<float, 1, true, 1, true, 1>(map, P, plan, st);
    return launch_nz<float, 1, true, 0, true, 1>(map, P, plan, st);
  }
  if (plan.half) {
    if (plan.lanes == 2) return plan.bz0 ? launch_nz<float, 1, true, 2, true, 2>(map, P, plan, st)
                                         : launch_nz<float, 1, true, 2, false, 2>(map, P, plan, st);
    if (plan.lanes == 1) return plan.bz0 ? launch_nz<float, 1, true, 1, true, 2>(map, P, plan, st)
                                         : launch_nz<float, 1, true, 1, false, 2>(map, P, plan, st);
    return plan.bz0 ? launch_nz<float, 1, true, 0, true, 2>(map, P, plan, st)
                    : launch_nz<float, 1, true, 0, false, 2>(map, P, plan, st);
  }
  if (plan.lanes == 2) return plan.bz0 ? launch_nz<float, 1, true, 2, true>(map, P, plan, st)
                                       : launch_nz<float, 1, true, 2, false>(map, P, plan, st);
  if (plan.lanes == 1) return plan.bz0 ? launch_nz<float, 1, true, 1, true>(map, P, plan, st)
                                       : launch_nz<float, 1, true, 1, false>(map, P, plan, st);
  return plan.bz0 ? launch_nz<float, 1, true, 0, true>(map, P, plan, st)
                  : launch_nz<float, 1, true, 0, false>(map, P, plan, st);
}

}  // namespace mtr
