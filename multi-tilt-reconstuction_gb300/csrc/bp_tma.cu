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

#include "bp_brick.cuh"

namespace mtr {
namespace {
// Polls of the pipeline waits before they give up (mtr_set_wait_limit).
std::atomic<unsigned> g_wait_iters{1u << 24};
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
    case 0: bp_brick<float, 1, false, 0, false, NZ>(map, P, b[0], b[1], b[2], smem, reinit); break;
    case 1: bp_brick<float, 1, false, 0, true, NZ>(map, P, b[0], b[1], b[2], smem, reinit); break;
    case 2: bp_brick<float, 1, false, 1, false, NZ>(map, P, b[0], b[1], b[2], smem, reinit); break;
    default: bp_brick<float, 1, false, 1, true, NZ>(map, P, b[0], b[1], b[2], smem, reinit); break;
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

namespace {

// The same for windows of 8-byte residual pairs: a voxel loads one pair per
// detector row.  A warp's 8-byte load is served per half-warp, and an element
// at index e covers banks 2e mod 32 and the next one, so per half-warp the
// wavefronts are the largest number of distinct elements sharing a bank pair;
// the result is normalised so that 1 is conflict-free (two wavefronts).
double pair_window_bank_cost(const std::vector<double>& xc, const std::vector<double>& yc, int A, int lanes, int nz,
                             int WX) {
  const int na = std::min(A, 16);
  double total = 0;
  int n = 0;
  int cnt[16];
  int seen[16][16];
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
        for (int t = 0; t < 2; ++t) {  // the two detector rows
          int wave = 0;
          for (int h = 0; h < 2; ++h) {
            std::fill(cnt, cnt + 16, 0);
            int worst = 0;
            for (int l = 16 * h; l < 16 * h + 16; ++l) {
              const int e = (r[l] + t) * WX + c[l];
              const int bank = e & 15;
              bool dup = false;
              for (int q = 0; q < cnt[bank]; ++q) dup = dup || seen[bank][q] == e;
              if (!dup) seen[bank][cnt[bank]++] = e;
              worst = std::max(worst, cnt[bank]);
            }
            wave += worst;
          }
          total += 0.5 * wave;
          ++n;
        }
      }
    }
  }
  return n ? total / n : 1.0;
}

}  // namespace

// Mean number of shared-memory wavefronts per tap load of one warp for a
// window row pitch WX: for a sample of angles, base fractions and depths the
// 32 lanes' tap addresses are laid out and, per tap, the largest number of
// distinct addresses that share a bank is counted (1 = conflict-free).
double window_bank_cost(const std::vector<double>& xc, const std::vector<double>& yc, int A, int lanes, int nz,
                        int WX, bool pairs) {
  if (pairs) return pair_window_bank_cost(xc, yc, A, lanes, nz, WX);
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
BpPlan plan_backproject_uncached(const std::vector<double>& xc, const std::vector<double>& yc, int A, int fmt,
                                 int nz, int lane) {
  BpPlan p;
  // FP32, planar and FP16 pair windows start on a 4-element (16-byte)
  // boundary; interleaved FP32 pair windows on an even pair column (16 bytes)
  const bool pairs = fmt == 1;
  p.align = pairs ? 2 : 4;
  p.pairs = fmt != 0;
  p.planar = fmt == 2;
  p.half = fmt == 3;
  p.nz = nz;
  const size_t es = pairs ? 8 : 4;          // bytes per window element
  const int planes = p.planar ? 2 : 1;      // window rows per detector row
  const size_t bes = p.pairs ? 8 : 4;       // bytes per blended-row element
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
    const size_t stage = (((size_t)WX * p.WY * planes * es) + 127) & ~(size_t)127;
    return 128 + ((((size_t)A * sizeof(WinConst)) + 127) & ~(size_t)127) + NST * stage +
           (((size_t)kConsumerWarps * WX * bes + 127) & ~(size_t)127);  // per-warp blended rows
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
  // (a TMA box row is at most 256 elements: 128 pairs)
  const int max_wx = pairs ? 128 : 256;
  for (int WX = wx_min; WX <= std::min(max_wx, wx_min + 16 * p.align); WX += p.align) {
    if (WX > wx_min && smem_for(WX) > (size_t)(228 * 1024 / 5 - 1024)) break;
    if (!known[WX & 31]) {
      // (planar: each of a voxel's four loads is a tap pattern of row pitch 2 WX)
      cost_of[WX & 31] = p.planar ? window_bank_cost(xc, yc, A, p.lanes, nz, 2 * WX, false)
                                  : window_bank_cost(xc, yc, A, p.lanes, nz, WX, pairs);
      known[WX & 31] = true;
    }
    const double c = cost_of[WX & 31];
    if (c < best - 1e-9) {
      best = c;
      p.WX = WX;
    }
  }
  p.ok = p.WX <= max_wx && p.WY * planes <= 256 && (nz == 4 || nz == 8 || nz == 16 || nz == 32) &&
         (!p.planar || bz0);  // (planar windows: y-maps without a Z term)
  p.smem = smem_for(p.WX);
  if (p.smem > 227 * 1024) p.ok = false;
  return p;
}

PlanMemo<BpPlan> g_bp_plans;

}  // namespace

BpPlan plan_backproject(const std::vector<double>& xc, const std::vector<double>& yc, int A, int fmt, int nz,
                        int lane) {
  return g_bp_plans.get(plan_key(xc, yc, A, {fmt, nz, lane}),
                        [&] { return plan_backproject_uncached(xc, yc, A, fmt, nz, lane); });
}

template <typename PT>
cudaError_t launch_backproject_tma(const CUtensorMap& map, const BpPlan& plan, const AxisDev& ax, const VolDev& vol,
                                   int mode, float step, float* vol_out, float* cbp, void* vol_copy, int copy_kind,
                                   int z0, int z1, int* err, cudaStream_t st) {
  BpArgs P{ax,        vol,      z0,       z1,   plan.WX, plan.WY, plan.align,
           mode,      step,     vol_out,  cbp,  vol_copy, copy_kind, err,
           g_wait_iters.load(std::memory_order_relaxed)};
  if (mode == 0) {
    if (plan.lanes == 2) return plan.bz0 ? launch_nz<PT, 0, false, 2, true>(map, P, plan, st)
                                         : launch_nz<PT, 0, false, 2, false>(map, P, plan, st);
    if (plan.lanes == 1) return plan.bz0 ? launch_nz<PT, 0, false, 1, true>(map, P, plan, st)
                                         : launch_nz<PT, 0, false, 1, false>(map, P, plan, st);
    return plan.bz0 ? launch_nz<PT, 0, false, 0, true>(map, P, plan, st) : launch_nz<PT, 0, false, 0, false>(map, P, plan, st);
  }
  if constexpr (std::is_same<PT, float>::value) {
    if (plan.pairs) return launch_backproject_tma_pairs(map, plan, P, st);
    if (plan.lanes == 2) return plan.bz0 ? launch_nz<PT, 1, false, 2, true>(map, P, plan, st)
                                         : launch_nz<PT, 1, false, 2, false>(map, P, plan, st);
    if (plan.lanes == 1) return plan.bz0 ? launch_nz<PT, 1, false, 1, true>(map, P, plan, st)
                                         : launch_nz<PT, 1, false, 1, false>(map, P, plan, st);
    return plan.bz0 ? launch_nz<PT, 1, false, 0, true>(map, P, plan, st) : launch_nz<PT, 1, false, 0, false>(map, P, plan, st);
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
