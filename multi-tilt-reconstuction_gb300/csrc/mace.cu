// Elementwise and MACE consensus kernels (sm_103a).  These are HBM-bound:
// grid-stride loops over the volume, sized to a multiple of the SM count.
#include <atomic>

#include "mtr_internal.h"

namespace mtr {
namespace {

constexpr int kThreads = 256;

unsigned grid_for(long long n) {
  long long b = (n + kThreads - 1) / kThreads;
  const long long cap = (long long)device_sm_count() * 8;  // 8 resident CTAs per SM
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return (unsigned)b;
}

__global__ void fill_kernel(float* __restrict__ p, long long n, float v) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    p[i] = v;
}

__global__ void add_kernel(float* __restrict__ dst, const float* __restrict__ src, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    dst[i] = __fadd_rn(dst[i], src[i]);
}

// z = 2*w_avg - w (FunctionOnGPU.cu:268-276).
__global__ void initial_z_kernel(const float* __restrict__ w, const float* __restrict__ wavg, float* __restrict__ z,
                                 long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    z[i] = __fsub_rn(2.f * wavg[i], w[i]);
}

// Mixed precision stores each MACE state as its FP16 deviation from the FP32
// consensus, d_k = w_k - w_avg: the axes' states differ from their consensus
// by much less than they differ from zero, so FP16 rounds d_k far more finely
// than it would round w_k.  The state's value is w_avg + d_k (one FP32 add).
__device__ __forceinline__ float state_of(float wavg, __half d) { return __fadd_rn(wavg, __half2float(d)); }

// z = 2*w_avg - w from a deviation state, w = w_avg + d.
__global__ void initial_z_half_kernel(const __half* __restrict__ d, const float* __restrict__ wavg,
                                      float* __restrict__ z, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float wa = wavg[i];
    z[i] = __fsub_rn(2.f * wa, state_of(wa, d[i]));
  }
}

// d = fp16(w - w_avg) and w = w_avg + d (state to and from its stored form).
__global__ void state_dev_kernel(const float* __restrict__ w, const float* __restrict__ wavg, __half* __restrict__ d,
                                 long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    d[i] = __float2half_rn(__fsub_rn(w[i], wavg[i]));
}
__global__ void state_value_kernel(const __half* __restrict__ d, const float* __restrict__ wavg, float* __restrict__ w,
                                   long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    w[i] = state_of(wavg[i], d[i]);
}

// w = step*(2v - z) + (1-step)*w, with the reference host loop's float
// rounding (MultiAxis.cpp:33-38; no fused multiply-add).
__device__ __forceinline__ float mann(float v, float z, float w, float step) {
  const float t1 = __fsub_rn(2.f * v, z);
  const float t2 = __fmul_rn(step, t1);
  const float t3 = __fmul_rn(__fsub_rn(1.f, step), w);
  return __fadd_rn(t2, t3);
}

__global__ void update_w_kernel(const float* __restrict__ v, const float* __restrict__ z, float* __restrict__ w,
                                long long n, float step) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    w[i] = mann(v[i], z[i], w[i], step);
}

__global__ void convert_kernel(const float* __restrict__ src, void* __restrict__ dst, int kind, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    if (kind == 1) static_cast<__nv_bfloat16*>(dst)[i] = __float2bfloat16_rn(src[i]);
    else static_cast<__half*>(dst)[i] = __float2half_rn(src[i]);
  }
}

__global__ void widen_kernel(const __half* __restrict__ src, float* __restrict__ dst, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    dst[i] = __half2float(src[i]);
}

// One MACE outer step for all K axes at once, replacing the reference's
// initialZdata + runMaceOnCPU + Reduce/Bcast consensus (FunctionOnGPU.cu:268-313,
// MultiAxis.cpp:48-67).  On entry x[k] holds v_k = SIRT(z_k), w[k] the state
// w_k and wavg the consensus that z_k was formed from (z_k = 2 wavg - w_k,
// recomputed here instead of stored).  On exit:
//   w[k] = rho*(2 v_k - z_k) + (1-rho) w_k
//   wavg = (sum_k w[k]) / K      (summed in FP64)
//   x[k] = 2 wavg - w[k]         (the next outer iteration's z_k)
// and, when copy_kind != 0, x_copy[k] = x[k] in bf16/f16 for the forward pass.
// With WH (mixed precision) w[k] holds the FP16 deviation d_k = w_k - w_avg
// (state_of): the new states are computed in FP32, the consensus averages
// them unrounded (so the output carries no rounding of the step that made
// it), then each is stored as fp16(w_k - w_avg_new) and the next z_k is formed
// from the stored value, exactly as the next step recomputes it.  REC: dchange
// (2 doubles) accumulates sum (wavg_new - wavg_old)^2 and sum wavg_new^2 in
// FP64, the convergence test's relative change (without it those FP64
// operations are not run).
constexpr int kMaxK = MTR_MAX_AXES;
struct MacePtrs {
  void* w[kMaxK];
  float* x[kMaxK];
  void* xc[kMaxK];
};

// The state w_k at voxel i (consensus wa at that voxel).
template <bool WH>
__device__ __forceinline__ float ld_state(const void* w, long long i, float wa) {
  if constexpr (WH) return state_of(wa, static_cast<const __half*>(w)[i]);
  else return static_cast<const float*>(w)[i];
}
// Stores the new state v against the new consensus na and returns the state
// as it will be read back.
template <bool WH>
__device__ __forceinline__ float st_state(void* w, long long i, float v, float na) {
  if constexpr (WH) {
    const __half h = __float2half_rn(__fsub_rn(v, na));
    static_cast<__half*>(w)[i] = h;
    return state_of(na, h);
  } else {
    static_cast<float*>(w)[i] = v;
    return v;
  }
}

template <bool REC, bool WH>
__global__ void __launch_bounds__(kThreads)
mace_kernel(int K, MacePtrs P, float* __restrict__ wavg, long long n, float rho, int copy_kind,
            double* __restrict__ dchange) {
  double acc = 0.0, acc2 = 0.0;
  const double inv_k = 1.0 / (double)K;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float wa = wavg[i];
    float wn[kMaxK];
    double sum = 0.0;
#pragma unroll
    for (int k = 0; k < kMaxK; ++k) {
      if (k < K) {
        const float wk = ld_state<WH>(P.w[k], i, wa);
        const float zk = __fsub_rn(2.f * wa, wk);
        wn[k] = mann(P.x[k][i], zk, wk, rho);
        sum += (double)wn[k];
      }
    }
    const float na = (float)(sum * inv_k);  // FP64 mean; the reciprocal spares an FP64 division
    wavg[i] = na;
    if (REC) {
      const double d = (double)na - (double)wa;
      acc += d * d;
      acc2 += (double)na * (double)na;
    }
#pragma unroll
    for (int k = 0; k < kMaxK; ++k) {
      if (k < K) {
        const float zn = __fsub_rn(2.f * na, st_state<WH>(P.w[k], i, wn[k], na));
        P.x[k][i] = zn;
        if (copy_kind == 1) static_cast<__nv_bfloat16*>(P.xc[k])[i] = __float2bfloat16_rn(zn);
        else if (copy_kind == 2) static_cast<__half*>(P.xc[k])[i] = __float2half_rn(zn);
      }
    }
  }
  if (REC) {
    for (int o = 16; o > 0; o >>= 1) {
      acc += __shfl_xor_sync(0xffffffffu, acc, o);
      acc2 += __shfl_xor_sync(0xffffffffu, acc2, o);
    }
    __shared__ double red[2][kThreads / 32];
    if ((threadIdx.x & 31) == 0) {
      red[0][threadIdx.x >> 5] = acc;
      red[1][threadIdx.x >> 5] = acc2;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0, t2 = 0.0;
      for (int w = 0; w < kThreads / 32; ++w) {
        t += red[0][w];
        t2 += red[1][w];
      }
      atomicAdd(dchange, t);
      atomicAdd(dchange + 1, t2);
    }
  }
}

// MACE step over many reconstructions: item = (descriptor, chunk of voxels);
// the arithmetic is mace_kernel's (reference float rounding, FP64 consensus).
__global__ void __launch_bounds__(kThreads)
mace_batch_kernel(const MaceBatchDesc* __restrict__ descs, const long long* __restrict__ first, int n_desc,
                  long long n_items) {
  for (long long it = blockIdx.x; it < n_items; it += gridDim.x) {
    const int2 item = work_item(first, n_desc, it);
    const MaceBatchDesc& D = descs[item.x];
    const long long i0 = (long long)item.y * kBatchChunk;
    const long long i1 = min(D.n, i0 + kBatchChunk);
    const int K = D.K;
    const double inv_k = 1.0 / (double)K;
    for (long long i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
      const float wa = D.wavg[i];
      float wn[kMaxK];
      double sum = 0.0;
#pragma unroll
      for (int k = 0; k < kMaxK; ++k) {
        if (k < K) {
          const float wk = D.w_half ? ld_state<true>(D.w[k], i, wa) : ld_state<false>(D.w[k], i, wa);
          wn[k] = mann(D.x[k][i], __fsub_rn(2.f * wa, wk), wk, D.rho);
          sum += (double)wn[k];
        }
      }
      const float na = (float)(sum * inv_k);  // FP64 mean; the reciprocal spares an FP64 division
      D.wavg[i] = na;
#pragma unroll
      for (int k = 0; k < kMaxK; ++k) {
        if (k < K) {
          const float ws = D.w_half ? st_state<true>(D.w[k], i, wn[k], na) : st_state<false>(D.w[k], i, wn[k], na);
          const float zn = __fsub_rn(2.f * na, ws);
          D.x[k][i] = zn;
          if (D.copy_kind == 1) static_cast<__nv_bfloat16*>(D.xc[k])[i] = __float2bfloat16_rn(zn);
          else if (D.copy_kind == 2) static_cast<__half*>(D.xc[k])[i] = __float2half_rn(zn);
        }
      }
    }
  }
}

}  // namespace

int device_sm_count() {
  constexpr int kMaxDevices = 64;
  static std::atomic<int> cached[kMaxDevices];  // 0 = not yet queried
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    dev = -1;
  }
  if (dev >= 0) {
    const int c = cached[dev].load(std::memory_order_relaxed);
    if (c > 0) return c;
  }
  int n = 0;
  if (dev < 0 || cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) {
    cudaGetLastError();
    return 1;  // a one-SM grid still covers everything through its grid-stride loop
  }
  cached[dev].store(n, std::memory_order_relaxed);
  return n;
}

void launch_mace_batch(const MaceBatchDesc* descs, const long long* first, int n_desc, long long n_items, int grid,
                       cudaStream_t st) {
  mace_batch_kernel<<<grid, kThreads, 0, st>>>(descs, first, n_desc, n_items);
}

void launch_fill(float* p, long long n, float v, cudaStream_t st) {
  fill_kernel<<<grid_for(n), kThreads, 0, st>>>(p, n, v);
}
void launch_axpy_acc(float* dst, const float* src, long long n, cudaStream_t st) {
  add_kernel<<<grid_for(n), kThreads, 0, st>>>(dst, src, n);
}
void launch_initial_z(const float* w, const float* wavg, float* z, long long n, cudaStream_t st) {
  initial_z_kernel<<<grid_for(n), kThreads, 0, st>>>(w, wavg, z, n);
}
void launch_initial_z_half(const __half* d, const float* wavg, float* z, long long n, cudaStream_t st) {
  initial_z_half_kernel<<<grid_for(n), kThreads, 0, st>>>(d, wavg, z, n);
}
void launch_state_dev(const float* w, const float* wavg, __half* d, long long n, cudaStream_t st) {
  state_dev_kernel<<<grid_for(n), kThreads, 0, st>>>(w, wavg, d, n);
}
void launch_state_value(const __half* d, const float* wavg, float* w, long long n, cudaStream_t st) {
  state_value_kernel<<<grid_for(n), kThreads, 0, st>>>(d, wavg, w, n);
}
void launch_update_w(const float* v, const float* z, float* w, long long n, float step, cudaStream_t st) {
  update_w_kernel<<<grid_for(n), kThreads, 0, st>>>(v, z, w, n, step);
}
void launch_convert_copy(const float* src, void* dst, int copy_kind, long long n, cudaStream_t st) {
  convert_kernel<<<grid_for(n), kThreads, 0, st>>>(src, dst, copy_kind, n);
}
void launch_widen(const __half* src, float* dst, long long n, cudaStream_t st) {
  widen_kernel<<<grid_for(n), kThreads, 0, st>>>(src, dst, n);
}
void launch_mace(int K, void* const* w, int w_half, float* const* x, float* wavg, long long n, float rho,
                 void* const* x_copy, int copy_kind, double* dchange, cudaStream_t st) {
  MacePtrs P{};
  for (int k = 0; k < K && k < kMaxK; ++k) {
    P.w[k] = w[k];
    P.x[k] = x[k];
    P.xc[k] = x_copy ? x_copy[k] : nullptr;
  }
  const unsigned g = grid_for(n);
  if (dchange) {
    if (w_half) mace_kernel<true, true><<<g, kThreads, 0, st>>>(K, P, wavg, n, rho, copy_kind, dchange);
    else mace_kernel<true, false><<<g, kThreads, 0, st>>>(K, P, wavg, n, rho, copy_kind, dchange);
  } else {
    if (w_half) mace_kernel<false, true><<<g, kThreads, 0, st>>>(K, P, wavg, n, rho, copy_kind, nullptr);
    else mace_kernel<false, false><<<g, kThreads, 0, st>>>(K, P, wavg, n, rho, copy_kind, nullptr);
  }
}

}  // namespace mtr
