// MRC stack data straight to device memory.  The reference reads a stack
// element by element with fread into host memory (MrcFileIOBaseFunction.cpp:
// 40-46) and its GPU code then copies it to the device every SIRT call.  Here
// the data block is read in large chunks into two pinned host buffers; each
// chunk's raw bytes are copied to the device and widened to float32 there,
// while the next chunk is read from the file.  The values are those of
// mtr_mrc_read_stack (same data offset rule, same per-mode conversion); the
// half-precision variant rounds them to FP16 on the device (round to nearest
// even), the storage precision of projections in the mixed-precision path.
#include <cstdint>
#include <cstdio>
#include <type_traits>
#include <sys/types.h>

#include <cuda_fp16.h>

#include "mtr_internal.h"
#include "mtr_runtime.h"

using namespace mtr;

namespace {

constexpr size_t kChunkBytes = size_t(32) << 20;

template <typename T>
__device__ __forceinline__ float widen(T v) { return (float)v; }
template <>
__device__ __forceinline__ float widen<__half>(__half v) { return __half2float(v); }

template <typename O>
__device__ __forceinline__ O narrow(float v);
template <>
__device__ __forceinline__ float narrow<float>(float v) { return v; }
template <>
__device__ __forceinline__ __half narrow<__half>(float v) { return __float2half_rn(v); }

template <typename T, typename O>
__global__ void convert_chunk_kernel(const T* __restrict__ src, O* __restrict__ dst, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    dst[i] = narrow<O>(widen(src[i]));
}

template <typename T, typename O>
void launch_convert_chunk(const void* src, O* dst, long long n, int sms, cudaStream_t st) {
  const long long blocks = std::min<long long>((n + 255) / 256, (long long)sms * 16);
  convert_chunk_kernel<T, O><<<(unsigned)std::max<long long>(blocks, 1), 256, 0, st>>>(static_cast<const T*>(src),
                                                                                       dst, n);
}

int mode_bytes(int mode) {
  switch (mode) {
    case MTR_MRC_MODE_BYTE: return 1;
    case MTR_MRC_MODE_SHORT: return 2;
    case MTR_MRC_MODE_FLOAT: return 4;
    case MTR_MRC_MODE_USHORT: return 2;
    case MTR_MRC_MODE_HALF: return 2;
    default: return 0;
  }
}

struct Staging {
  void* host[2] = {nullptr, nullptr};
  void* dev[2] = {nullptr, nullptr};
  cudaEvent_t done[2] = {nullptr, nullptr};
  FILE* f = nullptr;
  ~Staging() {
    for (int k = 0; k < 2; ++k) {
      if (done[k]) cudaEventSynchronize(done[k]);
      if (host[k]) cudaFreeHost(host[k]);
      if (dev[k]) cudaFree(dev[k]);
      if (done[k]) cudaEventDestroy(done[k]);
    }
    if (f) std::fclose(f);
  }
};

// The data block of `path` as n values of type O (float or __half) at d_out.
template <typename O>
mtr_status read_stack_device(mtr_context* ctx, const char* path, O* d_out, long long n) {
  if (!ctx || !path || !d_out || n <= 0) return set_error(ctx, MTR_ERR_INVALID_ARGUMENT, "invalid argument");
  DeviceGuard g(ctx->device);
  mtr_mrc_header h;
  mtr_status s = mtr_mrc_read_header(path, &h);
  if (s != MTR_OK) return set_error(ctx, s, std::string("cannot read the header of ") + path);
  const int nb = mode_bytes(h.mode);
  if (nb == 0) return set_error(ctx, MTR_ERR_UNSUPPORTED, "unsupported MRC mode");
  Staging stg;
  stg.f = std::fopen(path, "rb");
  if (!stg.f) return set_error(ctx, MTR_ERR_IO, std::string("cannot open ") + path);
  if (fseeko(stg.f, 0, SEEK_END) != 0) return set_error(ctx, MTR_ERR_IO, "seek");
  const long long size = (long long)ftello(stg.f);
  const long long need = n * nb;
  if (size < 1024 + need) return set_error(ctx, MTR_ERR_FORMAT, "file shorter than header + data");
  // the data block is the last n * bytes(mode) bytes of the file (as the host reader)
  if (fseeko(stg.f, (off_t)(size - need), SEEK_SET) != 0) return set_error(ctx, MTR_ERR_IO, "seek");
  const size_t chunk = std::min<size_t>(kChunkBytes, (size_t)need);
  // float32 data for a float32 result is copied as it is; everything else is
  // converted on the device from a raw staging chunk
  const bool direct = h.mode == MTR_MRC_MODE_FLOAT && std::is_same<O, float>::value;
  for (int k = 0; k < 2; ++k) {
    MTR_CK(ctx, cudaHostAlloc(&stg.host[k], chunk, cudaHostAllocDefault));
    if (!direct) MTR_CK(ctx, cudaMalloc(&stg.dev[k], chunk));
    MTR_CK(ctx, cudaEventCreateWithFlags(&stg.done[k], cudaEventDisableTiming));
  }
  const long long per_chunk = (long long)(chunk / (size_t)nb);
  long long done = 0;
  for (int c = 0; done < n; ++c) {
    const int k = c & 1;
    const long long m = std::min(per_chunk, n - done);
    // the copy that last read this pinned buffer (two chunks ago) must be done
    if (c >= 2) MTR_CK(ctx, cudaEventSynchronize(stg.done[k]));
    if (std::fread(stg.host[k], (size_t)nb, (size_t)m, stg.f) != (size_t)m)
      return set_error(ctx, MTR_ERR_IO, std::string("short read from ") + path);
    if (direct) {
      MTR_CK(ctx, cudaMemcpyAsync(d_out + done, stg.host[k], (size_t)m * 4, cudaMemcpyHostToDevice, ctx->stream));
    } else {
      MTR_CK(ctx, cudaMemcpyAsync(stg.dev[k], stg.host[k], (size_t)m * nb, cudaMemcpyHostToDevice, ctx->stream));
      O* dst = d_out + done;
      const int sms = ctx->num_sms;
      switch (h.mode) {
        case MTR_MRC_MODE_BYTE: launch_convert_chunk<uint8_t, O>(stg.dev[k], dst, m, sms, ctx->stream); break;
        case MTR_MRC_MODE_SHORT: launch_convert_chunk<int16_t, O>(stg.dev[k], dst, m, sms, ctx->stream); break;
        case MTR_MRC_MODE_USHORT: launch_convert_chunk<uint16_t, O>(stg.dev[k], dst, m, sms, ctx->stream); break;
        case MTR_MRC_MODE_FLOAT: launch_convert_chunk<float, O>(stg.dev[k], dst, m, sms, ctx->stream); break;
        default: launch_convert_chunk<__half, O>(stg.dev[k], dst, m, sms, ctx->stream); break;
      }
      MTR_CK_LAUNCH(ctx, "convert MRC chunk");
    }
    MTR_CK(ctx, cudaEventRecord(stg.done[k], ctx->stream));
    done += m;
  }
  MTR_CK(ctx, cudaStreamSynchronize(ctx->stream));
  return MTR_OK;
}

}  // namespace

extern "C" mtr_status mtr_mrc_read_stack_device(mtr_context* ctx, const char* path, float* d_out, long long n) {
  return read_stack_device<float>(ctx, path, d_out, n);
}

extern "C" mtr_status mtr_mrc_read_stack_device_half(mtr_context* ctx, const char* path, void* d_out, long long n) {
  return read_stack_device<__half>(ctx, path, static_cast<__half*>(d_out), n);
}
