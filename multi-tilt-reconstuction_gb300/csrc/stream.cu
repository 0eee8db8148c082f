// Single-GPU streaming slab loop (MTR_FLAG_STREAM_SLABS).
//
// The reference splits the volume into Z-slabs over MPI ranks (divideSlice,
// MultiAxis.cpp:13-31); each rank splats its slab into partial ray sums that
// are reduced in projection space every SIRT iteration before the residual
// (FunctionOnGPU.cu:218-238).  Here the slabs take turns on one GPU instead:
// the volume-sized arrays (iterates x_k, MACE states w_k, weight sums cbp_k,
// forward copies, consensus) stay in pinned host memory, and two slab slots
// of device memory rotate through them.  One SIRT iteration of axis k:
//
//   forward   for each slab j: copy x_k[j] in (stream `in`), splat it into
//             the axis' ray sums s_k (context stream) -- the ray sums of all
//             slabs add up in s_k, which is the cross-rank reduction;
//   residual  once, after the last slab (context stream);
//   update    for each slab j: copy x_k[j] and cbp_k[j] in, back-project the
//             residual into the slab (context stream), copy x_k[j] and its
//             forward copy out (stream `out`).
//
// Slot s is reused only after the copy out of its last slab (or, in the
// forward pass, its splat) has finished, so the copies of one slab overlap
// the kernels of the other.  The kernels are the device-resident path's
// (windowed where the windows fit, tiles tuned for one slab), given the slab
// as their Z range.  The WBP initialisation and the MACE steps move their
// slabs through the working set on the context stream.
#include <algorithm>
#include <memory>
#include <new>

#include "mtr_internal.h"
#include "mtr_runtime.h"

using namespace mtr;

SlabStream::~SlabStream() {
  for (cudaEvent_t e : loaded) if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : computed) if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : freed) if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : mark) if (e) cudaEventDestroy(e);
  if (in) cudaStreamDestroy(in);
  if (out) cudaStreamDestroy(out);
}

namespace {

// Z planes [z0, z1) of slab j and its offset (voxels) into the volume arrays.
struct SlabRange {
  int z0, z1;
  long long off, n;
};

SlabRange slab_range(const mtr_recon* r, int j, int depth) {
  const SlabStream& S = *r->slabs;
  const int z0 = r->vol.Zs + j * depth;
  const int z1 = std::min(z0 + depth, r->vol.Zs + r->vol.NZ);
  return SlabRange{z0, z1, (long long)(z0 - r->vol.Zs) * S.plane, (long long)(z1 - z0) * S.plane};
}

char* bytes_at(const DevBuf& b, long long elems, size_t esize) { return static_cast<char*>(b.p) + elems * esize; }

// `dst` waits for the work enqueued so far on `src` (mark[i] is the event used).
mtr_status after(mtr_context* ctx, SlabStream& S, int i, cudaStream_t dst, cudaStream_t src) {
  MTR_CK(ctx, cudaEventRecord(S.mark[i], src));
  MTR_CK(ctx, cudaStreamWaitEvent(dst, S.mark[i], 0));
  return MTR_OK;
}

// Forward splat of axis k, slab by slab, into its ray sums.
mtr_status forward_pass(mtr_recon* r, int k) {
  mtr_context* ctx = r->ctx;
  SlabStream& S = *r->slabs;
  AxisState& a = r->ax[k];
  const cudaStream_t c = ctx->stream;
  const int ck = recon_copy_kind(r);
  const size_t es = ck ? 2 : 4;               // the forward reads the copy (mixed) or x itself
  const DevBuf& src = ck ? a.xcopy : a.x;
  // the copies in read what the last update pass (or a MACE step) wrote out
  mtr_status st = after(ctx, S, 2, S.in, S.out);
  if (st != MTR_OK) return st;
  for (int j = 0; j < S.nslab; ++j) {
    const int s = j & 1;
    const SlabRange R = slab_range(r, j, S.depth);
    void* dst = ck ? S.xc[s].p : S.x[s].p;
    MTR_CK(ctx, cudaStreamWaitEvent(S.in, S.freed[s], 0));
    MTR_CK(ctx, cudaMemcpyAsync(dst, bytes_at(src, R.off, es), (size_t)R.n * es, cudaMemcpyDefault, S.in));
    MTR_CK(ctx, cudaEventRecord(S.loaded[s], S.in));
    MTR_CK(ctx, cudaStreamWaitEvent(c, S.loaded[s], 0));
    st = recon_enqueue_forward_span(r, k, VolSpan{R.z0, R.z1, S.x[s].as<float>(), S.cbp[s].as<float>(), S.xc[s].p});
    if (st != MTR_OK) return st;
    MTR_CK(ctx, cudaEventRecord(S.freed[s], c));
  }
  return MTR_OK;
}

// SIRT update of axis k from its residual, slab by slab.
mtr_status update_pass(mtr_recon* r, int k) {
  mtr_context* ctx = r->ctx;
  SlabStream& S = *r->slabs;
  AxisState& a = r->ax[k];
  const cudaStream_t c = ctx->stream;
  const int ck = recon_copy_kind(r);
  for (int j = 0; j < S.nslab; ++j) {
    const int s = j & 1;
    const SlabRange R = slab_range(r, j, S.depth);
    const size_t nb = (size_t)R.n * 4;
    MTR_CK(ctx, cudaStreamWaitEvent(S.in, S.freed[s], 0));
    MTR_CK(ctx, cudaMemcpyAsync(S.x[s].p, bytes_at(a.x, R.off, 4), nb, cudaMemcpyDefault, S.in));
    MTR_CK(ctx, cudaMemcpyAsync(S.cbp[s].p, bytes_at(a.cbp, R.off, 4), nb, cudaMemcpyDefault, S.in));
    MTR_CK(ctx, cudaEventRecord(S.loaded[s], S.in));
    MTR_CK(ctx, cudaStreamWaitEvent(c, S.loaded[s], 0));
    mtr_status st = recon_enqueue_bp_span(r, k, 1, VolSpan{R.z0, R.z1, S.x[s].as<float>(), S.cbp[s].as<float>(),
                                                           S.xc[s].p}, false);
    if (st != MTR_OK) return st;
    MTR_CK(ctx, cudaEventRecord(S.computed[s], c));
    MTR_CK(ctx, cudaStreamWaitEvent(S.out, S.computed[s], 0));
    MTR_CK(ctx, cudaMemcpyAsync(bytes_at(a.x, R.off, 4), S.x[s].p, nb, cudaMemcpyDefault, S.out));
    if (ck)
      MTR_CK(ctx, cudaMemcpyAsync(bytes_at(a.xcopy, R.off, 2), S.xc[s].p, (size_t)R.n * 2, cudaMemcpyDefault, S.out));
    MTR_CK(ctx, cudaEventRecord(S.freed[s], S.out));
  }
  return MTR_OK;
}

// MACE step `it` over all axes (the fused kernel of the device-resident
// path), chunk by chunk of mace_planes Z planes on the context stream.
mtr_status mace_pass(mtr_recon* r, int it) {
  mtr_context* ctx = r->ctx;
  SlabStream& S = *r->slabs;
  const cudaStream_t c = ctx->stream;
  const int K = r->K, ck = recon_copy_kind(r);
  mtr_status st = after(ctx, S, 2, c, S.out);  // the last update pass' copies out
  if (st != MTR_OK) return st;
  // chunk layout: x_k (FP32) x K, w_avg (FP32), w_k (FP16 in mixed precision,
  // else FP32) x K, forward copies (mixed) x K
  const long long cap = (long long)S.mace_planes * S.plane;
  const size_t ws_es = ck ? 2 : 4;
  char* base = static_cast<char*>(S.mace.p);
  void* ws[MTR_MAX_AXES];
  float* xs[MTR_MAX_AXES];
  void* xcs[MTR_MAX_AXES];
  float* wa = reinterpret_cast<float*>(base + (long long)K * cap * 4);
  char* wbase = base + (long long)(K + 1) * cap * 4;
  for (int k = 0; k < K; ++k) {
    xs[k] = reinterpret_cast<float*>(base + (long long)k * cap * 4);
    ws[k] = wbase + (long long)k * cap * ws_es;
    xcs[k] = ck ? static_cast<void*>(wbase + (long long)K * cap * ws_es + (long long)k * cap * 2) : nullptr;
  }
  for (int j = 0; j * S.mace_planes < r->vol.NZ; ++j) {
    const SlabRange R = slab_range(r, j, S.mace_planes);
    const size_t nb = (size_t)R.n * 4, nw = (size_t)R.n * ws_es;
    for (int k = 0; k < K; ++k) {
      MTR_CK(ctx, cudaMemcpyAsync(ws[k], bytes_at(r->ax[k].w, R.off, ws_es), nw, cudaMemcpyDefault, c));
      MTR_CK(ctx, cudaMemcpyAsync(xs[k], bytes_at(r->ax[k].x, R.off, 4), nb, cudaMemcpyDefault, c));
    }
    MTR_CK(ctx, cudaMemcpyAsync(wa, bytes_at(r->wavg, R.off, 4), nb, cudaMemcpyDefault, c));
    {
      ProfScope ps(ctx, MTR_KERNEL_MACE);
      launch_mace(K, ws, ck ? 1 : 0, xs, wa, R.n, r->p.mace_step, xcs, ck, recon_change_slot(r, it), c);
    }
    MTR_CK_LAUNCH(ctx, "mace (streamed)");
    for (int k = 0; k < K; ++k) {
      MTR_CK(ctx, cudaMemcpyAsync(bytes_at(r->ax[k].w, R.off, ws_es), ws[k], nw, cudaMemcpyDefault, c));
      MTR_CK(ctx, cudaMemcpyAsync(bytes_at(r->ax[k].x, R.off, 4), xs[k], nb, cudaMemcpyDefault, c));
      if (ck)
        MTR_CK(ctx, cudaMemcpyAsync(bytes_at(r->ax[k].xcopy, R.off, 2), xcs[k], (size_t)R.n * 2, cudaMemcpyDefault,
                                    c));
    }
    MTR_CK(ctx, cudaMemcpyAsync(bytes_at(r->wavg, R.off, 4), wa, nb, cudaMemcpyDefault, c));
  }
  // the next forward pass' copies in read what this step wrote out
  return after(ctx, S, 0, S.in, c);
}

}  // namespace

mtr_status mtr::stream_setup(mtr_recon* r) {
  mtr_context* ctx = r->ctx;
  std::unique_ptr<SlabStream> S(new (std::nothrow) SlabStream());
  if (!S) return set_error(ctx, MTR_ERR_OUT_OF_MEMORY, "host allocation");
  if (r->p.slab_depth < 0) return set_error(ctx, MTR_ERR_INVALID_ARGUMENT, "negative slab depth");
  const int NZ = r->vol.NZ;
  S->depth = std::min(r->p.slab_depth > 0 ? r->p.slab_depth : 32, NZ);
  S->nslab = (NZ + S->depth - 1) / S->depth;
  S->plane = (long long)r->vol.NX * r->vol.NY;
  const int K = r->K, ck = recon_copy_kind(r);
  const long long sv = S->plane * S->depth;  // voxels of one slab
  long long bytes = 0;
  for (int s = 0; s < 2; ++s) {
    MTR_CK(ctx, S->x[s].alloc_pooled((size_t)sv * 4, ctx));
    MTR_CK(ctx, S->cbp[s].alloc_pooled((size_t)sv * 4, ctx));
    if (ck) MTR_CK(ctx, S->xc[s].alloc_pooled((size_t)sv * 2, ctx));
    bytes += sv * (ck ? 10 : 8);
  }
  MTR_CK(ctx, S->acc.alloc_pooled((size_t)sv * 4, ctx));
  bytes += sv * 4;
  // A MACE chunk holds K + 1 FP32 volumes (x_k, w_avg), the K states w_k
  // (FP16 in mixed precision) and K forward copies (mixed) per voxel: sized
  // to about one slot's bytes.
  const long long mace_voxel_bytes = (K + 1LL) * 4 + (ck ? 2LL * K + 2LL * K : 4LL * K);
  S->mace_planes = (int)std::max(1LL, std::min<long long>(NZ, S->depth * (ck ? 10LL : 8LL) / mace_voxel_bytes));
  const long long mv = (long long)S->mace_planes * S->plane;
  MTR_CK(ctx, S->mace.alloc_pooled((size_t)(mv * mace_voxel_bytes), ctx));
  bytes += mv * mace_voxel_bytes;
  MTR_CK(ctx, cudaStreamCreateWithFlags(&S->in, cudaStreamNonBlocking));
  MTR_CK(ctx, cudaStreamCreateWithFlags(&S->out, cudaStreamNonBlocking));
  for (int s = 0; s < 2; ++s) {
    MTR_CK(ctx, cudaEventCreateWithFlags(&S->loaded[s], cudaEventDisableTiming));
    MTR_CK(ctx, cudaEventCreateWithFlags(&S->computed[s], cudaEventDisableTiming));
    MTR_CK(ctx, cudaEventCreateWithFlags(&S->freed[s], cudaEventDisableTiming));
  }
  for (cudaEvent_t& e : S->mark) MTR_CK(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  S->device_bytes = bytes;
  r->slabs = std::move(S);
  return MTR_OK;
}

// WBP initialisation slab by slab: every axis' WBP of the slab into slot 0
// (its weight sums copied out), summed into the initial model, which becomes
// w_avg, every w_k and every x_k (and the forward copies) of that slab.
mtr_status mtr::stream_enqueue_init(mtr_recon* r) {
  mtr_context* ctx = r->ctx;
  SlabStream& S = *r->slabs;
  const cudaStream_t c = ctx->stream;
  const int K = r->K, ck = recon_copy_kind(r);
  mtr_status st = after(ctx, S, 2, c, S.out);  // copies out of an earlier run
  if (st != MTR_OK) return st;
  MTR_CK(ctx, cudaMemsetAsync(r->err.p, 0, sizeof(int), c));
  for (int k = 0; k < K; ++k)
    if ((st = recon_enqueue_widen(r, k)) != MTR_OK) return st;
  for (int j = 0; j < S.nslab; ++j) {
    const SlabRange R = slab_range(r, j, S.depth);
    const size_t nb = (size_t)R.n * 4;
    for (int k = 0; k < K; ++k) {
      st = recon_enqueue_bp_span(r, k, 0, VolSpan{R.z0, R.z1, S.x[0].as<float>(), S.cbp[0].as<float>(), S.xc[0].p},
                                 false);
      if (st != MTR_OK) return st;
      MTR_CK(ctx, cudaMemcpyAsync(bytes_at(r->ax[k].cbp, R.off, 4), S.cbp[0].p, nb, cudaMemcpyDefault, c));
      ProfScope ps(ctx, MTR_KERNEL_OTHER);
      if (k == 0) {
        MTR_CK(ctx, cudaMemcpyAsync(S.acc.p, S.x[0].p, nb, cudaMemcpyDeviceToDevice, c));
      } else {
        launch_axpy_acc(S.acc.as<float>(), S.x[0].as<float>(), R.n, c);
        MTR_CK_LAUNCH(ctx, "initial model sum (streamed)");
      }
    }
    MTR_CK(ctx, cudaMemcpyAsync(bytes_at(r->wavg, R.off, 4), S.acc.p, nb, cudaMemcpyDefault, c));
    if (!ck) {  // w_k = x_k = w_avg
      for (int k = 0; k < K; ++k) {
        MTR_CK(ctx, cudaMemcpyAsync(bytes_at(r->ax[k].w, R.off, 4), S.acc.p, nb, cudaMemcpyDefault, c));
        MTR_CK(ctx, cudaMemcpyAsync(bytes_at(r->ax[k].x, R.off, 4), S.acc.p, nb, cudaMemcpyDefault, c));
      }
    } else {  // w_k = w_avg (a zero FP16 deviation), x_k = w_avg, and the forward copies
      MTR_CK(ctx, cudaMemsetAsync(S.xc[0].p, 0, (size_t)R.n * 2, c));
      for (int k = 0; k < K; ++k) {
        MTR_CK(ctx, cudaMemcpyAsync(bytes_at(r->ax[k].w, R.off, 2), S.xc[0].p, (size_t)R.n * 2, cudaMemcpyDefault,
                                    c));
        MTR_CK(ctx, cudaMemcpyAsync(bytes_at(r->ax[k].x, R.off, 4), S.acc.p, nb, cudaMemcpyDefault, c));
      }
      launch_convert_copy(S.acc.as<float>(), S.xc[0].p, ck, R.n, c);
      MTR_CK_LAUNCH(ctx, "volume copy (streamed)");
      for (int k = 0; k < K; ++k)
        MTR_CK(ctx, cudaMemcpyAsync(bytes_at(r->ax[k].xcopy, R.off, 2), S.xc[0].p, (size_t)R.n * 2,
                                    cudaMemcpyDefault, c));
    }
  }
  const int ni = r->p.sirt_inner, no = r->p.iter_times;
  if (r->norms.p) MTR_CK(ctx, cudaMemsetAsync(r->norms.p, 0, sizeof(double) * (size_t)no * K * ni, c));
  if (r->dchange.p) MTR_CK(ctx, cudaMemsetAsync(r->dchange.p, 0, sizeof(double) * 2 * (size_t)std::max(1, no), c));
  // slot 0 and the host arrays were written on the context stream
  if ((st = after(ctx, S, 0, S.in, c)) != MTR_OK) return st;
  return after(ctx, S, 1, S.out, c);
}

mtr_status mtr::stream_join(mtr_recon* r) {
  SlabStream& S = *r->slabs;
  mtr_status st = after(r->ctx, S, 0, S.in, r->ctx->stream);
  if (st == MTR_OK) st = after(r->ctx, S, 1, S.out, r->ctx->stream);
  return st;
}

mtr_status mtr::stream_enqueue_outer(mtr_recon* r, int first, int count) {
  for (int it = first; it < first + count; ++it) {
    for (int k = 0; k < r->K; ++k) {
      for (int j = 0; j < r->p.sirt_inner; ++j) {
        mtr_status st = forward_pass(r, k);
        if (st == MTR_OK) st = recon_enqueue_residual_norm(r, k, recon_norm_slot(r, it, k, j));
        if (st == MTR_OK) st = update_pass(r, k);
        if (st != MTR_OK) return st;
      }
    }
    mtr_status st = mace_pass(r, it);
    if (st != MTR_OK) return st;
  }
  return MTR_OK;
}
