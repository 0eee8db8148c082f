// Host runtime pieces shared by the C ABI translation units: the context,
// device buffers, error plumbing and the device-resident reconstruction.
#pragma once

#include <atomic>
#include <cstdint>
#include <cstdlib>
#include <memory>
#include <string>
#include <vector>

#include "mtr_internal.h"

struct mtr_context {
  int device = 0;
  int num_sms = 152;
  int cc_major = 0, cc_minor = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  std::string last_error;
  // Per-kernel-class event timing (mtr_context_set_profiling).
  bool profiling = false;
  struct ProfRec { int kind; cudaEvent_t a, b; };
  std::vector<ProfRec> prof_pending;
  std::vector<cudaEvent_t> event_pool;
  long long prof_count[MTR_KERNEL_CLASSES] = {};
  double prof_ms[MTR_KERNEL_CLASSES] = {};
  cudaEvent_t take_event() {
    if (!event_pool.empty()) {
      cudaEvent_t e = event_pool.back();
      event_pool.pop_back();
      return e;
    }
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
    return e;
  }
  // Side streams and fork/join events for work that runs concurrently with
  // the context stream (one per tilt axis), created on first use.
  std::vector<cudaStream_t> side_streams;
  std::vector<cudaEvent_t> sync_events;
  cudaStream_t side_stream(int k) {
    while ((int)side_streams.size() <= k) {
      cudaStream_t s = nullptr;
      if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return nullptr;
      side_streams.push_back(s);
    }
    return side_streams[(size_t)k];
  }
  cudaEvent_t sync_event(int i) {
    while ((int)sync_events.size() <= i) {
      cudaEvent_t e = nullptr;
      if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return nullptr;
      sync_events.push_back(e);
    }
    return sync_events[(size_t)i];
  }
  // Stream-ordered pool for the arrays of reconstructions, created on first
  // use.  Arrays freed by mtr_recon_destroy stay reserved in the pool (up to
  // its release threshold) and the next reconstruction of similar size takes
  // them without a cudaMalloc/cudaFree round trip.  nullptr when the device
  // has no pool support (plain cudaMalloc then).
  cudaMemPool_t pool = nullptr;
  bool pool_tried = false;
  cudaMemPool_t memory_pool() {
    if (pool_tried) return pool;
    pool_tried = true;
    int supported = 0;
    if (cudaDeviceGetAttribute(&supported, cudaDevAttrMemoryPoolsSupported, device) != cudaSuccess || !supported) {
      cudaGetLastError();
      return nullptr;
    }
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    if (cudaMemPoolCreate(&pool, &props) != cudaSuccess) {
      cudaGetLastError();
      pool = nullptr;
      return nullptr;
    }
    // Reserved bytes kept across synchronisations: MTR_POOL_KEEP_BYTES, else
    // a quarter of the device memory.
    size_t total = 0, free_b = 0;
    if (cudaMemGetInfo(&free_b, &total) != cudaSuccess) { cudaGetLastError(); total = 0; }
    uint64_t keep = (uint64_t)total / 4;
    if (const char* e = std::getenv("MTR_POOL_KEEP_BYTES")) keep = std::strtoull(e, nullptr, 10);
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    return pool;
  }
};

namespace mtr {

// Brackets the launches issued in its scope with events when profiling is on
// and the stream is not being captured into a graph.
struct ProfScope {
  mtr_context* c;
  int kind;
  cudaEvent_t a = nullptr;
  ProfScope(mtr_context* ctx, int k) : c(ctx), kind(k) {
    if (!c || !c->profiling) return;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(c->stream, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return;
    a = c->take_event();
    if (a) cudaEventRecord(a, c->stream);
  }
  ~ProfScope() {
    if (!a) return;
    cudaEvent_t b = c->take_event();
    if (!b) return;
    cudaEventRecord(b, c->stream);
    c->prof_pending.push_back({kind, a, b});
  }
};

// Process-wide count of libmtr kernel launches (graph replays add their node count).
extern std::atomic<long long> g_launches;

mtr_status set_error(mtr_context* ctx, mtr_status s, const std::string& msg);
mtr_status cuda_error(mtr_context* ctx, cudaError_t e, const char* what);
mtr_status check_volume(mtr_context* ctx, const mtr_volume_size& v);
// data_required false: prj_data may be null (projections uploaded later).
mtr_status check_axis(mtr_context* ctx, const mtr_axis& a, bool data_required = true);

// Side streams forked from the context stream and joined back to it.
// fork(n) makes side streams 0..n-1 wait for the work enqueued so far on the
// context stream; use(i) points the context at side stream i (use(-1) at the
// context stream).  The destructor, on every exit path, records a join event
// on each forked side stream, makes the context stream wait for it and
// restores the context stream: an error return in the middle of a section
// never leaves a stream capture with unjoined work, and later work on the
// context stream is ordered after everything the side streams received.
struct ForkJoin {
  mtr_context* ctx;
  cudaStream_t main;
  int forked = 0;
  explicit ForkJoin(mtr_context* c) : ctx(c), main(c->stream) {}
  ForkJoin(const ForkJoin&) = delete;
  ForkJoin& operator=(const ForkJoin&) = delete;
  mtr_status fork(int n) {
    cudaEvent_t f = ctx->sync_event(0);
    if (!f) return set_error(ctx, MTR_ERR_CUDA, "event creation");
    cudaError_t e = cudaEventRecord(f, main);
    if (e != cudaSuccess) return cuda_error(ctx, e, "cudaEventRecord(fork)");
    for (int i = forked; i < n; ++i) {
      cudaStream_t s = ctx->side_stream(i);
      if (!s || !ctx->sync_event(1 + i)) return set_error(ctx, MTR_ERR_CUDA, "side stream creation");
      e = cudaStreamWaitEvent(s, f, 0);
      if (e != cudaSuccess) return cuda_error(ctx, e, "cudaStreamWaitEvent(fork)");
      forked = i + 1;
    }
    return MTR_OK;
  }
  void use(int i) { ctx->stream = i < 0 ? main : ctx->side_streams[(size_t)i]; }
  ~ForkJoin() {
    ctx->stream = main;
    for (int i = 0; i < forked; ++i) {
      cudaEvent_t join = ctx->sync_event(1 + i);
      cudaEventRecord(join, ctx->side_streams[(size_t)i]);
      cudaStreamWaitEvent(main, join, 0);
    }
  }
};

// Makes a device current for a scope and restores the previous one.
struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DeviceGuard() {
    int cur = -1;
    if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
  }
};

// Owning allocation addressed by the device: device memory, or (alloc_mapped)
// pinned host memory mapped into the device address space, which kernels
// load and store directly (coherently over NVLink-C2C on Grace-based GPUs).
struct DevBuf {
  void* p = nullptr;     // device-side address
  void* host = nullptr;  // host allocation when mapped
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept : p(o.p), host(o.host), bytes(o.bytes), pooled(o.pooled), free_stream(o.free_stream) {
    o.p = o.host = nullptr;
    o.bytes = 0;
    o.pooled = false;
  }
  DevBuf& operator=(DevBuf&& o) noexcept {
    if (this != &o) {
      reset();
      p = o.p; host = o.host; bytes = o.bytes; pooled = o.pooled; free_stream = o.free_stream;
      o.p = o.host = nullptr;
      o.bytes = 0;
      o.pooled = false;
    }
    return *this;
  }
  ~DevBuf() { reset(); }
  cudaError_t alloc(size_t n) {
    reset();
    if (n == 0) return cudaSuccess;
    cudaError_t e = cudaMalloc(&p, n);
    if (e == cudaSuccess) bytes = n; else p = nullptr;
    return e;
  }
  cudaError_t alloc_mapped(size_t n) {
    reset();
    if (n == 0) return cudaSuccess;
    cudaError_t e = cudaHostAlloc(&host, n, cudaHostAllocMapped | cudaHostAllocPortable);
    if (e != cudaSuccess) { host = nullptr; return e; }
    e = cudaHostGetDevicePointer(&p, host, 0);
    if (e != cudaSuccess) { cudaFreeHost(host); host = p = nullptr; return e; }
    bytes = n;
    return cudaSuccess;
  }
  // device memory, or mapped host memory when `mapped`
  cudaError_t alloc_where(size_t n, bool mapped) { return mapped ? alloc_mapped(n) : alloc(n); }
  // Device memory from the context's pool, ordered on the context stream
  // (usable by work enqueued there after this call, and by any stream once
  // that stream has been synchronised).  Returned to the pool on the
  // context's own stream; the owner synchronises the streams that used the
  // array before releasing it.  Falls back to cudaMalloc without a pool.
  cudaError_t alloc_pooled(size_t n, mtr_context* ctx) {
    reset();
    if (n == 0) return cudaSuccess;
    cudaMemPool_t pool = ctx->memory_pool();
    if (!pool) return alloc(n);
    cudaError_t e = cudaMallocFromPoolAsync(&p, n, pool, ctx->stream);
    if (e != cudaSuccess) { p = nullptr; return e; }
    bytes = n;
    pooled = true;
    free_stream = ctx->own_stream;
    if (((uintptr_t)p & 255) != 0) {  // TMA and vector paths want aligned bases
      reset();
      return alloc(n);
    }
    return cudaSuccess;
  }
  // device memory (pooled when `ctx` is given), or mapped host memory
  cudaError_t alloc_where(size_t n, bool mapped, mtr_context* ctx) {
    return mapped ? alloc_mapped(n) : alloc_pooled(n, ctx);
  }
  void reset() {
    if (host) cudaFreeHost(host);
    else if (p && pooled) cudaFreeAsync(p, free_stream);
    else if (p) cudaFree(p);
    p = host = nullptr;
    bytes = 0;
    pooled = false;
  }
  bool pooled = false;
  cudaStream_t free_stream = nullptr;
  template <typename T> T* as() const { return static_cast<T*>(p); }
};

#define MTR_CK(ctx, call)                                       \
  do {                                                          \
    cudaError_t _e = (call);                                    \
    if (_e != cudaSuccess) return ::mtr::cuda_error((ctx), _e, #call); \
  } while (0)

#define MTR_CK_LAUNCH(ctx, what)                                \
  do {                                                          \
    ::mtr::g_launches.fetch_add(1, std::memory_order_relaxed);  \
    cudaError_t _e = cudaGetLastError();                        \
    if (_e != cudaSuccess) return ::mtr::cuda_error((ctx), _e, what); \
  } while (0)

// Per-axis device state of a reconstruction.
struct AxisState {
  int PX = 0, PY = 0, A = 0;
  int pitch = 0;          // row pitch of projection-space arrays (elements)
  int pitch2 = 0;         // row pitch of the residual in pair form (pairs, pair_pitch(PX))
  long long np = 0;       // A*PY*pitch
  std::vector<double> hxc, hyc;  // host copies of the maps (kernel planning)
  BpPlan plan;            // TMA back-projection window plan over r (FP32)
  BpPlan plan_b;          // WBP plan (FP32 windows, depth 8)
  CUtensorMap map_b{}, map_r{};  // WBP map over b (FP32) or over r holding b widened (mixed); map over r
  bool tma = false, tma_b = false;
  FwdPlan fplan;          // windowed forward splat plan
  CUtensorMap map_s{}, map_cf{};  // tensor maps over s and cf (valid when ftma)
  bool ftma = false;
  DevBuf xc, yc;          // [A*4] doubles
  DevBuf b;               // projections: float (FP32) or half (mixed)
  DevBuf s;               // forward accumulator, float
  DevBuf cf;              // forward row sums A 1, float
  DevBuf r;               // residual: FP32 [A][PY][pitch], or pairs [A][PY][pitch2] when the
                          // windowed back-projection reads it (tma)
  DevBuf cbp;             // back-projection weight sums A^T 1 (volume), float
  DevBuf w;               // MACE state w_k (volume), float
  DevBuf x;               // SIRT iterate z_k -> v_k (volume), float
  DevBuf xcopy;           // bf16/f16 copy of x read by the forward pass (mixed)
  AxisDev dev() const { return AxisDev{PX, PY, A, xc.as<double>(), yc.as<double>(), pitch}; }
};

// Tensor map over an axis' residual in pair form: FP32 elements, rows of
// 2 * pitch2 floats, boxes of 2 * WX floats (WX pairs) by WY rows; planar
// pairs as 2 * PY rows of pitch2 floats (each detector row's values, then its
// differences), boxes of WX floats by 2 * WY rows; FP16 pairs as 32-bit
// elements, rows of pitch2, boxes of WX by WY.
inline bool encode_pair_map(CUtensorMap* m, const AxisState& a, const BpPlan& p) {
  if (!p.pairs) return false;
  if (p.half) return encode_tensor_map_3d(m, a.r.p, false, a.pitch2, a.pitch2, a.PY, a.A, p.WX, p.WY);
  if (p.planar) return encode_tensor_map_3d(m, a.r.p, false, a.pitch2, a.pitch2, 2 * a.PY, a.A, p.WX, 2 * p.WY);
  return encode_tensor_map_3d(m, a.r.p, false, 2 * a.pitch2, 2 * a.pitch2, a.PY, a.A, 2 * p.WX, p.WY);
}
// Tensor map over an axis' residual in the form its SIRT update reads: pairs,
// or FP32 rows of `pitch` elements.
inline bool encode_residual_map(CUtensorMap* m, const AxisState& a, const BpPlan& p) {
  return p.pairs ? encode_pair_map(m, a, p)
                 : encode_tensor_map_3d(m, a.r.p, false, a.PX, a.pitch, a.PY, a.A, p.WX, p.WY);
}

// Disable the TMA kernels (MTR_DISABLE_TMA=1 in the environment) to run the
// plain global-memory kernels instead; used to cross-check the two paths.
bool tma_disabled();

// Autotuner (tune.cu): picks the brick depths of the SIRT back-projection and
// the forward splat for one axis, timing candidates on the axis' buffers
// before they hold data, and encodes the tensor maps.
bool autotune_enabled();
// Candidates run over the frame v on device scratch: scratch_vol / scratch_cbp
// (FP32) and, in mixed precision, scratch_copy (the BF16 / FP16 copy the
// forward splat reads); none of them holds data yet.
bool tune_axis(mtr_context* ctx, AxisState& a, const VolDev& v, int precision, float* scratch_vol,
               float* scratch_cbp, void* scratch_copy, int* err);

// The Z planes [z0, z1) one launch works on and the arrays that hold exactly
// those planes: an axis' whole volume arrays, or one slot of a streamed
// reconstruction's device working set.
struct VolSpan {
  int z0, z1;
  float* x;     // SIRT iterate (the WBP writes it)
  float* cbp;   // back-projection weight sums
  void* xcopy;  // BF16 / FP16 copy of x read by the forward splat (mixed), or null
};

// Device working set of a reconstruction whose volume-sized arrays live in
// host memory (MTR_FLAG_STREAM_SLABS, stream.cu).  The volume is cut into
// Z-slabs of `depth` planes; two slab slots rotate so that the copy of one
// slab overlaps the kernels of the other.  `in` carries host-to-device
// copies, `out` device-to-host copies, the context stream the kernels.
struct SlabStream {
  int depth = 0;           // Z planes per slab
  int nslab = 0;
  long long plane = 0;     // voxels per Z plane
  int mace_planes = 0;     // Z planes per MACE chunk
  DevBuf x[2], cbp[2], xc[2];  // slot arrays (x/cbp FP32, xc the forward copy in mixed precision)
  DevBuf acc;              // one slab of the WBP sum over axes (initialisation)
  DevBuf mace;             // one MACE chunk: w_k, x_k (FP32), w_avg, then the K forward copies
  cudaStream_t in = nullptr, out = nullptr;
  cudaEvent_t loaded[2] = {}, computed[2] = {}, freed[2] = {}, mark[3] = {};
  long long device_bytes = 0;
  ~SlabStream();
};

}  // namespace mtr

struct mtr_recon;
namespace mtr {
// WBP sum into w_avg, w_k = z_k = w_avg, records reset (recon.cu).
mtr_status recon_enqueue_init(mtr_recon* r);
// WBP of axis k alone: x_k = s/c and the weight sums cbp_k = c.
mtr_status recon_enqueue_wbp(mtr_recon* r, int k);
// One SIRT phase of axis k of a reconstruction, with its own kernels.
mtr_status recon_enqueue_forward(mtr_recon* r, int k);
mtr_status recon_enqueue_residual(mtr_recon* r, int k);
mtr_status recon_enqueue_sirt_bp(mtr_recon* r, int k);
// MACE step `it` (0-based outer iteration) over all axes of a reconstruction.
mtr_status recon_enqueue_mace(mtr_recon* r, int it);

// Descriptor tables of the persistent SIRT kernels over a set of
// reconstructions of one precision (batch.cu).  One SIRT iteration of every
// axis of every member = one forward, one residual and one back-projection
// launch over the small axes, plus the own launch chains of the other axes
// (large enough to fill the GPU alone, tiled as patches, or with windows that
// fit no TMA box), which run concurrently on side streams.  Device buffers
// only grow, so rebuilding for a changed set reallocates rarely.
struct SirtTables {
  int copy_kind = 0;
  DevBuf maps, bp_descs, fwd_descs, res_descs, bp_first, fwd_first, res_first;
  int n_bp_desc = 0, n_fwd_desc = 0, n_res_desc = 0;
  long long n_bp = 0, n_fwd = 0, n_res = 0;
  size_t bp_smem = 0, fwd_smem = 0;
  int bp_grid = 0, fwd_grid = 0, ew_grid = 0;
  std::vector<std::pair<mtr_recon*, int>> own;  // (reconstruction, axis) with their own launches
};
mtr_status build_sirt_tables(mtr_context* ctx, const std::vector<mtr_recon*>& recs, int precision, SirtTables& t);
mtr_status enqueue_sirt_iteration(mtr_context* ctx, const SirtTables& t, int* err);

}  // namespace mtr

struct mtr_recon {
  mtr_context* ctx = nullptr;
  mtr_volume_size vs{};
  mtr::VolDev vol{};
  mtr_params p{};
  int K = 0;
  long long nv = 0;
  std::vector<mtr::AxisState> ax;
  mtr::DevBuf wavg;       // consensus volume, float
  mtr::DevBuf norms;      // n_outer*K*n_inner doubles
  mtr::DevBuf dchange;    // n_outer doubles
  mtr::DevBuf err;        // device error flag written by bounded waits (int)
  long long bytes = 0;
  bool geometry_ready = false;  // cf and cbp computed
  bool record_changes = false;  // MACE steps accumulate the FP64 convergence record
  int outer_done = 0;           // MACE outer iterations the state has been through
  cudaGraphExec_t graph = nullptr;
  long long graph_nodes = 0;
  // Streamed slabs (MTR_FLAG_STREAM_SLABS): the volume-sized arrays above are
  // in pinned, mapped host memory and this is the device working set.
  std::unique_ptr<mtr::SlabStream> slabs;
  ~mtr_recon();
};

namespace mtr {
// Pieces of a reconstruction's schedule over one span of axis k's volume (recon.cu).
mtr_status recon_enqueue_forward_span(mtr_recon* r, int k, const VolSpan& sp);
// mode 0 WBP, 1 SIRT update; widen: widen FP16 projections for a windowed WBP first.
mtr_status recon_enqueue_bp_span(mtr_recon* r, int k, int mode, const VolSpan& sp, bool widen);
mtr_status recon_enqueue_widen(mtr_recon* r, int k);
// Residual of axis k; norm: FP64 sum of r^2 (null: not recorded).
mtr_status recon_enqueue_residual_norm(mtr_recon* r, int k, double* norm);
// Where the squared residual norm of (outer it, axis k, inner j) is recorded, or null.
double* recon_norm_slot(mtr_recon* r, int it, int k, int j);
// The MACE step's FP64 convergence sums of outer iteration it, or null.
double* recon_change_slot(mtr_recon* r, int it);
int recon_copy_kind(const mtr_recon* r);
// Streamed slabs (stream.cu): the device working set, the WBP initialisation
// and the MACE outer iterations with slabs streamed through it.
mtr_status stream_setup(mtr_recon* r);
mtr_status stream_enqueue_init(mtr_recon* r);
mtr_status stream_enqueue_outer(mtr_recon* r, int first, int count);
// The copy streams wait for the work enqueued so far on the context stream
// (after the context stream wrote the host-side volume arrays itself).
mtr_status stream_join(mtr_recon* r);
}  // namespace mtr
