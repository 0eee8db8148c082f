/*
 * mtr.h - C ABI of libmtr, a single-GPU (GB300, sm_103a) multi-axis
 * tomographic reconstruction library: weighted back-projection init, SIRT
 * with bilinear forward/back projectors, and MACE consensus over tilt axes.
 *
 * Plain C types only: pointers, sizes, status codes.  Every entry point
 * returns an mtr_status; nothing here prints or exits.  A context is bound
 * to one CUDA device and one stream and is not thread-safe (use one context
 * per host thread).
 *
 * Each entry point names the interface of the reference program
 * (Autumn1998/Multi-tilt-Reconstuction) that it replaces, as file:line.
 */
#ifndef MTR_H_
#define MTR_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MTR_ABI_VERSION 2
/* Maximum tilt axes per reconstruction (MAX_TILT, ReadAndInitialOptions.h:17). */
#define MTR_MAX_AXES 16
/* Default SIRT iterations per MACE iteration (hard-coded, FunctionOnGPU.cu:212). */
#define MTR_DEFAULT_SIRT_INNER 10

typedef enum mtr_status {
  MTR_OK = 0,
  MTR_ERR_INVALID_ARGUMENT = 1,
  MTR_ERR_CUDA = 2,
  MTR_ERR_OUT_OF_MEMORY = 3,
  MTR_ERR_IO = 4,
  MTR_ERR_FORMAT = 5,
  MTR_ERR_UNSUPPORTED = 6,
  MTR_ERR_NO_DEVICE = 7,
  MTR_ERR_TIMEOUT = 8,
  MTR_ERR_NOT_READY = 9,
  MTR_ERR_CAPACITY = 10
} mtr_status;

/* Storage precision.  FP32: everything float.  MIXED_*: projections stored
 * FP16, the volume copy read by the forward projector stored BF16 (or FP16),
 * the per-axis MACE states w_k stored as FP16 deviations from the FP32
 * consensus (w_k - w_avg, rounded once per outer iteration), and, where the
 * tuner finds it faster, the residual read by the back-projection stored as
 * FP16 (value, next - value) pairs computed in FP32; interpolation and
 * accumulation in FP32; residual norms and the MACE consensus sum in FP64;
 * the SIRT iterate (updated every iteration), the weight sums and the
 * consensus stay FP32.  Mixed storage takes less device memory than FP32;
 * values (and residual differences) must lie within the FP16 range.
 * MIXED_FP16 is the more accurate of the two (its copy keeps 11 bits). */
typedef enum mtr_precision {
  MTR_PREC_FP32 = 0,
  MTR_PREC_MIXED_BF16 = 1,
  MTR_PREC_MIXED_FP16 = 2
} mtr_precision;

/* Where a buffer passed to an entry point lives. */
typedef enum mtr_mem_kind { MTR_MEM_HOST = 0, MTR_MEM_DEVICE = 1 } mtr_mem_kind;

/* Volume frame, absolute voxel coordinates, end-exclusive, X = Xend-Xstart.
 * Same fields and order as VolumeSize (MrcFileIOBaseFunction.h:57-70). */
typedef struct mtr_volume_size {
  int Xstart, Xend, Ystart, Yend, Zstart, Zend;
  int X, Y, Z;
} mtr_volume_size;

/* Detector size and angle count.  Same fields as ProjectionSize
 * (MrcFileIOBaseFunction.h:73-78). */
typedef struct mtr_projection_size {
  int X, Y, AngN;
} mtr_projection_size;

/* One tilt axis: projections [AngN][Y][X] (x fastest) and per-angle affine
 * maps, 4 doubles per angle [const, X, Y, Z], detector coordinate
 * = c0 + c1*X + c2*Y + c3*Z - 1 (FunctionOnGPU.cu:12-25). */
typedef struct mtr_axis {
  mtr_projection_size prj;
  const double* x_coef; /* 4*AngN, host memory */
  const double* y_coef; /* 4*AngN, host memory */
  const float* prj_data; /* AngN*Y*X floats; host or device (see mem_kind) */
} mtr_axis;

typedef struct mtr_params {
  int iter_times;   /* -n: MACE outer iterations (ReadAndInitialOptions.h:38, default 5) */
  int sirt_inner;   /* SIRT iterations per MACE iteration (default 10) */
  float sirt_step;  /* -s: SIRT relaxation (default 0.5) */
  float mace_step;  /* -m: MACE Mann step rho (default 0.7) */
  int precision;    /* mtr_precision */
  int flags;        /* MTR_FLAG_* */
  int slab_depth;   /* Z planes per streamed slab (MTR_FLAG_STREAM_SLABS); 0 = automatic (32) */
} mtr_params;

/* Record the squared residual norm (FP64) of every SIRT iteration. */
#define MTR_FLAG_RECORD_NORMS 1
/* Capture a whole run (WBP init and every MACE iteration) in a CUDA graph on
 * the first mtr_recon_run and replay it on the next ones.  Ignored while
 * per-kernel profiling is on (mtr_context_set_profiling). */
#define MTR_FLAG_GRAPH 2
/* Keep the volume-sized arrays (iterates, MACE states, weight sums, forward
 * copies, consensus: 12-14 B per voxel and axis) in pinned host memory mapped
 * into the device address space, which the kernels load and store directly
 * (coherent NVLink-C2C on Grace-based GPUs), and only the projection arrays
 * in device memory: volumes larger than HBM.  No counterpart in the
 * reference, which splits Z over MPI ranks (MpiBigData.cpp). */
#define MTR_FLAG_HOST_VOLUMES 4
/* Keep the FP64 convergence record of the MACE loop (mtr_recon_changes): the
 * relative change of the consensus per outer iteration, two FP64 sums per
 * voxel in the MACE step.  mtr_recon_run_until turns it on by itself. */
#define MTR_FLAG_RECORD_CHANGES 8
/* Single-GPU streaming slab loop: the volume-sized arrays (iterates, MACE
 * states, weight sums, forward copies, consensus) live in pinned host memory,
 * and the device holds the projection-space arrays plus a working set of two
 * Z-slabs of slab_depth planes.  Each SIRT iteration of an axis splats the
 * slabs one after another into the axis' ray sums, forms the residual once
 * after the last slab, then back-projects the slabs one after another, each
 * slab's copies overlapping the other slab's kernels.  Replaces the
 * reference's Z-slab decomposition over MPI ranks (divideSlice,
 * MultiAxis.cpp:13-31), whose partial ray sums are reduced in projection
 * space every SIRT iteration (FunctionOnGPU.cu:218-238).  The axes run one
 * after another; MTR_FLAG_GRAPH is ignored. */
#define MTR_FLAG_STREAM_SLABS 16

/* Fill p with the reference defaults (Options(), ReadAndInitialOptions.h:33-42). */
void mtr_params_default(mtr_params* p);

typedef struct mtr_context mtr_context;

/* Library / error information. */
int mtr_abi_version(void);
const char* mtr_status_string(mtr_status s);
const char* mtr_context_last_error(const mtr_context* ctx);

/* Context: device, stream, scratch.  device < 0 selects the current device.
 * Replaces the per-call cudaSetDevice(rank%4)/cudaStreamCreate of the
 * reference entry points (FunctionOnGPU.cu:140,150-151,184,193-194). */
mtr_status mtr_context_create(int device, mtr_context** out);
mtr_status mtr_context_destroy(mtr_context* ctx);
/* Use an external cudaStream_t (NULL restores the context's own stream). */
mtr_status mtr_context_set_stream(mtr_context* ctx, void* cuda_stream);
mtr_status mtr_context_synchronize(mtr_context* ctx);
/* Reconstruction arrays come from a stream-ordered pool owned by the
 * context; after mtr_recon_destroy they stay reserved (up to a quarter of
 * the device memory, or MTR_POOL_KEEP_BYTES) so that the next reconstruction
 * of similar size allocates nothing.  Returns all reserved, unused pool
 * memory to the device. */
mtr_status mtr_context_trim(mtr_context* ctx);
/* Number of libmtr kernel launches issued by this process so far (graph
 * replays count every kernel node). */
mtr_status mtr_context_launch_count(const mtr_context* ctx, long long* out);
/* Of those, the launches of the TMA-windowed projector kernels: the
 * back-projection gather and the forward splat that stage detector windows
 * in shared memory (counted when issued; graph replays are not counted). */
mtr_status mtr_context_windowed_launch_count(const mtr_context* ctx, long long* out);
/* Failure-path hook, process-wide: the number of polls after which the
 * pipeline waits of the windowed back-projection (the producer waiting for a
 * free window stage, the consumers for a loaded window) give up, flag the
 * launch and return; the kernel still waits for its own copies in flight
 * before it exits.  A flagged run makes mtr_recon_check (and the host-buffer
 * downloads) report MTR_ERR_TIMEOUT; the context stays usable.  Negative
 * restores the default (2^24 polls); 0 makes every such wait give up at once.
 * Read when a launch is issued (a captured graph keeps the value it was
 * captured with).  The reference has no bounded waits (it only prints
 * kernel errors, FunctionOnGPU.cu:3-10). */
mtr_status mtr_set_wait_limit(long long polls);

/* Kernel classes for per-kernel timing. */
#define MTR_KERNEL_WBP 0
#define MTR_KERNEL_FORWARD 1
#define MTR_KERNEL_RESIDUAL 2
#define MTR_KERNEL_BACKPROJECT 3
#define MTR_KERNEL_MACE 4
#define MTR_KERNEL_OTHER 5
#define MTR_KERNEL_CLASSES 6
/* When enabled, every libmtr launch issued outside graph capture is
 * bracketed by CUDA events on the context stream. */
mtr_status mtr_context_set_profiling(mtr_context* ctx, int enable);
/* Synchronises the stream and returns the accumulated launch count and
 * device time (ms) of one kernel class since the last reset. */
mtr_status mtr_context_profile(mtr_context* ctx, int kernel_class, long long* launches, double* total_ms);
mtr_status mtr_context_profile_reset(mtr_context* ctx);

/* ---- Entry points replacing FunctionOnGPU.cuh:41-44 -------------------- */

/* Replaces ComputeInitialModel (FunctionOnGPU.cuh:41, FunctionOnGPU.cu:138-179).
 * Weighted back-projection of one axis over the Z-slab [slice_start,
 * slice_end) of vol: slab_out[(x)+(y)*X+(z-slice_start)*X*Y] = s/c where the
 * in-detector bilinear weight sum c != 0, else 0 (the reference adds into a
 * fresh device buffer; it is treated as zero).  slab_out is host memory. */
mtr_status mtr_wbp(mtr_context* ctx, const mtr_axis* axis, mtr_volume_size vol, int slice_start,
                   int slice_end, float* slab_out);

/* Replaces runSIRTOnGPU (FunctionOnGPU.cuh:42, FunctionOnGPU.cu:182-266) for
 * a caller that holds the whole Z range of its axis (no MPI communicator):
 * n_inner SIRT iterations x <- x + sirt_step * C A^T (b - R A x) on the
 * host slab, in place.  The reference hard-codes n_inner = 10. */
mtr_status mtr_sirt(mtr_context* ctx, const mtr_axis* axis, mtr_volume_size vol, int slice_start,
                    int slice_end, int n_inner, float sirt_step, float* slab_inout);

/* No counterpart in the reference.  The computation of mtr_sirt for callers
 * that cannot allocate device memory where they call it (cudaMalloc and
 * cudaFree synchronise the device and can fail, which a pipeline stage that
 * must not stall, or a program whose device memory belongs to another
 * allocator, cannot accept).  Inputs and outputs are device pointers owned by
 * the caller: x_coef_dev / y_coef_dev (4*AngN doubles each), prj_dev
 * (AngN*Y*X floats, x fastest) and slab_dev (X*Y*(slice_end-slice_start)
 * floats, updated in place), enqueued on the context stream.  The working
 * arrays live in one fixed device array of MTR_NOALLOC_SCRATCH_FLOATS floats
 * (32 MiB) compiled into the library: 3*AngN*Y*X + X*Y*(slice_end-slice_start)
 * must not exceed it, else MTR_ERR_CAPACITY.  The CUDA runtime loads a
 * library's device code lazily (the default since CUDA 12.2), so the array is
 * placed on a device by the first call there, which looks up its device
 * address; from then on the device holds it until the process exits.  That
 * first call can therefore still allocate (and fail when the device is out of
 * memory): make it at start-up, outside the stage that must not allocate, and
 * before any stream capture (a call with n_inner = 0 does only the set-up and
 * the geometry sums), or run with CUDA_MODULE_LOADING=EAGER.  All calls share
 * that array: calls that overlap on the GPU race, so issue them in order on
 * one stream. */
#define MTR_NOALLOC_SCRATCH_FLOATS (8 * 1024 * 1024)
mtr_status mtr_sirt_noalloc(mtr_context* ctx, mtr_projection_size prj, const double* x_coef_dev,
                            const double* y_coef_dev, const float* prj_dev, mtr_volume_size vol, int slice_start,
                            int slice_end, int n_inner, float sirt_step, float* slab_dev);

/* Replaces initialZdata (FunctionOnGPU.cuh:43, FunctionOnGPU.cu:291-313):
 * z = 2*w_avg - w over the whole volume (host buffers). */
mtr_status mtr_initial_z(mtr_context* ctx, mtr_volume_size vol, const float* w, const float* w_avg,
                         float* z);

/* Replaces runMaceOnGPU (FunctionOnGPU.cuh:44, FunctionOnGPU.cu:336-362) and
 * runMaceOnCPU (MultiAxis.cpp:33-38): w = step*(2v - z) + (1-step)*w. */
mtr_status mtr_update_w(mtr_context* ctx, mtr_volume_size vol, const float* v, const float* z, float* w,
                        float step);

/* Replaces the whole of MultiAxis.cpp:101-230 after option and file parsing:
 * per-axis WBP summed into the initial model (MultiAxis.cpp:172-200), then
 * iter_times MACE iterations of sirt_inner SIRT iterations per axis with the
 * consensus mean (MultiAxis.cpp:40-71), on one GPU.  out_volume receives
 * w_avg (X*Y*Z floats, x fastest), host memory. */
mtr_status mtr_reconstruct(mtr_context* ctx, int n_axes, const mtr_axis* axes, mtr_volume_size vol,
                           const mtr_params* params, float* out_volume);

/* The same reconstruction with every quantity in FP64 on the GPU (affine
 * map per voxel and angle, weights, sums, residual, MACE state), used as the
 * error reference for the FP32 and mixed-precision paths.  No reference
 * counterpart: the reference computes in FP64/float as the FP32 path does.
 * out_volume: X*Y*Z doubles, host or device memory per mem_kind; axes'
 * prj_data likewise. */
mtr_status mtr_reconstruct_fp64(mtr_context* ctx, int n_axes, const mtr_axis* axes, mtr_volume_size vol,
                                const mtr_params* params, double* out_volume, int mem_kind);

/* ---- Device-resident reconstruction object ------------------------------ */
/* The same computation as mtr_reconstruct, split so that uploads, the
 * on-device run and the download can be issued (and timed) separately. */
typedef struct mtr_recon mtr_recon;

/* axes[i].prj_data is host memory (mem_kind MTR_MEM_HOST) or device memory
 * (MTR_MEM_DEVICE, float, copied device-to-device).  It may be NULL: that
 * axis' projections are zero until mtr_recon_upload or mtr_recon_upload_half
 * supplies them. */
mtr_status mtr_recon_create(mtr_context* ctx, int n_axes, const mtr_axis* axes, mtr_volume_size vol,
                            const mtr_params* params, int mem_kind, mtr_recon** out);
/* Re-upload projection data for axis i (same shape). */
mtr_status mtr_recon_upload(mtr_recon* r, int axis, const float* prj_data, int mem_kind);
/* The same from IEEE FP16 projections (AngN*Y*X halves, host or device).  The
 * mixed-precision paths store projections in FP16 and take them as they are;
 * the FP32 path widens them on the device.  With mtr_mrc_read_stack_device_half
 * a stack goes from the file to the reconstruction in half width. */
mtr_status mtr_recon_upload_half(mtr_recon* r, int axis, const void* prj_f16, int mem_kind);
/* WBP init + MACE loop on the device (asynchronous on the context stream). */
mtr_status mtr_recon_run(mtr_recon* r);
/* The same run in pieces, and checkpoint/resume of the MACE state between
 * outer iterations.  No counterpart in the reference (its checkpoint code is
 * commented out, MultiAxis.cpp:208-214).
 *   mtr_recon_init      WBP init (asynchronous);
 *   mtr_recon_run_outer MACE outer iterations [first, first + count)
 *                       (asynchronous);
 *   mtr_recon_save      synchronises and writes w_avg, every w_k and the
 *                       number of outer iterations done;
 *   mtr_recon_load      recomputes the geometry sums (WBP init), then
 *                       restores the saved state and z_k = 2 w_avg - w_k;
 *                       *outer_done tells where to continue.  A file of
 *                       another volume or axis count is
 *                       MTR_ERR_INVALID_ARGUMENT, a damaged one MTR_ERR_FORMAT.
 * init + run_outer(0, n) is mtr_recon_run; a run resumed from a checkpoint
 * after outer iteration i equals the uninterrupted run up to the order of
 * floating-point additions in the forward splat. */
mtr_status mtr_recon_init(mtr_recon* r);
mtr_status mtr_recon_run_outer(mtr_recon* r, int first, int count);
mtr_status mtr_recon_save(mtr_recon* r, const char* path);
mtr_status mtr_recon_load(mtr_recon* r, const char* path, int* outer_done);
/* Copy w_avg out (host or device destination); synchronises for host. */
mtr_status mtr_recon_download(mtr_recon* r, float* out, int mem_kind);
/* Synchronises and reports MTR_ERR_TIMEOUT if a kernel of the last run gave
 * up on a bounded wait (the host-buffer download performs this check). */
mtr_status mtr_recon_check(mtr_recon* r);
/* Copy the K per-axis MACE states w_k (K*X*Y*Z floats). */
mtr_status mtr_recon_download_axes(mtr_recon* r, float* out, int mem_kind);
/* Squared residual norms, n_outer*K*n_inner doubles (MTR_FLAG_RECORD_NORMS). */
mtr_status mtr_recon_norms(mtr_recon* r, double* out, long long n);
/* FP64 convergence record of the MACE loop, computed on the GPU by the MACE
 * step when MTR_FLAG_RECORD_CHANGES is set (else MTR_ERR_INVALID_ARGUMENT): out[it] = ||w_avg(it) - w_avg(it-1)|| / ||w_avg(it)||, the relative
 * L2 change of the consensus in outer iteration it (w_avg(-1) = the WBP
 * init), for the first min(n, n_outer) iterations (0 for iterations not run).
 * The reference has no convergence test (fixed iteration counts,
 * MultiAxis.cpp:45). */
mtr_status mtr_recon_changes(mtr_recon* r, double* out, int n);
/* Outer iterations from `first` until the relative change of the last one
 * drops below tol or n_outer iterations are done; synchronises after each
 * outer iteration.  *outer_done = outer iterations done. */
mtr_status mtr_recon_run_until(mtr_recon* r, int first, double tol, int* outer_done);
/* Device bytes held by the object. */
mtr_status mtr_recon_footprint(const mtr_recon* r, long long* bytes);
/* JSON description of the kernels and tile shapes chosen per axis (TMA
 * windows, brick depths picked by the autotuner); NUL-terminated, truncated
 * to cap bytes. */
mtr_status mtr_recon_describe(const mtr_recon* r, char* buf, int cap);
mtr_status mtr_recon_destroy(mtr_recon* r);
/* Device bytes an object with these shapes would hold (admission control). */
mtr_status mtr_estimate_footprint(int n_axes, const mtr_projection_size* prjs, mtr_volume_size vol,
                                  int precision, long long* bytes);

/* ---- Batched reconstruction of many tilt series ------------------------- */
/* No counterpart in the reference (it reconstructs one series per MPI job).
 * Every instance gets its own device-resident reconstruction; the SIRT
 * phases of all instances run as one persistent launch per phase over a
 * cost-ordered work list of (instance, axis, brick) items, and the whole
 * schedule is captured once into a CUDA graph when params->flags has
 * MTR_FLAG_GRAPH.  All instances share params (iterations, steps, precision);
 * residual norms are not recorded in batch mode. */
typedef struct mtr_instance {
  int n_axes;
  const mtr_axis* axes;
  mtr_volume_size vol;
} mtr_instance;
typedef struct mtr_batch mtr_batch;
mtr_status mtr_batch_create(mtr_context* ctx, int n, const mtr_instance* instances, const mtr_params* params,
                            int mem_kind, mtr_batch** out);
/* WBP init + MACE loop of every instance (asynchronous on the context stream). */
mtr_status mtr_batch_run(mtr_batch* b);
/* Consensus volume of instance i (host: synchronises and checks the error flag). */
mtr_status mtr_batch_download(mtr_batch* b, int i, float* out, int mem_kind);
/* Voxel-updates per run, device bytes held, and work items per phase
 * (forward, residual, back-projection, MACE, axes on fallback kernels). */
mtr_status mtr_batch_info(const mtr_batch* b, long long* voxel_updates_per_run, long long* device_bytes,
                          long long* work_items5);
mtr_status mtr_batch_destroy(mtr_batch* b);

/* ---- Serving: continuous batching with admission by device footprint -----
 * No counterpart in the reference (MultiAxis.cpp runs one reconstruction per
 * process); this is the serving entry the batch layer feeds.
 *
 * Requests are queued by mtr_server_submit and admitted in arrival order
 * while the sum of admitted footprints (mtr_estimate_footprint) stays within
 * the server's byte budget.  Each mtr_server_step:
 *   1. waits for the previous step's GPU work,
 *   2. retires requests whose last MACE step has run: copies the consensus
 *      volume to the request's `out` buffer, frees its device memory and
 *      reports its id,
 *   3. admits queued requests that fit (device buffers, projection upload,
 *      tile tuning, WBP init),
 *   4. enqueues one SIRT iteration of every admitted request as one
 *      persistent launch per phase (forward, residual, back-projection),
 *      then the MACE step of each request that finished an outer iteration.
 * A request's `axes[].data` and `out` must stay valid until its id is
 * reported.  All requests of a server share one precision. */
typedef struct mtr_request {
  int n_axes;
  const mtr_axis* axes;   /* host projections */
  mtr_volume_size vol;
  int iter_times;         /* MACE outer iterations */
  int sirt_inner;         /* SIRT iterations per outer iteration */
  float sirt_step;
  float mace_step;
  float* out;             /* host, X*Y*Z floats: the consensus volume */
} mtr_request;
typedef struct mtr_server_stats {
  long long submitted, completed;
  long long queued, active;        /* now */
  long long bytes_in_use, peak_bytes, budget_bytes;
  long long steps;                 /* mtr_server_step calls that enqueued work */
  long long voxel_updates;         /* of completed requests */
} mtr_server_stats;
typedef struct mtr_server mtr_server;
mtr_status mtr_server_create(mtr_context* ctx, long long budget_bytes, int precision, mtr_server** out);
/* MTR_ERR_CAPACITY if the request alone exceeds the budget. */
mtr_status mtr_server_submit(mtr_server* s, const mtr_request* req, long long* id);
/* One scheduling step (see above); writes up to max_done retired ids. */
mtr_status mtr_server_step(mtr_server* s, int max_done, long long* done_ids, int* n_done);
mtr_status mtr_server_stats_get(const mtr_server* s, mtr_server_stats* st);
/* Waits for outstanding GPU work; queued and active requests are dropped. */
mtr_status mtr_server_destroy(mtr_server* s);

/* ---- MRC / TXBR / options (the reference's file I/O boundary) ----------- */

/* 1024-byte MRC header, same layout as MrcHeader (MrcFileIOBaseFunction.h:99-173). */
#pragma pack(push, 1)
typedef struct mtr_mrc_header {
  int nx, ny, nz, mode;
  int nxstart, nystart, nzstart;
  int mx, my, mz;
  float xlen, ylen, zlen;
  float alpha, beta, gamma;
  int mapc, mapr, maps;
  float amin, amax, amean;
  short ispg, nsymbt;
  int next;
  short creatid;
  char blank[30];
  short nint, nreal;
  short sub, zfac;
  float min2, max2, min3, max3, min4, max4;
  short idtype, lens, nd1, nd2, vd1, vd2;
  float tiltangles[6];
  float xorg, yorg, zorg;
  char cmap[4];
  char stamp[4];
  float rms;
  int nlabl;
  char labels[10][80];
} mtr_mrc_header;
#pragma pack(pop)

#define MTR_MRC_MODE_BYTE 0
#define MTR_MRC_MODE_SHORT 1
#define MTR_MRC_MODE_FLOAT 2
#define MTR_MRC_MODE_USHORT 6
#define MTR_MRC_MODE_HALF 12

/* Replaces mrcReadhead (MrcFileIOBaseFunction.cpp:11-16). */
mtr_status mtr_mrc_read_header(const char* path, mtr_mrc_header* out);
/* Replaces mrcReadAllData (MrcFileIOBaseFunction.cpp:18-70): n = nx*ny*nz
 * values converted to float.  The data block is the LAST n*bytes(mode)
 * bytes of the file (the reference takes file_size - n*2 for every mode,
 * which is the same offset for 16-bit modes).  Modes 0,1,2,6,12. */
mtr_status mtr_mrc_read_stack(const char* path, float* out, long long n);
/* The same values written straight into device memory (d_out: n floats on
 * the context's device).  No counterpart in the reference, which reads
 * element by element with fread (MrcFileIOBaseFunction.cpp:40-46): the data
 * block is read in 32 MiB chunks into two pinned buffers, and each chunk is
 * copied to the device and widened to float32 there while the next one is
 * read.  Synchronises the context stream before returning. */
mtr_status mtr_mrc_read_stack_device(mtr_context* ctx, const char* path, float* d_out, long long n);
/* The same values rounded to IEEE FP16 (round to nearest even) on the device:
 * d_out holds n halves.  Half the device bytes of the float32 variant. */
mtr_status mtr_mrc_read_stack_device_half(mtr_context* ctx, const char* path, void* d_out, long long n);
/* Replaces readCoef (MrcFileIOBaseFunction.cpp:72-134).  Appends x/y
 * coefficients (up to cap each), counts them in *n_x / *n_y, widens *vol by
 * the x->, y->, z-> bound lines and sets vol->X/Y/Z = end - start. */
mtr_status mtr_txbr_read(const char* path, double* x_coef, double* y_coef, int cap, int* n_x, int* n_y,
                         mtr_volume_size* vol);
/* ---- Geometry front end: tilt angles and 2-D alignments -> linear maps ----
 * No counterpart in the reference, which only reads precomputed linear maps
 * (readCoef, MrcFileIOBaseFunction.cpp:72-134).  These build the same
 * per-view maps x = c0 + c1 X + c2 Y + c3 Z (1-based detector pixel
 * coordinates of voxel (X, Y, Z), the TXBR coefficient order) from a
 * parallel-beam tilt series.
 *
 * Aligned view k of tilt angle t about an axis at in-plane angle phi:
 *   u_al - cu = cos(t) (cos(phi) (X-cx) + sin(phi) (Y-cy)) + sin(t) (Z-cz)
 *   v_al - cv = -sin(phi) (X-cx) + cos(phi) (Y-cy)
 * with detector centre (cu, cv) = ((det_x+1)/2, (det_y+1)/2) and volume
 * centre c = ((Xstart+Xend-1)/2, ...).  An alignment transform (IMOD .xf
 * convention: rows "a11 a12 a21 a22 dx dy", applied about the image centre)
 * maps raw view coordinates to aligned ones,
 *   al - C = A (raw - C) + (dx, dy),
 * so the maps returned address the RAW view: raw = C + A^-1 (al - C - d).
 * xf == NULL means identity for every view.  Fails with
 * MTR_ERR_INVALID_ARGUMENT for a singular A or a non-finite input. */
typedef struct mtr_xf {
  double a11, a12, a21, a22, dx, dy;
} mtr_xf;
mtr_status mtr_geometry_from_tilts(int n_views, const double* tilt_deg, const mtr_xf* xf, double phi_deg, int det_x,
                                   int det_y, mtr_volume_size vol, double* x_coef, double* y_coef);
/* Writes n_views linear maps (4 doubles per view each, TXBR coefficient
 * order) and the volume bounds of vol as a TXBR file in the grammar that
 * mtr_txbr_read and the reference's readCoef (MrcFileIOBaseFunction.cpp:72-134)
 * parse, every coefficient reading back exactly: maps built by
 * mtr_geometry_from_tilts from IMOD .tlt / .xf files become inputs of the
 * reference's command line (-i K,stacks,maps). */
mtr_status mtr_txbr_write(const char* path, int n_views, const double* x_coef, const double* y_coef,
                          mtr_volume_size vol);
/* One angle per line (IMOD .tlt); reads up to cap values into *n. */
mtr_status mtr_tlt_read(const char* path, double* tilt_deg, int cap, int* n);
/* Six numbers per line "a11 a12 a21 a22 dx dy" (IMOD .xf); up to cap views. */
mtr_status mtr_xf_read(const char* path, mtr_xf* xf, int cap, int* n);

/* Initialise a volume frame to the reference's empty bounds
 * (Xstart=999999, Xend=-999999, ..., MrcFileIO.h:22-28). */
void mtr_volume_size_empty(mtr_volume_size* vol);
/* Replaces updataAndWriteModel/writeModel (MrcFileIO.cpp:180-201): float32
 * MRC with the reference's header fields (MrcFileIO.cpp:3-61) and amin /
 * amax / amean computed from data (amean = mean of per-section means). */
mtr_status mtr_mrc_write_volume(const char* path, mtr_volume_size vol, const float* data);
/* Write a projection stack [nz][ny][nx] (modes 1, 2 or 12) with a minimal
 * header; used to produce test inputs in the reference's format. */
mtr_status mtr_mrc_write_stack(const char* path, int nx, int ny, int nz, int mode, const float* data);

/* Parsed command line (readOptions, ReadAndInitialOptions.cpp:127-172). */
typedef struct mtr_options {
  int number_tilt;
  char mrc_path[MTR_MAX_AXES][1024];
  char txbr_path[MTR_MAX_AXES][1024];
  char out_path[1024];
  int block_x, block_y, block_z; /* -x -y -z, kept as tile hints */
  int iter_times;                /* -n */
  float sirt_step;               /* -s */
  float mace_step;               /* -m */
  int sirt_inner;                /* --inner (long option; default 10) */
  int precision;                 /* --precision fp32|bf16|fp16 */
  int help;                      /* -h given */
} mtr_options;

/* Same short options as the reference (-h -i -o -x -y -z -n -s -m) plus the
 * long options --inner N and --precision P.  Unlike the reference, an
 * invalid option or a malformed -i list is an error (MTR_ERR_INVALID_ARGUMENT). */
mtr_status mtr_parse_options(int argc, char** argv, mtr_options* out);

#ifdef __cplusplus
}
#endif

#endif /* MTR_H_ */
