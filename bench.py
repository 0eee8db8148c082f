#!/usr/bin/env python
"""Benchmark: multi-axis SIRT + MACE reconstruction, voxel-updates/s on GB300.

One step = one complete reconstruction of the workload (per-axis WBP init,
n_outer MACE iterations of n_inner SIRT iterations per axis, consensus),
with inputs resident in HBM.  voxel-updates per step = V * K * n_outer * n_inner.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--config c2] [--impl ours|reference]

The default workload is the 3-axis 512x512x128 MACE configuration; the
headline value is the mixed-precision path (FP16 volume copy for the forward
splat, BF16 with --precision bf16; FP16 projections and MACE-state
deviations; FP32 interpolation, accumulation, iterate and residual; FP64
consensus sum), with the plain FP32 path timed beside it.  Multi-GPU runs
are independent replicas (the reconstruction is not sharded across GPUs).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
PKG = ROOT / "multi-tilt-reconstuction_gb300"
for p in (str(PKG), str(ROOT / "oracle"), str(ROOT)):
    if p not in sys.path:
        sys.path.insert(0, p)

METRIC = "SIRT voxel-updates/s mixed vs FP32 @<=1e-3 rel-L2 vs FP64"
UNIT = "voxel-updates/s"

CONFIGS = {
    "c1": dict(workload="single-axis SIRT 128x128x32, 61 tilts (+-60 step 2) x 128^2 px, WBP + 10 SIRT, lambda 0.5",
               vol=(0, 128, 0, 128, 0, 32), px=128, tilts=(-60, 61, 2), phis=(0.0,), n_ell=20,
               noise=("gaussian", 0.02), seed=1001, n_outer=1, n_inner=10, sirt_step=0.5, mace_step=0.5),
    "c2": dict(workload="3-axis MACE 512x512x128, axes 0/60/120 deg, 61 tilts (+-60 step 2) x 512^2 px, "
                        "2 MACE x 10 SIRT per axis, lambda 0.5, rho 0.8",
               vol=(0, 512, 0, 512, 0, 128), px=512, tilts=(-60, 61, 2), phis=(0.0, 60.0, 120.0), n_ell=50,
               noise=("gaussian", 0.05), seed=1002, n_outer=2, n_inner=10, sirt_step=0.5, mace_step=0.8),
    "c3": dict(workload="4-axis 2048x2048x256, axes 0/45/90/135 deg, 121 tilts (+-60 step 1) x 2048^2 px, "
                        "3 MACE x 10 SIRT per axis, lambda 0.5, rho 0.7, Poisson dose 50",
               vol=(0, 2048, 0, 2048, 0, 256), px=2048, tilts=(-60, 61, 1), phis=(0.0, 45.0, 90.0, 135.0), n_ell=200,
               noise=("poisson", 50.0), seed=1003, n_outer=3, n_inner=10, sirt_step=0.5, mace_step=0.7),
}


# Per-launch DRAM traffic and instruction count of the dominant kernel, from
# the ncu captures summarised in profiles/ (one launch of axis 0).
NCU_PROFILES = {
    ("c2", "backproject"): {"traffic": 390_982_656 + 167_104_768, "warp_inst": 828_349_812,
                            "duration_ms": 0.937248, "sm_ghz": 2.070, "sms": 152,
                            "source": "profiles/bp_tma_kernel_3axis_512x512x128.md"},
    ("c2", "forward"): {"traffic": 128_399_104 + 40_043_008, "warp_inst": 1_279_387_488,
                        "duration_ms": 1.282304, "sm_ghz": 2.047, "sms": 152,
                        "source": "profiles/fwd_tma_kernel_3axis_512x512x128.md"},
}


def cfg_voxel_angles(cfg: dict) -> int:
    """Voxel-angle evaluations of one projector launch (one axis, all angles)."""
    x0, x1, y0, y1, z0, z1 = cfg["vol"]
    t0, t1, dt = cfg["tilts"]
    return (x1 - x0) * (y1 - y0) * (z1 - z0) * len(range(t0, t1, dt))


def peaks() -> tuple[dict, str]:
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        return json.loads(f.read_text()), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def reduce_max(x: float, device=None) -> float:
    """Max of x over all ranks of the default process group (identity when not
    distributed).  Works on NCCL (CUDA tensor) and gloo (CPU tensor)."""
    import torch

    if not (torch.distributed.is_available() and torch.distributed.is_initialized()):
        return x
    dev = device if torch.distributed.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def replica_value(units_per_rank: float, world: int, max_ms_per_step: float) -> float:
    """Whole-job throughput of N independent replicas: every rank's units over
    the slowest rank's time per step."""
    return units_per_rank * world / (max_ms_per_step * 1e-3)


def voxel_updates(cfg: dict) -> int:
    v = cfg["vol"]
    V = (v[1] - v[0]) * (v[3] - v[2]) * (v[5] - v[4])
    return V * len(cfg["phis"]) * cfg["n_outer"] * cfg["n_inner"]


def n_angles(cfg: dict) -> int:
    return len(range(*cfg["tilts"]))


L2_BYTES = 129 * 10**6  # GB300 L2


def l2_note(cfg: dict) -> str:
    """How the timed step's arrays compare with L2 (no flush between steps)."""
    v = cfg["vol"]
    vb = (v[1] - v[0]) * (v[3] - v[2]) * (v[5] - v[4]) * 4
    pb = cfg["px"] * cfg["px"] * n_angles(cfg) * 4
    K = len(cfg["phis"])
    total = K * (3 * vb + 4 * pb) + vb
    if vb > L2_BYTES:
        return (f"inputs larger than L2: each FP32 volume array {vb / 1e6:.0f} MB, projection arrays "
                f"{pb / 1e6:.0f} MB per axis, {total / 1e9:.1f} GB of arrays in all (L2 129 MB)")
    return (f"each FP32 volume array {vb / 1e6:.1f} MB and projection array {pb / 1e6:.1f} MB fit L2 (129 MB); "
            f"{total / 1e6:.0f} MB of arrays in all, no flush between steps: an L2-resident workload")


# ----------------------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []
        self.t = None

    def start(self) -> None:
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, ValueError):
            self.proc = None

    def _read(self) -> None:
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        # A timed region shorter than nvidia-smi's start-up and sampling period
        # has no sample of its own: take the first one, right after it.
        after = not self.lines
        deadline = time.time() + 3.0
        while not self.lines and time.time() < deadline and self.proc.poll() is None:
            time.sleep(0.01)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.t:
            self.t.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        out = {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
               "reasons": sorted(reasons), "samples": len(sm)}
        if after and sm:
            out["sampled"] = "right after the timed region (shorter than the sampling period)"
        return out


# ----------------------------------------------------------------------------------------
def make_inputs(cfg: dict, device: str):
    import mtr
    import phantom

    vol = mtr.VolumeSize.make(*cfg["vol"])
    tilts = np.arange(*cfg["tilts"], dtype=np.float64)
    kind, level = cfg["noise"]
    case = phantom.make_case_torch(vol, cfg["px"], tilts, list(cfg["phis"]), cfg["n_ell"], kind, level, cfg["seed"],
                                   device=device)
    axes = [mtr.AxisData(xc, yc, d) for (xc, yc, d) in case["axes"]]
    return vol, axes, case["meta"]


def mrc_load_throughput(torch, mtr, ctx, data: np.ndarray) -> dict:
    """Axis 0 written as an int16 MRC stack (scaled to +-30000), then loaded
    into device memory twice: the host reader (float32 array) followed by a
    copy to the device, and mtr_mrc_read_stack_device.  The file was just
    written, so both read it from the page cache."""
    import tempfile

    d = tempfile.mkdtemp(prefix="mtr_io_")
    path = os.path.join(d, "axis0.mrc")
    try:
        scale = 30000.0 / max(float(np.abs(data).max()), 1e-30)
        mtr.write_mrc_stack(path, data * scale, 1)
        nbytes = data.size * 2
        dev = torch.empty(data.size, dtype=torch.float32, device="cuda")
        out = {"file_bytes": nbytes, "mode": 1}
        for name, fn in (("host_read_then_copy", lambda: dev.copy_(torch.from_numpy(mtr.read_mrc_stack(path).reshape(-1)))),
                         ("device_read", lambda: mtr.read_mrc_stack_device(ctx, path, dev))):
            fn()  # warm the page cache and the code path
            torch.cuda.synchronize()
            t = time.perf_counter()
            for _ in range(3):
                fn()
            torch.cuda.synchronize()
            out[name + "_gbs"] = 3 * nbytes / (time.perf_counter() - t) / 1e9
        out["speedup"] = out["device_read_gbs"] / out["host_read_then_copy_gbs"]
        del dev
        return out
    finally:
        if os.path.exists(path):
            os.remove(path)
        os.rmdir(d)


def rel_l2_np(a, b) -> float:
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-30))


def time_steps(torch, stream, recon, steps: int) -> float:
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    start.record(stream)
    for _ in range(steps):
        recon.run()
    end.record(stream)
    end.synchronize()
    return start.elapsed_time(end) / steps


def algorithmic_bytes(kind: str, cfg: dict, prec: int) -> tuple[float, str]:
    """Compulsory HBM bytes of one launch of a kernel class (one axis)."""
    import mtr

    v = cfg["vol"]
    V = (v[1] - v[0]) * (v[3] - v[2]) * (v[5] - v[4])
    P = cfg["px"] * cfg["px"] * n_angles(cfg)
    pe = 2 if prec != mtr.PREC_FP32 else 4
    if kind == "backproject":
        # read r (FP32, P), read+write the FP32 iterate, read the weight sums (+ write the 16-bit copy when mixed)
        b = P * 4 + V * 12 + (V * 2 if prec != mtr.PREC_FP32 else 0)
        return b, f"P*4 (residual) + V*12 (iterate r/w, weight sums){' + V*2 (16-bit copy)' if pe == 2 else ''}"
    if kind == "forward":
        vb = 2 if prec != mtr.PREC_FP32 else 4
        return P * 4 + V * vb, f"V*{vb} (volume read) + P*4 (ray-sum write)"
    if kind == "residual":
        return P * (4 + 4 + 4 + pe + pe), f"P*(s r/w 8 + c 4 + b {pe} + r {pe})"
    if kind == "mace":
        K = len(cfg["phis"])
        return V * 4 * (2 + 4 * K), "V*4*(2 + 4K) (w_avg r/w, w_k r/w, x_k r/w)"
    return 0.0, "n/a"


# ----------------------------------------------------------------------------------------
def run_ours(args, rank: int, world: int, local_rank: int) -> dict | None:
    import torch

    import mtr

    cfg = CONFIGS[args.config]
    torch.cuda.set_device(local_rank)
    device = f"cuda:{local_rank}"
    # A dedicated stream: libmtr launches on it and the timing events are
    # recorded on it (the legacy default stream's handle is 0, which the
    # library would read as "use your own stream").
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx = mtr.Context(local_rank)
    ctx.set_stream(stream.cuda_stream)
    assert stream.cuda_stream != 0
    t0 = time.time()
    vol, axes, meta = make_inputs(cfg, device)
    gen_s = time.time() - t0
    no, ni = cfg["n_outer"], cfg["n_inner"]
    prec = {"bf16": mtr.PREC_MIXED_BF16, "fp16": mtr.PREC_MIXED_FP16, "fp32": mtr.PREC_FP32}[args.precision]
    mk = lambda pr: mtr.params(iter_times=no, sirt_inner=ni, sirt_step=cfg["sirt_step"], mace_step=cfg["mace_step"],
                               precision=pr)

    def mk_timed(pr):  # the device-resident runs replay one CUDA graph per run
        p = mk(pr)
        p.flags = mtr.FLAG_GRAPH if args.graph else 0
        return p

    rec = mtr.Recon(ctx, axes, vol, mk_timed(prec), mem_kind=mtr.MEM_DEVICE)
    tiles = rec.describe()
    ref32 = mtr.Recon(ctx, axes, vol, mk_timed(mtr.PREC_FP32), mem_kind=mtr.MEM_DEVICE) if prec != mtr.PREC_FP32 else rec

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    def max_over_ranks(x: float) -> float:
        return reduce_max(x, device)

    # warm-up
    for _ in range(args.warmup):
        rec.run()
        if ref32 is not rec:
            ref32.run()
    torch.cuda.synchronize()

    # timed region: headline precision, clocks sampled
    clocks = ClockSampler(local_rank)
    launches0 = ctx.launch_count()
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    ms = time_steps(torch, stream, rec, args.steps)
    clk = clocks.stop()
    launches = ctx.launch_count() - launches0
    barrier()
    ms = max_over_ranks(ms)

    # one more step with every launch bracketed by CUDA events (per kernel
    # class device time for the roofline; the axes then run one after another)
    ctx.profile_reset()
    ctx.set_profiling(True)
    rec.run()
    torch.cuda.synchronize()
    ctx.set_profiling(False)
    prof = ctx.profile()

    # plain FP32 path, same workload
    ms32 = time_steps(torch, stream, ref32, args.steps) if ref32 is not rec else ms
    ms32 = max_over_ranks(ms32)

    # the naive global-atomic kernels, FP32: the reference's kernel structure
    # (a global-memory gather and a global float-atomic splat) in this library
    # (MTR_DISABLE_TMA=1 is read at creation and at every launch, so it is set
    # only around this run).  Not the plain FP32 path: that is `fp32` above.
    naive = None
    if args.extras and args.config in ("c1", "c2"):
        os.environ["MTR_DISABLE_TMA"] = "1"
        try:
            rp = mtr.Recon(ctx, axes, vol, mk(mtr.PREC_FP32), mem_kind=mtr.MEM_DEVICE)
            rp.run()
            ms_naive = max_over_ranks(time_steps(torch, stream, rp, 1))
            err_naive = rel_l2_np(rp.download(), ref32.download())
            rp.close()
        finally:
            del os.environ["MTR_DISABLE_TMA"]
        naive = {"ms_per_step": ms_naive, "mixed_over_naive": ms_naive / ms, "fp32_over_naive": ms_naive / ms32,
                 "rel_l2_vs_fp32": err_naive,
                 "kernels": "bp_gather_kernel + fwd_splat_kernel (global float atomics), FP32"}

    # the streaming slab loop: volume arrays in host memory, two device slabs
    streamed = None
    if args.stream_slabs:
        ps = mk(prec)
        ps.flags = mtr.FLAG_STREAM_SLABS
        ps.slab_depth = args.stream_slabs
        t0 = time.time()
        rs = mtr.Recon(ctx, axes, vol, ps, mem_kind=mtr.MEM_DEVICE)
        create_s = time.time() - t0
        rs.run()  # warm-up
        ms_s = max_over_ranks(time_steps(torch, stream, rs, 1))
        streamed = {"ms_per_step": ms_s, "value": voxel_updates(cfg) / (ms_s * 1e-3), "slab_depth": args.stream_slabs,
                    "device_bytes": rs.footprint(), "device_bytes_resident": rec.footprint(),
                    "vs_device_resident": ms_s / ms, "rel_l2_vs_device_resident": rel_l2_np(rs.download(), rec.download()),
                    "create_s": round(create_s, 1),
                    "host_bytes": (4 + len(axes) * (14 if prec != mtr.PREC_FP32 else 12)) * vol.X * vol.Y * vol.Z}
        rs.close()

    # volumes in mapped host memory (MTR_FLAG_HOST_VOLUMES), same precision and inputs
    host_vol = None
    if args.extras and args.config in ("c1", "c2"):
        ph = mk(prec)
        ph.flags = mtr.FLAG_HOST_VOLUMES
        rh = mtr.Recon(ctx, axes, vol, ph, mem_kind=mtr.MEM_DEVICE)
        rh.run()
        ms_h = max_over_ranks(time_steps(torch, stream, rh, 1))
        host_vol = {"ms_per_step": ms_h, "device_bytes": rh.footprint(), "vs_device_resident": ms_h / ms,
                    "rel_l2_vs_device_resident": rel_l2_np(rh.download(), rec.download())}
        rh.close()

    out_mixed = rec.download()
    out_fp32 = ref32.download()
    footprint = {args.precision: rec.footprint(), "fp32": ref32.footprint()}
    # free both device-resident runs before the end-to-end calls allocate their own
    rec.close()
    if ref32 is not rec:
        ref32.close()

    # end to end through the public host-buffer API: H2D of the projections from
    # pinned memory, device allocation, geometry sums, the run, D2H of the volume
    host_axes = []
    h2d = 0
    for a in axes:
        pinned = torch.empty(a.data.shape, dtype=torch.float32, pin_memory=True)
        pinned.copy_(a.data)
        host_axes.append(mtr.AxisData(a.x_coef, a.y_coef, pinned.numpy()))
        h2d += pinned.numel() * 4 + a.x_coef.nbytes + a.y_coef.nbytes
    del axes, a
    torch.cuda.empty_cache()
    out_pinned = torch.empty(vol.shape, dtype=torch.float32, pin_memory=True).numpy()
    p_e2e = mk(prec)
    arr_ms = []
    import ctypes as C

    arr = (mtr.AxisC * len(host_axes))(*[a.c_struct() for a in host_axes])
    first_ms = None
    for i in range(1 + max(1, args.e2e_steps)):
        torch.cuda.synchronize()
        t = time.perf_counter()
        ctx.check(ctx.lib.mtr_reconstruct(ctx.h, len(host_axes), arr, vol, C.byref(p_e2e), out_pinned.ctypes.data),
                  "mtr_reconstruct")
        dt = time.perf_counter() - t
        if i > 0:
            arr_ms.append(dt * 1e3)
        else:
            first_ms = dt * 1e3  # this process' first call of this geometry (tile plans already cached by the runs above)
    # median of the calls: one call is one full reconstruction, and host-side
    # stalls (page faults, scheduling) make single calls vary by several %
    e2e_ms = max_over_ranks(statistics.median(arr_ms))

    io = mrc_load_throughput(torch, mtr, ctx, host_axes[0].data) if args.extras else None

    # error of both paths against the all-FP64 GPU reconstruction of the same inputs
    err64 = None
    if args.fp64 and args.config != "c3":
        t = time.time()
        out64 = ctx.reconstruct_fp64(host_axes, vol, mk(mtr.PREC_FP32))
        n64 = max(float(np.linalg.norm(out64)), 1e-300)
        err64 = {"mixed_vs_fp64_rel_l2": float(np.linalg.norm(out_mixed - out64) / n64),
                 "fp32_vs_fp64_rel_l2": float(np.linalg.norm(out_fp32 - out64) / n64),
                 "fp64_run_s": round(time.time() - t, 1), "on": "the whole workload"}
    elif args.fp64:
        # The all-FP64 run of the whole 4-axis 2048x2048x256 workload would take
        # the FP64 pipe many minutes: the error is stated on an 8-plane Z-slab
        # of it (full 2048^2 lateral extent, the full detector and every tilt),
        # 1 MACE x 10 SIRT, with the same maps and projections.
        t = time.time()
        zc = (vol.Zstart + vol.Zend) // 2
        sub = mtr.VolumeSize.make(vol.Xstart, vol.Xend, vol.Ystart, vol.Yend, zc - 4, zc + 4)
        psub = lambda pr: mtr.params(iter_times=1, sirt_inner=ni, sirt_step=cfg["sirt_step"],
                                     mace_step=cfg["mace_step"], precision=pr)
        out64 = ctx.reconstruct_fp64(host_axes, sub, psub(mtr.PREC_FP32))
        mx_s = ctx.reconstruct(host_axes, sub, psub(prec))
        f32_s = ctx.reconstruct(host_axes, sub, psub(mtr.PREC_FP32))
        n64 = max(float(np.linalg.norm(out64)), 1e-300)
        err64 = {"mixed_vs_fp64_rel_l2": float(np.linalg.norm(mx_s - out64) / n64),
                 "fp32_vs_fp64_rel_l2": float(np.linalg.norm(f32_s - out64) / n64),
                 "fp64_run_s": round(time.time() - t, 1),
                 "on": f"an 8-plane Z-slab [{zc - 4}, {zc + 4}) of the volume (full lateral extent, detector and "
                       f"tilts), 1 MACE x {ni} SIRT"}

    vu = voxel_updates(cfg)
    res = {"tiles": tiles, "ms": ms, "ms32": ms32, "e2e_ms": e2e_ms, "e2e_first_ms": first_ms, "h2d": h2d,
           "d2h": vol.X * vol.Y * vol.Z * 4, "clk": clk,
           "prof": prof, "launches": launches, "gen_s": gen_s, "meta": meta, "vu": vu,
           "mixed_vs_fp32": float(np.linalg.norm(out_mixed.astype(np.float64) - out_fp32) /
                                  max(np.linalg.norm(out_fp32.astype(np.float64)), 1e-30)),
           "axes_host": host_axes, "vol": vol, "prec": prec, "err64": err64, "io": io, "naive": naive,
           "host_vol": host_vol, "streamed": streamed, "footprint": footprint}
    rec.close()
    if ref32 is not rec:
        ref32.close()
    ctx.close()
    return res


C4 = dict(workload="64 seeded tilt series, detector and volume lateral size U{128..1024} px, tilts U{41..121} "
                   "over +-60 deg, axes U{1..4} (in-plane angles k*180/K), depth U{32..256}, 8 ellipsoids each, "
                   "Gaussian noise 0.02; WBP init, 1 MACE x 3 SIRT, lambda 0.5, rho 0.7",
          n=64, seed=1004, n_ell=8, n_outer=1, n_inner=3)


def make_batch_instances(device: str, n: int | None = None, seed: int | None = None):
    """Uneven instances of the batched workload's size distribution (host
    float32 projections; generated on the GPU)."""
    import torch

    import mtr
    import phantom

    seed = C4["seed"] if seed is None else seed
    rng = np.random.default_rng(seed)
    inst = []
    for i in range(C4["n"] if n is None else n):
        px = int(rng.integers(128, 1025))
        A = int(rng.integers(41, 122))
        K = int(rng.integers(1, 5))
        Z = int(rng.integers(32, 257))
        vol = mtr.VolumeSize.make(0, px, 0, px, 0, Z)
        tilts = np.linspace(-60.0, 60.0, A)
        phis = [k * 180.0 / K for k in range(K)]
        case = phantom.make_case_torch(vol, px, tilts, phis, C4["n_ell"], "gaussian", 0.02, seed * 100 + i,
                                       device=device)
        axes = [mtr.AxisData(xc, yc, d.cpu().numpy()) for (xc, yc, d) in case["axes"]]
        del case
        torch.cuda.empty_cache()
        inst.append((axes, vol))
    return inst


def run_batch_bench(args) -> dict:
    """Config 4: all instances in one batch (one persistent launch per SIRT phase,
    CUDA graph, mixed storage) against looping the plain FP32 path over them."""
    import torch

    import mtr

    torch.cuda.set_device(0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx = mtr.Context(0)
    ctx.set_stream(stream.cuda_stream)
    t0 = time.time()
    inst = make_batch_instances("cuda:0")
    gen_s = time.time() - t0
    prec = {"bf16": mtr.PREC_MIXED_BF16, "fp16": mtr.PREC_MIXED_FP16, "fp32": mtr.PREC_FP32}[args.precision]
    p = mtr.params(iter_times=C4["n_outer"], sirt_inner=C4["n_inner"], sirt_step=0.5, mace_step=0.7, precision=prec,
                   flags=mtr.FLAG_GRAPH)
    t0 = time.time()
    batch = mtr.Batch(ctx, inst, p)
    create_s = time.time() - t0
    info = batch.info()
    for _ in range(max(1, args.warmup)):
        batch.run()
    launches0 = ctx.launch_count()
    ms = time_steps(torch, stream, batch, args.steps)
    launches = (ctx.launch_count() - launches0) // max(1, args.steps)
    batched = [batch.download(i) for i in range(len(inst))]
    batch.close()
    # per-phase device time of one run, without the graph (events around each launch)
    pn = mtr.params(iter_times=C4["n_outer"], sirt_inner=C4["n_inner"], sirt_step=0.5, mace_step=0.7, precision=prec)
    batch = mtr.Batch(ctx, inst, pn)
    batch.run()
    torch.cuda.synchronize()
    ctx.profile_reset()
    ctx.set_profiling(True)
    batch.run()
    torch.cuda.synchronize()
    ctx.set_profiling(False)
    batch_prof = {k: round(v[1], 2) for k, v in ctx.profile().items()}
    batch.close()
    # plain FP32 path looped over the instances (device-resident inputs, run only timed)
    pf = mtr.params(iter_times=C4["n_outer"], sirt_inner=C4["n_inner"], sirt_step=0.5, mace_step=0.7)
    loop_ms, errs = 0.0, []
    ctx.profile_reset()
    for i, (axes, vol) in enumerate(inst):
        r = mtr.Recon(ctx, axes, vol, pf)
        r.run()  # warm-up (module load, first-touch)
        loop_ms += time_steps(torch, stream, r, 1)
        ctx.set_profiling(True)
        r.run()
        torch.cuda.synchronize()
        ctx.set_profiling(False)
        ref = r.download()
        r.close()
        errs.append(float(np.linalg.norm(batched[i] - ref) / max(np.linalg.norm(ref), 1e-30)))
    vu = info["voxel_updates"]
    sizes = [vol.X for _, vol in inst]
    return {"metric": METRIC, "value": vu / (ms * 1e-3), "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": C4["workload"], "precision": args.precision, "instances": len(inst),
                       "axes_total": sum(len(a) for a, _ in inst), "voxel_updates_per_step": vu,
                       "device_bytes": info["bytes"], "work_items": info["items"],
                       "lateral_px": [min(sizes), max(sizes)], "seed": C4["seed"],
                       "l2": "inputs larger than L2", "generation_s": round(gen_s, 1),
                       "create_and_tune_s": round(create_s, 1)},
            "phase_ms": {"batched": batch_prof, "fp32_loop": {k: round(v[1], 2) for k, v in ctx.profile().items()}},
            "fp32_loop": {"value": vu / (loop_ms * 1e-3), "ms_per_step": loop_ms,
                          "batched_over_loop": loop_ms / ms,
                          "rel_l2_batched_vs_fp32_max": max(errs), "rel_l2_batched_vs_fp32_median": float(np.median(errs))},
            "gpu_launches": launches, "e2e": None}


C5 = dict(workload="serving: Poisson arrivals of reconstruction requests drawn from a pool of 12 seeded instances "
                   "of the batched workload's size distribution (lateral U{128..1024} px, tilts U{41..121}, axes "
                   "U{1..4}, depth U{32..256}); each request 1..3 MACE x 10 SIRT (10-30 iterations), lambda 0.5, "
                   "rho 0.7; admission by device footprint under a 180 GB budget; continuous batching",
          pool=12, seed=1005, budget=180 * 10**9, rates=(0.5, 1, 2, 5, 10, 50), per_rate=12)


def serve_rate(mtr, ctx, pool, rate: float, n_req: int, precision: int, rng, keep: int = 0) -> dict:
    """Serve n_req Poisson arrivals at `rate` req/s; latency = retire time - arrival time."""
    srv = mtr.Server(ctx, C5["budget"], precision)
    gaps = rng.exponential(1.0 / rate, n_req)
    arrive = np.cumsum(gaps) - gaps[0]
    picks = rng.integers(0, len(pool), n_req)
    outer = rng.integers(1, 4, n_req)
    ids, lat, kept, vu = {}, {}, {}, 0
    t0 = time.perf_counter()
    nxt = 0
    while len(lat) < n_req:
        now = time.perf_counter() - t0
        while nxt < n_req and arrive[nxt] <= now:
            axes, vol = pool[picks[nxt]]
            ids[srv.submit(axes, vol, int(outer[nxt]), 10, 0.5, 0.7)] = nxt
            vu += vol.X * vol.Y * vol.Z * len(axes) * int(outer[nxt]) * 10
            nxt += 1
        st = srv.stats()
        if st["queued"] == 0 and st["active"] == 0 and nxt < n_req:
            time.sleep(max(0.0, arrive[nxt] - (time.perf_counter() - t0)))
            continue
        for rid, v in srv.step():
            i = ids[rid]
            lat[i] = time.perf_counter() - t0 - arrive[i]
            if i < keep:
                kept[i] = v
    wall = time.perf_counter() - t0
    st = srv.stats()
    srv.close()
    ls = np.array([lat[i] for i in range(n_req)]) * 1e3
    return {"rate_req_s": rate, "requests": n_req, "p50_ms": float(np.percentile(ls, 50)),
            "p99_ms": float(np.percentile(ls, 99)), "throughput_req_s": n_req / wall,
            "voxel_updates_per_s": vu / wall, "steps": st["steps"], "peak_bytes": st["peak_bytes"],
            "wall_s": wall, "_kept": kept, "_picks": picks[:keep].tolist(), "_outer": outer[:keep].tolist()}


def run_serve_bench(args) -> dict:
    """Config 5: rate sweep of the continuous-batching server, mixed storage
    and FP32; the first requests of the lowest rate are compared
    between the two precisions."""
    import torch

    import mtr

    torch.cuda.set_device(0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx = mtr.Context(0)
    ctx.set_stream(stream.cuda_stream)
    t0 = time.time()
    pool = make_batch_instances("cuda:0", n=C5["pool"], seed=C5["seed"])
    gen_s = time.time() - t0
    torch.cuda.empty_cache()
    prec = {"bf16": mtr.PREC_MIXED_BF16, "fp16": mtr.PREC_MIXED_FP16, "fp32": mtr.PREC_FP32}[args.precision]
    # warm-up: every pool member once (tile tuning, module load)
    for p in (prec, mtr.PREC_FP32):
        srv = mtr.Server(ctx, C5["budget"], p)
        for axes, vol in pool:
            srv.submit(axes, vol, 1, 1)
        srv.drain()
        srv.close()
    rates = C5["rates"]
    out = {}
    for name, p in ((args.precision, prec), ("fp32", mtr.PREC_FP32)):
        rng = np.random.default_rng(C5["seed"])
        out[name] = [serve_rate(mtr, ctx, pool, r, C5["per_rate"], p, rng, keep=4 if r == rates[0] else 0)
                     for r in rates]
    a, b = out[args.precision][0]["_kept"], out["fp32"][0]["_kept"]
    errs = [float(np.linalg.norm(a[i] - b[i]) / max(np.linalg.norm(b[i]), 1e-30)) for i in sorted(a)]
    for rows in out.values():
        for r in rows:
            for k in ("_kept", "_picks", "_outer"):
                r.pop(k)
    top = out[args.precision][-1]
    return {"metric": METRIC, "value": top["voxel_updates_per_s"], "unit": UNIT, "n_gpus": 1, "steps": len(rates),
            "warmup": 1, "ms_per_step": None, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": C5["workload"], "precision": args.precision, "budget_bytes": C5["budget"],
                       "rates_req_s": list(rates), "requests_per_rate": C5["per_rate"], "seed": C5["seed"],
                       "pool_generation_s": round(gen_s, 1), "value_at": f"{rates[-1]} req/s (saturated)"},
            "serve": out, "error": {"mixed_vs_fp32_rel_l2_max": max(errs), "requests_compared": len(errs)},
            "gpu_launches": None, "e2e": None}


def cpu_slab(vol, n_angles: int) -> int:
    """Z planes of the CPU sample: the whole volume up to ~2 G voxel-angle
    evaluations per SIRT iteration (a few seconds on the host cores)."""
    return int(max(1, min(vol.Z, round(2e9 / (vol.X * vol.Y * n_angles)))))


def cpu_baseline(cfg: dict, vol, axes_host, budget_s: float = 20.0) -> dict:
    """Reference-faithful CPU oracle on the host cores: SIRT iterations of axis 0
    over a Z-slab (the whole volume up to ~2 G voxel-angle evaluations per
    iteration; each iteration = slab-voxels voxel-updates)."""
    import oracle

    n = os.cpu_count() or 1
    oracle.set_threads(n)
    a = axes_host[0]
    dz = cpu_slab(vol, a.data.shape[0])
    z0, z1 = vol.Zstart, vol.Zstart + dz
    x0 = np.zeros((dz, vol.Y, vol.X), np.float64)
    t = time.perf_counter()
    it = 0
    while True:
        oracle.sirt(oracle.REF_FAITHFUL, a, vol, x0, 1, cfg["sirt_step"], z0, z1)
        it += 1
        el = time.perf_counter() - t
        if el > budget_s / 2 or it >= 3:
            break
    V = vol.X * vol.Y * dz
    where = (f"the full {vol.X}x{vol.Y}x{vol.Z} volume" if dz == vol.Z else
             f"a {dz}-plane Z-slab of the {vol.X}x{vol.Y}x{vol.Z} volume")
    return {"value": V * it / el, "unit": UNIT, "cores": n, "kind": "port",
            "sample": f"{it} reference-faithful SIRT iteration(s) (forward splat + residual + back-projection) of "
                      f"axis 0 over {where}, OpenMP over {n} host threads, {el:.1f} s"}


def run_reference(args) -> dict:
    """The reference path on the host cores: its own implementation is CUDA+MPI
    with no CPU version, so the oracle restatement (reference-faithful precision)
    stands in; one step = one SIRT iteration of axis 0 on the full volume."""
    import torch

    import mtr
    import oracle

    cfg = CONFIGS[args.config]
    vol, axes, _ = make_inputs(cfg, "cuda:0" if torch.cuda.is_available() else "cpu")
    a = axes[0]
    host = mtr.AxisData(a.x_coef, a.y_coef, a.data.cpu().numpy() if hasattr(a.data, "cpu") else a.data)
    n = os.cpu_count() or 1
    oracle.set_threads(n)
    dz = cpu_slab(vol, host.data.shape[0])
    z0, z1 = vol.Zstart, vol.Zstart + dz
    x0 = np.zeros((dz, vol.Y, vol.X), np.float64)
    for _ in range(args.warmup):
        oracle.sirt(oracle.REF_FAITHFUL, host, vol, x0, 1, cfg["sirt_step"], z0, z1)
    t = time.perf_counter()
    for _ in range(args.steps):
        oracle.sirt(oracle.REF_FAITHFUL, host, vol, x0, 1, cfg["sirt_step"], z0, z1)
    el = time.perf_counter() - t
    V = vol.X * vol.Y * dz
    where = "the full volume" if dz == vol.Z else f"a {dz}-plane Z-slab"
    value = V * args.steps / el
    return {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": cfg["workload"], "step": "one SIRT iteration of axis 0 (bounded sample)"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": n, "kind": "port",
                             "sample": f"reference-faithful CPU restatement (the reference's path is CUDA+MPI only), "
                                       f"one SIRT iteration of axis 0 over {where} per step, {n} threads"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--config", default="c2", choices=sorted(CONFIGS) + ["c4", "c5"])
    ap.add_argument("--precision", default="fp16", choices=["bf16", "fp16", "fp32"],
                    help="mixed storage of the forward copy (fp16: FP16, bf16: BF16), or fp32 throughout")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--fp64", type=int, default=1, help="1: state both paths' error against the FP64 GPU run")
    ap.add_argument("--extras", type=int, default=1,
                    help="1: also time the naive global-atomic kernels, host-resident volumes and MRC loading (c1/c2)")
    ap.add_argument("--graph", type=int, default=1,
                    help="1: the device-resident timed runs replay a CUDA graph of the whole run")
    ap.add_argument("--stream-slabs", type=int, default=0,
                    help="D > 0: also time the streaming slab loop (volume arrays in host memory, D-plane slabs)")
    args = ap.parse_args()

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if rank != 0:
            return 0
        print(json.dumps(run_reference(args)), flush=True)
        return 0

    import __graft_entry__

    if args.config in ("c4", "c5"):
        __graft_entry__.build()
        line = run_batch_bench(args) if args.config == "c4" else run_serve_bench(args)
        print(json.dumps(line), flush=True)
        return 0

    if rank == 0 or world == 1:
        __graft_entry__.build()
    if world > 1:
        import torch

        torch.distributed.init_process_group("nccl", device_id=torch.device(f"cuda:{local_rank}"))
        torch.distributed.barrier()
        if rank != 0:
            __graft_entry__.build()

    r = run_ours(args, rank, world, local_rank)
    cfg = CONFIGS[args.config]
    if rank == 0:
        import mtr

        pk, pk_kind = peaks()
        prof = r["prof"]
        dom = max((k for k in prof if prof[k][0] > 0), key=lambda k: prof[k][1])
        n_l, tot = prof[dom]
        per_launch_ms = tot / n_l
        alg, alg_desc = algorithmic_bytes(dom, cfg, r["prec"])
        achieved = alg / (per_launch_ms * 1e-3) / 1e9
        ncu = NCU_PROFILES.get((args.config, dom))
        roof = {"bound": "hbm", "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
                "frac": achieved / pk["hbm_gbs"], "traffic": ncu["traffic"] if ncu else None, "kernel": dom,
                "peak_source": pk_kind,
                "algorithmic_bytes_per_launch": alg, "algorithmic_bytes": alg_desc,
                "avg_launch_ms": per_launch_ms, "launches": n_l,
                "kernel_share": {k: prof[k][1] / max(sum(x[1] for x in prof.values()), 1e-9) for k in prof}}
        if ncu:
            # the roof that binds is instruction issue; figures of the captured
            # launch (axis 0) against 4 issue slots per SM per clock
            issue_peak = ncu["sms"] * 4 * ncu["sm_ghz"] * 1e9
            inst_rate = ncu["warp_inst"] / (ncu["duration_ms"] * 1e-3)
            roof["binding"] = {"resource": "instruction issue", "achieved": inst_rate, "peak": issue_peak,
                               "unit": "warp-instructions/s", "frac": inst_rate / issue_peak,
                               "warp_inst_per_voxel_angle": ncu["warp_inst"] / cfg_voxel_angles(cfg),
                               "launch": "axis 0 (ncu)", "source": ncu["source"]}
        vu = r["vu"] * world
        value = replica_value(r["vu"], world, r["ms"])
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": r["ms"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": cfg["workload"], "precision": args.precision,
                       "storage": f"{args.precision} volume copy for the forward pass, fp16 projections, "
                                  "fp16 MACE-state deviations from the consensus, fp32 iterate/residual/weight sums/consensus"
                                  if args.precision != "fp32"
                       else "fp32", "voxel_updates_per_step": r["vu"], "parallelism": f"replicas x{world}",
                       "l2": l2_note(cfg),
                       "seed": cfg["seed"],
                       "tiles": [{"bp_depth": t["back_projection"]["depth"], "fwd_depth": t["forward"]["depth"],
                                  "bp_lanes": t["back_projection"]["lanes"], "fwd_lanes": t["forward"]["lanes"],
                                  "bp_window": t["back_projection"].get("window_format"),
                                  "tma": t["back_projection"]["tma"] and t["forward"]["tma"]} for t in r["tiles"]]},
            "fp32": {"value": vu / (r["ms32"] * 1e-3), "ms_per_step": r["ms32"],
                     "mixed_over_fp32": r["ms32"] / r["ms"]},
            "footprint_bytes": r["footprint"],
            "naive_atomic_fp32": None if r["naive"] is None else {"value": vu / (r["naive"]["ms_per_step"] * 1e-3),
                                                                  **r["naive"]},
            "host_volumes": r["host_vol"],
            "streamed_slabs": r["streamed"],
            "error": {"mixed_vs_fp32_rel_l2": r["mixed_vs_fp32"], **(r["err64"] or {})},
            "e2e": {"value": vu / (r["e2e_ms"] * 1e-3), "unit": UNIT, "h2d_bytes_per_step": r["h2d"],
                    "d2h_bytes_per_step": r["d2h"], "ms_per_step": r["e2e_ms"],
                    "first_call_ms": r["e2e_first_ms"], "statistic": f"median of {max(1, args.e2e_steps)} calls",
                    "api": "mtr_reconstruct (host buffers, pinned)"},
            "gpu_launches": r["launches"],
            "io": r["io"],
            "roofline": roof,
            "clocks": r["clk"],
        }
        if not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(cfg, r["vol"], r["axes_host"])
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch

        torch.distributed.barrier()
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
