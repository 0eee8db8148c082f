// Autotuner for the projector tile shapes.
//
// Two shape parameters decide the projectors' speed and depend on the
// geometry:
//  * brick depth (voxels per thread along Z): deep bricks amortise the
//    per-angle window work and, in the forward splat, merge more of a
//    column's taps; shallow bricks give more CTAs on small volumes and use
//    fewer registers;
//  * warp layout: lines along X keep volume accesses coalesced, lines along
//    the volume axis that detector x follows keep shared-memory gathers free
//    of bank conflicts, and (back-projection) 8x4 patches keep the taps of an
//    oblique axis compact in the window;
//  * the SIRT back-projection's window format: FP32 residual values, or
//    (value, next - value) pairs that halve the tap loads but double the
//    window and load 8 bytes per lane (faster where a warp's lanes share
//    detector rows, slower where their 8-byte loads conflict in the banks),
//    or the same pairs as two FP32 planes per row (4-byte loads with the FP32
//    window's bank pattern, one FFMA per row), or (mixed precision) FP16
//    pairs in 32 bits (one 4-byte load per row: half the shared-memory bytes).
// For each tilt axis the tuner times every candidate (3 formats x depth
// 4/8/16/32 x lines along X / lines along Y / patches for the SIRT
// back-projection, depth 8/16/32 x the same three layouts for the forward
// splat) with CUDA events on the reconstruction's own buffers, over a Z-slab
// of the frame sized for 8 waves of the deepest tile, before they hold data
// (each candidate launch writes only scratch that the run overwrites), and
// keeps the fastest.  Results are cached per process by a geometry key and,
// when MTR_AUTOTUNE_CACHE names a file, persisted there as JSON ({"key":
// [bp_depth, fwd_depth, bp_lane, fwd_lane, bp_format], ...}; bp_format 0 FP32
// windows, 1 interleaved pairs, 2 planar pairs, 3 FP16 pairs in mixed precision).  MTR_AUTOTUNE=0 disables
// tuning (depths 8 and 16, lane axis by slope, FP32 windows);
// MTR_FORCE_DEPTHS=bp,fwd[,bp_lane,fwd_lane[,bp_format]] pins the choice;
// MTR_AUTOTUNE_LOG=1 prints every candidate's time to stderr.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <functional>
#include <iterator>
#include <map>
#include <mutex>
#include <sstream>
#include <string>

#include "mtr_internal.h"
#include "mtr_runtime.h"

namespace mtr {
namespace {

struct Choice {
  int bp_nz = 8, fwd_nz = 16, bp_lane = -1, fwd_lane = -1;
  int bp_pairs = 0;  // SIRT update window format: 0 FP32, 1 interleaved residual pairs, 2 planar pairs
};

std::mutex g_mu;
std::map<std::string, Choice> g_cache;
bool g_loaded = false;

const char* cache_path() {
  const char* p = std::getenv("MTR_AUTOTUNE_CACHE");
  return (p && *p) ? p : nullptr;
}

void load_file() {
  if (g_loaded) return;
  g_loaded = true;
  const char* path = cache_path();
  if (!path) return;
  std::ifstream f(path);
  if (!f) return;
  std::stringstream ss;
  ss << f.rdbuf();
  const std::string s = ss.str();
  // minimal parser for {"key": [a, b, c, d], ...} as written by save_file()
  size_t i = 0;
  while ((i = s.find('"', i)) != std::string::npos) {
    const size_t j = s.find('"', i + 1);
    if (j == std::string::npos) break;
    const std::string key = s.substr(i + 1, j - i - 1);
    const size_t lb = s.find('[', j), rb = s.find(']', j);
    if (lb == std::string::npos || rb == std::string::npos) break;
    Choice c;
    if (std::sscanf(s.c_str() + lb, "[%d , %d , %d , %d , %d]", &c.bp_nz, &c.fwd_nz, &c.bp_lane, &c.fwd_lane,
                    &c.bp_pairs) == 5)
      g_cache[key] = c;
    i = rb + 1;
  }
}

void save_file() {
  const char* path = cache_path();
  if (!path) return;
  std::ofstream f(path, std::ios::trunc);
  if (!f) return;
  f << "{\n";
  size_t n = 0;
  for (const auto& kv : g_cache)
    f << "  \"" << kv.first << "\": [" << kv.second.bp_nz << ", " << kv.second.fwd_nz << ", " << kv.second.bp_lane
      << ", " << kv.second.fwd_lane << ", " << kv.second.bp_pairs << "]" << (++n < g_cache.size() ? ",\n" : "\n");
  f << "}\n";
}

std::string geometry_key(const AxisState& a, const VolDev& v, int precision) {
  double m[6] = {0, 0, 0, 0, 0, 0};
  bool bz0 = true;
  for (int k = 0; k < a.A; ++k) {
    for (int c = 0; c < 3; ++c) m[c] = std::max(m[c], std::fabs(a.hxc[4 * k + 1 + c]));
    for (int c = 0; c < 3; ++c) m[3 + c] = std::max(m[3 + c], std::fabs(a.hyc[4 * k + 1 + c]));
    if (a.hyc[4 * k + 3] != 0.0) bz0 = false;
  }
  char buf[256];
  // the trailing tag names the timing method, so choices cached by an older one are not reused
  std::snprintf(buf, sizeof(buf), "p%dx%dx%d_v%dx%dx%d_m%.2f,%.2f,%.2f,%.2f,%.2f,%.2f_z%d_prec%d_t8", a.PX, a.PY,
                a.A, v.NX, v.NY, v.NZ, m[0], m[1], m[2], m[3], m[4], m[5], bz0 ? 0 : 1, precision);
  return buf;
}

// Times every candidate launch and returns the index of the fastest (-1 if
// none ran).  Each candidate is launched once untimed, then the candidates
// are timed round-robin for kRounds rounds and each keeps its minimum, so a
// clock ramp during tuning does not favour the candidates timed last.
constexpr int kRounds = 3;
int fastest(cudaStream_t st, const std::vector<std::function<cudaError_t()>>& cands, const char* log_to = nullptr,
            const std::vector<std::string>* what = nullptr) {
  const size_t n = cands.size();
  std::vector<float> best(n, 1e30f);
  std::vector<bool> ok(n, false);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    cudaGetLastError();
    return -1;
  }
  for (size_t i = 0; i < n; ++i) ok[i] = cands[i]() == cudaSuccess;  // warm-up: module load, attributes
  cudaGetLastError();
  for (int r = 0; r < kRounds; ++r)
    for (size_t i = 0; i < n; ++i) {
      if (!ok[i]) continue;
      float ms = 0.f;
      cudaEventRecord(e0, st);
      const cudaError_t e = cands[i]();
      cudaEventRecord(e1, st);
      if (e != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
          cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
        ok[i] = false;
        cudaGetLastError();
        continue;
      }
      best[i] = std::min(best[i], ms);
    }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  int arg = -1;
  for (size_t i = 0; i < n; ++i)
    if (ok[i] && (arg < 0 || best[i] < best[arg])) arg = (int)i;
  if (log_to) {
    for (size_t i = 0; i < n; ++i)
      std::fprintf(stderr, "mtr autotune %s %s %s: %.4f ms%s\n", log_to, what ? (*what)[i].c_str() : "", ok[i] ? "" : "failed",
                   ok[i] ? best[i] : 0.f, (int)i == arg ? "  <- chosen" : "");
  }
  return arg;
}

// MTR_AUTOTUNE_LOG=1 prints every candidate's best time to stderr.
bool autotune_log() {
  const char* e = std::getenv("MTR_AUTOTUNE_LOG");
  return e && e[0] == '1';
}

}  // namespace

bool autotune_enabled() {
  const char* e = std::getenv("MTR_AUTOTUNE");
  return !(e && e[0] == '0');
}

// Chooses a.plan (SIRT back-projection over r) and a.fplan (forward splat
// over s) for one axis and encodes the matching tensor maps.  Leaves s zeroed.
bool tune_axis(mtr_context* ctx, AxisState& a, const VolDev& v, int precision, float* scratch_vol,
               float* scratch_cbp, void* scratch_copy, int* err) {
  const int copy_kind = precision == MTR_PREC_MIXED_BF16 ? 1 : precision == MTR_PREC_MIXED_FP16 ? 2 : 0;
  const std::string key = geometry_key(a, v, precision);
  Choice ch;
  bool known = false;
  if (const char* f = std::getenv("MTR_FORCE_DEPTHS")) {
    Choice c;
    const int n = std::sscanf(f, "%d,%d,%d,%d,%d", &c.bp_nz, &c.fwd_nz, &c.bp_lane, &c.fwd_lane, &c.bp_pairs);
    if (n >= 2) {
      if (n < 4) c.bp_lane = c.fwd_lane = -1;
      if (n < 5) c.bp_pairs = 0;
      ch = c;
      known = true;
    }
  }
  if (!known) {
    std::lock_guard<std::mutex> lock(g_mu);
    load_file();
    auto it = g_cache.find(key);
    if (it != g_cache.end()) {
      ch = it->second;
      known = true;
    }
  }
  // Candidates are timed over a Z-slab of the frame with enough bricks for
  // 8 waves of the deepest tile (32 planes, 3 CTAs per SM), at least 32
  // planes: a launch's cost grows with its planes, but the ranking of tiles
  // stays the frame's only while no tile runs a partly filled last wave.
  VolDev tv = v;
  {
    const long long cols = (long long)((v.NX + 31) / 32) * ((v.NY + 7) / 8);  // bricks per 32-plane layer
    const long long layers = (8LL * ctx->num_sms * 3 + cols - 1) / cols;
    tv.NZ = (int)std::min<long long>(v.NZ, 32 * std::max(1LL, layers));
  }
  const int z0 = tv.Zs, z1 = tv.Zs + tv.NZ;
  if (!known && autotune_enabled()) {
    // Non-zero weight sums, so that every candidate's SIRT epilogue reads and
    // writes the volume as a real run does (with zeros it would skip the
    // update, hiding the cost of strided lanes-along-Y stores).
    launch_fill(scratch_cbp, (long long)tv.NX * tv.NY * tv.NZ, 1.f, ctx->stream);
    // back-projection candidates: window format x depth x lane axis
    std::vector<std::function<cudaError_t()>> cands;
    std::vector<Choice> what;
    std::vector<BpPlan> bps;
    std::vector<CUtensorMap> bmaps;
    // (the candidates keep pointers into these: no reallocation)
    // (FP16 residual pairs only in mixed precision)
    const int n_fmt = copy_kind != 0 ? 4 : 3;
    bps.reserve(12 * std::size(kBpDepths));  // formats x 3 lane layouts x the depths
    bmaps.reserve(12 * std::size(kBpDepths));
    for (int fmt = 0; fmt < n_fmt; ++fmt)
      for (int lane = 0; lane < 3; ++lane)
        for (int nz : kBpDepths) {
          BpPlan p = plan_backproject(a.hxc, a.hyc, a.A, fmt, nz, lane);
          CUtensorMap m;
          if (!p.ok || !encode_residual_map(&m, a, p)) continue;
          bps.push_back(p);
          bmaps.push_back(m);
          const BpPlan* pp = &bps.back();
          const CUtensorMap* mp = &bmaps.back();
          cands.push_back([=, &a, &tv] {
            return launch_backproject_tma<float>(*mp, *pp, a.dev(), tv, 1, 0.5f, scratch_vol, scratch_cbp,
                                                 scratch_copy, copy_kind, z0, z1, err, ctx->stream);
          });
          Choice c;
          c.bp_nz = nz;
          c.bp_lane = lane;
          c.bp_pairs = fmt;
          what.push_back(c);
        }
    const bool log = autotune_log();
    std::vector<std::string> labels;
    char lb[96];
    for (const Choice& c : what) {
      std::snprintf(lb, sizeof(lb), "bp fmt %d lane %d depth %d", c.bp_pairs, c.bp_lane, c.bp_nz);
      labels.push_back(lb);
    }
    int k = fastest(ctx->stream, cands, log ? key.c_str() : nullptr, &labels);
    if (k >= 0) {
      ch.bp_nz = what[k].bp_nz;
      ch.bp_lane = what[k].bp_lane;
      ch.bp_pairs = what[k].bp_pairs;
    }
    // forward candidates
    cands.clear();
    what.clear();
    std::vector<FwdPlan> fps;
    std::vector<CUtensorMap> fmaps;
    fps.reserve(9);
    fmaps.reserve(9);
    for (int lane = 0; lane < 3; ++lane)
      for (int nz : kFwdDepths) {
        FwdPlan p = plan_forward(a.hxc, a.hyc, a.A, a.PX, a.PY, a.pitch, nz, lane);
        CUtensorMap m;
        if (!p.ok || p.nz != nz || !encode_tensor_map_3d(&m, a.s.p, false, a.pitch, a.pitch, a.PY, a.A, p.WX, p.WY))
          continue;
        fps.push_back(p);
        fmaps.push_back(m);
        const FwdPlan* pp = &fps.back();
        const CUtensorMap* mp = &fmaps.back();
        cands.push_back([=, &a, &tv] {
          if (copy_kind == 1)
            return launch_forward_tma<__nv_bfloat16>(*mp, *pp, a.dev(), tv,
                                                     static_cast<const __nv_bfloat16*>(scratch_copy), z0, z1, err,
                                                     ctx->stream);
          if (copy_kind == 2)
            return launch_forward_tma<__half>(*mp, *pp, a.dev(), tv, static_cast<const __half*>(scratch_copy), z0, z1,
                                              err, ctx->stream);
          return launch_forward_tma<float>(*mp, *pp, a.dev(), tv, scratch_vol, z0, z1, err, ctx->stream);
        });
        Choice c;
        c.fwd_nz = nz;
        c.fwd_lane = lane;
        what.push_back(c);
      }
    labels.clear();
    for (const Choice& c : what) {
      std::snprintf(lb, sizeof(lb), "fwd lane %d depth %d", c.fwd_lane, c.fwd_nz);
      labels.push_back(lb);
    }
    k = fastest(ctx->stream, cands, log ? key.c_str() : nullptr, &labels);
    if (k >= 0) {
      ch.fwd_nz = what[k].fwd_nz;
      ch.fwd_lane = what[k].fwd_lane;
    }
    std::lock_guard<std::mutex> lock(g_mu);
    g_cache[key] = ch;
    save_file();
  }
  // the timing runs wrote into s and the tuner's scratch: restore the zeros
  cudaMemsetAsync(a.s.p, 0, (size_t)a.np * 4, ctx->stream);
  a.plan = plan_backproject(a.hxc, a.hyc, a.A, std::min(std::max(ch.bp_pairs, 0), copy_kind != 0 ? 3 : 2), ch.bp_nz,
                            ch.bp_lane);
  a.tma = a.plan.ok && encode_residual_map(&a.map_r, a, a.plan);
  a.fplan = plan_forward(a.hxc, a.hyc, a.A, a.PX, a.PY, a.pitch, ch.fwd_nz, ch.fwd_lane);
  a.ftma = a.fplan.ok &&
           encode_tensor_map_3d(&a.map_s, a.s.p, false, a.pitch, a.pitch, a.PY, a.A, a.fplan.WX, a.fplan.WY) &&
           encode_tensor_map_3d(&a.map_cf, a.cf.p, false, a.pitch, a.pitch, a.PY, a.A, a.fplan.WX, a.fplan.WY);
  return a.tma || a.ftma;
}

}  // namespace mtr
