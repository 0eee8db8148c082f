// CPU oracle for the multi-axis WBP -> SIRT -> MACE path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the oracle: the parity tests, the
// smoke check and the CPU-baseline leg of the benchmark call it to produce the
// expected answer.  It is never linked into the product library and the
// product never falls back to it.
//
// It restates, in plain C++ with OpenMP, the arithmetic of the reference
// program (Autumn1998/Multi-tilt-Reconstuction):
//   projection map        FunctionOnGPU.cu:12-25   (computeWeight)
//   bilinear splat        FunctionOnGPU.cu:27-52   (Reproj) + :316-333 (computeDivisor)
//   bilinear gather       FunctionOnGPU.cu:54-79   (BilinearValue)
//   WBP                   FunctionOnGPU.cu:82-109  (backProjOnGPU)
//   SIRT update           FunctionOnGPU.cu:111-135 (sirtBackProjOnGPU)
//   SIRT inner loop       FunctionOnGPU.cu:182-266 (runSIRTOnGPU; residual :228-236)
//   MACE z / w updates    FunctionOnGPU.cu:268-288, MultiAxis.cpp:33-38
//   MACE outer loop       MultiAxis.cpp:40-71      (reconstructModel)
//   initial model (sum)   MultiAxis.cpp:172-200
//   Z-slab split          MultiAxis.cpp:13-31      (divideSlice)
//
// Two precision modes:
//   mode 0 "reference-faithful": FP64 coordinates and gather sums, splat
//          products rounded to float and accumulated in float, residual and
//          MACE in float, exactly as the reference's kernels and host loops do
//          (the reference's atomics add in an unspecified order; here the
//          order is voxel-index order within each angle plane).
//   mode 1 "FP64": every quantity in double.  This is the error reference for
//          reduced-precision runs.
//
// Build: g++ -O2 -fopenmp -ffp-contract=off -shared -fPIC (see oracle/build.py).

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <omp.h>

extern "C" {

typedef struct { int Xstart, Xend, Ystart, Yend, Zstart, Zend, X, Y, Z; } orc_vol;
typedef struct { int X, Y, AngN; } orc_prj;

}  // extern "C"

namespace {

struct Tap {
  int ix, iy;
  double dx, dy;
};

// FunctionOnGPU.cu:12-25.  Affine voxel -> detector map, 1-based -> 0-based.
inline Tap map_voxel(const double* xc, const double* yc, int ang, int X, int Y, int Z) {
  const int k = 4 * ang;
  const double x = xc[k] + xc[k + 1] * X + xc[k + 2] * Y + xc[k + 3] * Z - 1;
  const double y = yc[k] + yc[k + 1] * X + yc[k + 2] * Y + yc[k + 3] * Z - 1;
  Tap t;
  t.ix = (int)std::floor(x);
  t.iy = (int)std::floor(y);
  t.dx = x - t.ix;
  t.dy = y - t.iy;
  return t;
}

inline bool inside(int ix, int iy, const orc_prj& p) {
  return ix >= 0 && ix < p.X && iy >= 0 && iy < p.Y;
}

// FunctionOnGPU.cu:54-79 + the angle loops of :97-101 / :126-130.
// Sums over all angles in double, as the reference kernels do.
template <typename P>
inline void gather_voxel(const orc_prj& prj, const double* xc, const double* yc, const P* data,
                         int X, int Y, int Z, double& s, double& c) {
  s = 0.0;
  c = 0.0;
  const long long plane = (long long)prj.X * prj.Y;
  for (int a = 0; a < prj.AngN; ++a) {
    const Tap t = map_voxel(xc, yc, a, X, Y, Z);
    const P* img = data + plane * a;
    const double w00 = (1 - t.dx) * (1 - t.dy), w10 = t.dx * (1 - t.dy);
    const double w01 = (1 - t.dx) * t.dy, w11 = t.dx * t.dy;
    if (inside(t.ix, t.iy, prj)) { s += w00 * img[t.ix + (long long)t.iy * prj.X]; c += w00; }
    if (inside(t.ix + 1, t.iy, prj)) { s += w10 * img[t.ix + 1 + (long long)t.iy * prj.X]; c += w10; }
    if (inside(t.ix, t.iy + 1, prj)) { s += w01 * img[t.ix + (long long)(t.iy + 1) * prj.X]; c += w01; }
    if (inside(t.ix + 1, t.iy + 1, prj)) { s += w11 * img[t.ix + 1 + (long long)(t.iy + 1) * prj.X]; c += w11; }
  }
}

// Voxel-driven bilinear splat of a slab (FunctionOnGPU.cu:27-52, 316-333).
// S is the accumulator type: float in mode 0 (the reference's float atomics),
// double in mode 1.  Parallel over angles: each angle plane is owned by one
// thread, so the result does not depend on the thread count.
template <typename V, typename S>
void splat(const orc_prj& prj, const orc_vol& vol, const double* xc, const double* yc,
           const V* slab, int z0, int z1, S* s, S* c) {
  const long long plane = (long long)prj.X * prj.Y;
#pragma omp parallel for schedule(dynamic, 1)
  for (int a = 0; a < prj.AngN; ++a) {
    S* sp = s + plane * a;
    S* cp = c + plane * a;
    for (long long i = 0; i < plane; ++i) { sp[i] = 0; cp[i] = 0; }
    for (int z = z0; z < z1; ++z)
      for (int y = vol.Ystart; y < vol.Yend; ++y)
        for (int x = vol.Xstart; x < vol.Xend; ++x) {
          const long long vi = (long long)(x - vol.Xstart) + (long long)(y - vol.Ystart) * vol.X +
                               (long long)(z - z0) * vol.X * vol.Y;
          const double v = (double)slab[vi];
          const Tap t = map_voxel(xc, yc, a, x, y, z);
          const double w00 = (1 - t.dx) * (1 - t.dy), w10 = t.dx * (1 - t.dy);
          const double w01 = (1 - t.dx) * t.dy, w11 = t.dx * t.dy;
          if (inside(t.ix, t.iy, prj)) {
            const long long n = t.ix + (long long)t.iy * prj.X;
            sp[n] += (S)(w00 * v); cp[n] += (S)w00;
          }
          if (inside(t.ix + 1, t.iy, prj)) {
            const long long n = t.ix + 1 + (long long)t.iy * prj.X;
            sp[n] += (S)(w10 * v); cp[n] += (S)w10;
          }
          if (inside(t.ix, t.iy + 1, prj)) {
            const long long n = t.ix + (long long)(t.iy + 1) * prj.X;
            sp[n] += (S)(w01 * v); cp[n] += (S)w01;
          }
          if (inside(t.ix + 1, t.iy + 1, prj)) {
            const long long n = t.ix + 1 + (long long)(t.iy + 1) * prj.X;
            sp[n] += (S)(w11 * v); cp[n] += (S)w11;
          }
        }
  }
}

// Residual (FunctionOnGPU.cu:228-236): s <- s/c where c != 0, r = b - s.
template <typename S, typename P>
double residual(long long n, const P* b, const S* s, const S* c, S* r) {
  double norm2 = 0.0;
#pragma omp parallel for reduction(+ : norm2) schedule(static)
  for (long long k = 0; k < n; ++k) {
    S sk = s[k];
    if (c[k] != 0) sk = sk / c[k];
    const S rk = (S)b[k] - sk;
    r[k] = rk;
    norm2 += (double)rk * (double)rk;
  }
  return norm2;
}

// WBP (FunctionOnGPU.cu:82-109) into a zero slab: out = s/c where c != 0.
template <typename V>
void wbp(const orc_prj& prj, const orc_vol& vol, const double* xc, const double* yc, const float* data,
         int z0, int z1, V* out) {
  const int nz = z1 - z0;
#pragma omp parallel for collapse(2) schedule(static)
  for (int z = 0; z < nz; ++z)
    for (int y = 0; y < vol.Y; ++y)
      for (int x = 0; x < vol.X; ++x) {
        double s, c;
        gather_voxel(prj, xc, yc, data, x + vol.Xstart, y + vol.Ystart, z + z0, s, c);
        const long long vi = (long long)x + (long long)y * vol.X + (long long)z * vol.X * vol.Y;
        V v = 0;
        if (c != 0.0) v = (V)(s / c);
        out[vi] = v;
      }
}

// SIRT back-projection update (FunctionOnGPU.cu:111-135).
template <typename V, typename R>
void sirt_update(const orc_prj& prj, const orc_vol& vol, const double* xc, const double* yc, const R* r,
                 int z0, int z1, double step, V* slab) {
  const int nz = z1 - z0;
#pragma omp parallel for collapse(2) schedule(static)
  for (int z = 0; z < nz; ++z)
    for (int y = 0; y < vol.Y; ++y)
      for (int x = 0; x < vol.X; ++x) {
        double s, c;
        gather_voxel(prj, xc, yc, r, x + vol.Xstart, y + vol.Ystart, z + z0, s, c);
        const long long vi = (long long)x + (long long)y * vol.X + (long long)z * vol.X * vol.Y;
        if (c != 0.0) {
          if (sizeof(V) == sizeof(float))
            slab[vi] = (V)((double)slab[vi] + (double)(float)(s / c) * step);
          else
            slab[vi] = (V)((double)slab[vi] + (s / c) * step);
        }
      }
}

// runSIRTOnGPU (FunctionOnGPU.cu:182-266) for one axis whose slab is the
// whole [z0,z1) range.  c = A*1 is identical every iteration, so it is
// accumulated once; the reference recomputes the same values each time.
template <typename V>
void sirt(const orc_prj& prj, const orc_vol& vol, const double* xc, const double* yc, const float* data,
          int z0, int z1, int n_inner, double step, V* slab, double* norms) {
  const long long np = (long long)prj.X * prj.Y * prj.AngN;
  std::vector<V> s(np), c(np), r(np);
  for (int it = 0; it < n_inner; ++it) {
    splat(prj, vol, xc, yc, slab, z0, z1, s.data(), c.data());
    const double n2 = residual(np, data, s.data(), c.data(), r.data());
    if (norms) norms[it] = n2;
    sirt_update(prj, vol, xc, yc, r.data(), z0, z1, step, slab);
  }
}

template <typename V>
void reconstruct(int K, const orc_prj* prjs, const double* const* xcs, const double* const* ycs,
                 const float* const* datas, const orc_vol& vol, int n_outer, int n_inner,
                 double sirt_step, double mace_step, double* out_wavg, double* out_w, double* norms) {
  const long long nv = (long long)vol.X * vol.Y * vol.Z;
  const int z0 = vol.Zstart, z1 = vol.Zend;
  // Initial model: sum over axes of the per-axis WBP (MultiAxis.cpp:181-200).
  std::vector<V> init(nv, (V)0), x0(nv);
  for (int k = 0; k < K; ++k) {
    wbp(prjs[k], vol, xcs[k], ycs[k], datas[k], z0, z1, x0.data());
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < nv; ++i) init[i] = init[i] + x0[i];
  }
  std::vector<std::vector<V>> w(K, init);
  std::vector<V> wavg(init), zv(nv);
  const V step = (V)mace_step;
  for (int it = 0; it < n_outer; ++it) {
    for (int k = 0; k < K; ++k) {
      V* wk = w[k].data();
      // z = 2*w_avg - w (FunctionOnGPU.cu:268-276)
#pragma omp parallel for schedule(static)
      for (long long i = 0; i < nv; ++i) zv[i] = 2 * wavg[i] - wk[i];
      std::vector<V> v(zv);
      sirt(prjs[k], vol, xcs[k], ycs[k], datas[k], z0, z1, n_inner, sirt_step, v.data(),
           norms ? norms + ((long long)it * K + k) * n_inner : nullptr);
      // w = step*(2v - z) + (1-step)*w (MultiAxis.cpp:33-38)
#pragma omp parallel for schedule(static)
      for (long long i = 0; i < nv; ++i) {
        const V t1 = 2 * v[i] - zv[i];
        const V t2 = step * t1;
        const V t3 = (1 - step) * wk[i];
        wk[i] = t2 + t3;
      }
    }
    // Consensus: sum over axes, divide by the axis count (MultiAxis.cpp:63-66).
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < nv; ++i) {
      V acc = 0;
      for (int k = 0; k < K; ++k) acc = acc + w[k][i];
      wavg[i] = acc / (V)K;
    }
  }
  for (long long i = 0; i < nv; ++i) out_wavg[i] = (double)wavg[i];
  if (out_w)
    for (int k = 0; k < K; ++k)
      for (long long i = 0; i < nv; ++i) out_w[(long long)k * nv + i] = (double)w[k][i];
}

}  // namespace

extern "C" {

int orc_num_threads(void) { return omp_get_max_threads(); }
void orc_set_threads(int n) { if (n > 0) omp_set_num_threads(n); }

// MultiAxis.cpp:13-31.
void orc_divide_slice(int myid, int N, int Z, int S, int* z_start, int* z_end) {
  const int zrem = Z % N;
  int height, start;
  if (myid < zrem) {
    height = Z / N + 1;
    start = height * myid + S;
  } else {
    height = Z / N;
    start = height * myid + zrem + S;
  }
  *z_start = start;
  *z_end = start + height;
}

// WBP of one axis over [z0,z1): out (slab, x fastest) = s/c, 0 where c == 0.
int orc_wbp(int mode, orc_prj prj, orc_vol vol, const double* xc, const double* yc, const float* data,
            int z0, int z1, double* out) {
  const long long n = (long long)vol.X * vol.Y * (z1 - z0);
  if (mode == 0) {
    std::vector<float> tmp(n);
    wbp(prj, vol, xc, yc, data, z0, z1, tmp.data());
    for (long long i = 0; i < n; ++i) out[i] = tmp[i];
  } else {
    wbp(prj, vol, xc, yc, data, z0, z1, out);
  }
  return 0;
}

// Forward splat of a slab: s = A x, c = A 1 (projection layout [AngN][Y][X]).
int orc_forward(int mode, orc_prj prj, orc_vol vol, const double* xc, const double* yc, const double* slab,
                int z0, int z1, double* s, double* c) {
  const long long nv = (long long)vol.X * vol.Y * (z1 - z0);
  const long long np = (long long)prj.X * prj.Y * prj.AngN;
  if (mode == 0) {
    std::vector<float> sl(nv), sf(np), cf(np);
    for (long long i = 0; i < nv; ++i) sl[i] = (float)slab[i];
    splat(prj, vol, xc, yc, sl.data(), z0, z1, sf.data(), cf.data());
    for (long long i = 0; i < np; ++i) { s[i] = sf[i]; c[i] = cf[i]; }
  } else {
    splat(prj, vol, xc, yc, slab, z0, z1, s, c);
  }
  return 0;
}

// Back-projection gather of a projection-space array r: s_bp = A^T r, c_bp = A^T 1
// (both over in-detector taps), as the reference's gather kernels accumulate them.
int orc_backproject(orc_prj prj, orc_vol vol, const double* xc, const double* yc, const double* r,
                    int z0, int z1, double* s_out, double* c_out) {
  const int nz = z1 - z0;
#pragma omp parallel for collapse(2) schedule(static)
  for (int z = 0; z < nz; ++z)
    for (int y = 0; y < vol.Y; ++y)
      for (int x = 0; x < vol.X; ++x) {
        double s, c;
        gather_voxel(prj, xc, yc, r, x + vol.Xstart, y + vol.Ystart, z + z0, s, c);
        const long long vi = (long long)x + (long long)y * vol.X + (long long)z * vol.X * vol.Y;
        s_out[vi] = s;
        c_out[vi] = c;
      }
  return 0;
}

// n_inner SIRT iterations of one axis on slab (in place), optional residual norms.
int orc_sirt(int mode, orc_prj prj, orc_vol vol, const double* xc, const double* yc, const float* data,
             int z0, int z1, int n_inner, double step, double* slab, double* norms) {
  const long long nv = (long long)vol.X * vol.Y * (z1 - z0);
  if (mode == 0) {
    std::vector<float> tmp(nv);
    for (long long i = 0; i < nv; ++i) tmp[i] = (float)slab[i];
    sirt(prj, vol, xc, yc, data, z0, z1, n_inner, (double)(float)step, tmp.data(), norms);
    for (long long i = 0; i < nv; ++i) slab[i] = tmp[i];
  } else {
    sirt(prj, vol, xc, yc, data, z0, z1, n_inner, step, slab, norms);
  }
  return 0;
}

// Full reconstruction: WBP sum init, n_outer MACE iterations of n_inner SIRT
// iterations per axis, consensus mean.  out_wavg receives the consensus
// volume (the reference's output); out_w (optional) the K per-axis w.
// norms (optional) receives n_outer*K*n_inner squared residual norms.
int orc_reconstruct(int mode, int K, const orc_prj* prjs, const double* const* xcs, const double* const* ycs,
                    const float* const* datas, orc_vol vol, int n_outer, int n_inner, double sirt_step,
                    double mace_step, double* out_wavg, double* out_w, double* norms) {
  if (K <= 0) return 1;
  if (mode == 0)
    reconstruct<float>(K, prjs, xcs, ycs, datas, vol, n_outer, n_inner, (double)(float)sirt_step,
                       (double)(float)mace_step, out_wavg, out_w, norms);
  else
    reconstruct<double>(K, prjs, xcs, ycs, datas, vol, n_outer, n_inner, sirt_step, mace_step, out_wavg,
                        out_w, norms);
  return 0;
}

}  // extern "C"
