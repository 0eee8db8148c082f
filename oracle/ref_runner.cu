// Runs the reference's OWN CUDA kernels (FunctionOnGPU.cu compiled, unmodified,
// into oracle/_ref/ref_kernels.cubin by oracle/build.py) on the GPU, driven by a
// restatement of the reference's host logic with one rank per tilt axis.
//
// TEST INFRASTRUCTURE ONLY: this pins the CPU oracle and the product to the
// reference's actual arithmetic (FP64 coordinates, float atomics).  It is
// never linked into libmtr.
//
// Host logic restated here:
//   ComputeInitialModel   FunctionOnGPU.cu:138-179 (device slab zeroed first:
//                         the reference adds into a fresh cudaMalloc)
//   runSIRTOnGPU          FunctionOnGPU.cu:182-266 (1-rank communicator:
//                         reductions and broadcasts are identities)
//   initialZdata          FunctionOnGPU.cu:291-313
//   runMaceOnCPU          MultiAxis.cpp:33-38
//   reconstructModel      MultiAxis.cpp:40-71 with numprocs = K
//   initial model         MultiAxis.cpp:172-200 (float sum over axes)
// Launch shape: block (8,8,8), grid ceil(X/8) x ceil(Y/8) x ceil(Z/8)
// (ReadAndInitialOptions.h:35-37, FunctionOnGPU.cu:162-163).
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace {

// Same layout as the reference's ProjectionSize / VolumeSize
// (MrcFileIOBaseFunction.h:57-78), passed by value to its kernels.
struct RefPrj { int X, Y, AngN; };
struct RefVol { int Xstart, Xend, Ystart, Yend, Zstart, Zend, X, Y, Z; };

cudaLibrary_t g_lib = nullptr;
cudaKernel_t k_bp = nullptr, k_fwd = nullptr, k_sirt = nullptr, k_z = nullptr;
std::string g_err;

int fail(const char* what, cudaError_t e) {
  g_err = std::string(what) + ": " + cudaGetErrorString(e);
  return 1;
}

#define RR(call) do { cudaError_t _e = (call); if (_e != cudaSuccess) return fail(#call, _e); } while (0)

int launch(cudaKernel_t k, dim3 grid, dim3 block, void** args) {
  RR(cudaLaunchKernel((const void*)k, grid, block, args, 0, 0));
  RR(cudaGetLastError());
  return 0;
}

dim3 grid_of(int X, int Y, int Z) { return dim3((X + 7) / 8, (Y + 7) / 8, (Z + 7) / 8); }

struct DevAxis {
  double* xc = nullptr;
  double* yc = nullptr;
  float* prj = nullptr;
  ~DevAxis() { cudaFree(xc); cudaFree(yc); cudaFree(prj); }
};

int upload_axis(const RefPrj& p, const double* xc, const double* yc, const float* data, DevAxis& d) {
  // The reference sizes the coefficient buffers AngN*10 entries (FunctionOnGPU.cu:145).
  const size_t cb = sizeof(double) * (size_t)p.AngN * 10;
  std::vector<double> hx(p.AngN * 10, 0.0), hy(p.AngN * 10, 0.0);
  std::memcpy(hx.data(), xc, sizeof(double) * 4 * p.AngN);
  std::memcpy(hy.data(), yc, sizeof(double) * 4 * p.AngN);
  RR(cudaMalloc(&d.xc, cb));
  RR(cudaMalloc(&d.yc, cb));
  RR(cudaMalloc(&d.prj, sizeof(float) * (size_t)p.X * p.Y * p.AngN));
  RR(cudaMemcpy(d.xc, hx.data(), cb, cudaMemcpyHostToDevice));
  RR(cudaMemcpy(d.yc, hy.data(), cb, cudaMemcpyHostToDevice));
  RR(cudaMemcpy(d.prj, data, sizeof(float) * (size_t)p.X * p.Y * p.AngN, cudaMemcpyHostToDevice));
  return 0;
}

int wbp(const RefPrj& p, const RefVol& v, DevAxis& d, int z0, int z1, float* out) {
  const size_t n = (size_t)v.X * v.Y * (z1 - z0);
  float* dm = nullptr;
  RR(cudaMalloc(&dm, n * 4));
  RR(cudaMemset(dm, 0, n * 4));
  RefPrj pp = p;
  RefVol vv = v;
  int a6 = z0, a7 = z1;
  void* args[] = {&pp, &vv, &d.xc, &d.yc, &d.prj, &dm, &a6, &a7};
  int rc = launch(k_bp, grid_of(v.X, v.Y, z1 - z0), dim3(8, 8, 8), args);
  if (!rc) rc = cudaMemcpy(out, dm, n * 4, cudaMemcpyDeviceToHost) != cudaSuccess;
  cudaFree(dm);
  if (rc && g_err.empty()) g_err = "wbp copy";
  return rc;
}

int sirt(const RefPrj& p, const RefVol& v, DevAxis& d, const float* b, int z0, int z1, int n_inner, float step,
         float* slab, double* norms) {
  const size_t np = (size_t)p.X * p.Y * p.AngN;
  const size_t ns = (size_t)v.X * v.Y * (z1 - z0);
  float *ds = nullptr, *dc = nullptr, *dm = nullptr;
  RR(cudaMalloc(&ds, np * 4));
  RR(cudaMalloc(&dc, np * 4));
  RR(cudaMalloc(&dm, ns * 4));
  RR(cudaMemcpy(dm, slab, ns * 4, cudaMemcpyHostToDevice));
  std::vector<float> hs(np), hc(np);
  RefPrj pp = p;
  RefVol vv = v;
  int a7 = z0, a8 = z1;
  double lam = (double)step;  // opts->sirt_step (float) passed as double
  for (int it = 0; it < n_inner; ++it) {
    RR(cudaMemset(ds, 0, np * 4));
    RR(cudaMemset(dc, 0, np * 4));
    void* fa[] = {&pp, &vv, &d.xc, &d.yc, &ds, &dc, &dm, &a7, &a8};
    if (launch(k_fwd, grid_of(v.X, v.Y, z1 - z0), dim3(8, 8, 8), fa)) return 1;
    RR(cudaMemcpy(hc.data(), dc, np * 4, cudaMemcpyDeviceToHost));
    RR(cudaMemcpy(hs.data(), ds, np * 4, cudaMemcpyDeviceToHost));
    double n2 = 0.0;
    for (size_t k = 0; k < np; ++k) {  // FunctionOnGPU.cu:230-234
      if (hc[k] != 0) hs[k] /= hc[k];
      hs[k] = b[k] - hs[k];
      n2 += (double)hs[k] * hs[k];
    }
    if (norms) norms[it] = n2;
    RR(cudaMemcpy(ds, hs.data(), np * 4, cudaMemcpyHostToDevice));
    void* ba[] = {&pp, &vv, &d.xc, &d.yc, &ds, &dm, &a7, &a8, &lam};
    if (launch(k_sirt, grid_of(v.X, v.Y, z1 - z0), dim3(8, 8, 8), ba)) return 1;
  }
  RR(cudaMemcpy(slab, dm, ns * 4, cudaMemcpyDeviceToHost));
  cudaFree(ds);
  cudaFree(dc);
  cudaFree(dm);
  return 0;
}

}  // namespace

extern "C" {

const char* rr_last_error(void) { return g_err.c_str(); }

// Load the cubin built from the reference's FunctionOnGPU.cu.
int rr_load(const char* cubin_path) {
  if (g_lib) return 0;
  RR(cudaLibraryLoadFromFile(&g_lib, cubin_path, nullptr, nullptr, 0, nullptr, nullptr, 0));
  RR(cudaLibraryGetKernel(&k_bp, g_lib, "_Z13backProjOnGPU14ProjectionSize10VolumeSizePdS1_PfS2_ii"));
  RR(cudaLibraryGetKernel(&k_fwd, g_lib, "_Z14computeDivisor14ProjectionSize10VolumeSizePdS1_PfS2_S2_ii"));
  RR(cudaLibraryGetKernel(&k_sirt, g_lib, "_Z17sirtBackProjOnGPU14ProjectionSize10VolumeSizePdS1_PfS2_iid"));
  RR(cudaLibraryGetKernel(&k_z, g_lib, "_Z13initialZOnGPU10VolumeSizePfS0_S0_"));
  return 0;
}

// ComputeInitialModel for one axis over [z0,z1).
int rr_wbp(const int* prj3, const int* vol9, const double* xc, const double* yc, const float* data, int z0, int z1,
           float* out) {
  RefPrj p{prj3[0], prj3[1], prj3[2]};
  RefVol v;
  std::memcpy(&v, vol9, sizeof(v));
  DevAxis d;
  if (upload_axis(p, xc, yc, data, d)) return 1;
  return wbp(p, v, d, z0, z1, out);
}

// runSIRTOnGPU for one axis, n_inner iterations on slab (in place).
int rr_sirt(const int* prj3, const int* vol9, const double* xc, const double* yc, const float* data, int z0, int z1,
            int n_inner, float step, float* slab, double* norms) {
  RefPrj p{prj3[0], prj3[1], prj3[2]};
  RefVol v;
  std::memcpy(&v, vol9, sizeof(v));
  DevAxis d;
  if (upload_axis(p, xc, yc, data, d)) return 1;
  return sirt(p, v, d, data, z0, z1, n_inner, step, slab, norms);
}

// Whole reconstruction with K axes (one rank each): WBP sum init, n_outer MACE
// iterations, output w_avg.  prj3: 3*K ints; xcs/ycs/datas: K pointers.
int rr_reconstruct(int K, const int* prj3, const double* const* xcs, const double* const* ycs,
                   const float* const* datas, const int* vol9, int n_outer, int n_inner, float sirt_step,
                   float mace_step, float* out_wavg) {
  RefVol v;
  std::memcpy(&v, vol9, sizeof(v));
  const size_t nv = (size_t)v.X * v.Y * v.Z;
  std::vector<DevAxis> dev(K);
  std::vector<RefPrj> prj(K);
  std::vector<float> init(nv, 0.f), x0(nv);
  for (int k = 0; k < K; ++k) {
    prj[k] = RefPrj{prj3[3 * k], prj3[3 * k + 1], prj3[3 * k + 2]};
    if (upload_axis(prj[k], xcs[k], ycs[k], datas[k], dev[k])) return 1;
    if (wbp(prj[k], v, dev[k], v.Zstart, v.Zend, x0.data())) return 1;
    for (size_t i = 0; i < nv; ++i) init[i] = init[i] + x0[i];
  }
  std::vector<std::vector<float>> w(K, init);
  std::vector<float> wavg(init), z(nv);
  float *dw = nullptr, *da = nullptr, *dz = nullptr;
  RR(cudaMalloc(&dw, nv * 4));
  RR(cudaMalloc(&da, nv * 4));
  RR(cudaMalloc(&dz, nv * 4));
  for (int it = 0; it < n_outer; ++it) {
    for (int k = 0; k < K; ++k) {
      // initialZdata on the GPU (FunctionOnGPU.cu:291-313)
      RR(cudaMemcpy(dw, w[k].data(), nv * 4, cudaMemcpyHostToDevice));
      RR(cudaMemcpy(da, wavg.data(), nv * 4, cudaMemcpyHostToDevice));
      RefVol vv = v;
      void* za[] = {&vv, &dw, &da, &dz};
      if (launch(k_z, grid_of(v.X, v.Y, v.Z), dim3(8, 8, 8), za)) return 1;
      RR(cudaMemcpy(z.data(), dz, nv * 4, cudaMemcpyDeviceToHost));
      std::vector<float> vk(z);
      if (sirt(prj[k], v, dev[k], datas[k], v.Zstart, v.Zend, n_inner, sirt_step, vk.data(), nullptr)) return 1;
      float* wk = w[k].data();
      for (size_t i = 0; i < nv; ++i) wk[i] = mace_step * (2 * vk[i] - z[i]) + (1 - mace_step) * wk[i];
    }
    for (size_t i = 0; i < nv; ++i) {
      float acc = 0.f;
      for (int k = 0; k < K; ++k) acc = acc + w[k][i];
      wavg[i] = acc / K;
    }
  }
  cudaFree(dw);
  cudaFree(da);
  cudaFree(dz);
  std::memcpy(out_wavg, wavg.data(), nv * 4);
  return 0;
}

}  // extern "C"
