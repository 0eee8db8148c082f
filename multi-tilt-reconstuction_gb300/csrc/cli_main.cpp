// mtr_multiaxis: drop-in replacement for the reference's MultiAxis executable
// (MultiAxis.cpp:101-230) on one GPU.  Same options, same inputs (MRC stacks
// + TXBR maps, one pair per tilt axis), same output (MRC float32 volume of
// the MACE consensus w_avg, x fastest).  Where the reference needs one MPI
// rank per axis slab, this runs every axis on one device.
//
//   mtr_multiaxis -i K,a.st,...,a.txbr,... -o out.mrc [-n 5] [-s 0.5] [-m 0.7]
//                 [--inner 10] [--precision fp32|bf16|fp16]
//   mtr_multiaxis tilts2txbr TLT OUT DET_X DET_Y XS XE YS YE ZS ZE [PHI_DEG [XF]]
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/mtr.h"

namespace {

void help() {
  std::printf(
      "mtr_multiaxis - multi-axis WBP/SIRT/MACE reconstruction on one GPU\n"
      "  -i K,st_1,...,st_K,txbr_1,...,txbr_K   projection stacks (MRC) and TXBR maps\n"
      "  -o FILE                                output MRC volume (float32)\n"
      "  -n N                                   MACE iterations (default 5)\n"
      "  -s F                                   SIRT relaxation (default 0.5)\n"
      "  -m F                                   MACE step rho (default 0.7)\n"
      "  -x/-y/-z N                             block-size hints (accepted, default 8)\n"
      "  --inner N                              SIRT iterations per MACE iteration (default 10)\n"
      "  --precision fp32|bf16|fp16             storage precision (default fp32)\n"
      "  -h                                     this help\n");
}

int fail(const char* what, mtr_status s, const char* detail = nullptr) {
  std::fprintf(stderr, "mtr_multiaxis: %s: %s%s%s\n", what, mtr_status_string(s), detail ? " - " : "",
               detail ? detail : "");
  return 1;
}

// mtr_multiaxis tilts2txbr TLT OUT DET_X DET_Y XS XE YS YE ZS ZE [PHI_DEG [XF]]
// The linear maps of a parallel-beam tilt series (IMOD .tlt angles, optional
// .xf alignments, tilt axis at in-plane angle PHI) over the volume frame
// [XS,XE) x [YS,YE) x [ZS,ZE), written as a TXBR file for -i.
int tilts_to_txbr(int argc, char** argv) {
  if (argc < 12 || argc > 14) {
    std::fprintf(stderr, "usage: mtr_multiaxis tilts2txbr TLT OUT DET_X DET_Y XS XE YS YE ZS ZE [PHI_DEG [XF]]\n");
    return 2;
  }
  const int cap = 100000;
  std::vector<double> tilt((size_t)cap);
  int n = 0;
  mtr_status s = mtr_tlt_read(argv[2], tilt.data(), cap, &n);
  if (s != MTR_OK) return fail("read .tlt", s, argv[2]);
  std::vector<mtr_xf> xf;
  if (argc == 14) {
    xf.resize((size_t)cap);
    int nx = 0;
    s = mtr_xf_read(argv[13], xf.data(), cap, &nx);
    if (s != MTR_OK) return fail("read .xf", s, argv[13]);
    if (nx != n) return fail(".xf", MTR_ERR_FORMAT, "one transform per tilt angle is needed");
  }
  int v[8];
  for (int i = 0; i < 8; ++i) {
    char* end = nullptr;
    v[i] = (int)std::strtol(argv[4 + i], &end, 10);
    if (!end || *end) return fail("arguments", MTR_ERR_INVALID_ARGUMENT, argv[4 + i]);
  }
  const double phi = argc >= 13 ? std::strtod(argv[12], nullptr) : 0.0;
  mtr_volume_size vol{v[2], v[3], v[4], v[5], v[6], v[7], v[3] - v[2], v[5] - v[4], v[7] - v[6]};
  std::vector<double> xc(4 * (size_t)n), yc(4 * (size_t)n);
  s = mtr_geometry_from_tilts(n, tilt.data(), xf.empty() ? nullptr : xf.data(), phi, v[0], v[1], vol, xc.data(),
                              yc.data());
  if (s != MTR_OK) return fail("geometry", s);
  s = mtr_txbr_write(argv[3], n, xc.data(), yc.data(), vol);
  if (s != MTR_OK) return fail("write TXBR", s, argv[3]);
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc > 1 && std::strcmp(argv[1], "tilts2txbr") == 0) return tilts_to_txbr(argc, argv);
  mtr_options opt;
  mtr_status s = mtr_parse_options(argc, argv, &opt);
  if (s != MTR_OK) {
    help();
    return fail("options", s);
  }
  if (opt.help) {
    help();
    return 0;
  }
  if (opt.number_tilt < 1 || opt.out_path[0] == '\0') {
    help();
    return fail("options", MTR_ERR_INVALID_ARGUMENT, "-i and -o are required");
  }
  const int K = opt.number_tilt;
  std::vector<std::vector<float>> data(K);
  std::vector<std::vector<double>> xc(K), yc(K);
  std::vector<mtr_axis> axes(K);
  mtr_volume_size vol;
  mtr_volume_size_empty(&vol);
  for (int k = 0; k < K; ++k) {
    mtr_mrc_header h;
    s = mtr_mrc_read_header(opt.mrc_path[k], &h);
    if (s != MTR_OK) return fail("read MRC header", s, opt.mrc_path[k]);
    if (h.nx <= 0 || h.ny <= 0 || h.nz <= 0) return fail("MRC header", MTR_ERR_FORMAT, opt.mrc_path[k]);
    const long long n = (long long)h.nx * h.ny * h.nz;
    data[k].resize((size_t)n);
    s = mtr_mrc_read_stack(opt.mrc_path[k], data[k].data(), n);
    if (s != MTR_OK) return fail("read MRC data", s, opt.mrc_path[k]);
    const int cap = 4 * h.nz;
    xc[k].assign((size_t)cap, 0.0);
    yc[k].assign((size_t)cap, 0.0);
    int nxc = 0, nyc = 0;
    s = mtr_txbr_read(opt.txbr_path[k], xc[k].data(), yc[k].data(), cap, &nxc, &nyc, &vol);
    if (s != MTR_OK) return fail("read TXBR", s, opt.txbr_path[k]);
    if (nxc != cap || nyc != cap)
      return fail("TXBR", MTR_ERR_FORMAT, "coefficient count must be 4 per section of the stack");
    axes[k].prj = mtr_projection_size{h.nx, h.ny, h.nz};
    axes[k].x_coef = xc[k].data();
    axes[k].y_coef = yc[k].data();
    axes[k].prj_data = data[k].data();
  }
  mtr_params p;
  mtr_params_default(&p);
  p.iter_times = opt.iter_times;
  p.sirt_inner = opt.sirt_inner;
  p.sirt_step = opt.sirt_step;
  p.mace_step = opt.mace_step;
  p.precision = opt.precision;
  mtr_context* ctx = nullptr;
  s = mtr_context_create(-1, &ctx);
  if (s != MTR_OK) return fail("CUDA context", s);
  std::vector<float> out((size_t)vol.X * vol.Y * vol.Z);
  const auto t0 = std::chrono::steady_clock::now();
  s = mtr_reconstruct(ctx, K, axes.data(), vol, &p, out.data());
  const double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (s != MTR_OK) {
    const int rc = fail("reconstruct", s, mtr_context_last_error(ctx));
    mtr_context_destroy(ctx);
    return rc;
  }
  mtr_context_destroy(ctx);
  std::printf("Total time: %f s\n", sec);
  s = mtr_mrc_write_volume(opt.out_path, vol, out.data());
  if (s != MTR_OK) return fail("write MRC", s, opt.out_path);
  return 0;
}
