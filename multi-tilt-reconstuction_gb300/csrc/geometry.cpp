// Geometry front end: per-view linear maps (the TXBR coefficient order the
// reference's readCoef consumes, MrcFileIOBaseFunction.cpp:72-134) from tilt
// angles, the tilt axis' in-plane angle and optional 2-D alignment
// transforms.  The reference has no such converter; its maps come from TxBR.
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "../../include/mtr.h"

namespace {

bool is_finite(double v) { return std::isfinite(v); }

// Reads whitespace-separated numbers line by line; each non-blank line must
// hold exactly `per_line` numbers.  Returns MTR_OK, MTR_ERR_IO or MTR_ERR_FORMAT.
mtr_status read_rows(const char* path, int per_line, double* out, int cap_rows, int* n_rows) {
  *n_rows = 0;
  FILE* f = std::fopen(path, "r");
  if (!f) return MTR_ERR_IO;
  char line[4096];
  mtr_status st = MTR_OK;
  while (std::fgets(line, sizeof line, f)) {
    if (!std::strchr(line, '\n') && !std::feof(f)) {
      st = MTR_ERR_FORMAT;  // line longer than the buffer
      break;
    }
    const char* p = line;
    double vals[8];
    int k = 0;
    for (;;) {
      while (*p == ' ' || *p == '\t' || *p == '\r' || *p == '\n') ++p;
      if (!*p) break;
      char* end = nullptr;
      errno = 0;
      const double v = std::strtod(p, &end);
      if (end == p || errno == ERANGE || !is_finite(v) || k == per_line) {
        st = MTR_ERR_FORMAT;
        break;
      }
      vals[k++] = v;
      p = end;
    }
    if (st != MTR_OK) break;
    if (k == 0) continue;  // blank line
    if (k != per_line) {
      st = MTR_ERR_FORMAT;
      break;
    }
    if (*n_rows < cap_rows)
      for (int i = 0; i < per_line; ++i) out[(size_t)*n_rows * per_line + i] = vals[i];
    ++*n_rows;
  }
  std::fclose(f);
  if (st == MTR_OK && *n_rows > cap_rows) *n_rows = cap_rows;
  return st;
}

}  // namespace

extern "C" {

mtr_status mtr_geometry_from_tilts(int n_views, const double* tilt_deg, const mtr_xf* xf, double phi_deg, int det_x,
                                   int det_y, mtr_volume_size vol, double* x_coef, double* y_coef) {
  if (n_views <= 0 || !tilt_deg || !x_coef || !y_coef || det_x <= 0 || det_y <= 0 || !is_finite(phi_deg))
    return MTR_ERR_INVALID_ARGUMENT;
  const double kDeg = 3.14159265358979323846 / 180.0;
  const double cx = (vol.Xstart + vol.Xend - 1) / 2.0, cy = (vol.Ystart + vol.Yend - 1) / 2.0,
               cz = (vol.Zstart + vol.Zend - 1) / 2.0;
  const double cu = (det_x + 1) / 2.0, cv = (det_y + 1) / 2.0;
  const double sf = std::sin(phi_deg * kDeg), cf = std::cos(phi_deg * kDeg);
  // in-plane detector v direction (independent of the tilt)
  const double a[3] = {-sf, cf, 0.0};
  for (int k = 0; k < n_views; ++k) {
    if (!is_finite(tilt_deg[k])) return MTR_ERR_INVALID_ARGUMENT;
    const double t = tilt_deg[k] * kDeg;
    const double e[3] = {std::cos(t) * cf, std::cos(t) * sf, std::sin(t)};
    // aligned coordinates relative to the detector centre: (e.(p-c), a.(p-c))
    double m11 = 1, m12 = 0, m21 = 0, m22 = 1, dx = 0, dy = 0;
    if (xf) {
      const mtr_xf& T = xf[k];
      const double all[6] = {T.a11, T.a12, T.a21, T.a22, T.dx, T.dy};
      for (double v : all)
        if (!is_finite(v)) return MTR_ERR_INVALID_ARGUMENT;
      const double det = T.a11 * T.a22 - T.a12 * T.a21;
      if (!(std::fabs(det) > 1e-12)) return MTR_ERR_INVALID_ARGUMENT;
      m11 = T.a22 / det;
      m12 = -T.a12 / det;
      m21 = -T.a21 / det;
      m22 = T.a11 / det;
      dx = T.dx;
      dy = T.dy;
    }
    // raw - C = M (al - C - d)
    double lx[3], ly[3];
    for (int i = 0; i < 3; ++i) {
      lx[i] = m11 * e[i] + m12 * a[i];
      ly[i] = m21 * e[i] + m22 * a[i];
    }
    const double ec = e[0] * cx + e[1] * cy + e[2] * cz, ac = a[0] * cx + a[1] * cy + a[2] * cz;
    x_coef[4 * k + 0] = cu - m11 * (ec + dx) - m12 * (ac + dy);
    y_coef[4 * k + 0] = cv - m21 * (ec + dx) - m22 * (ac + dy);
    for (int i = 0; i < 3; ++i) {
      x_coef[4 * k + 1 + i] = lx[i];
      y_coef[4 * k + 1 + i] = ly[i];
    }
  }
  return MTR_OK;
}

mtr_status mtr_tlt_read(const char* path, double* tilt_deg, int cap, int* n) {
  if (!path || !n || cap < 0 || (cap > 0 && !tilt_deg)) return MTR_ERR_INVALID_ARGUMENT;
  return read_rows(path, 1, tilt_deg, cap, n);
}

mtr_status mtr_xf_read(const char* path, mtr_xf* xf, int cap, int* n) {
  if (!path || !n || cap < 0 || (cap > 0 && !xf)) return MTR_ERR_INVALID_ARGUMENT;
  static_assert(sizeof(mtr_xf) == 6 * sizeof(double), "mtr_xf is six packed doubles");
  return read_rows(path, 6, reinterpret_cast<double*>(xf), cap, n);
}

}  // extern "C"
