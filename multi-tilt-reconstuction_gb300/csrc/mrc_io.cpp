// MRC and TXBR file I/O with the reference's formats and volume layout
// (MrcFileIO.cpp, MrcFileIOBaseFunction.cpp), returning status codes.
//
// Deliberate differences from the reference, all on inputs it mishandles:
//  * the data block is taken as the last n*bytes(mode) bytes of the file for
//    every mode (the reference uses n*2 for every mode and reads modes 0, 2
//    and 6 one byte at a time, MrcFileIOBaseFunction.cpp:20-66); for mode 1
//    stacks, the only mode the reference reads correctly, the result is the
//    same float array;
//  * TXBR lines are read whole and tokenised on any blank; a trailing blank
//    does not append a zero coefficient, and a non-numeric coefficient or a
//    bounds line with fewer than four ':' fields is a format error instead of
//    a silent 0 or a crash (MrcFileIOBaseFunction.cpp:72-134);
//  * the output header's amin/amax are taken from the data (the reference
//    seeds them from an uninitialised buffer, MrcFileIO.cpp:68) and the
//    header fields it leaves uninitialised are zero.
#include <algorithm>
#include <cerrno>
#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/mtr.h"

namespace {

struct File {
  FILE* f = nullptr;
  File(const char* path, const char* mode) { f = std::fopen(path, mode); }
  ~File() { if (f) std::fclose(f); }
};

long long file_size(FILE* f) {
  if (std::fseek(f, 0, SEEK_END) != 0) return -1;
  const long long n = (long long)std::ftell(f);
  std::rewind(f);
  return n;
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

// IEEE binary16 -> float (MRC mode 12), written out from the format definition.
float half_to_float(uint16_t h) {
  const uint32_t sign = (uint32_t)(h >> 15) << 31;
  const int exp = (h >> 10) & 0x1f;
  const uint32_t man = h & 0x3ffu;
  float v;
  if (exp == 0) v = std::ldexp((float)man, -24);
  else if (exp == 31) v = man ? NAN : INFINITY;
  else v = std::ldexp((float)(man | 0x400u), exp - 25);
  uint32_t bits;
  std::memcpy(&bits, &v, 4);
  bits |= sign;
  std::memcpy(&v, &bits, 4);
  return v;
}

uint16_t float_to_half(float f) {
  // Round-to-nearest-even conversion, finite range only (test inputs).
  uint32_t x;
  std::memcpy(&x, &f, 4);
  const uint32_t sign = (x >> 16) & 0x8000u;
  const float a = std::fabs(f);
  if (!(a == a)) return (uint16_t)(sign | 0x7e00u);
  if (a >= 65520.f) return (uint16_t)(sign | 0x7c00u);
  if (a < 6.103515625e-05f) {  // subnormal half: quantum 2^-24
    const float q = std::nearbyint(a * 16777216.f);
    return (uint16_t)(sign | (uint32_t)q);
  }
  int e;
  const float m = std::frexp(a, &e);  // a = m * 2^e, m in [0.5,1)
  float q = std::nearbyint(m * 2048.f);  // 11 significant bits
  if (q >= 2048.f) { q = 1024.f; ++e; }
  const uint32_t he = (uint32_t)(e + 14);
  return (uint16_t)(sign | (he << 10) | ((uint32_t)q & 0x3ffu));
}

bool is_blank(char c) { return c == ' ' || c == '\t' || c == '\r' || c == '\n' || c == '\v' || c == '\f'; }

std::vector<std::string> split_blank(const std::string& s) {
  std::vector<std::string> out;
  size_t i = 0;
  while (i < s.size()) {
    while (i < s.size() && is_blank(s[i])) ++i;
    size_t j = i;
    while (j < s.size() && !is_blank(s[j])) ++j;
    if (j > i) out.push_back(s.substr(i, j - i));
    i = j;
  }
  return out;
}

bool parse_double(const std::string& t, double* v) {
  errno = 0;
  char* end = nullptr;
  *v = std::strtod(t.c_str(), &end);
  return end && end != t.c_str() && *end == '\0' && errno != ERANGE;
}

bool parse_int_prefix(const std::string& t, int* v) {
  // atoi semantics on the leading digits, but the field must start with a number.
  const char* p = t.c_str();
  while (is_blank(*p)) ++p;
  char* end = nullptr;
  errno = 0;
  const long x = std::strtol(p, &end, 10);
  if (end == p || errno == ERANGE || x < -2147483647L || x > 2147483647L) return false;
  *v = (int)x;
  return true;
}

}  // namespace

extern "C" {

void mtr_volume_size_empty(mtr_volume_size* vol) {
  if (!vol) return;
  vol->Xstart = 999999; vol->Xend = -999999;
  vol->Ystart = 999999; vol->Yend = -999999;
  vol->Zstart = 999999; vol->Zend = -999999;
  vol->X = vol->Y = 0;
  vol->Z = 91;  // the reference's InputData() default (MrcFileIO.h:27)
}

mtr_status mtr_mrc_read_header(const char* path, mtr_mrc_header* out) {
  static_assert(sizeof(mtr_mrc_header) == 1024, "MRC header must be 1024 bytes");
  if (!path || !out) return MTR_ERR_INVALID_ARGUMENT;
  File f(path, "rb");
  if (!f.f) return MTR_ERR_IO;
  if (std::fread(out, 1, 1024, f.f) != 1024) return MTR_ERR_FORMAT;
  return MTR_OK;
}

mtr_status mtr_mrc_read_stack(const char* path, float* out, long long n) {
  if (!path || !out || n <= 0) return MTR_ERR_INVALID_ARGUMENT;
  File f(path, "rb");
  if (!f.f) return MTR_ERR_IO;
  mtr_mrc_header h;
  if (std::fread(&h, 1, 1024, f.f) != 1024) return MTR_ERR_FORMAT;
  const int nb = mode_bytes(h.mode);
  if (nb == 0) return MTR_ERR_UNSUPPORTED;
  const long long size = file_size(f.f);
  const long long need = n * nb;
  if (size < 1024 + need) return MTR_ERR_FORMAT;
  if (std::fseek(f.f, (long)(size - need), SEEK_SET) != 0) return MTR_ERR_IO;
  std::vector<unsigned char> buf;
  const long long chunk = 1 << 24;
  long long done = 0;
  buf.resize((size_t)std::min(need, chunk * nb));
  while (done < n) {
    const long long m = std::min(chunk, n - done);
    if (std::fread(buf.data(), (size_t)nb, (size_t)m, f.f) != (size_t)m) return MTR_ERR_IO;
    float* o = out + done;
    const unsigned char* b = buf.data();
    switch (h.mode) {
      case MTR_MRC_MODE_BYTE:
        for (long long i = 0; i < m; ++i) o[i] = (float)b[i];
        break;
      case MTR_MRC_MODE_SHORT:
        for (long long i = 0; i < m; ++i) {
          int16_t v;
          std::memcpy(&v, b + 2 * i, 2);
          o[i] = (float)v;
        }
        break;
      case MTR_MRC_MODE_USHORT:
        for (long long i = 0; i < m; ++i) {
          uint16_t v;
          std::memcpy(&v, b + 2 * i, 2);
          o[i] = (float)v;
        }
        break;
      case MTR_MRC_MODE_FLOAT:
        std::memcpy(o, b, (size_t)m * 4);
        break;
      case MTR_MRC_MODE_HALF:
        for (long long i = 0; i < m; ++i) {
          uint16_t v;
          std::memcpy(&v, b + 2 * i, 2);
          o[i] = half_to_float(v);
        }
        break;
    }
    done += m;
  }
  return MTR_OK;
}

mtr_status mtr_txbr_read(const char* path, double* x_coef, double* y_coef, int cap, int* n_x, int* n_y,
                         mtr_volume_size* vol) {
  if (!path || !n_x || !n_y || !vol || cap < 0 || (cap > 0 && (!x_coef || !y_coef))) return MTR_ERR_INVALID_ARGUMENT;
  File f(path, "rb");
  if (!f.f) return MTR_ERR_IO;
  int nx = 0, ny = 0;
  std::string line;
  int ch;
  bool eof = false;
  while (!eof) {
    line.clear();
    while ((ch = std::fgetc(f.f)) != EOF && ch != '\n') line.push_back((char)ch);
    if (ch == EOF) {
      eof = true;
      if (line.empty()) break;
    }
    if (line.size() < 2) continue;
    const char c0 = line[0], c1 = line[1];
    const bool arrow = line.size() >= 3 && line[2] == '>';
    if ((c0 == 'x' || c0 == 'y') && c1 == '-' && !arrow) {
      // "x-<label> c0 c1 c2 c3 ..." : every blank-separated token after the first.
      const std::vector<std::string> tok = split_blank(line);
      for (size_t t = 1; t < tok.size(); ++t) {
        double v;
        if (!parse_double(tok[t], &v)) return MTR_ERR_FORMAT;
        if (c0 == 'x') {
          if (nx < cap) x_coef[nx] = v;
          ++nx;
        } else {
          if (ny < cap) y_coef[ny] = v;
          ++ny;
        }
      }
    } else if ((c0 == 'x' || c0 == 'y' || c0 == 'z') && c1 == '-' && arrow) {
      // "x->START:STEP:END" -> fields 2 and 4 of the ':'-split with '>' as ':'.
      std::string s = line;
      s[2] = ':';
      std::vector<std::string> fld;
      size_t i = 0;
      while (i <= s.size()) {
        size_t j = s.find(':', i);
        if (j == std::string::npos) j = s.size();
        if (j > i) fld.push_back(s.substr(i, j - i));  // strtok skips empty fields
        i = j + 1;
      }
      int a, b;
      if (fld.size() < 4 || !parse_int_prefix(fld[1], &a) || !parse_int_prefix(fld[3], &b)) return MTR_ERR_FORMAT;
      if (c0 == 'x') { vol->Xstart = std::min(vol->Xstart, a); vol->Xend = std::max(vol->Xend, b); }
      if (c0 == 'y') { vol->Ystart = std::min(vol->Ystart, a); vol->Yend = std::max(vol->Yend, b); }
      if (c0 == 'z') { vol->Zstart = std::min(vol->Zstart, a); vol->Zend = std::max(vol->Zend, b); }
    }
  }
  vol->X = vol->Xend - vol->Xstart;
  vol->Y = vol->Yend - vol->Ystart;
  vol->Z = vol->Zend - vol->Zstart;
  *n_x = nx;
  *n_y = ny;
  if (nx > cap || ny > cap) return MTR_ERR_CAPACITY;
  return MTR_OK;
}

// The grammar mtr_txbr_read (and the reference's readCoef,
// MrcFileIOBaseFunction.cpp:72-134) parses: per view an "l k" line and
// "x-k:" / "y-k:" lines of the four coefficients [const, X, Y, Z], then the
// "x->start:1:end" bound lines (fields 2 and 4 are start and end).  Numbers
// are the shortest text that reads back to the same double (std::to_chars:
// independent of the C locale), and no line ends in a blank (the reference
// would read a trailing blank as one more coefficient).
mtr_status mtr_txbr_write(const char* path, int n_views, const double* x_coef, const double* y_coef,
                          mtr_volume_size vol) {
  if (!path || n_views <= 0 || !x_coef || !y_coef) return MTR_ERR_INVALID_ARGUMENT;
  for (int i = 0; i < 4 * n_views; ++i)
    if (!std::isfinite(x_coef[i]) || !std::isfinite(y_coef[i])) return MTR_ERR_INVALID_ARGUMENT;
  if (vol.Xend <= vol.Xstart || vol.Yend <= vol.Ystart || vol.Zend <= vol.Zstart) return MTR_ERR_INVALID_ARGUMENT;
  std::string out;
  out.reserve((size_t)n_views * 220 + 64);
  char num[64];
  auto append_num = [&](double v) {
    const std::to_chars_result r = std::to_chars(num, num + sizeof num, v);
    out.append(num, r.ptr);
  };
  for (int k = 0; k < n_views; ++k) {
    const std::string label = std::to_string(k);
    out += "l " + label + "\n";
    for (int m = 0; m < 2; ++m) {
      const double* c = (m == 0 ? x_coef : y_coef) + 4 * k;
      out += (m == 0 ? "x-" : "y-") + label + ":";
      for (int j = 0; j < 4; ++j) {
        out += ' ';
        append_num(c[j]);
      }
      out += '\n';
    }
  }
  out += "x->" + std::to_string(vol.Xstart) + ":1:" + std::to_string(vol.Xend) + "\n";
  out += "y->" + std::to_string(vol.Ystart) + ":1:" + std::to_string(vol.Yend) + "\n";
  out += "z->" + std::to_string(vol.Zstart) + ":1:" + std::to_string(vol.Zend) + "\n";
  File f(path, "wb");
  if (!f.f) return MTR_ERR_IO;
  if (std::fwrite(out.data(), 1, out.size(), f.f) != out.size()) return MTR_ERR_IO;
  return std::fflush(f.f) == 0 ? MTR_OK : MTR_ERR_IO;
}

mtr_status mtr_mrc_write_volume(const char* path, mtr_volume_size vol, const float* data) {
  if (!path || !data || vol.X <= 0 || vol.Y <= 0 || vol.Z <= 0) return MTR_ERR_INVALID_ARGUMENT;
  mtr_mrc_header h;
  std::memset(&h, 0, sizeof(h));
  // MrcFileIO.cpp:3-61 (headerInitialize + headerSetValue).
  h.nx = vol.X; h.ny = vol.Y; h.nz = vol.Z;
  h.mode = MTR_MRC_MODE_FLOAT;
  h.nxstart = vol.Xstart; h.nystart = vol.Ystart; h.nzstart = vol.Zstart;
  h.mx = vol.X; h.my = vol.Y; h.mz = vol.Z;
  h.xlen = h.ylen = h.zlen = 1.f;
  h.alpha = h.beta = h.gamma = 90.f;
  h.mapc = 1; h.mapr = 2; h.maps = 3;
  h.ispg = 0; h.nsymbt = 0; h.next = 0;
  h.creatid = 1000;
  h.cmap[0] = 'M'; h.cmap[1] = 'A'; h.cmap[2] = 'P'; h.cmap[3] = ' ';
  h.stamp[0] = 'D';
  // updateHeader (MrcFileIO.cpp:63-88): min, max, mean of per-section means.
  const long long sec = (long long)vol.X * vol.Y;
  float amin = data[0], amax = data[0];
  double sum_of_means = 0.0;
  for (int z = 0; z < vol.Z; ++z) {
    const float* p = data + sec * z;
    double m = 0.0;
    for (long long i = 0; i < sec; ++i) {
      const float v = p[i];
      if (v > amax) amax = v;
      if (v < amin) amin = v;
      m += v;
    }
    sum_of_means += m / (double)sec;
  }
  h.amin = amin;
  h.amax = amax;
  h.amean = (float)(sum_of_means / vol.Z);
  File f(path, "wb");
  if (!f.f) return MTR_ERR_IO;
  if (std::fwrite(&h, 1, 1024, f.f) != 1024) return MTR_ERR_IO;
  const size_t n = (size_t)sec * vol.Z;
  if (std::fwrite(data, sizeof(float), n, f.f) != n) return MTR_ERR_IO;
  return MTR_OK;
}

mtr_status mtr_mrc_write_stack(const char* path, int nx, int ny, int nz, int mode, const float* data) {
  if (!path || !data || nx <= 0 || ny <= 0 || nz <= 0) return MTR_ERR_INVALID_ARGUMENT;
  if (mode != MTR_MRC_MODE_SHORT && mode != MTR_MRC_MODE_FLOAT && mode != MTR_MRC_MODE_HALF)
    return MTR_ERR_UNSUPPORTED;
  mtr_mrc_header h;
  std::memset(&h, 0, sizeof(h));
  h.nx = nx; h.ny = ny; h.nz = nz; h.mode = mode;
  h.mx = nx; h.my = ny; h.mz = nz;
  h.xlen = (float)nx; h.ylen = (float)ny; h.zlen = (float)nz;
  h.alpha = h.beta = h.gamma = 90.f;
  h.mapc = 1; h.mapr = 2; h.maps = 3;
  h.cmap[0] = 'M'; h.cmap[1] = 'A'; h.cmap[2] = 'P'; h.cmap[3] = ' ';
  h.stamp[0] = 'D'; h.stamp[1] = 'A';
  const long long n = (long long)nx * ny * nz;
  float amin = data[0], amax = data[0];
  double sum = 0.0;
  for (long long i = 0; i < n; ++i) {
    amin = std::min(amin, data[i]);
    amax = std::max(amax, data[i]);
    sum += data[i];
  }
  h.amin = amin; h.amax = amax; h.amean = (float)(sum / (double)n);
  File f(path, "wb");
  if (!f.f) return MTR_ERR_IO;
  if (std::fwrite(&h, 1, 1024, f.f) != 1024) return MTR_ERR_IO;
  std::vector<unsigned char> buf;
  const long long chunk = 1 << 22;
  for (long long done = 0; done < n; done += chunk) {
    const long long m = std::min(chunk, n - done);
    const float* d = data + done;
    if (mode == MTR_MRC_MODE_FLOAT) {
      if (std::fwrite(d, 4, (size_t)m, f.f) != (size_t)m) return MTR_ERR_IO;
      continue;
    }
    buf.resize((size_t)m * 2);
    for (long long i = 0; i < m; ++i) {
      uint16_t v;
      if (mode == MTR_MRC_MODE_SHORT) {
        float r = std::nearbyint(d[i]);
        r = std::fmin(std::fmax(r, -32768.f), 32767.f);
        const int16_t s = (int16_t)r;
        std::memcpy(&v, &s, 2);
      } else {
        v = float_to_half(d[i]);
      }
      std::memcpy(buf.data() + 2 * i, &v, 2);
    }
    if (std::fwrite(buf.data(), 2, (size_t)m, f.f) != (size_t)m) return MTR_ERR_IO;
  }
  return MTR_OK;
}

}  // extern "C"
