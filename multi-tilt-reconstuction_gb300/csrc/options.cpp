// Command-line parsing with the reference's options (readOptions,
// ReadAndInitialOptions.cpp:104-172; defaults ReadAndInitialOptions.h:33-42):
//   -i K,st_1,...,st_K,txbr_1,...,txbr_K   input stacks and TXBR maps
//   -o FILE                                output MRC volume
//   -x/-y/-z N                             CUDA block size (kept as tile hints)
//   -n N                                   MACE outer iterations (default 5)
//   -s F                                   SIRT relaxation (default 0.5)
//   -m F                                   MACE step rho (default 0.7)
//   -h                                     help
// plus long-only options: --inner N (SIRT iterations per MACE iteration,
// hard-coded 10 in the reference) and --precision fp32|bf16|fp16.
//
// The option character is held in an int, so the loop terminates on hosts
// where char is unsigned (the reference's `char ch` loop does not).  Invalid
// options, missing arguments and malformed -i lists are errors.
#include <getopt.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/mtr.h"

namespace {

bool parse_int(const char* s, int* out) {
  if (!s || !*s) return false;
  char* end = nullptr;
  const long v = std::strtol(s, &end, 10);
  if (*end != '\0' || v < -2147483647L || v > 2147483647L) return false;
  *out = (int)v;
  return true;
}

bool parse_float(const char* s, float* out) {
  if (!s || !*s) return false;
  char* end = nullptr;
  const double v = std::strtod(s, &end);
  if (*end != '\0') return false;
  *out = (float)v;
  return true;
}

bool copy_path(char* dst, const std::string& src) {
  if (src.empty() || src.size() >= 1024) return false;
  std::memcpy(dst, src.c_str(), src.size() + 1);
  return true;
}

// praseInputAddr (ReadAndInitialOptions.cpp:104-125): "K,st..,txbr..".
bool parse_inputs(const char* arg, mtr_options* o) {
  std::vector<std::string> f;
  std::string cur;
  for (const char* p = arg; *p; ++p) {
    if (*p == ',') { f.push_back(cur); cur.clear(); }
    else cur.push_back(*p);
  }
  f.push_back(cur);
  int k = 0;
  if (!parse_int(f[0].c_str(), &k) || k < 1 || k > MTR_MAX_AXES) return false;
  if ((int)f.size() != 1 + 2 * k) return false;
  for (int i = 0; i < k; ++i) {
    if (!copy_path(o->mrc_path[i], f[1 + i])) return false;
    if (!copy_path(o->txbr_path[i], f[1 + k + i])) return false;
  }
  o->number_tilt = k;
  return true;
}

}  // namespace

extern "C" mtr_status mtr_parse_options(int argc, char** argv, mtr_options* o) {
  if (!o || argc < 0 || (argc > 0 && !argv)) return MTR_ERR_INVALID_ARGUMENT;
  std::memset(o, 0, sizeof(*o));
  o->block_x = o->block_y = o->block_z = 8;
  o->iter_times = 5;
  o->sirt_step = 0.5f;
  o->mace_step = 0.7f;
  o->sirt_inner = MTR_DEFAULT_SIRT_INNER;
  o->precision = MTR_PREC_FP32;
  static const struct option longopts[] = {
      {"help", no_argument, nullptr, 'h'},
      {"inner", required_argument, nullptr, 1001},
      {"precision", required_argument, nullptr, 1002},
      {nullptr, 0, nullptr, 0},
  };
  optind = 0;  // full re-initialisation of getopt (glibc): the parser may be called repeatedly
  opterr = 0;
  int ch;
  mtr_status st = MTR_OK;
  while ((ch = getopt_long(argc, argv, ":hi:o:x:y:z:n:s:m:", longopts, nullptr)) != -1) {
    switch (ch) {
      case 'h': o->help = 1; break;
      case 'i': if (!parse_inputs(optarg, o)) st = MTR_ERR_INVALID_ARGUMENT; break;
      case 'o': if (!copy_path(o->out_path, optarg ? optarg : "")) st = MTR_ERR_INVALID_ARGUMENT; break;
      case 'x': if (!parse_int(optarg, &o->block_x) || o->block_x <= 0) st = MTR_ERR_INVALID_ARGUMENT; break;
      case 'y': if (!parse_int(optarg, &o->block_y) || o->block_y <= 0) st = MTR_ERR_INVALID_ARGUMENT; break;
      case 'z': if (!parse_int(optarg, &o->block_z) || o->block_z <= 0) st = MTR_ERR_INVALID_ARGUMENT; break;
      case 'n': if (!parse_int(optarg, &o->iter_times) || o->iter_times < 0) st = MTR_ERR_INVALID_ARGUMENT; break;
      case 's': if (!parse_float(optarg, &o->sirt_step)) st = MTR_ERR_INVALID_ARGUMENT; break;
      case 'm': if (!parse_float(optarg, &o->mace_step)) st = MTR_ERR_INVALID_ARGUMENT; break;
      case 1001: if (!parse_int(optarg, &o->sirt_inner) || o->sirt_inner < 0) st = MTR_ERR_INVALID_ARGUMENT; break;
      case 1002:
        if (std::strcmp(optarg, "fp32") == 0) o->precision = MTR_PREC_FP32;
        else if (std::strcmp(optarg, "bf16") == 0) o->precision = MTR_PREC_MIXED_BF16;
        else if (std::strcmp(optarg, "fp16") == 0) o->precision = MTR_PREC_MIXED_FP16;
        else st = MTR_ERR_INVALID_ARGUMENT;
        break;
      default: st = MTR_ERR_INVALID_ARGUMENT; break;  // '?' unknown option, ':' missing argument
    }
    if (st != MTR_OK) break;
  }
  if (st == MTR_OK && optind < argc) st = MTR_ERR_INVALID_ARGUMENT;  // stray positional arguments
  optind = 0;
  return st;
}
