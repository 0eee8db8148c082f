// Golden-vector generator built ON the reference's own CPU sources
// (ReadAndInitialOptions.cpp, MrcFileIO.cpp, MrcFileIOBaseFunction.cpp,
// compiled from where they lie by oracle/build.py into oracle/_ref/).
//
// TEST INFRASTRUCTURE ONLY.  tests/golden/make_golden.py runs it to record
// how the reference parses options, reads MRC stacks and TXBR maps, and
// writes the output volume; the product's I/O is tested against those
// records.  Output: one line "JSON:{...}" on stdout.
//
//   ref_golden options <argv...>            readOptions (ReadAndInitialOptions.cpp:127-172)
//   ref_golden read <stack.st> <map.txbr>   readMrcHeader + readMrcAndTXBR (MrcFileIO.cpp:107-178)
//   ref_golden write <out.mrc> Xs Xe Ys Ye Zs Ze <data.f32>
//                                           OutputModel + updataAndWriteModel (MrcFileIO.cpp:3-105,180-201)
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "MrcFileIO.h"
#include "ReadAndInitialOptions.h"

static void print_json_options(int rc, const Options& o) {
  std::printf("JSON:{\"rc\":%d,\"number_tilt\":%d,\"block\":[%d,%d,%d],\"iter_times\":%d,"
              "\"sirt_step\":%.9g,\"mace_step\":%.9g,\"out\":\"%s\",\"mrc\":[",
              rc, o.number_tilt, o.block_x, o.block_y, o.block_z, o.iter_times, (double)o.sirt_step,
              (double)o.mace_step, o.out_dir ? o.out_dir : "");
  for (int i = 0; i < o.number_tilt && i < 16; ++i) std::printf("%s\"%s\"", i ? "," : "", o.mrc_dir[i].c_str());
  std::printf("],\"txbr\":[");
  for (int i = 0; i < o.number_tilt && i < 16; ++i) std::printf("%s\"%s\"", i ? "," : "", o.txbr_dir[i].c_str());
  std::printf("]}\n");
}

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  const std::string cmd = argv[1];
  if (cmd == "options") {
    Options o;
    o.number_tilt = 0;
    o.out_dir = nullptr;
    o.mrc_dir = nullptr;
    o.txbr_dir = nullptr;
    Options* po = &o;
    const int rc = readOptions(argc - 1, argv + 1, po);
    std::printf("\n");
    print_json_options(rc, o);
    return 0;
  }
  if (cmd == "read" && argc >= 4) {
    Options o;
    o.number_tilt = 1;
    o.mrc_dir = new std::string[1];
    o.txbr_dir = new std::string[1];
    o.mrc_dir[0] = argv[2];
    o.txbr_dir[0] = argv[3];
    InputData in;
    in.group_id = 0;
    const int h = readMrcHeader(&o, &in);
    DataToUse d;
    const long long n = (long long)in.prj.X * in.prj.Y * in.prj.AngN;
    d.mrc_data = (float*)std::calloc((size_t)n, sizeof(float));
    d.x_coef = (double*)std::calloc((size_t)in.prj.AngN * 10, sizeof(double));
    d.y_coef = (double*)std::calloc((size_t)in.prj.AngN * 10, sizeof(double));
    const int r = readMrcAndTXBR(&o, &in, &d);
    std::printf("\nJSON:{\"header_rc\":%d,\"read_rc\":%d,\"prj\":[%d,%d,%d],\"mode\":%d,\"vol\":[%d,%d,%d,%d,%d,%d,%d,%d,%d],",
                h, r, in.prj.X, in.prj.Y, in.prj.AngN, in.mrc_header.mode, in.vol.Xstart, in.vol.Xend, in.vol.Ystart,
                in.vol.Yend, in.vol.Zstart, in.vol.Zend, in.vol.X, in.vol.Y, in.vol.Z);
    std::printf("\"x_coef\":[");
    for (int i = 0; i < 4 * in.prj.AngN; ++i) std::printf("%s%.17g", i ? "," : "", d.x_coef[i]);
    std::printf("],\"y_coef\":[");
    for (int i = 0; i < 4 * in.prj.AngN; ++i) std::printf("%s%.17g", i ? "," : "", d.y_coef[i]);
    std::printf("],\"data\":[");
    for (long long i = 0; i < n; ++i) std::printf("%s%.9g", i ? "," : "", (double)d.mrc_data[i]);
    std::printf("]}\n");
    return 0;
  }
  if (cmd == "write" && argc >= 10) {
    VolumeSize v;
    v.Xstart = std::atoi(argv[3]); v.Xend = std::atoi(argv[4]);
    v.Ystart = std::atoi(argv[5]); v.Yend = std::atoi(argv[6]);
    v.Zstart = std::atoi(argv[7]); v.Zend = std::atoi(argv[8]);
    v.X = v.Xend - v.Xstart; v.Y = v.Yend - v.Ystart; v.Z = v.Zend - v.Zstart;
    const size_t n = (size_t)v.X * v.Y * v.Z;
    std::vector<float> data(n);
    FILE* f = std::fopen(argv[9], "rb");
    if (!f || std::fread(data.data(), 4, n, f) != n) return 3;
    std::fclose(f);
    Options o;
    o.out_dir = argv[2];
    OutputModel res;
    res.slc.z_start = v.Zstart;
    res.slc.z_end = v.Zend;
    res.initialize(v);
    // The reference seeds amin/amax from this (otherwise uninitialised) buffer
    // (MrcFileIO.cpp:68); filling it with the data makes the record deterministic.
    std::memcpy(res.output_data, data.data(), n * 4);
    const int rc = updataAndWriteModel(&o, &res, data.data());
    std::printf("\nJSON:{\"rc\":%d}\n", rc);
    return 0;
  }
  return 2;
}
