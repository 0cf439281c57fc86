// TEST INFRASTRUCTURE ONLY. Golden outputs of the reference's own sky and sun code (kit-sim_daylight src/sky.cpp
// gendaymtx_step / make_patches, src/solar.cpp sun_noaa, compiled unchanged from the reference tree by oracle/Makefile)
// for the engine's FP64 GPU sky (kgb_sky, kgb_sun_noaa). Driven by tests/golden/make_golden.py:
//   ref_sky_golden sun IN OUT N        IN: N x 7 doubles (lat, lon, tz, month, day, hour, leap); OUT: N x 6 doubles
//   ref_sky_golden sky IN OUT N MF SUN SKY VIS GREFL
//                                      IN: N x 5 doubles (jd, alt, azi, dni, dhi); OUT: N x 3 (P + 1) floats
#include "internal.h"
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

using namespace daylight;

int main(int argc, char** argv) {
  if (argc < 5) return 2;
  const size_t n = std::strtoul(argv[4], nullptr, 10);
  std::FILE* fi = std::fopen(argv[2], "rb");
  std::FILE* fo = std::fopen(argv[3], "wb");
  if (!fi || !fo) return 3;
  if (!std::strcmp(argv[1], "sun")) {
    std::vector<double> in(7 * n), out(6 * n);
    if (std::fread(in.data(), 8, in.size(), fi) != in.size()) return 4;
    for (size_t k = 0; k < n; ++k) {
      const double* p = &in[7 * k];
      const Sun s = sun_noaa(p[0], p[1], p[2], int(p[3]), int(p[4]), p[5], p[6] != 0);
      double* o = &out[6 * k];
      o[0] = s.alt; o[1] = s.azi; o[2] = s.up ? 1 : 0; o[3] = s.vec.x; o[4] = s.vec.y; o[5] = s.vec.z;
    }
    std::fwrite(out.data(), 8, out.size(), fo);
  } else {
    if (argc < 10) return 2;
    const int mf = std::atoi(argv[5]);
    const bool sun = std::atoi(argv[6]) != 0, sky = std::atoi(argv[7]) != 0, vis = std::atoi(argv[8]) != 0;
    const double grefl = std::atof(argv[9]);
    const Patches pa = make_patches(mf);
    std::vector<double> in(5 * n);
    if (std::fread(in.data(), 8, in.size(), fi) != in.size()) return 4;
    std::vector<float> row(3 * size_t(pa.P + 1));
    for (size_t k = 0; k < n; ++k) {
      const double* p = &in[5 * k];
      gendaymtx_step(pa, int(p[0]), p[1], p[2], p[3], p[4], grefl, sun, sky, vis, row.data());
      std::fwrite(row.data(), 4, row.size(), fo);
    }
  }
  std::fclose(fi);
  std::fclose(fo);
  return 0;
}
