// TEST INFRASTRUCTURE ONLY. Golden outputs of the reference's own sky and sun code (kit-sim_daylight src/sky.cpp
// gendaymtx_step / make_patches, src/solar.cpp sun_noaa, compiled unchanged from the reference tree by oracle/Makefile)
// for the engine's FP64 GPU sky (kgb_sky, kgb_sun_noaa). Driven by tests/golden/make_golden.py:
//   ref_sky_golden sun IN OUT N        IN: N x 7 doubles (lat, lon, tz, month, day, hour, leap); OUT: N x 6 doubles
//   ref_sky_golden sky IN OUT N MF SUN SKY VIS GREFL
//                                      IN: N x 5 doubles (jd, alt, azi, dni, dhi); OUT: N x 3 (P + 1) floats
//   ref_sky_golden year IN OUT N MF    the sky build of a weather year as the engine's precision benchmark runs it on
//                                      the GPU (NOAA sun per hour at 52.52 N, 13.41 E, tz 1; per hour the sky alone and
//                                      the binned sun alone, ground 0.2), on the reference's own host code, serial as in
//                                      run.cpp:372-446. IN: N x 2 doubles (DNI, DHI) per hour of a non-leap year;
//                                      OUT: 1 double, the seconds it took
#include "internal.h"
#include <chrono>
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
  } else if (!std::strcmp(argv[1], "year")) {
    if (argc < 6) return 2;
    const int mf = std::atoi(argv[5]);
    std::vector<double> w(2 * n);
    if (std::fread(w.data(), 8, w.size(), fi) != w.size()) return 4;
    static const int dim[12] = {31, 28, 31, 30, 31, 30, 31, 31, 30, 31, 30, 31};
    const auto t0 = std::chrono::steady_clock::now();
    const Patches pa = make_patches(mf);
    std::vector<float> row(3 * size_t(pa.P + 1));
    double sink = 0;
    size_t k = 0;
    for (int m = 1; m <= 12 && k < n; ++m)
      for (int d = 1; d <= dim[m - 1] && k < n; ++d)
        for (int h = 0; h < 24 && k < n; ++h, ++k) {
          const Sun s = sun_noaa(52.52, 13.41, 1.0, m, d, h + 0.5, false);
          const int jd = int(k / 24) + 1;
          const double alt = s.alt * 3.141592653589793 / 180, azi = s.azi * 3.141592653589793 / 180;
          gendaymtx_step(pa, jd, alt, azi, w[2 * k], w[2 * k + 1], 0.2, false, true, false, row.data());
          sink += row[3];
          gendaymtx_step(pa, jd, alt, azi, w[2 * k], w[2 * k + 1], 0.2, true, false, false, row.data());
          sink += row[3];
        }
    const double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::fwrite(&sec, 8, 1, fo);
    std::fprintf(stderr, "%zu steps, check %g\n", k, sink);
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
