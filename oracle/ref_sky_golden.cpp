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
//   ref_sky_golden ladybug EPW OUT 0 MF GREFL
//                                      ladybug mode's sky (the reference's run.cpp:362-398 and 447-470, restated here
//                                      over the reference's own read_epw, make_steps, sun_radiance, gendaymtx_step and
//                                      round_fmt) for the annual steps of the EPW. OUT: 7 doubles (T, P, Tup,
//                                      durationHours, lat, lon, tz), steps [T x 4] doubles (jd, hour, DNI, DHI), the float
//                                      accumulators [4 P + 6] (accDir, accDif, ground direct, ground diffuse), the weights
//                                      [3 P + 1] doubles (skyDirLB, skyDifLB, skyRad, gndLB), S [P x Tup] and g [Tup] floats
//   ref_sky_golden mesh IN OUT 0       the reference's triangulate_into and thin_solid (src/mesh.cpp) on one mesh.
//                                      IN: u64 nPoints, nFaces, nIdx; 3 doubles c; points [nPoints x 3] doubles; counts
//                                      [nFaces] i32; indices [nIdx] i32; slots [nFaces] u16. OUT: u64 made, i64 skipped,
//                                      u64 nSlots; v [nPoints x 3] f32; tri [made x 3] u32; slot [made] u32 (slot base
//                                      0, vertex base 0); thin_solid of each slot [nSlots] u32
//   ref_sky_golden dmesh IN OUT 0      the reference's read_dmesh (src/mesh.cpp:476-478) on one image named "case".
//                                      IN: the image's bytes. OUT: u64 ok, u64 meshes read, u64 message length, the
//                                      message; per mesh read u64 nPoints, nFaces, nIndices, nSlots and its arrays
//                                      (points f64, counts i32, indices i32, slots u16)
#include "internal.h"
#include <cmath>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

using namespace daylight;

// run.cpp:23-27
constexpr double kRf = 0.265074126, kGf = 0.670114631, kBf = 0.064811243;
inline double bright(const float* rgb) { return kRf * rgb[0] + kGf * rgb[1] + kBf * rgb[2]; }

static int ladybug(const char* epw, std::FILE* fo, int mf, double grefl) {
  Weather w;
  std::string err;
  if (!read_epw(epw, w, err)) { std::fprintf(stderr, "%s\n", err.c_str()); return 5; }
  Options opt;
  opt.t0 = NAN;
  opt.t1 = NAN;
  std::vector<Step> steps;
  if (!make_steps(opt, &w, steps, err, 0)) { std::fprintf(stderr, "%s\n", err.c_str()); return 6; }
  const size_t T = steps.size();
  const Patches pa = make_patches(mf);
  const size_t Pz = size_t(pa.P);
  double durationHours = 0;
  for (const Step& st : steps) durationHours += st.dt;
  const double lat = w.lat, lon = w.lon, tz = w.tz;
  const double latW = round_fmt(lat, "%.2f"), lonWestW = round_fmt(-lon, "%.2f"), meridW = static_cast<double>(static_cast<int>(-w.tz * 15.0));
  std::vector<int> colOf(T, -1);
  int Tup = 0;
  for (size_t t = 0; t < T; ++t) if (steps[t].dni + steps[t].dhi > 1e-4) colOf[t] = Tup++;
  std::vector<float> S(Pz * size_t(Tup), 0.f), gS(size_t(Tup), 0.f), buf(3 * (Pz + 1)), buf2(3 * (Pz + 1));
  std::vector<float> accDir(Pz, 0.f), accDif(3 * Pz, 0.f), gDif(3, 0.f), gDir(3, 0.f);
  for (size_t t = 0; t < T; ++t) {
    const Step& st = steps[t];
    const int col = colOf[t];
    double altS, aziS;
    sun_radiance(latW, lonWestW, meridW, st.jd, st.hour, altS, aziS);
    const double dniW = static_cast<double>(static_cast<int>(st.dni)), dhiW = static_cast<double>(static_cast<int>(st.dhi));
    gendaymtx_step(pa, st.jd, altS, aziS, dniW, dhiW, grefl, true, false, false, buf.data());
    gendaymtx_step(pa, st.jd, altS, aziS, dniW, dhiW, grefl, false, true, false, buf2.data());
    for (int ch = 0; ch < 3; ++ch) { gDir[size_t(ch)] += buf[size_t(ch)]; gDif[size_t(ch)] += buf2[size_t(ch)]; }
    double meanPatch = 0;
    for (size_t p = 0; p < Pz; ++p) {
      const float* dr = &buf[3 * (p + 1)];
      const float* df = &buf2[3 * (p + 1)];
      accDir[p] += dr[0];
      for (int ch = 0; ch < 3; ++ch) accDif[3 * p + size_t(ch)] += df[ch];
      if (col >= 0) {
        const double Lp = bright(df) + dr[0];
        S[p * size_t(Tup) + size_t(col)] = static_cast<float>(Lp);
        meanPatch += Lp * pa.omega[p];
      }
    }
    if (col >= 0) gS[size_t(col)] = static_cast<float>(grefl * meanPatch / static_cast<double>(pa.P));
  }
  const float inv = static_cast<float>(1.0 / static_cast<double>(T));
  std::vector<double> lb(3 * Pz + 1, 0.0);
  double mean = 0;
  for (size_t p = 0; p < Pz; ++p) {
    const float avgDir = T > 1 ? accDir[p] * inv : accDir[p];
    const float r = T > 1 ? accDif[3 * p] * inv : accDif[3 * p];
    const float gch = T > 1 ? accDif[3 * p + 1] * inv : accDif[3 * p + 1];
    const float b = T > 1 ? accDif[3 * p + 2] * inv : accDif[3 * p + 2];
    const double rd = round_fmt(avgDir, "%.3g"), rr = round_fmt(r, "%.3g"), rg = round_fmt(gch, "%.3g"), rb = round_fmt(b, "%.3g");
    lb[p] = rd * pa.omega[p] * durationHours / 1000.0;
    lb[Pz + p] = (kRf * rr + kGf * rg + kBf * rb) * pa.omega[p] * durationHours / 1000.0;
    lb[2 * Pz + p] = lb[p] + lb[Pz + p];
    mean += lb[2 * Pz + p];
  }
  lb[3 * Pz] = grefl * mean / static_cast<double>(pa.P);
  const double head[7] = {double(T), double(Pz), double(Tup), durationHours, lat, lon, tz};
  std::fwrite(head, 8, 7, fo);
  for (const Step& st : steps) {
    const double row[4] = {double(st.jd), st.hour, double(st.dni), double(st.dhi)};
    std::fwrite(row, 8, 4, fo);
  }
  std::fwrite(accDir.data(), 4, Pz, fo);
  std::fwrite(accDif.data(), 4, 3 * Pz, fo);
  std::fwrite(gDir.data(), 4, 3, fo);
  std::fwrite(gDif.data(), 4, 3, fo);
  std::fwrite(lb.data(), 8, lb.size(), fo);
  std::fwrite(S.data(), 4, S.size(), fo);
  std::fwrite(gS.data(), 4, gS.size(), fo);
  return 0;
}

static int mesh(std::FILE* fi, std::FILE* fo) {
  uint64_t head[3];
  double c[3];
  if (std::fread(head, 8, 3, fi) != 3 || std::fread(c, 8, 3, fi) != 3) return 4;
  SimulationMesh m;
  m.points.resize(3 * head[0]);
  m.counts.resize(head[1]);
  m.indices.resize(head[2]);
  m.slot.resize(head[1]);
  if (std::fread(m.points.data(), 8, m.points.size(), fi) != m.points.size() || std::fread(m.counts.data(), 4, m.counts.size(), fi) != m.counts.size() ||
      std::fread(m.indices.data(), 4, m.indices.size(), fi) != m.indices.size() || std::fread(m.slot.data(), 2, m.slot.size(), fi) != m.slot.size())
    return 4;
  const size_t cap = tri_cap(m);
  std::vector<float3> v(m.numPoints());
  std::vector<uint3> tri(cap);
  std::vector<uint32_t> slots(cap);
  int skipped = 0;
  const size_t made = triangulate_into(m, c, v.data(), tri.data(), slots.data(), 0, 0, skipped);
  const uint64_t nSlots = m.slot.empty() ? 1 : uint64_t(slot_count(m));
  std::vector<uint32_t> thin(nSlots);
  for (uint64_t s = 0; s < nSlots; ++s) thin[s] = thin_solid(m, unsigned(s), c);
  const uint64_t out[3] = {uint64_t(made), uint64_t(int64_t(skipped)), nSlots};
  std::fwrite(out, 8, 3, fo);
  std::fwrite(v.data(), 4, 3 * v.size(), fo);
  std::fwrite(tri.data(), 4, 3 * made, fo);
  std::fwrite(slots.data(), 4, made, fo);
  std::fwrite(thin.data(), 4, thin.size(), fo);
  return 0;
}

static int dmesh(std::FILE* fi, std::FILE* fo) {
  std::vector<char> img;
  char buf[65536];
  for (size_t n; (n = std::fread(buf, 1, sizeof buf, fi)) > 0;) img.insert(img.end(), buf, buf + n);
  std::vector<SimulationMesh> out;
  std::string err;
  const bool ok = read_dmesh(img.data(), img.size(), "case", out, err);
  const uint64_t head[3] = {uint64_t(ok), uint64_t(out.size()), uint64_t(err.size())};
  std::fwrite(head, 8, 3, fo);
  std::fwrite(err.data(), 1, err.size(), fo);
  for (const SimulationMesh& m : out) {
    const uint64_t n[4] = {uint64_t(m.numPoints()), uint64_t(m.counts.size()), uint64_t(m.indices.size()), uint64_t(m.slot.size())};
    std::fwrite(n, 8, 4, fo);
    std::fwrite(m.points.data(), 8, m.points.size(), fo);
    std::fwrite(m.counts.data(), 4, m.counts.size(), fo);
    std::fwrite(m.indices.data(), 4, m.indices.size(), fo);
    std::fwrite(m.slot.data(), 2, m.slot.size(), fo);
  }
  return 0;
}

int main(int argc, char** argv) {
  if (argc >= 4 && !std::strcmp(argv[1], "dmesh")) {
    std::FILE* fi = std::fopen(argv[2], "rb");
    std::FILE* fo = std::fopen(argv[3], "wb");
    if (!fi || !fo) return 3;
    const int rc = dmesh(fi, fo);
    std::fclose(fi);
    std::fclose(fo);
    return rc;
  }
  if (argc >= 4 && !std::strcmp(argv[1], "mesh")) {
    std::FILE* fi = std::fopen(argv[2], "rb");
    std::FILE* fo = std::fopen(argv[3], "wb");
    if (!fi || !fo) return 3;
    const int rc = mesh(fi, fo);
    std::fclose(fi);
    std::fclose(fo);
    return rc;
  }
  if (argc >= 7 && !std::strcmp(argv[1], "ladybug")) {
    std::FILE* fo = std::fopen(argv[3], "wb");
    if (!fo) return 3;
    const int rc = ladybug(argv[2], fo, std::atoi(argv[5]), std::atof(argv[6]));
    std::fclose(fo);
    return rc;
  }
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
