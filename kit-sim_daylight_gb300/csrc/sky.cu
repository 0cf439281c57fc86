// The sky side of the path in FP64 on the GPU: NOAA sun positions per step and the Perez all-weather sky per step and
// patch, restating the reference's host code (src/solar.cpp:66-105 sun_noaa; src/sky.cpp:240-283 make_patches,
// :297-474 gendaymtx_step, a port of Radiance gendaymtx's ComputeSky + AddDirect) so that a whole year's sky matrix
// [T x P] is built beside the contraction that consumes it.
//
// k_sky: one CTA per time step. The per-step scalars (zenith, air mass, clearness category, illuminances, Perez
// parameters) on one thread; the patch luminances (exp / acos / cos in FP64) on all threads; the normalising sum and
// the four patches nearest the sun on one thread in the reference's order (sequential sums, first-wins ties), so the
// float outputs round as the reference's do.
// k_sun: one thread per step.
#include "engine.h"
#include "kgb_detmath.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace kgb {

// Perez, Seals, Michalsky 1993 (Solar Energy 50(3):235-245) Table 1, with the 1993 erratum: the all-weather model's
// coefficients per sky clearness category, 5 parameters x 4 terms (published data; the model needs these values).
__constant__ double kPerez[8][20] = {
    {1.3525, -0.2576, -0.2690, -1.4366, -0.7670, 0.0007, 1.2734, -0.1233, 2.8000, 0.6004, 1.2375, 1.0000, 1.8734, 0.6297, 0.9738, 0.2809,
     0.0356, -0.1246, -0.5718, 0.9938},
    {-1.2219, -0.7730, 1.4148, 1.1016, -0.2054, 0.0367, -3.9128, 0.9156, 6.9750, 0.1774, 6.4477, -0.1239, -1.5798, -0.5081, -1.7812,
     0.1080, 0.2624, 0.0672, -0.2190, -0.4285},
    {-1.1000, -0.2515, 0.8952, 0.0156, 0.2782, -0.1812, -4.5000, 1.1766, 24.7219, -13.0812, -37.7000, 34.8438, -5.0000, 1.5218, 3.9229,
     -2.6204, -0.0156, 0.1597, 0.4199, -0.5562},
    {-0.5484, -0.6654, -0.2672, 0.7117, 0.7234, -0.6219, -5.6812, 2.6297, 33.3389, -18.3000, -62.2500, 52.0781, -3.5000, 0.0016, 1.1477,
     0.1062, 0.4659, -0.3296, -0.0876, -0.0329},
    {-0.6000, -0.3566, -2.5000, 2.3250, 0.2937, 0.0496, -5.6812, 1.8415, 21.0000, -4.7656, -21.5906, 7.2492, -3.5000, -0.1554, 1.4062,
     0.3988, 0.0032, 0.0766, -0.0656, -0.1294},
    {-1.0156, -0.3670, 1.0078, 1.4051, 0.2875, -0.5328, -3.8500, 3.3750, 14.0000, -0.9999, -7.1406, 7.5469, -3.4000, -0.1078, -1.0750,
     1.5702, -0.0672, 0.4016, 0.3017, -0.4844},
    {-1.0000, 0.0211, 0.5025, -0.5119, -0.3000, 0.1922, 0.7023, -1.6317, 19.0000, -5.0000, 1.2438, -1.9094, -4.0000, 0.0250, 0.3844,
     0.2656, 1.0468, -0.3788, -2.4517, 1.4656},
    {-1.0500, 0.0289, 0.4260, 0.3590, -0.3250, 0.1156, 0.7781, 0.0025, 31.0625, -14.5000, -46.1148, 55.3750, -7.2312, 0.4050, 13.3500,
     0.6234, 1.5000, -0.6426, 1.8564, 0.5636}};
// Perez et al. 1990 (Solar Energy 44(5):271-289) Table 1 clearness bounds and Table 4 luminous efficacy (a, b, c, d).
__constant__ double kClearLo[8] = {1.000, 1.065, 1.230, 1.500, 1.950, 2.800, 4.500, 6.200};
__constant__ double kClearHi[8] = {1.065, 1.230, 1.500, 1.950, 2.800, 4.500, 6.200, 12.01};
__constant__ double kDiffLum[8][4] = {{97.24, -0.46, 12.00, -8.91},    {107.22, 1.15, 0.59, -3.95},  {104.97, 2.96, -5.53, -8.77},
                                      {102.39, 5.59, -13.95, -13.90}, {100.71, 5.94, -22.75, -23.74}, {106.42, 3.83, -36.15, -28.83},
                                      {141.88, 1.90, -53.24, -14.03}, {152.23, 0.35, -45.27, -7.98}};
__constant__ double kDirLum[8][4] = {{57.20, -4.55, -2.98, 117.12}, {98.99, -3.46, -1.21, 12.38},  {109.83, -4.90, -1.71, -8.81},
                                     {110.34, -5.84, -1.99, -4.56},  {106.36, -3.97, -1.75, -6.16}, {107.19, -1.25, -1.51, -26.73},
                                     {105.75, 0.77, -1.26, -34.44},  {101.18, 1.58, -1.10, -8.29}};

constexpr double PI = 3.14159265358979323846;
constexpr double WHTEFFICACY = 179.;

struct SkyArgs {
  const kgb_sky_step* steps;
  uint32_t T, P;
  const float* alt;      // [P] patch centre altitude (float, as the reference's Patches)
  const float* azi;
  const float* omega;
  const double* costab;  // [1025] Radiance tcos table
  double grefl;
  int sun, sky, visible;
  float* out;            // [T x 3 (P + 1)]
};

__device__ __forceinline__ double tcos_d(const double* costab, double x) {   // Radiance tcos.c, NCOSENTRY 1024
  const int N = 1024;
  if (x < 0.) x = -x;
  int i = (int)((N * 2. / PI) * x + 0.5);
  while (i >= 4 * N) i -= 4 * N;
  switch (i / N) {
    case 0: return costab[i];
    case 1: return -costab[2 * N - i];
    case 2: return -costab[i - 2 * N];
    default: return costab[4 * N - i];
  }
}

__global__ void __launch_bounds__(128) k_sky(SkyArgs a) {
  extern __shared__ double sh[];   // [P] terms, then [P] sun dot products
  __shared__ double sPar[5], sScal[6];
  __shared__ int sNight;
  const uint32_t t = blockIdx.x;
  const kgb_sky_step st = a.steps[t];
  float* parr = a.out + size_t(t) * 3 * (a.P + 1);
  const uint32_t nsp = a.P + 1;
  if (threadIdx.x == 0) {
    sNight = st.dni + st.dhi <= 1e-4;
    const double altitude = st.alt, dir_irrad = st.dni, diff_irrad = st.dhi;
    const double apwc = exp(0.07 * 11.0 - 0.075);
    double sz;
    if (altitude <= 0.0) sz = 90.0 * (PI / 180.);
    else if (altitude >= 87.0 * (PI / 180.)) sz = 3.0 * (PI / 180.);
    else sz = 90.0 * (PI / 180.) - altitude;
    const double day_angle = (st.jd - 1.0) * (2.0 * PI / 365.0);
    const double E0 = 1.00011 + 0.034221 * cos(day_angle) + 0.00128 * sin(day_angle) + 0.000719 * cos(2.0 * day_angle) + 0.000077 * sin(2.0 * day_angle);
    const double air_mass = 1.0 / (cos(sz) + 0.15 * pow(93.885 - sz * (180. / PI), -1.253));
    double bright = diff_irrad * air_mass / (1367.0 * E0);
    const double sz3 = sz * sz * sz;
    double clear = ((diff_irrad + dir_irrad) / diff_irrad + 1.041 * sz3) / (1.0 + 1.041 * sz3);
    if (clear > 11.9) clear = 11.9;
    if (bright < 0.01) bright = 0.01;
    int index;
    for (index = 0; index < 8; index++)
      if (clear >= kClearLo[index] && clear < kClearHi[index]) break;
    if (index > 7) index = 7;
    double diff_illum, dir_illum;
    if (a.visible) {
      diff_illum = diff_irrad * (kDiffLum[index][0] + kDiffLum[index][1] * apwc + kDiffLum[index][2] * cos(sz) + kDiffLum[index][3] * log(bright));
      const double r = kDirLum[index][0] + kDirLum[index][1] * apwc + kDirLum[index][2] * exp(5.73 * sz - 5.0) + kDirLum[index][3] * bright;
      dir_illum = dir_irrad * (r > 0.0 ? r : 0.0);
    } else {
      diff_illum = diff_irrad * WHTEFFICACY;
      dir_illum = dir_irrad * WHTEFFICACY;
    }
    // ground (float / double mixing as the reference's)
    if (!sNight) {
      float g0 = (float)diff_illum;
      if (altitude > 0) g0 = (float)(g0 + dir_illum * sin(altitude));
      g0 = (float)(g0 * (1. / PI / WHTEFFICACY));
      const float gr = a.sky ? (float)a.grefl : 0.f;
      parr[0] = parr[1] = parr[2] = g0 * gr;
    }
    // Perez parameters
    double delta = bright;
    if (clear > 1.065 && clear < 2.8 && delta < 0.2) delta = 0.2;
    const double* x = kPerez[index];
    if (index != 0) {
      for (int i = 0; i < 5; i++) sPar[i] = x[4 * i] + x[4 * i + 1] * sz + delta * (x[4 * i + 2] + x[4 * i + 3] * sz);
    } else {
      sPar[0] = x[0] + x[1] * sz + delta * (x[2] + x[3] * sz);
      sPar[1] = x[4] + x[5] * sz + delta * (x[6] + x[7] * sz);
      sPar[4] = x[16] + x[17] * sz + delta * (x[18] + x[19] * sz);
      sPar[2] = exp(pow(delta * (x[8] + x[9] * sz), x[10])) - x[11];
      sPar[3] = -exp(delta * (x[12] + x[13] * sz)) + x[14] + delta * x[15];
    }
    sScal[0] = sz; sScal[1] = diff_illum; sScal[2] = dir_illum; sScal[3] = altitude; sScal[4] = st.azi;
  }
  __syncthreads();
  if (sNight) {
    for (uint32_t k = threadIdx.x; k < 3 * nsp; k += blockDim.x) parr[k] = 0.f;
    return;
  }
  const double sz = sScal[0], diff_illum = sScal[1], dir_illum = sScal[2], altitude = sScal[3], azimuth = sScal[4];
  const float skyc[3] = {a.sky ? .96f : 0.f, a.sky ? 1.004f : 0.f, a.sky ? 1.118f : 0.f};
  double* term = sh;
  double* dprod = sh + a.P;
  if (!a.sky) {
    for (uint32_t k = threadIdx.x + 3; k < 3 * nsp; k += blockDim.x) parr[k] = 0.f;
  } else {
    // patch luminance (Perez all-weather relative luminance), then the normalisation term
    for (uint32_t p = threadIdx.x; p < a.P; p += blockDim.x) {
      const double aas = fabs((double)a.azi[p] - azimuth);
      const double zsa = PI * 0.5 - (double)a.alt[p];
      const double sspa = acos(cos(sz) * cos(zsa) + sin(sz) * sin(zsa) * cos(aas));
      float v = (float)((1.0 + sPar[0] * exp(sPar[1] / cos(zsa))) * (1.0 + sPar[2] * exp(sPar[3] * sspa) + sPar[4] * cos(sspa) * cos(sspa)));
      if (v < 0) v = 0;
      parr[3 * (p + 1)] = v;
      term[p] = v * tcos_d(a.costab, (double)a.alt[p] - (PI / 2.)) * a.omega[p];
    }
    __syncthreads();
    __shared__ double sNorm;
    __shared__ int sUniform;
    if (threadIdx.x == 0) {   // the reference's order: one sum, patch by patch
      double norm = 0.0;
      for (uint32_t p = 0; p < a.P; ++p) norm += term[p];
      sUniform = norm <= 1e-6;
      if (sUniform) norm = PI;
      sNorm = diff_illum / norm;
    }
    __syncthreads();
    const double sf = sNorm * (1. / WHTEFFICACY);
    for (uint32_t p = threadIdx.x; p < a.P; p += blockDim.x) {
      const float v = sUniform ? 1.f : parr[3 * (p + 1)];
      parr[3 * (p + 1)] = (float)(v * sf) * skyc[0];
      parr[3 * (p + 1) + 1] = (float)(v * sf) * skyc[1];
      parr[3 * (p + 1) + 2] = (float)(v * sf) * skyc[2];
    }
  }
  // AddDirect: the sun into the four nearest patches by proximity weight
  if (dir_illum <= 1e-4 || !a.sun) return;
  double sv[3];
  sv[1] = cos(altitude); sv[0] = sv[1] * sin(azimuth); sv[1] *= cos(azimuth); sv[2] = sin(altitude);
  for (uint32_t p = threadIdx.x; p < a.P; p += blockDim.x) {
    double pv[3];
    pv[1] = cos((double)a.alt[p]); pv[0] = pv[1] * sin((double)a.azi[p]); pv[1] *= cos((double)a.azi[p]); pv[2] = sin((double)a.alt[p]);
    dprod[p] = pv[0] * sv[0] + pv[1] * sv[1] + pv[2] * sv[2];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double near_d[4] = {-1., -1., -1., -1.};
    int near_p[4] = {0, 0, 0, 0};
    for (uint32_t p = 0; p < a.P; ++p) {
      const double d = dprod[p];
      for (int i = 0; i < 4; i++)
        if (d > near_d[i]) {
          for (int j = 3; j > i; --j) { near_d[j] = near_d[j - 1]; near_p[j] = near_p[j - 1]; }
          near_d[i] = d;
          near_p[i] = int(p) + 1;
          break;
        }
    }
    double wta[4], wtot = 0;
    for (int i = 4; i--;) wtot += wta[i] = 1. / (1.002 - near_d[i]);
    for (int i = 4; i--;) {
      float* pd = parr + 3 * near_p[i];
      float v = (float)(wta[i] * dir_illum / (WHTEFFICACY * wtot));
      v /= a.omega[near_p[i] - 1];
      pd[0] += v; pd[1] += v; pd[2] += v;
    }
  }
}

// NOAA solar position with ladybug's conventions (the reference's sun_noaa, solar.cpp:66-105), one thread per step.
struct SunArgs {
  const double* in;   // [T x 7]: lat, lon, tz, month, day, hourFrac, leap
  uint32_t T;
  double* out;        // [T x 6]: alt (deg), azi (deg), up, vec x, y, z (float values)
};
__device__ __forceinline__ double pymod(double a, double m) { const double r = fmod(a, m); return r < 0 ? r + m : r; }
// strtod(snprintf("%.2f", x)): x's exact binary value to 2 decimals, ties to even. x*100 as hi + lo (lo exact by fma),
// rint on hi, then the exact remainder decides the cases rint on the rounded product got wrong.
__device__ __forceinline__ double round2(double x) {
  const double hi = x * 100.0, lo = fma(x, 100.0, -hi);
  double n = rint(hi);
  const double f = (hi - n) + lo;
  if (f > 0.5) n += 1;
  else if (f < -0.5) n -= 1;
  return n / 100.0;
}
__global__ void k_sun(SunArgs a) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= a.T) return;
  const double* p = a.in + 7 * size_t(t);
  const double lat = p[0], lon = p[1], tz = p[2], hourFrac = p[5];
  const int month = int(p[3]), day = int(p[4]);
  const bool leap = p[6] != 0;
  const auto rad = [](double d) { return d * PI / 180; };
  const auto deg = [](double r) { return r * 180 / PI; };
  int hour = (int)hourFrac, minute = (int)llrint((hourFrac - hour) * 60);
  if (minute == 60) { ++hour; minute = 0; }
  const int dim[12] = {31, 28, 31, 30, 31, 30, 31, 31, 30, 31, 30, 31};
  int doy = day;
  for (int m = 1; m < month; ++m) doy += dim[m - 1] + (leap && m == 2 ? 1 : 0);
  const double jd = (leap ? 42368.0 : 42734.0) + doy + 1 + 2415018.5 + round2((minute + hour * 60) / 1440.0) - tz / 24;
  const double jc = (jd - 2451545) / 36525;
  const double L0 = pymod(280.46646 + jc * (36000.76983 + jc * 0.0003032), 360);
  const double M = 357.52911 + jc * (35999.05029 - 0.0001537 * jc);
  const double e = 0.016708634 - jc * (0.000042037 + 0.0000001267 * jc);
  const double C = sin(rad(M)) * (1.914602 - jc * (0.004817 + 0.000014 * jc)) + sin(rad(2 * M)) * (0.019993 - 0.000101 * jc) + sin(rad(3 * M)) * 0.000289;
  const double omega = rad(125.04 - 1934.136 * jc);
  const double lambda = rad(L0 + C - 0.00569 - 0.00478 * sin(omega));
  const double eps0 = 23 + (26 + (21.448 - jc * (46.815 + jc * (0.00059 - jc * 0.001813))) / 60) / 60;
  const double eps = rad(eps0 + 0.00256 * cos(omega));
  const double dec = asin(sin(eps) * sin(lambda));
  double y = tan(eps / 2);
  y *= y;
  const double eot = 4 * deg(y * sin(2 * rad(L0)) - 2 * e * sin(rad(M)) + 4 * e * y * sin(rad(M)) * cos(2 * rad(L0)) - 0.5 * y * y * sin(4 * rad(L0)) -
                             1.25 * e * e * sin(2 * rad(M)));
  const double tst = pymod(hourFrac * 60 + eot + 4 * lon - 60 * tz, 1440);
  const double H = tst < 0 ? tst / 4 + 180 : tst / 4 - 180;
  const double la = rad(lat);
  const double zen = acos(sin(la) * sin(dec) + cos(la) * cos(dec) * cos(rad(H)));
  const double alt = 90 - deg(zen), tt = tan(rad(alt));
  double r;
  if (alt > 85) r = 0;
  else if (alt > 5) r = 58.1 / tt - 0.07 / (tt * tt * tt) + 0.000086 / (tt * tt * tt * tt * tt);
  else if (alt > -0.575) r = 1735 + alt * (-518.2 + alt * (103.4 + alt * (-12.79 + alt * 0.711)));
  else r = -20.772 / tt;
  const double salt = alt + r / 3600;
  const double c = (sin(la) * cos(zen) - sin(dec)) / (cos(la) * sin(zen));
  double azi;
  if (c >= -1 && c <= 1) azi = pymod(H > 0 ? deg(acos(c)) + 180 : 540 - deg(acos(c)), 360);
  else azi = c > 0 ? 180 : 0;
  double* o = a.out + 6 * size_t(t);
  o[0] = salt; o[1] = azi; o[2] = salt >= 0 ? 1 : 0;
  const double ar = rad(salt), zr = rad(azi);
  double v1 = cos(ar);
  const double v0 = v1 * sin(zr);
  v1 *= cos(zr);
  o[3] = (float)v0; o[4] = (float)v1; o[5] = (float)sin(ar);
}

// ---------------------------------------------------------------------------------------------- ladybug mode
// The reference's --mode ladybug emulates gendaymtx -A as ladybug runs it (src/run.cpp:362-398 per step, 447-470 at the
// end): the sun by Radiance's sun.c at the site ladybug writes into its .wea (latitude and west longitude to 0.01
// degree, the zone's integer meridian), each step's DNI and DHI truncated to integers, the sky of each step twice (the
// sun alone, gendaymtx -d; the sky alone, -s), and per patch float sums over all steps in step order, averaged and
// printed to three significant digits.

// Radiance sun.c (rad5R4: sdec, stadj, salt, sazi), the reference's sun_radiance (src/sky.cpp:477-486), in FP64.
__device__ __forceinline__ void sun_rad(double latDeg, double lonW, double meridW, int jd, double hour, double& alt, double& azi) {
  const double lat = latDeg * (PI / 180.), lon = lonW * (PI / 180.), mer = meridW * (PI / 180.);
  const double sd = 0.4093 * sin((2. * PI / 365.) * (jd - 81));
  const double sta = 0.170 * sin((4. * PI / 373.) * (jd - 80)) - 0.129 * sin((2. * PI / 355.) * (jd - 8)) + (12. / PI) * (mer - lon);
  const double st = hour + sta;
  alt = asin(sin(lat) * sin(sd) - cos(lat) * cos(sd) * cos(st * (PI / 12.)));
  azi = -atan2(cos(sd) * sin(st * (PI / 12.)), -cos(lat) * sin(sd) - sin(lat) * cos(sd) * cos(st * (PI / 12.))) + PI;
}
// per step: the sky step of the .wea (jd, the sun by sun.c, DNI and DHI truncated to integers)
__global__ void k_lb_steps(const double* in, uint32_t T, double latW, double lonW, double meridW, kgb_sky_step* out) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  const double* p = in + 4 * size_t(t);
  kgb_sky_step s{};
  s.jd = int(p[0]);
  sun_rad(latW, lonW, meridW, s.jd, p[1], s.alt, s.azi);
  s.dni = double(int(p[2]));
  s.dhi = double(int(p[3]));
  out[t] = s;
}
// The float sums over the steps, in step order: accDir [P] (red of the sun rows), accDif [3 P], the ground row of the
// sun rows [3], of the sky rows [3]. One thread per sum.
__global__ void k_lb_acc(const float* dir, const float* dif, uint32_t T, uint32_t P, float* acc) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= 4 * P + 6) return;
  const float* src;
  uint32_t off;
  if (k < P) { src = dir; off = 3 * (k + 1); }
  else if (k < 4 * P) { src = dif; off = 3 + (k - P); }
  else if (k < 4 * P + 3) { src = dir; off = k - 4 * P; }
  else { src = dif; off = k - 4 * P - 3; }
  const size_t row = 3 * size_t(P + 1);
  float s = 0.f;
  for (uint32_t t = 0; t < T; ++t) s = __fadd_rn(s, src[t * row + off]);
  acc[k] = s;
}
// The series columns of the steps with DNI + DHI > 1e-4: S [p, col] = float(bright(sky row) + the sun row's red),
// g [col] = float(grefl x sum_p L_p omega_p / P), the sum in patch order. One block per step.
__global__ void k_lb_series(const float* dir, const float* dif, const int32_t* colOf, uint32_t T, uint32_t P, uint32_t Tup,
                            const float* omega, double grefl, float* S, float* g) {
  const uint32_t t = blockIdx.x;
  const int32_t col = colOf[t];
  if (col < 0) return;
  const size_t row = 3 * size_t(P + 1) * t;
  const auto L = [&](uint32_t p) {
    const float* df = dif + row + 3 * (p + 1);
    return __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(0.265074126, double(df[0])), __dmul_rn(0.670114631, double(df[1]))),
                               __dmul_rn(0.064811243, double(df[2]))), double(dir[row + 3 * (p + 1)]));
  };
  for (uint32_t p = threadIdx.x; p < P; p += blockDim.x) S[size_t(p) * Tup + uint32_t(col)] = __double2float_rn(L(p));
  if (threadIdx.x == 0) {
    double mean = 0;
    for (uint32_t p = 0; p < P; ++p) mean = __dadd_rn(mean, __dmul_rn(L(p), double(omega[p])));
    g[col] = __double2float_rn(__ddiv_rn(__dmul_rn(grefl, mean), double(P)));
  }
}

// make_patches (sky.cpp:240-270): Reinhart / Tregenza patch centres and solid angles, float as the reference's.
void make_patches(int mf, std::vector<float>& alt, std::vector<float>& azi, std::vector<float>& omega) {
  static const int tnaz[7] = {30, 30, 24, 24, 18, 12, 6};
  const double alpha = (PI / 2.) / (7 * mf + .5);
  alt.clear(); azi.clear(); omega.clear();
  for (int i = 0; i < 7 * mf; i++) {
    const float ralt = (float)(alpha * (i + .5));
    const int ninrow = tnaz[i / mf] * mf;
    const float dom = (float)(2. * PI * (std::sin(alpha * (i + 1)) - std::sin(alpha * i)) / (double)ninrow);
    for (int j = 0; j < ninrow; j++) {
      alt.push_back(ralt);
      azi.push_back((float)(2. * PI * j / (double)ninrow));
      omega.push_back(dom);
    }
  }
  alt.push_back((float)(PI / 2.));
  azi.push_back(0.f);
  omega.push_back((float)(2. * PI * (1. - std::cos(alpha * .5))));
}

const char* sky_steps(int mf, const kgb_sky_step* hsteps, size_t T, double grefl, int sun, int sky, int visible, float* hout, cudaStream_t st) {
  if (mf != 1 && mf != 2 && mf != 4) return "kgb_sky: sky density must be 1, 2 or 4";
  if (!T) return nullptr;
  std::vector<float> alt, azi, omega;
  make_patches(mf, alt, azi, omega);
  const uint32_t P = uint32_t(alt.size());
  std::vector<double> costab(1025);
  for (int i = 0; i <= 1024; i++) costab[i] = std::cos((PI / 2. / 1024) * i);
  const size_t outN = T * 3 * (P + 1);
  void* d = nullptr;
  const size_t bytes = T * sizeof(kgb_sky_step) + 3 * P * 4 + 1025 * 8 + outN * 4 + 1024;
  if (cudaMallocAsync(&d, bytes, st) != cudaSuccess) return "kgb_sky: device memory";
  char* b = static_cast<char*>(d);
  kgb_sky_step* dsteps = reinterpret_cast<kgb_sky_step*>(b);
  float* dalt = reinterpret_cast<float*>(b + ((T * sizeof(kgb_sky_step) + 255) & ~size_t(255)));
  float* dazi = dalt + P;
  float* dom = dazi + P;
  double* dcos = reinterpret_cast<double*>(reinterpret_cast<uintptr_t>(dom + P + 1) & ~uintptr_t(7));
  float* dout = reinterpret_cast<float*>(dcos + 1025);
  cudaMemcpyAsync(dsteps, hsteps, T * sizeof(kgb_sky_step), cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(dalt, alt.data(), P * 4, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(dazi, azi.data(), P * 4, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(dom, omega.data(), P * 4, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(dcos, costab.data(), 1025 * 8, cudaMemcpyHostToDevice, st);
  SkyArgs a{dsteps, uint32_t(T), P, dalt, dazi, dom, dcos, grefl, sun, sky, visible, dout};
  k_sky<<<uint32_t(T), 128, 2 * P * sizeof(double), st>>>(a);
  cudaMemcpyAsync(hout, dout, outN * 4, cudaMemcpyDeviceToHost, st);
  cudaFreeAsync(d, st);
  if (cudaStreamSynchronize(st) != cudaSuccess || cudaGetLastError() != cudaSuccess) return "kgb_sky: kernel failed";
  return nullptr;
}

// ladybug mode: the steps' sky rows on the device (k_sky twice), the float sums, the series columns; the weights (the
// averages printed to three significant digits, run.cpp:447-470) on the host from the downloaded sums, by the same
// snprintf / strtod round trip as the reference's round_fmt.
static double round_fmt(double x, const char* fmt) {
  char buf[64];
  std::snprintf(buf, sizeof buf, fmt, x);
  return std::strtod(buf, nullptr);
}
const char* sky_ladybug(int mf, const double* hsteps, size_t T, double lat, double lon, double tz, double grefl, double durationHours,
                        double* lb, float* hacc, float* hS, float* hg, cudaStream_t st) {
  if (mf != 1 && mf != 2) return "kgb_sky_ladybug: ladybug mode supports sky density 1 or 2 (the reference's rule)";
  if (!T) return nullptr;
  std::vector<float> alt, azi, omega;
  make_patches(mf, alt, azi, omega);
  const uint32_t P = uint32_t(alt.size());
  std::vector<double> costab(1025);
  for (int i = 0; i <= 1024; i++) costab[i] = std::cos((PI / 2. / 1024) * i);
  std::vector<int32_t> colOf(T, -1);
  uint32_t Tup = 0;
  for (size_t t = 0; t < T; ++t)
    if (float(hsteps[4 * t + 2]) + float(hsteps[4 * t + 3]) > 1e-4) colOf[t] = int32_t(Tup++);   // the Step's float DNI + DHI
  const size_t rowN = 3 * size_t(P + 1), nAcc = 4 * size_t(P) + 6;
  const auto a256 = [](size_t x) { return (x + 255) & ~size_t(255); };
  const size_t oSteps = 0, oSky = a256(oSteps + T * 4 * 8), oPatch = a256(oSky + T * sizeof(kgb_sky_step)), oCos = a256(oPatch + 3 * P * 4),
               oCol = a256(oCos + 1025 * 8), oDir = a256(oCol + T * 4), oDif = a256(oDir + T * rowN * 4), oAcc = a256(oDif + T * rowN * 4),
               oS = a256(oAcc + nAcc * 4), oG = a256(oS + size_t(P) * Tup * 4), total = a256(oG + size_t(Tup) * 4);
  void* d = nullptr;
  if (cudaMallocAsync(&d, total, st) != cudaSuccess) return "kgb_sky_ladybug: device memory";
  char* b = static_cast<char*>(d);
  double* dsteps = reinterpret_cast<double*>(b + oSteps);
  kgb_sky_step* dsky = reinterpret_cast<kgb_sky_step*>(b + oSky);
  float* dalt = reinterpret_cast<float*>(b + oPatch);
  float* dazi = dalt + P;
  float* dom = dazi + P;
  double* dcos = reinterpret_cast<double*>(b + oCos);
  int32_t* dcol = reinterpret_cast<int32_t*>(b + oCol);
  float* ddir = reinterpret_cast<float*>(b + oDir);
  float* ddif = reinterpret_cast<float*>(b + oDif);
  float* dacc = reinterpret_cast<float*>(b + oAcc);
  float* dS = reinterpret_cast<float*>(b + oS);
  float* dg = reinterpret_cast<float*>(b + oG);
  cudaMemcpyAsync(dsteps, hsteps, T * 4 * 8, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(dalt, alt.data(), P * 4, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(dazi, azi.data(), P * 4, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(dom, omega.data(), P * 4, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(dcos, costab.data(), 1025 * 8, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(dcol, colOf.data(), T * 4, cudaMemcpyHostToDevice, st);
  // the .wea's site: latitude and west longitude printed to 0.01 degree, the zone's meridian an integer of degrees west
  const double latW = round_fmt(lat, "%.2f"), lonW = round_fmt(-lon, "%.2f"), meridW = static_cast<double>(static_cast<int>(-tz * 15.0));
  k_lb_steps<<<uint32_t((T + 127) / 128), 128, 0, st>>>(dsteps, uint32_t(T), latW, lonW, meridW, dsky);
  SkyArgs a{dsky, uint32_t(T), P, dalt, dazi, dom, dcos, grefl, 1, 0, 0, ddir};
  k_sky<<<uint32_t(T), 128, 2 * P * sizeof(double), st>>>(a);   // -d: the sun alone
  a.sun = 0; a.sky = 1; a.out = ddif;
  k_sky<<<uint32_t(T), 128, 2 * P * sizeof(double), st>>>(a);   // -s: the sky alone
  k_lb_acc<<<uint32_t((nAcc + 127) / 128), 128, 0, st>>>(ddir, ddif, uint32_t(T), P, dacc);
  if (hS || hg) k_lb_series<<<uint32_t(T), 128, 0, st>>>(ddir, ddif, dcol, uint32_t(T), P, Tup, dom, grefl, dS, dg);
  std::vector<float> acc(nAcc);
  cudaMemcpyAsync(acc.data(), dacc, nAcc * 4, cudaMemcpyDeviceToHost, st);
  if (hS) cudaMemcpyAsync(hS, dS, size_t(P) * Tup * 4, cudaMemcpyDeviceToHost, st);
  if (hg) cudaMemcpyAsync(hg, dg, size_t(Tup) * 4, cudaMemcpyDeviceToHost, st);
  cudaFreeAsync(d, st);
  if (cudaStreamSynchronize(st) != cudaSuccess || cudaGetLastError() != cudaSuccess) return "kgb_sky_ladybug: kernel failed";
  if (hacc) std::memcpy(hacc, acc.data(), nAcc * 4);
  // run.cpp:447-470: averages over all steps in float, printed %.3g; weights kWh/m2 per unit of radiance x solid angle
  const float inv = static_cast<float>(1.0 / static_cast<double>(T));
  double mean = 0;
  for (uint32_t p = 0; p < P; ++p) {
    const float avgDir = T > 1 ? acc[p] * inv : acc[p];
    const float r = T > 1 ? acc[P + 3 * p] * inv : acc[P + 3 * p];
    const float gch = T > 1 ? acc[P + 3 * p + 1] * inv : acc[P + 3 * p + 1];
    const float bch = T > 1 ? acc[P + 3 * p + 2] * inv : acc[P + 3 * p + 2];
    const double rd = round_fmt(avgDir, "%.3g"), rr = round_fmt(r, "%.3g"), rg = round_fmt(gch, "%.3g"), rb = round_fmt(bch, "%.3g");
    lb[p] = rd * omega[p] * durationHours / 1000.0;
    lb[P + p] = (0.265074126 * rr + 0.670114631 * rg + 0.064811243 * rb) * omega[p] * durationHours / 1000.0;
    lb[2 * P + p] = lb[p] + lb[P + p];
    mean += lb[2 * P + p];
  }
  lb[3 * P] = grefl * mean / static_cast<double>(P);
  return nullptr;
}

const char* sun_steps(const double* hin, size_t T, double* hout, cudaStream_t st) {
  if (!T) return nullptr;
  void* d = nullptr;
  if (cudaMallocAsync(&d, T * 13 * 8, st) != cudaSuccess) return "kgb_sun_noaa: device memory";
  double* din = static_cast<double*>(d);
  double* dout = din + 7 * T;
  cudaMemcpyAsync(din, hin, T * 7 * 8, cudaMemcpyHostToDevice, st);
  k_sun<<<uint32_t((T + 127) / 128), 128, 0, st>>>(SunArgs{din, uint32_t(T), dout});
  cudaMemcpyAsync(hout, dout, T * 6 * 8, cudaMemcpyDeviceToHost, st);
  cudaFreeAsync(d, st);
  if (cudaStreamSynchronize(st) != cudaSuccess || cudaGetLastError() != cudaSuccess) return "kgb_sun_noaa: kernel failed";
  return nullptr;
}

}  // namespace kgb
