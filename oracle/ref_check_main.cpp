// TEST INFRASTRUCTURE ONLY. Runs the reference's own module checks (kit-sim_daylight tests/check_sky.cpp,
// tests/check_gpu.cpp, tests/check_views.cpp, tests/check_mesh.cpp, compiled unchanged from the reference tree) against
// the oracle behind the engine's C++ shim; check_mesh's n-gon cases run on the engine's restatement of earcut
// (include/kgb_earcut.h, through oracle/ref_shims/mapbox/earcut.hpp). check_solar needs an EPW file the reference tree
// lacks, so it is not run.
#include <cstdio>
#include <cstring>
int check_sky(const char* testsDir);
int check_gpu(const char* testsDir);
int check_views(const char* testsDir);
int check_mesh(const char* testsDir);
int main(int argc, char** argv) {
  const char* dir = argc > 1 ? argv[1] : "tests";
  const char* only = argc > 2 ? argv[2] : "";
  int failures = 0;
  if (!*only || !std::strcmp(only, "sky")) failures += check_sky(dir);
  if (!*only || !std::strcmp(only, "gpu")) failures += check_gpu(dir);
  if (!*only || !std::strcmp(only, "views")) failures += check_views(dir);
  if (!*only || !std::strcmp(only, "mesh")) failures += check_mesh(dir);
  std::printf("%s: %d failure(s)\n", failures ? "FAIL" : "OK", failures);
  return failures ? 1 : 0;
}
