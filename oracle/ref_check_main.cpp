// TEST INFRASTRUCTURE ONLY. Runs the reference's own module checks (kit-sim_daylight tests/check_sky.cpp,
// tests/check_gpu.cpp, tests/check_views.cpp, compiled unchanged from the reference tree) against the oracle behind
// the engine's C++ shim. check_solar needs an EPW file the reference tree lacks, check_mesh's n-gon cases need earcut:
// neither is on the ray-cast-and-accumulate path, so they are not run (check_mesh.cpp is linked for box_mesh).
#include <cstdio>
#include <cstring>
int check_sky(const char* testsDir);
int check_gpu(const char* testsDir);
int check_views(const char* testsDir);
int main(int argc, char** argv) {
  const char* dir = argc > 1 ? argv[1] : "tests";
  const char* only = argc > 2 ? argv[2] : "";
  int failures = 0;
  if (!*only || !std::strcmp(only, "sky")) failures += check_sky(dir);
  if (!*only || !std::strcmp(only, "gpu")) failures += check_gpu(dir);
  if (!*only || !std::strcmp(only, "views")) failures += check_views(dir);
  std::printf("%s: %d failure(s)\n", failures ? "FAIL" : "OK", failures);
  return failures ? 1 : 0;
}
