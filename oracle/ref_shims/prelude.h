/* TEST INFRASTRUCTURE ONLY. Force-included when the reference's host sources (kit-sim_daylight src/*.cpp, tests/*.cpp)
 * are compiled on Linux with g++ for the oracle harness (oracle/Makefile, target `ref`):
 *  - glibc's <time.h> declares a global `int daylight`, which clashes with the reference's `namespace daylight`: the
 *    header is included first, then the namespace is renamed for the whole translation unit;
 *  - _ftelli64 (MSVC, src/mesh.cpp:356, 484) is ftello64 on glibc. */
#include <time.h>
#include <stdio.h>
#define daylight dlref
#define _ftelli64 ftello64
