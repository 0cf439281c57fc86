// kgb_reduce_noalloc: kgb_reduce for callers that must not allocate device memory when they call it.
//
// Who cannot allocate: a host application that reserves the GPU's memory for its own pool when it starts and leaves
// nothing for a plugin's cudaMalloc, or a plugin host whose processing loop forbids device allocation (an allocation
// there fails, or stalls the loop and breaks the host's accounting). kgb_reduce stages the host weights and the
// per-sensor sums in engine buffers that it grows on demand, so its first call, or a call with more sensors than
// before, allocates. This entry point runs the same reduce kernels on the same trace and stages the weights and the
// sums in one fixed array of device memory that is part of the library image instead: it calls no cudaMalloc,
// cudaFree or allocating library routine.
//
// Limits and sharing:
//  - the array is kNoAllocScratchBytes (1 MiB) on each device, held by every GPU that loads the library until the
//    process exits. The nDir weights (4 bytes each, rounded up to 256 bytes) plus the nc sums (8 bytes each) must
//    fit: with 5610 directions that is up to 128,256 sensors per call. A larger call fails with a message that gives
//    the limit;
//  - every call on a device uses the same array, so calls whose work overlaps on the GPU (from other threads, or
//    other engines on the same device) race. Each call waits for its own work before it returns, so calls made one
//    after another do not overlap;
//  - the array keeps the last call's contents; nothing in it needs clearing, because the weights are copied in and
//    every sum is written before it is read;
//  - the first call on a device looks up the array's device address (cudaGetSymbolAddress, with that device
//    current) and keeps it for the process: make that first call before any stream capture.
#include "engine.h"

#include <mutex>
#include <string>

namespace kgb {

constexpr size_t kNoAllocScratchBytes = size_t(1) << 20;
constexpr int kNoAllocMaxDevices = 64;
// In host code this name stands for the array; its device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_reduce_scratch[kNoAllocScratchBytes];

// The array's device address on the given device (looked up once per device); null and a message on failure.
static unsigned char* scratch_on(int device, std::string& err) {
  static std::mutex m;
  static unsigned char* addr[kNoAllocMaxDevices] = {};
  if (device < 0 || device >= kNoAllocMaxDevices) { err = "kgb_reduce_noalloc: device index beyond 63"; return nullptr; }
  std::lock_guard<std::mutex> lk(m);
  if (!addr[device]) {
    int prev = 0;
    if (cudaGetDevice(&prev) != cudaSuccess) { err = "kgb_reduce_noalloc: cudaGetDevice failed"; return nullptr; }
    if (prev != device && cudaSetDevice(device) != cudaSuccess) { err = "kgb_reduce_noalloc: cannot make the engine's device current"; return nullptr; }
    unsigned char* p = nullptr;
    const cudaError_t rc = cudaGetSymbolAddress(reinterpret_cast<void**>(&p), g_reduce_scratch);
    if (prev != device) cudaSetDevice(prev);
    if (rc != cudaSuccess) { err = std::string("kgb_reduce_noalloc: cudaGetSymbolAddress failed: ") + cudaGetErrorString(rc); return nullptr; }
    addr[device] = p;
  }
  return addr[device];
}

}  // namespace kgb

using namespace kgb;

extern "C" KGB_API int kgb_reduce_noalloc(kgb_engine* e, size_t nc, const float* W, int useCos, double* out) {
  if (!e) return set_error("kgb_reduce_noalloc: no engine");
  ReduceInputs in{};
  engine_reduce_inputs(e, in);
  if (nc == 0) return 1;
  if (nc != in.visN) return set_error("kgb_reduce_noalloc: no trace of this chunk");
  const size_t wBytes = (in.nDir * 4 + 255) & ~size_t(255);
  if (wBytes + nc * 8 > kNoAllocScratchBytes) {
    const size_t most = wBytes < kNoAllocScratchBytes ? (kNoAllocScratchBytes - wBytes) / 8 : 0;
    return set_error("kgb_reduce_noalloc: " + std::to_string(nc) + " sensors x 8 bytes + " + std::to_string(in.nDir) +
                     " weights x 4 bytes exceed its " + std::to_string(kNoAllocScratchBytes) + "-byte array (at most " +
                     std::to_string(most) + " sensors per call with these directions)");
  }
  std::string err;
  unsigned char* s = scratch_on(in.device, err);
  if (!s) return set_error(err);
  float* dW = reinterpret_cast<float*>(s);
  double* dOut = reinterpret_cast<double*>(s + wBytes);
  if (cudaMemcpyAsync(dW, W, in.nDir * 4, cudaMemcpyHostToDevice, in.st) != cudaSuccess)
    return set_error("kgb_reduce_noalloc: the weights' upload failed");
  if (in.bytes) launch_reduce_bytes(in.bytesVis, uint32_t(nc), uint32_t(in.nDir), in.N, in.D, dW, useCos, dOut, in.st);
  else launch_reduce_bits(in.bitsVis, uint32_t(nc), uint32_t(in.nWords), uint32_t(in.nDir), in.N, in.D, dW, useCos, dOut, in.st);
  if (cudaGetLastError() != cudaSuccess) return set_error("kgb_reduce_noalloc: the reduce launch failed");
  if (cudaMemcpyAsync(out, dOut, nc * 8, cudaMemcpyDeviceToHost, in.st) != cudaSuccess)
    return set_error("kgb_reduce_noalloc: the sums' download failed");
  if (cudaStreamSynchronize(in.st) != cudaSuccess) return set_error("kgb_reduce_noalloc: the reduce failed");
  return 1;
}
