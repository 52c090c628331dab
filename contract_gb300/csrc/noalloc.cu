// Fixed-size device scratch for the allocation-free entry point
// (contract_baryon_all_types_noalloc in contract_gb300.h).
//
// Some callers cannot let the library call cudaMalloc: a host framework whose
// pool allocator already owns the free device memory (QUDA/PyQUDA-style
// setups reserve most of it up front), code that must not hit cudaMalloc's
// implicit device synchronisation in a latency-critical loop, or plugin hosts
// that require, as CLQCD/contract's own library does, that a contraction
// library allocate nothing.  For them the per-timeslice partial sums go into
// this file-scope array instead of the growable per-device workspace.
//
// The array is part of the module image: every GPU that loads the library
// holds its kStaticScratchBytes until the process exits.  In host code the
// symbol is only a host-side stand-in, so its device address is looked up
// once per device, with that device current, via cudaGetSymbolAddress.
#include <mutex>

#include "launch.hpp"

namespace cgb {

constexpr size_t kStaticScratchBytes = size_t(16) << 20;  // 16 MiB

static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

// Device address of g_static_scratch on the current device.  The first call on
// a device resolves it (cudaGetSymbolAddress); later calls reuse the cached
// address.  Resolving is not a stream operation, but it should happen before
// any stream capture that includes the entry point.
cudaError_t static_scratch(void **ptr, size_t *bytes)
{
  static std::mutex mu;
  static void *addr[64] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(mu);
  if (!addr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess) return e;
    addr[dev] = p;
  }
  *ptr = addr[dev];
  *bytes = kStaticScratchBytes;
  return cudaSuccess;
}

} // namespace cgb
