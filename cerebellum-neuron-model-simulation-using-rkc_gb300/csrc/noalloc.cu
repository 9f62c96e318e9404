// Launch scratch for gbrkc_advance_noalloc (engine.cpp): the persistent
// launch's per-role work-queue counters and per-CTA start / end timestamps,
// held in this file's static device array instead of memory the engine
// allocates.  Every GPU that loads the library holds the array
// (NOALLOC_SCRATCH_WORDS * 8 bytes = 16.6 KB) until the process exits.
//
// Host code may not use the array's name as a device address (on the host it
// names a host-side stand-in): the address is looked up here, once per
// device, with cudaGetSymbolAddress while that device is current.
#include <cuda_runtime.h>

#include "noalloc.h"

namespace gbrkc {

namespace {

static __device__ __align__(256) unsigned long long g_scratch[NOALLOC_SCRATCH_WORDS];

constexpr int MAX_DEVICES = 64;
unsigned long long *g_addr[MAX_DEVICES] = {};

}  // namespace

int noalloc_scratch(unsigned long long **ptr) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return (int)e;
  if (dev < 0 || dev >= MAX_DEVICES) return (int)cudaErrorInvalidDevice;
  if (!g_addr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess) return (int)e;
    g_addr[dev] = (unsigned long long *)p;
  }
  *ptr = g_addr[dev];
  return 0;
}

}  // namespace gbrkc
