// Launch scratch for gbrkc_advance_noalloc (engine.cpp): the persistent
// launch's per-role work-queue counters and per-CTA start / end timestamps,
// held in this file's static device array instead of memory the engine
// allocates.  Every GPU that loads the library holds the array
// (NOALLOC_SCRATCH_WORDS * 8 bytes = 16.6 KB) until the process exits.
//
// Host code may not use the array's name as a device address (on the host it
// names a host-side stand-in): the address is looked up here with
// cudaGetSymbolAddress while the engine's device is current.  gbrkc_build
// calls this once per persistent engine and keeps the result in the engine,
// so an engine built after a device reset (which reloads this module) gets
// the reloaded array's address, and the advance itself looks nothing up.
#include <cuda_runtime.h>

#include "noalloc.h"

namespace gbrkc {

namespace {

static __device__ __align__(256) unsigned long long g_scratch[NOALLOC_SCRATCH_WORDS];

}  // namespace

int noalloc_scratch(unsigned long long **ptr) {
  void *p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
  if (e != cudaSuccess) return (int)e;
  *ptr = (unsigned long long *)p;
  return 0;
}

}  // namespace gbrkc
