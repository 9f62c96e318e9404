// Static launch scratch of gbrkc_advance_noalloc (noalloc.cu).
#pragma once

namespace gbrkc {

// Most CTAs a persistent launch may have on this path (one GB300 runs 152).
constexpr int NOALLOC_MAX_CTAS = 1024;
// Layout in 8-byte words: [0, 32) the work-queue counters (as ints, one per
// role), then NOALLOC_MAX_CTAS start stamps, then NOALLOC_MAX_CTAS end stamps.
constexpr int NOALLOC_QUEUE_WORDS = 32;
constexpr int NOALLOC_SCRATCH_WORDS = NOALLOC_QUEUE_WORDS + 2 * NOALLOC_MAX_CTAS;

// Device address of the scratch on the current device (a fresh lookup on
// every call; gbrkc_build makes it once per persistent engine).  Returns 0 or
// a cudaError_t code.
int noalloc_scratch(unsigned long long **ptr);

}  // namespace gbrkc
