// oic_prims.cuh -- device-wide primitives written for the engine: exclusive scan and a
// stable LSD radix sort of (uint64 key, uint32 value) pairs.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace oic {

// Kernels this host thread has launched through the library (for launch accounting).
// Per thread: a context is driven by one thread at a time, so the difference across a
// call counts that call's launches even while other threads drive other contexts.
extern thread_local unsigned long long g_launches;

// Scratch bytes oic_scan_u32 needs for n elements.
size_t scan_u32_scratch(uint64_t n);
// out[i] = sum(in[0..i)) for i < n, and *total (device pointer, may be null) = sum(in).
// `in` and `out` may alias.  n < 2^32.
cudaError_t scan_u32(const uint32_t *in, uint32_t *out, uint64_t n, uint32_t *total, void *scratch, cudaStream_t st);

// Scratch bytes radix_sort needs for n elements (double buffers are separate).
size_t radix_sort_scratch(uint64_t n);
// Stable ascending sort of keys/vals on key bits [0, bits).  keys/vals are sorted in
// place; keysAlt/valsAlt are buffers of the same size used for ping-pong.  With nDev
// non-null the launches are sized for n keys and sort the first min(n, *nDev) (a count
// known only on the device, e.g. inside a captured graph).
cudaError_t radix_sort_u64_u32(unsigned long long *keys, uint32_t *vals, unsigned long long *keysAlt, uint32_t *valsAlt, uint64_t n,
                               int bits, void *scratch, cudaStream_t st, const uint32_t *nDev = nullptr);

}  // namespace oic
