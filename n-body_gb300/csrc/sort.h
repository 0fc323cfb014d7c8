// Stable radix sort of (63-bit key, 32-bit value) pairs (internal to the library).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace nbody {

// Scratch bytes sort_pairs needs for n pairs.
size_t sort_scratch_bytes(int64_t n);

// Sorts (keys, vals) stably by the low 8 * passes bits of the key (passes
// 1..8; 8 covers a 63-bit key); keys_alt / vals_alt are ping-pong buffers of
// the same size. On return *result_in_alt says which pair of buffers holds the
// sorted result. `status` is the device status word. Launch attributes are set
// on the first call per device (sort_prepare), so later calls may be captured
// into a CUDA graph.
cudaError_t sort_pairs(uint64_t *keys, uint32_t *vals, uint64_t *keys_alt, uint32_t *vals_alt, int64_t n,
                       void *scratch, cudaStream_t stream, int *status, int *result_in_alt, int passes = 8);
cudaError_t sort_prepare(int device);

}  // namespace nbody
