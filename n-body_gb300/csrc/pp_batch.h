// Direct sum over an ensemble of packed systems (internal to the library).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace nbody {

// Launch shapes (threads x i-bodies per thread).
constexpr int kPPBatch128x2 = 0;
constexpr int kPPBatch256x2 = 1;
constexpr int kPPBatch256x4 = 2;
constexpr int kPPBatch128x4 = 3;
constexpr int kPPBatchShapes = 4;

// i-bodies per work item for a shape.
int pp_batch_bodies_per_item(int shape);
// Persistent grid: min(items, resident CTAs on the device).
int pp_batch_ctas(int shape, int device, int nitems);

// One step of every system: items[k] = {system, first i-body}, largest
// systems first; sys_range[s] = {first body, count, -, -}; sys_prm[s] = {dt,
// eps2, -, euler}. sched = 2 unsigned that must be 0 before the first launch
// (the kernel leaves them at 0). pos -> pos_out, vel / acc in place.
cudaError_t pp_batch_launch(int shape, int ctas, const float4 *pos, float4 *pos_out, float4 *vel, float4 *acc,
                            const int2 *items, int nitems, const int4 *sys_range, const float4 *sys_prm,
                            unsigned *sched, cudaStream_t st, int *status);

}  // namespace nbody
