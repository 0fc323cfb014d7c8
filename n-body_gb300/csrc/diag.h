// FP64 conservation diagnostics (internal to the library).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace nbody {

constexpr int kDiagBlocks = 512;

// Scratch for diag_momenta (block partials and a counter that must start at 0).
size_t diag_scratch_bytes();

// out_dev[0..7] (device, double) = kinetic energy, potential energy
// (0.5 sum m_i phi_i, or 0 when phi is null), linear momentum xyz, angular
// momentum xyz, for n bodies (pos float4 with mass in w, vel float4).
cudaError_t diag_momenta(const float4 *pos, const float4 *vel, const float *phi, int64_t n, void *scratch,
                         double *out_dev, cudaStream_t st);

// Direct-sum potential per body (self pair excluded), FP32.
cudaError_t diag_pp_potential(const float4 *pos, int64_t n, float eps2, float *phi, cudaStream_t st);

}  // namespace nbody
