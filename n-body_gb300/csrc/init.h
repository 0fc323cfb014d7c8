// Seeded device-side initial conditions (internal to the library).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "nbody_gb300.h"

namespace nbody {

struct InitParams {
    float p[NBODY_INIT_MAX_PARAMS];
};

bool init_kind_valid(int kind);
InitParams init_defaults(int kind);

// Writes pos (x, y, z, m), vel (x, y, z, 0) and acc = 0 for n bodies of the
// given NBODY_INIT_* kind on stream st.
cudaError_t init_state(int kind, uint64_t seed, int64_t n, const InitParams &prm, float4 *pos, float4 *vel,
                       float4 *acc, cudaStream_t st);

}  // namespace nbody
