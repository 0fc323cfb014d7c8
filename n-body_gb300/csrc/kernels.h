// Host-side declarations of the kernel launchers (internal to the library).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace nbody {

// Reference-order integrator outputs (include/ParticleSystem.h:52-69).
// pos_out == nullptr means "forces only".
struct Integrate {
    float4 *pos_out = nullptr;
    float4 *vel = nullptr;
    float4 *acc = nullptr;
    float4 *force = nullptr;  // optional copy of the new acceleration
    float dt = 0.f;
    int euler = 0;  // 1: the GLSL path's semi-implicit Euler (updateParticles.glsl:44-55)
};

// Optional per-stage timing: when set, launchers record a CUDA event pair
// around each kernel on the launch stream (see capi.cu: nbody_profile_*).
enum Stage {
    kStagePPForce = 0,
    kStagePack,
    kStageBBox,
    kStageMorton,
    kStageSort,
    kStageGather,
    kStageBuild,
    kStageUpsweep,
    kStageTraverse,
    kStageCount
};

struct StageTimer {
    virtual ~StageTimer() = default;
    virtual void begin(int stage, cudaStream_t s) = 0;
    virtual void end(int stage, cudaStream_t s) = 0;
};

// Launch shape of the direct-sum force kernel for one n.
struct PPPlan {
    int k = 4;          // i-bodies per thread
    int threads = 128;  // threads per CTA
    int slices = 1;     // j-slices (CTAs per i-block); 0 with the linear split
    int iblocks = 0;    // i-blocks of threads*k bodies
    int linear_ctas = 0;  // > 0: linear split of the (i-block, j-pair) work over this many CTAs
    size_t arrivals_bytes = 0; // per-i-block arrival counters at the start of scratch (zeroed once)
    size_t partial_bytes = 0;  // total scratch: counters + per-slice partial accelerations
};

PPPlan pp_plan(int64_t n, int device, bool allow_linear = true);

// pp_plan with the slice count lowered until the scratch it needs fits in
// `scratch_bytes` (one slice needs none).
PPPlan pp_plan_within(int64_t n, int device, size_t scratch_bytes);

// Direct-sum forces at `pos` (float4 x,y,z,m) followed by the integrator
// (or a plain force write when g.pos_out is null). When plan.slices > 1 or
// plan.linear_ctas > 0, `scratch` must hold plan.partial_bytes and its first plan.arrivals_bytes
// must be zero before the first launch (the kernel leaves them zero again).
// `status` is a device int.
cudaError_t pp_launch(const PPPlan &plan, const float4 *pos, int64_t n, float eps2, const Integrate &g,
                      void *scratch, cudaStream_t stream, int *status, StageTimer *timer = nullptr);

// Packs the reference host layout into the device layout and back.
cudaError_t pack_state(const float4 *positions4, const float4 *masses4, float4 *pos_mass, int64_t n,
                       cudaStream_t stream);
cudaError_t unpack_positions(const float4 *pos_mass, float4 *positions4, int64_t n, cudaStream_t stream);
// masses4[ids ? ids[i] : i] = (m_i, 0, 0, 0): the reference's vec4 mass layout.
cudaError_t unpack_masses(const float4 *pos_mass, const int *ids, float4 *masses4, int64_t n, cudaStream_t stream,
                          int *status);
// The same moves straight between device state and page-locked host buffers,
// given their device-mapped addresses (hostio.cu): vel_h / acc_h may be null
// (zeros in); any output may be null; with ids (device) the state is in sorted
// order and out[ids[i]] = in[i], through the inverse order built in `inv`
// (n ints of device scratch).
// host_mapped: the address on `device` of a page-locked host buffer registered
// with that device whose page-locked range holds all `bytes` from p, or
// nullptr for any other pointer (pageable memory, device memory, another
// device's page-locked memory, a range shorter than `bytes`, or not 16-byte
// aligned).
float4 *host_mapped(const void *p, size_t bytes, int device);
// pos_mass[i].w = masses4[i].x (device arrays).
cudaError_t merge_masses(float4 *pos_mass, const float4 *masses4, int64_t n, cudaStream_t stream);
cudaError_t host_gather(const float4 *positions4, const float4 *masses4, const float4 *vel_h, const float4 *acc_h,
                        float4 *pos_mass, float4 *vel, float4 *acc, int64_t n, cudaStream_t stream);
cudaError_t host_scatter(const float4 *pos_mass, const float4 *vel, const float4 *acc, const int *ids, int *inv,
                         float4 *positions4, float4 *vel_h, float4 *acc_h, float4 *force_h, float4 *masses_h,
                         int64_t n, cudaStream_t stream, int *status);

}  // namespace nbody
