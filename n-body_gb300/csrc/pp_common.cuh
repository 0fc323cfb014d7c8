// Direct-sum pieces shared by the single-system and the ensemble kernels
// (internal to the library).
#pragma once

#include "common.cuh"
#include "kernels.h"

namespace nbody {

constexpr int kPPTile = 256;    // j-bodies per stage (4 KiB)
constexpr int kPPStages = 3;

__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }

// Reference integrator, one body. Each operation is rounded on its own
// (no FMA contraction), matching the reference's scalar evaluation.
__device__ __forceinline__ void integrate_body(int64_t i, float4 p, float fx, float fy, float fz,
                                               const Integrate &g) {
    const float dt = g.dt;
    const float h = __fmul_rn(dt, 0.5f);
    float4 v = g.vel[i];
    const float4 anew = make_float4(fx, fy, fz, 0.f);
    if (g.euler) {
        // updateParticles.glsl:44-55: v += F dt, then x += v dt.
        v.x = __fadd_rn(v.x, __fmul_rn(fx, dt));
        v.y = __fadd_rn(v.y, __fmul_rn(fy, dt));
        v.z = __fadd_rn(v.z, __fmul_rn(fz, dt));
        p.x = __fadd_rn(p.x, __fmul_rn(v.x, dt));
        p.y = __fadd_rn(p.y, __fmul_rn(v.y, dt));
        p.z = __fadd_rn(p.z, __fmul_rn(v.z, dt));
        g.pos_out[i] = p;
        g.vel[i] = v;
        g.acc[i] = anew;
        if (g.force) g.force[i] = anew;
        return;
    }
    const float4 a = g.acc[i];
    v.x = __fadd_rn(v.x, __fmul_rn(a.x, h));
    v.y = __fadd_rn(v.y, __fmul_rn(a.y, h));
    v.z = __fadd_rn(v.z, __fmul_rn(a.z, h));
    p.x = __fadd_rn(p.x, __fmul_rn(v.x, dt));
    p.y = __fadd_rn(p.y, __fmul_rn(v.y, dt));
    p.z = __fadd_rn(p.z, __fmul_rn(v.z, dt));
    v.x = __fadd_rn(v.x, __fmul_rn(fx, h));
    v.y = __fadd_rn(v.y, __fmul_rn(fy, h));
    v.z = __fadd_rn(v.z, __fmul_rn(fz, h));
    g.pos_out[i] = p;  // w keeps the mass
    g.vel[i] = v;
    g.acc[i] = anew;
    if (g.force) g.force[i] = anew;
}

}  // namespace nbody
