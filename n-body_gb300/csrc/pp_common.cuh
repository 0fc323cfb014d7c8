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

// The inner loop: forces on this thread's K i-bodies from npr j-pairs laid out
// {x0 x1 y0 y1}{z0 z1 m0 m1}, two interactions per packed f32x2 instruction
// (12 FADD2/FFMA2/FMUL2 + 2 MUFU.RSQ per pair of interactions). nx/ny/nz hold
// the negated i-positions duplicated in both halves. GUARD drops pairs at zero
// distance (needed when eps2 == 0).
template <int K, bool GUARD>
__device__ __forceinline__ void pair_forces(const float4 *__restrict__ pr, int npr, const float2 (&nx)[K],
                                            const float2 (&ny)[K], const float2 (&nz)[K], float2 e2,
                                            float2 (&ax)[K], float2 (&ay)[K], float2 (&az)[K]) {
#pragma unroll 2
    for (int q = 0; q < npr; ++q) {
        const float4 u = pr[2 * q];
        const float4 v = pr[2 * q + 1];
        const float2 xj = f2(u.x, u.y), yj = f2(u.z, u.w), zj = f2(v.x, v.y), mj = f2(v.z, v.w);
#pragma unroll
        for (int r = 0; r < K; ++r) {
            const float2 dx = __fadd2_rn(xj, nx[r]);
            const float2 dy = __fadd2_rn(yj, ny[r]);
            const float2 dz = __fadd2_rn(zj, nz[r]);
            float2 r2 = __ffma2_rn(dx, dx, e2);
            r2 = __ffma2_rn(dy, dy, r2);
            r2 = __ffma2_rn(dz, dz, r2);
            float2 inv = f2(rsqrt_ftz(r2.x), rsqrt_ftz(r2.y));
            if (GUARD) {
                inv.x = r2.x > 0.f ? inv.x : 0.f;
                inv.y = r2.y > 0.f ? inv.y : 0.f;
            }
            const float2 inv2 = __fmul2_rn(inv, inv);
            const float2 s = __fmul2_rn(__fmul2_rn(mj, inv), inv2);
            ax[r] = __ffma2_rn(dx, s, ax[r]);
            ay[r] = __ffma2_rn(dy, s, ay[r]);
            az[r] = __ffma2_rn(dz, s, az[r]);
        }
    }
}

// Shared-memory staging of one CTA: the TMA landing ring and the j-pair tile.
struct Ring {
    float4 (*tile)[kPPTile];
    float4 *pairs;
    uint64_t *full;
};

// Accumulates the forces on this thread's K i-bodies from bodies [j0, j1),
// through the TMA ring; `gt` counts the tiles this CTA has consumed (ring
// position and mbarrier phase). Returns false if a copy never landed.
template <int K, int T, bool GUARD>
__device__ bool item_forces(const float4 *__restrict__ pos, int64_t j0, int64_t j1, const float2 (&nx)[K],
                            const float2 (&ny)[K], const float2 (&nz)[K], float2 (&ax)[K], float2 (&ay)[K],
                            float2 (&az)[K], float eps2, Ring ring, uint32_t &gt, int *status) {
    const int tid = threadIdx.x;
    const int64_t len = j1 - j0;
    const int ntiles = static_cast<int>((len + kPPTile - 1) / kPPTile);
    auto issue = [&](int t) {
        const uint32_t g = gt + static_cast<uint32_t>(t);
        const int stage = static_cast<int>(g % kPPStages);
        const int64_t jt = j0 + static_cast<int64_t>(t) * kPPTile;
        const int cnt = static_cast<int>((j1 - jt) < kPPTile ? (j1 - jt) : kPPTile);
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(&ring.full[stage], static_cast<uint32_t>(cnt) * 16u);
        tma_bulk_g2s(&ring.tile[stage][0], pos + jt, static_cast<uint32_t>(cnt) * 16u, &ring.full[stage]);
    };
    if (tid == 0)
        for (int t = 0; t < kPPStages && t < ntiles; ++t) issue(t);
    const float2 e2 = f2(eps2, eps2);
    for (int t = 0; t < ntiles; ++t) {
        const uint32_t g = gt + static_cast<uint32_t>(t);
        const int stage = static_cast<int>(g % kPPStages);
        const uint32_t parity = (g / kPPStages) & 1u;
        const bool ok = mbar_wait_bounded(&ring.full[stage], parity, status);
        if (!__syncthreads_and(ok)) {
            // Drain the copies still in flight before shared memory goes away.
            if (tid == 0)
                for (int u = t; u < ntiles && u < t + kPPStages; ++u) {
                    const uint32_t gu = gt + static_cast<uint32_t>(u);
                    mbar_wait_bounded(&ring.full[gu % kPPStages], (gu / kPPStages) & 1u, status);
                }
            __syncthreads();
            return false;
        }
        const int64_t jt = j0 + static_cast<int64_t>(t) * kPPTile;
        const int cnt = static_cast<int>((j1 - jt) < kPPTile ? (j1 - jt) : kPPTile);
        const int npr = (cnt + 1) >> 1;
        for (int q = tid; q < npr; q += T) {
            const float4 a = ring.tile[stage][2 * q];
            const float4 b = (2 * q + 1 < cnt) ? ring.tile[stage][2 * q + 1] : make_float4(0.f, 0.f, 0.f, 0.f);
            ring.pairs[2 * q] = make_float4(a.x, b.x, a.y, b.y);
            ring.pairs[2 * q + 1] = make_float4(a.z, b.z, a.w, b.w);
        }
        __syncthreads();
        if (tid == 0 && t + kPPStages < ntiles) issue(t + kPPStages);
        pair_forces<K, GUARD>(ring.pairs, npr, nx, ny, nz, e2, ax, ay, az);
    }
    gt += static_cast<uint32_t>(ntiles);
    return true;
}

}  // namespace nbody
