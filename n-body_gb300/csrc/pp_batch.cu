// Direct sum over an ensemble of independent systems packed back to back:
// one persistent kernel per step.
//
// Work items are (system, i-block of T*K bodies); the host lists them largest
// system first, and each CTA takes the next item from an atomic counter, so
// the long items start early and the short ones fill the tail. An item streams
// its system's bodies through the same TMA ring and packed f32x2 inner loop as
// the single-system kernel (no j-slices: the ensemble itself fills the GPU),
// then applies the integrator with that system's dt. The sum for a body runs
// over its system in j order, independent of which other systems share the
// launch, so a system's result does not depend on the ensemble around it.
#include <cuda_runtime.h>

#include <mutex>

#include "common.cuh"
#include "kernels.h"
#include "pp_batch.h"
#include "pp_common.cuh"

namespace nbody {

namespace {

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
        const float4 *pr = ring.pairs;
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
    gt += static_cast<uint32_t>(ntiles);
    return true;
}

template <int K, int T>
__global__ void __launch_bounds__(T)
    pp_batch_kernel(const float4 *__restrict__ pos, float4 *__restrict__ pos_out, float4 *__restrict__ vel,
                    float4 *__restrict__ acc, const int2 *__restrict__ items, int nitems,
                    const int4 *__restrict__ sys_range, const float4 *__restrict__ sys_prm,
                    unsigned *__restrict__ sched, int *status) {
    __shared__ __align__(128) float4 tile[kPPStages][kPPTile];
    __shared__ __align__(128) float4 pairs[kPPTile];
    __shared__ __align__(8) uint64_t full[kPPStages];
    __shared__ int s_item;
    const int tid = threadIdx.x;
    if (tid == 0) {
        for (int s = 0; s < kPPStages; ++s) mbar_init(&full[s], 1);
        mbar_init_fence();
    }
    __syncthreads();
    const Ring ring{tile, pairs, full};
    uint32_t gt = 0;
    for (;;) {
        if (tid == 0) s_item = static_cast<int>(atomicAdd(&sched[0], 1u));
        __syncthreads();
        const int it = s_item;
        __syncthreads();  // everyone has the item before thread 0 fetches again
        if (it >= nitems) break;
        const int2 wi = items[it];
        const int4 sr = sys_range[wi.x];  // first body, body count
        const float4 pr = sys_prm[wi.x];   // dt, eps2, -, euler
        const int64_t j0 = sr.x, j1 = static_cast<int64_t>(sr.x) + sr.y;
        float2 nx[K], ny[K], nz[K], ax[K], ay[K], az[K];
        float4 pi[K];
#pragma unroll
        for (int r = 0; r < K; ++r) {
            const int64_t i = static_cast<int64_t>(wi.y) + tid + r * T;
            pi[r] = i < j1 ? pos[i] : make_float4(0.f, 0.f, 0.f, 0.f);
            nx[r] = f2(-pi[r].x, -pi[r].x);
            ny[r] = f2(-pi[r].y, -pi[r].y);
            nz[r] = f2(-pi[r].z, -pi[r].z);
            ax[r] = ay[r] = az[r] = f2(0.f, 0.f);
        }
        const bool ok = pr.y > 0.f ? item_forces<K, T, false>(pos, j0, j1, nx, ny, nz, ax, ay, az, pr.y, ring, gt, status)
                                   : item_forces<K, T, true>(pos, j0, j1, nx, ny, nz, ax, ay, az, pr.y, ring, gt, status);
        if (!ok) return;  // status raised; the host resets the schedule
        Integrate g{pos_out, vel, acc, nullptr, pr.x, pr.w != 0.f ? 1 : 0};
#pragma unroll
        for (int r = 0; r < K; ++r) {
            const int64_t i = static_cast<int64_t>(wi.y) + tid + r * T;
            if (i < j1) integrate_body(i, pi[r], ax[r].x + ax[r].y, ay[r].x + ay[r].y, az[r].x + az[r].y, g);
        }
    }
    if (tid == 0) {
        // The last CTA out re-arms the schedule for the next launch.
        __threadfence();
        if (atomicAdd(&sched[1], 1u) == gridDim.x - 1) {
            sched[0] = 0u;
            sched[1] = 0u;
        }
    }
}

template <int K, int T>
int batch_ctas_per_sm() {
    int c = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&c, pp_batch_kernel<K, T>, T, 0);
    return c > 0 ? c : 1;
}

}  // namespace

int pp_batch_bodies_per_item(int shape) { return shape == kPPBatch128x2 ? 256 : shape == kPPBatch256x4 ? 1024 : 512; }

int pp_batch_ctas(int shape, int device, int nitems) {
    static std::mutex mu;
    static int cps[64][3] = {};
    static int sms[64] = {};
    std::lock_guard<std::mutex> lk(mu);
    const int d = device >= 0 && device < 64 ? device : 0;
    if (sms[d] == 0) {
        cudaDeviceGetAttribute(&sms[d], cudaDevAttrMultiProcessorCount, device);
        cps[d][kPPBatch128x2] = batch_ctas_per_sm<2, 128>();
        cps[d][kPPBatch256x2] = batch_ctas_per_sm<2, 256>();
        cps[d][kPPBatch256x4] = batch_ctas_per_sm<4, 256>();
        if (sms[d] <= 0) sms[d] = 1;
    }
    const int resident = sms[d] * cps[d][shape];
    return nitems < resident ? nitems : resident;
}

cudaError_t pp_batch_launch(int shape, int ctas, const float4 *pos, float4 *pos_out, float4 *vel, float4 *acc,
                            const int2 *items, int nitems, const int4 *sys_range, const float4 *sys_prm,
                            unsigned *sched, cudaStream_t st, int *status) {
    if (nitems <= 0 || ctas <= 0) return cudaSuccess;
    switch (shape) {
        case kPPBatch128x2:
            pp_batch_kernel<2, 128><<<ctas, 128, 0, st>>>(pos, pos_out, vel, acc, items, nitems, sys_range, sys_prm,
                                                          sched, status);
            break;
        case kPPBatch256x4:
            pp_batch_kernel<4, 256><<<ctas, 256, 0, st>>>(pos, pos_out, vel, acc, items, nitems, sys_range, sys_prm,
                                                          sched, status);
            break;
        default:
            pp_batch_kernel<2, 256><<<ctas, 256, 0, st>>>(pos, pos_out, vel, acc, items, nitems, sys_range, sys_prm,
                                                          sched, status);
            break;
    }
    return cudaGetLastError();
}

}  // namespace nbody
