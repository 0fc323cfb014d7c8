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

// K >= 4: up to 255 registers (all K accumulators and the unrolled j-pairs in
// registers; fewer, ILP-rich warps), as the single-system kernel.
template <int K, int T>
__global__ void __launch_bounds__(T, K >= 4 ? 1 : 0)
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

int pp_batch_bodies_per_item(int shape) {
    return shape == kPPBatch128x2 ? 256 : shape == kPPBatch256x4 ? 1024 : 512;  // 256x2 and 128x4: 512
}

int pp_batch_ctas(int shape, int device, int nitems) {
    static std::mutex mu;
    static int cps[64][kPPBatchShapes] = {};
    static int sms[64] = {};
    std::lock_guard<std::mutex> lk(mu);
    const int d = device >= 0 && device < 64 ? device : 0;
    if (sms[d] == 0) {
        cudaDeviceGetAttribute(&sms[d], cudaDevAttrMultiProcessorCount, device);
        cps[d][kPPBatch128x2] = batch_ctas_per_sm<2, 128>();
        cps[d][kPPBatch256x2] = batch_ctas_per_sm<2, 256>();
        cps[d][kPPBatch256x4] = batch_ctas_per_sm<4, 256>();
        cps[d][kPPBatch128x4] = batch_ctas_per_sm<4, 128>();
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
        case kPPBatch128x4:
            pp_batch_kernel<4, 128><<<ctas, 128, 0, st>>>(pos, pos_out, vel, acc, items, nitems, sys_range, sys_prm,
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
