// Conservation diagnostics: total kinetic and potential energy, linear and
// angular momentum. The reference has no diagnostics; these reductions are
// the only FP64 arithmetic on the GPU. Per-body terms are formed and summed
// in FP64 (grid-stride per thread, then per block, then the blocks in index
// order by the last block to finish), so a given launch shape always gives
// the same bits. The potential per body comes in as FP32 (direct sum or the
// Barnes-Hut walk) and is reduced here.
#include <cuda_runtime.h>

#include "common.cuh"
#include "diag.h"

namespace nbody {

namespace {

constexpr int kDiagThreads = 256;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    return v;
}

__global__ void __launch_bounds__(kDiagThreads)
    momenta_kernel(const float4 *__restrict__ pos, const float4 *__restrict__ vel, const float *__restrict__ phi,
                   int64_t n, double *__restrict__ partial, unsigned *__restrict__ counter,
                   double *__restrict__ out) {
    double v[8] = {0, 0, 0, 0, 0, 0, 0, 0};  // ke, pe, px, py, pz, lx, ly, lz
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
        const float4 p = pos[i];
        const float4 u = vel[i];
        const double m = p.w, x = p.x, y = p.y, z = p.z, vx = u.x, vy = u.y, vz = u.z;
        v[0] += 0.5 * m * (vx * vx + vy * vy + vz * vz);
        if (phi) v[1] += 0.5 * m * static_cast<double>(phi[i]);
        v[2] += m * vx;
        v[3] += m * vy;
        v[4] += m * vz;
        v[5] += m * (y * vz - z * vy);
        v[6] += m * (z * vx - x * vz);
        v[7] += m * (x * vy - y * vx);
    }
    __shared__ double ws[kDiagThreads / 32][8];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < 8; ++k) v[k] = warp_sum(v[k]);
    if (lane == 0)
        for (int k = 0; k < 8; ++k) ws[warp][k] = v[k];
    __syncthreads();
    if (threadIdx.x < 8) {
        double t = 0;
        for (int w = 0; w < kDiagThreads / 32; ++w) t += ws[w][threadIdx.x];
        partial[blockIdx.x * 8 + threadIdx.x] = t;
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(counter, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    if (threadIdx.x < 8) {
        double t = 0;
        for (unsigned b = 0; b < gridDim.x; ++b) t += __ldcg(&partial[b * 8 + threadIdx.x]);
        out[threadIdx.x] = t;
    }
    if (threadIdx.x == 0) *counter = 0u;
}

// phi_i = -sum_{j != i} m_j / sqrt(|x_j - x_i|^2 + eps2), FP32, j-tiles in
// shared memory (the self pair is excluded by index: its term is not zero).
__global__ void __launch_bounds__(kDiagThreads) pp_potential_kernel(const float4 *__restrict__ pos, int64_t n,
                                                                     float eps2, float *__restrict__ phi) {
    __shared__ float4 tile[kDiagThreads];
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const float4 me = i < n ? pos[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    float acc = 0.f;
    for (int64_t j0 = 0; j0 < n; j0 += kDiagThreads) {
        __syncthreads();
        const int64_t j = j0 + threadIdx.x;
        tile[threadIdx.x] = j < n ? pos[j] : make_float4(0.f, 0.f, 0.f, 0.f);
        __syncthreads();
        const int cnt = (n - j0) < kDiagThreads ? static_cast<int>(n - j0) : kDiagThreads;
        for (int q = 0; q < cnt; ++q) {
            if (j0 + q == i) continue;
            const float4 o = tile[q];
            const float dx = o.x - me.x, dy = o.y - me.y, dz = o.z - me.z;
            const float r2 = fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, eps2)));
            if (r2 > 0.f) acc = fmaf(-o.w, rsqrtf(r2), acc);
        }
    }
    if (i < n) phi[i] = acc;
}

}  // namespace

size_t diag_scratch_bytes() { return sizeof(double) * (8 * kDiagBlocks + 16) + 256; }

cudaError_t diag_momenta(const float4 *pos, const float4 *vel, const float *phi, int64_t n, void *scratch,
                         double *out_dev, cudaStream_t st) {
    double *partial = static_cast<double *>(scratch);
    unsigned *counter = reinterpret_cast<unsigned *>(partial + 8 * kDiagBlocks);
    int blocks = static_cast<int>((n + kDiagThreads - 1) / kDiagThreads);
    if (blocks > kDiagBlocks) blocks = kDiagBlocks;
    if (blocks < 1) blocks = 1;
    momenta_kernel<<<blocks, kDiagThreads, 0, st>>>(pos, vel, phi, n, partial, counter, out_dev);
    return cudaGetLastError();
}

cudaError_t diag_pp_potential(const float4 *pos, int64_t n, float eps2, float *phi, cudaStream_t st) {
    pp_potential_kernel<<<static_cast<unsigned>((n + kDiagThreads - 1) / kDiagThreads), kDiagThreads, 0, st>>>(
        pos, n, eps2, phi);
    return cudaGetLastError();
}

}  // namespace nbody
