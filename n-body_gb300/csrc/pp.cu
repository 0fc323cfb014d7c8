// Direct-sum (particle-particle) gravity for sm_103a.
//
// Replaces the reference's PP solvers: the CPU -v 2 force loop
// (src/ParticleSolver/ParticleSolverCPUParallel/ParticleSolverCPUParallel.cpp:27-40)
// and the GLSL -v 3 / -v 4 shaders (forceCalculation.glsl:24-49,
// forceCalculationOptimized.glsl:28-76) plus the integrator, which here keeps
// the CPU order (include/ParticleSystem.h:52-69), not the shaders' Euler step.
//
// Shape of the work: every CTA owns an i-block of T*K bodies (K per thread,
// held in registers) and one j-slice. The j-slice streams through shared
// memory in tiles of 256 float4 (x, y, z, m) bodies, each fetched by one
// non-tensor TMA bulk copy into a 3-stage ring completed on mbarriers; each
// landed tile is re-laid as j-pairs. The inner loop takes two j-bodies at a
// time so that every FP32 instruction is a packed f32x2 one
// (FADD2/FFMA2/FMUL2): 12 packed ops + 2 MUFU.RSQ per pair of interactions.
// j-slices exist to fill 152 SMs when n is small; the CTA that completes an
// i-block last sums its slices' partial accelerations in slice order
// (deterministic) and applies the integrator. With one slice the integrator
// runs in the force kernel's epilogue.
//
// Self-interaction: the reference skips j == i by index. Here the i == j term
// has dx = 0 and contributes exactly 0 when eps2 > 0; with eps2 == 0 the GUARD
// variant drops every pair at zero distance (r^2 == 0), which for j == i is the
// same thing.
#include <algorithm>
#include <cstdlib>
#include <mutex>

#include "common.cuh"
#include "kernels.h"
#include "pp_common.cuh"

namespace nbody {

constexpr int kPPMinThreads = 128;

// Launch bounds: K <= 2 takes the compiler's register choice (64 registers,
// 4 CTAs of 256 per SM); K >= 4 allows up to 255 registers per thread so that
// all K i-bodies' accumulators and the unrolled j-pairs stay in registers:
// fewer warps, more independent FMA chains per thread.
template <int K>
constexpr int pp_min_blocks() {
    return K >= 4 ? 1 : 0;
}

template <int K, int T, bool GUARD>
__global__ void __launch_bounds__(T, pp_min_blocks<K>())
    pp_force_kernel(const float4 *__restrict__ pos, int64_t n, float eps2, int nslices,
                    float4 *__restrict__ partial, unsigned *__restrict__ arrivals, Integrate g, int *status) {
    // tile: TMA landing zone, bodies as float4 (x, y, z, m).
    // pairs: two tiles re-laid as j-pairs {x0 x1 y0 y1}{z0 z1 m0 m1}, so that
    // one 16-byte shared load yields two packed f32x2 operands.
    __shared__ __align__(128) float4 tile[kPPStages][kPPTile];
    __shared__ __align__(128) float4 pairs[2][kPPTile];
    __shared__ __align__(8) uint64_t full[kPPStages];
    __shared__ int last_cta;

    const int tid = threadIdx.x;
    const int64_t ib0 = static_cast<int64_t>(blockIdx.x) * (T * K);
    const int slice = blockIdx.y;
    // The slice boundaries sit on even bodies so that j-pairs never straddle.
    const int64_t npairs = (n + 1) / 2;
    const int64_t p0 = npairs * slice / nslices;
    const int64_t p1 = npairs * (slice + 1) / nslices;
    const int64_t j0 = 2 * p0;
    const int64_t j1 = (2 * p1 < n) ? 2 * p1 : n;
    const int64_t len = j1 > j0 ? j1 - j0 : 0;
    const int ntiles = static_cast<int>((len + kPPTile - 1) / kPPTile);

    // Producer: thread 0 fetches tile t of this slice into stage t % kPPStages.
    auto issue = [&](int t) {
        const int stage = t % kPPStages;
        const int64_t jt = j0 + static_cast<int64_t>(t) * kPPTile;
        const int cnt = static_cast<int>((j1 - jt) < kPPTile ? (j1 - jt) : kPPTile);
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(&full[stage], static_cast<uint32_t>(cnt) * 16u);
        tma_bulk_g2s(&tile[stage][0], pos + jt, static_cast<uint32_t>(cnt) * 16u, &full[stage]);
    };
    // The first tiles are requested before the i-bodies are loaded, so that
    // the two memory latencies overlap; the barrier below publishes the
    // mbarrier initialisation to the other threads before any of them waits.
    if (tid == 0) {
        for (int s = 0; s < kPPStages; ++s) mbar_init(&full[s], 1);
        mbar_init_fence();
        for (int t = 0; t < kPPStages && t < ntiles; ++t) issue(t);
    }

    float2 nx[K], ny[K], nz[K], ax[K], ay[K], az[K];
    float4 pi[K];
#pragma unroll
    for (int r = 0; r < K; ++r) {
        const int64_t i = ib0 + tid + r * T;
        pi[r] = i < n ? pos[i] : make_float4(0.f, 0.f, 0.f, 0.f);
        nx[r] = f2(-pi[r].x, -pi[r].x);
        ny[r] = f2(-pi[r].y, -pi[r].y);
        nz[r] = f2(-pi[r].z, -pi[r].z);
        ax[r] = ay[r] = az[r] = f2(0.f, 0.f);
    }
    const float2 e2 = f2(eps2, eps2);
    __syncthreads();

    // Waits for tile t and re-lays it as j-pairs into pairs[t & 1] (an odd
    // last body is paired with m = 0). Returns false if the copy never landed.
    auto stage_in = [&](int t) -> bool {
        const int stage = t % kPPStages;
        const uint32_t parity = static_cast<uint32_t>(t / kPPStages) & 1u;
        if (!mbar_wait_bounded(&full[stage], parity, status)) return false;
        const int64_t jt = j0 + static_cast<int64_t>(t) * kPPTile;
        const int cnt = static_cast<int>((j1 - jt) < kPPTile ? (j1 - jt) : kPPTile);
        const int npr = (cnt + 1) >> 1;
        float4 *dst = pairs[t & 1];
        for (int q = tid; q < npr; q += T) {
            const float4 a = tile[stage][2 * q];
            const float4 b = (2 * q + 1 < cnt) ? tile[stage][2 * q + 1] : make_float4(0.f, 0.f, 0.f, 0.f);
            dst[2 * q] = make_float4(a.x, b.x, a.y, b.y);
            dst[2 * q + 1] = make_float4(a.z, b.z, a.w, b.w);
        }
        return true;
    };

    // Tile t is computed from pairs[t & 1] while tile t + 1 is re-laid into
    // the other buffer: one block barrier per tile. After the barrier that
    // ends tile t, tile t + 1's ring stage is free and takes tile t + 1 + stages.
    bool failed = false;
    int fail_at = 0;  // first tile whose copy may still be in flight
    if (ntiles > 0) {
        if (!__syncthreads_and(stage_in(0))) {
            failed = true;
        } else if (tid == 0 && kPPStages < ntiles) {
            issue(kPPStages);
        }
    }
    for (int t = 0; t < ntiles && !failed; ++t) {
        const bool ok = (t + 1 < ntiles) ? stage_in(t + 1) : true;
        const int64_t jt = j0 + static_cast<int64_t>(t) * kPPTile;
        const int cnt = static_cast<int>((j1 - jt) < kPPTile ? (j1 - jt) : kPPTile);
        const int npr = (cnt + 1) >> 1;
        pair_forces<K, GUARD>(pairs[t & 1], npr, nx, ny, nz, e2, ax, ay, az);
        if (!__syncthreads_and(ok)) {  // also: every thread is done with pairs[t & 1]
            failed = true;
            fail_at = t + 1;
            break;
        }
        if (tid == 0 && t + 1 + kPPStages < ntiles) issue(t + 1 + kPPStages);
    }

    if (failed) {
        // Drain this CTA's copies still in flight before shared memory goes away.
        if (tid == 0) {
            for (int u = fail_at; u < ntiles && u < fail_at + kPPStages; ++u)
                mbar_wait_bounded(&full[u % kPPStages], static_cast<uint32_t>(u / kPPStages) & 1u, status);
        }
        __syncthreads();
        return;
    }

    if (nslices == 1) {
#pragma unroll
        for (int r = 0; r < K; ++r) {
            const int64_t i = ib0 + tid + r * T;
            if (i >= n) continue;
            const float fx = ax[r].x + ax[r].y;
            const float fy = ay[r].x + ay[r].y;
            const float fz = az[r].x + az[r].y;
            if (g.pos_out) integrate_body(i, pi[r], fx, fy, fz, g);
            else if (g.force) g.force[i] = make_float4(fx, fy, fz, 0.f);
        }
        return;
    }

    // Several j-slices: publish this slice's partial accelerations; the CTA
    // that completes an i-block last sums all slices in slice order (so the
    // result does not depend on which CTA ran when) and integrates.
#pragma unroll
    for (int r = 0; r < K; ++r) {
        const int64_t i = ib0 + tid + r * T;
        if (i < n)
            partial[static_cast<int64_t>(slice) * n + i] =
                make_float4(ax[r].x + ax[r].y, ay[r].x + ay[r].y, az[r].x + az[r].y, 0.f);
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) {
        const unsigned prev = atomicAdd(&arrivals[blockIdx.x], 1u);
        last_cta = (prev == static_cast<unsigned>(nslices - 1));
        if (last_cta) arrivals[blockIdx.x] = 0u;  // ready for the next launch
    }
    __syncthreads();
    if (!last_cta) return;
    __threadfence();
    // kBatch slices x K bodies of partial loads in flight at once (16 float4),
    // each body still summed in slice order.
    constexpr int kBatch = K >= 16 ? 1 : 16 / K;
    float fx[K], fy[K], fz[K];
#pragma unroll
    for (int r = 0; r < K; ++r) fx[r] = fy[r] = fz[r] = 0.f;
    for (int sl0 = 0; sl0 < nslices; sl0 += kBatch) {
        float4 q[kBatch][K];
#pragma unroll
        for (int b = 0; b < kBatch; ++b) {
#pragma unroll
            for (int r = 0; r < K; ++r) {
                const int64_t i = ib0 + tid + r * T;
                q[b][r] = (sl0 + b < nslices && i < n) ? __ldcg(&partial[static_cast<int64_t>(sl0 + b) * n + i])
                                                       : make_float4(0.f, 0.f, 0.f, 0.f);
            }
        }
#pragma unroll
        for (int b = 0; b < kBatch; ++b) {
            if (sl0 + b < nslices) {
#pragma unroll
                for (int r = 0; r < K; ++r) {
                    fx[r] += q[b][r].x;
                    fy[r] += q[b][r].y;
                    fz[r] += q[b][r].z;
                }
            }
        }
    }
#pragma unroll
    for (int r = 0; r < K; ++r) {
        const int64_t i = ib0 + tid + r * T;
        if (i >= n) continue;
        if (g.pos_out) integrate_body(i, pi[r], fx[r], fy[r], fz[r], g);
        else if (g.force) g.force[i] = make_float4(fx[r], fy[r], fz[r], 0.f);
    }
}

// Linear split, for the shapes that run one ILP-bound CTA per SM: the work
// space of (i-block, j-pair) units, i-block major, is cut into gridDim.x equal
// contiguous ranges, so every CTA evaluates the same number of pairs and no SM
// idles for want of a CTA. With gridDim.x >= i-blocks a range covers the end of
// one i-block and the start of the next at most: a CTA computes its (one or
// two) segments first, publishing one partial per segment (slot 0 or 1), and
// only then takes part in the reductions: the last CTA to arrive for an
// i-block sums the partials of all CTAs that touched it, in CTA order
// (deterministic), and integrates.
__device__ __forceinline__ int64_t linear_begin(int64_t W, int64_t C, int64_t c) { return W * c / C; }
// The CTA whose range holds unit x.
__device__ __forceinline__ int64_t linear_cta(int64_t W, int64_t C, int64_t x) { return ((x + 1) * C + W - 1) / W - 1; }

template <int K, int T, bool GUARD>
__global__ void __launch_bounds__(T, pp_min_blocks<K>())
    pp_force_linear_kernel(const float4 *__restrict__ pos, int64_t n, float eps2, float4 *__restrict__ partial,
                           unsigned *__restrict__ arrivals, Integrate g, int *status) {
    __shared__ __align__(128) float4 tile[kPPStages][kPPTile];
    __shared__ __align__(128) float4 pairs[kPPTile];
    __shared__ __align__(8) uint64_t full[kPPStages];
    __shared__ int last_cta;
    __shared__ long long s_first, s_last;
    const int tid = threadIdx.x;
    if (tid == 0) {
        for (int s = 0; s < kPPStages; ++s) mbar_init(&full[s], 1);
        mbar_init_fence();
    }
    __syncthreads();
    const Ring ring{tile, pairs, full};
    constexpr int64_t TK = static_cast<int64_t>(T) * K;
    const int64_t npairs = (n + 1) / 2;
    const int64_t iblocks = (n + TK - 1) / TK;
    const int64_t W = iblocks * npairs;
    const int64_t C = gridDim.x, c = blockIdx.x;
    const int64_t u0 = linear_begin(W, C, c), u1 = linear_begin(W, C, c + 1);
    uint32_t gt = 0;
    int64_t blocks_of[2] = {-1, -1};
    int nseg = 0;
    for (int64_t u = u0; u < u1; ++nseg) {
        const int64_t b = u / npairs;
        const int64_t p0 = u - b * npairs;
        const int64_t pend = (npairs - p0) < (u1 - u) ? npairs : p0 + (u1 - u);
        const int64_t j0 = 2 * p0, j1 = (2 * pend < n) ? 2 * pend : n;
        const int64_t ib0 = b * TK;
        if (nseg > 1) {  // cannot happen with gridDim.x >= i-blocks: report, stop
            record_error(status, NBODY_ERR_CAPACITY);
            return;
        }
        float2 nx[K], ny[K], nz[K], ax[K], ay[K], az[K];
#pragma unroll
        for (int r = 0; r < K; ++r) {
            const int64_t i = ib0 + tid + r * T;
            const float4 p = i < n ? pos[i] : make_float4(0.f, 0.f, 0.f, 0.f);
            nx[r] = f2(-p.x, -p.x);
            ny[r] = f2(-p.y, -p.y);
            nz[r] = f2(-p.z, -p.z);
            ax[r] = ay[r] = az[r] = f2(0.f, 0.f);
        }
        if (!item_forces<K, T, GUARD>(pos, j0, j1, nx, ny, nz, ax, ay, az, eps2, ring, gt, status)) return;
        float4 *mine = partial + (c * 2 + nseg) * TK;
#pragma unroll
        for (int r = 0; r < K; ++r)
            mine[tid + r * T] = make_float4(ax[r].x + ax[r].y, ay[r].x + ay[r].y, az[r].x + az[r].y, 0.f);
        blocks_of[nseg] = b;
        u = (b + 1) * npairs;
    }
    __threadfence();
    __syncthreads();
    for (int sg = 0; sg < nseg; ++sg) {
        const int64_t b = blocks_of[sg];
        if (tid == 0) {
            const int64_t first = linear_cta(W, C, b * npairs), last = linear_cta(W, C, (b + 1) * npairs - 1);
            const unsigned prev = atomicAdd(&arrivals[b], 1u);
            last_cta = prev == static_cast<unsigned>(last - first);
            if (last_cta) arrivals[b] = 0u;  // ready for the next launch
            s_first = first;
            s_last = last;
        }
        __syncthreads();
        if (last_cta) {
            __threadfence();
            const int64_t ib0 = b * TK;
            float fx[K], fy[K], fz[K];
#pragma unroll
            for (int r = 0; r < K; ++r) fx[r] = fy[r] = fz[r] = 0.f;
            constexpr int kB = 4;  // CTAs' partials in flight at a time
            for (int64_t c0 = s_first; c0 <= s_last; c0 += kB) {
                float4 q[kB][K];
#pragma unroll
                for (int bb = 0; bb < kB; ++bb) {
                    const int64_t cc = c0 + bb;
                    if (cc > s_last) continue;
                    const int64_t sl = b - linear_begin(W, C, cc) / npairs;  // the i-block's slot in CTA cc
                    const float4 *src = partial + (cc * 2 + sl) * TK + tid;
#pragma unroll
                    for (int r = 0; r < K; ++r) q[bb][r] = __ldcg(src + r * T);
                }
#pragma unroll
                for (int bb = 0; bb < kB; ++bb) {
                    if (c0 + bb > s_last) continue;
#pragma unroll
                    for (int r = 0; r < K; ++r) {
                        fx[r] += q[bb][r].x;
                        fy[r] += q[bb][r].y;
                        fz[r] += q[bb][r].z;
                    }
                }
            }
#pragma unroll
            for (int r = 0; r < K; ++r) {
                const int64_t i = ib0 + tid + r * T;
                if (i >= n) continue;
                if (g.pos_out) integrate_body(i, pos[i], fx[r], fy[r], fz[r], g);
                else if (g.force) g.force[i] = make_float4(fx[r], fy[r], fz[r], 0.f);
            }
        }
        __syncthreads();  // last_cta and s_first / s_last are rewritten for the next i-block
    }
}

__global__ void pack_kernel(const float4 *__restrict__ positions4, const float4 *__restrict__ masses4,
                            float4 *__restrict__ pos_mass, int64_t n) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p = positions4[i];
    pos_mass[i] = make_float4(p.x, p.y, p.z, masses4[i].x);
}

__global__ void unpack_kernel(const float4 *__restrict__ pos_mass, float4 *__restrict__ positions4, int64_t n) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p = pos_mass[i];
    positions4[i] = make_float4(p.x, p.y, p.z, 0.f);
}

__global__ void unpack_masses_kernel(const float4 *__restrict__ pos_mass, const int *__restrict__ ids,
                                     float4 *__restrict__ masses4, int64_t n, int *status) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int64_t d = ids ? ids[i] : i;
    if (d < 0 || d >= n) {
        record_error(status, NBODY_ERR_CAPACITY);
        return;
    }
    masses4[d] = make_float4(pos_mass[i].w, 0.f, 0.f, 0.f);
}

// ---------------------------------------------------------------- host side
namespace {

template <int K, int T>
int ctas_per_sm() {
    int c = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&c, pp_force_kernel<K, T, false>, T, 0);
    return c > 0 ? c : 1;
}

struct DeviceInfo {
    int sms = 0;
    int cps[2][4] = {{0, 0, 0, 0}, {0, 0, 0, 0}};  // CTAs per SM for T = 128, 256 and K = 1, 2, 4, 8
};

DeviceInfo device_info(int device) {
    static std::mutex mu;
    static DeviceInfo cache[64];
    static bool have[64] = {};
    std::lock_guard<std::mutex> lk(mu);
    if (device < 0 || device >= 64) device = 0;
    if (!have[device]) {
        DeviceInfo d;
        cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, device);
        d.cps[0][0] = ctas_per_sm<1, 128>();
        d.cps[0][1] = ctas_per_sm<2, 128>();
        d.cps[0][2] = ctas_per_sm<4, 128>();
        d.cps[0][3] = ctas_per_sm<8, 128>();
        d.cps[1][0] = ctas_per_sm<1, 256>();
        d.cps[1][1] = ctas_per_sm<2, 256>();
        d.cps[1][2] = ctas_per_sm<4, 256>();
        d.cps[1][3] = ctas_per_sm<8, 256>();
        cache[device] = d;
        have[device] = true;
    }
    return cache[device];
}

int k_index(int k) { return k == 1 ? 0 : k == 2 ? 1 : k == 4 ? 2 : 3; }

}  // namespace

PPPlan pp_plan(int64_t n, int device, bool allow_linear) {
    PPPlan p;
    const DeviceInfo d = device_info(device);
    // Default shapes from sweeps on GB300 (T x K in {128, 256} x {1, 2, 4, 8},
    // N = 4,096 ... 131,072): from N = 8,192 on, 256 threads with 4 i-bodies
    // each (one CTA per SM at 140 registers, ILP-bound) is fastest; below it 2
    // i-bodies per thread give the j-slicing enough CTAs.
    int k = n >= 8192 ? 4 : 2;
    if (const char *e = std::getenv("NBODY_PP_K")) {
        const int v = std::atoi(e);
        if (v == 1 || v == 2 || v == 4 || v == 8) k = v;
    } else if (n <= 2 * kPPMinThreads) {
        k = 1;
    }
    p.k = k;
    int threads = n <= 2 * kPPMinThreads ? 128 : 256;
    if (const char *e = std::getenv("NBODY_PP_THREADS")) {
        const int v = std::atoi(e);
        if (v == 128 || v == 256) threads = v;
    }
    p.threads = threads;
    const int64_t per_block = static_cast<int64_t>(threads) * k;
    p.iblocks = static_cast<int>((n + per_block - 1) / per_block);
    const int64_t sms = d.sms > 0 ? d.sms : 1;
    const int ti = threads == 256 ? 1 : 0;
    const int64_t cps = d.cps[ti][k_index(k)] > 0 ? d.cps[ti][k_index(k)] : 1;
    const int64_t npairs = (n + 1) / 2;
    // Slice count: each slice keeps at least one full tile of j-bodies. The
    // cost model charges every SM for the waves of CTAs it must run (a partial
    // wave costs a full one, since a lone CTA cannot fill an SM), each CTA for
    // its j-pairs plus a fixed overhead (pipeline fill, i-loads, epilogue: about
    // 24 pairs' time), and the final sum for reading one partial per slice
    // (about one pair's time: the loads of 16 / K slices are in flight at once).
    // On GB300 at N = 16,384 this takes 19 slices in two full waves over 152 SMs
    // (110.7 us) over 9 slices in one wave over 144 SMs (112.0 us).
    int64_t smax = std::max<int64_t>(1, std::min<int64_t>(npairs / (kPPTile / 2), 64));
    double best = 1e300;
    int best_s = 1;
    for (int64_t sl = 1; sl <= smax; ++sl) {
        const int64_t total = static_cast<int64_t>(p.iblocks) * sl;
        const int64_t per_sm = (total + sms - 1) / sms;
        const int64_t waves = (per_sm + cps - 1) / cps;
        const double cta_cost = static_cast<double>(npairs) / static_cast<double>(sl) + 24.0;
        const double cost = static_cast<double>(waves * cps) * cta_cost + static_cast<double>(sl);
        if (cost < best * (1.0 - 1e-9)) {
            best = cost;
            best_s = static_cast<int>(sl);
        }
    }
    if (const char *e = std::getenv("NBODY_PP_SLICES")) {
        const int v = std::atoi(e);
        if (v >= 1) best_s = static_cast<int>(std::min<int64_t>(v, std::max<int64_t>(1, npairs)));
    }
    p.slices = best_s;
    // Shapes with one ILP-bound CTA per SM take the linear split (exactly
    // filled SMs) from N = 32,768 on, where it measured 1-4% faster on GB300
    // (below, the end-of-kernel reductions of every CTA cost more than the idle
    // SMs of the sliced plan), unless a slice count is forced; NBODY_PP_LINEAR
    // = 1 / 0 forces it on / off.
    const char *lin = std::getenv("NBODY_PP_LINEAR");
    const bool lin_on = lin && std::atoi(lin) == 1, lin_off = lin && std::atoi(lin) == 0;
    const bool want_linear = allow_linear && k >= 4 && !std::getenv("NBODY_PP_SLICES") && !lin_off &&
                             n >= static_cast<int64_t>(threads) * k && (lin_on || n >= 32768);
    if (want_linear) {
        const int64_t resident = sms * cps;
        p.linear_ctas = static_cast<int>(resident * ((p.iblocks + resident - 1) / resident));
        p.slices = 0;
        p.arrivals_bytes = (static_cast<size_t>(p.iblocks) * sizeof(unsigned) + 255) & ~static_cast<size_t>(255);
        p.partial_bytes = p.arrivals_bytes + static_cast<size_t>(p.linear_ctas) * 2 * static_cast<size_t>(per_block) *
                                                 sizeof(float4);
        return p;
    }
    if (p.slices > 1) {
        p.arrivals_bytes = (static_cast<size_t>(p.iblocks) * sizeof(unsigned) + 255) & ~static_cast<size_t>(255);
        p.partial_bytes = p.arrivals_bytes + static_cast<size_t>(p.slices) * static_cast<size_t>(n) * sizeof(float4);
    }
    return p;
}

PPPlan pp_plan_within(int64_t n, int device, size_t scratch_bytes) {
    PPPlan p = pp_plan(n, device);
    if (p.linear_ctas > 0 && p.partial_bytes > scratch_bytes) p = pp_plan(n, device, false);
    while (p.slices > 1 && p.partial_bytes > scratch_bytes) {
        const int64_t fit = static_cast<int64_t>((scratch_bytes > p.arrivals_bytes ? scratch_bytes - p.arrivals_bytes : 0) /
                                                 (static_cast<size_t>(n) * sizeof(float4)));
        p.slices = static_cast<int>(std::max<int64_t>(1, std::min<int64_t>(fit, p.slices - 1)));
        p.arrivals_bytes = p.slices > 1 ? p.arrivals_bytes : 0;
        p.partial_bytes =
            p.slices > 1 ? p.arrivals_bytes + static_cast<size_t>(p.slices) * static_cast<size_t>(n) * sizeof(float4) : 0;
    }
    return p;
}

template <int K, int T>
static cudaError_t launch_kt(const PPPlan &plan, const float4 *pos, int64_t n, float eps2, const Integrate &g,
                             float4 *partial, unsigned *arrivals, cudaStream_t stream, int *status) {
    if (plan.linear_ctas > 0) {
        if (eps2 > 0.f)
            pp_force_linear_kernel<K, T, false>
                <<<plan.linear_ctas, T, 0, stream>>>(pos, n, eps2, partial, arrivals, g, status);
        else
            pp_force_linear_kernel<K, T, true>
                <<<plan.linear_ctas, T, 0, stream>>>(pos, n, eps2, partial, arrivals, g, status);
        return cudaGetLastError();
    }
    const dim3 grid(plan.iblocks, plan.slices);
    if (eps2 > 0.f)
        pp_force_kernel<K, T, false><<<grid, T, 0, stream>>>(pos, n, eps2, plan.slices, partial, arrivals, g, status);
    else
        pp_force_kernel<K, T, true><<<grid, T, 0, stream>>>(pos, n, eps2, plan.slices, partial, arrivals, g, status);
    return cudaGetLastError();
}

template <int K>
static cudaError_t launch_k(const PPPlan &plan, const float4 *pos, int64_t n, float eps2, const Integrate &g,
                            float4 *partial, unsigned *arrivals, cudaStream_t stream, int *status) {
    if (plan.threads == 256) return launch_kt<K, 256>(plan, pos, n, eps2, g, partial, arrivals, stream, status);
    return launch_kt<K, 128>(plan, pos, n, eps2, g, partial, arrivals, stream, status);
}

cudaError_t pp_launch(const PPPlan &plan, const float4 *pos, int64_t n, float eps2, const Integrate &g,
                      void *scratch, cudaStream_t stream, int *status, StageTimer *timer) {
    if (n <= 0) return cudaSuccess;
    unsigned *arrivals = nullptr;
    float4 *partial = nullptr;
    if (plan.slices > 1 || plan.linear_ctas > 0) {
        if (!scratch) return cudaErrorInvalidValue;
        arrivals = static_cast<unsigned *>(scratch);
        partial = reinterpret_cast<float4 *>(static_cast<char *>(scratch) + plan.arrivals_bytes);
    }
    cudaError_t e;
    if (timer) timer->begin(kStagePPForce, stream);
    switch (plan.k) {
        case 1: e = launch_k<1>(plan, pos, n, eps2, g, partial, arrivals, stream, status); break;
        case 2: e = launch_k<2>(plan, pos, n, eps2, g, partial, arrivals, stream, status); break;
        case 8: e = launch_k<8>(plan, pos, n, eps2, g, partial, arrivals, stream, status); break;
        default: e = launch_k<4>(plan, pos, n, eps2, g, partial, arrivals, stream, status); break;
    }
    if (timer) timer->end(kStagePPForce, stream);
    return e;
}

cudaError_t pack_state(const float4 *positions4, const float4 *masses4, float4 *pos_mass, int64_t n,
                       cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    const int threads = 256;
    pack_kernel<<<static_cast<unsigned>((n + threads - 1) / threads), threads, 0, stream>>>(positions4, masses4,
                                                                                           pos_mass, n);
    return cudaGetLastError();
}

cudaError_t unpack_positions(const float4 *pos_mass, float4 *positions4, int64_t n, cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    const int threads = 256;
    unpack_kernel<<<static_cast<unsigned>((n + threads - 1) / threads), threads, 0, stream>>>(pos_mass,
                                                                                             positions4, n);
    return cudaGetLastError();
}

cudaError_t unpack_masses(const float4 *pos_mass, const int *ids, float4 *masses4, int64_t n, cudaStream_t stream,
                          int *status) {
    if (n <= 0) return cudaSuccess;
    const int threads = 256;
    unpack_masses_kernel<<<static_cast<unsigned>((n + threads - 1) / threads), threads, 0, stream>>>(
        pos_mass, ids, masses4, n, status);
    return cudaGetLastError();
}

}  // namespace nbody
