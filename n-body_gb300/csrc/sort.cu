// Stable LSD radix sort of (63-bit key, 32-bit value) pairs: a onesweep-style
// design (one global histogram pass, then one pass per 8-bit digit with a
// decoupled look-back across tiles).
//
// Replaces the reference's unstable global bitonic sort
// (src/shaders/ComputeShaders/bitonicSort.glsl:23-50, driven by the host loop in
// src/ParticleSystem/ParticleSystem.cpp:142-151) and its rearrange pass: the
// sort here is stable, so equal keys keep their input order, and the result is
// the permutation std::stable_sort would produce.
//
// Per digit pass, a CTA takes the next tile index from an atomic counter (so
// every tile it waits on belongs to a CTA that is already running), ranks its
// 4096 keys per digit with warp match-any (stable: item order inside a warp,
// warps in order), publishes its per-digit counts, looks back over earlier
// tiles for their running totals (bounded waits; a timeout raises the status
// word and the pass gives up), stages the tile in shared memory in digit order
// and writes it out.
#include <cuda_runtime.h>

#include <mutex>

#include "common.cuh"
#include "sort.h"

namespace nbody {

namespace {

constexpr int kRadixBits = 8;
constexpr int kBins = 1 << kRadixBits;
constexpr int kSortThreads = 256;
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kItems = 16;  // keys per thread
constexpr int kTile = kSortThreads * kItems;  // 4096 keys per tile
constexpr int kPasses = 8;                    // 63 key bits = 8 digits of 8 bits

constexpr uint32_t kFlagAgg = 1u << 30;   // tile count published
constexpr uint32_t kFlagIncl = 2u << 30;  // inclusive running total published
constexpr uint32_t kValueMask = (1u << 30) - 1u;

__device__ __forceinline__ uint32_t digit_of(uint64_t k, int pass) {
    return static_cast<uint32_t>(k >> (pass * kRadixBits)) & (kBins - 1);
}

// Global histograms of the first `passes` digits in one read of the keys.
__global__ void __launch_bounds__(kSortThreads) histogram_kernel(const uint64_t *__restrict__ keys, int64_t n,
                                                                 int passes,
                                                                 uint32_t *__restrict__ hist /* [kPasses][kBins] */) {
    __shared__ uint32_t h[kPasses][kBins];
    for (int i = threadIdx.x; i < kPasses * kBins; i += blockDim.x) (&h[0][0])[i] = 0;
    __syncthreads();
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint64_t k = keys[i];
#pragma unroll
        for (int p = 0; p < kPasses; ++p)
            if (p < passes) atomicAdd(&h[p][digit_of(k, p)], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < passes * kBins; i += blockDim.x) {
        const uint32_t v = (&h[0][0])[i];
        if (v) atomicAdd(&hist[i], v);
    }
}

// Exclusive scan of each digit's histogram (one CTA of kBins threads per pass).
__global__ void __launch_bounds__(kBins) histogram_scan_kernel(uint32_t *__restrict__ hist) {
    __shared__ uint32_t s[kBins];
    uint32_t *h = hist + blockIdx.x * kBins;
    const int t = threadIdx.x;
    s[t] = h[t];
    __syncthreads();
    for (int off = 1; off < kBins; off <<= 1) {
        const uint32_t v = t >= off ? s[t - off] : 0u;
        __syncthreads();
        s[t] += v;
        __syncthreads();
    }
    h[t] = s[t] - h[t];  // exclusive
}

struct __align__(16) SortSmem {
    uint32_t warp_hist[kSortWarps][kBins];  // per-warp digit counts, then per-warp prefixes
    uint32_t tile_bin_start[kBins];         // exclusive prefix of the tile's digit counts
    uint32_t global_base[kBins];            // where this tile's digit-b run starts in the output
    uint64_t keys[kTile];
    uint32_t vals[kTile];
    int tile_id;
    int failed;
};

// Three CTAs per SM (80 registers, no spills; shared memory 3 x 58 KB): the
// pass is latency-bound, and the third CTA took a 2^24-key sort from 2.17 to
// 1.55 ms on GB300.
__global__ void __launch_bounds__(kSortThreads, 3)
    onesweep_kernel(const uint64_t *__restrict__ keys_in, const uint32_t *__restrict__ vals_in,
                    uint64_t *__restrict__ keys_out, uint32_t *__restrict__ vals_out, int64_t n, int pass,
                    const uint32_t *__restrict__ digit_base /* [kBins] */, uint32_t *tile_counter,
                    uint32_t *desc /* [ntiles][kBins] */, int *status) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SortSmem &S = *reinterpret_cast<SortSmem *>(smem_raw);
    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const int warp = tid >> 5;

    if (tid == 0) {
        S.tile_id = static_cast<int>(atomicAdd(tile_counter, 1u));
        S.failed = 0;
    }
    for (int i = tid; i < kSortWarps * kBins; i += kSortThreads) (&S.warp_hist[0][0])[i] = 0;
    __syncthreads();
    const int tile = S.tile_id;
    const int64_t base = static_cast<int64_t>(tile) * kTile;

    // Load: warp w owns keys [base + w*32*kItems, ...), lane l holds item j at
    // offset j*32 + l (coalesced), i.e. items in ascending input order by (j, l).
    uint64_t k[kItems];
    uint32_t v[kItems];
    uint32_t d[kItems];
    uint32_t rank[kItems];
    const int64_t wbase = base + static_cast<int64_t>(warp) * 32 * kItems;
#pragma unroll
    for (int j = 0; j < kItems; ++j) {
        const int64_t i = wbase + j * 32 + lane;
        const bool ok = i < n;
        k[j] = ok ? keys_in[i] : ~0ull;
        v[j] = ok ? vals_in[i] : 0u;
        d[j] = ok ? digit_of(k[j], pass) : kBins;  // out-of-range items get no digit
    }
    // Stable warp-level ranking per item row.
    const uint32_t lt = (1u << lane) - 1u;
#pragma unroll
    for (int j = 0; j < kItems; ++j) {
        const uint32_t peers = __match_any_sync(0xffffffffu, d[j]);
        const uint32_t leader = __ffs(peers) - 1;
        uint32_t before = 0;
        if (d[j] < kBins && lane == static_cast<int>(leader)) before = S.warp_hist[warp][d[j]];
        before = __shfl_sync(0xffffffffu, before, leader);
        rank[j] = before + __popc(peers & lt);
        __syncwarp();
        if (d[j] < kBins && lane == static_cast<int>(leader)) S.warp_hist[warp][d[j]] = before + __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    // Per digit: tile count and exclusive prefix over warps (thread b owns digit b).
    uint32_t tile_count = 0;
    if (tid < kBins) {
        uint32_t run = 0;
        for (int w = 0; w < kSortWarps; ++w) {
            const uint32_t c = S.warp_hist[w][tid];
            S.warp_hist[w][tid] = run;
            run += c;
        }
        tile_count = run;
        // Publish this tile's count (or, for tile 0, its inclusive total).
        volatile uint32_t *dd = desc + static_cast<int64_t>(tile) * kBins + tid;
        *dd = (tile == 0 ? kFlagIncl : kFlagAgg) | tile_count;
    }
    // Exclusive prefix of tile counts over digits -> tile-local start of each digit run.
    {
        __shared__ uint32_t scan[kBins];
        if (tid < kBins) scan[tid] = tile_count;
        __syncthreads();
        for (int off = 1; off < kBins; off <<= 1) {
            uint32_t t2 = 0;
            if (tid < kBins && tid >= off) t2 = scan[tid - off];
            __syncthreads();
            if (tid < kBins) scan[tid] += t2;
            __syncthreads();
        }
        if (tid < kBins) S.tile_bin_start[tid] = scan[tid] - tile_count;
    }
    // Decoupled look-back: running total of digit tid over all earlier tiles.
    if (tid < kBins) {
        uint32_t excl = 0;
        bool ok = true;
        for (int p = tile - 1; p >= 0 && ok;) {
            volatile const uint32_t *dd = desc + static_cast<int64_t>(p) * kBins + tid;
            uint32_t w = *dd;
            if ((w & ~kValueMask) == 0) {
                const unsigned long long t0 = global_ns();
                uint32_t spin = 0;
                while (((w = *dd) & ~kValueMask) == 0) {
                    if (++spin >= kWaitSpinCap || ((spin & 1023u) == 0 && global_ns() - t0 > kWaitLimitNs)) {
                        record_error(status, NBODY_ERR_TIMEOUT);
                        ok = false;
                        break;
                    }
                }
                if (!ok) break;
            }
            excl += w & kValueMask;
            if (w & kFlagIncl) break;
            --p;
        }
        if (!ok) atomicExch(&S.failed, 1);
        if (tile > 0) {
            volatile uint32_t *dd = desc + static_cast<int64_t>(tile) * kBins + tid;
            *dd = kFlagIncl | ((excl + tile_count) & kValueMask);
        }
        S.global_base[tid] = digit_base[tid] + excl;
    }
    __syncthreads();
    if (S.failed) return;
    // Stage the tile in digit order (stable), then write it out.
#pragma unroll
    for (int j = 0; j < kItems; ++j) {
        if (d[j] < kBins) {
            const uint32_t pos = S.tile_bin_start[d[j]] + S.warp_hist[warp][d[j]] + rank[j];
            if (pos < static_cast<uint32_t>(kTile)) {
                S.keys[pos] = k[j];
                S.vals[pos] = v[j];
            } else {
                record_error(status, NBODY_ERR_CAPACITY);
            }
        }
    }
    __syncthreads();
    const int64_t valid = (n - base) < kTile ? (n - base) : kTile;
    for (int i = tid; i < valid; i += kSortThreads) {
        const uint64_t key = S.keys[i];
        const uint32_t b = digit_of(key, pass);
        const int64_t dst = static_cast<int64_t>(S.global_base[b]) + (i - static_cast<int64_t>(S.tile_bin_start[b]));
        if (dst < 0 || dst >= n) {  // broken offsets: report, never write out of bounds
            record_error(status, NBODY_ERR_CAPACITY);
            continue;
        }
        keys_out[dst] = key;
        vals_out[dst] = S.vals[i];
    }
}

}  // namespace

size_t sort_scratch_bytes(int64_t n) {
    const int64_t tiles = (n + kTile - 1) / kTile;
    size_t b = 0;
    b += sizeof(uint32_t) * kPasses * kBins;                       // histograms
    b += sizeof(uint32_t) * 64;                                    // tile counters (one per pass)
    b += sizeof(uint32_t) * static_cast<size_t>(tiles) * kBins * kPasses;  // look-back descriptors
    return (b + 255) & ~static_cast<size_t>(255);
}

cudaError_t sort_prepare(int device) {
    static std::mutex mu;
    static bool done[64] = {};
    std::lock_guard<std::mutex> lk(mu);
    if (device >= 0 && device < 64 && done[device]) return cudaSuccess;
    const cudaError_t e = cudaFuncSetAttribute(onesweep_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               static_cast<int>(sizeof(SortSmem)));
    if (e == cudaSuccess && device >= 0 && device < 64) done[device] = true;
    return e;
}

cudaError_t sort_pairs(uint64_t *keys, uint32_t *vals, uint64_t *keys_alt, uint32_t *vals_alt, int64_t n,
                       void *scratch, cudaStream_t stream, int *status, int *result_in_alt, int passes) {
    *result_in_alt = 0;
    if (n <= 1 || passes <= 0) return cudaSuccess;
    if (passes > kPasses) return cudaErrorInvalidValue;
    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e == cudaSuccess) e = sort_prepare(device);
    if (e != cudaSuccess) return e;
    const int64_t tiles = (n + kTile - 1) / kTile;
    uint32_t *hist = static_cast<uint32_t *>(scratch);
    uint32_t *counters = hist + kPasses * kBins;
    uint32_t *desc = counters + 64;
    // Only what this sort uses must start at zero: histograms, tile counters and
    // the look-back descriptors of `passes` passes.
    const size_t used = sizeof(uint32_t) * (kPasses * kBins + 64 + static_cast<size_t>(tiles) * kBins * passes);
    e = cudaMemsetAsync(scratch, 0, used, stream);
    if (e != cudaSuccess) return e;
    int hist_blocks = static_cast<int>((n + 8191) / 8192);
    if (hist_blocks > 1024) hist_blocks = 1024;
    histogram_kernel<<<hist_blocks, kSortThreads, 0, stream>>>(keys, n, passes, hist);
    histogram_scan_kernel<<<passes, kBins, 0, stream>>>(hist);
    uint64_t *ki = keys, *ko = keys_alt;
    uint32_t *vi = vals, *vo = vals_alt;
    for (int p = 0; p < passes; ++p) {
        onesweep_kernel<<<static_cast<unsigned>(tiles), kSortThreads, sizeof(SortSmem), stream>>>(
            ki, vi, ko, vo, n, p, hist + p * kBins, counters + p, desc + static_cast<int64_t>(p) * tiles * kBins,
            status);
        uint64_t *tk = ki; ki = ko; ko = tk;
        uint32_t *tv = vi; vi = vo; vo = tv;
    }
    *result_in_alt = (ki == keys_alt) ? 1 : 0;  // an odd pass count leaves the result in the alternates
    return cudaGetLastError();
}

}  // namespace nbody
