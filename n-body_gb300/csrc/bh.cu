// Barnes-Hut gravity for sm_103a: per-step bounding box, 63-bit Morton keys,
// stable radix sort, state gather, octree from sorted keys, bottom-up mass /
// centre of mass, and a warp-cooperative walk with the reference's opening
// criterion and integrator fused in: by default the cell walk (a cell's
// children decided for whole sets of bodies from their box, body by body only
// where the set disagrees), or the stackless union walk (NBODY_BH_WALK=union);
// both give every body exactly the records its own reference walk accepts.
//
// Replaces the reference's -v 6 CPU path (ParticleSolverBHutCPUParallel,
// src/ParticleSolver/ParticleSolverBHutCPUParallel/ParticleSolverBHutCPUParallel.cpp:18-41
// over ParallelOctreeCPU, src/Octree/ParallelOctreeCPU.cpp) and the -v 7 GLSL
// path (ParallelOctreeGPU + shaders #18-32).
//
// Tree. The reference inserts bodies one by one into an octree over the
// per-step box, subdividing a leaf until its two bodies separate, then prunes
// empty children (Octree.cpp:81-294). The cells it ends up with are the
// dyadic cells of the box that hold >= 2 bodies (plus chains of cells with a
// single occupied child, which a traversal treats exactly like their only
// child) and single-body leaves. With the bodies sorted by 63-bit Morton key,
// those cells are the octree levels L = floor(delta / 3) of a binary radix
// tree over the keys (delta = common prefix length in bits; Karras 2012): a
// radix-tree node is a cell top when its level exceeds its parent's. Cells
// are laid out in depth-first pre-order, so a cell's first child is the next
// record and `next` (the escape link of Octree.cpp:303-338) is the first
// record after its subtree. For a body b let mask[b] be the set of levels of
// cells whose first body is b and cnt[b] = |mask[b]| + (b is a lone body);
// with P the exclusive prefix sum of cnt, the cells starting at b occupy
// records P[b] .. in order of level and b's own leaf comes last; a cell whose
// bodies are [lo, hi] has next = P[hi + 1]. Bodies with identical 63-bit keys
// share one leaf record (a "bucket") and interact one by one.
//
// Cell geometry follows the reference bit for bit: a cell's box is the root
// box halved level by level in FP32 as Octree::subdivide does
// (Octree.cpp:159-231: w = max - min; centre = min + w / 2), and the opening
// test is s*s < theta2 * d2 with s the largest side, d2 = dx*dx + dy*dy + dz*dz
// evaluated without FMA contraction (Octree.cpp:303-338).
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cstdlib>
#include <cstring>

#include "bh.h"
#include "common.cuh"
#include "sort.h"

namespace nbody {

namespace {

constexpr int kMaxLevel = 21;

__device__ __forceinline__ int level_of(int delta) {
    const int l = delta / 3;
    return l < kMaxLevel ? l : kMaxLevel;
}

// Several systems packed back to back (an ensemble) are told apart by the
// per-body system id sv.seg. The radix tree then runs over the composite keys
// (system id as 32 leading bits, then the 63-bit key, then the index), so
// delta between bodies of different systems is below 32 and inside a system it
// is 32 + the key's delta. Nodes with delta < 32 join systems and are no
// octree cell (level -1); below them each system's subtree is exactly the tree
// of that system alone. sv.seg == nullptr is the single-system solver.
__device__ __forceinline__ int level_c(int delta, int base) {
    return delta < base ? -1 : level_of(delta - base);
}

__device__ __forceinline__ bool same_key(const uint64_t *__restrict__ k, const SegView &sv, int64_t a, int64_t b) {
    return k[a] == k[b] && (sv.seg == nullptr || sv.seg[a] == sv.seg[b]);
}

__device__ __forceinline__ const float *box_of(const SegView &sv, const float *box, int64_t body) {
    return sv.seg ? sv.boxes + 8 * sv.seg[body] : box;
}

// ------------------------------------------------------------- bounding box
// Reference seeds: min = FLT_MAX, max = FLT_MIN (ParallelOctreeCPU.cpp:77-82),
// strict comparisons. min/max are order-independent, so the result is exact.
__global__ void bbox_kernel(const float4 *__restrict__ pos, int64_t n, float *__restrict__ partial,
                            unsigned *__restrict__ counter, float *__restrict__ box) {
    float mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX};
    float mx[3] = {FLT_MIN, FLT_MIN, FLT_MIN};
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
        const float4 p = pos[i];
        if (p.x < mn[0]) mn[0] = p.x;
        if (p.y < mn[1]) mn[1] = p.y;
        if (p.z < mn[2]) mn[2] = p.z;
        if (p.x > mx[0]) mx[0] = p.x;
        if (p.y > mx[1]) mx[1] = p.y;
        if (p.z > mx[2]) mx[2] = p.z;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const float o1 = __shfl_down_sync(0xffffffffu, mn[a], off);
            const float o2 = __shfl_down_sync(0xffffffffu, mx[a], off);
            if (o1 < mn[a]) mn[a] = o1;
            if (o2 > mx[a]) mx[a] = o2;
        }
    }
    __shared__ float wm[32][6];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (lane == 0) {
        for (int a = 0; a < 3; ++a) {
            wm[warp][a] = mn[a];
            wm[warp][3 + a] = mx[a];
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < nw; ++w)
            for (int a = 0; a < 3; ++a) {
                if (wm[w][a] < wm[0][a]) wm[0][a] = wm[w][a];
                if (wm[w][3 + a] > wm[0][3 + a]) wm[0][3 + a] = wm[w][3 + a];
            }
        for (int a = 0; a < 6; ++a) partial[blockIdx.x * 6 + a] = wm[0][a];
        __threadfence();
        last = atomicAdd(counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    // Last block: every thread folds a strided share of the partials, then
    // the block reduces as above.
    __threadfence();
    float r[6] = {FLT_MAX, FLT_MAX, FLT_MAX, FLT_MIN, FLT_MIN, FLT_MIN};
    for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x)
        for (int a = 0; a < 3; ++a) {
            const float lo = __ldcg(&partial[b * 6 + a]);
            const float hi = __ldcg(&partial[b * 6 + 3 + a]);
            if (lo < r[a]) r[a] = lo;
            if (hi > r[3 + a]) r[3 + a] = hi;
        }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const float o1 = __shfl_down_sync(0xffffffffu, r[a], off);
            const float o2 = __shfl_down_sync(0xffffffffu, r[3 + a], off);
            if (o1 < r[a]) r[a] = o1;
            if (o2 > r[3 + a]) r[3 + a] = o2;
        }
    }
    __syncthreads();
    if (lane == 0)
        for (int a = 0; a < 6; ++a) wm[warp][a] = r[a];
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < nw; ++w)
            for (int a = 0; a < 3; ++a) {
                if (wm[w][a] < wm[0][a]) wm[0][a] = wm[w][a];
                if (wm[w][3 + a] > wm[0][3 + a]) wm[0][3 + a] = wm[w][3 + a];
            }
        for (int a = 0; a < 6; ++a) box[a] = wm[0][a];
        *counter = 0u;
    }
}

// ------------------------------------------------------------- Morton keys
__device__ __forceinline__ uint64_t expand21(uint64_t v) {
    v &= 0x1FFFFFull;
    v = (v | (v << 32)) & 0x001F00000000FFFFull;
    v = (v | (v << 16)) & 0x001F0000FF0000FFull;
    v = (v | (v << 8)) & 0x100F00F00F00F00Full;
    v = (v | (v << 4)) & 0x10C30C30C30C30C3ull;
    v = (v | (v << 2)) & 0x1249249249249249ull;
    return v;
}

// morton.glsl:49-51,68-75 with 2^21 cells per axis, each step one IEEE op.
__device__ __forceinline__ uint32_t quantize21(float p, float lo, float hi) {
    float ext = __fsub_rn(hi, lo);
    if (!(ext > 1e-6f)) ext = 1e-6f;
    float t = __fdiv_rn(__fsub_rn(p, lo), ext);
    if (t < 0.f) t = 0.f;
    if (t > 1.f) t = 1.f;
    float g = __fmul_rn(t, 2097152.0f);
    if (g > 2097151.0f) g = 2097151.0f;
    return __float2uint_rz(g);
}

// The reference's own octree descent (Octree::getNextNode with the child
// boxes of Octree::subdivide, src/Octree/Octree.cpp:148-231) taken 21 levels
// deep from the root box: per level and axis, centre = min + (max - min) / 2 in
// FP32 and the body goes to the upper half unless pos < centre. The key bits
// are the halves taken (1 = upper), x highest in each triple, so cells of
// this key are exactly the reference's cells and body membership is decided
// by the same comparisons.
__device__ __forceinline__ uint64_t octree_key(float px, float py, float pz, const float *__restrict__ box) {
    float mn[3] = {box[0], box[1], box[2]};
    float mx[3] = {box[3], box[4], box[5]};
    const float p[3] = {px, py, pz};
    uint64_t key = 0;
    for (int l = 0; l < 21; ++l) {
        uint32_t digit = 0;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const float c = __fadd_rn(mn[a], __fmul_rn(__fsub_rn(mx[a], mn[a]), 0.5f));
            const bool upper = !(p[a] < c);
            if (upper) mn[a] = c; else mx[a] = c;
            digit |= static_cast<uint32_t>(upper) << (2 - a);
        }
        key = (key << 3) | digit;
    }
    return key;
}

template <int MODE>
__global__ void morton_kernel(const float4 *__restrict__ pos, int64_t n, const float *__restrict__ box,
                              uint64_t *__restrict__ keys, uint32_t *__restrict__ vals) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p = pos[i];
    if (MODE == NBODY_KEYS_MORTON) {
        const uint64_t qx = quantize21(p.x, box[0], box[3]);
        const uint64_t qy = quantize21(p.y, box[1], box[4]);
        const uint64_t qz = quantize21(p.z, box[2], box[5]);
        keys[i] = (expand21(qx) << 2) | (expand21(qy) << 1) | expand21(qz);
    } else {
        keys[i] = octree_key(p.x, p.y, p.z, box);
    }
    if (vals) vals[i] = static_cast<uint32_t>(i);
}

// ------------------------------------------- ensemble: per-system boxes
// Float min / max through unsigned atomics on an order-preserving encoding
// (exact and order-independent, as the single-system reduction).
__device__ __forceinline__ unsigned ord_of(float f) {
    const unsigned u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float float_of(unsigned o) {
    return __uint_as_float((o & 0x80000000u) ? (o & 0x7fffffffu) : ~o);
}

// One CTA per chunk of one system (chunk = {system, first, end, chunks of the
// system}). Accumulators start at the reference's seeds (min FLT_MAX, max
// FLT_MIN); the system's last chunk writes the box and re-seeds them.
__global__ void __launch_bounds__(256) bbox_seg_kernel(const float4 *__restrict__ pos,
                                                       const int4 *__restrict__ chunks,
                                                       unsigned *__restrict__ acc, float *__restrict__ boxes) {
    const int4 c = chunks[blockIdx.x];
    float mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX};
    float mx[3] = {FLT_MIN, FLT_MIN, FLT_MIN};
    for (int i = c.y + threadIdx.x; i < c.z; i += blockDim.x) {
        const float4 p = pos[i];
        if (p.x < mn[0]) mn[0] = p.x;
        if (p.y < mn[1]) mn[1] = p.y;
        if (p.z < mn[2]) mn[2] = p.z;
        if (p.x > mx[0]) mx[0] = p.x;
        if (p.y > mx[1]) mx[1] = p.y;
        if (p.z > mx[2]) mx[2] = p.z;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const float o1 = __shfl_down_sync(0xffffffffu, mn[a], off);
            const float o2 = __shfl_down_sync(0xffffffffu, mx[a], off);
            if (o1 < mn[a]) mn[a] = o1;
            if (o2 > mx[a]) mx[a] = o2;
        }
    }
    __shared__ float wm[8][6];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0)
        for (int a = 0; a < 3; ++a) {
            wm[warp][a] = mn[a];
            wm[warp][3 + a] = mx[a];
        }
    __syncthreads();
    if (threadIdx.x != 0) return;
    for (int w = 1; w < static_cast<int>(blockDim.x >> 5); ++w)
        for (int a = 0; a < 3; ++a) {
            if (wm[w][a] < wm[0][a]) wm[0][a] = wm[w][a];
            if (wm[w][3 + a] > wm[0][3 + a]) wm[0][3 + a] = wm[w][3 + a];
        }
    unsigned *A = acc + 8 * c.x;
    for (int a = 0; a < 3; ++a) {
        atomicMin(&A[a], ord_of(wm[0][a]));
        atomicMax(&A[3 + a], ord_of(wm[0][3 + a]));
    }
    __threadfence();
    if (atomicAdd(&A[6], 1u) != static_cast<unsigned>(c.w - 1)) return;
    __threadfence();
    float *B = boxes + 8 * c.x;
    for (int a = 0; a < 6; ++a) B[a] = float_of(atomicAdd(&A[a], 0u));
    for (int a = 0; a < 3; ++a) {
        A[a] = ord_of(FLT_MAX);
        A[3 + a] = ord_of(FLT_MIN);
    }
    A[6] = 0u;
}

__global__ void seed_box_acc_kernel(unsigned *__restrict__ acc, int systems) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= systems) return;
    for (int a = 0; a < 3; ++a) {
        acc[8 * s + a] = ord_of(FLT_MAX);
        acc[8 * s + 3 + a] = ord_of(FLT_MIN);
    }
    acc[8 * s + 6] = 0u;
    acc[8 * s + 7] = 0u;
}

// Keys over each body's own system box; the unsorted keys are kept for the
// gather (the segment passes of the sort overwrite the key array).
template <int MODE>
__global__ void keys_seg_kernel(const float4 *__restrict__ pos, int64_t n, const int *__restrict__ seg,
                                const float *__restrict__ boxes, uint64_t *__restrict__ keys,
                                uint64_t *__restrict__ keys_orig, uint32_t *__restrict__ vals) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p = pos[i];
    const float *box = boxes + 8 * seg[i];
    uint64_t key;
    if (MODE == NBODY_KEYS_MORTON) {
        const uint64_t qx = quantize21(p.x, box[0], box[3]);
        const uint64_t qy = quantize21(p.y, box[1], box[4]);
        const uint64_t qz = quantize21(p.z, box[2], box[5]);
        key = (expand21(qx) << 2) | (expand21(qy) << 1) | expand21(qz);
    } else {
        key = octree_key(p.x, p.y, p.z, box);
    }
    keys[i] = key;
    keys_orig[i] = key;
    vals[i] = static_cast<uint32_t>(i);
}

// Sort key of the segment passes: the system of the body now at slot j.
__global__ void seg_keys_kernel(const uint32_t *__restrict__ vals, int64_t n, const int *__restrict__ seg,
                                uint64_t *__restrict__ out, int *status) {
    const int64_t j = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j >= n) return;
    uint32_t v = vals[j];
    if (v >= static_cast<uint64_t>(n)) {
        record_error(status, NBODY_ERR_CAPACITY);
        v = 0;
    }
    out[j] = static_cast<uint64_t>(seg[v]);
}

// ------------------------------------------------------------------ gather
__global__ void gather_kernel(const uint32_t *__restrict__ perm, int64_t n, const float4 *__restrict__ pos_in,
                              const float4 *__restrict__ vel_in, const float4 *__restrict__ acc_in,
                              const int *__restrict__ id_in, float4 *__restrict__ pos_out,
                              float4 *__restrict__ vel_out, float4 *__restrict__ acc_out,
                              int *__restrict__ id_out, int *status, const uint64_t *__restrict__ key_in,
                              uint64_t *__restrict__ key_out) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t j = perm[i];
    if (j >= static_cast<uint64_t>(n)) {  // not a permutation: report, read in bounds
        record_error(status, NBODY_ERR_CAPACITY);
        j = 0;
    }
    pos_out[i] = pos_in[j];
    if (vel_out) vel_out[i] = vel_in[j];
    if (acc_out) acc_out[i] = acc_in[j];
    if (id_out) id_out[i] = id_in ? id_in[j] : static_cast<int>(j);
    if (key_out) key_out[i] = key_in[j];
}

// ------------------------------------------------------ binary radix tree
__device__ __forceinline__ int delta_at(const uint64_t *__restrict__ k, const int *__restrict__ seg, int64_t n,
                                        int64_t i, int64_t j) {
    if (j < 0 || j >= n) return -1;
    int base = 0;
    if (seg) {
        const int si = seg[i], sj = seg[j];
        if (si != sj) return __clz(si ^ sj);
        base = 32;
    }
    const uint64_t a = k[i], b = k[j];
    if (a != b) return base + __clzll(static_cast<long long>(a ^ b)) - 1;  // bit 63 is always 0
    return base + 63 + __clz(static_cast<int>(i ^ j));                        // equal keys: break ties by index
}

__global__ void radix_tree_kernel(const uint64_t *__restrict__ k, int64_t n, BinaryTree t, SegView sv,
                                  uint32_t *__restrict__ mask, int base) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    const int *seg = sv.seg;
    const int dl = delta_at(k, seg, n, i, i - 1), dr = delta_at(k, seg, n, i, i + 1);
    const int d = dr > dl ? 1 : -1;
    const int dmin = d > 0 ? dl : dr;
    int64_t lmax = 2;
    while (delta_at(k, seg, n, i, i + lmax * d) > dmin) lmax *= 2;
    int64_t l = 0;
    for (int64_t s = lmax / 2; s >= 1; s /= 2)
        if (delta_at(k, seg, n, i, i + (l + s) * d) > dmin) l += s;
    const int64_t j = i + l * d;
    const int dnode = delta_at(k, seg, n, i, j);
    int64_t s = 0;
    int64_t step = l;
    do {
        step = (step + 1) >> 1;
        if (delta_at(k, seg, n, i, i + (s + step) * d) > dnode) s += step;
    } while (step > 1);
    const int64_t gamma = i + s * d + (d < 0 ? -1 : 0);
    const int64_t lo = i < j ? i : j, hi = i < j ? j : i;
    const int left = (lo == gamma) ? ~static_cast<int>(gamma) : static_cast<int>(gamma);
    const int right = (hi == gamma + 1) ? ~static_cast<int>(gamma + 1) : static_cast<int>(gamma + 1);
    t.lo[i] = static_cast<int>(lo);
    t.hi[i] = static_cast<int>(hi);
    t.left[i] = left;
    t.right[i] = right;
    t.delta[i] = dnode;
    if (left < 0) t.lparent[~left] = static_cast<int>(i); else t.iparent[left] = static_cast<int>(i);
    if (right < 0) t.lparent[~right] = static_cast<int>(i); else t.iparent[right] = static_cast<int>(i);
    if (i == 0) t.iparent[0] = -1;
    // Cell top: a node whose octree level exceeds its parent's. A node is the
    // maximal range sharing its prefix, so its parent extends it across the
    // end whose neighbour is the more similar one, and the parent's delta is
    // the larger of the deltas across the two ends (-1 past the array).
    const int L = level_c(dnode, base);
    const int dp = i == 0 ? -1 : max(delta_at(k, seg, n, lo, lo - 1), delta_at(k, seg, n, hi, hi + 1));
    const int Lp = i == 0 ? -1 : level_c(dp, base);
    const bool top = L > Lp;
    t.top[i] = top ? 1 : 0;
    if (top) atomicOr(&mask[lo], 1u << L);
}

__global__ void count_nodes_kernel(const uint64_t *__restrict__ k, int64_t n, const uint32_t *__restrict__ mask,
                                   uint32_t *__restrict__ cnt, SegView sv) {
    const int64_t b = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (b >= n) return;
    const bool lone = !((b > 0 && same_key(k, sv, b, b - 1)) || (b + 1 < n && same_key(k, sv, b, b + 1)));
    cnt[b] = __popc(mask[b]) + (lone ? 1u : 0u);
}

// Side^2 of the level-L cell holding `key`: the root box halved L times in
// FP32 exactly as Octree::subdivide computes child boxes.
__device__ __forceinline__ float cell_side2(uint64_t key, int L, const float *__restrict__ box) {
    float mn[3] = {box[0], box[1], box[2]};
    float mx[3] = {box[3], box[4], box[5]};
    for (int l = 1; l <= L; ++l) {
        const uint32_t dgt = static_cast<uint32_t>(key >> (63 - 3 * l)) & 7u;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const float w = __fsub_rn(mx[a], mn[a]);
            const float c = __fadd_rn(mn[a], __fmul_rn(w, 0.5f));
            // key bit 1 = upper half [min + w/2, max]; 0 = lower half [min, min + w/2]
            if ((dgt >> (2 - a)) & 1u) mn[a] = c; else mx[a] = c;
        }
    }
    const float sx = __fsub_rn(mx[0], mn[0]), sy = __fsub_rn(mx[1], mn[1]), sz = __fsub_rn(mx[2], mn[2]);
    const float sxy = sx < sy ? sy : sx;
    const float s = sxy < sz ? sz : sxy;
    return __fmul_rn(s, s);
}

// Record index of the cell whose top radix-tree node is p.
__device__ __forceinline__ int record_of(const BinaryTree &t, const uint32_t *__restrict__ mask,
                                         const uint32_t *__restrict__ P, int p, int base) {
    const int L = level_c(t.delta[p], base);
    const int lo = t.lo[p];
    return static_cast<int>(P[lo] + __popc(mask[lo] & ((1u << L) - 1u)));
}

// Octree parent of a record: the nearest radix-tree ancestor that is a cell
// top (the nodes in between split the same cell; at most 6 of them).
__device__ __forceinline__ int octree_parent(const BinaryTree &t, const uint32_t *__restrict__ mask,
                                             const uint32_t *__restrict__ P, int p, int base) {
    // At most 6 nodes per octree level inside a system, and at most 32 joining
    // nodes (strictly decreasing delta < 32) above a system's subtree.
    for (int guard = 0; p >= 0 && !t.top[p] && guard < 160; ++guard) p = t.iparent[p];
    return (p >= 0 && t.top[p]) ? record_of(t, mask, P, p, base) : -1;
}

__global__ void emit_cells_kernel(const uint64_t *__restrict__ k, int64_t n, BinaryTree t,
                                  const uint32_t *__restrict__ mask, const uint32_t *__restrict__ P,
                                  const float *__restrict__ box, BHNode *__restrict__ nodes, Records r, SegView sv,
                                  bool parents) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    if (!t.top[i]) return;
    const int base = sv.seg ? 32 : 0;
    const int L = level_c(t.delta[i], base);
    const int lo = t.lo[i], hi = t.hi[i];
    const int idx = record_of(t, mask, P, static_cast<int>(i), base);
    int4 meta;
    if (L < kMaxLevel) {
        meta = make_int4(__float_as_int(cell_side2(k[lo], L, box_of(sv, box, lo))), static_cast<int>(P[hi + 1]), lo,
                         0);
    } else {  // bucket of bodies with identical keys: a leaf
        meta = make_int4(__float_as_int(-1.f), static_cast<int>(P[hi + 1]), lo, hi - lo + 1);
    }
    nodes[idx].meta = meta;
    r.level[idx] = L;
    if (parents) {  // the climbing upsweep's links
        const int par = i == 0 ? -1 : octree_parent(t, mask, P, t.iparent[i], base);
        r.parent[idx] = par;
        if (par >= 0) atomicAdd(&r.nchild[par], 1);
    }
}

__global__ void emit_leaves_kernel(const uint64_t *__restrict__ k, int64_t n, const float4 *__restrict__ pos,
                                   BinaryTree t, const uint32_t *__restrict__ mask, const uint32_t *__restrict__ P,
                                   BHNode *__restrict__ nodes, Records r, SegView sv, bool parents) {
    const int64_t b = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (b >= n) return;
    const bool lone = !((b > 0 && same_key(k, sv, b, b - 1)) || (b + 1 < n && same_key(k, sv, b, b + 1)));
    if (!lone) return;
    const int idx = static_cast<int>(P[b] + __popc(mask[b]));
    nodes[idx].cm = pos[b];
    nodes[idx].meta = make_int4(__float_as_int(-1.f), static_cast<int>(P[b + 1]), static_cast<int>(b), 1);
    r.level[idx] = kMaxLevel + 1;  // a lone body
    if (parents) {
        const int par = n < 2 ? -1 : octree_parent(t, mask, P, t.lparent[b], sv.seg ? 32 : 0);
        r.parent[idx] = par;
        if (par >= 0) atomicAdd(&r.nchild[par], 1);
    }
}

// kids[8 r + j]: the record of the j-th child of cell r in pre-order (the
// chain r + 1, next(r + 1), ... before next(r)), -1 after the last; a cell
// has at most 8. Leaves and buckets get no entry. For the cell walk, which
// decides a cell's children side by side.
__global__ void kids_kernel(const BHNode *__restrict__ nodes, const uint32_t *__restrict__ total, int64_t cap,
                            int *__restrict__ kids, int *status) {
    const int64_t r = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const int64_t m = static_cast<int64_t>(*total) < cap ? static_cast<int64_t>(*total) : cap;
    if (r >= m) return;
    const int4 meta = nodes[r].meta;
    if (__int_as_float(meta.x) < 0.f) return;  // a leaf or a bucket
    const int64_t end = meta.y < m ? meta.y : m;
    int k[8];
    int64_t c = r + 1;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        k[j] = -1;
        if (c < end) {
            k[j] = static_cast<int>(c);
            const int64_t nx = nodes[c].meta.y;
            c = nx > c ? nx : end;
        }
    }
    if (c < end) record_error(status, NBODY_ERR_CAPACITY);  // more than 8 children: broken tree
    int4 *out = reinterpret_cast<int4 *>(kids + 8 * r);
    out[0] = make_int4(k[0], k[1], k[2], k[3]);
    out[1] = make_int4(k[4], k[5], k[6], k[7]);
}

// The reference's child order (Octree::getNextNode, src/Octree/Octree.cpp:148-153):
// index bit a is set when the body lies below the centre on axis a (x = bit 0),
// while a Morton digit bit is set for the upper half (x = bit 2).
__device__ __forceinline__ int reference_child_index(uint32_t digit) {
    return static_cast<int>(((~digit >> 2) & 1u) | ((~digit) & 2u) | (((~digit) & 1u) << 2));
}

// Bottom-up centres of mass in the reference's arithmetic
// (ParallelOctreeCPU::propagate / Octree::propagate, Octree.cpp:238-258): a
// cell's centre is sum(child centre * child mass) / sum(child mass) over its
// occupied children in the reference's child order, every step rounded on its
// own. A cell of the reference's tree that has a single occupied child is
// skipped here but leaves its trace: (c * m) / m once per skipped level. The
// reference also keeps lone bodies no shallower than its fixed top levels
// (depth `father_depth`). A cell all of whose children are leaves is flagged
// (meta.w = -bodies) so the traversal can sum its bodies directly. Two
// schedules give the same bits: the climb (one launch; the last child to
// arrive at a cell computes it and climbs on) and the level schedule (bucket
// leaves, then one launch per octree level from the deepest up, no atomics),
// which is faster from about 2^21 bodies and for ensembles.
// A cell's children by the reference's child index, in registers: each store
// is eight predicated selects, so no slot is addressed dynamically. The level
// schedule uses it (0.375 vs 0.481 ms at 4M bodies against an array in local
// memory, whose traffic reached DRAM); the climb keeps the local array, which
// costs it fewer registers and so more threads in flight (0.189 vs 0.258 ms
// at 2^20).
struct ChildSlots {
    float4 s[8];
    unsigned used = 0;
    __device__ __forceinline__ void put(int j, float4 v) {
#pragma unroll
        for (int q = 0; q < 8; ++q) s[q] = j == q ? v : s[q];
        used |= 1u << j;
    }
    // Sum(c * m) / Sum(m) over the occupied slots in index order, every step
    // rounded on its own.
    __device__ __forceinline__ float4 centre() const {
        float cx = 0.f, cy = 0.f, cz = 0.f, m = 0.f;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            if (!((used >> j) & 1u)) continue;
            cx = __fadd_rn(cx, __fmul_rn(s[j].x, s[j].w));
            cy = __fadd_rn(cy, __fmul_rn(s[j].y, s[j].w));
            cz = __fadd_rn(cz, __fmul_rn(s[j].z, s[j].w));
            m = __fadd_rn(m, s[j].w);
        }
        return m > 0.f ? make_float4(__fdiv_rn(cx, m), __fdiv_rn(cy, m), __fdiv_rn(cz, m), m)
                       : make_float4(0.f, 0.f, 0.f, 0.f);
    }
};

__device__ __forceinline__ float4 round_trips(float4 c, int times) {
    for (int q = 0; q < times; ++q) {
        c.x = __fdiv_rn(__fmul_rn(c.x, c.w), c.w);
        c.y = __fdiv_rn(__fmul_rn(c.y, c.w), c.w);
        c.z = __fdiv_rn(__fmul_rn(c.z, c.w), c.w);
    }
    return c;
}

// Centre of mass of the bucket (bodies with identical keys) whose first body
// is b: its occupied bodies in body order, each step rounded on its own.
__device__ __forceinline__ float4 bucket_cm(const uint64_t *__restrict__ k, int64_t n, const float4 *__restrict__ pos,
                                            const SegView &sv, int64_t b) {
    float cx = 0.f, cy = 0.f, cz = 0.f, m = 0.f;
    for (int64_t q = b; q < n && same_key(k, sv, q, b); ++q) {
        const float4 o = pos[q];
        if (!(o.w > 0.f)) continue;
        cx = __fadd_rn(cx, __fmul_rn(o.x, o.w));
        cy = __fadd_rn(cy, __fmul_rn(o.y, o.w));
        cz = __fadd_rn(cz, __fmul_rn(o.z, o.w));
        m = __fadd_rn(m, o.w);
    }
    return m > 0.f ? make_float4(__fdiv_rn(cx, m), __fdiv_rn(cy, m), __fdiv_rn(cz, m), m)
                   : make_float4(0.f, 0.f, 0.f, 0.f);
}

__global__ void upsweep_climb_kernel(const uint64_t *__restrict__ k, int64_t n, const float4 *__restrict__ pos,
                                     const uint32_t *__restrict__ mask, const uint32_t *__restrict__ P,
                                     BHNode *__restrict__ nodes, Records r, int father_depth, int *status,
                                     SegView sv) {
    const int64_t b = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (b >= n) return;
    if (sv.seg) father_depth = sv.fdepth[sv.seg[b]];
    const bool left_eq = b > 0 && same_key(k, sv, b, b - 1);
    const bool right_eq = b + 1 < n && same_key(k, sv, b, b + 1);
    int rec;
    if (!left_eq && !right_eq) {
        rec = static_cast<int>(P[b] + __popc(mask[b]));  // lone body: already written
    } else if (!left_eq) {
        // first body of a bucket: its record is the level-21 cell starting here
        rec = static_cast<int>(P[b] + __popc(mask[b] & ((1u << kMaxLevel) - 1u)));
        nodes[rec].cm = bucket_cm(k, n, pos, sv, b);
    } else {
        return;
    }
    for (int depth = 0; depth <= kMaxLevel + 2; ++depth) {
        const int par = r.parent[rec];
        if (par < 0) return;
        __threadfence();
        const int done = static_cast<int>(atomicAdd(&r.arrive[par], 1u)) + 1;
        if (done < __ldcg(&r.nchild[par])) return;
        __threadfence();
        const int L = __ldcg(&r.level[par]);
        const int4 pm = __ldcg(&nodes[par].meta);
        float4 slot[8];
        bool used[8] = {false, false, false, false, false, false, false, false};
        bool all_leaves = true;
        int bodies = 0;
        int c = par + 1;
        for (int guard = 0; c < pm.y && guard < 8; ++guard) {
            const int4 cmeta = __ldcg(&nodes[c].meta);
            float4 cc = __ldcg(&nodes[c].cm);
            const int cl = __ldcg(&r.level[c]);
            const uint32_t digit = static_cast<uint32_t>(k[cmeta.z] >> (63 - 3 * (L + 1))) & 7u;
            int trips;
            if (cl > kMaxLevel || cl == kMaxLevel) {  // a leaf (lone body or bucket)
                trips = father_depth - (L + 1) > 0 ? father_depth - (L + 1) : 0;
                bodies += cmeta.w;
            } else {
                trips = cl - L - 1;
                all_leaves = false;
            }
            if (cc.w > 0.f) {
                const int j = reference_child_index(digit);
                slot[j] = round_trips(cc, trips);
                used[j] = true;
            }
            c = cmeta.y;
        }
        if (c != pm.y) record_error(status, NBODY_ERR_CAPACITY);  // more than 8 children: broken tree
        float cx = 0.f, cy = 0.f, cz = 0.f, m = 0.f;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            if (!used[j]) continue;
            cx = __fadd_rn(cx, __fmul_rn(slot[j].x, slot[j].w));
            cy = __fadd_rn(cy, __fmul_rn(slot[j].y, slot[j].w));
            cz = __fadd_rn(cz, __fmul_rn(slot[j].z, slot[j].w));
            m = __fadd_rn(m, slot[j].w);
        }
        nodes[par].cm = m > 0.f ? make_float4(__fdiv_rn(cx, m), __fdiv_rn(cy, m), __fdiv_rn(cz, m), m)
                                : make_float4(0.f, 0.f, 0.f, 0.f);
        if (all_leaves) nodes[par].meta.w = -bodies;
        rec = par;
    }
    record_error(status, NBODY_ERR_CAPACITY);  // deeper than any octree: broken tree
}

// Buckets (bodies with identical keys; a level-kMaxLevel leaf): the centre of
// mass of their occupied bodies, in body order. Lone-body leaves already hold
// their body.
__global__ void bucket_cm_kernel(const uint64_t *__restrict__ k, int64_t n, const float4 *__restrict__ pos,
                                 const uint32_t *__restrict__ mask, const uint32_t *__restrict__ P,
                                 BHNode *__restrict__ nodes, SegView sv) {
    const int64_t b = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (b >= n) return;
    const bool left_eq = b > 0 && same_key(k, sv, b, b - 1);
    const bool right_eq = b + 1 < n && same_key(k, sv, b, b + 1);
    if (left_eq || !right_eq) return;  // not the first body of a bucket
    const int rec = static_cast<int>(P[b] + __popc(mask[b] & ((1u << kMaxLevel) - 1u)));
    nodes[rec].cm = bucket_cm(k, n, pos, sv, b);
}

// Cells per octree level (levels 0 .. kMaxLevel - 1) over records [0, *total).
__global__ void level_count_kernel(const int *__restrict__ level, const uint32_t *__restrict__ total,
                                   unsigned *__restrict__ lvl) {
    __shared__ unsigned h[kMaxLevel];
    if (threadIdx.x < kMaxLevel) h[threadIdx.x] = 0u;
    __syncthreads();
    const int64_t nrec = *total;
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t r = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; r < nrec; r += stride) {
        const int L = level[r];
        if (L >= 0 && L < kMaxLevel) atomicAdd(&h[L], 1u);
    }
    __syncthreads();
    if (threadIdx.x < kMaxLevel && h[threadIdx.x]) atomicAdd(&lvl[threadIdx.x], h[threadIdx.x]);
}

// Groups the cell records by level into list (one record per thread; the grid
// covers the record capacity): a block reserves one range per level with a
// single global atomic, its records take consecutive places in it.
__global__ void level_scatter_kernel(const int *__restrict__ level, const uint32_t *__restrict__ total,
                                     unsigned *__restrict__ lvl, unsigned *__restrict__ list, int64_t cap,
                                     int *status) {
    __shared__ unsigned h[kMaxLevel], base[kMaxLevel], off[kMaxLevel];
    if (threadIdx.x == 0) {
        unsigned run = 0;
        for (int L = 0; L < kMaxLevel; ++L) {
            off[L] = run;
            run += lvl[L];
        }
    }
    if (threadIdx.x < kMaxLevel) h[threadIdx.x] = 0u;
    __syncthreads();
    if (blockIdx.x == 0 && threadIdx.x < kMaxLevel) lvl[32 + threadIdx.x] = off[threadIdx.x];
    const int64_t r = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const int L = r < *total ? level[r] : -1;
    const bool cell = L >= 0 && L < kMaxLevel;
    const unsigned local = cell ? atomicAdd(&h[L], 1u) : 0u;
    __syncthreads();
    if (threadIdx.x < kMaxLevel && h[threadIdx.x])
        base[threadIdx.x] = off[threadIdx.x] + atomicAdd(&lvl[64 + threadIdx.x], h[threadIdx.x]);
    __syncthreads();
    if (!cell) return;
    const int64_t at = static_cast<int64_t>(base[L]) + local;
    if (at >= cap) {
        record_error(status, NBODY_ERR_CAPACITY);
        return;
    }
    list[at] = static_cast<unsigned>(r);
}

// The cells of one level: each sums its children (already final) in the
// reference's child order.
// Four CTAs per SM (64 registers): the eight register slots fit without spills.
__global__ void __launch_bounds__(256, 4)
    level_cm_kernel(int L, const uint64_t *__restrict__ k, int64_t n, BHNode *__restrict__ nodes,
                    const int *__restrict__ level, const unsigned *__restrict__ list, const unsigned *__restrict__ lvl,
                    int father_depth, int *status, SegView sv) {
    const unsigned count = lvl[L], first = lvl[32 + L];
    const unsigned stride = gridDim.x * blockDim.x;
    for (unsigned q = blockIdx.x * blockDim.x + threadIdx.x; q < count; q += stride) {
        const int par = static_cast<int>(list[first + q]);
        const int4 pm = nodes[par].meta;
        const int fd = sv.seg ? sv.fdepth[sv.seg[pm.z]] : father_depth;
        ChildSlots slot;
        bool all_leaves = true;
        int bodies = 0;
        int c = par + 1;
        for (int guard = 0; c < pm.y && guard < 8; ++guard) {
            const int4 cmeta = nodes[c].meta;
            const float4 cc = nodes[c].cm;
            const int cl = level[c];
            const uint32_t digit = static_cast<uint32_t>(k[cmeta.z] >> (63 - 3 * (L + 1))) & 7u;
            int trips;
            if (cl >= kMaxLevel) {  // a leaf (lone body or bucket)
                trips = fd - (L + 1) > 0 ? fd - (L + 1) : 0;
                bodies += cmeta.w;
            } else {
                trips = cl - L - 1;
                all_leaves = false;
            }
            if (cc.w > 0.f) slot.put(reference_child_index(digit), round_trips(cc, trips));
            c = cmeta.y;
        }
        if (c != pm.y) record_error(status, NBODY_ERR_CAPACITY);  // more than 8 children: broken tree
        nodes[par].cm = slot.centre();
        if (all_leaves) nodes[par].meta.w = -bodies;
    }
}

// --------------------------------------------------------------- traversal
// One warp walks the pre-order records of the tree for its 32 bodies. A lane
// evaluates the reference criterion on each record it has not already
// covered (skip <= i); an accepted record adds its force and sets skip to
// the record's `next`. The warp descends (i + 1) if any lane opened the
// record, otherwise it jumps to the smallest `skip` of its lanes. Every lane
// therefore sees exactly the records its own reference walk would accept.
// Both bodies of a lane summing the same run of bodies in one packed loop;
// side A takes part when doA, side B when doB. Per side the arithmetic and
// its rounding are those of direct_sum_range: a side that does not take part,
// or a pair it skips (m == 0 or r^2 == 0), adds dx * 0 = +0 to its sums.
__device__ __forceinline__ void direct_sum_range2(const float4 *__restrict__ pos, int64_t n, int first, int count,
                                                  float2 nx, float2 ny, float2 nz, float eps2, bool doA, bool doB,
                                                  float2 &ax, float2 &ay, float2 &az) {
    const int q0 = first < 0 ? 0 : first;
    const int q1 = first + count < n ? first + count : static_cast<int>(n);
    for (int q = q0; q < q1; ++q) {
        const float4 o = pos[q];
        const float2 ex = __fadd2_rn(make_float2(o.x, o.x), nx);
        const float2 ey = __fadd2_rn(make_float2(o.y, o.y), ny);
        const float2 ez = __fadd2_rn(make_float2(o.z, o.z), nz);
        const float2 r2 = __fadd2_rn(__fadd2_rn(__fmul2_rn(ex, ex), __fmul2_rn(ey, ey)), __fmul2_rn(ez, ez));
        const float2 iv = make_float2(rsqrt_ftz(r2.x + eps2), rsqrt_ftz(r2.y + eps2));
        const float2 w = __fmul2_rn(__fmul2_rn(__fmul2_rn(make_float2(o.w, o.w), iv), iv), iv);
        const bool ua = doA && o.w > 0.f && r2.x > 0.f, ub = doB && o.w > 0.f && r2.y > 0.f;
        const float2 ws = make_float2(ua ? w.x : 0.f, ub ? w.y : 0.f);
        ax = __ffma2_rn(ex, ws, ax);
        ay = __ffma2_rn(ey, ws, ay);
        az = __ffma2_rn(ez, ws, az);
    }
}

__device__ __forceinline__ void integrate_sorted(int64_t b, float4 p, float fx, float fy, float fz, float dt,
                                                 float4 *__restrict__ pos_out, float4 *__restrict__ vel,
                                                 float4 *__restrict__ acc, float4 *__restrict__ force_out,
                                                 const int *__restrict__ ids, int64_t n, int euler,
                                                 const HostOut &host = HostOut{});

// COUNT adds up (per warp, one atomic each) the pairwise force evaluations
// and the records the warp visited; used for measurement only.
template <bool COUNT>
__global__ void __launch_bounds__(256) traverse_kernel(const BHNode *__restrict__ nodes,
                                                       const uint32_t *__restrict__ node_total,
                                                       const float4 *__restrict__ pos, int64_t n, float eps2,
                                                       float theta2, float dt, float4 *__restrict__ pos_out,
                                                       float4 *__restrict__ vel, float4 *__restrict__ acc,
                                                       float4 *__restrict__ force_out, const int *__restrict__ ids,
                                                       unsigned long long *__restrict__ counters, int euler) {
    unsigned long long n_pairs = 0, n_visits = 0;
    const int64_t b = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const bool valid = b < n;
    const int m_nodes = static_cast<int>(*node_total);
    const float4 me = valid ? pos[b] : make_float4(0.f, 0.f, 0.f, 0.f);
    int skip = valid ? 0 : m_nodes;
    float fx = 0.f, fy = 0.f, fz = 0.f;
    int i = 0;
    while (i < m_nodes) {
        const float4 cm = __ldg(&nodes[i].cm);
        const int4 meta = __ldg(&nodes[i].meta);
        const bool act = skip <= i;
        const float dx = __fsub_rn(cm.x, me.x), dy = __fsub_rn(cm.y, me.y), dz = __fsub_rn(cm.z, me.z);
        const float d2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
        const float s2 = __int_as_float(meta.x);
        // Octree.cpp:318: accept a leaf, or a cell with s^2 < theta^2 d^2.
        const bool acc = act && (s2 < 0.f || s2 < __fmul_rn(theta2, d2));
        // Force from the record itself (a cell's centre of mass or a lone
        // body). A branch, not a select: records every active lane opens (the
        // upper levels) then cost no force arithmetic at all.
        if (acc && meta.w <= 1 && cm.w > 0.f && d2 > 0.f) {
            if (COUNT) ++n_pairs;
            const float inv = rsqrt_ftz(d2 + eps2);
            const float w = cm.w * inv * inv * inv;
            fx = fmaf(dx, w, fx);
            fy = fmaf(dy, w, fy);
            fz = fmaf(dz, w, fz);
        }
        if (meta.w != 0 && meta.w != 1) {  // warp-uniform: a bucket or a terminal cell
            // A bucket (meta.w >= 2) accepted, or a terminal cell (meta.w < 0)
            // opened: every body in it interacts one by one.
            if ((meta.w >= 2 && acc) || (meta.w < 0 && act && !acc)) {
                const int cntb = meta.w >= 2 ? meta.w : -meta.w;
                const int q0 = meta.z < 0 ? 0 : meta.z;
                const int q1 = meta.z + cntb < n ? meta.z + cntb : static_cast<int>(n);
                for (int q = q0; q < q1; ++q) {
                    const float4 o = pos[q];
                    const float ex = __fsub_rn(o.x, me.x), ey = __fsub_rn(o.y, me.y), ez = __fsub_rn(o.z, me.z);
                    const float e2 =
                        __fadd_rn(__fadd_rn(__fmul_rn(ex, ex), __fmul_rn(ey, ey)), __fmul_rn(ez, ez));
                    if (o.w > 0.f && e2 > 0.f) {
                        if (COUNT) ++n_pairs;
                        const float iv = rsqrt_ftz(e2 + eps2);
                        const float wq = o.w * iv * iv * iv;
                        fx = fmaf(ex, wq, fx);
                        fy = fmaf(ey, wq, fy);
                        fz = fmaf(ez, wq, fz);
                    }
                }
            }
        }
        // A lane is done with this subtree if it accepted the record or summed
        // a terminal cell's bodies; otherwise an active lane opens it.
        const bool done = acc || (act && meta.w < 0);
        if (done) skip = meta.y;
        const bool open = act && !done;
        if (COUNT) ++n_visits;
        if (__any_sync(0xffffffffu, open)) {
            ++i;
        } else {
            // Every `next` lies beyond its record; max() keeps the walk finite
            // (at most m_nodes iterations) whatever the records hold.
            const int nx = static_cast<int>(__reduce_min_sync(0xffffffffu, static_cast<unsigned>(skip)));
            i = nx > i ? nx : i + 1;
        }
    }
    if (COUNT) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) n_pairs += __shfl_down_sync(0xffffffffu, n_pairs, off);
        if ((threadIdx.x & 31) == 0) {
            atomicAdd(&counters[0], n_pairs);
            atomicAdd(&counters[1], n_visits);
        }
    }
    if (!valid) return;
    integrate_sorted(b, me, fx, fy, fz, dt, pos_out, vel, acc, force_out, ids, n, euler);
}

// Two bodies per lane: a warp serves 64 consecutive sorted bodies (lane l
// holds bodies base + l and base + 32 + l), so each record load, vote and
// branch is shared by twice the bodies. The criterion and forces use packed
// f32x2 arithmetic, each lane of a pair rounded exactly as the scalar walk.
__device__ __forceinline__ void direct_sum_range(const float4 *__restrict__ pos, int64_t n, int first, int count,
                                                 float4 me, float eps2, float &fx, float &fy, float &fz,
                                                 unsigned long long &n_pairs, bool count_pairs, float &phi,
                                                 bool pot) {
    const int q0 = first < 0 ? 0 : first;
    const int q1 = first + count < n ? first + count : static_cast<int>(n);
    for (int q = q0; q < q1; ++q) {
        const float4 o = pos[q];
        const float ex = __fsub_rn(o.x, me.x), ey = __fsub_rn(o.y, me.y), ez = __fsub_rn(o.z, me.z);
        const float e2 = __fadd_rn(__fadd_rn(__fmul_rn(ex, ex), __fmul_rn(ey, ey)), __fmul_rn(ez, ez));
        if (o.w > 0.f && e2 > 0.f) {
            if (count_pairs) ++n_pairs;
            const float iv = rsqrt_ftz(e2 + eps2);
            const float wq = o.w * iv * iv * iv;
            fx = fmaf(ex, wq, fx);
            fy = fmaf(ey, wq, fy);
            fz = fmaf(ez, wq, fz);
            if (pot) phi = fmaf(-o.w, iv, phi);
        }
    }
}

// Body b's new state into the caller's arrays at its caller index.
__device__ __forceinline__ void write_host(const HostOut host, const int *__restrict__ ids, int64_t b, int64_t n,
                                        float4 p, float4 v, float4 a) {
    const int d = ids ? ids[b] : static_cast<int>(b);
    if (d < 0 || d >= n) return;
    host.pos[d] = make_float4(p.x, p.y, p.z, 0.f);
    host.vel[d] = v;
    host.acc[d] = a;
    if (host.force) host.force[d] = a;
}

__device__ __forceinline__ void integrate_sorted(int64_t b, float4 p, float fx, float fy, float fz, float dt,
                                                 float4 *__restrict__ pos_out, float4 *__restrict__ vel,
                                                 float4 *__restrict__ acc, float4 *__restrict__ force_out,
                                                 const int *__restrict__ ids, int64_t n, int euler,
                                                 const HostOut &host) {
    const float4 anew = make_float4(fx, fy, fz, 0.f);
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    if (pos_out && euler) {
        // updateParticles.glsl:44-55: v += F dt, then x += v dt.
        v = vel[b];
        v.x = __fadd_rn(v.x, __fmul_rn(fx, dt));
        v.y = __fadd_rn(v.y, __fmul_rn(fy, dt));
        v.z = __fadd_rn(v.z, __fmul_rn(fz, dt));
        p.x = __fadd_rn(p.x, __fmul_rn(v.x, dt));
        p.y = __fadd_rn(p.y, __fmul_rn(v.y, dt));
        p.z = __fadd_rn(p.z, __fmul_rn(v.z, dt));
        pos_out[b] = p;
        vel[b] = v;
        acc[b] = anew;
    } else if (pos_out) {
        // Reference integrator (include/ParticleSystem.h:52-69), no contraction.
        const float h = __fmul_rn(dt, 0.5f);
        v = vel[b];
        const float4 a = acc[b];
        v.x = __fadd_rn(v.x, __fmul_rn(a.x, h));
        v.y = __fadd_rn(v.y, __fmul_rn(a.y, h));
        v.z = __fadd_rn(v.z, __fmul_rn(a.z, h));
        p.x = __fadd_rn(p.x, __fmul_rn(v.x, dt));
        p.y = __fadd_rn(p.y, __fmul_rn(v.y, dt));
        p.z = __fadd_rn(p.z, __fmul_rn(v.z, dt));
        v.x = __fadd_rn(v.x, __fmul_rn(fx, h));
        v.y = __fadd_rn(v.y, __fmul_rn(fy, h));
        v.z = __fadd_rn(v.z, __fmul_rn(fz, h));
        pos_out[b] = p;
        vel[b] = v;
        acc[b] = anew;
    }
    if (force_out) {
        const int d = ids ? ids[b] : static_cast<int>(b);
        if (d >= 0 && d < n) force_out[d] = anew;
    }
    if (host.pos && pos_out) write_host(host, ids, b, n, p, v, anew);
}

// The union walk over the records [i, iend) (the whole tree, or the subtree
// of record i) for the lane's bodies whose flags vA / vB are set, all active
// at record i: each evaluates the reference criterion on the records it has
// not covered (skip <= i); an accepted record adds its force and sets skip to
// the record's `next`; the warp descends if any lane opened the record, else
// jumps to the smallest skip. Sums go to fx, fy, fz (x: body A, y: body B).
template <bool COUNT, bool POT, bool GUARD>
__device__ __forceinline__ void union_range(const BHNode *__restrict__ nodes, const float4 *__restrict__ pos,
                                            int64_t n, int i, const int iend, const bool vA, const bool vB,
                                            const float2 nx, const float2 ny, const float2 nz, const float2 th,
                                            const float eps2, float2 &fx, float2 &fy, float2 &fz, float &phiA,
                                            float &phiB, unsigned long long &n_pairs,
                                            unsigned long long &n_visits) {
    const float2 e2 = make_float2(eps2, eps2);
    int skipA = vA ? i : iend, skipB = vB ? i : iend;
    while (i < iend) {
        const float4 cm = __ldg(&nodes[i].cm);
        const int4 meta = __ldg(&nodes[i].meta);
        const bool actA = skipA <= i, actB = skipB <= i;
        const float2 dx = __fadd2_rn(make_float2(cm.x, cm.x), nx);
        const float2 dy = __fadd2_rn(make_float2(cm.y, cm.y), ny);
        const float2 dz = __fadd2_rn(make_float2(cm.z, cm.z), nz);
        const float2 d2 = __fadd2_rn(__fadd2_rn(__fmul2_rn(dx, dx), __fmul2_rn(dy, dy)), __fmul2_rn(dz, dz));
        const float s2 = __int_as_float(meta.x);
        const float2 rhs = __fmul2_rn(th, d2);
        bool accA, accB, useA, useB;
        if (GUARD) {
            accA = actA && (s2 < 0.f || s2 < rhs.x);
            accB = actB && (s2 < 0.f || s2 < rhs.y);
            const bool self = meta.w <= 1 && cm.w > 0.f;
            useA = accA && self && d2.x > 0.f;
            useB = accB && self && d2.y > 0.f;
        } else {
            accA = actA && s2 < rhs.x;
            accB = actB && s2 < rhs.y;
            const bool self = meta.w <= 1;  // a bucket's bodies are summed one by one below
            useA = accA && self;
            useB = accB && self;
        }
        if (useA || useB) {
            if (COUNT) n_pairs += (useA ? 1u : 0u) + (useB ? 1u : 0u);
            const float2 e = __fadd2_rn(d2, e2);
            const float2 inv = make_float2(rsqrt_ftz(e.x), rsqrt_ftz(e.y));
            const float2 inv3 = __fmul2_rn(__fmul2_rn(inv, inv), inv);
            const float2 mw = __fmul2_rn(make_float2(cm.w, cm.w), inv3);
            const float2 w = make_float2(useA ? mw.x : 0.f, useB ? mw.y : 0.f);
            fx = __ffma2_rn(dx, w, fx);
            fy = __ffma2_rn(dy, w, fy);
            fz = __ffma2_rn(dz, w, fz);
            if (POT) {
                phiA = fmaf(useA ? -cm.w : 0.f, inv.x, phiA);
                phiB = fmaf(useB ? -cm.w : 0.f, inv.y, phiB);
            }
        }
        if (meta.w != 0 && meta.w != 1) {  // warp-uniform: a bucket or a terminal cell
            const int cntb = meta.w >= 2 ? meta.w : -meta.w;
            const bool doA = (meta.w >= 2 && accA) || (meta.w < 0 && actA && !accA);
            const bool doB = (meta.w >= 2 && accB) || (meta.w < 0 && actB && !accB);
            if (COUNT || POT) {
                const float4 meA = make_float4(-nx.x, -ny.x, -nz.x, 0.f), meB = make_float4(-nx.y, -ny.y, -nz.y, 0.f);
                if (doA) direct_sum_range(pos, n, meta.z, cntb, meA, eps2, fx.x, fy.x, fz.x, n_pairs, COUNT, phiA, POT);
                if (doB) direct_sum_range(pos, n, meta.z, cntb, meB, eps2, fx.y, fy.y, fz.y, n_pairs, COUNT, phiB, POT);
            } else if (doA || doB) {
                direct_sum_range2(pos, n, meta.z, cntb, nx, ny, nz, eps2, doA, doB, fx, fy, fz);
            }
        }
        const bool doneA = accA || (actA && meta.w < 0), doneB = accB || (actB && meta.w < 0);
        if (doneA) skipA = meta.y;
        if (doneB) skipB = meta.y;
        const bool open = (actA && !doneA) || (actB && !doneB);
        if (COUNT) ++n_visits;
        if (__any_sync(0xffffffffu, open)) {
            ++i;
        } else {
            const int mine = skipA < skipB ? skipA : skipB;
            const int nx2 = static_cast<int>(__reduce_min_sync(0xffffffffu, static_cast<unsigned>(mine)));
            i = nx2 > i ? nx2 : i + 1;
        }
    }
}

// POT also accumulates the potential -sum m / sqrt(d^2 + eps^2) over the same
// accepted records (for the energy diagnostic) into phi_out[ids[b]].
// SEG: an ensemble of systems; warp w serves work[w] = {system, first body
// of the warp, first body of the system, end of the system}, walks only the
// system's records [P[first], P[end]) and takes dt, eps2, theta2 and the
// integrator from params[system] = {dt, eps2, theta2, euler}.
// GUARD keeps the reference's explicit d2 > 0 and leaf tests; without it
// (eps2 > 0, no potential) they are implied: a leaf's s2 = -1 is below
// theta2 * d2 >= 0, and a record at zero distance adds dx * w = +0 to every
// component, so the accepted set and the sums are the same bit for bit.
template <bool COUNT, bool POT, bool SEG, bool GUARD>
__global__ void __launch_bounds__(256, SEG ? 5 : (POT ? 1 : 6)) traverse2_kernel(const BHNode *__restrict__ nodes,
                                                        const uint32_t *__restrict__ node_total,
                                                        const float4 *__restrict__ pos, int64_t n, float eps2,
                                                        float theta2, float dt, float4 *__restrict__ pos_out,
                                                        float4 *__restrict__ vel, float4 *__restrict__ acc,
                                                        float4 *__restrict__ force_out, const int *__restrict__ ids,
                                                        unsigned long long *__restrict__ counters,
                                                        float *__restrict__ phi_out, int euler,
                                                        const int4 *__restrict__ work, int nwork,
                                                        const float4 *__restrict__ params,
                                                        const uint32_t *__restrict__ P) {
    unsigned long long n_pairs = 0, n_visits = 0;
    float phiA = 0.f, phiB = 0.f;
    const int lane = threadIdx.x & 31;
    const int64_t warp = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    int64_t base, end;
    int i, m_nodes;
    if (SEG) {
        // Only what the walk needs stays live through it; the body range, dt
        // and the integrator are read again afterwards.
        if (warp >= nwork) return;  // whole warps
        const int4 ww = work[warp];
        const float4 prm = params[ww.x];
        eps2 = prm.y;
        theta2 = prm.z;
        base = ww.y;
        end = ww.w;
        i = static_cast<int>(P[ww.z]);
        m_nodes = static_cast<int>(P[ww.w]);
    } else {
        base = warp * 64;
        end = n;
        i = 0;
        m_nodes = static_cast<int>(*node_total);
    }
    bool vA = base + lane < end, vB = base + lane + 32 < end;
    const float4 meA0 = vA ? pos[base + lane] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 meB0 = vB ? pos[base + lane + 32] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float2 nx = make_float2(-meA0.x, -meB0.x), ny = make_float2(-meA0.y, -meB0.y),
                 nz = make_float2(-meA0.z, -meB0.z);
    const float2 th = make_float2(theta2, theta2);
    // Force sums of the lane's two bodies as packed pairs (x: body A, y: body B);
    // an FFMA2 rounds each half exactly as a scalar FFMA.
    float2 fx = make_float2(0.f, 0.f), fy = make_float2(0.f, 0.f), fz = make_float2(0.f, 0.f);
    union_range<COUNT, POT, GUARD>(nodes, pos, n, i, m_nodes, vA, vB, nx, ny, nz, th, eps2, fx, fy, fz, phiA, phiB,
                                   n_pairs, n_visits);
    if (COUNT) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) n_pairs += __shfl_down_sync(0xffffffffu, n_pairs, off);
        if (lane == 0) {
            atomicAdd(&counters[0], n_pairs);
            atomicAdd(&counters[1], n_visits);
        }
    }
    if (SEG) {
        const int4 ww = work[warp];
        const float4 prm = params[ww.x];
        dt = prm.x;
        euler = prm.w != 0.f ? 1 : 0;
        base = ww.y;
        end = ww.w;
    }
    const int64_t bA = base + lane, bB = bA + 32;
    vA = bA < end;
    vB = bB < end;
    if (POT) {
        if (vA) {
            const int d = ids ? ids[bA] : static_cast<int>(bA);
            if (d >= 0 && d < n) phi_out[d] = phiA;
        }
        if (vB) {
            const int d = ids ? ids[bB] : static_cast<int>(bB);
            if (d >= 0 && d < n) phi_out[d] = phiB;
        }
        return;
    }
    // SEG reads the positions again (an L1/L2 hit) to keep registers free
    // during the walk; the single-system walk keeps them.
    if (vA) integrate_sorted(bA, SEG ? pos[bA] : meA0, fx.x, fy.x, fz.x, dt, pos_out, vel, acc, force_out, ids, n, euler);
    if (vB) integrate_sorted(bB, SEG ? pos[bB] : meB0, fx.y, fy.y, fz.y, dt, pos_out, vel, acc, force_out, ids, n, euler);
}

// ------------------------------------------------- deciding for a set
// From the box of a set of bodies, a record is
//   accepted by all  when s^2 < theta^2 * d2lo, d2lo the least squared
//                    distance to the box in the walk's own rounding (each
//                    step is monotone, so every body's d^2 >= d2lo and its
//                    product >= theta^2 * d2lo: the body accepts), or when it
//                    is a lone body (every body accepts a leaf);
//   opened by all    when it is a plain cell and s^2 >= theta^2 * d2hi, d2hi
//                    the largest squared distance in the same rounding;
//   ambiguous        otherwise (and for buckets and terminal cells that are
//                    not accepted by all), to be decided body by body.
struct SetBox {
    float lx, ly, lz, hx, hy, hz;
};

// 0: accepted by every body in the box; 1: opened by every body (a plain
// cell); 2: ambiguous.
__device__ __forceinline__ int certify(const float4 cm, const int4 meta, const SetBox &b, const float theta2) {
    if (meta.w == 1) return 0;  // a lone body: a leaf is always accepted
    if (meta.w >= 2) return 2;  // a bucket: its bodies are summed one by one in the walk
    const float s2 = __int_as_float(meta.x);
    // per axis, the least |dx| over the box (0 inside it) and the largest, both
    // rounded as the walk rounds cm - p
    const float gx = fmaxf(fmaxf(__fsub_rn(b.lx, cm.x), __fsub_rn(cm.x, b.hx)), 0.f);
    const float gy = fmaxf(fmaxf(__fsub_rn(b.ly, cm.y), __fsub_rn(cm.y, b.hy)), 0.f);
    const float gz = fmaxf(fmaxf(__fsub_rn(b.lz, cm.z), __fsub_rn(cm.z, b.hz)), 0.f);
    const float lo2 = __fadd_rn(__fadd_rn(__fmul_rn(gx, gx), __fmul_rn(gy, gy)), __fmul_rn(gz, gz));
    if (s2 < __fmul_rn(theta2, lo2)) return 0;
    if (meta.w != 0) return 2;
    const float ux = fmaxf(fabsf(__fsub_rn(cm.x, b.lx)), fabsf(__fsub_rn(b.hx, cm.x)));
    const float uy = fmaxf(fabsf(__fsub_rn(cm.y, b.ly)), fabsf(__fsub_rn(b.hy, cm.y)));
    const float uz = fmaxf(fabsf(__fsub_rn(cm.z, b.lz)), fabsf(__fsub_rn(b.hz, cm.z)));
    const float hi2 = __fadd_rn(__fadd_rn(__fmul_rn(ux, ux), __fmul_rn(uy, uy)), __fmul_rn(uz, uz));
    return s2 < __fmul_rn(theta2, hi2) ? 2 : 1;
}

// ------------------------------------------------------------ cell walk
// Same per-body acceptance as traverse2_kernel, organised by cells. A warp
// holds a stack of cells that some of its bodies opened, each with the masks
// of those bodies (first and second body of each lane) and their box. For a
// cell popped (up to four at a time), eight lanes load its children and
// decide each one for the whole set from the box (certify: accepted by all of them, opened by all of
// them, or ambiguous) while leaving its cm in shared memory. Accepted
// children are summed by those bodies with no criterion, in batches read from
// shared memory (3.51 against 4.05 ms at 2^20 when each was fetched on its own
// by record index); children opened by all are pushed with the same set and box;
// each ambiguous child gets the per-body criterion, its accepting bodies sum
// it (or a bucket's bodies), the bodies that open a terminal cell sum its
// bodies, and the bodies that open a plain cell are pushed with it as a new,
// smaller set with its own box. A body thus meets exactly the records of its
// own reference walk, and decides by itself only those its set disagrees on.
constexpr int kCellWarps = 2;   // 64-thread CTAs: finer blocks shorten the grid's uneven last wave
constexpr int kCellDepth = 48;  // stack entries per warp; a full stack sends a cell to union_range

// Box of the bodies in masks sa / sb (exact min / max on the order-preserving
// integer image).
__device__ __forceinline__ SetBox box_of(unsigned sa, unsigned sb, int lane, float4 pa, float4 pb) {
    const bool ia = (sa >> lane) & 1u, ib = (sb >> lane) & 1u;
    const float xa[3] = {pa.x, pa.y, pa.z}, xb[3] = {pb.x, pb.y, pb.z};
    unsigned lo[3], hi[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const unsigned oa = ord_of(xa[a]), ob = ord_of(xb[a]);
        lo[a] = __reduce_min_sync(0xffffffffu, min(ia ? oa : 0xffffffffu, ib ? ob : 0xffffffffu));
        hi[a] = __reduce_max_sync(0xffffffffu, max(ia ? oa : 0u, ib ? ob : 0u));
    }
    SetBox b;
    b.lx = float_of(lo[0]);
    b.ly = float_of(lo[1]);
    b.lz = float_of(lo[2]);
    b.hx = float_of(hi[0]);
    b.hy = float_of(hi[1]);
    b.hz = float_of(hi[2]);
    return b;
}

// The record's force on each of the lane's bodies whose flag is set (the
// walk's arithmetic; GUARD keeps the explicit zero-distance and massless
// tests).
template <bool COUNT, bool POT, bool GUARD>
__device__ __forceinline__ void add_record(const float4 cm, bool useA, bool useB, const float2 nx, const float2 ny,
                                           const float2 nz, const float2 e2, float2 &fx, float2 &fy, float2 &fz,
                                           float &phiA, float &phiB, unsigned long long &n_pairs) {
    const float2 dx = __fadd2_rn(make_float2(cm.x, cm.x), nx);
    const float2 dy = __fadd2_rn(make_float2(cm.y, cm.y), ny);
    const float2 dz = __fadd2_rn(make_float2(cm.z, cm.z), nz);
    const float2 d2 = __fadd2_rn(__fadd2_rn(__fmul2_rn(dx, dx), __fmul2_rn(dy, dy)), __fmul2_rn(dz, dz));
    if (GUARD) {
        useA = useA && cm.w > 0.f && d2.x > 0.f;
        useB = useB && cm.w > 0.f && d2.y > 0.f;
    }
    const float2 ee = __fadd2_rn(d2, e2);
    const float2 inv = make_float2(rsqrt_ftz(ee.x), rsqrt_ftz(ee.y));
    const float2 inv3 = __fmul2_rn(__fmul2_rn(inv, inv), inv);
    const float2 mw = __fmul2_rn(make_float2(cm.w, cm.w), inv3);
    const float2 w = make_float2(useA ? mw.x : 0.f, useB ? mw.y : 0.f);
    fx = __ffma2_rn(dx, w, fx);
    fy = __ffma2_rn(dy, w, fy);
    fz = __ffma2_rn(dz, w, fz);
    if (COUNT) n_pairs += (useA ? 1u : 0u) + (useB ? 1u : 0u);
    if (POT) {
        phiA = fmaf(useA ? -cm.w : 0.f, inv.x, phiA);
        phiB = fmaf(useB ? -cm.w : 0.f, inv.y, phiB);
    }
}

// 64-thread CTAs. One system: twenty-four per SM (40 registers, 48 warps):
// 4.05 ms at 2^20 against 4.18 at twenty (48 registers) and 4.21 at
// twenty-eight or thirty-two, 14.4 vs 15.4 ms at 4M (GB300, before the
// children's cm moved to shared memory; with them there twenty still loses,
// 4.0 vs 3.67 ms). An ensemble's
// form also holds each system's eps^2 and theta^2 in registers and runs best
// at sixteen (64 registers, no spills; 33.7 vs 30.8 ms at twenty for a
// 512-system ensemble). Against 256-thread CTAs at the same occupancy the
// finer blocks shorten the uneven last wave (4.19 vs 4.28 ms at 2^20).
template <bool COUNT, bool POT, bool SEG, bool GUARD, bool HOST = false>
__global__ void __launch_bounds__(64, (COUNT || SEG) ? 16 : 24) cell_walk_kernel(
    const BHNode *__restrict__ nodes, const int *__restrict__ kids, const uint32_t *__restrict__ node_total,
    const float4 *__restrict__ pos, int64_t n, float eps2, float theta2, float dt, float4 *__restrict__ pos_out,
    float4 *__restrict__ vel, float4 *__restrict__ acc, float4 *__restrict__ force_out, const int *__restrict__ ids,
    unsigned long long *__restrict__ counters, float *__restrict__ phi_out, int euler, const int4 *__restrict__ work,
    int nwork, const float4 *__restrict__ params, const uint32_t *__restrict__ P, const HostOut host) {
    // One block of shared memory per warp, addressed from one base.
    struct __align__(16) WarpArea {
        int4 stk_i[kCellDepth];     // cell, mask A, mask B, box hz (float bits)
        float4 stk_lo[kCellDepth];  // box: lx, ly, lz, hx
        float stk_hy[kCellDepth];   // box: hy
        int4 bat_i[4];              // the cells of a round, as popped
        float4 bat_lo[4];
        float bat_hy[4];
        float4 ch_cm[32];           // the round's children's cm, by the lane that loaded them
    };
    __shared__ WarpArea area[kCellWarps];
    WarpArea &A = area[threadIdx.x >> 5];
    unsigned long long n_pairs = 0, n_visits = 0;
    float phiA = 0.f, phiB = 0.f;
    const int lane = threadIdx.x & 31;
    int4 *si = A.stk_i;
    float4 *slo = A.stk_lo;
    float *shy = A.stk_hy;
    int4 *bi = A.bat_i;
    float4 *blo = A.bat_lo;
    float *bhy = A.bat_hy;
    float4 *ccm = A.ch_cm;
    const int64_t warp = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    int64_t base, end;
    int root, rend;
    if (SEG) {
        if (warp >= nwork) return;  // whole warps
        const int4 ww = work[warp];
        const float4 prm = params[ww.x];
        eps2 = prm.y;
        theta2 = prm.z;
        base = ww.y;
        end = ww.w;
        root = static_cast<int>(P[ww.z]);
        rend = static_cast<int>(P[ww.w]);
    } else {
        base = warp * 64;
        end = n;
        root = 0;
        rend = static_cast<int>(*node_total);
    }
    bool vA = base + lane < end, vB = base + lane + 32 < end;
    const float4 meA0 = vA ? pos[base + lane] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 meB0 = vB ? pos[base + lane + 32] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float2 nx = make_float2(-meA0.x, -meB0.x), ny = make_float2(-meA0.y, -meB0.y),
                 nz = make_float2(-meA0.z, -meB0.z);
    const float2 th = make_float2(theta2, theta2);
    const float2 e2 = make_float2(eps2, eps2);
    float2 fx = make_float2(0.f, 0.f), fy = make_float2(0.f, 0.f), fz = make_float2(0.f, 0.f);
    int sp = 0;

    // Record k decided body by body for the bodies in (sa, sb); the bodies
    // that open a plain cell are pushed with it (or, on a full stack, walk
    // its subtree with union_range).
    auto decide = [&](int k, const float4 cm, const int4 meta, unsigned sa, unsigned sb) {
        const bool actA = (sa >> lane) & 1u, actB = (sb >> lane) & 1u;
        const float2 dx = __fadd2_rn(make_float2(cm.x, cm.x), nx);
        const float2 dy = __fadd2_rn(make_float2(cm.y, cm.y), ny);
        const float2 dz = __fadd2_rn(make_float2(cm.z, cm.z), nz);
        const float2 d2 = __fadd2_rn(__fadd2_rn(__fmul2_rn(dx, dx), __fmul2_rn(dy, dy)), __fmul2_rn(dz, dz));
        const float s2 = __int_as_float(meta.x);
        const float2 rhs = __fmul2_rn(th, d2);
        bool accA, accB, useA, useB;
        if (GUARD) {
            accA = actA && (s2 < 0.f || s2 < rhs.x);
            accB = actB && (s2 < 0.f || s2 < rhs.y);
            const bool self = meta.w <= 1 && cm.w > 0.f;
            useA = accA && self && d2.x > 0.f;
            useB = accB && self && d2.y > 0.f;
        } else {
            accA = actA && s2 < rhs.x;
            accB = actB && s2 < rhs.y;
            const bool self = meta.w <= 1;
            useA = accA && self;
            useB = accB && self;
        }
        if (COUNT) ++n_visits;
        {
            const float2 ee = __fadd2_rn(d2, e2);
            const float2 inv = make_float2(rsqrt_ftz(ee.x), rsqrt_ftz(ee.y));
            const float2 inv3 = __fmul2_rn(__fmul2_rn(inv, inv), inv);
            const float2 mw = __fmul2_rn(make_float2(cm.w, cm.w), inv3);
            const float2 w = make_float2(useA ? mw.x : 0.f, useB ? mw.y : 0.f);
            fx = __ffma2_rn(dx, w, fx);
            fy = __ffma2_rn(dy, w, fy);
            fz = __ffma2_rn(dz, w, fz);
            if (COUNT) n_pairs += (useA ? 1u : 0u) + (useB ? 1u : 0u);
            if (POT) {
                phiA = fmaf(useA ? -cm.w : 0.f, inv.x, phiA);
                phiB = fmaf(useB ? -cm.w : 0.f, inv.y, phiB);
            }
        }
        if (meta.w != 0 && meta.w != 1) {  // a bucket accepted, or a terminal cell opened: body by body
            const int cntb = meta.w >= 2 ? meta.w : -meta.w;
            const bool doA = (meta.w >= 2 && accA) || (meta.w < 0 && actA && !accA);
            const bool doB = (meta.w >= 2 && accB) || (meta.w < 0 && actB && !accB);
            if (COUNT || POT) {
                const float4 meA = make_float4(-nx.x, -ny.x, -nz.x, 0.f), meB = make_float4(-nx.y, -ny.y, -nz.y, 0.f);
                if (doA) direct_sum_range(pos, n, meta.z, cntb, meA, eps2, fx.x, fy.x, fz.x, n_pairs, COUNT, phiA, POT);
                if (doB) direct_sum_range(pos, n, meta.z, cntb, meB, eps2, fx.y, fy.y, fz.y, n_pairs, COUNT, phiB, POT);
            } else if (doA || doB) {
                direct_sum_range2(pos, n, meta.z, cntb, nx, ny, nz, eps2, doA, doB, fx, fy, fz);
            }
            return;
        }
        if (meta.w != 0) return;
        const unsigned oa = __ballot_sync(0xffffffffu, actA && !accA);
        const unsigned ob = __ballot_sync(0xffffffffu, actB && !accB);
        if (!(oa | ob)) return;
        if (sp < kCellDepth) {
            const SetBox b = box_of(oa, ob, lane, meA0, meB0);
            if (lane == 0) {
                si[sp] = make_int4(k, static_cast<int>(oa), static_cast<int>(ob), __float_as_int(b.hz));
                slo[sp] = make_float4(b.lx, b.ly, b.lz, b.hx);
                shy[sp] = b.hy;
            }
            ++sp;
        } else {
            union_range<COUNT, POT, GUARD>(nodes, pos, n, k + 1, meta.y, (oa >> lane) & 1u, (ob >> lane) & 1u, nx,
                                           ny, nz, th, eps2, fx, fy, fz, phiA, phiB, n_pairs, n_visits);
        }
    };

    if (root < rend)
        decide(root, __ldg(&nodes[root].cm), __ldg(&nodes[root].meta), __ballot_sync(0xffffffffu, vA),
               __ballot_sync(0xffffffffu, vB));
    // Up to four cells per round: lanes 8g .. 8g + 7 take the children of cell
    // g and decide them for its set; the popped entries move to a batch area
    // that the round's pushes cannot reach.
    const int grp = lane >> 3;
    // Accepted children summed per batch: eight for one system (3.51 vs 3.58
    // ms at four, 2^20 Plummer), four for ensembles (28.9 vs 29.5 ms, 512
    // systems), whose form holds more registers.
    constexpr int kBatch = SEG ? 4 : 8;
    while (sp > 0) {
        const int nb = sp < 4 ? sp : 4;
        sp -= nb;
        __syncwarp();  // lane 0's writes of the entries before the lanes read them
        int kid = -1, cls = 3;
        if (grp < nb) {
            const int4 t = si[sp + grp];
            const float4 bl = slo[sp + grp];
            const float hy = shy[sp + grp];
            if ((lane & 7) == 0) {
                bi[grp] = t;
                blo[grp] = bl;
                bhy[grp] = hy;
            }
            SetBox box;
            box.lx = bl.x;
            box.ly = bl.y;
            box.lz = bl.z;
            box.hx = bl.w;
            box.hy = hy;
            box.hz = __int_as_float(t.w);
            kid = __ldg(&kids[8 * static_cast<int64_t>(t.x) + (lane & 7)]);
            if (kid >= 0) {
                const float4 cm = __ldg(&nodes[kid].cm);
                ccm[lane] = cm;
                cls = certify(cm, __ldg(&nodes[kid].meta), box, theta2);
            }
        }
        __syncwarp();  // the batch written, and the popped slots read, before pushes reuse them
        const unsigned bAcc = __ballot_sync(0xffffffffu, cls == 0);
        const unsigned bOpen = __ballot_sync(0xffffffffu, cls == 1);
        const unsigned bAmb = __ballot_sync(0xffffffffu, cls == 2);
        if (COUNT) n_visits += __popc(bAcc | bOpen | bAmb);
        for (int q = 0; q < nb; ++q) {
            const unsigned gm = 0xffu << (8 * q);
            const int4 t = bi[q];
            const unsigned sa = static_cast<unsigned>(t.y), sb = static_cast<unsigned>(t.z);
            const bool actA = (sa >> lane) & 1u, actB = (sb >> lane) & 1u;
            for (unsigned m = bOpen & gm; m; m &= m - 1) {
                const int k = __shfl_sync(0xffffffffu, kid, __ffs(m) - 1);
                if (sp < kCellDepth) {
                    if (lane == 0) {
                        si[sp] = make_int4(k, static_cast<int>(sa), static_cast<int>(sb), t.w);
                        slo[sp] = blo[q];
                        shy[sp] = bhy[q];
                    }
                    ++sp;
                } else {
                    const int kend = __ldg(&nodes[k].meta).y;
                    union_range<COUNT, POT, GUARD>(nodes, pos, n, k + 1, kend, actA, actB, nx, ny, nz, th, eps2, fx,
                                                   fy, fz, phiA, phiB, n_pairs, n_visits);
                }
            }
            // Accepted children in batches: their cm come from shared memory
            // (bit c of the mask is lane c's child), all loads of a batch
            // before its sums.
            unsigned m = bAcc & gm;
            while (__popc(m) >= kBatch) {
                float4 c[kBatch];
#pragma unroll
                for (int j = 0; j < kBatch; ++j) {
                    c[j] = ccm[__ffs(m) - 1];
                    m &= m - 1;
                }
#pragma unroll
                for (int j = 0; j < kBatch; ++j)
                    add_record<COUNT, POT, GUARD>(c[j], actA, actB, nx, ny, nz, e2, fx, fy, fz, phiA, phiB, n_pairs);
            }
            for (; m; m &= m - 1)
                add_record<COUNT, POT, GUARD>(ccm[__ffs(m) - 1], actA, actB, nx, ny, nz, e2, fx, fy, fz, phiA, phiB,
                                              n_pairs);
            for (m = bAmb & gm; m; m &= m - 1) {
                const int c = __ffs(m) - 1;
                const int k = __shfl_sync(0xffffffffu, kid, c);
                decide(k, ccm[c], __ldg(&nodes[k].meta), sa, sb);
            }
        }
    }

    if (COUNT) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) n_pairs += __shfl_down_sync(0xffffffffu, n_pairs, off);
        if (lane == 0) {
            atomicAdd(&counters[0], n_pairs);
            atomicAdd(&counters[1], n_visits);
        }
    }
    if (SEG) {
        const int4 ww = work[warp];
        const float4 prm = params[ww.x];
        dt = prm.x;
        euler = prm.w != 0.f ? 1 : 0;
        base = ww.y;
        end = ww.w;
    }
    const int64_t bA = base + lane, bB = bA + 32;
    vA = bA < end;
    vB = bB < end;
    if (POT) {
        if (vA) {
            const int d = ids ? ids[bA] : static_cast<int>(bA);
            if (d >= 0 && d < n) phi_out[d] = phiA;
        }
        if (vB) {
            const int d = ids ? ids[bB] : static_cast<int>(bB);
            if (d >= 0 && d < n) phi_out[d] = phiB;
        }
        return;
    }
    // HOST: a separate instance (even an unused store to the caller's arrays
    // here added spills to the walk above).
    if (vA)
        integrate_sorted(bA, SEG ? pos[bA] : meA0, fx.x, fy.x, fz.x, dt, pos_out, vel, acc, force_out, ids, n, euler,
                         HOST ? host : HostOut{});
    if (vB)
        integrate_sorted(bB, SEG ? pos[bB] : meB0, fx.y, fy.y, fz.y, dt, pos_out, vel, acc, force_out, ids, n, euler,
                         HOST ? host : HostOut{});
}

// out[ids[i]] = in[i] (back to the caller's body order), positions with w = 0.
__global__ void unpermute_kernel(const int *__restrict__ ids, int64_t n, const float4 *__restrict__ in,
                                 float4 *__restrict__ out, int zero_w, int *status) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 v = in[i];
    if (zero_w) v.w = 0.f;
    const int d = ids[i];
    if (d < 0 || d >= n) {
        record_error(status, NBODY_ERR_CAPACITY);
        return;
    }
    out[d] = v;
}

// exclusive scan of cnt[0..n) into P[0..n], P[n] = total (three phases).
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

__global__ void __launch_bounds__(kScanThreads) scan_tiles_kernel(const uint32_t *__restrict__ in, int64_t n,
                                                                  uint32_t *__restrict__ out,
                                                                  uint32_t *__restrict__ tile_sums) {
    __shared__ uint32_t warp_sums[32];
    const int64_t base = static_cast<int64_t>(blockIdx.x) * kScanTile + threadIdx.x * kScanItems;
    uint32_t v[kScanItems];
    uint32_t run = 0;
#pragma unroll
    for (int j = 0; j < kScanItems; ++j) {
        v[j] = base + j < n ? in[base + j] : 0u;
        const uint32_t t2 = v[j];
        v[j] = run;
        run += t2;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = run;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, off);
        if (lane >= off) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = warp_sums[lane];
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, w, off);
            if (lane >= off) w += y;
        }
        warp_sums[lane] = w;
    }
    __syncthreads();
    const uint32_t offset = (x - run) + (warp > 0 ? warp_sums[warp - 1] : 0u);
#pragma unroll
    for (int j = 0; j < kScanItems; ++j)
        if (base + j < n) out[base + j] = v[j] + offset;
    if (threadIdx.x == kScanThreads - 1) tile_sums[blockIdx.x] = offset + run;
}

__global__ void __launch_bounds__(1024) scan_sums_kernel(uint32_t *__restrict__ tile_sums, int tiles,
                                                         uint32_t *__restrict__ total_out) {
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < tiles; base += 1024) {
        const int i = base + threadIdx.x;
        const uint32_t v = i < tiles ? tile_sums[i] : 0u;
        uint32_t x = v;
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, off);
            if (lane >= off) x += y;
        }
        __shared__ uint32_t ws[32];
        if (lane == 31) ws[warp] = x;
        __syncthreads();
        if (warp == 0) {
            uint32_t w = ws[lane];
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, w, off);
                if (lane >= off) w += y;
            }
            ws[lane] = w;
        }
        __syncthreads();
        const uint32_t incl = x + (warp > 0 ? ws[warp - 1] : 0u);
        if (i < tiles) tile_sums[i] = carry + incl - v;
        __syncthreads();
        if (threadIdx.x == 1023) carry += incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) *total_out = carry;
}

__global__ void scan_add_kernel(uint32_t *__restrict__ out, int64_t n, const uint32_t *__restrict__ tile_sums) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] += tile_sums[i / kScanTile];
}

unsigned grid_for(int64_t n, int threads) { return static_cast<unsigned>((n + threads - 1) / threads); }

// Depth of the reference's fully expanded top levels for n bodies
// (ParallelOctreeCPU::ParallelOctreeCPU, src/Octree/ParallelOctreeCPU.cpp:7-23):
// the deepest d <= 3 with 1 + 8 + ... + 8^d < n.
int father_depth(int64_t n) {
    int64_t nodes = 0, p8 = 1;
    int d = -1;
    while (nodes < n && d < 3) {
        if (nodes + p8 >= n) break;
        nodes += p8;
        ++d;
        p8 *= 8;
    }
    return d;
}

}  // namespace

int bh_father_depth(int64_t n) { return father_depth(n); }

// ------------------------------------------------------------------- host
size_t bh_workspace_bytes(int64_t n) {
    BHWorkspace w;
    return bh_workspace_layout(n, nullptr, &w);
}

size_t bh_workspace_layout(int64_t n, void *base, BHWorkspace *w) {
    size_t off = 0;
    auto take = [&](size_t bytes) -> void * {
        off = (off + 255) & ~static_cast<size_t>(255);
        void *p = base ? static_cast<char *>(base) + off : nullptr;
        off += bytes;
        return p;
    };
    const size_t nn = static_cast<size_t>(n > 1 ? n : 2);
    const int64_t tiles = (n + kScanTile - 1) / kScanTile;
    w->n = n;
    w->keys[0] = static_cast<uint64_t *>(take(sizeof(uint64_t) * nn));
    w->keys[1] = static_cast<uint64_t *>(take(sizeof(uint64_t) * nn));
    w->vals[0] = static_cast<uint32_t *>(take(sizeof(uint32_t) * nn));
    w->vals[1] = static_cast<uint32_t *>(take(sizeof(uint32_t) * nn));
    w->sort_scratch = take(sort_scratch_bytes(n));
    w->box = static_cast<float *>(take(sizeof(float) * 8));
    w->bbox_partial = static_cast<float *>(take(sizeof(float) * 6 * kBBoxBlocks));
    w->bbox_counter = static_cast<unsigned *>(take(sizeof(unsigned) * 4));
    w->tree.lo = static_cast<int *>(take(sizeof(int) * nn));
    w->tree.hi = static_cast<int *>(take(sizeof(int) * nn));
    w->tree.left = static_cast<int *>(take(sizeof(int) * nn));
    w->tree.right = static_cast<int *>(take(sizeof(int) * nn));
    w->tree.delta = static_cast<int *>(take(sizeof(int) * nn));
    w->tree.iparent = static_cast<int *>(take(sizeof(int) * nn));
    w->tree.lparent = static_cast<int *>(take(sizeof(int) * nn));
    w->tree.top = static_cast<int *>(take(sizeof(int) * nn));
    w->rec.level = static_cast<int *>(take(sizeof(int) * 2 * nn));
    w->rec.parent = static_cast<int *>(take(sizeof(int) * 2 * nn));
    w->rec.nchild = static_cast<int *>(take(sizeof(int) * 2 * nn));
    w->rec.arrive = static_cast<unsigned *>(take(sizeof(unsigned) * 2 * nn));
    w->rec.list = w->rec.arrive;  // one schedule or the other per build
    w->rec.lvl = static_cast<unsigned *>(take(sizeof(unsigned) * 96));
    w->mask = static_cast<uint32_t *>(take(sizeof(uint32_t) * nn));
    w->cnt = static_cast<uint32_t *>(take(sizeof(uint32_t) * nn));
    w->P = static_cast<uint32_t *>(take(sizeof(uint32_t) * (nn + 1)));
    w->scan_sums = static_cast<uint32_t *>(take(sizeof(uint32_t) * static_cast<size_t>(tiles + 1)));
    w->nodes = static_cast<BHNode *>(take(sizeof(BHNode) * 2 * nn));
    w->kids = static_cast<int *>(take(sizeof(int) * 8 * 2 * nn));
    w->counter_mem = static_cast<unsigned long long *>(take(sizeof(unsigned long long) * 2));
    w->counters = nullptr;
    w->node_count_host = 0;
    return (off + 255) & ~static_cast<size_t>(255);
}

cudaError_t bh_bbox(const float4 *pos, int64_t n, BHWorkspace &w, cudaStream_t st, StageTimer *timer) {
    if (timer) timer->begin(kStageBBox, st);
    int blocks = static_cast<int>((n + 255) / 256);
    if (blocks > kBBoxBlocks) blocks = kBBoxBlocks;
    if (blocks < 1) blocks = 1;
    bbox_kernel<<<blocks, 256, 0, st>>>(pos, n, w.bbox_partial, w.bbox_counter, w.box);
    if (timer) timer->end(kStageBBox, st);
    return cudaGetLastError();
}

cudaError_t bh_keys(const float4 *pos, int64_t n, BHWorkspace &w, int mode, cudaStream_t st, StageTimer *timer) {
    if (timer) timer->begin(kStageMorton, st);
    if (mode == NBODY_KEYS_MORTON)
        morton_kernel<NBODY_KEYS_MORTON><<<grid_for(n, 256), 256, 0, st>>>(pos, n, w.box, w.keys[0], w.vals[0]);
    else
        morton_kernel<NBODY_KEYS_OCTREE><<<grid_for(n, 256), 256, 0, st>>>(pos, n, w.box, w.keys[0], w.vals[0]);
    if (timer) timer->end(kStageMorton, st);
    return cudaGetLastError();
}

cudaError_t bh_sort(int64_t n, BHWorkspace &w, cudaStream_t st, int *status, StageTimer *timer) {
    if (timer) timer->begin(kStageSort, st);
    int alt = 0;
    cudaError_t e = sort_pairs(w.keys[0], w.vals[0], w.keys[1], w.vals[1], n, w.sort_scratch, st, status, &alt);
    if (timer) timer->end(kStageSort, st);
    if (e != cudaSuccess) return e;
    if (alt) {  // keep the sorted pairs in slot 0
        uint64_t *tk = w.keys[0]; w.keys[0] = w.keys[1]; w.keys[1] = tk;
        uint32_t *tv = w.vals[0]; w.vals[0] = w.vals[1]; w.vals[1] = tv;
    }
    return cudaSuccess;
}

cudaError_t bh_gather(int64_t n, const BHWorkspace &w, const float4 *pos_in, const float4 *vel_in,
                      const float4 *acc_in, const int *id_in, float4 *pos_out, float4 *vel_out, float4 *acc_out,
                      int *id_out, cudaStream_t st, int *status, StageTimer *timer) {
    if (timer) timer->begin(kStageGather, st);
    gather_kernel<<<grid_for(n, 256), 256, 0, st>>>(w.vals[0], n, pos_in, vel_in, acc_in, id_in, pos_out, vel_out,
                                                    acc_out, id_out, status, nullptr, nullptr);
    if (timer) timer->end(kStageGather, st);
    return cudaGetLastError();
}

bool bh_upsweep_by_levels(int64_t n, bool ensemble) {
    // Same bits either way: the climb below 2^21 bodies of one system, where
    // one launch beats one per level; NBODY_UPSWEEP = "climb" or "levels"
    // forces one.
    bool levels = ensemble || n >= (int64_t(1) << 21);
    if (const char *env = std::getenv("NBODY_UPSWEEP")) {
        if (std::strcmp(env, "climb") == 0) levels = false;
        if (std::strcmp(env, "levels") == 0) levels = true;
    }
    return levels;
}

int bh_upsweep_launches(int64_t n, bool ensemble) { return bh_upsweep_by_levels(n, ensemble) ? 3 + kMaxLevel : 1; }

cudaError_t bh_build(const float4 *pos_sorted, int64_t n, BHWorkspace &w, cudaStream_t st, int *status,
                     StageTimer *timer, const SegView &sv) {
    if (timer) timer->begin(kStageBuild, st);
    const uint64_t *k = w.keys[0];
    cudaError_t e = cudaMemsetAsync(w.mask, 0, sizeof(uint32_t) * static_cast<size_t>(n), st);
    if (e != cudaSuccess) return e;
    if (n >= 2) {
        radix_tree_kernel<<<grid_for(n - 1, 256), 256, 0, st>>>(k, n, w.tree, sv, w.mask, sv.seg ? 32 : 0);
    }
    count_nodes_kernel<<<grid_for(n, 256), 256, 0, st>>>(k, n, w.mask, w.cnt, sv);
    const int tiles = static_cast<int>((n + kScanTile - 1) / kScanTile);
    scan_tiles_kernel<<<tiles, kScanThreads, 0, st>>>(w.cnt, n, w.P, w.scan_sums);
    scan_sums_kernel<<<1, 1024, 0, st>>>(w.scan_sums, tiles, w.P + n);
    scan_add_kernel<<<grid_for(n, 256), 256, 0, st>>>(w.P, n, w.scan_sums);
    const bool levels = bh_upsweep_by_levels(n, sv.seg != nullptr);
    // Records: at most 2n (n - 1 cells and n leaves).
    const int64_t cap = 2 * (n > 1 ? n : 2);
    if (!levels) {
        e = cudaMemsetAsync(w.rec.nchild, 0, sizeof(int) * static_cast<size_t>(cap), st);
        if (e == cudaSuccess) e = cudaMemsetAsync(w.rec.arrive, 0, sizeof(unsigned) * static_cast<size_t>(cap), st);
        if (e != cudaSuccess) return e;
    }
    if (n >= 2)
        emit_cells_kernel<<<grid_for(n - 1, 256), 256, 0, st>>>(k, n, w.tree, w.mask, w.P, w.box, w.nodes, w.rec,
                                                                sv, !levels);
    emit_leaves_kernel<<<grid_for(n, 256), 256, 0, st>>>(k, n, pos_sorted, w.tree, w.mask, w.P, w.nodes, w.rec, sv,
                                                         !levels);
    if (w.walk == kWalkCell) {
        const int64_t cap = 2 * (n > 1 ? n : 2);
        kids_kernel<<<grid_for(cap, 256), 256, 0, st>>>(w.nodes, w.P + n, cap, w.kids, status);
    }
    if (timer) timer->end(kStageBuild, st);
    if (timer) timer->begin(kStageUpsweep, st);
    if (!levels) {
        upsweep_climb_kernel<<<grid_for(n, 256), 256, 0, st>>>(k, n, pos_sorted, w.mask, w.P, w.nodes, w.rec,
                                                               father_depth(n), status, sv);
        if (timer) timer->end(kStageUpsweep, st);
        return cudaGetLastError();
    }
    e = cudaMemsetAsync(w.rec.lvl, 0, sizeof(unsigned) * 96, st);
    if (e != cudaSuccess) return e;
    bucket_cm_kernel<<<grid_for(n, 256), 256, 0, st>>>(k, n, pos_sorted, w.mask, w.P, w.nodes, sv);
    const unsigned spread = static_cast<unsigned>(std::min<int64_t>(grid_for(n, 256), 1216));
    level_count_kernel<<<spread, 256, 0, st>>>(w.rec.level, w.P + n, w.rec.lvl);
    level_scatter_kernel<<<grid_for(cap, 256), 256, 0, st>>>(w.rec.level, w.P + n, w.rec.lvl, w.rec.list, cap,
                                                             status);
    const int fd = father_depth(n);
    for (int L = kMaxLevel - 1; L >= 0; --L)
        level_cm_kernel<<<spread, 256, 0, st>>>(L, k, n, w.nodes, w.rec.level, w.rec.list, w.rec.lvl, fd, status, sv);
    if (timer) timer->end(kStageUpsweep, st);
    return cudaGetLastError();
}

// One launch of the walk in the workspace's form (the same accepted records
// per body in both forms).
template <bool COUNT, bool POT, bool SEG, bool GUARD>
void launch_walk(const BHWorkspace &w, unsigned blocks, cudaStream_t st, const uint32_t *node_total,
                 const float4 *pos, int64_t n, float eps2, float theta2, float dt, float4 *pos_out, float4 *vel,
                 float4 *acc, float4 *force_out, const int *ids, unsigned long long *counters, float *phi_out,
                 int euler, const int4 *work, int nwork, const float4 *params, const uint32_t *P,
                 const HostOut &host = HostOut{}) {
    if constexpr (!SEG && !POT) {
        if (w.walk == kWalkCell && host.pos) {
            cell_walk_kernel<COUNT, POT, SEG, GUARD, true><<<blocks * 4, 64, 0, st>>>(
                w.nodes, w.kids, node_total, pos, n, eps2, theta2, dt, pos_out, vel, acc, force_out, ids, counters,
                phi_out, euler, work, nwork, params, P, host);
            return;
        }
    }
    if (w.walk == kWalkCell)
        cell_walk_kernel<COUNT, POT, SEG, GUARD><<<blocks * 4, 64, 0, st>>>(w.nodes, w.kids, node_total, pos, n, eps2,
                                                                         theta2, dt, pos_out, vel, acc, force_out,
                                                                         ids, counters, phi_out, euler, work, nwork,
                                                                         params, P, host);
    else
        traverse2_kernel<COUNT, POT, SEG, GUARD><<<blocks, 256, 0, st>>>(w.nodes, node_total, pos, n, eps2, theta2,
                                                                         dt, pos_out, vel, acc, force_out, ids,
                                                                         counters, phi_out, euler, work, nwork,
                                                                         params, P);
}

bool bh_walk_writes_host(const BHWorkspace &w) { return w.walk == kWalkCell && w.bodies_per_lane == 2; }

int bh_walk_form() {
    const char *e = std::getenv("NBODY_BH_WALK");
    return (e && std::strcmp(e, "union") == 0) ? kWalkUnion : kWalkCell;
}

cudaError_t bh_traverse(const float4 *pos_sorted, int64_t n, const BHWorkspace &w, float eps2, float theta2,
                        float dt, float4 *pos_out, float4 *vel, float4 *acc, float4 *force_out, const int *ids,
                        int euler, cudaStream_t st, StageTimer *timer, const HostOut &host) {
    if (host.pos && !bh_walk_writes_host(w)) return cudaErrorInvalidValue;
    if (timer) timer->begin(kStageTraverse, st);
    // The record count P[n] stays on the device; the kernel reads it.
    if (w.bodies_per_lane == 2) {
        const int64_t warps = (n + 63) / 64;
        const unsigned blocks = static_cast<unsigned>((warps * 32 + 255) / 256);
        if (w.counters)
            launch_walk<true, false, false, true>(w, blocks, st, w.P + n, pos_sorted, n, eps2, theta2, dt, pos_out, vel,
                                                 acc, force_out, ids, w.counters, nullptr, euler, nullptr, 0, nullptr,
                                                 nullptr, host);
        else if (eps2 > 0.f && theta2 > 0.f)
            launch_walk<false, false, false, false>(w, blocks, st, w.P + n, pos_sorted, n, eps2, theta2, dt, pos_out,
                                                   vel, acc, force_out, ids, nullptr, nullptr, euler, nullptr, 0,
                                                   nullptr, nullptr, host);
        else
            launch_walk<false, false, false, true>(w, blocks, st, w.P + n, pos_sorted, n, eps2, theta2, dt, pos_out,
                                                  vel, acc, force_out, ids, nullptr, nullptr, euler, nullptr, 0,
                                                  nullptr, nullptr, host);
    } else if (w.counters)
        traverse_kernel<true><<<grid_for(n, 256), 256, 0, st>>>(w.nodes, w.P + n, pos_sorted, n, eps2, theta2, dt,
                                                                pos_out, vel, acc, force_out, ids, w.counters, euler);
    else
        traverse_kernel<false><<<grid_for(n, 256), 256, 0, st>>>(w.nodes, w.P + n, pos_sorted, n, eps2, theta2, dt,
                                                                 pos_out, vel, acc, force_out, ids, nullptr, euler);
    if (timer) timer->end(kStageTraverse, st);
    return cudaGetLastError();
}

cudaError_t bh_potential(const float4 *pos_sorted, int64_t n, const BHWorkspace &w, float eps2, float theta2,
                         float *phi_out, const int *ids, cudaStream_t st) {
    const int64_t warps = (n + 63) / 64;
    const unsigned blocks = static_cast<unsigned>((warps * 32 + 255) / 256);
    launch_walk<false, true, false, true>(w, blocks, st, w.P + n, pos_sorted, n, eps2, theta2, 0.f, nullptr, nullptr,
                                          nullptr, nullptr, ids, nullptr, phi_out, 0, nullptr, 0, nullptr, nullptr);
    return cudaGetLastError();
}

cudaError_t bh_seed_boxes(const BHEnsembleTables &e, cudaStream_t st) {
    if (e.systems <= 0) return cudaSuccess;
    seed_box_acc_kernel<<<grid_for(e.systems, 256), 256, 0, st>>>(e.box_acc, e.systems);
    return cudaGetLastError();
}

cudaError_t bh_ensemble_step(int64_t n, BHWorkspace &w, const BHEnsembleTables &e, int key_mode, float4 *P,
                             float4 *Po, float4 *V, float4 *Vo, float4 *A, float4 *Ao, const int *I, int *Io,
                             cudaStream_t st, int *status, StageTimer *tm) {
    if (n <= 0 || e.systems <= 0) return cudaSuccess;
    cudaError_t err;
    if (tm) tm->begin(kStageBBox, st);
    bbox_seg_kernel<<<e.nchunks, 256, 0, st>>>(P, e.chunks, e.box_acc, e.boxes);
    if (tm) tm->end(kStageBBox, st);
    if (tm) tm->begin(kStageMorton, st);
    if (key_mode == NBODY_KEYS_MORTON)
        keys_seg_kernel<NBODY_KEYS_MORTON><<<grid_for(n, 256), 256, 0, st>>>(P, n, e.seg, e.boxes, w.keys[0],
                                                                              e.keys_orig, w.vals[0]);
    else
        keys_seg_kernel<NBODY_KEYS_OCTREE><<<grid_for(n, 256), 256, 0, st>>>(P, n, e.seg, e.boxes, w.keys[0],
                                                                              e.keys_orig, w.vals[0]);
    if (tm) tm->end(kStageMorton, st);
    if (tm) tm->begin(kStageSort, st);
    // Stable by key over all systems, then stable by system: within each
    // system the order is the single-system sort's.
    int alt = 0;
    err = sort_pairs(w.keys[0], w.vals[0], w.keys[1], w.vals[1], n, w.sort_scratch, st, status, &alt, 8);
    if (err != cudaSuccess) return err;
    uint64_t *k0 = alt ? w.keys[1] : w.keys[0], *k1 = alt ? w.keys[0] : w.keys[1];
    uint32_t *v0 = alt ? w.vals[1] : w.vals[0], *v1 = alt ? w.vals[0] : w.vals[1];
    if (e.systems > 1) {
        seg_keys_kernel<<<grid_for(n, 256), 256, 0, st>>>(v0, n, e.seg, k0, status);
        err = sort_pairs(k0, v0, k1, v1, n, w.sort_scratch, st, status, &alt, e.seg_passes);
        if (err != cudaSuccess) return err;
        if (alt) {
            uint32_t *tv = v0; v0 = v1; v1 = tv;
        }
    }
    if (tm) tm->end(kStageSort, st);
    if (tm) tm->begin(kStageGather, st);
    // Sorted keys into keys[0] (the build reads them there), permutation in vals[0].
    uint64_t *ksorted = w.keys[0];
    gather_kernel<<<grid_for(n, 256), 256, 0, st>>>(v0, n, P, V, A, I, Po, Vo, Ao, Io, status, e.keys_orig, ksorted);
    if (tm) tm->end(kStageGather, st);
    err = cudaGetLastError();
    if (err != cudaSuccess) return err;
    SegView sv;
    sv.seg = e.seg;
    sv.boxes = e.boxes;
    sv.fdepth = e.fdepth;
    err = bh_build(Po, n, w, st, status, tm, sv);
    if (err != cudaSuccess) return err;
    if (tm) tm->begin(kStageTraverse, st);
    const unsigned blocks = static_cast<unsigned>((static_cast<int64_t>(e.nwarps) * 32 + 255) / 256);
    if (w.counters)
        launch_walk<true, false, true, true>(w, blocks, st, nullptr, Po, n, 0.f, 0.f, 0.f, P, Vo, Ao, nullptr, nullptr,
                                             w.counters, nullptr, 0, e.warps, e.nwarps, e.params, w.P);
    else if (e.all_soft)
        launch_walk<false, false, true, false>(w, blocks, st, nullptr, Po, n, 0.f, 0.f, 0.f, P, Vo, Ao, nullptr,
                                               nullptr, nullptr, nullptr, 0, e.warps, e.nwarps, e.params, w.P);
    else
        launch_walk<false, false, true, true>(w, blocks, st, nullptr, Po, n, 0.f, 0.f, 0.f, P, Vo, Ao, nullptr, nullptr,
                                              nullptr, nullptr, 0, e.warps, e.nwarps, e.params, w.P);
    if (tm) tm->end(kStageTraverse, st);
    return cudaGetLastError();
}

cudaError_t bh_unpermute(const int *ids, int64_t n, const float4 *in, float4 *out, bool zero_w, cudaStream_t st,
                         int *status) {
    unpermute_kernel<<<grid_for(n, 256), 256, 0, st>>>(ids, n, in, out, zero_w ? 1 : 0, status);
    return cudaGetLastError();
}

}  // namespace nbody
