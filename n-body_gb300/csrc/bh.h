// Barnes-Hut pipeline internals (bounding box, keys, sort, gather, tree,
// upsweep, traversal); internal to the library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "kernels.h"

namespace nbody {

constexpr int kBBoxBlocks = 1024;

// One pre-order tree record (32 bytes). cm = centre of mass and mass (for a
// lone-body leaf: its position and mass). meta.x = s^2 of the cell as float
// bits (-1 for leaves), meta.y = next record after the subtree, meta.z =
// first body (sorted order), meta.w = body count of a leaf, 0 for a cell, or
// minus the body count of a cell whose children are all leaves.
struct __align__(16) BHNode {
    float4 cm;
    int4 meta;
};

// Binary radix tree over sorted keys: internal node i covers bodies
// [lo, hi]; a child < 0 is body ~child.
struct BinaryTree {
    int *lo, *hi, *left, *right, *delta, *iparent, *lparent, *top;
};

// Per-record bookkeeping for the bottom-up pass: level[r] = octree level of
// record r (kMaxLevel for a bucket, kMaxLevel + 1 for a lone body). The
// climbing schedule uses parent (octree parent record), nchild and arrive;
// the level schedule uses list (the cell records grouped by level; it shares
// arrive's storage) and lvl: lvl[0..32) = cells per level, lvl[32..64) = where
// each level's group starts in list, lvl[64..96) = fill cursors.
struct Records {
    int *level, *parent, *nchild;
    unsigned *arrive;
    unsigned *list;
    unsigned *lvl;
};

// Systems packed back to back (an ensemble): seg[b] = system of body b,
// boxes = 8 floats per system (min xyz, max xyz, 2 unused), fdepth = the
// reference's fixed top-level depth per system. seg == nullptr: one system.
struct SegView {
    const int *seg = nullptr;
    const float *boxes = nullptr;
    const int *fdepth = nullptr;
};

// Walk forms over the same records (same accepted set per body).
constexpr int kWalkUnion = 0;  // one record at a time for the warp's bodies, per-lane skip links
constexpr int kWalkCell = 1;   // cell by cell: a cell's children decided side by side for the bodies
                               // that opened it (from their box), per body only where they differ

struct BHWorkspace {
    int64_t n = 0;
    uint64_t *keys[2] = {nullptr, nullptr};
    uint32_t *vals[2] = {nullptr, nullptr};
    void *sort_scratch = nullptr;
    float *box = nullptr;  // min xyz, max xyz
    float *bbox_partial = nullptr;
    unsigned *bbox_counter = nullptr;
    BinaryTree tree{};
    Records rec{};
    uint32_t *mask = nullptr;
    uint32_t *cnt = nullptr;
    uint32_t *P = nullptr;  // n + 1 entries; P[n] = record count
    uint32_t *scan_sums = nullptr;
    BHNode *nodes = nullptr;  // up to 2n records
    int *kids = nullptr;      // 8 child records per cell record (cell walk)
    // Traversal counters (pairwise evaluations, warp record visits): the
    // traversal counts into `counters` when it is set (= counter_mem).
    unsigned long long *counter_mem = nullptr;
    unsigned long long *counters = nullptr;
    int bodies_per_lane = 1;  // traversal shape: 1 or 2 bodies per lane
    int walk = kWalkCell;     // with 2 bodies per lane: kWalkCell or kWalkUnion
    int64_t node_count_host = 0;
};

// The walk form: kWalkCell, or kWalkUnion when NBODY_BH_WALK=union.
int bh_walk_form();

// Bytes of device memory for a workspace of n bodies, and its layout inside
// `base` (base == nullptr only computes the size). The bbox counter must be
// zero before first use.
size_t bh_workspace_bytes(int64_t n);
size_t bh_workspace_layout(int64_t n, void *base, BHWorkspace *w);

cudaError_t bh_bbox(const float4 *pos, int64_t n, BHWorkspace &w, cudaStream_t st, StageTimer *timer);
// Keys of `mode` (NBODY_KEYS_OCTREE or NBODY_KEYS_MORTON) into keys[0], index into vals[0].
cudaError_t bh_keys(const float4 *pos, int64_t n, BHWorkspace &w, int mode, cudaStream_t st, StageTimer *timer);
cudaError_t bh_sort(int64_t n, BHWorkspace &w, cudaStream_t st, int *status, StageTimer *timer);
cudaError_t bh_gather(int64_t n, const BHWorkspace &w, const float4 *pos_in, const float4 *vel_in,
                      const float4 *acc_in, const int *id_in, float4 *pos_out, float4 *vel_out, float4 *acc_out,
                      int *id_out, cudaStream_t st, int *status, StageTimer *timer);
// Upsweep schedule of bh_build: true = one launch per octree level (ensembles,
// and systems from 2^21 bodies), false = the single-launch climb; and the
// kernel launches it takes.
bool bh_upsweep_by_levels(int64_t n, bool ensemble);
int bh_upsweep_launches(int64_t n, bool ensemble);
cudaError_t bh_build(const float4 *pos_sorted, int64_t n, BHWorkspace &w, cudaStream_t st, int *status,
                     StageTimer *timer, const SegView &sv = SegView{});
// The caller's arrays in the reference layout (device-mapped page-locked host
// memory), written by the walk itself at index ids[b]: positions with w = 0,
// velocities, accelerations and (if set) forces.
struct HostOut {
    float4 *pos = nullptr, *vel = nullptr, *acc = nullptr, *force = nullptr;
};
// Whether the workspace's walk form writes HostOut (the cell walk does).
bool bh_walk_writes_host(const BHWorkspace &w);
// Forces for every sorted body; with pos_out set, also the reference
// integrator (pos_out must not alias pos_sorted). force_out, if set, receives
// the acceleration at index ids[b] (or b when ids is null). host.pos set (and
// bh_walk_writes_host): the new state also goes to the caller's arrays.
// euler = 1 applies the GLSL path's semi-implicit Euler instead of the CPU order.
cudaError_t bh_traverse(const float4 *pos_sorted, int64_t n, const BHWorkspace &w, float eps2, float theta2,
                        float dt, float4 *pos_out, float4 *vel, float4 *acc, float4 *force_out, const int *ids,
                        int euler, cudaStream_t st, StageTimer *timer, const HostOut &host = HostOut{});
// Potential -sum m / sqrt(d^2 + eps^2) of every sorted body over the same
// accepted records as the forces, into phi_out[ids[b]] (or phi_out[b]).
cudaError_t bh_potential(const float4 *pos_sorted, int64_t n, const BHWorkspace &w, float eps2, float theta2,
                         float *phi_out, const int *ids, cudaStream_t st);
// Tables of an ensemble of Barnes-Hut systems packed back to back in one
// workspace (all body indices are global positions in the packed arrays).
struct BHEnsembleTables {
    int systems = 0;
    int *seg = nullptr;             // per body: its system
    int4 *chunks = nullptr;         // bounding-box chunks: system, first, end, chunks of the system
    int nchunks = 0;
    unsigned *box_acc = nullptr;    // per system, 8: encoded min xyz, max xyz, arrivals, unused
    float *boxes = nullptr;         // per system, 8: min xyz, max xyz, unused
    int *fdepth = nullptr;          // per system: the reference's fixed top-level depth
    int4 *warps = nullptr;          // traversal work: system, first body, system first, system end
    int nwarps = 0;
    float4 *params = nullptr;       // per system: dt, eps2, theta2, euler (0 / 1)
    uint64_t *keys_orig = nullptr;  // per body: unsorted key
    int seg_passes = 1;             // 8-bit digits of the system id
    bool all_soft = false;          // every system has eps2 > 0 and theta2 > 0
};

// Host helper: the reference's fixed top-level depth for n bodies.
int bh_father_depth(int64_t n);
// Seeds the per-system box accumulators (once after the tables are made).
cudaError_t bh_seed_boxes(const BHEnsembleTables &e, cudaStream_t st);
// One step of every system: positions P (updated in place), velocity and
// acceleration V, A -> Vo, Ao, ids I -> Io (I null: identity), Po scratch.
cudaError_t bh_ensemble_step(int64_t n, BHWorkspace &w, const BHEnsembleTables &e, int key_mode, float4 *P,
                             float4 *Po, float4 *V, float4 *Vo, float4 *A, float4 *Ao, const int *I, int *Io,
                             cudaStream_t st, int *status, StageTimer *tm);

cudaError_t bh_unpermute(const int *ids, int64_t n, const float4 *in, float4 *out, bool zero_w, cudaStream_t st,
                         int *status);

}  // namespace nbody
