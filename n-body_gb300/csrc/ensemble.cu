// Ensembles: many independent systems of uneven size stepped together (C ABI
// in include/nbody_gb300.h, nbody_ensemble_*). The reference steps one system
// per process; this is the batched form of its two solver paths.
//
// Layout. Systems below the crossover size go to the direct-sum group, the
// others to the Barnes-Hut group; each group packs its systems back to back
// (largest first) with an offset table, so one persistent direct-sum launch
// and one segmented Barnes-Hut pipeline step every system of the ensemble. The
// direct-sum launch runs on a side stream forked from the ensemble's stream,
// beside the Barnes-Hut stages. A step's launches can be captured k steps at a
// time into CUDA graphs (cached per k and buffer parity).
//
// Membership. Systems are added and removed at any time between steps; the
// layout is rebuilt lazily (new packed arrays from a private stream-ordered
// memory pool, states of the remaining systems moved device to device), which
// is what a serving loop needs to fold arrivals into the next launch.
//
// Independence. Every per-system quantity (box, keys, tree, sums) is computed
// from that system alone, in an order that does not depend on the other
// systems, so a system's trajectory is the same alone and in any mix.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <new>
#include <string>
#include <tuple>
#include <vector>

#include "bh.h"
#include "init.h"
#include "kernels.h"
#include "nbody_gb300.h"
#include "pp_batch.h"
#include "sort.h"
#include "timer.h"

namespace {

constexpr int kBBoxChunk = 4096;  // bodies per bounding-box CTA
constexpr int kWarpBodies = 64;   // bodies per traversal warp (two per lane)

__global__ void iota_kernel(int *__restrict__ out, int64_t n) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) out[i] = static_cast<int>(i);
}

unsigned blocks_for(int64_t n, int t) { return static_cast<unsigned>((n + t - 1) / t); }

struct Sys {
    int64_t n = 0;
    float dt = 0.f, eps2 = 0.f, theta2 = 0.25f;
    int mode = NBODY_MODE_PP;
    int euler = 0;
    bool alive = true;
    bool ready = false;  // state uploaded or generated
    // placement in the current layout (-1: not placed yet)
    int group_index = -1;
    int64_t first = -1;
};

template <typename T>
T *take(char *&p, size_t count) {
    T *r = reinterpret_cast<T *>(p);
    p += (count * sizeof(T) + 255) & ~static_cast<size_t>(255);
    return r;
}

template <typename T>
size_t bytes_of(size_t count) {
    return (count * sizeof(T) + 255) & ~static_cast<size_t>(255);
}

}  // namespace

struct nbody_ensemble {
    int device = 0;
    int64_t crossover = 4096;
    int pp_shape = nbody::kPPBatch256x2;
    int key_mode = NBODY_KEYS_OCTREE;
    cudaStream_t own_stream = nullptr, stream = nullptr, side = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    cudaMemPool_t pool = nullptr;
    int *status = nullptr;
    std::string last_error;
    std::vector<Sys> sys;
    bool dirty = true;

    // direct-sum group
    std::vector<int> pp_order;  // system ids in group order
    int64_t pp_n = 0;
    float4 *pp_pos[2] = {nullptr, nullptr};
    int pp_cur = 0;
    float4 *pp_vel = nullptr, *pp_acc = nullptr;
    void *pp_tab = nullptr;
    int2 *pp_items = nullptr;
    int pp_nitems = 0, pp_ctas = 0;
    int4 *pp_range = nullptr;
    float4 *pp_prm = nullptr;
    unsigned *pp_sched = nullptr;

    // Barnes-Hut group
    std::vector<int> bh_order;
    int64_t bh_n = 0;
    float4 *bh_pos[2] = {nullptr, nullptr};
    float4 *bh_vel[2] = {nullptr, nullptr}, *bh_acc[2] = {nullptr, nullptr};
    int *bh_ids[2] = {nullptr, nullptr};
    int bh_va = 0;
    void *bh_tab_mem = nullptr;
    nbody::BHEnsembleTables tab;
    void *ws_mem = nullptr;
    int64_t ws_cap = 0;
    nbody::BHWorkspace ws;

    // staging for one system's upload / download (2 float4 per body)
    float4 *stage = nullptr;
    int64_t stage_cap = 0;

    struct Graph {
        cudaGraphExec_t exec = nullptr;
        int end_pp_cur = 0, end_bh_va = 0;
    };
    std::map<std::tuple<int, int, int>, Graph> graphs;
    int64_t steps_done = 0;
    nbody::EventTimer *timer = nullptr;  // non-null while profiling (steps then run without graphs)
};

namespace {

int efail(nbody_ensemble *e, cudaError_t err) {
    e->last_error = cudaGetErrorString(err);
    if (err == cudaErrorMemoryAllocation) return NBODY_ERR_NOMEM;
    return NBODY_ERR_CUDA;
}

#define EN_CK(e, call)                                  \
    do {                                                \
        cudaError_t err_ = (call);                      \
        if (err_ != cudaSuccess) return efail(e, err_); \
    } while (0)

struct DevGuard {
    int prev = -1;
    bool ok = true;
    explicit DevGuard(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != dev) ok = cudaSetDevice(dev) == cudaSuccess;
    }
    ~DevGuard() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

void pool_free(nbody_ensemble *e, void *&p) {
    if (p) cudaFreeAsync(p, e->stream);
    p = nullptr;
}

template <typename T>
cudaError_t pool_alloc(nbody_ensemble *e, T **p, size_t bytes) {
    void *q = nullptr;
    const cudaError_t err = cudaMallocFromPoolAsync(&q, bytes > 0 ? bytes : 256, e->pool, e->stream);
    *p = static_cast<T *>(q);
    return err;
}

cudaError_t pool_alloc_raw(nbody_ensemble *e, void **p, size_t bytes) {
    return cudaMallocFromPoolAsync(p, bytes > 0 ? bytes : 256, e->pool, e->stream);
}

// Every block of the current layout back to the pool (stream ordered).
void free_layout(nbody_ensemble *e) {
    void *blocks[] = {e->pp_pos[0], e->pp_pos[1], e->pp_vel,    e->pp_acc,    e->bh_pos[0], e->bh_pos[1],
                      e->bh_vel[0], e->bh_vel[1], e->bh_acc[0], e->bh_acc[1], e->bh_ids[0], e->bh_ids[1],
                      e->pp_tab,    e->bh_tab_mem, e->ws_mem,   e->stage};
    for (void *p : blocks) pool_free(e, p);
    e->pp_pos[0] = e->pp_pos[1] = e->pp_vel = e->pp_acc = nullptr;
    e->bh_pos[0] = e->bh_pos[1] = e->bh_vel[0] = e->bh_vel[1] = e->bh_acc[0] = e->bh_acc[1] = nullptr;
    e->bh_ids[0] = e->bh_ids[1] = nullptr;
    e->pp_tab = e->bh_tab_mem = e->ws_mem = nullptr;
    e->stage = nullptr;
    e->ws_cap = e->stage_cap = 0;
}

void clear_graphs(nbody_ensemble *e) {
    for (auto &kv : e->graphs)
        if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
    e->graphs.clear();
}

int read_status(nbody_ensemble *e) {
    int h = 0;
    EN_CK(e, cudaMemcpyAsync(&h, e->status, sizeof(int), cudaMemcpyDeviceToHost, e->stream));
    EN_CK(e, cudaStreamSynchronize(e->stream));
    if (h != NBODY_OK) {
        // Re-arm everything a failed kernel may have left half way.
        cudaMemsetAsync(e->status, 0, sizeof(int), e->stream);
        if (e->pp_sched) cudaMemsetAsync(e->pp_sched, 0, 2 * sizeof(unsigned), e->stream);
        if (e->tab.systems > 0) nbody::bh_seed_boxes(e->tab, e->stream);
        cudaStreamSynchronize(e->stream);
        e->last_error = nbody_status_string(h);
    }
    return h;
}

// Rebuilds the packed layout of the live systems and moves the states of the
// ones already placed. Called lazily before anything that needs placements.
int relayout(nbody_ensemble *e) {
    if (!e->dirty) return NBODY_OK;
    clear_graphs(e);
    std::vector<int> pp, bh;
    for (int id = 0; id < static_cast<int>(e->sys.size()); ++id) {
        const Sys &s = e->sys[id];
        if (!s.alive) continue;
        (s.mode == NBODY_MODE_PP ? pp : bh).push_back(id);
    }
    auto by_size = [&](int a, int b) { return e->sys[a].n != e->sys[b].n ? e->sys[a].n > e->sys[b].n : a < b; };
    std::stable_sort(pp.begin(), pp.end(), by_size);
    std::stable_sort(bh.begin(), bh.end(), by_size);
    int64_t pp_n = 0, bh_n = 0;
    std::vector<int64_t> new_first(e->sys.size(), -1);
    for (int id : pp) { new_first[id] = pp_n; pp_n += e->sys[id].n; }
    for (int id : bh) { new_first[id] = bh_n; bh_n += e->sys[id].n; }
    if (pp_n > INT32_MAX || bh_n > INT32_MAX) {
        e->last_error = "ensemble larger than 2^31 bodies per group";
        return NBODY_ERR_CAPACITY;
    }

    // --- new state arrays; move the placed systems
    float4 *npp_pos = nullptr, *npp_vel = nullptr, *npp_acc = nullptr, *npp_pos_alt = nullptr;
    float4 *nbh_pos = nullptr, *nbh_pos_alt = nullptr, *nbh_vel[2] = {nullptr, nullptr}, *nbh_acc[2] = {nullptr, nullptr};
    int *nbh_ids[2] = {nullptr, nullptr};
    const size_t p4 = static_cast<size_t>(pp_n) * sizeof(float4), b4 = static_cast<size_t>(bh_n) * sizeof(float4);
    EN_CK(e, pool_alloc(e, &npp_pos, p4));
    EN_CK(e, pool_alloc(e, &npp_pos_alt, p4));
    EN_CK(e, pool_alloc(e, &npp_vel, p4));
    EN_CK(e, pool_alloc(e, &npp_acc, p4));
    EN_CK(e, pool_alloc(e, &nbh_pos, b4));
    EN_CK(e, pool_alloc(e, &nbh_pos_alt, b4));
    for (int k = 0; k < 2; ++k) {
        EN_CK(e, pool_alloc(e, &nbh_vel[k], b4));
        EN_CK(e, pool_alloc(e, &nbh_acc[k], b4));
        EN_CK(e, pool_alloc(e, &nbh_ids[k], static_cast<size_t>(bh_n) * sizeof(int)));
    }
    for (int id = 0; id < static_cast<int>(e->sys.size()); ++id) {
        Sys &s = e->sys[id];
        if (!s.alive || s.first < 0 || !s.ready) continue;
        const size_t nb = static_cast<size_t>(s.n) * sizeof(float4);
        const int64_t of = s.first, nf = new_first[id];
        if (s.mode == NBODY_MODE_PP) {
            EN_CK(e, cudaMemcpyAsync(npp_pos + nf, e->pp_pos[e->pp_cur] + of, nb, cudaMemcpyDeviceToDevice, e->stream));
            EN_CK(e, cudaMemcpyAsync(npp_vel + nf, e->pp_vel + of, nb, cudaMemcpyDeviceToDevice, e->stream));
            EN_CK(e, cudaMemcpyAsync(npp_acc + nf, e->pp_acc + of, nb, cudaMemcpyDeviceToDevice, e->stream));
        } else {
            EN_CK(e, cudaMemcpyAsync(nbh_pos + nf, e->bh_pos[0] + of, nb, cudaMemcpyDeviceToDevice, e->stream));
            EN_CK(e, cudaMemcpyAsync(nbh_vel[0] + nf, e->bh_vel[e->bh_va] + of, nb, cudaMemcpyDeviceToDevice,
                                     e->stream));
            EN_CK(e, cudaMemcpyAsync(nbh_acc[0] + nf, e->bh_acc[e->bh_va] + of, nb, cudaMemcpyDeviceToDevice,
                                     e->stream));
            EN_CK(e, cudaMemcpyAsync(nbh_ids[0] + nf, e->bh_ids[e->bh_va] + of, static_cast<size_t>(s.n) * sizeof(int),
                                     cudaMemcpyDeviceToDevice, e->stream));
        }
    }
    // The side stream may still be reading the old arrays: order the frees after it.
    EN_CK(e, cudaEventRecord(e->join, e->side));
    EN_CK(e, cudaStreamWaitEvent(e->stream, e->join, 0));
    void *old[] = {e->pp_pos[0], e->pp_pos[1], e->pp_vel, e->pp_acc, e->bh_pos[0], e->bh_pos[1],
                   e->bh_vel[0], e->bh_vel[1], e->bh_acc[0], e->bh_acc[1], e->bh_ids[0], e->bh_ids[1]};
    for (void *p : old) pool_free(e, p);
    e->pp_pos[0] = npp_pos;
    e->pp_pos[1] = npp_pos_alt;
    e->pp_cur = 0;
    e->pp_vel = npp_vel;
    e->pp_acc = npp_acc;
    e->bh_pos[0] = nbh_pos;
    e->bh_pos[1] = nbh_pos_alt;
    for (int k = 0; k < 2; ++k) {
        e->bh_vel[k] = nbh_vel[k];
        e->bh_acc[k] = nbh_acc[k];
        e->bh_ids[k] = nbh_ids[k];
    }
    e->bh_va = 0;
    for (int id = 0; id < static_cast<int>(e->sys.size()); ++id) e->sys[id].first = new_first[id];
    for (size_t g = 0; g < pp.size(); ++g) e->sys[pp[g]].group_index = static_cast<int>(g);
    for (size_t g = 0; g < bh.size(); ++g) e->sys[bh[g]].group_index = static_cast<int>(g);
    e->pp_order = pp;
    e->bh_order = bh;
    e->pp_n = pp_n;
    e->bh_n = bh_n;

    // --- direct-sum tables
    pool_free(e, e->pp_tab);
    {
        const int per = nbody::pp_batch_bodies_per_item(e->pp_shape);
        std::vector<int2> items;
        std::vector<int4> range(pp.size());
        std::vector<float4> prm(pp.size());
        for (size_t g = 0; g < pp.size(); ++g) {
            const Sys &s = e->sys[pp[g]];
            range[g] = make_int4(static_cast<int>(s.first), static_cast<int>(s.n), 0, 0);
            prm[g] = make_float4(s.dt, s.eps2, 0.f, s.euler ? 1.f : 0.f);
            for (int64_t b = 0; b < s.n; b += per)
                items.push_back(make_int2(static_cast<int>(g), static_cast<int>(s.first + b)));
        }
        const size_t bytes = bytes_of<int2>(items.size()) + bytes_of<int4>(range.size()) +
                             bytes_of<float4>(prm.size()) + bytes_of<unsigned>(2);
        EN_CK(e, pool_alloc_raw(e, &e->pp_tab, bytes));
        char *p = static_cast<char *>(e->pp_tab);
        e->pp_items = take<int2>(p, items.size());
        e->pp_range = take<int4>(p, range.size());
        e->pp_prm = take<float4>(p, prm.size());
        e->pp_sched = take<unsigned>(p, 2);
        e->pp_nitems = static_cast<int>(items.size());
        e->pp_ctas = nbody::pp_batch_ctas(e->pp_shape, e->device, e->pp_nitems);
        if (!items.empty())
            EN_CK(e, cudaMemcpyAsync(e->pp_items, items.data(), items.size() * sizeof(int2), cudaMemcpyHostToDevice,
                                     e->stream));
        if (!range.empty()) {
            EN_CK(e, cudaMemcpyAsync(e->pp_range, range.data(), range.size() * sizeof(int4), cudaMemcpyHostToDevice,
                                     e->stream));
            EN_CK(e, cudaMemcpyAsync(e->pp_prm, prm.data(), prm.size() * sizeof(float4), cudaMemcpyHostToDevice,
                                     e->stream));
        }
        EN_CK(e, cudaMemsetAsync(e->pp_sched, 0, 2 * sizeof(unsigned), e->stream));
    }

    // --- Barnes-Hut tables and workspace
    pool_free(e, e->bh_tab_mem);
    e->tab = nbody::BHEnsembleTables{};
    if (!bh.empty()) {
        std::vector<int> seg(static_cast<size_t>(bh_n));
        std::vector<int4> chunks, warps;
        std::vector<int> fdepth(bh.size());
        std::vector<float4> prm(bh.size());
        for (size_t g = 0; g < bh.size(); ++g) {
            const Sys &s = e->sys[bh[g]];
            const int f = static_cast<int>(s.first), end = static_cast<int>(s.first + s.n);
            std::fill(seg.begin() + f, seg.begin() + end, static_cast<int>(g));
            const int nch = static_cast<int>((s.n + kBBoxChunk - 1) / kBBoxChunk);
            for (int c = 0; c < nch; ++c)
                chunks.push_back(make_int4(static_cast<int>(g), f + c * kBBoxChunk,
                                           std::min(end, f + (c + 1) * kBBoxChunk), nch));
            for (int b = f; b < end; b += kWarpBodies) warps.push_back(make_int4(static_cast<int>(g), b, f, end));
            fdepth[g] = nbody::bh_father_depth(s.n);
            prm[g] = make_float4(s.dt, s.eps2, s.theta2, s.euler ? 1.f : 0.f);
        }
        const size_t nsys = bh.size();
        const size_t bytes = bytes_of<int>(seg.size()) + bytes_of<int4>(chunks.size()) + bytes_of<unsigned>(8 * nsys) +
                             bytes_of<float>(8 * nsys) + bytes_of<int>(nsys) + bytes_of<int4>(warps.size()) +
                             bytes_of<float4>(nsys) + bytes_of<uint64_t>(static_cast<size_t>(bh_n));
        EN_CK(e, pool_alloc_raw(e, &e->bh_tab_mem, bytes));
        char *p = static_cast<char *>(e->bh_tab_mem);
        nbody::BHEnsembleTables &t = e->tab;
        t.systems = static_cast<int>(nsys);
        t.seg = take<int>(p, seg.size());
        t.chunks = take<int4>(p, chunks.size());
        t.nchunks = static_cast<int>(chunks.size());
        t.box_acc = take<unsigned>(p, 8 * nsys);
        t.boxes = take<float>(p, 8 * nsys);
        t.fdepth = take<int>(p, nsys);
        t.warps = take<int4>(p, warps.size());
        t.nwarps = static_cast<int>(warps.size());
        t.params = take<float4>(p, nsys);
        t.keys_orig = take<uint64_t>(p, static_cast<size_t>(bh_n));
        t.seg_passes = nsys <= 256 ? 1 : nsys <= 65536 ? 2 : 3;
        t.all_soft = true;
        for (int id : bh) t.all_soft = t.all_soft && e->sys[id].eps2 > 0.f && e->sys[id].theta2 > 0.f;
        EN_CK(e, cudaMemcpyAsync(t.seg, seg.data(), seg.size() * sizeof(int), cudaMemcpyHostToDevice, e->stream));
        EN_CK(e, cudaMemcpyAsync(t.chunks, chunks.data(), chunks.size() * sizeof(int4), cudaMemcpyHostToDevice,
                                 e->stream));
        EN_CK(e, cudaMemcpyAsync(t.fdepth, fdepth.data(), nsys * sizeof(int), cudaMemcpyHostToDevice, e->stream));
        EN_CK(e, cudaMemcpyAsync(t.warps, warps.data(), warps.size() * sizeof(int4), cudaMemcpyHostToDevice,
                                 e->stream));
        EN_CK(e, cudaMemcpyAsync(t.params, prm.data(), nsys * sizeof(float4), cudaMemcpyHostToDevice, e->stream));
        EN_CK(e, nbody::bh_seed_boxes(t, e->stream));
        // The order-dependent vectors above must outlive their copies.
        EN_CK(e, cudaStreamSynchronize(e->stream));
        if (bh_n > e->ws_cap) {
            pool_free(e, e->ws_mem);
            const int64_t cap = bh_n + bh_n / 4;
            nbody::BHWorkspace w;
            const size_t wb = nbody::bh_workspace_layout(cap, nullptr, &w);
            EN_CK(e, pool_alloc_raw(e, &e->ws_mem, wb));
            nbody::bh_workspace_layout(cap, e->ws_mem, &e->ws);
            EN_CK(e, cudaMemsetAsync(e->ws.bbox_counter, 0, sizeof(unsigned) * 4, e->stream));
            EN_CK(e, cudaMemsetAsync(e->ws.counter_mem, 0, sizeof(unsigned long long) * 2, e->stream));
            e->ws.bodies_per_lane = 2;
            e->ws.walk = nbody::bh_walk_form();
            e->ws_cap = cap;
        }
    }
    // staging for the largest system
    int64_t nmax = 0;
    for (const Sys &s : e->sys)
        if (s.alive) nmax = std::max(nmax, s.n);
    if (nmax > e->stage_cap) {
        void *st = e->stage;
        pool_free(e, st);
        EN_CK(e, pool_alloc(e, &e->stage, 2 * static_cast<size_t>(nmax) * sizeof(float4)));
        e->stage_cap = nmax;
    }
    EN_CK(e, cudaStreamSynchronize(e->stream));
    e->dirty = false;
    return NBODY_OK;
}

int check_system(nbody_ensemble *e, int id) {
    if (!e || id < 0 || id >= static_cast<int>(e->sys.size()) || !e->sys[id].alive) return NBODY_ERR_ARG;
    return NBODY_OK;
}

// One step of every system: direct sum on the side stream, Barnes-Hut on the main stream.
int step_once(nbody_ensemble *e) {
    if (e->pp_nitems > 0) {
        EN_CK(e, cudaEventRecord(e->fork, e->stream));
        EN_CK(e, cudaStreamWaitEvent(e->side, e->fork, 0));
        if (e->timer) e->timer->begin(nbody::kStagePPForce, e->side);
        EN_CK(e, nbody::pp_batch_launch(e->pp_shape, e->pp_ctas, e->pp_pos[e->pp_cur], e->pp_pos[e->pp_cur ^ 1],
                                        e->pp_vel, e->pp_acc, e->pp_items, e->pp_nitems, e->pp_range, e->pp_prm,
                                        e->pp_sched, e->side, e->status));
        if (e->timer) e->timer->end(nbody::kStagePPForce, e->side);
        e->pp_cur ^= 1;
    }
    if (e->bh_n > 0) {
        const int va = e->bh_va;
        EN_CK(e, nbody::bh_ensemble_step(e->bh_n, e->ws, e->tab, e->key_mode, e->bh_pos[0], e->bh_pos[1],
                                         e->bh_vel[va], e->bh_vel[va ^ 1], e->bh_acc[va], e->bh_acc[va ^ 1],
                                         e->bh_ids[va], e->bh_ids[va ^ 1], e->stream, e->status, e->timer));
        e->bh_va ^= 1;
    }
    if (e->pp_nitems > 0) {
        EN_CK(e, cudaEventRecord(e->join, e->side));
        EN_CK(e, cudaStreamWaitEvent(e->stream, e->join, 0));
    }
    ++e->steps_done;
    return NBODY_OK;
}

int run_graph(nbody_ensemble *e, int k) {
    const auto key = std::make_tuple(k, e->pp_cur, e->bh_va);
    auto it = e->graphs.find(key);
    if (it == e->graphs.end()) {
        const int pc = e->pp_cur, va = e->bh_va;
        const int64_t done = e->steps_done;
        EN_CK(e, cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
        int rc = NBODY_OK;
        for (int s = 0; s < k && rc == NBODY_OK; ++s) rc = step_once(e);
        cudaGraph_t g = nullptr;
        const cudaError_t ec = cudaStreamEndCapture(e->stream, &g);
        if (rc != NBODY_OK) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        if (ec != cudaSuccess) return efail(e, ec);
        nbody_ensemble::Graph gr;
        gr.end_pp_cur = e->pp_cur;
        gr.end_bh_va = e->bh_va;
        const cudaError_t ei = cudaGraphInstantiate(&gr.exec, g, 0);
        cudaGraphDestroy(g);
        if (ei != cudaSuccess) return efail(e, ei);
        e->pp_cur = pc;
        e->bh_va = va;
        e->steps_done = done;
        it = e->graphs.emplace(key, gr).first;
    }
    EN_CK(e, cudaGraphLaunch(it->second.exec, e->stream));
    e->pp_cur = it->second.end_pp_cur;
    e->bh_va = it->second.end_bh_va;
    e->steps_done += k;
    return NBODY_OK;
}

}  // namespace

extern "C" {

int nbody_ensemble_create(nbody_ensemble **out, int device, int64_t crossover) {
    if (!out || device < 0 || crossover < 0) return NBODY_ERR_ARG;
    *out = nullptr;
    nbody_ensemble *e = new (std::nothrow) nbody_ensemble();
    if (!e) return NBODY_ERR_NOMEM;
    e->device = device;
    e->crossover = crossover;
    DevGuard dg(device);
    int rc = dg.ok ? NBODY_OK : NBODY_ERR_CUDA;
    auto ck = [&](cudaError_t err) {
        if (rc == NBODY_OK && err != cudaSuccess) rc = efail(e, err);
    };
    ck(cudaStreamCreateWithFlags(&e->own_stream, cudaStreamNonBlocking));
    e->stream = e->own_stream;
    ck(cudaStreamCreateWithFlags(&e->side, cudaStreamNonBlocking));
    ck(cudaEventCreateWithFlags(&e->fork, cudaEventDisableTiming));
    ck(cudaEventCreateWithFlags(&e->join, cudaEventDisableTiming));
    if (rc == NBODY_OK) {
        cudaMemPoolProps props{};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = device;
        ck(cudaMemPoolCreate(&e->pool, &props));
        uint64_t keep = UINT64_MAX;  // keep freed blocks for the next layout
        if (rc == NBODY_OK) ck(cudaMemPoolSetAttribute(e->pool, cudaMemPoolAttrReleaseThreshold, &keep));
    }
    ck(cudaMalloc(&e->status, sizeof(int)));
    if (rc == NBODY_OK) ck(cudaMemsetAsync(e->status, 0, sizeof(int), e->stream));
    if (rc == NBODY_OK) ck(nbody::sort_prepare(device));
    if (rc == NBODY_OK) ck(cudaStreamSynchronize(e->stream));
    if (rc != NBODY_OK) {
        nbody_ensemble_destroy(e);
        return rc;
    }
    *out = e;
    return NBODY_OK;
}

int nbody_ensemble_destroy(nbody_ensemble *e) {
    if (!e) return NBODY_ERR_ARG;
    {
        DevGuard dg(e->device);
        if (e->side) cudaStreamSynchronize(e->side);
        if (e->stream) cudaStreamSynchronize(e->stream);
        clear_graphs(e);
        delete e->timer;
        e->timer = nullptr;
        if (e->pool && e->stream) {
            free_layout(e);
            cudaStreamSynchronize(e->stream);
        }
        if (e->pool) cudaMemPoolDestroy(e->pool);
        if (e->status) cudaFree(e->status);
        if (e->fork) cudaEventDestroy(e->fork);
        if (e->join) cudaEventDestroy(e->join);
        if (e->side) cudaStreamDestroy(e->side);
        if (e->own_stream) cudaStreamDestroy(e->own_stream);
    }
    delete e;
    return NBODY_OK;
}

const char *nbody_ensemble_last_error(const nbody_ensemble *e) { return e ? e->last_error.c_str() : "null ensemble"; }

int nbody_ensemble_set_stream(nbody_ensemble *e, void *stream) {
    if (!e) return NBODY_ERR_ARG;
    DevGuard dg(e->device);
    // Work already queued on the old streams finishes first.
    if (e->stream) EN_CK(e, cudaStreamSynchronize(e->stream));
    if (e->side) EN_CK(e, cudaStreamSynchronize(e->side));
    e->stream = stream ? static_cast<cudaStream_t>(stream) : e->own_stream;
    // The side stream (direct-sum launch) takes the caller's stream priority.
    int prio = 0, side_prio = 0;
    EN_CK(e, cudaStreamGetPriority(e->stream, &prio));
    EN_CK(e, cudaStreamGetPriority(e->side, &side_prio));
    if (prio != side_prio) {
        cudaStream_t ns = nullptr;
        EN_CK(e, cudaStreamCreateWithPriority(&ns, cudaStreamNonBlocking, prio));
        cudaStreamDestroy(e->side);
        e->side = ns;
    }
    clear_graphs(e);
    return NBODY_OK;
}

int nbody_ensemble_set_options(nbody_ensemble *e, int pp_shape, int key_mode) {
    if (!e || pp_shape < 0 || pp_shape >= nbody::kPPBatchShapes ||
        (key_mode != NBODY_KEYS_OCTREE && key_mode != NBODY_KEYS_MORTON))
        return NBODY_ERR_ARG;
    if (pp_shape != e->pp_shape) e->dirty = true;  // the work items change
    e->pp_shape = pp_shape;
    e->key_mode = key_mode;
    clear_graphs(e);
    return NBODY_OK;
}

int nbody_ensemble_add(nbody_ensemble *e, int64_t n, float dt, float eps2, float theta2, int mode, int integrator,
                       int *system) {
    if (!e || !system || n <= 0 || n > INT32_MAX || !(eps2 >= 0.f) ||
        (mode != -1 && mode != NBODY_MODE_PP && mode != NBODY_MODE_BH) ||
        (integrator != NBODY_INTEGRATOR_CPU && integrator != NBODY_INTEGRATOR_GPU_EULER))
        return NBODY_ERR_ARG;
    Sys s;
    s.n = n;
    s.dt = dt;
    s.eps2 = eps2;
    s.theta2 = theta2 > 0.f ? theta2 : 0.25f;
    s.mode = mode >= 0 ? mode : (n < e->crossover ? NBODY_MODE_PP : NBODY_MODE_BH);
    s.euler = integrator == NBODY_INTEGRATOR_GPU_EULER ? 1 : 0;
    e->sys.push_back(s);
    e->dirty = true;
    *system = static_cast<int>(e->sys.size()) - 1;
    return NBODY_OK;
}

int nbody_ensemble_remove(nbody_ensemble *e, int system) {
    const int rc = check_system(e, system);
    if (rc != NBODY_OK) return rc;
    e->sys[system].alive = false;
    e->dirty = true;
    return NBODY_OK;
}

int nbody_ensemble_system_info(nbody_ensemble *e, int system, int *mode, int64_t *n) {
    const int rc = check_system(e, system);
    if (rc != NBODY_OK) return rc;
    if (mode) *mode = e->sys[system].mode;
    if (n) *n = e->sys[system].n;
    return NBODY_OK;
}

int nbody_ensemble_upload(nbody_ensemble *e, int system, const float *positions4, const float *velocities4,
                          const float *accelerations4, const float *masses4) {
    int rc = check_system(e, system);
    if (rc != NBODY_OK) return rc;
    if (!positions4 || !masses4) return NBODY_ERR_ARG;
    DevGuard dg(e->device);
    if ((rc = relayout(e)) != NBODY_OK) return rc;
    Sys &s = e->sys[system];
    const size_t nb = static_cast<size_t>(s.n) * sizeof(float4);
    const bool pp = s.mode == NBODY_MODE_PP;
    float4 *pos = pp ? e->pp_pos[e->pp_cur] + s.first : e->bh_pos[0] + s.first;
    float4 *vel = pp ? e->pp_vel + s.first : e->bh_vel[e->bh_va] + s.first;
    float4 *acc = pp ? e->pp_acc + s.first : e->bh_acc[e->bh_va] + s.first;
    // Page-locked host arrays are read in place by one kernel; otherwise one
    // copy per array into the staging area, then the pack kernel.
    const float4 *mp = nbody::host_mapped(positions4, nb, e->device);
    const float4 *mm = nbody::host_mapped(masses4, nb, e->device);
    const float4 *mv = velocities4 ? nbody::host_mapped(velocities4, nb, e->device) : nullptr;
    const float4 *ma = accelerations4 ? nbody::host_mapped(accelerations4, nb, e->device) : nullptr;
    if (mp && mm && (!velocities4 || mv) && (!accelerations4 || ma)) {
        EN_CK(e, nbody::host_gather(mp, mm, mv, ma, pos, vel, acc, s.n, e->stream));
    } else {
        EN_CK(e, cudaMemcpyAsync(e->stage, positions4, nb, cudaMemcpyHostToDevice, e->stream));
        EN_CK(e, cudaMemcpyAsync(e->stage + s.n, masses4, nb, cudaMemcpyHostToDevice, e->stream));
        EN_CK(e, nbody::pack_state(e->stage, e->stage + s.n, pos, s.n, e->stream));
        if (velocities4) EN_CK(e, cudaMemcpyAsync(vel, velocities4, nb, cudaMemcpyHostToDevice, e->stream));
        else EN_CK(e, cudaMemsetAsync(vel, 0, nb, e->stream));
        if (accelerations4) EN_CK(e, cudaMemcpyAsync(acc, accelerations4, nb, cudaMemcpyHostToDevice, e->stream));
        else EN_CK(e, cudaMemsetAsync(acc, 0, nb, e->stream));
    }
    if (!pp) {
        iota_kernel<<<blocks_for(s.n, 256), 256, 0, e->stream>>>(e->bh_ids[e->bh_va] + s.first, s.n);
        EN_CK(e, cudaGetLastError());
    }
    // The host arrays may be reused once this returns.
    EN_CK(e, cudaStreamSynchronize(e->stream));
    s.ready = true;
    return NBODY_OK;
}

int nbody_ensemble_init_device(nbody_ensemble *e, int system, int kind, uint64_t seed, const float *params,
                               int nparams) {
    int rc = check_system(e, system);
    if (rc != NBODY_OK) return rc;
    if (!nbody::init_kind_valid(kind) || nparams < 0 || nparams > NBODY_INIT_MAX_PARAMS || (nparams > 0 && !params))
        return NBODY_ERR_ARG;
    Sys &s = e->sys[system];
    if (kind == NBODY_INIT_TWO_DISCS && (s.n < 2 || s.n % 2 != 0)) return NBODY_ERR_ARG;
    DevGuard dg(e->device);
    if ((rc = relayout(e)) != NBODY_OK) return rc;
    nbody::InitParams prm = nbody::init_defaults(kind);
    for (int k = 0; k < nparams; ++k) prm.p[k] = params[k];
    const bool pp = s.mode == NBODY_MODE_PP;
    float4 *pos = pp ? e->pp_pos[e->pp_cur] + s.first : e->bh_pos[0] + s.first;
    float4 *vel = pp ? e->pp_vel + s.first : e->bh_vel[e->bh_va] + s.first;
    float4 *acc = pp ? e->pp_acc + s.first : e->bh_acc[e->bh_va] + s.first;
    EN_CK(e, nbody::init_state(kind, seed, s.n, prm, pos, vel, acc, e->stream));
    if (!pp) {
        iota_kernel<<<blocks_for(s.n, 256), 256, 0, e->stream>>>(e->bh_ids[e->bh_va] + s.first, s.n);
        EN_CK(e, cudaGetLastError());
    }
    s.ready = true;
    return NBODY_OK;
}

int nbody_ensemble_step(nbody_ensemble *e, int steps, int graph_steps) {
    if (!e || steps < 0 || graph_steps < 0) return NBODY_ERR_ARG;
    DevGuard dg(e->device);
    int rc = relayout(e);
    if (rc != NBODY_OK) return rc;
    for (const Sys &s : e->sys)
        if (s.alive && !s.ready) return NBODY_ERR_STATE;
    int left = steps;
    if (graph_steps > 0 && !e->timer)
        while (rc == NBODY_OK && left >= graph_steps) {
            rc = run_graph(e, graph_steps);
            left -= graph_steps;
        }
    while (rc == NBODY_OK && left > 0) {
        rc = step_once(e);
        --left;
    }
    return rc;
}

int nbody_ensemble_download(nbody_ensemble *e, int system, float *positions4, float *velocities4,
                            float *accelerations4, float *masses4) {
    int rc = check_system(e, system);
    if (rc != NBODY_OK) return rc;
    DevGuard dg(e->device);
    if ((rc = relayout(e)) != NBODY_OK) return rc;
    Sys &s = e->sys[system];
    if (!s.ready) return NBODY_ERR_STATE;
    const size_t nb = static_cast<size_t>(s.n) * sizeof(float4);
    {
        // Page-locked host arrays are written in place by one kernel, in the
        // caller's order (a Barnes-Hut system through the inverse of its key
        // order, built in the staging area).
        const int dev = e->device;
        float4 *mp = positions4 ? nbody::host_mapped(positions4, nb, dev) : nullptr;
        float4 *mv = velocities4 ? nbody::host_mapped(velocities4, nb, dev) : nullptr;
        float4 *ma = accelerations4 ? nbody::host_mapped(accelerations4, nb, dev) : nullptr;
        float4 *mm = masses4 ? nbody::host_mapped(masses4, nb, dev) : nullptr;
        if ((!positions4 || mp) && (!velocities4 || mv) && (!accelerations4 || ma) && (!masses4 || mm)) {
            const bool pp = s.mode == NBODY_MODE_PP;
            if (mp || mv || ma || mm)
                EN_CK(e, nbody::host_scatter(pp ? e->pp_pos[e->pp_cur] + s.first : e->bh_pos[0] + s.first,
                                             pp ? e->pp_vel + s.first : e->bh_vel[e->bh_va] + s.first,
                                             pp ? e->pp_acc + s.first : e->bh_acc[e->bh_va] + s.first,
                                             pp ? nullptr : e->bh_ids[e->bh_va] + s.first,
                                             reinterpret_cast<int *>(e->stage), mp, mv, ma, nullptr, mm, s.n,
                                             e->stream, e->status));
            return read_status(e);
        }
    }
    if (s.mode == NBODY_MODE_PP) {
        const float4 *pos = e->pp_pos[e->pp_cur] + s.first;
        if (positions4) {
            EN_CK(e, nbody::unpack_positions(pos, e->stage, s.n, e->stream));
            EN_CK(e, cudaMemcpyAsync(positions4, e->stage, nb, cudaMemcpyDeviceToHost, e->stream));
        }
        if (masses4) {
            EN_CK(e, nbody::unpack_masses(pos, nullptr, e->stage + s.n, s.n, e->stream, e->status));
            EN_CK(e, cudaMemcpyAsync(masses4, e->stage + s.n, nb, cudaMemcpyDeviceToHost, e->stream));
        }
        if (velocities4)
            EN_CK(e, cudaMemcpyAsync(velocities4, e->pp_vel + s.first, nb, cudaMemcpyDeviceToHost, e->stream));
        if (accelerations4)
            EN_CK(e, cudaMemcpyAsync(accelerations4, e->pp_acc + s.first, nb, cudaMemcpyDeviceToHost, e->stream));
        return read_status(e);
    }
    // Barnes-Hut state is in key order; ids hold each slot's body index.
    const int *ids = e->bh_ids[e->bh_va] + s.first;
    auto out = [&](const float4 *src, float *dst, bool zero_w, int half) -> int {
        if (!dst) return NBODY_OK;
        float4 *tmp = e->stage + half * s.n;
        EN_CK(e, nbody::bh_unpermute(ids, s.n, src + s.first, tmp, zero_w, e->stream, e->status));
        EN_CK(e, cudaMemcpyAsync(dst, tmp, nb, cudaMemcpyDeviceToHost, e->stream));
        return NBODY_OK;
    };
    rc = out(e->bh_pos[0], positions4, true, 0);
    if (rc == NBODY_OK) rc = out(e->bh_vel[e->bh_va], velocities4, false, 1);
    if (rc == NBODY_OK && accelerations4) {
        EN_CK(e, cudaStreamSynchronize(e->stream));  // stage half 0 is free again
        rc = out(e->bh_acc[e->bh_va], accelerations4, false, 0);
    }
    if (rc == NBODY_OK && masses4) {
        EN_CK(e, cudaStreamSynchronize(e->stream));
        EN_CK(e, nbody::unpack_masses(e->bh_pos[0] + s.first, ids, e->stage + s.n, s.n, e->stream, e->status));
        EN_CK(e, cudaMemcpyAsync(masses4, e->stage + s.n, nb, cudaMemcpyDeviceToHost, e->stream));
    }
    if (rc != NBODY_OK) return rc;
    return read_status(e);
}

int nbody_ensemble_sync(nbody_ensemble *e) {
    if (!e) return NBODY_ERR_ARG;
    DevGuard dg(e->device);
    return read_status(e);
}

int nbody_ensemble_counts(nbody_ensemble *e, int *systems, int64_t *pp_bodies, int64_t *bh_bodies,
                          int *launches_per_step) {
    if (!e) return NBODY_ERR_ARG;
    DevGuard dg(e->device);
    const int rc = relayout(e);
    if (rc != NBODY_OK) return rc;
    int live = 0;
    for (const Sys &s : e->sys) live += s.alive ? 1 : 0;
    if (systems) *systems = live;
    if (pp_bodies) *pp_bodies = e->pp_n;
    if (bh_bodies) *bh_bodies = e->bh_n;
    if (launches_per_step) {
        // direct sum: 1; Barnes-Hut: bbox, keys, histogram + scan + 8 key
        // passes, segment keys + histogram + scan + passes, gather, 7 build
        // kernels (+ the cell walk's child table), the upsweep's, traversal
        int l = e->pp_nitems > 0 ? 1 : 0;
        if (e->bh_n > 0)
            l += 2 + (2 + 8) + (e->tab.systems > 1 ? 3 + e->tab.seg_passes : 0) + 1 + 7 +
                 (e->ws.walk == nbody::kWalkCell ? 1 : 0) + nbody::bh_upsweep_launches(e->bh_n, true) + 1;
        *launches_per_step = l;
    }
    return NBODY_OK;
}

int nbody_ensemble_profile_enable(nbody_ensemble *e, int on) {
    if (!e) return NBODY_ERR_ARG;
    if (on && !e->timer) {
        e->timer = new (std::nothrow) nbody::EventTimer();
        if (!e->timer) return NBODY_ERR_NOMEM;
    } else if (!on && e->timer) {
        DevGuard dg(e->device);
        cudaStreamSynchronize(e->stream);
        cudaStreamSynchronize(e->side);
        delete e->timer;
        e->timer = nullptr;
    }
    return NBODY_OK;
}

int nbody_ensemble_profile_read(nbody_ensemble *e, double *ms, int *launches, int nstages) {
    if (!e || nstages < 0) return NBODY_ERR_ARG;
    for (int k = 0; k < nstages; ++k) {
        if (ms) ms[k] = 0.0;
        if (launches) launches[k] = 0;
    }
    if (!e->timer) return NBODY_OK;
    DevGuard dg(e->device);
    EN_CK(e, e->timer->read(ms, launches, nstages));
    return NBODY_OK;
}

int64_t nbody_ensemble_footprint(int64_t n, int mode) {
    if (n <= 0) return 0;
    const int64_t state = (mode == NBODY_MODE_PP ? 4 : 6) * 16 * n + (mode == NBODY_MODE_BH ? 8 * n : 0);
    if (mode == NBODY_MODE_PP) return state + 64 * 1024;
    const int64_t tables = 4 * n + 8 * n + 16 * ((n + 63) / 64);
    const int64_t work = static_cast<int64_t>(nbody::bh_workspace_bytes(n + n / 4));
    return state + tables + work + 64 * 1024;
}

}  // extern "C"
