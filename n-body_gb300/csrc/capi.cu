// C ABI of the library (declared in include/nbody_gb300.h): solver contexts,
// host-layout and resident-state steps, device-pointer entry points.
//
// A context owns, on one device: the double-buffered pos_mass state, vel and
// acc, a staging area for the reference's host layout, a status word that
// kernels raise on a failed bounded wait or a capacity overflow, the scratch
// memory its kernels need, and a non-blocking stream (replaceable with
// nbody_set_stream).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "bh.h"
#include "diag.h"
#include "init.h"
#include "kernels.h"
#include "nbody_gb300.h"
#include "sort.h"
#include "timer.h"

// What a captured Barnes-Hut step depends on: a replay is valid while all of
// it is unchanged (buffers, parameters, kernel forms, host arrays).
struct GraphKey {
    const void *ws = nullptr;
    int64_t n = 0;
    int va = -1, key_mode = -1, integrator = -1, walk = -1, bodies_per_lane = -1;
    float dt = 0.f, eps2 = 0.f, theta2 = 0.f;
    const void *host[9] = {};
    bool operator==(const GraphKey &o) const {
        if (ws != o.ws || n != o.n || va != o.va || key_mode != o.key_mode || integrator != o.integrator ||
            walk != o.walk || bodies_per_lane != o.bodies_per_lane || dt != o.dt || eps2 != o.eps2 ||
            theta2 != o.theta2)
            return false;
        for (int i = 0; i < 9; ++i)
            if (host[i] != o.host[i]) return false;
        return true;
    }
};

struct StepGraph {
    cudaGraphExec_t exec = nullptr;
    GraphKey key;
};

struct nbody_ctx {
    int device = 0;
    int mode = NBODY_MODE_PP;
    int64_t n = 0;
    float dt = 0.f, eps2 = 0.f, theta2 = 0.25f;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    float4 *pos[2] = {nullptr, nullptr};
    int cur = 0;
    float4 *vel = nullptr;
    float4 *acc = nullptr;
    float4 *stage = nullptr;  // 2n float4: reference-layout positions, then masses
    int *status = nullptr;    // device status word
    int *status_host = nullptr;  // page-locked copy of it, read after a stream sync
    void *scratch = nullptr;
    size_t scratch_bytes = 0;
    bool uploaded = false;
    nbody::EventTimer *timer = nullptr;  // non-null while profiling is enabled
    std::string last_error;

    // Barnes-Hut resident state, kept in the order of the last sort: pos[bh_pos],
    // vel2[bh_va] / acc2[bh_va] and ids[bh_va] (ids[k] = caller's body index).
    float4 *vel2[2] = {nullptr, nullptr};
    float4 *acc2[2] = {nullptr, nullptr};
    int *ids[2] = {nullptr, nullptr};
    int bh_pos = 0, bh_va = 0;
    int key_mode = NBODY_KEYS_OCTREE;
    int integrator = NBODY_INTEGRATOR_CPU;
    bool ids_valid = false;  // false until the first step after an upload
    // Barnes-Hut workspace (keys, sort scratch, tree), grown on demand.
    void *ws_mem = nullptr;
    size_t ws_bytes = 0;
    nbody::BHWorkspace ws;
    // Buffers for the device-pointer Barnes-Hut entry point.
    float4 *dev_pos = nullptr;
    int *dev_ids = nullptr;
    int64_t dev_cap = 0;
    // Diagnostics: reduction scratch, 8 doubles of output, per-body potential.
    void *diag_mem = nullptr;
    float *diag_phi = nullptr;
    // Side stream and events of the overlapped host step (made on first use).
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    // Barnes-Hut steps replayed as CUDA graphs: the resident step by the
    // parity of its velocity buffers, and the host step of nbody_update_host.
    StepGraph graph_step[2], graph_host;
    bool graphs_off = false;  // capture failed once (or NBODY_GRAPHS=0)
};

namespace {

struct DeviceGuard {
    int prev = -1;
    bool ok = true;
    explicit DeviceGuard(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != dev) ok = cudaSetDevice(dev) == cudaSuccess;
    }
    ~DeviceGuard() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

int fail(nbody_ctx *ctx, cudaError_t e) {
    if (ctx) ctx->last_error = cudaGetErrorString(e);
    cudaGetLastError();  // clear a non-sticky error
    return e == cudaErrorMemoryAllocation ? NBODY_ERR_NOMEM : NBODY_ERR_CUDA;
}

#define NB_CK(ctx, expr)                              \
    do {                                              \
        cudaError_t e_ = (expr);                      \
        if (e_ != cudaSuccess) return fail(ctx, e_);  \
    } while (0)

bool aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

int ensure_scratch(nbody_ctx *ctx, size_t bytes) {
    if (bytes <= ctx->scratch_bytes) return NBODY_OK;
    if (ctx->scratch) {
        NB_CK(ctx, cudaStreamSynchronize(ctx->stream));
        cudaFree(ctx->scratch);
        ctx->scratch = nullptr;
        ctx->scratch_bytes = 0;
    }
    NB_CK(ctx, cudaMalloc(&ctx->scratch, bytes));
    NB_CK(ctx, cudaMemsetAsync(ctx->scratch, 0, bytes, ctx->stream));
    ctx->scratch_bytes = bytes;
    return NBODY_OK;
}

int read_status(nbody_ctx *ctx) {
    int h = NBODY_OK;
    if (ctx->status_host) {
        NB_CK(ctx, cudaMemcpyAsync(ctx->status_host, ctx->status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        NB_CK(ctx, cudaMemsetAsync(ctx->status, 0, sizeof(int), ctx->stream));
        NB_CK(ctx, cudaStreamSynchronize(ctx->stream));
        h = *ctx->status_host;
    } else {
        NB_CK(ctx, cudaMemcpyAsync(&h, ctx->status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        NB_CK(ctx, cudaMemsetAsync(ctx->status, 0, sizeof(int), ctx->stream));
        NB_CK(ctx, cudaStreamSynchronize(ctx->stream));
    }
    if (h != NBODY_OK && ctx->scratch) {
        // A kernel gave up part-way: its arrival counters may be left non-zero.
        NB_CK(ctx, cudaMemsetAsync(ctx->scratch, 0, ctx->scratch_bytes, ctx->stream));
        NB_CK(ctx, cudaStreamSynchronize(ctx->stream));
    }
    return h;
}

int pp_steps(nbody_ctx *ctx, int steps) {
    const nbody::PPPlan plan = nbody::pp_plan(ctx->n, ctx->device);
    int rc = ensure_scratch(ctx, plan.partial_bytes);
    if (rc != NBODY_OK) return rc;
    for (int s = 0; s < steps; ++s) {
        nbody::Integrate g;
        g.pos_out = ctx->pos[ctx->cur ^ 1];
        g.vel = ctx->vel;
        g.acc = ctx->acc;
        g.dt = ctx->dt;
        g.euler = ctx->integrator == NBODY_INTEGRATOR_GPU_EULER;
        NB_CK(ctx, nbody::pp_launch(plan, ctx->pos[ctx->cur], ctx->n, ctx->eps2, g, ctx->scratch, ctx->stream,
                                    ctx->status, ctx->timer));
        ctx->cur ^= 1;
    }
    return NBODY_OK;
}

int ensure_dev_buffers(nbody_ctx *ctx, int64_t n) {
    if (ctx->dev_cap >= n) return NBODY_OK;
    NB_CK(ctx, cudaStreamSynchronize(ctx->stream));
    cudaFree(ctx->dev_pos);
    cudaFree(ctx->dev_ids);
    ctx->dev_pos = nullptr;
    ctx->dev_ids = nullptr;
    ctx->dev_cap = 0;
    NB_CK(ctx, cudaMalloc(&ctx->dev_pos, sizeof(float4) * static_cast<size_t>(n)));
    NB_CK(ctx, cudaMalloc(&ctx->dev_ids, sizeof(int) * static_cast<size_t>(n)));
    ctx->dev_cap = n;
    return NBODY_OK;
}

int ensure_workspace(nbody_ctx *ctx, int64_t n) {
    if (ctx->ws_mem && ctx->ws.n >= n) return NBODY_OK;
    const size_t bytes = nbody::bh_workspace_bytes(n);
    if (ctx->ws_mem) {
        NB_CK(ctx, cudaStreamSynchronize(ctx->stream));
        cudaFree(ctx->ws_mem);
        ctx->ws_mem = nullptr;
    }
    NB_CK(ctx, cudaMalloc(&ctx->ws_mem, bytes));
    NB_CK(ctx, cudaMemsetAsync(ctx->ws_mem, 0, bytes, ctx->stream));
    ctx->ws_bytes = bytes;
    const bool counting = ctx->ws.counters != nullptr;
    nbody::bh_workspace_layout(n, ctx->ws_mem, &ctx->ws);
    if (counting) ctx->ws.counters = ctx->ws.counter_mem;
    // Two bodies per lane measured faster at N = 2^20 (Plummer): 62M instead
    // of 110M warp record visits per step, traversal 5.95 ms instead of 7.12 ms.
    ctx->ws.bodies_per_lane = 2;
    if (const char *e = std::getenv("NBODY_BH_BODIES_PER_LANE")) {
        if (std::atoi(e) == 1) ctx->ws.bodies_per_lane = 1;
    }
    ctx->ws.walk = nbody::bh_walk_form();
    return NBODY_OK;
}

// One Barnes-Hut step on the resident state (see nbody_ctx for the layout).
// join: when set, the step waits for it before its gather and first merges
// the masses in `masses4` (device, reference layout) into the positions,
// which were copied in with w = 0 (the overlapped host step).
int bh_step(nbody_ctx *ctx, cudaEvent_t join = nullptr, const float4 *masses4 = nullptr,
            const nbody::HostOut &host = nbody::HostOut{}) {
    nbody::BHWorkspace &w = ctx->ws;
    const int64_t n = ctx->n;
    float4 *P = ctx->pos[ctx->bh_pos], *Po = ctx->pos[ctx->bh_pos ^ 1];
    float4 *V = ctx->vel2[ctx->bh_va], *Vo = ctx->vel2[ctx->bh_va ^ 1];
    float4 *A = ctx->acc2[ctx->bh_va], *Ao = ctx->acc2[ctx->bh_va ^ 1];
    const int *I = ctx->ids_valid ? ctx->ids[ctx->bh_va] : nullptr;
    int *Io = ctx->ids[ctx->bh_va ^ 1];
    nbody::StageTimer *tm = ctx->timer;
    NB_CK(ctx, nbody::bh_bbox(P, n, w, ctx->stream, tm));
    NB_CK(ctx, nbody::bh_keys(P, n, w, ctx->key_mode, ctx->stream, tm));
    NB_CK(ctx, nbody::bh_sort(n, w, ctx->stream, ctx->status, tm));
    if (join) {
        NB_CK(ctx, cudaStreamWaitEvent(ctx->stream, join, 0));
        NB_CK(ctx, nbody::merge_masses(P, masses4, n, ctx->stream));
    }
    NB_CK(ctx, nbody::bh_gather(n, w, P, V, A, I, Po, Vo, Ao, Io, ctx->stream, ctx->status, tm));
    NB_CK(ctx, nbody::bh_build(Po, n, w, ctx->stream, ctx->status, tm));
    // New positions go to the buffer the gather just read from.
    NB_CK(ctx, nbody::bh_traverse(Po, n, w, ctx->eps2, ctx->theta2, ctx->dt, P, Vo, Ao, nullptr, host.pos ? Io : nullptr,
                                  ctx->integrator == NBODY_INTEGRATOR_GPU_EULER, ctx->stream, tm, host));
    ctx->bh_va ^= 1;
    ctx->ids_valid = true;
    return NBODY_OK;
}

GraphKey graph_key(const nbody_ctx *ctx) {
    GraphKey k;
    k.ws = ctx->ws_mem;
    k.n = ctx->n;
    k.va = ctx->bh_va;
    k.key_mode = ctx->key_mode;
    k.integrator = ctx->integrator;
    k.walk = ctx->ws.walk;
    k.bodies_per_lane = ctx->ws.bodies_per_lane;
    k.dt = ctx->dt;
    k.eps2 = ctx->eps2;
    k.theta2 = ctx->theta2;
    k.host[8] = reinterpret_cast<const void *>(static_cast<uintptr_t>(ctx->bh_pos + 1));
    return k;
}

// Whether steps may run as graphs: not while per-stage timing or pair
// counting is on (their launches differ), nor after a capture failed.
bool graphs_usable(nbody_ctx *ctx) {
    if (ctx->graphs_off || ctx->timer || ctx->ws.counters) return false;
    const char *e = std::getenv("NBODY_GRAPHS");  // "0": launch every kernel directly
    return !(e && std::strcmp(e, "0") == 0);
}

void drop_graph(StepGraph &g) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    g.exec = nullptr;
}

// Runs `body` (stream work on ctx->stream, possibly forking to ctx->side and
// joining back) as the graph cached in g, capturing it first when g is empty
// or was captured under another key. The host-side state that body changes
// (buffer parities, id validity) is put back after a capture, so the caller
// applies it once per replay. Returns NBODY_OK, or an error before anything
// was launched, with *replayed = false when the caller should run body itself
// (capture unavailable).
template <class Body>
int replay(nbody_ctx *ctx, StepGraph &g, const GraphKey &key, Body &&body, bool *replayed) {
    *replayed = false;
    if (!(g.exec && g.key == key)) {
        drop_graph(g);
        const int va = ctx->bh_va, pos = ctx->bh_pos, cur = ctx->cur;
        const bool iv = ctx->ids_valid, up = ctx->uploaded;
        if (cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            cudaGetLastError();
            ctx->graphs_off = true;
            return NBODY_OK;
        }
        const int rc = body();
        cudaGraph_t graph = nullptr;
        const cudaError_t e = cudaStreamEndCapture(ctx->stream, &graph);
        ctx->bh_va = va;
        ctx->bh_pos = pos;
        ctx->cur = cur;
        ctx->ids_valid = iv;
        ctx->uploaded = up;
        if (rc != NBODY_OK || e != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            cudaGetLastError();
            ctx->graphs_off = true;  // run this and later steps directly
            return NBODY_OK;
        }
        const cudaError_t ei = cudaGraphInstantiate(&g.exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ei != cudaSuccess) {
            g.exec = nullptr;
            cudaGetLastError();
            ctx->graphs_off = true;
            return NBODY_OK;
        }
        g.key = key;
    }
    NB_CK(ctx, cudaGraphLaunch(g.exec, ctx->stream));
    *replayed = true;
    return NBODY_OK;
}

// Steps on the resident state. From the second step after an upload (ids
// valid, the same launches every step) each step is one graph launch, one
// graph per parity of the velocity buffers: one host call instead of some
// thirty, so a slow or busy host no longer leaves gaps between the step's
// short kernels.
int bh_steps(nbody_ctx *ctx, int steps) {
    int rc = ensure_workspace(ctx, ctx->n);
    for (int s = 0; rc == NBODY_OK && s < steps; ++s) {
        if (ctx->ids_valid && graphs_usable(ctx)) {
            bool replayed = false;
            rc = replay(ctx, ctx->graph_step[ctx->bh_va], graph_key(ctx), [&] { return bh_step(ctx); }, &replayed);
            if (rc != NBODY_OK) break;
            if (replayed) {
                ctx->bh_va ^= 1;
                ctx->ids_valid = true;
                continue;
            }
        }
        rc = bh_step(ctx);
    }
    return rc;
}

}  // namespace

extern "C" {

const char *nbody_status_string(int status) {
    switch (status) {
        case NBODY_OK: return "ok";
        case NBODY_ERR_ARG: return "invalid argument";
        case NBODY_ERR_CUDA: return "CUDA error";
        case NBODY_ERR_NOMEM: return "out of memory";
        case NBODY_ERR_CAPACITY: return "capacity exceeded";
        case NBODY_ERR_TIMEOUT: return "device wait timed out";
        case NBODY_ERR_STATE: return "call out of order";
        default: return "unknown status";
    }
}

const char *nbody_last_error(const nbody_ctx *ctx) { return ctx ? ctx->last_error.c_str() : ""; }

int nbody_create(nbody_ctx **out, int device, int mode, int64_t n, float dt, float eps2, float theta2) {
    if (!out) return NBODY_ERR_ARG;
    *out = nullptr;
    if (n <= 0 || device < 0 || !(eps2 >= 0.f) || (mode != NBODY_MODE_PP && mode != NBODY_MODE_BH))
        return NBODY_ERR_ARG;
    nbody_ctx *ctx = new (std::nothrow) nbody_ctx();
    if (!ctx) return NBODY_ERR_NOMEM;
    ctx->device = device;
    ctx->mode = mode;
    ctx->n = n;
    ctx->dt = dt;
    ctx->eps2 = eps2;
    ctx->theta2 = theta2 > 0.f ? theta2 : 0.25f;
    DeviceGuard dg(device);
    int rc = NBODY_OK;
    auto alloc = [&](void **p, size_t bytes) {
        if (rc != NBODY_OK) return;
        cudaError_t e = cudaMalloc(p, bytes);
        if (e != cudaSuccess) rc = fail(ctx, e);
    };
    if (!dg.ok) rc = NBODY_ERR_CUDA;
    const size_t b4 = static_cast<size_t>(n) * sizeof(float4);
    alloc(reinterpret_cast<void **>(&ctx->pos[0]), b4);
    alloc(reinterpret_cast<void **>(&ctx->pos[1]), b4);
    alloc(reinterpret_cast<void **>(&ctx->vel), b4);
    alloc(reinterpret_cast<void **>(&ctx->acc), b4);
    alloc(reinterpret_cast<void **>(&ctx->stage), 2 * b4);
    alloc(reinterpret_cast<void **>(&ctx->status), sizeof(int));
    if (rc == NBODY_OK && cudaMallocHost(reinterpret_cast<void **>(&ctx->status_host), sizeof(int)) != cudaSuccess) {
        cudaGetLastError();  // the status is then read into pageable memory
        ctx->status_host = nullptr;
    }
    if (mode == NBODY_MODE_BH) {
        ctx->vel2[0] = ctx->vel;
        ctx->acc2[0] = ctx->acc;
        alloc(reinterpret_cast<void **>(&ctx->vel2[1]), b4);
        alloc(reinterpret_cast<void **>(&ctx->acc2[1]), b4);
        alloc(reinterpret_cast<void **>(&ctx->ids[0]), sizeof(int) * static_cast<size_t>(n));
        alloc(reinterpret_cast<void **>(&ctx->ids[1]), sizeof(int) * static_cast<size_t>(n));
    }
    if (rc == NBODY_OK) {
        cudaError_t e = cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) rc = fail(ctx, e);
        ctx->stream = ctx->own_stream;
    }
    if (rc == NBODY_OK && mode == NBODY_MODE_BH) rc = ensure_workspace(ctx, n);
    if (rc == NBODY_OK) {
        cudaError_t e = cudaMemsetAsync(ctx->status, 0, sizeof(int), ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) rc = fail(ctx, e);
    }
    if (rc != NBODY_OK) {
        nbody_destroy(ctx);
        return rc;
    }
    *out = ctx;
    return NBODY_OK;
}

int nbody_destroy(nbody_ctx *ctx) {
    if (!ctx) return NBODY_ERR_ARG;
    {
        DeviceGuard dg(ctx->device);
        if (ctx->stream) cudaStreamSynchronize(ctx->stream);
        cudaFree(ctx->pos[0]);
        cudaFree(ctx->pos[1]);
        cudaFree(ctx->vel);
        cudaFree(ctx->acc);
        cudaFree(ctx->stage);
        cudaFree(ctx->status);
        if (ctx->status_host) cudaFreeHost(ctx->status_host);
        cudaFree(ctx->scratch);
        cudaFree(ctx->vel2[1]);
        cudaFree(ctx->acc2[1]);
        cudaFree(ctx->ids[0]);
        cudaFree(ctx->ids[1]);
        cudaFree(ctx->ws_mem);
        cudaFree(ctx->dev_pos);
        cudaFree(ctx->dev_ids);
        cudaFree(ctx->diag_mem);
        cudaFree(ctx->diag_phi);
        delete ctx->timer;
        drop_graph(ctx->graph_step[0]);
        drop_graph(ctx->graph_step[1]);
        drop_graph(ctx->graph_host);
        if (ctx->side) cudaStreamDestroy(ctx->side);
        if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
        if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
        if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
    }
    delete ctx;
    return NBODY_OK;
}

int nbody_set_stream(nbody_ctx *ctx, void *stream) {
    if (!ctx) return NBODY_ERR_ARG;
    ctx->stream = stream ? static_cast<cudaStream_t>(stream) : ctx->own_stream;
    return NBODY_OK;
}

float nbody_get_squared_softening(const nbody_ctx *ctx) { return ctx ? ctx->eps2 : 0.f; }

int nbody_upload(nbody_ctx *ctx, const float *positions4, const float *velocities4, const float *accelerations4,
                 const float *masses4) {
    if (!ctx || !positions4 || !masses4) return NBODY_ERR_ARG;
    DeviceGuard dg(ctx->device);
    const size_t b4 = static_cast<size_t>(ctx->n) * sizeof(float4);
    // Page-locked host buffers are read in place by one kernel; otherwise one
    // copy per array into the staging area, then the pack kernel.
    const float4 *mp = nbody::host_mapped(positions4, b4, ctx->device);
    const float4 *mm = nbody::host_mapped(masses4, b4, ctx->device);
    const float4 *mv = velocities4 ? nbody::host_mapped(velocities4, b4, ctx->device) : nullptr;
    const float4 *ma = accelerations4 ? nbody::host_mapped(accelerations4, b4, ctx->device) : nullptr;
    if (mp && mm && (!velocities4 || mv) && (!accelerations4 || ma)) {
        NB_CK(ctx, nbody::host_gather(mp, mm, mv, ma, ctx->pos[0], ctx->vel, ctx->acc, ctx->n, ctx->stream));
    } else {
        NB_CK(ctx, cudaMemcpyAsync(ctx->stage, positions4, b4, cudaMemcpyHostToDevice, ctx->stream));
        NB_CK(ctx, cudaMemcpyAsync(ctx->stage + ctx->n, masses4, b4, cudaMemcpyHostToDevice, ctx->stream));
        if (velocities4)
            NB_CK(ctx, cudaMemcpyAsync(ctx->vel, velocities4, b4, cudaMemcpyHostToDevice, ctx->stream));
        else
            NB_CK(ctx, cudaMemsetAsync(ctx->vel, 0, b4, ctx->stream));
        if (accelerations4)
            NB_CK(ctx, cudaMemcpyAsync(ctx->acc, accelerations4, b4, cudaMemcpyHostToDevice, ctx->stream));
        else
            NB_CK(ctx, cudaMemsetAsync(ctx->acc, 0, b4, ctx->stream));
        NB_CK(ctx, nbody::pack_state(ctx->stage, ctx->stage + ctx->n, ctx->pos[0], ctx->n, ctx->stream));
    }
    ctx->cur = 0;
    ctx->bh_pos = 0;
    ctx->bh_va = 0;
    ctx->ids_valid = false;
    ctx->uploaded = true;
    return NBODY_OK;
}

int nbody_step(nbody_ctx *ctx, int steps) {
    if (!ctx || steps < 0) return NBODY_ERR_ARG;
    if (!ctx->uploaded) return NBODY_ERR_STATE;
    DeviceGuard dg(ctx->device);
    if (ctx->mode == NBODY_MODE_PP) return pp_steps(ctx, steps);
    return bh_steps(ctx, steps);
}

int nbody_download(nbody_ctx *ctx, float *positions4, float *velocities4, float *accelerations4, float *forces4) {
    if (!ctx) return NBODY_ERR_ARG;
    if (!ctx->uploaded) return NBODY_ERR_STATE;
    DeviceGuard dg(ctx->device);
    const size_t b4 = static_cast<size_t>(ctx->n) * sizeof(float4);
    const int64_t n = ctx->n;
    {
        // Page-locked host buffers are written in place by one kernel, in the
        // caller's order (through the inverse of the sorted order, built in the
        // staging area, when the state is sorted).
        const int dev = ctx->device;
        float4 *mp = positions4 ? nbody::host_mapped(positions4, b4, dev) : nullptr;
        float4 *mv = velocities4 ? nbody::host_mapped(velocities4, b4, dev) : nullptr;
        float4 *ma = accelerations4 ? nbody::host_mapped(accelerations4, b4, dev) : nullptr;
        float4 *mf = forces4 ? nbody::host_mapped(forces4, b4, dev) : nullptr;
        if ((!positions4 || mp) && (!velocities4 || mv) && (!accelerations4 || ma) && (!forces4 || mf)) {
            const bool bh = ctx->mode == NBODY_MODE_BH;
            const int *ids = (bh && ctx->ids_valid) ? ctx->ids[ctx->bh_va] : nullptr;
            if (mp || mv || ma || mf)
                NB_CK(ctx, nbody::host_scatter(bh ? ctx->pos[ctx->bh_pos] : ctx->pos[ctx->cur],
                                               bh ? ctx->vel2[ctx->bh_va] : ctx->vel,
                                               bh ? ctx->acc2[ctx->bh_va] : ctx->acc, ids,
                                               reinterpret_cast<int *>(ctx->stage), mp, mv, ma, mf, nullptr, n,
                                               ctx->stream, ctx->status));
            return read_status(ctx);
        }
    }
    if (ctx->mode == NBODY_MODE_BH && ctx->ids_valid) {
        // Resident state is in the last sort's order: scatter back by id.
        const int *ids = ctx->ids[ctx->bh_va];
        float4 *half[2] = {ctx->stage, ctx->stage + n};
        int h = 0;
        auto out = [&](const float4 *src, float *dst, bool zero_w) -> int {
            if (!dst) return NBODY_OK;
            NB_CK(ctx, nbody::bh_unpermute(ids, n, src, half[h], zero_w, ctx->stream, ctx->status));
            NB_CK(ctx, cudaMemcpyAsync(dst, half[h], b4, cudaMemcpyDeviceToHost, ctx->stream));
            h ^= 1;
            return NBODY_OK;
        };
        int rc = out(ctx->pos[ctx->bh_pos], positions4, true);
        if (rc == NBODY_OK) rc = out(ctx->vel2[ctx->bh_va], velocities4, false);
        if (rc == NBODY_OK) rc = out(ctx->acc2[ctx->bh_va], accelerations4, false);
        if (rc == NBODY_OK) rc = out(ctx->acc2[ctx->bh_va], forces4, false);
        if (rc != NBODY_OK) return rc;
        return read_status(ctx);
    }
    float4 *pos = ctx->mode == NBODY_MODE_BH ? ctx->pos[ctx->bh_pos] : ctx->pos[ctx->cur];
    float4 *vel = ctx->mode == NBODY_MODE_BH ? ctx->vel2[ctx->bh_va] : ctx->vel;
    float4 *acc = ctx->mode == NBODY_MODE_BH ? ctx->acc2[ctx->bh_va] : ctx->acc;
    if (positions4) {
        NB_CK(ctx, nbody::unpack_positions(pos, ctx->stage, ctx->n, ctx->stream));
        NB_CK(ctx, cudaMemcpyAsync(positions4, ctx->stage, b4, cudaMemcpyDeviceToHost, ctx->stream));
    }
    if (velocities4) NB_CK(ctx, cudaMemcpyAsync(velocities4, vel, b4, cudaMemcpyDeviceToHost, ctx->stream));
    if (accelerations4) NB_CK(ctx, cudaMemcpyAsync(accelerations4, acc, b4, cudaMemcpyDeviceToHost, ctx->stream));
    if (forces4) NB_CK(ctx, cudaMemcpyAsync(forces4, acc, b4, cudaMemcpyDeviceToHost, ctx->stream));
    return read_status(ctx);
}

int nbody_download_masses(nbody_ctx *ctx, float *masses4) {
    if (!ctx || !masses4) return NBODY_ERR_ARG;
    if (!ctx->uploaded) return NBODY_ERR_STATE;
    DeviceGuard dg(ctx->device);
    const bool bh = ctx->mode == NBODY_MODE_BH;
    const float4 *pos = bh ? ctx->pos[ctx->bh_pos] : ctx->pos[ctx->cur];
    const int *ids = (bh && ctx->ids_valid) ? ctx->ids[ctx->bh_va] : nullptr;
    NB_CK(ctx, nbody::unpack_masses(pos, ids, ctx->stage, ctx->n, ctx->stream, ctx->status));
    NB_CK(ctx, cudaMemcpyAsync(masses4, ctx->stage, static_cast<size_t>(ctx->n) * sizeof(float4),
                               cudaMemcpyDeviceToHost, ctx->stream));
    return read_status(ctx);
}

int nbody_sync(nbody_ctx *ctx) {
    if (!ctx) return NBODY_ERR_ARG;
    DeviceGuard dg(ctx->device);
    return read_status(ctx);
}

int nbody_host_in_place(const void *p, int64_t bytes, int device) {
    if (!p || bytes <= 0 || device < 0) return NBODY_ERR_ARG;
    DeviceGuard dg(device);
    return nbody::host_mapped(p, static_cast<size_t>(bytes), device) ? 1 : 0;
}

namespace {

// nbody_update_host for Barnes-Hut with page-locked host arrays: positions come
// in first by a DMA copy (the reference layout's w = 0), velocities,
// accelerations and masses by DMA copies on a side stream while the first
// step's box, keys and sort run on the SMs; the step merges the masses into
// the positions just before its gather, the first use of any of them. With
// `host` set, the last step's walk writes the new state into the caller's
// arrays as each body finishes (over the host link while the walk runs; the
// inputs were copied in before). Same values as nbody_upload + nbody_step +
// nbody_download.
int bh_update_overlapped(nbody_ctx *ctx, const float *positions4, const float *velocities4,
                         const float *accelerations4, const float *masses4, int steps,
                         const nbody::HostOut &host = nbody::HostOut{}) {
    DeviceGuard dg(ctx->device);
    int rc = ensure_workspace(ctx, ctx->n);
    if (rc != NBODY_OK) return rc;
    if (!ctx->side) {
        NB_CK(ctx, cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking));
        NB_CK(ctx, cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming));
        NB_CK(ctx, cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming));
    }
    const size_t b4 = static_cast<size_t>(ctx->n) * sizeof(float4);
    const nbody::HostOut first_out = steps == 1 ? host : nbody::HostOut{};
    // The copies in and the first step: the same launches on every call with
    // the same arrays, so they replay as one graph.
    auto first = [&]() -> int {
        NB_CK(ctx, cudaEventRecord(ctx->ev_fork, ctx->stream));
        NB_CK(ctx, cudaMemcpyAsync(ctx->pos[0], positions4, b4, cudaMemcpyHostToDevice, ctx->stream));
        NB_CK(ctx, cudaStreamWaitEvent(ctx->side, ctx->ev_fork, 0));
        NB_CK(ctx, cudaMemcpyAsync(ctx->vel, velocities4, b4, cudaMemcpyHostToDevice, ctx->side));
        NB_CK(ctx, cudaMemcpyAsync(ctx->acc, accelerations4, b4, cudaMemcpyHostToDevice, ctx->side));
        NB_CK(ctx, cudaMemcpyAsync(ctx->stage, masses4, b4, cudaMemcpyHostToDevice, ctx->side));
        NB_CK(ctx, cudaEventRecord(ctx->ev_join, ctx->side));
        ctx->cur = 0;
        ctx->bh_pos = 0;
        ctx->bh_va = 0;
        ctx->ids_valid = false;
        ctx->uploaded = true;
        return bh_step(ctx, ctx->ev_join, ctx->stage, first_out);
    };
    bool replayed = false;
    if (graphs_usable(ctx)) {
        NB_CK(ctx, nbody::sort_prepare(ctx->device));  // launch attributes before any capture
        GraphKey key = graph_key(ctx);
        key.va = 0;
        const void *arrays[9] = {positions4, velocities4, accelerations4, masses4, first_out.pos, first_out.vel,
                                 first_out.acc, first_out.force, nullptr};
        for (int i = 0; i < 9; ++i) key.host[i] = arrays[i];
        rc = replay(ctx, ctx->graph_host, key, first, &replayed);
        if (rc != NBODY_OK) return rc;
    }
    if (replayed) {  // the state the first step leaves
        ctx->cur = 0;
        ctx->bh_pos = 0;
        ctx->bh_va = 1;
        ctx->ids_valid = true;
        ctx->uploaded = true;
    } else {
        rc = first();
    }
    if (rc == NBODY_OK && steps > 1) rc = bh_steps(ctx, steps - 2);
    if (rc == NBODY_OK && steps > 1) rc = bh_step(ctx, nullptr, nullptr, host);
    return rc;
}

// nbody_update_host for one direct-sum step with page-locked arrays: the
// gather kernel in, the step and the scatter kernel out replay as one graph
// (the same launches on every call with the same arrays). Returns false, with
// nothing launched, when the call does not qualify; else *rc is the call's
// status.
bool pp_update_graphed(nbody_ctx *ctx, const float *positions4, float *velocities4, float *accelerations4,
                       const float *masses4, float *forces4, int *rc) {
    DeviceGuard dg(ctx->device);
    if (!graphs_usable(ctx)) return false;
    const size_t b4 = static_cast<size_t>(ctx->n) * sizeof(float4);
    const int dev = ctx->device;
    float4 *mp = nbody::host_mapped(positions4, b4, dev), *mv = nbody::host_mapped(velocities4, b4, dev),
           *ma = nbody::host_mapped(accelerations4, b4, dev), *mm = nbody::host_mapped(masses4, b4, dev);
    float4 *mf = forces4 ? nbody::host_mapped(forces4, b4, dev) : nullptr;
    if (!(mp && mv && ma && mm && (!forces4 || mf))) return false;
    const nbody::PPPlan plan = nbody::pp_plan(ctx->n, ctx->device);
    *rc = ensure_scratch(ctx, plan.partial_bytes);  // allocation stays outside the capture
    if (*rc != NBODY_OK) return true;
    auto body = [&]() -> int {
        NB_CK(ctx, nbody::host_gather(mp, mm, mv, ma, ctx->pos[0], ctx->vel, ctx->acc, ctx->n, ctx->stream));
        nbody::Integrate g;
        g.pos_out = ctx->pos[1];
        g.vel = ctx->vel;
        g.acc = ctx->acc;
        g.dt = ctx->dt;
        g.euler = ctx->integrator == NBODY_INTEGRATOR_GPU_EULER;
        NB_CK(ctx, nbody::pp_launch(plan, ctx->pos[0], ctx->n, ctx->eps2, g, ctx->scratch, ctx->stream, ctx->status,
                                    nullptr));
        NB_CK(ctx, nbody::host_scatter(ctx->pos[1], ctx->vel, ctx->acc, nullptr, nullptr, mp, mv, ma, mf, nullptr,
                                       ctx->n, ctx->stream, ctx->status));
        return NBODY_OK;
    };
    GraphKey key = graph_key(ctx);
    key.ws = ctx->scratch;
    const void *arrays[9] = {mp, mv, ma, mm, mf, nullptr, nullptr, nullptr, nullptr};
    for (int i = 0; i < 9; ++i) key.host[i] = arrays[i];
    bool replayed = false;
    *rc = replay(ctx, ctx->graph_host, key, body, &replayed);
    if (*rc != NBODY_OK) return true;
    if (!replayed) return false;  // capture unavailable: the caller's path runs the call
    ctx->cur = 1;  // the step's new state is in pos[1]
    ctx->bh_pos = 0;
    ctx->bh_va = 0;
    ctx->ids_valid = false;
    ctx->uploaded = true;
    *rc = read_status(ctx);
    return true;
}

}  // namespace

int nbody_update_host(nbody_ctx *ctx, float *positions4, float *velocities4, float *accelerations4,
                      const float *masses4, float *forces4, int steps) {
    if (!ctx || !positions4 || !velocities4 || !accelerations4 || !masses4 || steps < 0) return NBODY_ERR_ARG;
    if (ctx->mode == NBODY_MODE_PP && steps == 1) {
        int rc = NBODY_OK;
        if (pp_update_graphed(ctx, positions4, velocities4, accelerations4, masses4, forces4, &rc)) return rc;
    }
    if (ctx->mode == NBODY_MODE_BH && steps >= 1) {
        const size_t b4 = static_cast<size_t>(ctx->n) * sizeof(float4);
        const int dev = ctx->device;
        DeviceGuard dg(dev);
        float4 *mp = nbody::host_mapped(positions4, b4, dev), *mv = nbody::host_mapped(velocities4, b4, dev),
               *ma = nbody::host_mapped(accelerations4, b4, dev);
        float4 *mf = forces4 ? nbody::host_mapped(forces4, b4, dev) : nullptr;
        if (mp && mv && ma && nbody::host_mapped(masses4, b4, dev)) {
            int rc = ensure_workspace(ctx, ctx->n);
            if (rc != NBODY_OK) return rc;
            if (nbody::bh_walk_writes_host(ctx->ws) && (!forces4 || mf)) {
                nbody::HostOut host;
                host.pos = mp;
                host.vel = mv;
                host.acc = ma;
                host.force = mf;
                rc = bh_update_overlapped(ctx, positions4, velocities4, accelerations4, masses4, steps, host);
                return rc == NBODY_OK ? read_status(ctx) : rc;
            }
            rc = bh_update_overlapped(ctx, positions4, velocities4, accelerations4, masses4, steps);
            if (rc == NBODY_OK) rc = nbody_download(ctx, positions4, velocities4, accelerations4, forces4);
            return rc;
        }
    }
    int rc = nbody_upload(ctx, positions4, velocities4, accelerations4, masses4);
    if (rc == NBODY_OK) rc = nbody_step(ctx, steps);
    if (rc == NBODY_OK) rc = nbody_download(ctx, positions4, velocities4, accelerations4, forces4);
    return rc;
}

int nbody_device_state(nbody_ctx *ctx, void **pos_mass4, void **vel4, void **acc4) {
    if (!ctx) return NBODY_ERR_ARG;
    const bool bh = ctx->mode == NBODY_MODE_BH;
    if (pos_mass4) *pos_mass4 = bh ? ctx->pos[ctx->bh_pos] : ctx->pos[ctx->cur];
    if (vel4) *vel4 = bh ? ctx->vel2[ctx->bh_va] : ctx->vel;
    if (acc4) *acc4 = bh ? ctx->acc2[ctx->bh_va] : ctx->acc;
    return NBODY_OK;
}

int nbody_device_order(nbody_ctx *ctx, void **ids) {
    if (!ctx || !ids) return NBODY_ERR_ARG;
    *ids = (ctx->mode == NBODY_MODE_BH && ctx->ids_valid) ? static_cast<void *>(ctx->ids[ctx->bh_va]) : nullptr;
    return NBODY_OK;
}

int nbody_bh_keys_device(nbody_ctx *ctx, const void *pos_mass4, int64_t n, void *keys_out, void *box_out) {
    if (!ctx || !pos_mass4 || n <= 0 || !aligned16(pos_mass4)) return NBODY_ERR_ARG;
    DeviceGuard dg(ctx->device);
    int rc = ensure_workspace(ctx, n);
    if (rc != NBODY_OK) return rc;
    nbody::BHWorkspace &w = ctx->ws;
    const float4 *p = static_cast<const float4 *>(pos_mass4);
    NB_CK(ctx, nbody::bh_bbox(p, n, w, ctx->stream, ctx->timer));
    NB_CK(ctx, nbody::bh_keys(p, n, w, ctx->key_mode, ctx->stream, ctx->timer));
    if (keys_out)
        NB_CK(ctx, cudaMemcpyAsync(keys_out, w.keys[0], sizeof(uint64_t) * static_cast<size_t>(n),
                                   cudaMemcpyDeviceToDevice, ctx->stream));
    if (box_out) NB_CK(ctx, cudaMemcpyAsync(box_out, w.box, sizeof(float) * 6, cudaMemcpyDeviceToDevice, ctx->stream));
    return NBODY_OK;
}

int nbody_sort_pairs_device(nbody_ctx *ctx, void *keys, void *vals, int64_t n) {
    if (!ctx || !keys || !vals || n < 0) return NBODY_ERR_ARG;
    if (n <= 1) return NBODY_OK;
    DeviceGuard dg(ctx->device);
    int rc = ensure_workspace(ctx, n);
    if (rc != NBODY_OK) return rc;
    nbody::BHWorkspace &w = ctx->ws;
    int alt = 0;
    NB_CK(ctx, nbody::sort_pairs(static_cast<uint64_t *>(keys), static_cast<uint32_t *>(vals), w.keys[1], w.vals[1], n,
                                 w.sort_scratch, ctx->stream, ctx->status, &alt));
    if (alt) {
        NB_CK(ctx, cudaMemcpyAsync(keys, w.keys[1], sizeof(uint64_t) * static_cast<size_t>(n), cudaMemcpyDeviceToDevice,
                                   ctx->stream));
        NB_CK(ctx, cudaMemcpyAsync(vals, w.vals[1], sizeof(uint32_t) * static_cast<size_t>(n), cudaMemcpyDeviceToDevice,
                                   ctx->stream));
    }
    return NBODY_OK;
}

int nbody_bh_forces_device(nbody_ctx *ctx, const void *pos_mass4, void *force4, int64_t n) {
    if (!ctx || !pos_mass4 || !force4 || n <= 0 || !aligned16(pos_mass4) || !aligned16(force4))
        return NBODY_ERR_ARG;
    DeviceGuard dg(ctx->device);
    int rc = ensure_workspace(ctx, n);
    if (rc == NBODY_OK) rc = ensure_dev_buffers(ctx, n);
    if (rc != NBODY_OK) return rc;
    nbody::BHWorkspace &w = ctx->ws;
    const float4 *p = static_cast<const float4 *>(pos_mass4);
    nbody::StageTimer *tm = ctx->timer;
    NB_CK(ctx, nbody::bh_bbox(p, n, w, ctx->stream, tm));
    NB_CK(ctx, nbody::bh_keys(p, n, w, ctx->key_mode, ctx->stream, tm));
    NB_CK(ctx, nbody::bh_sort(n, w, ctx->stream, ctx->status, tm));
    NB_CK(ctx, nbody::bh_gather(n, w, p, nullptr, nullptr, nullptr, ctx->dev_pos, nullptr, nullptr, ctx->dev_ids,
                                ctx->stream, ctx->status, tm));
    NB_CK(ctx, nbody::bh_build(ctx->dev_pos, n, w, ctx->stream, ctx->status, tm));
    NB_CK(ctx, nbody::bh_traverse(ctx->dev_pos, n, w, ctx->eps2, ctx->theta2, 0.f, nullptr, nullptr, nullptr,
                                  static_cast<float4 *>(force4), ctx->dev_ids, 0, ctx->stream, tm));
    return NBODY_OK;
}

int nbody_bh_tree_export(nbody_ctx *ctx, float *records_host, int64_t cap, int64_t *count, float *box_host) {
    if (!ctx || !count) return NBODY_ERR_ARG;
    *count = 0;
    if (!ctx->ws_mem) return NBODY_ERR_STATE;
    DeviceGuard dg(ctx->device);
    const nbody::BHWorkspace &w = ctx->ws;
    uint32_t m = 0;
    NB_CK(ctx, cudaMemcpyAsync(&m, w.P + w.n, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
    NB_CK(ctx, cudaStreamSynchronize(ctx->stream));
    *count = m;
    if (box_host) NB_CK(ctx, cudaMemcpy(box_host, w.box, sizeof(float) * 6, cudaMemcpyDeviceToHost));
    if (records_host && cap > 0) {
        const int64_t k = std::min<int64_t>(cap, m);
        NB_CK(ctx, cudaMemcpy(records_host, w.nodes, sizeof(nbody::BHNode) * static_cast<size_t>(k),
                              cudaMemcpyDeviceToHost));
    }
    return NBODY_OK;
}

int nbody_pp_forces_device(nbody_ctx *ctx, const void *pos_mass4, void *force4, int64_t n) {
    if (!ctx || !pos_mass4 || !force4 || n <= 0) return NBODY_ERR_ARG;
    if (!aligned16(pos_mass4) || !aligned16(force4)) return NBODY_ERR_ARG;
    DeviceGuard dg(ctx->device);
    const nbody::PPPlan plan = nbody::pp_plan(n, ctx->device);
    int rc = ensure_scratch(ctx, plan.partial_bytes);
    if (rc != NBODY_OK) return rc;
    nbody::Integrate g;
    g.force = static_cast<float4 *>(force4);
    NB_CK(ctx, nbody::pp_launch(plan, static_cast<const float4 *>(pos_mass4), n, ctx->eps2, g, ctx->scratch,
                                ctx->stream, ctx->status, ctx->timer));
    return NBODY_OK;
}

int nbody_pp_step_device(nbody_ctx *ctx, const void *pos_in, void *pos_out, void *vel4, void *acc4, void *force4,
                         int64_t n) {
    if (!ctx || !pos_in || !pos_out || !vel4 || !acc4 || n <= 0 || pos_in == pos_out) return NBODY_ERR_ARG;
    if (!aligned16(pos_in) || !aligned16(pos_out) || !aligned16(vel4) || !aligned16(acc4) ||
        (force4 && !aligned16(force4)))
        return NBODY_ERR_ARG;
    DeviceGuard dg(ctx->device);
    const nbody::PPPlan plan = nbody::pp_plan(n, ctx->device);
    int rc = ensure_scratch(ctx, plan.partial_bytes);
    if (rc != NBODY_OK) return rc;
    nbody::Integrate g;
    g.pos_out = static_cast<float4 *>(pos_out);
    g.vel = static_cast<float4 *>(vel4);
    g.acc = static_cast<float4 *>(acc4);
    g.force = static_cast<float4 *>(force4);
    g.dt = ctx->dt;
    g.euler = ctx->integrator == NBODY_INTEGRATOR_GPU_EULER;
    NB_CK(ctx, nbody::pp_launch(plan, static_cast<const float4 *>(pos_in), n, ctx->eps2, g, ctx->scratch,
                                ctx->stream, ctx->status, ctx->timer));
    return NBODY_OK;
}

int nbody_pp_config(nbody_ctx *ctx, int64_t n, int *bodies_per_thread, int *slices, int *ctas) {
    if (!ctx || n <= 0) return NBODY_ERR_ARG;
    DeviceGuard dg(ctx->device);
    const nbody::PPPlan plan = nbody::pp_plan(n, ctx->device);
    if (bodies_per_thread) *bodies_per_thread = plan.k;
    if (slices) *slices = plan.slices;
    if (ctas) *ctas = plan.linear_ctas > 0 ? plan.linear_ctas : plan.iblocks * plan.slices;
    return NBODY_OK;
}

const char *nbody_stage_name(int stage) {
    switch (stage) {
        case nbody::kStagePPForce: return "pp_force";
        case nbody::kStagePack: return "pack";
        case nbody::kStageBBox: return "bh_bbox";
        case nbody::kStageMorton: return "bh_morton";
        case nbody::kStageSort: return "bh_sort";
        case nbody::kStageGather: return "bh_gather";
        case nbody::kStageBuild: return "bh_build";
        case nbody::kStageUpsweep: return "bh_upsweep";
        case nbody::kStageTraverse: return "bh_traverse";
        default: return "";
    }
}

int nbody_stage_count(void) { return nbody::kStageCount; }

int nbody_profile_enable(nbody_ctx *ctx, int on) {
    if (!ctx) return NBODY_ERR_ARG;
    DeviceGuard dg(ctx->device);
    if (on && !ctx->timer) {
        ctx->timer = new (std::nothrow) nbody::EventTimer();
        if (!ctx->timer) return NBODY_ERR_NOMEM;
    } else if (!on && ctx->timer) {
        NB_CK(ctx, cudaStreamSynchronize(ctx->stream));
        delete ctx->timer;
        ctx->timer = nullptr;
    }
    return NBODY_OK;
}

int nbody_profile_read(nbody_ctx *ctx, double *ms, int *launches, int nstages) {
    if (!ctx || nstages < 0) return NBODY_ERR_ARG;
    for (int i = 0; i < nstages; ++i) {
        if (ms) ms[i] = 0.0;
        if (launches) launches[i] = 0;
    }
    if (!ctx->timer) return NBODY_OK;
    DeviceGuard dg(ctx->device);
    NB_CK(ctx, ctx->timer->read(ms, launches, nstages));
    return NBODY_OK;
}

int nbody_diagnostics(nbody_ctx *ctx, double *out) {
    if (!ctx || !out) return NBODY_ERR_ARG;
    if (!ctx->uploaded) return NBODY_ERR_STATE;
    DeviceGuard dg(ctx->device);
    const int64_t n = ctx->n;
    if (!ctx->diag_mem) {
        NB_CK(ctx, cudaMalloc(&ctx->diag_mem, nbody::diag_scratch_bytes() + 256));
        NB_CK(ctx, cudaMemsetAsync(ctx->diag_mem, 0, nbody::diag_scratch_bytes() + 256, ctx->stream));
        NB_CK(ctx, cudaMalloc(&ctx->diag_phi, sizeof(float) * static_cast<size_t>(n)));
    }
    double *out_dev = reinterpret_cast<double *>(static_cast<char *>(ctx->diag_mem) + nbody::diag_scratch_bytes());
    const float4 *P, *V;
    if (ctx->mode == NBODY_MODE_PP) {
        P = ctx->pos[ctx->cur];
        V = ctx->vel;
        NB_CK(ctx, nbody::diag_pp_potential(P, n, ctx->eps2, ctx->diag_phi, ctx->stream));
    } else {
        // A tree over the current positions (the last step's tree predates the
        // integrator), built on copies so that the resident order is kept.
        P = ctx->pos[ctx->bh_pos];
        V = ctx->vel2[ctx->bh_va];
        int rc = ensure_workspace(ctx, n);
        if (rc == NBODY_OK) rc = ensure_dev_buffers(ctx, n);
        if (rc != NBODY_OK) return rc;
        nbody::BHWorkspace &w = ctx->ws;
        NB_CK(ctx, nbody::bh_bbox(P, n, w, ctx->stream, nullptr));
        NB_CK(ctx, nbody::bh_keys(P, n, w, ctx->key_mode, ctx->stream, nullptr));
        NB_CK(ctx, nbody::bh_sort(n, w, ctx->stream, ctx->status, nullptr));
        NB_CK(ctx, nbody::bh_gather(n, w, P, nullptr, nullptr, nullptr, ctx->dev_pos, nullptr, nullptr, ctx->dev_ids,
                                    ctx->stream, ctx->status, nullptr));
        NB_CK(ctx, nbody::bh_build(ctx->dev_pos, n, w, ctx->stream, ctx->status, nullptr));
        NB_CK(ctx, nbody::bh_potential(ctx->dev_pos, n, w, ctx->eps2, ctx->theta2, ctx->diag_phi, ctx->dev_ids,
                                       ctx->stream));
    }
    NB_CK(ctx, nbody::diag_momenta(P, V, ctx->diag_phi, n, ctx->diag_mem, out_dev, ctx->stream));
    NB_CK(ctx, cudaMemcpyAsync(out, out_dev, sizeof(double) * 8, cudaMemcpyDeviceToHost, ctx->stream));
    return read_status(ctx);
}

int nbody_init_device(nbody_ctx *ctx, int kind, uint64_t seed, const float *params, int nparams) {
    if (!ctx || !nbody::init_kind_valid(kind) || nparams < 0 || nparams > NBODY_INIT_MAX_PARAMS ||
        (nparams > 0 && !params))
        return NBODY_ERR_ARG;
    if (kind == NBODY_INIT_TWO_DISCS && (ctx->n < 2 || ctx->n % 2 != 0)) return NBODY_ERR_ARG;
    nbody::InitParams prm = nbody::init_defaults(kind);
    for (int k = 0; k < nparams; ++k) prm.p[k] = params[k];
    DeviceGuard dg(ctx->device);
    NB_CK(ctx, nbody::init_state(kind, seed, ctx->n, prm, ctx->pos[0], ctx->vel, ctx->acc, ctx->stream));
    ctx->cur = 0;
    ctx->bh_pos = 0;
    ctx->bh_va = 0;
    ctx->ids_valid = false;
    ctx->uploaded = true;
    return NBODY_OK;
}

int nbody_set_integrator(nbody_ctx *ctx, int integrator) {
    if (!ctx || (integrator != NBODY_INTEGRATOR_CPU && integrator != NBODY_INTEGRATOR_GPU_EULER))
        return NBODY_ERR_ARG;
    ctx->integrator = integrator;
    return NBODY_OK;
}

int nbody_set_key_mode(nbody_ctx *ctx, int mode) {
    if (!ctx || (mode != NBODY_KEYS_OCTREE && mode != NBODY_KEYS_MORTON)) return NBODY_ERR_ARG;
    ctx->key_mode = mode;
    return NBODY_OK;
}

int nbody_bh_counters(nbody_ctx *ctx, int enable, int64_t *pair_evaluations, int64_t *warp_visits) {
    if (!ctx) return NBODY_ERR_ARG;
    DeviceGuard dg(ctx->device);
    int rc = ensure_workspace(ctx, ctx->n);
    if (rc != NBODY_OK) return rc;
    unsigned long long h[2] = {0ull, 0ull};
    NB_CK(ctx, cudaMemcpyAsync(h, ctx->ws.counter_mem, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
    NB_CK(ctx, cudaMemsetAsync(ctx->ws.counter_mem, 0, sizeof(h), ctx->stream));
    NB_CK(ctx, cudaStreamSynchronize(ctx->stream));
    if (pair_evaluations) *pair_evaluations = static_cast<int64_t>(h[0]);
    if (warp_visits) *warp_visits = static_cast<int64_t>(h[1]);
    ctx->ws.counters = enable ? ctx->ws.counter_mem : nullptr;
    return NBODY_OK;
}

}  // extern "C"
