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
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "kernels.h"
#include "nbody_gb300.h"

namespace {

// Records a CUDA event pair around each launcher stage on the launch stream;
// read back (and reset) by nbody_profile_read.
struct EventTimer : nbody::StageTimer {
    struct Rec {
        int stage;
        cudaEvent_t a, b;
    };
    std::vector<cudaEvent_t> pool;
    size_t used = 0;
    std::vector<Rec> recs;
    cudaEvent_t open[nbody::kStageCount] = {};

    cudaEvent_t get() {
        if (used == pool.size()) {
            cudaEvent_t e = nullptr;
            if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
            pool.push_back(e);
        }
        return pool[used++];
    }
    void begin(int st, cudaStream_t s) override {
        cudaEvent_t e = get();
        if (e) cudaEventRecord(e, s);
        open[st] = e;
    }
    void end(int st, cudaStream_t s) override {
        cudaEvent_t e = get();
        if (e) cudaEventRecord(e, s);
        if (e && open[st]) recs.push_back({st, open[st], e});
        open[st] = nullptr;
    }
    cudaError_t read(double *ms, int *count, int nstages) {
        for (const Rec &r : recs) {
            cudaError_t e = cudaEventSynchronize(r.b);
            if (e != cudaSuccess) return e;
            float t = 0.f;
            e = cudaEventElapsedTime(&t, r.a, r.b);
            if (e != cudaSuccess) return e;
            if (r.stage < nstages) {
                if (ms) ms[r.stage] += t;
                if (count) count[r.stage] += 1;
            }
        }
        recs.clear();
        used = 0;
        return cudaSuccess;
    }
    ~EventTimer() override {
        for (cudaEvent_t e : pool) cudaEventDestroy(e);
    }
};

}  // namespace

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
    void *scratch = nullptr;
    size_t scratch_bytes = 0;
    bool uploaded = false;
    EventTimer *timer = nullptr;  // non-null while profiling is enabled
    std::string last_error;
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
    NB_CK(ctx, cudaMemcpyAsync(&h, ctx->status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    NB_CK(ctx, cudaMemsetAsync(ctx->status, 0, sizeof(int), ctx->stream));
    NB_CK(ctx, cudaStreamSynchronize(ctx->stream));
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
        NB_CK(ctx, nbody::pp_launch(plan, ctx->pos[ctx->cur], ctx->n, ctx->eps2, g, ctx->scratch, ctx->stream,
                                    ctx->status, ctx->timer));
        ctx->cur ^= 1;
    }
    return NBODY_OK;
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
    if (rc == NBODY_OK) {
        cudaError_t e = cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) rc = fail(ctx, e);
        ctx->stream = ctx->own_stream;
    }
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
        cudaFree(ctx->scratch);
        delete ctx->timer;
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
    ctx->cur = 0;
    NB_CK(ctx, nbody::pack_state(ctx->stage, ctx->stage + ctx->n, ctx->pos[0], ctx->n, ctx->stream));
    ctx->uploaded = true;
    return NBODY_OK;
}

int nbody_step(nbody_ctx *ctx, int steps) {
    if (!ctx || steps < 0) return NBODY_ERR_ARG;
    if (!ctx->uploaded) return NBODY_ERR_STATE;
    DeviceGuard dg(ctx->device);
    if (ctx->mode == NBODY_MODE_PP) return pp_steps(ctx, steps);
    return NBODY_ERR_ARG;
}

int nbody_download(nbody_ctx *ctx, float *positions4, float *velocities4, float *accelerations4, float *forces4) {
    if (!ctx) return NBODY_ERR_ARG;
    if (!ctx->uploaded) return NBODY_ERR_STATE;
    DeviceGuard dg(ctx->device);
    const size_t b4 = static_cast<size_t>(ctx->n) * sizeof(float4);
    if (positions4) {
        NB_CK(ctx, nbody::unpack_positions(ctx->pos[ctx->cur], ctx->stage, ctx->n, ctx->stream));
        NB_CK(ctx, cudaMemcpyAsync(positions4, ctx->stage, b4, cudaMemcpyDeviceToHost, ctx->stream));
    }
    if (velocities4) NB_CK(ctx, cudaMemcpyAsync(velocities4, ctx->vel, b4, cudaMemcpyDeviceToHost, ctx->stream));
    if (accelerations4)
        NB_CK(ctx, cudaMemcpyAsync(accelerations4, ctx->acc, b4, cudaMemcpyDeviceToHost, ctx->stream));
    if (forces4) NB_CK(ctx, cudaMemcpyAsync(forces4, ctx->acc, b4, cudaMemcpyDeviceToHost, ctx->stream));
    return read_status(ctx);
}

int nbody_sync(nbody_ctx *ctx) {
    if (!ctx) return NBODY_ERR_ARG;
    DeviceGuard dg(ctx->device);
    return read_status(ctx);
}

int nbody_update_host(nbody_ctx *ctx, float *positions4, float *velocities4, float *accelerations4,
                      const float *masses4, float *forces4, int steps) {
    if (!ctx || !positions4 || !velocities4 || !accelerations4 || !masses4 || steps < 0) return NBODY_ERR_ARG;
    int rc = nbody_upload(ctx, positions4, velocities4, accelerations4, masses4);
    if (rc == NBODY_OK) rc = nbody_step(ctx, steps);
    if (rc == NBODY_OK) rc = nbody_download(ctx, positions4, velocities4, accelerations4, forces4);
    return rc;
}

int nbody_device_state(nbody_ctx *ctx, void **pos_mass4, void **vel4, void **acc4) {
    if (!ctx) return NBODY_ERR_ARG;
    if (pos_mass4) *pos_mass4 = ctx->pos[ctx->cur];
    if (vel4) *vel4 = ctx->vel;
    if (acc4) *acc4 = ctx->acc;
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
    if (ctas) *ctas = plan.iblocks * plan.slices;
    return NBODY_OK;
}

const char *nbody_stage_name(int stage) {
    switch (stage) {
        case nbody::kStagePPForce: return "pp_force";
        case nbody::kStagePack: return "pack";
        default: return "";
    }
}

int nbody_stage_count(void) { return nbody::kStageCount; }

int nbody_profile_enable(nbody_ctx *ctx, int on) {
    if (!ctx) return NBODY_ERR_ARG;
    DeviceGuard dg(ctx->device);
    if (on && !ctx->timer) {
        ctx->timer = new (std::nothrow) EventTimer();
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

}  // extern "C"
