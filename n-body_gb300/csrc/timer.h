// CUDA-event timing of launcher stages (internal to the library).
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "kernels.h"

namespace nbody {

// Records a CUDA event pair around each launcher stage on the launch stream;
// read back (and reset) by nbody_profile_read.
struct EventTimer : StageTimer {
    struct Rec {
        int stage;
        cudaEvent_t a, b;
    };
    std::vector<cudaEvent_t> pool;
    size_t used = 0;
    std::vector<Rec> recs;
    cudaEvent_t open[kStageCount] = {};

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


}  // namespace nbody
