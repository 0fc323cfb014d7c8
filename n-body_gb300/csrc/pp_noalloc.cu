// Direct-sum forces through an entry point that allocates nothing.
//
// Some callers cannot let a library call cudaMalloc: a frame or control loop
// that must never stall on an allocation (cudaMalloc and cudaFree can
// synchronise the whole device), or a host application that owns all device
// memory through its own pool, so that memory appearing behind its back would
// break its budget. nbody_pp_forces_device needs a context, and a context
// allocates its state and scratch. This entry point takes only the caller's
// input and output buffers; the kernel's scratch (status word, per-i-block
// arrival counters, per-slice partial accelerations) lives in one fixed-size
// array in device memory defined in this file.
#include <cuda_runtime.h>

#include <mutex>

#include "kernels.h"
#include "nbody_gb300.h"

namespace {

constexpr size_t kScratchBytes = 8u << 20;  // 8 MiB on every device that loads the library
constexpr size_t kStatusBytes = 256;        // status word, padded so the rest stays 256-byte aligned

// Device-side scratch. In host code this name is a host-side stand-in, not a
// device address: host code must use the address cudaGetSymbolAddress gives.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
unsigned char *g_scratch_addr[kMaxDevices] = {};

// Set-up, once per device, with that device current.
cudaError_t scratch_address(int device, unsigned char **out) {
    if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (!g_scratch_addr[device]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_addr[device] = static_cast<unsigned char *>(p);
    }
    *out = g_scratch_addr[device];
    return cudaSuccess;
}

}  // namespace

extern "C" int nbody_pp_forces_noalloc(const void *pos_mass4, void *force4, int64_t n, float eps2, void *stream,
                                       int *kernel_status) {
    if (!pos_mass4 || !force4 || n <= 0 || !(eps2 >= 0.f)) return NBODY_ERR_ARG;
    if ((reinterpret_cast<uintptr_t>(pos_mass4) & 15u) || (reinterpret_cast<uintptr_t>(force4) & 15u))
        return NBODY_ERR_ARG;
    if (n > NBODY_NOALLOC_MAX_BODIES) return NBODY_ERR_CAPACITY;
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess) return NBODY_ERR_CUDA;
    unsigned char *scratch = nullptr;
    if (scratch_address(device, &scratch) != cudaSuccess) return NBODY_ERR_CUDA;
    const cudaStream_t st = static_cast<cudaStream_t>(stream);
    const nbody::PPPlan plan = nbody::pp_plan_within(n, device, kScratchBytes - kStatusBytes);
    // The array keeps the previous call's contents: clear the status word and
    // the arrival counters, which must start at zero.
    if (cudaMemsetAsync(scratch, 0, kStatusBytes + plan.arrivals_bytes, st) != cudaSuccess) return NBODY_ERR_CUDA;
    nbody::Integrate g;
    g.force = static_cast<float4 *>(force4);
    if (nbody::pp_launch(plan, static_cast<const float4 *>(pos_mass4), n, eps2, g, scratch + kStatusBytes, st,
                         reinterpret_cast<int *>(scratch)) != cudaSuccess)
        return NBODY_ERR_CUDA;
    if (kernel_status) {
        if (cudaMemcpyAsync(kernel_status, scratch, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess)
            return NBODY_ERR_CUDA;
        if (cudaStreamSynchronize(st) != cudaSuccess) return NBODY_ERR_CUDA;
    }
    return NBODY_OK;
}
