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
#include <cuda.h>
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
unsigned long long g_scratch_ctx[kMaxDevices] = {};

// Driver entry points looked up through the runtime (the library links no
// libcuda): cuCtxGetCurrent and cuCtxGetId.
using CtxGetCurrentFn = CUresult (*)(CUcontext *);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long *);

void *driver_fn(const char *name) {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion(name, &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return f;
}

// The id of the context current on this thread (unique for the life of the
// process, so a context made anew after cudaDeviceReset has another), or 0.
unsigned long long current_ctx_id() {
    static const CtxGetCurrentFn get = reinterpret_cast<CtxGetCurrentFn>(driver_fn("cuCtxGetCurrent"));
    static const CtxGetIdFn get_id = reinterpret_cast<CtxGetIdFn>(driver_fn("cuCtxGetId"));
    CUcontext cur = nullptr;
    unsigned long long id = 0;
    if (!get || !get_id || get(&cur) != CUDA_SUCCESS || !cur || get_id(cur, &id) != CUDA_SUCCESS) return 0;
    return id;
}

// Set-up, once per device, with that device current: the array's device
// address. The address is kept with the id of the context it belongs to and
// looked up again when the current context is another one (after
// cudaDeviceReset the module, and with it the array, is loaded anew).
cudaError_t scratch_address(int device, unsigned char **out) {
    if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_setup_mu);
    unsigned long long ctx = current_ctx_id();
    if (!ctx || !g_scratch_addr[device] || g_scratch_ctx[device] != ctx) {
        // The lookup binds the device's context to this thread if none was
        // yet, so the context is read again after it.
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        if (!(ctx = current_ctx_id())) return cudaErrorInitializationError;
        g_scratch_addr[device] = static_cast<unsigned char *>(p);
        g_scratch_ctx[device] = ctx;
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
