// Self-test of the bounded device waits (C ABI nbody_selftest_wait): a kernel
// waits on an mbarrier that nothing ever arrives at, through the same helper
// the force kernels use, and must give up after the limit with
// NBODY_ERR_TIMEOUT in its status word, leaving the context usable. This is
// how a lost copy or a broken invariant surfaces instead of a hung GPU.
#include <cuda_runtime.h>

#include "common.cuh"
#include "nbody_gb300.h"

namespace {

__global__ void wait_selftest_kernel(unsigned long long limit_ns, int *status, unsigned long long *waited_ns) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        nbody::mbar_init(&bar, 1);
        nbody::mbar_init_fence();
    }
    __syncthreads();
    const unsigned long long t0 = nbody::global_ns();
    // No thread arrives and no copy completes on `bar`: phase 0 never ends.
    const bool done = nbody::mbar_wait_bounded_ns(&bar, 0, status, limit_ns);
    __syncthreads();
    if (threadIdx.x == 0) {
        waited_ns[0] = nbody::global_ns() - t0;
        if (done) nbody::record_error(status, NBODY_ERR_STATE);  // cannot happen: report it
    }
}

}  // namespace

extern "C" int nbody_selftest_wait(int device, int64_t limit_us, int *kernel_status, double *waited_ms) {
    if (!kernel_status || limit_us < 1 || limit_us > 1000000) return NBODY_ERR_ARG;
    int prev = -1;
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    if (cudaSetDevice(device) != cudaSuccess) return NBODY_ERR_CUDA;
    int rc = NBODY_OK;
    void *mem = nullptr;
    if (cudaMalloc(&mem, 16) != cudaSuccess) {
        rc = NBODY_ERR_NOMEM;
    } else {
        int *status = static_cast<int *>(mem);
        auto *waited = reinterpret_cast<unsigned long long *>(static_cast<char *>(mem) + 8);
        unsigned long long host[2] = {0ull, 0ull};
        if (cudaMemset(mem, 0, 16) != cudaSuccess) rc = NBODY_ERR_CUDA;
        if (rc == NBODY_OK) {
            wait_selftest_kernel<<<1, 32>>>(static_cast<unsigned long long>(limit_us) * 1000ull, status, waited);
            if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) rc = NBODY_ERR_CUDA;
        }
        if (rc == NBODY_OK && cudaMemcpy(host, mem, 16, cudaMemcpyDeviceToHost) != cudaSuccess) rc = NBODY_ERR_CUDA;
        if (rc == NBODY_OK) {
            *kernel_status = static_cast<int>(host[0] & 0xffffffffull);
            if (waited_ms) *waited_ms = static_cast<double>(host[1]) * 1e-6;
        }
        cudaFree(mem);
    }
    if (prev >= 0) cudaSetDevice(prev);
    return rc;
}
