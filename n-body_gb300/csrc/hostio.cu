// Host-layout state moved by kernels that read and write page-locked host
// buffers directly (mapped into the device address space; on GB300 over the
// coherent NVLink-C2C link): one launch in and one launch out per call instead
// of a copy per array plus pack / unpack kernels. The bytes that cross the link
// are the same as with cudaMemcpyAsync. Callers pass device-mapped addresses
// only, as host_mapped returns them.
#include <cuda.h>

#include "common.cuh"
#include "kernels.h"

namespace nbody {

namespace {

// positions4 / masses4 (reference layout: vec4 each) -> pos_mass (x, y, z, m);
// vel / acc copied, or zeroed when the caller passed none.
__global__ void host_gather_kernel(const float4 *__restrict__ positions4, const float4 *__restrict__ masses4,
                                   const float4 *__restrict__ vel_h, const float4 *__restrict__ acc_h,
                                   float4 *__restrict__ pos_mass, float4 *__restrict__ vel,
                                   float4 *__restrict__ acc, int64_t n) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p = positions4[i];
    pos_mass[i] = make_float4(p.x, p.y, p.z, masses4[i].x);
    vel[i] = vel_h ? vel_h[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    acc[i] = acc_h ? acc_h[i] : make_float4(0.f, 0.f, 0.f, 0.f);
}

// inv[ids[i]] = i: the inverse of the sorted order's body ids (inv is filled
// with -1 first, so an id that no body carries stays detectable).
__global__ void invert_ids_kernel(const int *__restrict__ ids, int *__restrict__ inv, int64_t n, int *status) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int d = ids[i];
    if (d < 0 || d >= n) {
        record_error(status, NBODY_ERR_CAPACITY);
        return;
    }
    inv[d] = static_cast<int>(i);
}

// pos_mass[i].w = masses4[i].x: the masses of the reference layout (brought in
// by a copy) merged into positions copied with w = 0.
__global__ void merge_masses_kernel(float4 *__restrict__ pos_mass, const float4 *__restrict__ masses4, int64_t n) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    pos_mass[i].w = masses4[i].x;
}

// Device state -> the caller's arrays, walking the caller's order d so that
// the writes into host memory are contiguous: body d is state row inv[d] (or
// d without inv). Positions leave with w = 0, masses in the reference's vec4
// layout (m, 0, 0, 0); any output may be absent.
__global__ void host_scatter_kernel(const float4 *__restrict__ pos_mass, const float4 *__restrict__ vel,
                                    const float4 *__restrict__ acc, const int *__restrict__ inv,
                                    float4 *__restrict__ positions4, float4 *__restrict__ vel_h,
                                    float4 *__restrict__ acc_h, float4 *__restrict__ force_h,
                                    float4 *__restrict__ masses_h, int64_t n, int *status) {
    const int64_t d = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (d >= n) return;
    const int64_t i = inv ? inv[d] : d;
    if (i < 0 || i >= n) {
        record_error(status, NBODY_ERR_CAPACITY);
        return;
    }
    if (positions4 || masses_h) {
        const float4 p = pos_mass[i];
        if (positions4) positions4[d] = make_float4(p.x, p.y, p.z, 0.f);
        if (masses_h) masses_h[d] = make_float4(p.w, 0.f, 0.f, 0.f);
    }
    if (vel_h) vel_h[d] = vel[i];
    if (acc_h || force_h) {
        const float4 a = acc[i];
        if (acc_h) acc_h[d] = a;
        if (force_h) force_h[d] = a;
    }
}

}  // namespace

namespace {

// cuPointerGetAttribute from the driver, looked up through the runtime so the
// library links no libcuda; null when the driver does not offer it.
using PointerAttrFn = CUresult (*)(void *, CUpointer_attribute, CUdeviceptr);

PointerAttrFn pointer_attr() {
    static PointerAttrFn fn = [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuPointerGetAttribute", &f, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            return static_cast<PointerAttrFn>(nullptr);
        }
        return reinterpret_cast<PointerAttrFn>(f);
    }();
    return fn;
}

// True when [addr, addr + bytes) lies inside the registered or allocated range
// that the driver reports for addr.
bool range_holds(uintptr_t addr, size_t bytes) {
    const PointerAttrFn fn = pointer_attr();
    if (!fn) return false;
    CUdeviceptr start = 0;
    size_t size = 0;
    if (fn(&start, CU_POINTER_ATTRIBUTE_RANGE_START_ADDR, static_cast<CUdeviceptr>(addr)) != CUDA_SUCCESS ||
        fn(&size, CU_POINTER_ATTRIBUTE_RANGE_SIZE, static_cast<CUdeviceptr>(addr)) != CUDA_SUCCESS)
        return false;
    const uintptr_t lo = static_cast<uintptr_t>(start);
    return addr >= lo && bytes <= size && addr - lo <= size - bytes;
}

}  // namespace

float4 *host_mapped(const void *p, size_t bytes, int device) {
    if (!p || (reinterpret_cast<uintptr_t>(p) & 15u) != 0) return nullptr;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type != cudaMemoryTypeHost || a.device != device || !a.devicePointer ||
        (reinterpret_cast<uintptr_t>(a.devicePointer) & 15u) != 0)
        return nullptr;
    // The kernels touch all `bytes` through the mapped address: a buffer that
    // is page-locked only in part (or shorter than the call's bodies) takes
    // the copy path, whose host-side reads the driver stages itself.
    if (!range_holds(reinterpret_cast<uintptr_t>(p), bytes) &&
        !range_holds(reinterpret_cast<uintptr_t>(a.devicePointer), bytes))
        return nullptr;
    return static_cast<float4 *>(a.devicePointer);
}

cudaError_t merge_masses(float4 *pos_mass, const float4 *masses4, int64_t n, cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    const int threads = 256;
    merge_masses_kernel<<<static_cast<unsigned>((n + threads - 1) / threads), threads, 0, stream>>>(pos_mass, masses4,
                                                                                                   n);
    return cudaGetLastError();
}

cudaError_t host_gather(const float4 *positions4, const float4 *masses4, const float4 *vel_h, const float4 *acc_h,
                        float4 *pos_mass, float4 *vel, float4 *acc, int64_t n, cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    const int threads = 256;
    host_gather_kernel<<<static_cast<unsigned>((n + threads - 1) / threads), threads, 0, stream>>>(
        positions4, masses4, vel_h, acc_h, pos_mass, vel, acc, n);
    return cudaGetLastError();
}

cudaError_t host_scatter(const float4 *pos_mass, const float4 *vel, const float4 *acc, const int *ids, int *inv,
                         float4 *positions4, float4 *vel_h, float4 *acc_h, float4 *force_h, float4 *masses_h,
                         int64_t n, cudaStream_t stream, int *status) {
    if (n <= 0) return cudaSuccess;
    const int threads = 256;
    const unsigned blocks = static_cast<unsigned>((n + threads - 1) / threads);
    if (ids) {
        cudaError_t e = cudaMemsetAsync(inv, 0xff, static_cast<size_t>(n) * sizeof(int), stream);
        if (e != cudaSuccess) return e;
        invert_ids_kernel<<<blocks, threads, 0, stream>>>(ids, inv, n, status);
    }
    host_scatter_kernel<<<blocks, threads, 0, stream>>>(pos_mass, vel, acc, ids ? inv : nullptr, positions4, vel_h,
                                                        acc_h, force_h, masses_h, n, status);
    return cudaGetLastError();
}

}  // namespace nbody
