// g5_common.cuh -- shared definitions of the libg5bfs CUDA sources.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>

#include "g5bfs.h"

#define G5_NUM_SMS_DEFAULT 152

namespace g5 {

// Maps a CUDA error to a status code (allocation failures are OOM).
inline g5_status cuda_status(cudaError_t e)
{
    if (e == cudaSuccess) return G5_OK;
    if (e == cudaErrorMemoryAllocation) return G5_ERR_OOM;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return G5_ERR_NO_DEVICE;
    return G5_ERR_CUDA;
}

// Returns from the enclosing function with a status if a CUDA call fails.
#define G5_CUDA(call)                                                            \
    do {                                                                         \
        cudaError_t g5_e_ = (call);                                              \
        if (g5_e_ != cudaSuccess) {                                              \
            if (getenv("G5_VERBOSE"))                                            \
                fprintf(stderr, "g5: %s failed at %s:%d: %s\n", #call, __FILE__, \
                        __LINE__, cudaGetErrorString(g5_e_));                    \
            return ::g5::cuda_status(g5_e_);                                     \
        }                                                                        \
    } while (0)

#define G5_TRY(call)                       \
    do {                                   \
        g5_status g5_s_ = (call);          \
        if (g5_s_ != G5_OK) return g5_s_;  \
    } while (0)

// Number of SMs of the current device (cached per process).
int num_sms();

// True if p is a device or managed pointer.
bool is_device_ptr(const void *p);

// Grid of `per_sm` blocks per SM.
inline int grid_for(int per_sm) { return num_sms() * per_sm; }

// Owning device buffer (freed on scope exit unless released).
template <class T>
struct DevBuf {
    T *p = nullptr;
    ~DevBuf()
    {
        if (p) cudaFree(p);
    }
    g5_status alloc(size_t count)
    {
        G5_CUDA(cudaMalloc(&p, sizeof(T) * (count ? count : 1)));
        return G5_OK;
    }
    T *release()
    {
        T *r = p;
        p = nullptr;
        return r;
    }
};

// Launches kern on s; with pdl, as a programmatic dependent of the kernel
// before it on the stream (the kernel must call g5_pdl_sync first).
template <typename... KArgs, typename... Args>
cudaError_t launch(bool pdl, void (*kern)(KArgs...), dim3 grid, dim3 block, cudaStream_t s, Args... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kern, args...);
}

// As launch(), with smem bytes of dynamic shared memory.
template <typename... KArgs, typename... Args>
cudaError_t launch_dyn(bool pdl, void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                       Args... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kern, args...);
}

}  // namespace g5

// Device-side error flags (bit set in a status word).
enum : uint32_t {
    G5_DEVERR_CAPACITY = 1u,
    G5_DEVERR_CORRUPT = 2u,
    G5_DEVERR_MISMATCH = 4u,
    G5_DEVERR_LEVELS = 8u,
    G5_DEVERR_WAIT = 16u,  // a bounded device wait ran out
};

__device__ __forceinline__ int g5_lane() { return threadIdx.x & 31; }

// Programmatic dependent launch: waits until the kernel before this one on
// the stream has finished and its writes are visible, then lets the next
// launch start setting up while this one runs.  Both are no-ops for an
// ordinary launch; a kernel calls this before it reads anything.
__device__ __forceinline__ void g5_pdl_sync()
{
    asm volatile("griddepcontrol.wait;\n" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
}
__device__ __forceinline__ unsigned g5_lanemask_lt()
{
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}
