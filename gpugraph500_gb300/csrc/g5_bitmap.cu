// g5_bitmap.cu -- frontier-bitmap OR reduction.
//
// The reference merges frontier bitmaps of the column ranks inside vreduce
// (cpu_2d/vreduce.hpp:112,257-259,359-361) with CPUBFS_bin::reduce_fq_out,
// fq_out[i] |= in[i] over uint64 words (cpu_2d/cpubfs_bin.cpp:55-65).  On one
// GPU the k logical blocks are k device bitmaps OR-ed into dst in one pass:
// each thread streams 16-byte vectors of all k sources, so dst is read and
// written once and every source read once ((k+1)*8 + 8 bytes per word pair).
#include "g5_common.cuh"

namespace {

constexpr int kMaxSrc = 64;

struct Srcs {
    const uint64_t *p[kMaxSrc];
};

__global__ void __launch_bounds__(256) k_or_vec(ulonglong2 *__restrict__ dst, Srcs s, int k, uint64_t nvec)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nvec;
         i += (uint64_t)gridDim.x * blockDim.x) {
        ulonglong2 acc = dst[i];
        for (int j = 0; j < k; ++j) {
            const ulonglong2 x = __ldcs(reinterpret_cast<const ulonglong2 *>(s.p[j]) + i);
            acc.x |= x.x;
            acc.y |= x.y;
        }
        dst[i] = acc;
    }
}

__global__ void __launch_bounds__(256) k_or_tail(uint64_t *__restrict__ dst, Srcs s, int k, uint64_t w0,
                                                 uint64_t words)
{
    for (uint64_t i = w0 + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < words;
         i += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t acc = dst[i];
        for (int j = 0; j < k; ++j) acc |= s.p[j][i];
        dst[i] = acc;
    }
}

}  // namespace

extern "C" g5_status g5_bitmap_or(uint64_t *dst, const uint64_t *const *srcs, int k, size_t words, void *stream)
{
    if (!dst || k < 0 || k > kMaxSrc || (k && !srcs)) return G5_ERR_INVALID_ARG;
    if (words == 0 || k == 0) return G5_OK;
    Srcs s;
    bool aligned = ((uintptr_t)dst & 15) == 0;
    for (int j = 0; j < k; ++j) {
        if (!srcs[j]) return G5_ERR_INVALID_ARG;
        s.p[j] = srcs[j];
        aligned = aligned && ((uintptr_t)srcs[j] & 15) == 0;
    }
    cudaStream_t st = (cudaStream_t)stream;
    uint64_t done = 0;
    if (aligned) {
        const uint64_t nvec = words / 2;
        if (nvec) k_or_vec<<<g5::grid_for(8), 256, 0, st>>>(reinterpret_cast<ulonglong2 *>(dst), s, k, nvec);
        done = nvec * 2;
    }
    if (done < words) k_or_tail<<<g5::grid_for(1), 256, 0, st>>>(dst, s, k, done, words);
    G5_CUDA(cudaGetLastError());
    return G5_OK;
}
