// g5_bitmap.cu -- frontier-bitmap OR reduction.
//
// The reference merges frontier bitmaps of the column ranks inside vreduce
// (cpu_2d/vreduce.hpp:112,257-259,359-361) with CPUBFS_bin::reduce_fq_out,
// fq_out[i] |= in[i] over uint64 words (cpu_2d/cpubfs_bin.cpp:55-65).  On one
// GPU the k logical blocks are k device bitmaps OR-ed into dst in one pass
// (up to 8 sources; more take one pass per 8): each thread streams 16-byte
// vectors of all sources, so dst is read and written once per pass and every
// source read once ((k+2)*8 bytes per word for k <= 8).
#include "g5_common.cuh"

namespace {

constexpr int kMaxSrc = 64;

struct Srcs {
    const uint64_t *p[kMaxSrc];
};

// K sources (a compile-time count) and V 16-byte vectors per thread: the
// V x (K + 1) loads of a thread are independent and issued together, then
// OR-ed, so a thread keeps all of them in flight instead of waiting on one
// source at a time.  Streaming loads: nothing here is read twice.  The
// library launches V = 1.
template <int K, int V>
__global__ void __launch_bounds__(256) k_or_vec(ulonglong2 *__restrict__ dst, Srcs s, uint64_t nvec)
{
    g5_pdl_sync();
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i0 = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i0 < nvec; i0 += stride * V) {
        ulonglong2 acc[V];
#pragma unroll
        for (int v = 0; v < V; ++v) {
            const uint64_t i = i0 + v * stride;
            acc[v] = i < nvec ? __ldcs(dst + i) : make_ulonglong2(0, 0);
        }
        ulonglong2 x[K][V];
#pragma unroll
        for (int j = 0; j < K; ++j)
#pragma unroll
            for (int v = 0; v < V; ++v) {
                const uint64_t i = i0 + v * stride;
                x[j][v] = i < nvec ? __ldcs(reinterpret_cast<const ulonglong2 *>(s.p[j]) + i)
                                   : make_ulonglong2(0, 0);
            }
#pragma unroll
        for (int j = 0; j < K; ++j)
#pragma unroll
            for (int v = 0; v < V; ++v) {
                acc[v].x |= x[j][v].x;
                acc[v].y |= x[j][v].y;
            }
#pragma unroll
        for (int v = 0; v < V; ++v) {
            const uint64_t i = i0 + v * stride;
            if (i < nvec) dst[i] = acc[v];
        }
    }
}

// one vector per thread and grid step: 4.85 TB/s on 8 x 2^24-bit sources
// against 3.18 TB/s with two (measured in one graph of 24 calls; the
// threads' 9 loads of one vector keep enough bytes in flight, and a second
// vector only halves the threads and unbalances the SMs)
constexpr int kVec = 1;
constexpr int kPassSrc = 8;  // sources per pass for k > kPassSrc

template <int K>
void launch_or(ulonglong2 *dst, const Srcs &s, uint64_t nvec, cudaStream_t st)
{
    // one grid step covers the bitmap when it is small (every thread busy
    // once), a grid-stride loop over 8 blocks per SM when it is large
    const uint64_t per_block = 256ull * kVec;
    const uint64_t want = (nvec + per_block - 1) / per_block;
    const uint64_t cap = (uint64_t)g5::grid_for(8);
    const int grid = (int)(want < cap ? want : cap);
    // a programmatic dependent launch: it may begin while the previous
    // kernel on the stream drains; the kernel's first instruction keeps the
    // data dependence
    g5::launch(true, k_or_vec<K, kVec>, grid, 256, st, dst, s, nvec);
}

void dispatch_or(ulonglong2 *dst, const Srcs &s, int k, uint64_t nvec, cudaStream_t st)
{
    switch (k) {
    case 1: launch_or<1>(dst, s, nvec, st); break;
    case 2: launch_or<2>(dst, s, nvec, st); break;
    case 3: launch_or<3>(dst, s, nvec, st); break;
    case 4: launch_or<4>(dst, s, nvec, st); break;
    case 5: launch_or<5>(dst, s, nvec, st); break;
    case 6: launch_or<6>(dst, s, nvec, st); break;
    case 7: launch_or<7>(dst, s, nvec, st); break;
    default: launch_or<8>(dst, s, nvec, st); break;
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
        if (nvec) {
            // up to kPassSrc sources per pass (dst read and written once per pass)
            for (int j0 = 0; j0 < k; j0 += kPassSrc) {
                Srcs part;
                const int kk = k - j0 < kPassSrc ? k - j0 : kPassSrc;
                for (int j = 0; j < kk; ++j) part.p[j] = s.p[j0 + j];
                dispatch_or(reinterpret_cast<ulonglong2 *>(dst), part, kk, nvec, st);
            }
        }
        done = nvec * 2;
    }
    if (done < words) k_or_tail<<<g5::grid_for(1), 256, 0, st>>>(dst, s, k, done, words);
    G5_CUDA(cudaGetLastError());
    return G5_OK;
}
