// g5_graph.cu -- resident CSR graphs: upload, GPU Kronecker generation and
// GPU CSR construction.
//
// The generator restates the Graph500 Kronecker generator of the reference
// (cpu_2d/generator/graph_generator.c:45-187, splittable_mrg.c:79-127,
// utils.c:60-67) one edge per thread; the CSR build does on the device what
// DistMatrix2d::setupMatrix2 does at 1x1 (cpu_2d/distmatrix2d.hh:745-1166):
// append reversed edges, sort by (v0, v1), drop self loops and duplicates.
#include <cub/cub.cuh>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "g5_common.cuh"
#include "g5_internal.h"

namespace g5 {

int num_sms()
{
    static int sms = 0;
    if (!sms) {
        int dev = 0, v = 0;
        if (cudaGetDevice(&dev) == cudaSuccess &&
            cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && v > 0)
            sms = v;
        else
            sms = G5_NUM_SMS_DEFAULT;
    }
    return sms;
}

bool is_device_ptr(const void *p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// ---- MRG skip table ------------------------------------------------------

static const uint32_t kP = 0x7FFFFFFFu;

static void mat_mul_host(const uint32_t *a, const uint32_t *b, uint32_t *r)
{
    uint32_t t[25];
    for (int i = 0; i < 5; ++i)
        for (int j = 0; j < 5; ++j) {
            uint64_t s = 0;
            for (int k = 0; k < 5; ++k) s = (s + (uint64_t)a[i * 5 + k] * b[k * 5 + j]) % kP;
            t[i * 5 + j] = (uint32_t)s;
        }
    memcpy(r, t, sizeof t);
}

// The reference ships these powers of the one-step matrix as a generated
// table (cpu_2d/generator/mrg_transitions.c); here they are computed once.
const uint32_t *mrg_skip_table_host()
{
    static std::vector<uint32_t> tab;
    static std::once_flag once;
    std::call_once(once, [] {
        tab.assign(24 * 256 * 25, 0);
        uint32_t base[25] = {0};
        base[0] = 107374182u;
        base[4] = 104480u;
        base[5] = base[11] = base[17] = base[23] = 1;
        for (int k = 0; k < 24; ++k) {
            uint32_t *row = &tab[(size_t)k * 256 * 25];
            for (int i = 0; i < 5; ++i) row[i * 6] = 1;
            for (int v = 1; v < 256; ++v) mat_mul_host(row + (v - 1) * 25, base, row + v * 25);
            uint32_t nb[25];
            mat_mul_host(row + 255 * 25, base, nb);
            memcpy(base, nb, sizeof nb);
        }
    });
    return tab.data();
}

}  // namespace g5

// ---- device generator ------------------------------------------------------

namespace {

// x mod (2^31 - 1) for x < 2^64 by folding (exact, same value as %).
__device__ __forceinline__ uint32_t mod_p(uint64_t x)
{
    x = (x & 0x7FFFFFFFull) + (x >> 31);
    x = (x & 0x7FFFFFFFull) + (x >> 31);
    uint32_t r = (uint32_t)x;
    return r >= 0x7FFFFFFFu ? r - 0x7FFFFFFFu : r;
}

struct Mrg {
    uint32_t z[5];
};

__device__ __forceinline__ void mrg_apply(const uint32_t *__restrict__ m, Mrg &s)
{
    uint32_t o[5];
#pragma unroll
    for (int i = 0; i < 5; ++i) {
        // each product < 2^62, the sum of five < 2^65: fold pairwise
        uint64_t acc = (uint64_t)__ldg(m + i * 5) * s.z[0] + (uint64_t)__ldg(m + i * 5 + 1) * s.z[1];
        acc = mod_p(acc) + (uint64_t)__ldg(m + i * 5 + 2) * s.z[2];
        acc = mod_p(acc) + (uint64_t)__ldg(m + i * 5 + 3) * s.z[3];
        acc = mod_p(acc) + (uint64_t)__ldg(m + i * 5 + 4) * s.z[4];
        o[i] = mod_p(acc);
    }
#pragma unroll
    for (int i = 0; i < 5; ++i) s.z[i] = o[i];
}

__device__ __forceinline__ uint32_t mrg_next(Mrg &s)
{
    uint32_t nz = mod_p((uint64_t)107374182u * s.z[0] + (uint64_t)104480u * s.z[4]);
    s.z[4] = s.z[3];
    s.z[3] = s.z[2];
    s.z[2] = s.z[1];
    s.z[1] = s.z[0];
    s.z[0] = nz;
    return nz;
}

__device__ __forceinline__ int bernoulli4(Mrg &s)
{
    const uint32_t limit = 0xFFFFFFFFu % 10000u;
    uint32_t v = mrg_next(s);
    while (v < limit) v = mrg_next(s);
    v %= 10000u;
    if (v < 1900u) return 1;
    v -= 1900u;
    if (v < 1900u) return 2;
    v -= 1900u;
    if (v < 5700u) return 0;
    return 3;
}

__device__ __forceinline__ uint64_t scramble(uint64_t v, int lg, uint64_t val0, uint64_t val1)
{
    v += val0 + val1;
    v *= (val0 | 0x4519840211493211ull);
    v = __brevll(v) >> (64 - lg);
    v *= (val1 | 0x3050852102C843A5ull);
    v = __brevll(v) >> (64 - lg);
    return v;
}

struct GenParams {
    Mrg seed;
    uint64_t val0, val1;
    int scale;
};

// Edge ei of the generator, as (src, dst).
__device__ __forceinline__ void gen_edge(const GenParams &p, const uint32_t *__restrict__ skip,
                                         uint64_t ei, uint64_t &a, uint64_t &b)
{
    Mrg s = p.seed;
    // mrg_skip(&s, 0, ei, 0): the middle 64-bit word maps to byte tables 8..15
    uint64_t e = ei;
    for (int bi = 8; e; ++bi, e >>= 8) {
        uint32_t v = (uint32_t)(e & 0xFF);
        if (v) mrg_apply(skip + ((size_t)bi * 256 + v) * 25, s);
    }
    int64_t bs = 0, bt = 0, nv = (int64_t)1 << p.scale;
    while (nv > 1) {
        int sq = bernoulli4(s);
        int so = sq >> 1, to = sq & 1;
        if (bs == bt && so > to) {
            int t = so;
            so = to;
            to = t;
        }
        nv >>= 1;
        bs += nv * so;
        bt += nv * to;
    }
    a = scramble((uint64_t)bs, p.scale, p.val0, p.val1);
    b = scramble((uint64_t)bt, p.scale, p.val0, p.val1);
}

// Writes both orientations as dense keys (src << scale | dst).
__global__ void k_gen_keys(GenParams p, const uint32_t *__restrict__ skip, uint64_t m,
                           uint64_t *__restrict__ keys)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m;
         i += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t a, b;
        gen_edge(p, skip, i, a, b);
        keys[i] = (a << p.scale) | b;
        keys[m + i] = (b << p.scale) | a;
    }
}

__global__ void k_gen_pairs(GenParams p, const uint32_t *__restrict__ skip, uint64_t start, uint64_t cnt,
                            int64_t *__restrict__ out)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < cnt;
         i += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t a, b;
        gen_edge(p, skip, start + i, a, b);
        out[2 * i] = (int64_t)a;
        out[2 * i + 1] = (int64_t)b;
    }
}

// row_off[v] = first index with (key >> shift) >= v, for sorted keys.
__global__ void k_row_bounds(const uint64_t *__restrict__ keys, uint64_t cnt, int shift, int64_t n,
                             int64_t *__restrict__ row_off)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i <= cnt;
         i += (uint64_t)gridDim.x * blockDim.x) {
        int64_t cur = i < cnt ? (int64_t)(keys[i] >> shift) : n;
        int64_t prev = i > 0 ? (int64_t)(keys[i - 1] >> shift) : -1;
        for (int64_t v = prev + 1; v <= cur && v <= n; ++v) row_off[v] = (int64_t)i;
    }
}

__global__ void k_degrees_u32(const int64_t *__restrict__ row_off, int64_t n, uint32_t *__restrict__ deg)
{
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n;
         v += (int64_t)gridDim.x * blockDim.x)
        deg[v] = (uint32_t)(row_off[v + 1] - row_off[v]);
}

struct NotSelfLoop {
    int scale;
    uint64_t mask;
    __host__ __device__ bool operator()(uint64_t k) const { return (k >> scale) != (k & mask); }
};

__global__ void k_low_bits(const uint64_t *__restrict__ keys, uint64_t cnt, uint64_t mask,
                           uint32_t *__restrict__ col)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < cnt;
         i += (uint64_t)gridDim.x * blockDim.x)
        col[i] = (uint32_t)(keys[i] & mask);
}

// Checks the uploaded CSR: offsets monotone, ids < n, rows strictly sorted.
__global__ void k_check_csr(const int64_t *__restrict__ row_off, const uint32_t *__restrict__ col,
                            int64_t n, int64_t nnz, unsigned *__restrict__ bad)
{
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n;
         v += (int64_t)gridDim.x * blockDim.x) {
        int64_t s = row_off[v], e = row_off[v + 1];
        if (s < 0 || e < s || e > nnz) {
            atomicOr(bad, 1u);
            continue;
        }
        for (int64_t j = s; j < e; ++j) {
            if (col[j] >= (uint64_t)n) atomicOr(bad, 1u);
            if (j > s && col[j] <= col[j - 1]) atomicOr(bad, 2u);
        }
    }
}

GenParams make_params(int scale, uint64_t seed1, uint64_t seed2)
{
    GenParams p;
    // utils.c:60-67 make_mrg_seed
    p.seed.z[0] = (uint32_t)((seed1 & 0x3FFFFFFF) + 1);
    p.seed.z[1] = (uint32_t)(((seed1 >> 30) & 0x3FFFFFFF) + 1);
    p.seed.z[2] = (uint32_t)((seed2 & 0x3FFFFFFF) + 1);
    p.seed.z[3] = (uint32_t)(((seed2 >> 30) & 0x3FFFFFFF) + 1);
    p.seed.z[4] = (uint32_t)(((seed2 >> 60) << 4) + (seed1 >> 60) + 1);
    p.scale = scale;
    // graph_generator.c:168-178: skip(50, 7, 0) then two 62-bit values
    const uint32_t *tab = g5::mrg_skip_table_host();
    uint32_t z[5];
    memcpy(z, p.seed.z, sizeof z);
    auto apply = [&](int bi, int v) {
        const uint32_t *m = tab + ((size_t)bi * 256 + v) * 25;
        uint32_t o[5];
        for (int i = 0; i < 5; ++i) {
            uint64_t acc = 0;
            for (int k = 0; k < 5; ++k) acc = (acc + (uint64_t)m[i * 5 + k] * z[k]) % g5::kP;
            o[i] = (uint32_t)acc;
        }
        memcpy(z, o, sizeof o);
    };
    apply(8, 7);
    apply(16, 50);
    auto next = [&]() {
        uint32_t nz = (uint32_t)(((uint64_t)107374182u * z[0] + (uint64_t)104480u * z[4]) % g5::kP);
        z[4] = z[3];
        z[3] = z[2];
        z[2] = z[1];
        z[1] = z[0];
        z[0] = nz;
        return nz;
    };
    uint64_t v0 = next();
    v0 *= 0xFFFFFFFFull;
    v0 += next();
    uint64_t v1 = next();
    v1 *= 0xFFFFFFFFull;
    v1 += next();
    p.val0 = v0;
    p.val1 = v1;
    return p;
}

struct DevSkip {
    uint32_t *ptr = nullptr;
    ~DevSkip()
    {
        if (ptr) cudaFree(ptr);
    }
    g5_status load()
    {
        const size_t bytes = 24 * 256 * 25 * sizeof(uint32_t);
        G5_CUDA(cudaMalloc(&ptr, bytes));
        G5_CUDA(cudaMemcpy(ptr, g5::mrg_skip_table_host(), bytes, cudaMemcpyHostToDevice));
        return G5_OK;
    }
};

using g5::DevBuf;

}  // namespace

namespace g5 {

g5_status graph_degree(const g5_graph *g, int64_t v, int64_t *deg)
{
    int64_t ro[2];
    G5_CUDA(cudaMemcpy(ro, g->row_off + v, sizeof ro, cudaMemcpyDeviceToHost));
    *deg = ro[1] - ro[0];
    return G5_OK;
}

}  // namespace g5

namespace {

// On-disk header of the binary CSR cache (64 bytes, little-endian).
constexpr char kFileMagic[8] = {'G', '5', 'C', 'S', 'R', 0, 0, 1};  // format version 1
struct FileHeader {
    char magic[8];
    int64_t n;
    int64_t nnz;
    int32_t scale;      // Kronecker scale, -1 if not generated
    uint32_t flags;     // bit 0: generated endpoint counts follow the columns
    int64_t gen_edges;  // generated (undirected) edges, 0 if not generated
    uint8_t pad[24];
};
static_assert(sizeof(FileHeader) == 64, "graph file header is 64 bytes");

constexpr size_t kIoChunk = size_t(64) << 20;  // bytes per staged copy

// Device array -> file, through a pinned staging buffer.
g5_status stream_out(FILE *f, const void *dev, size_t bytes)
{
    void *stage = nullptr;
    if (cudaMallocHost(&stage, std::min(bytes, kIoChunk) + 1) != cudaSuccess) return G5_ERR_OOM;
    g5_status st = G5_OK;
    for (size_t off = 0; off < bytes && st == G5_OK; off += kIoChunk) {
        const size_t len = std::min(kIoChunk, bytes - off);
        if (cudaMemcpy(stage, (const char *)dev + off, len, cudaMemcpyDeviceToHost) != cudaSuccess)
            st = G5_ERR_CUDA;
        else if (fwrite(stage, 1, len, f) != len)
            st = G5_ERR_IO;
    }
    cudaFreeHost(stage);
    return st;
}

// File -> device array, through a pinned staging buffer.
g5_status stream_in(FILE *f, void *dev, size_t bytes)
{
    void *stage = nullptr;
    if (cudaMallocHost(&stage, std::min(bytes, kIoChunk) + 1) != cudaSuccess) return G5_ERR_OOM;
    g5_status st = G5_OK;
    for (size_t off = 0; off < bytes && st == G5_OK; off += kIoChunk) {
        const size_t len = std::min(kIoChunk, bytes - off);
        if (fread(stage, 1, len, f) != len)
            st = G5_ERR_IO;
        else if (cudaMemcpy((char *)dev + off, stage, len, cudaMemcpyHostToDevice) != cudaSuccess)
            st = G5_ERR_CUDA;
    }
    cudaFreeHost(stage);
    return st;
}

}  // namespace

extern "C" {

const char *g5_status_str(g5_status s)
{
    switch (s) {
    case G5_OK: return "ok";
    case G5_ERR_OOM: return "out of memory";
    case G5_ERR_CAPACITY: return "capacity exceeded";
    case G5_ERR_INVALID_ARG: return "invalid argument";
    case G5_ERR_TIMEOUT: return "timeout";
    case G5_ERR_CORRUPT_STREAM: return "corrupt codec stream";
    case G5_ERR_CUDA: return "CUDA error";
    case G5_ERR_NO_DEVICE: return "no CUDA device";
    case G5_ERR_MISMATCH: return "round-trip mismatch";
    case G5_ERR_IO: return "graph file I/O error or not a graph file";
    }
    return "unknown status";
}

uint32_t g5_version(void) { return 0x000100; }

g5_status g5_graph_create(const int64_t *row_off, const uint32_t *col, int64_t n, int64_t nnz,
                          g5_graph **out)
{
    if (!out || !row_off || (nnz > 0 && !col) || n <= 0 || nnz < 0 || n > ((int64_t)1 << 32))
        return G5_ERR_INVALID_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return G5_ERR_NO_DEVICE;
    }
    DevBuf<int64_t> ro;
    DevBuf<uint32_t> cl;
    G5_TRY(ro.alloc((size_t)n + 1));
    G5_TRY(cl.alloc((size_t)nnz));
    G5_CUDA(cudaMemcpy(ro.p, row_off, sizeof(int64_t) * (size_t)(n + 1), cudaMemcpyDefault));
    if (nnz) G5_CUDA(cudaMemcpy(cl.p, col, sizeof(uint32_t) * (size_t)nnz, cudaMemcpyDefault));
    int64_t last = 0, first = 0;
    G5_CUDA(cudaMemcpy(&first, ro.p, sizeof(int64_t), cudaMemcpyDeviceToHost));
    G5_CUDA(cudaMemcpy(&last, ro.p + n, sizeof(int64_t), cudaMemcpyDeviceToHost));
    if (first != 0 || last != nnz) return G5_ERR_INVALID_ARG;
    DevBuf<unsigned> bad;
    G5_TRY(bad.alloc(1));
    G5_CUDA(cudaMemset(bad.p, 0, sizeof(unsigned)));
    k_check_csr<<<g5::grid_for(4), 256>>>(ro.p, cl.p, n, nnz, bad.p);
    G5_CUDA(cudaGetLastError());
    unsigned hbad = 0;
    G5_CUDA(cudaMemcpy(&hbad, bad.p, sizeof hbad, cudaMemcpyDeviceToHost));
    if (hbad & 1u) return G5_ERR_INVALID_ARG;
    g5_graph *g = new g5_graph();
    cudaGetDevice(&g->device);
    g->n = n;
    g->nnz = nnz;
    g->row_off = ro.release();
    g->col = cl.release();
    *out = g;
    return G5_OK;
}

g5_status g5_kronecker_edges(int scale, uint64_t seed1, uint64_t seed2, int64_t start, int64_t end,
                             int64_t *edges_host)
{
    if (scale < 1 || scale > 32 || start < 0 || end < start || !edges_host) return G5_ERR_INVALID_ARG;
    DevSkip skip;
    G5_TRY(skip.load());
    GenParams p = make_params(scale, seed1, seed2);
    const int64_t slice = (int64_t)1 << 24;
    DevBuf<int64_t> buf;
    G5_TRY(buf.alloc((size_t)2 * (size_t)std::min<int64_t>(slice, end - start)));
    for (int64_t s = start; s < end; s += slice) {
        int64_t cnt = std::min<int64_t>(slice, end - s);
        k_gen_pairs<<<g5::grid_for(8), 256>>>(p, skip.ptr, (uint64_t)s, (uint64_t)cnt, buf.p);
        G5_CUDA(cudaGetLastError());
        G5_CUDA(cudaMemcpy(edges_host + 2 * (s - start), buf.p, sizeof(int64_t) * 2 * (size_t)cnt,
                           cudaMemcpyDeviceToHost));
    }
    return G5_OK;
}

g5_status g5_graph_generate_kronecker(int scale, int edgefactor, uint64_t seed1, uint64_t seed2,
                                      g5_graph **out)
{
    if (!out || scale < 1 || scale > 30 || edgefactor < 1) return G5_ERR_INVALID_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return G5_ERR_NO_DEVICE;
    }
    const int64_t n = (int64_t)1 << scale;
    const uint64_t m = (uint64_t)edgefactor << scale;
    const uint64_t m2 = 2 * m;
    const uint64_t mask = ((uint64_t)1 << scale) - 1;
    DevSkip skip;
    G5_TRY(skip.load());
    GenParams p = make_params(scale, seed1, seed2);

    DevBuf<uint64_t> keys, alt;
    G5_TRY(keys.alloc(m2));
    G5_TRY(alt.alloc(m2));
    k_gen_keys<<<g5::grid_for(8), 256>>>(p, skip.ptr, m, keys.p);
    G5_CUDA(cudaGetLastError());

    // sort the doubled list by (v0, v1): cpu_2d/distmatrix2d.hh:838-840
    cub::DoubleBuffer<uint64_t> db(keys.p, alt.p);
    size_t tmp_bytes = 0;
    G5_CUDA(cub::DeviceRadixSort::SortKeys(nullptr, tmp_bytes, db, (int64_t)m2, 0, 2 * scale));
    DevBuf<unsigned char> tmp;
    G5_TRY(tmp.alloc(tmp_bytes));
    G5_CUDA(cub::DeviceRadixSort::SortKeys(tmp.p, tmp_bytes, db, (int64_t)m2, 0, 2 * scale));
    uint64_t *sorted = db.Current();
    uint64_t *other = db.Alternate();

    // endpoint counts of the generated list (duplicates and self loops kept)
    DevBuf<int64_t> row_off;
    G5_TRY(row_off.alloc((size_t)n + 1));
    k_row_bounds<<<g5::grid_for(8), 256>>>(sorted, m2, scale, n, row_off.p);
    G5_CUDA(cudaGetLastError());
    DevBuf<uint32_t> end_deg;
    G5_TRY(end_deg.alloc((size_t)n));
    k_degrees_u32<<<g5::grid_for(8), 256>>>(row_off.p, n, end_deg.p);
    G5_CUDA(cudaGetLastError());

    // drop duplicates, then self loops: distmatrix2d.hh:856-1010
    DevBuf<int64_t> nsel;
    G5_TRY(nsel.alloc(1));
    size_t t2 = 0;
    G5_CUDA(cub::DeviceSelect::Unique(nullptr, t2, sorted, other, nsel.p, (int64_t)m2));
    if (t2 > tmp_bytes) {
        cudaFree(tmp.p);
        tmp.p = nullptr;
        G5_TRY(tmp.alloc(t2));
        tmp_bytes = t2;
    }
    G5_CUDA(cub::DeviceSelect::Unique(tmp.p, t2, sorted, other, nsel.p, (int64_t)m2));
    int64_t nuniq = 0;
    G5_CUDA(cudaMemcpy(&nuniq, nsel.p, sizeof nuniq, cudaMemcpyDeviceToHost));
    NotSelfLoop pred{scale, mask};
    size_t t3 = 0;
    G5_CUDA(cub::DeviceSelect::If(nullptr, t3, other, sorted, nsel.p, nuniq, pred));
    if (t3 > tmp_bytes) {
        cudaFree(tmp.p);
        tmp.p = nullptr;
        G5_TRY(tmp.alloc(t3));
        tmp_bytes = t3;
    }
    G5_CUDA(cub::DeviceSelect::If(tmp.p, t3, other, sorted, nsel.p, nuniq, pred));
    int64_t nnz = 0;
    G5_CUDA(cudaMemcpy(&nnz, nsel.p, sizeof nnz, cudaMemcpyDeviceToHost));

    k_row_bounds<<<g5::grid_for(8), 256>>>(sorted, (uint64_t)nnz, scale, n, row_off.p);
    G5_CUDA(cudaGetLastError());
    DevBuf<uint32_t> col;
    G5_TRY(col.alloc((size_t)nnz));
    k_low_bits<<<g5::grid_for(8), 256>>>(sorted, (uint64_t)nnz, mask, col.p);
    G5_CUDA(cudaGetLastError());
    G5_CUDA(cudaDeviceSynchronize());

    g5_graph *g = new g5_graph();
    cudaGetDevice(&g->device);
    g->n = n;
    g->nnz = nnz;
    g->row_off = row_off.release();
    g->col = col.release();
    g->end_deg = end_deg.release();
    g->scale = scale;
    g->gen_edges = (int64_t)m;
    *out = g;
    return G5_OK;
}

g5_status g5_graph_info(const g5_graph *g, int64_t *n, int64_t *nnz)
{
    if (!g) return G5_ERR_INVALID_ARG;
    if (n) *n = g->n;
    if (nnz) *nnz = g->nnz;
    return G5_OK;
}

g5_status g5_graph_copy_csr(const g5_graph *g, int64_t *row_off_host, uint32_t *col_host)
{
    if (!g) return G5_ERR_INVALID_ARG;
    if (row_off_host)
        G5_CUDA(cudaMemcpy(row_off_host, g->row_off, sizeof(int64_t) * (size_t)(g->n + 1),
                           cudaMemcpyDeviceToHost));
    if (col_host && g->nnz)
        G5_CUDA(cudaMemcpy(col_host, g->col, sizeof(uint32_t) * (size_t)g->nnz, cudaMemcpyDeviceToHost));
    return G5_OK;
}

g5_status g5_graph_device_csr(const g5_graph *g, const int64_t **row_off, const uint32_t **col)
{
    if (!g) return G5_ERR_INVALID_ARG;
    if (row_off) *row_off = g->row_off;
    if (col) *col = g->col;
    return G5_OK;
}

g5_status g5_graph_kronecker_info(const g5_graph *g, int *scale, int64_t *gen_edges)
{
    if (!g) return G5_ERR_INVALID_ARG;
    if (scale) *scale = g->end_deg ? g->scale : -1;
    if (gen_edges) *gen_edges = g->end_deg ? g->gen_edges : 0;
    return G5_OK;
}

g5_status g5_graph_save(const g5_graph *g, const char *path)
{
    if (!g || !path) return G5_ERR_INVALID_ARG;
    FileHeader h;
    memset(&h, 0, sizeof h);
    memcpy(h.magic, kFileMagic, sizeof h.magic);
    h.n = g->n;
    h.nnz = g->nnz;
    h.scale = g->end_deg ? g->scale : -1;
    h.flags = g->end_deg ? 1u : 0u;
    h.gen_edges = g->end_deg ? g->gen_edges : 0;
    FILE *f = fopen(path, "wb");
    if (!f) return G5_ERR_IO;
    g5_status st = G5_OK;
    if (fwrite(&h, sizeof h, 1, f) != 1) st = G5_ERR_IO;
    if (st == G5_OK) st = stream_out(f, g->row_off, sizeof(int64_t) * (size_t)(g->n + 1));
    if (st == G5_OK) st = stream_out(f, g->col, sizeof(uint32_t) * (size_t)g->nnz);
    if (st == G5_OK && g->end_deg) st = stream_out(f, g->end_deg, sizeof(uint32_t) * (size_t)g->n);
    if (fclose(f) != 0 && st == G5_OK) st = G5_ERR_IO;
    return st;
}

g5_status g5_graph_load(const char *path, g5_graph **out)
{
    if (!path || !out) return G5_ERR_INVALID_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return G5_ERR_NO_DEVICE;
    }
    FILE *f = fopen(path, "rb");
    if (!f) return G5_ERR_IO;
    struct Closer {
        FILE *f;
        ~Closer() { fclose(f); }
    } closer{f};
    FileHeader h;
    if (fread(&h, sizeof h, 1, f) != 1 || memcmp(h.magic, kFileMagic, sizeof h.magic) != 0) return G5_ERR_IO;
    if (h.n <= 0 || h.n > ((int64_t)1 << 32) || h.nnz < 0 || (h.flags & ~1u)) return G5_ERR_IO;
    // the file must hold exactly the arrays the header announces
    const uint64_t body = sizeof(int64_t) * (uint64_t)(h.n + 1) + sizeof(uint32_t) * (uint64_t)h.nnz +
                          ((h.flags & 1u) ? sizeof(uint32_t) * (uint64_t)h.n : 0);
    if (fseeko(f, 0, SEEK_END) != 0) return G5_ERR_IO;
    const off_t size = ftello(f);
    if (size < 0 || (uint64_t)size != sizeof h + body || fseeko(f, (off_t)sizeof h, SEEK_SET) != 0)
        return G5_ERR_IO;
    DevBuf<int64_t> ro;
    DevBuf<uint32_t> cl, ed;
    G5_TRY(ro.alloc((size_t)h.n + 1));
    G5_TRY(cl.alloc((size_t)h.nnz));
    G5_TRY(stream_in(f, ro.p, sizeof(int64_t) * (size_t)(h.n + 1)));
    G5_TRY(stream_in(f, cl.p, sizeof(uint32_t) * (size_t)h.nnz));
    if (h.flags & 1u) {
        G5_TRY(ed.alloc((size_t)h.n));
        G5_TRY(stream_in(f, ed.p, sizeof(uint32_t) * (size_t)h.n));
    }
    int64_t first = -1, last = -1;
    G5_CUDA(cudaMemcpy(&first, ro.p, sizeof(int64_t), cudaMemcpyDeviceToHost));
    G5_CUDA(cudaMemcpy(&last, ro.p + h.n, sizeof(int64_t), cudaMemcpyDeviceToHost));
    if (first != 0 || last != h.nnz) return G5_ERR_INVALID_ARG;
    DevBuf<unsigned> bad;
    G5_TRY(bad.alloc(1));
    G5_CUDA(cudaMemset(bad.p, 0, sizeof(unsigned)));
    k_check_csr<<<g5::grid_for(4), 256>>>(ro.p, cl.p, h.n, h.nnz, bad.p);
    G5_CUDA(cudaGetLastError());
    unsigned hbad = 0;
    G5_CUDA(cudaMemcpy(&hbad, bad.p, sizeof hbad, cudaMemcpyDeviceToHost));
    if (hbad & 1u) return G5_ERR_INVALID_ARG;
    g5_graph *g = new g5_graph();
    cudaGetDevice(&g->device);
    g->n = h.n;
    g->nnz = h.nnz;
    g->row_off = ro.release();
    g->col = cl.release();
    if (h.flags & 1u) {
        g->end_deg = ed.release();
        g->scale = h.scale;
        g->gen_edges = h.gen_edges;
    }
    *out = g;
    return G5_OK;
}

g5_status g5_graph_destroy(g5_graph *g)
{
    if (!g) return G5_ERR_INVALID_ARG;
    if (g->row_off) cudaFree(g->row_off);
    if (g->col) cudaFree(g->col);
    if (g->end_deg) cudaFree(g->end_deg);
    delete g;
    return G5_OK;
}

}  // extern "C"
