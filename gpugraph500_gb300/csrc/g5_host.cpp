// g5_host.cpp -- host-side parts of libg5bfs that are not kernels: root
// selection of the reference driver and the CpuSimd-shaped codec plugin.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <random>
#include <unordered_map>
#include <vector>

#include "g5_internal.h"
#include "g5bfs.h"

namespace {

// Process-wide device buffers of the codec plugin (grown on demand).
struct PluginState {
    std::mutex mu;
    g5_codec *codec = nullptr;
    size_t cap_n = 0;
    uint32_t *d_in = nullptr;
    uint32_t *d_out = nullptr;
    size_t cap_words = 0;
    uint32_t *h_buf = nullptr;  // pinned staging
    size_t h_cap = 0;
};

PluginState &plugin()
{
    static PluginState p;
    return p;
}

// Drops every buffer, so that the next call after a failed growth
// reallocates all of them instead of trusting stale capacities.
void reset(PluginState &p)
{
    if (p.codec) g5_codec_destroy(p.codec);
    cudaFree(p.d_in);
    cudaFree(p.d_out);
    cudaFreeHost(p.h_buf);
    p.codec = nullptr;
    p.d_in = p.d_out = p.h_buf = nullptr;
    p.cap_n = p.cap_words = p.h_cap = 0;
}

g5_status grow(PluginState &p, size_t n, size_t words)
{
    if (n > p.cap_n || !p.codec) {
        size_t c = std::max<size_t>(n, 1 << 16);
        if (p.codec) g5_codec_destroy(p.codec);
        p.codec = nullptr;
        g5_status s = g5_codec_create(c, &p.codec);
        if (s != G5_OK) return s;
        cudaFree(p.d_in);
        p.d_in = nullptr;
        if (cudaMalloc(&p.d_in, sizeof(uint32_t) * (c + 256)) != cudaSuccess) return G5_ERR_OOM;
        p.cap_n = c;
    }
    size_t w = std::max(words, g5_codec_bound(p.cap_n));
    if (w > p.cap_words) {
        cudaFree(p.d_out);
        p.d_out = nullptr;
        if (cudaMalloc(&p.d_out, sizeof(uint32_t) * w) != cudaSuccess) return G5_ERR_OOM;
        p.cap_words = w;
    }
    size_t hb = std::max(p.cap_words, p.cap_n + 256);
    if (hb > p.h_cap) {
        cudaFreeHost(p.h_buf);
        p.h_buf = nullptr;
        if (cudaMallocHost(&p.h_buf, sizeof(uint32_t) * hb) != cudaSuccess) return G5_ERR_OOM;
        p.h_cap = hb;
    }
    return G5_OK;
}

g5_status ensure(PluginState &p, size_t n, size_t words)
{
    const g5_status s = grow(p, n, words);
    if (s != G5_OK) reset(p);
    return s;
}

}  // namespace

extern "C" {

g5_status g5_select_roots(const g5_graph *g, int nroots, int64_t maxgen, int64_t *roots_host, int *found)
{
    if (!g || nroots < 0 || maxgen < 1 || (nroots && !roots_host) || !found) return G5_ERR_INVALID_ARG;
    // cpu_2d/main.cpp:351-392
    std::knuth_b gen;
    std::uniform_int_distribution<int64_t> dist(0, g->n - 1);
    std::vector<int64_t> tries;
    std::unordered_map<int64_t, int64_t> deg_cache;
    int64_t attempts = 0;
    const int64_t maxattempts = (int64_t)nroots * maxgen;
    while ((int)tries.size() < nroots && attempts < maxattempts) {
        ++attempts;
        const int64_t s = dist(gen);
        if (std::find(tries.begin(), tries.end(), s) != tries.end()) continue;
        int64_t d;
        auto it = deg_cache.find(s);
        if (it != deg_cache.end()) d = it->second;
        else {
            g5_status st = g5::graph_degree(g, s, &d);
            if (st != G5_OK) return st;
            deg_cache[s] = d;
        }
        if (d > 0) tries.push_back(s);
    }
    for (size_t i = 0; i < tries.size(); ++i) roots_host[i] = tries[i];
    *found = (int)tries.size();
    return G5_OK;
}

g5_status g5_plugin_compress(const int64_t *fq_host, size_t size, uint32_t **compressed, size_t *compressedsize,
                             uint32_t threshold, int mode)
{
    if ((size && !fq_host) || !compressed || !compressedsize || threshold == 0) return G5_ERR_INVALID_ARG;
    if (mode != G5_CODEC_D4 && mode != G5_CODEC_DM) return G5_ERR_INVALID_ARG;
    // cpusimd.hh:84-90: every id must fit in 32 bits
    for (size_t i = 0; i < size; ++i)
        if (fq_host[i] < 0 || fq_host[i] > (int64_t)0xFFFFFFFFll) return G5_ERR_INVALID_ARG;
    if (size <= threshold) {
        // cpusimd.hh:102-117: small queues travel as raw uint32
        uint32_t *o = (uint32_t *)malloc(sizeof(uint32_t) * (size ? size : 1));
        if (!o) return G5_ERR_OOM;
        for (size_t i = 0; i < size; ++i) o[i] = (uint32_t)fq_host[i];
        *compressed = o;
        *compressedsize = size;
        return G5_OK;
    }
    PluginState &p = plugin();
    std::lock_guard<std::mutex> lk(p.mu);
    g5_status s = ensure(p, size, g5_codec_bound(size));
    if (s != G5_OK) return s;
    for (size_t i = 0; i < size; ++i) p.h_buf[i] = (uint32_t)fq_host[i];
    if (cudaMemcpy(p.d_in, p.h_buf, sizeof(uint32_t) * size, cudaMemcpyHostToDevice) != cudaSuccess)
        return G5_ERR_CUDA;
    size_t words = 0;
    s = g5_codec_encode(p.codec, p.d_in, size, p.d_out, &words, mode, nullptr);
    if (s != G5_OK) return s;
    uint32_t *o = (uint32_t *)malloc(sizeof(uint32_t) * (words ? words : 1));
    if (!o) return G5_ERR_OOM;
    if (cudaMemcpy(o, p.d_out, sizeof(uint32_t) * words, cudaMemcpyDeviceToHost) != cudaSuccess) {
        free(o);
        return G5_ERR_CUDA;
    }
    *compressed = o;
    *compressedsize = words;
    return G5_OK;
}

g5_status g5_plugin_decompress(const uint32_t *compressed_host, size_t compressedsize, int64_t **uncompressed,
                               size_t *uncompressedsize, uint32_t threshold, int mode)
{
    if ((compressedsize && !compressed_host) || !uncompressed || !uncompressedsize || threshold == 0)
        return G5_ERR_INVALID_ARG;
    if (mode != G5_CODEC_D4 && mode != G5_CODEC_DM) return G5_ERR_INVALID_ARG;
    const size_t n = *uncompressedsize;
    // cpusimd.hh:169-173 isCompressed
    if (!(n > threshold && n != compressedsize)) {
        int64_t *o = (int64_t *)malloc(sizeof(int64_t) * (compressedsize ? compressedsize : 1));
        if (!o) return G5_ERR_OOM;
        for (size_t i = 0; i < compressedsize; ++i) o[i] = compressed_host[i];
        *uncompressed = o;
        *uncompressedsize = compressedsize;
        return G5_OK;
    }
    PluginState &p = plugin();
    std::lock_guard<std::mutex> lk(p.mu);
    g5_status s = ensure(p, n, compressedsize + 4);
    if (s != G5_OK) return s;
    if (cudaMemcpy(p.d_out, compressed_host, sizeof(uint32_t) * compressedsize, cudaMemcpyHostToDevice) !=
        cudaSuccess)
        return G5_ERR_CUDA;
    size_t got = 0;
    s = g5_codec_decode(p.codec, p.d_out, compressedsize, p.d_in, n, &got, mode, nullptr);
    if (s != G5_OK) return s;
    if (cudaMemcpy(p.h_buf, p.d_in, sizeof(uint32_t) * got, cudaMemcpyDeviceToHost) != cudaSuccess)
        return G5_ERR_CUDA;
    int64_t *o = (int64_t *)malloc(sizeof(int64_t) * (got ? got : 1));
    if (!o) return G5_ERR_OOM;
    for (size_t i = 0; i < got; ++i) o[i] = p.h_buf[i];
    *uncompressed = o;
    *uncompressedsize = got;
    return G5_OK;
}

}  // extern "C"
