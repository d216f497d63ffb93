// Compiles include/g5bfs.hpp against libg5bfs and runs the parts of it that
// need no GPU: errors carry their status, the CSR is checked before any
// device work, and the codec plugin's raw path (queues up to the threshold)
// round-trips on the host with the reference plugin's ownership (malloc'd
// buffers the caller frees).  Exit code 0 = pass; otherwise the failed step.
#include <cstdio>
#include <cstdlib>

#include "g5bfs.hpp"

// stands in for the reference's Compression<int64_t, uint32_t> base class
struct PluginBase {
    virtual ~PluginBase() = default;
};

int main()
{
    try {
        g5::check(G5_ERR_INVALID_ARG, "step");
        return 1;
    } catch (const g5::Error &e) {
        if (e.code != G5_ERR_INVALID_ARG) return 2;
    }
    try {
        const int64_t ro[2] = {0, 0};
        g5::Graph g(ro, nullptr, -1, 0);  // n < 1
        return 3;
    } catch (const g5::Error &e) {
        if (e.code != G5_ERR_INVALID_ARG) return 4;
    }
    try {
        g5::Graph::load("/nonexistent-dir/graph.g5csr");
        return 5;
    } catch (const g5::Error &e) {
        if (e.code != G5_ERR_IO && e.code != G5_ERR_NO_DEVICE) return 6;
    }

    g5::GpuSimd<PluginBase> c;
    c.reconfigure(64, "s4-bp128-d4");
    if (c.mode() != G5_CODEC_DM || c.threshold() != 64 || c.name() != "gpusimd") return 7;
    g5::GpuSimd<PluginBase> d(true);
    d.reconfigure(32, "s4-bp128-d4");
    if (d.mode() != G5_CODEC_D4 || d.threshold() != 32) return 8;
    if (c.isCompressed(64, 10) || !c.isCompressed(65, 10) || c.isCompressed(100, 100)) return 9;

    int64_t q[40];
    for (int i = 0; i < 40; ++i) q[i] = 7 + 3 * i;
    uint32_t *z = nullptr;
    size_t zs = 0;
    c.compress(q, 40, &z, zs);  // 40 <= 64: raw uint32
    if (!z || zs != 40 || c.isCompressed(40, zs)) return 10;
    int64_t *back = nullptr;
    size_t n = 40;
    c.decompress(z, (int)zs, &back, n);
    if (!back || n != 40) return 11;
    for (int i = 0; i < 40; ++i)
        if (back[i] != q[i]) return 12;
    free(z);
    free(back);
    int64_t bad = -1;
    try {
        c.compress(&bad, 1, &z, zs);  // ids must fit in 32 bits
        return 13;
    } catch (const g5::Error &e) {
        if (e.code != G5_ERR_INVALID_ARG) return 14;
    }
    std::puts("g5bfs.hpp ok");
    return 0;
}
