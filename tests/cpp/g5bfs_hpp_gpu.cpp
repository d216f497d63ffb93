// The C++ host classes of include/g5bfs.hpp on a GPU: builds the Graph500
// Kronecker graph of the given scale on the device, runs g5::CudaBFS for
// each root given, checks the device validator, and writes the parents
// (int64, n per root) to the output file for comparison with the oracle;
// then round-trips a queue longer than the threshold through g5::GpuSimd
// (the device codec).  Exit code 0 = pass; otherwise the failed step.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "g5bfs.hpp"

struct PluginBase {
    virtual ~PluginBase() = default;
};

static int run(int argc, char **argv);

int main(int argc, char **argv)
{
    try {
        return run(argc, argv);
    } catch (const g5::Error &e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 50;
    }
}

static int run(int argc, char **argv)
{
    if (argc < 4) return 100;
    const int scale = std::atoi(argv[1]);
    FILE *f = std::fopen(argv[2], "wb");
    if (!f) return 101;
    g5::Graph g = g5::Graph::kronecker(scale);
    g5::CudaBFS bfs(g);
    for (int i = 3; i < argc; ++i) {
        const int64_t root = std::atoll(argv[i]);
        bfs.runBFS(root);
        bool minp = false;
        if (!bfs.validate(&minp) || !minp) return 1;
        if (bfs.getPredecessor()[root] != root) return 2;
        if (std::fwrite(bfs.getPredecessor(), sizeof(int64_t), (size_t)g.n(), f) != (size_t)g.n()) return 3;
    }
    std::fclose(f);

    g5::GpuSimd<PluginBase> c;
    c.reconfigure(64, "s4-bp128-d4");
    std::vector<int64_t> q(5000);
    for (size_t i = 0; i < q.size(); ++i) q[i] = (int64_t)(11 + 13 * i + (i * i) % 7);
    uint32_t *z = nullptr;
    size_t zs = 0;
    c.compress(q.data(), q.size(), &z, zs);
    if (!z || !c.isCompressed(q.size(), zs) || zs >= q.size()) return 4;
    int64_t *back = nullptr;
    size_t n = q.size();
    c.decompress(z, (int)zs, &back, n);
    if (!back || n != q.size()) return 5;
    for (size_t i = 0; i < n; ++i)
        if (back[i] != q[i]) return 6;
    std::free(z);
    std::free(back);
    std::puts("g5bfs.hpp gpu ok");
    return 0;
}
