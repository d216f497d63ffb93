// The C++ host classes of include/g5bfs.hpp on a GPU: builds the Graph500
// Kronecker graph of the given scale on the device; for the roots given runs
// g5::CudaBFS (device validator checked), one g5::Batch over all of them and
// one g5::Server query each, and writes the three sets of parents to the
// output file for comparison with the oracle (plain: int64 [root][v];
// batch: uint32 [v][root]; server: int64 [root][v]); then round-trips a queue
// longer than the threshold through g5::GpuSimd (the device codec).
// Exit code 0 = pass; otherwise the failed step.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include <cuda_runtime_api.h>

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
    const size_t n = (size_t)g.n();
    std::vector<int64_t> roots;
    for (int i = 3; i < argc; ++i) roots.push_back(std::atoll(argv[i]));
    g5::CudaBFS bfs(g);
    std::vector<std::vector<int64_t>> alone;
    for (int64_t root : roots) {
        bfs.runBFS(root);
        bool minp = false;
        if (!bfs.validate(&minp) || !minp) return 1;
        if (bfs.getPredecessor()[root] != root) return 2;
        if (std::fwrite(bfs.getPredecessor(), sizeof(int64_t), n, f) != n) return 3;
        alone.push_back(bfs.parents());
    }
    // all roots in one pipelined call: the same parents
    {
        std::vector<std::vector<int64_t>> many(roots.size(), std::vector<int64_t>(n, 7));
        std::vector<int64_t *> outs;
        for (auto &m : many) outs.push_back(m.data());
        std::vector<double> ms;
        bfs.runMany(roots, outs, &ms);
        for (size_t i = 0; i < roots.size(); ++i)
            if (many[i] != alone[i] || !(ms[i] > 0)) return 7;
    }

    g5::Batch bt({&g});
    const int R = (int)roots.size();
    uint32_t *pred_dev = nullptr;
    if (cudaMalloc((void **)&pred_dev, sizeof(uint32_t) * n * R) != cudaSuccess) return 20;
    bt.run(roots, {R}, pred_dev);
    std::vector<uint32_t> bp(n * R);
    if (cudaMemcpy(bp.data(), pred_dev, sizeof(uint32_t) * n * R, cudaMemcpyDeviceToHost) != cudaSuccess) return 21;
    cudaFree(pred_dev);
    if (std::fwrite(bp.data(), sizeof(uint32_t), n * R, f) != n * R) return 22;

    {
        g5::Server sv({&g}, (size_t)1 << 30);
        std::vector<uint64_t> tickets;
        for (int64_t root : roots) tickets.push_back(sv.submit(0, root));
        for (uint64_t t : tickets) {
            if (!sv.wait(t, 60.0)) return 30;
            double lat = -1;
            const std::vector<int64_t> p = sv.result(t, 0, &lat);
            if (p.size() != n || lat < 0) return 31;
            if (std::fwrite(p.data(), sizeof(int64_t), n, f) != n) return 32;
        }
    }
    {
        // cohort mode on the same graph: every query's parents as alone
        g5::Server sv({&g}, (size_t)1 << 30, G5_SERVE_COHORTS);
        sv.cohortPolicy(2, 1.0);
        std::vector<uint64_t> tickets;
        for (int64_t root : roots) tickets.push_back(sv.submit(0, root));
        for (size_t i = 0; i < tickets.size(); ++i) {
            if (!sv.wait(tickets[i], 60.0)) return 33;
            if (sv.result(tickets[i], 0) != alone[i]) return 34;
        }
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
    size_t m = q.size();
    c.decompress(z, (int)zs, &back, m);
    if (!back || m != q.size()) return 5;
    for (size_t i = 0; i < m; ++i)
        if (back[i] != q[i]) return 6;
    std::free(z);
    std::free(back);
    std::puts("g5bfs.hpp gpu ok");
    return 0;
}
