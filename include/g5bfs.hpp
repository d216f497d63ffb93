/* g5bfs.hpp -- C++ host classes over the C ABI of g5bfs.h, keeping the
 * reference's names so that a 1x1 gpugraph500 driver uses them unchanged:
 *
 *   g5::CudaBFS  runBFS(start) / getPredecessor(), the shape of CUDA_BFS
 *                (cpu_2d/cuda/cuda_bfs.h:39-84) as the driver calls it
 *                (cpu_2d/main.cpp:425-459,512);
 *   g5::GpuSimd  compress / decompress / isCompressed / reconfigure / name of
 *                the Compression<T, T_C> plugin (cpu_2d/compression/
 *                compression.hh:11-28), over g5_plugin_compress/decompress;
 *                malloc-owned buffers, freed by the caller as with the
 *                reference's cpusimd plugin (globalbfs.hh:903,
 *                vreduce.hpp:263-265).
 *
 * Header only; link with -lg5bfs.  Errors throw g5::Error (carrying the
 * g5_status) instead of the reference's abort paths; callers that must not
 * throw use the C ABI directly. */
#ifndef G5BFS_HPP
#define G5BFS_HPP

#include <cstdint>
#include <cstdlib>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "g5bfs.h"

namespace g5 {

class Error : public std::runtime_error {
public:
    g5_status code;
    Error(g5_status s, const char *what) : std::runtime_error(std::string(what) + ": " + g5_status_str(s)), code(s) {}
};

inline void check(g5_status s, const char *what)
{
    if (s != G5_OK) throw Error(s, what);
}

// A CSR resident on the current device (g5_graph), owned.
class Graph {
    g5_graph *g_ = nullptr;
    explicit Graph(g5_graph *g) : g_(g) {}

public:
    // row_off: n+1 int64 offsets; col: nnz uint32 ids, rows sorted ascending
    Graph(const int64_t *row_off, const uint32_t *col, int64_t n, int64_t nnz)
    {
        check(g5_graph_create(row_off, col, n, nnz, &g_), "g5_graph_create");
    }
    // Graph500 Kronecker graph generated and built on the GPU (seeds as the
    // reference driver's userseed1/2, cpu_2d/main.cpp:221)
    static Graph kronecker(int scale, int edgefactor = 16, uint64_t seed1 = 1, uint64_t seed2 = 2)
    {
        g5_graph *g = nullptr;
        check(g5_graph_generate_kronecker(scale, edgefactor, seed1, seed2, &g), "g5_graph_generate_kronecker");
        return Graph(g);
    }
    static Graph load(const std::string &path)
    {
        g5_graph *g = nullptr;
        check(g5_graph_load(path.c_str(), &g), "g5_graph_load");
        return Graph(g);
    }
    void save(const std::string &path) const { check(g5_graph_save(g_, path.c_str()), "g5_graph_save"); }
    int64_t n() const
    {
        int64_t n = 0, nnz = 0;
        check(g5_graph_info(g_, &n, &nnz), "g5_graph_info");
        return n;
    }
    g5_graph *get() const { return g_; }

    Graph(Graph &&o) noexcept : g_(std::exchange(o.g_, nullptr)) {}
    Graph &operator=(Graph &&o) noexcept
    {
        if (this != &o) {
            if (g_) g5_graph_destroy(g_);
            g_ = std::exchange(o.g_, nullptr);
        }
        return *this;
    }
    Graph(const Graph &) = delete;
    Graph &operator=(const Graph &) = delete;
    ~Graph()
    {
        if (g_) g5_graph_destroy(g_);
    }
};

// One-root search workspace with the backend interface the driver uses.
// The graph must outlive it.
class CudaBFS {
    g5_bfs *b_ = nullptr;
    std::vector<int64_t> pred_;
    int64_t root_ = -1;

public:
    explicit CudaBFS(const Graph &g, const g5_bfs_config *cfg = nullptr)
    {
        g5_bfs_config c;
        g5_bfs_config_default(&c);
        if (cfg) c = *cfg;
        check(g5_bfs_create(g.get(), &c, &b_), "g5_bfs_create");
        pred_.assign((size_t)g.n(), -1);
    }
    // parents into host memory: -1 unvisited, root -> root, otherwise the
    // smallest previous-level neighbour (the reference CPU BFS's choice)
    void runBFS(int64_t start, g5_bfs_stats *stats = nullptr)
    {
        check(g5_bfs_run(b_, start, pred_.data(), nullptr, stats), "g5_bfs_run");
        root_ = start;
    }
    int64_t *getPredecessor() { return pred_.data(); }
    const std::vector<int64_t> &parents() const { return pred_; }
    // every root, root i's parents into outs[i] (host or device, n entries;
    // nullptr skips it) while root i + 1 runs; pinned host buffers overlap
    void runMany(const std::vector<int64_t> &roots, const std::vector<int64_t *> &outs,
                 std::vector<double> *device_ms = nullptr)
    {
        if (!outs.empty() && outs.size() != roots.size()) throw Error(G5_ERR_INVALID_ARG, "runMany");
        if (device_ms) device_ms->assign(roots.size(), 0.0);
        check(g5_bfs_run_many(b_, roots.data(), (int)roots.size(), outs.empty() ? nullptr : outs.data(),
                              device_ms ? device_ms->data() : nullptr),
              "g5_bfs_run_many");
        if (!roots.empty()) root_ = roots.back();
    }
    // Graph500 validation of the last search on the device
    bool validate(bool *min_parent = nullptr)
    {
        int valid = 0, minp = 0;
        check(g5_bfs_validate(b_, root_, &valid, min_parent ? &minp : nullptr), "g5_bfs_validate");
        if (min_parent) *min_parent = minp != 0;
        return valid != 0;
    }
    // TEPS edge count of the last search (generated graphs)
    int64_t teps_edges()
    {
        int64_t ne = 0;
        check(g5_bfs_teps_edges(b_, &ne), "g5_bfs_teps_edges");
        return ne;
    }
    g5_bfs *get() const { return b_; }

    CudaBFS(const CudaBFS &) = delete;
    CudaBFS &operator=(const CudaBFS &) = delete;
    ~CudaBFS()
    {
        if (b_) g5_bfs_destroy(b_);
    }
};

// Batched search: up to 64 roots per graph over one or more resident graphs
// in one level loop.  Parents go to a device buffer the caller owns, per
// graph vertex-major ([v][roots of the graph]) and graphs one after another.
class Batch {
    g5_batch *bt_ = nullptr;

public:
    explicit Batch(const std::vector<const Graph *> &graphs)
    {
        std::vector<g5_graph *> gs;
        for (const Graph *g : graphs) gs.push_back(g->get());
        check(g5_batch_create(gs.data(), (int)gs.size(), &bt_), "g5_batch_create");
    }
    void set_direction(double alpha, double beta)
    {
        check(g5_batch_set_direction(bt_, alpha, beta), "g5_batch_set_direction");
    }
    // roots: graph-major, nroots[g] of them per graph; returns device ms
    double run(const std::vector<int64_t> &roots, const std::vector<int> &nroots, uint32_t *pred_dev)
    {
        double ms = 0;
        check(g5_batch_run(bt_, roots.data(), nroots.data(), pred_dev, &ms), "g5_batch_run");
        return ms;
    }
    g5_batch *get() const { return bt_; }

    Batch(const Batch &) = delete;
    Batch &operator=(const Batch &) = delete;
    ~Batch()
    {
        if (bt_) g5_batch_destroy(bt_);
    }
};

// Serving: resident graphs, queries submitted as they arrive and batched
// on the GPU (continuous batching), results fetched by ticket.
class Server {
    g5_server *sv_ = nullptr;
    std::vector<int64_t> n_;

public:
    Server(const std::vector<const Graph *> &graphs, size_t mem_budget, int mode = G5_SERVE_STREAMS,
           bool keep_results = true)
    {
        std::vector<g5_graph *> gs;
        for (const Graph *g : graphs) {
            gs.push_back(g->get());
            n_.push_back(g->n());
        }
        check(g5_server_create(gs.data(), (int)gs.size(), mem_budget, keep_results ? 1 : 0, mode, &sv_),
              "g5_server_create");
    }
    // cohort mode: a cohort starts at min_roots waiting queries or after max_wait_ms
    void cohortPolicy(int min_roots, double max_wait_ms)
    {
        check(g5_server_cohort_policy(sv_, min_roots, max_wait_ms), "g5_server_cohort_policy");
    }
    uint64_t submit(int graph, int64_t root)
    {
        uint64_t t = 0;
        check(g5_server_submit(sv_, graph, root, &t), "g5_server_submit");
        return t;
    }
    // true once the query has finished (false on timeout)
    bool wait(uint64_t ticket, double timeout_s)
    {
        int done = 0;
        check(g5_server_wait(sv_, ticket, timeout_s, &done), "g5_server_wait");
        return done != 0;
    }
    // the query's parents (graph's vertex count entries); latency in ms
    std::vector<int64_t> result(uint64_t ticket, int graph, double *latency_ms = nullptr)
    {
        std::vector<int64_t> pred((size_t)n_.at((size_t)graph));
        double lat = 0, queue = 0;
        check(g5_server_result(sv_, ticket, pred.data(), &lat, &queue), "g5_server_result");
        if (latency_ms) *latency_ms = lat;
        return pred;
    }
    g5_server *get() const { return sv_; }

    Server(const Server &) = delete;
    Server &operator=(const Server &) = delete;
    ~Server()
    {
        if (sv_) g5_server_destroy(sv_);
    }
};

// The codec plugin.  Base is the reference's Compression<int64_t, uint32_t>
// (a template parameter, so this header needs none of the reference's).
// The plugin emits the stream of the reference's cpusimd plugin: by default
// the dm form, which that plugin produces whatever name reconfigure gets;
// exact_d4 = true follows the name instead.
template <typename Base>
class GpuSimd : public Base {
    uint32_t thr_ = 64;
    int mode_ = G5_CODEC_DM;
    bool exact_d4_;

public:
    explicit GpuSimd(bool exact_d4 = false) : exact_d4_(exact_d4) {}
    void reconfigure(int threshold, std::string codec)
    {
        thr_ = (uint32_t)threshold;
        mode_ = (exact_d4_ && codec == "s4-bp128-d4") ? G5_CODEC_D4 : G5_CODEC_DM;
    }
    void compress(int64_t *fq, const size_t &size, uint32_t **compressed, size_t &compressedsize) const
    {
        check(g5_plugin_compress(fq, size, compressed, &compressedsize, thr_, mode_), "g5_plugin_compress");
    }
    void decompress(uint32_t *compressed, const int compressedsize, int64_t **uncompressed,
                    size_t &uncompressedsize) const
    {
        check(g5_plugin_decompress(compressed, (size_t)compressedsize, uncompressed, &uncompressedsize, thr_, mode_),
              "g5_plugin_decompress");
    }
    bool isCompressed(const size_t originalsize, const size_t compressedsize) const
    {
        return originalsize > thr_ && originalsize != compressedsize;
    }
    std::string name() const { return "gpusimd"; }
    uint32_t threshold() const { return thr_; }
    int mode() const { return mode_; }
};

}  // namespace g5

#endif
