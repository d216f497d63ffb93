// ref_driver.cpp -- drives the reference's own sources, compiled unmodified
// from the gpugraph500 tree against the single-rank MPI shim, to produce
// golden vectors for the oracle restatement and the CUDA path.
//
// TEST INFRASTRUCTURE ONLY (built into oracle/_ref, never into the product).
// Follows the 1x1 order of cpu_2d/main.cpp:219-248 (make_graph,
// setupMatrix2), :351-392 (roots), cpu_2d/globalbfs.hh:657-1128 (the hook
// sequence of runBFS, driven directly on CPUBFS_bin because runBFS does not
// compile for it) and cpu_2d/main.cpp:511-513 (validation).
#include <mpi.h>
#include <cstdint>
#include <algorithm>
#include <cstring>
#include <random>
#include <vector>

#include "cpubfs_bin.h"
#include "generator/make_graph.h"
#include "validate/validate.h"

namespace {

struct RefState {
    int scale = 0;
    packed_edge *edges = nullptr;
    int64_t nedges = 0;  // after setupMatrix2: the doubled, sorted list
    CPUBFS_bin::MatrixT *store = nullptr;
    CPUBFS_bin *bfs = nullptr;
};
RefState g;

void reset()
{
    delete g.bfs;
    delete g.store;
    free(g.edges);
    g = RefState();
}

}  // namespace

extern "C" {

// Generates the scale-`scale` Kronecker graph with the reference generator
// and returns the raw edge list (before symmetrisation) in out[2*M].
int64_t ref_make_graph(int scale, int edgefactor, uint64_t seed1, uint64_t seed2, int64_t *out)
{
    int64_t ne = 0;
    packed_edge *e = nullptr;
    make_graph(scale, (int64_t)edgefactor << scale, seed1, seed2, &ne, &e);
    if (out) for (int64_t i = 0; i < ne; ++i) { out[2 * i] = e[i].v0; out[2 * i + 1] = e[i].v1; }
    free(e);
    return ne;
}

// Builds the reference CSR (setupMatrix2) and a CPUBFS_bin on it from an
// edge list given as int64 pairs.  Returns the number of local rows.
int64_t ref_setup(const int64_t *edges, int64_t nedges)
{
    reset();
    g.edges = (packed_edge *)malloc(sizeof(packed_edge) * (size_t)(nedges > 0 ? nedges : 1));
    for (int64_t i = 0; i < nedges; ++i) { g.edges[i].v0 = edges[2 * i]; g.edges[i].v1 = edges[2 * i + 1]; }
    g.nedges = nedges;
    g.store = new CPUBFS_bin::MatrixT(1, 1);
    g.store->setupMatrix2(g.edges, g.nedges);
    g.bfs = new CPUBFS_bin(*g.store, 0);
    return g.store->getLocRowLength();
}

int64_t ref_nnz() { return g.store->getRowPointer()[g.store->getLocRowLength()]; }

void ref_csr(int64_t *row_off, int64_t *col)
{
    const int64_t n = g.store->getLocRowLength();
    std::memcpy(row_off, g.store->getRowPointer(), sizeof(int64_t) * (size_t)(n + 1));
    std::memcpy(col, g.store->getColumnIndex(), sizeof(int64_t) * (size_t)ref_nnz());
}

// cpu_2d/main.cpp:351-392 root selection on the reference CSR.
int ref_roots(int nroots, int64_t *roots)
{
    const int64_t vertices = g.store->getLocRowLength();
    std::knuth_b generator;
    std::uniform_int_distribution<int64_t> distribution(0, vertices - 1);
    std::vector<int64_t> tries;
    int64_t giteration = 0, maxiterations = (int64_t)nroots * 32;
    while ((int)tries.size() < nroots && giteration < maxiterations) {
        ++giteration;
        int64_t start = distribution(generator);
        if (std::find(tries.begin(), tries.end(), start) != tries.end()) continue;
        int64_t elem = 0;
        if (g.store->isLocalRow(start)) {
            int64_t loc = g.store->globaltolocalRow(start);
            elem = g.store->getRowPointer()[loc + 1] - g.store->getRowPointer()[loc];
        }
        if (elem > 0) tries.push_back(start);
    }
    for (size_t i = 0; i < tries.size(); ++i) roots[i] = tries[i];
    return (int)tries.size();
}

// One BFS in the runBFS hook order for a 1x1 grid; copies the predecessor
// array out, then runs the reference validator on it.  Returns the depth
// (levels run) and writes validity and the TEPS edge count.
int ref_bfs(int64_t root, int64_t *pred_out, int *valid, int64_t *nedge)
{
    CPUBFS_bin &b = *g.bfs;
    const int64_t n = g.store->getLocColLength();
    b.setStartVertex(root);
    int depth = 0;
    for (;;) {
        b.runLocalBFS();
        if (!b.istheresomethingnew()) break;
        uint64_t *fq = nullptr;
        long sz = 0;
        b.getOutgoingFQ(fq, sz);
        b.setModOutgoingFQ(nullptr, sz);
        uint64_t *rowfq = nullptr;
        long rowsz = 0;
        b.getOutgoingFQ(0, g.store->getLocRowLength(), rowfq, rowsz);
        long insize = rowsz;
        b.setIncommingFQ(0, g.store->getLocRowLength(), rowfq, insize);
        ++depth;
    }
    int64_t *pred = b.getPredecessor();
    std::memcpy(pred_out, pred, sizeof(int64_t) * (size_t)n);
    int64_t ne = 0;
    int level = 0;
    std::vector<int64_t> work(pred, pred + n);
    *valid = validate_bfs_result<CPUBFS_bin::MatrixT>(*g.store, g.edges, g.nedges, n, root,
                                                     work.data(), &ne, &level);
    *nedge = ne;
    return depth + 1;
}

// Runs the reference validator on a caller-supplied predecessor array.
int ref_validate(int64_t root, const int64_t *pred, int64_t *nedge)
{
    const int64_t n = g.store->getLocColLength();
    std::vector<int64_t> work(pred, pred + n);
    int64_t ne = 0;
    int level = 0;
    int ok = validate_bfs_result<CPUBFS_bin::MatrixT>(*g.store, g.edges, g.nedges, n, root,
                                                     work.data(), &ne, &level);
    *nedge = ne;
    return ok;
}

void ref_free() { reset(); }

}  // extern "C"
