// g5_internal.h -- library-internal types shared by the libg5bfs sources.
#pragma once

#include <cstdint>
#include <cstddef>

#include "g5bfs.h"

struct g5_graph {
    int device = 0;
    int64_t n = 0;
    int64_t nnz = 0;
    int64_t *row_off = nullptr;  // device, n + 1
    uint32_t *col = nullptr;     // device, nnz, rows sorted ascending
    uint32_t *end_deg = nullptr; // device, n: generated edge endpoints per vertex
                                 // (duplicates and self loops included), or null
    int scale = -1;              // Kronecker scale when generated on the device
    int64_t gen_edges = 0;       // generated (undirected) edges
};

namespace g5 {

// Host side of the MRG skip table: A^(val * 256^byte) for byte 0..23,
// 25 entries each (row-major 5x5 mod 2^31-1).
const uint32_t *mrg_skip_table_host();

// Degree of vertex v of a device graph (reads two row offsets).
g5_status graph_degree(const g5_graph *g, int64_t v, int64_t *deg);

// A batch workspace over the same graphs as `owner` that borrows owner's
// degree-ordered graph copies (owner must outlive it).
g5_status batch_create_sharing(g5_batch *owner, g5_batch **out);
// Device bytes of a batch workspace on one graph without its graph copy and
// parent output, and of the degree-ordered copy alone.
size_t batch_workspace_bytes(const g5_graph *g);
size_t batch_copy_bytes(const g5_graph *g);

}  // namespace g5
