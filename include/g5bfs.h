/*
 * g5bfs.h -- C ABI of the GB300-native gpugraph500 BFS hot path.
 *
 * One library, libg5bfs.so, with hand-written sm_103a kernels behind plain
 * C entry points: no C++ or torch types cross this boundary, only pointers,
 * sizes and status codes.  Each entry point names the reference interface it
 * replaces (paths relative to the gpugraph500 project root).
 *
 * Pointers documented as "device" must be CUDA device (or managed) memory.
 * Pointers documented as "host or device" are classified with
 * cudaPointerGetAttributes; host memory is copied inside the call.
 * Nothing here aborts the process: every failure is a g5_status.
 */
#ifndef G5BFS_H
#define G5BFS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* The reference reports CUDA failures with B40CPerror + MPI_Abort
 * (cpu_2d/cuda/cuda_bfs.cu:567-574,605-611,652-658) and codec misuse with
 * assert (cpu_2d/compression/cpusimd.hh:49-57,84-90); these codes replace
 * both. */
typedef enum g5_status {
    G5_OK = 0,
    G5_ERR_OOM = 1,            /* device or pinned allocation failed       */
    G5_ERR_CAPACITY = 2,       /* a buffer or limit is too small           */
    G5_ERR_INVALID_ARG = 3,    /* bad pointer, size, root or mode          */
    G5_ERR_TIMEOUT = 4,        /* a bounded device wait or level cap ran out */
    G5_ERR_CORRUPT_STREAM = 5, /* codec stream fails validation            */
    G5_ERR_CUDA = 6,           /* any other CUDA runtime error             */
    G5_ERR_NO_DEVICE = 7,      /* no CUDA device visible                   */
    G5_ERR_MISMATCH = 8,       /* an in-loop round-trip check failed       */
    G5_ERR_IO = 9              /* a graph file cannot be read or written, or
                                  is not a well-formed graph file          */
} g5_status;

/* Human-readable name of a status code (static storage). */
const char *g5_status_str(g5_status s);

/* Library/ABI version, 0xMMmmpp. */
uint32_t g5_version(void);

/* ------------------------------------------------------------------------ */
/* Graphs: a symmetric CSR resident in HBM                                   */
/* ------------------------------------------------------------------------ */

typedef struct g5_graph g5_graph;

/* Uploads a host CSR (int64 row offsets, n+1 entries; uint32 sorted column
 * ids, nnz entries) to the current device.  Replaces
 * CsrProblem::FromHostProblem (b40c/graph/bfs/csr_problem_2d.cuh:314-394),
 * which the reference calls from CUDA_BFS's constructor
 * (cpu_2d/cuda/cuda_bfs.cu:15-60).  Column ids must be < n and each row
 * sorted ascending without duplicates (the shape setupMatrix2 builds,
 * cpu_2d/distmatrix2d.hh:1033-1164); rows that are not sorted still give
 * valid BFS trees, but not the reference's parent choice. */
g5_status g5_graph_create(const int64_t *row_off, const uint32_t *col, int64_t n,
                          int64_t nnz, g5_graph **out);

/* Generates the Graph500 Kronecker graph of the given scale on the GPU and
 * builds its symmetric CSR there (self loops and duplicates dropped), the
 * work of make_graph (cpu_2d/main.cpp:221, cpu_2d/generator/make_graph.c:34-69)
 * plus DistMatrix2d::setupMatrix2 (cpu_2d/distmatrix2d.hh:745-1166) at 1x1.
 * n = 2^scale.  Also keeps, per vertex, the number of generated edge
 * endpoints (duplicates and self loops included) so that the Graph500 TEPS
 * edge count of a search (cpu_2d/validate/validate.h:440-443,485) can be
 * computed on the device. */
g5_status g5_graph_generate_kronecker(int scale, int edgefactor, uint64_t seed1,
                                      uint64_t seed2, g5_graph **out);

/* Copies the raw generated edge list [start, end) (int64 pairs) of a
 * Kronecker graph to host memory, generating it again on the device in
 * slices (cpu_2d/generator/graph_generator.c:157-187). */
g5_status g5_kronecker_edges(int scale, uint64_t seed1, uint64_t seed2,
                             int64_t start, int64_t end, int64_t *edges_host);

g5_status g5_graph_info(const g5_graph *g, int64_t *n, int64_t *nnz);

/* Copies the CSR back (either pointer may be NULL). */
g5_status g5_graph_copy_csr(const g5_graph *g, int64_t *row_off_host, uint32_t *col_host);

/* Device pointers of the resident CSR (for callers that run their own
 * kernels on it).  Valid until g5_graph_destroy. */
g5_status g5_graph_device_csr(const g5_graph *g, const int64_t **row_off,
                              const uint32_t **col);

g5_status g5_graph_destroy(g5_graph *g);

/* Binary CSR cache on disk, so a large graph is built once: the reference
 * rebuilds the graph on every run (generator + setupMatrix2,
 * cpu_2d/main.cpp:221-260, cpu_2d/distmatrix2d.hh:745-1166).  The file holds
 * a 64-byte header (magic "G5CSR", format version, n, nnz, Kronecker scale and
 * generated edge count when known), the int64 row offsets, the uint32
 * columns and, for generated graphs, the per-vertex generated endpoint counts
 * (little-endian).  g5_graph_load uploads it to the current device and checks
 * its structure like g5_graph_create (offsets from 0 to nnz, columns < n,
 * rows sorted without duplicates); a short, truncated or foreign file gives
 * G5_ERR_IO, a malformed CSR G5_ERR_INVALID_ARG. */
g5_status g5_graph_save(const g5_graph *g, const char *path);
g5_status g5_graph_load(const char *path, g5_graph **out);

/* Kronecker scale and generated edge count of a generated (or loaded
 * generated) graph; scale -1 and 0 edges for a CSR built from arrays. */
g5_status g5_graph_kronecker_info(const g5_graph *g, int *scale, int64_t *gen_edges);

/* Root selection of the reference driver (cpu_2d/main.cpp:351-392):
 * default-seeded std::knuth_b, uniform_int_distribution<int64_t>(0, n-1),
 * skipping repeats and CSR-degree-0 vertices, at most nroots*maxgen draws
 * (the driver uses maxgen = 32). *found = roots written. */
g5_status g5_select_roots(const g5_graph *g, int nroots, int64_t maxgen,
                          int64_t *roots_host, int *found);

/* ------------------------------------------------------------------------ */
/* Plain BFS: one root per search (the drop-in for CUDA_BFS)                 */
/* ------------------------------------------------------------------------ */

typedef struct g5_bfs g5_bfs;

enum {
    G5_CODEC_NONE = 0, /* no codec pass                                        */
    G5_CODEC_D4 = 1,   /* s4-bp128-d4: CompositeCodec<SIMDBinaryPacking<
                          SIMDIntegratedBlockPacker<CoarseDelta4SIMD>>,
                          VariableByte<true>> (codecfactory.h:103-105)        */
    G5_CODEC_DM = 2    /* s4-bp128-dm: same with Max4DeltaSIMD (:106-108); the
                          stream the reference's CpuSimd plugin actually emits,
                          see g5_plugin_compress                             */
};

typedef struct g5_bfs_config {
    double alpha;        /* top-down -> bottom-up when m_f > m_u / alpha (Beamer) */
    double beta;         /* bottom-up -> top-down when n_f < n / beta           */
    int codec;           /* G5_CODEC_*: round-trip every level's sorted queue   */
    uint32_t codec_threshold; /* raw below or at this length (cpusimd.hh:27,44) */
    int use_graph;       /* 1: level loop as one CUDA graph (conditional while
                            node); 0: host-driven loop, one sync per level       */
    int max_levels;      /* safety cap on levels (G5_ERR_TIMEOUT past it)       */
    int want_levels;     /* keep a per-vertex level array                        */
    int profile;         /* with use_graph = 0: time every launch with CUDA events
                            into g5_bfs_stats.kernel_ms                          */
    int parent_mode;     /* how a top-down level finds parents (same result):
                            0 atomicMin per edge; 1 atomicMin for vertices of
                            degree > 64, a scan of the adjacency for the rest;
                            2 as 1, but the first discoverer's atomicMin stands
                            unless the vertex is reached twice               */
    uint32_t tile_edges; /* frontier edges per top-down warp tile: a power of
                            two from 32 to 4096 (default 256)                  */
    int bu_serial;       /* adjacency entries a bottom-up lane scans alone
                            before its warp scans the rest together: 1..64
                            (default 8)                                        */
} g5_bfs_config;

/* Fills the defaults: alpha 14, beta 24, no codec, threshold 64, CUDA graph,
 * 4096 levels, no level array, no profiling, parent_mode 0. */
void g5_bfs_config_default(g5_bfs_config *cfg);

/* Per-search workspace on one graph; not thread safe (one per host thread),
 * like a CUDA_BFS instance (cpu_2d/cuda/cuda_bfs.h:39-84). */
g5_status g5_bfs_create(g5_graph *g, const g5_bfs_config *cfg, g5_bfs **out);
g5_status g5_bfs_destroy(g5_bfs *b);

typedef struct g5_bfs_stats {
    int32_t levels;           /* BFS depth + 1 (levels run)                      */
    int32_t bottom_up_levels; /* levels expanded bottom-up                        */
    int64_t visited;          /* vertices reached                                 */
    int64_t edges_td;         /* adjacency entries read top-down                  */
    int64_t edges_bu;         /* adjacency entries examined bottom-up             */
    int64_t queue_total;      /* sum of frontier queue lengths                    */
    int64_t codec_words;      /* sum of encoded words over levels                 */
    int64_t codec_values;     /* sum of values that went through the codec        */
    int64_t alg_bytes;        /* algorithmic HBM bytes of the search: per level,
                                 top-down 20|F| + 4 E + N/8; bottom-up (a sweep
                                 of the unvisited list) (2 off + 8) C + 4 E +
                                 N/8 (C candidates, off row-offset bytes); + 13
                                 or 9 bytes per vertex added (queue, parent,
                                 level)                                          */
    double device_ms;         /* device time of the search (CUDA events)          */
    double kernel_ms[8];      /* profile mode: prologue, expand, fixup, count,
                                 scan, write, codec, and the host loop's gap
                                 after each level (ms, summed)                    */
} g5_bfs_stats;

/* One BFS from root: GlobalBFS::runBFS (cpu_2d/globalbfs.hh:548-1263) at 1x1
 * with CUDA_BFS's hooks (cpu_2d/cuda/cuda_bfs.cu:230-659) followed by
 * getBackPredecessor/getPredecessor (cuda_bfs.cu:328-378).  pred_out (host or
 * device, n entries, may be NULL) receives the parent array in the
 * reference's convention: -1 unvisited, root -> root, otherwise the smallest
 * vertex of the previous level adjacent to the vertex (the parent
 * CPUBFS_bin's ascending first-writer sweep picks, cpu_2d/cpubfs_bin.cpp:
 * 143-180).  level_out (host or device, may be NULL; needs want_levels)
 * receives levels, -1 unvisited.  stats may be NULL. */
g5_status g5_bfs_run(g5_bfs *b, int64_t root, int64_t *pred_out, int32_t *level_out,
                     g5_bfs_stats *stats);

/* Asynchronous form of g5_bfs_run for a CUDA-graph workspace: launches the
 * search on the workspace's own stream and returns; g5_bfs_poll sets *done
 * once it has finished (and its status is the search's).  Parents stay in
 * the workspace (g5_bfs_device_pred).  Workspaces on one graph run
 * concurrently. */
g5_status g5_bfs_launch(g5_bfs *b, int64_t root);
g5_status g5_bfs_poll(g5_bfs *b, int *done, double *device_ms);

/* Many searches in one call, pipelined: search i+1 runs while search i's
 * parents travel to pred_out[i] (host or device, n entries each; a NULL
 * array or entry skips that copy) on a second stream, with two parent
 * buffers on the device.  The per-root loop of the reference driver
 * (cpu_2d/main.cpp:419-462: runBFS then getPredecessor for each root) with
 * the copy of one search hidden behind the next.  Host buffers should be
 * pinned (cudaMallocHost) for the copies to overlap; pageable ones still
 * give the same results.  device_ms (nullable, k entries) receives each
 * search's device time.  Same parents as g5_bfs_run root by root; afterwards
 * g5_bfs_device_pred, g5_bfs_teps_edges and g5_bfs_validate refer to the
 * last root.  The first call allocates the second parent buffer (8n bytes)
 * and builds its CUDA graph. */
g5_status g5_bfs_run_many(g5_bfs *b, const int64_t *roots, int k, int64_t *const *pred_out, double *device_ms);

/* Per-level record of the last search, 4 int64 per level: direction
 * (0 top-down, 1 bottom-up), frontier vertices, their adjacency entries, and
 * adjacency entries the expansion read.  *rows = levels written. */
g5_status g5_bfs_level_log(g5_bfs *b, int64_t *out, int max_rows, int *rows);

/* Profile mode: per launch of the last search, the kernel kind (index into
 * g5_bfs_stats.kernel_ms) and its CUDA-event time in ms. */
g5_status g5_bfs_profile_log(g5_bfs *b, int32_t *kinds, double *ms, int max_rows, int *rows);

/* Capture of the in-loop codec's output (workspaces created with codec !=
 * G5_CODEC_NONE), so that a caller can compare every level's stream with
 * the one the reference encoder produces for that level's queue (the
 * reference encodes each level's queue at cpu_2d/globalbfs.hh:853,873-877
 * and cpu_2d/vreduce.hpp:426 through cpu_2d/compression/cpusimd.hh:70-118).
 * From the next search on, each level's stream is also copied to buf_dev
 * (device, cap_words words; each stream starts at a multiple of 4 words)
 * and rec_dev (device, 4 x max_levels uint64) receives per level: the level
 * index of the encoded queue, its length, the stream's words and its offset
 * in buf_dev.  buf_dev = NULL turns the copy off.  g5_bfs_codec_captured
 * gives the levels recorded by the last search and whether a stream or
 * record did not fit (the rest were then dropped). */
g5_status g5_bfs_codec_capture(g5_bfs *b, uint32_t *buf_dev, uint64_t cap_words, uint64_t *rec_dev,
                               int max_levels);
g5_status g5_bfs_codec_captured(g5_bfs *b, int *levels, int *overflow);

/* Device pointer to the workspace's int64 parent array of the last search. */
g5_status g5_bfs_device_pred(g5_bfs *b, const int64_t **pred);

/* Graph500 TEPS edge count of the last search, computed on the device: the
 * number of generated input edges (self loops and duplicates included) with a
 * visited endpoint (validate.h:440-443,485).  Needs a generated graph. */
g5_status g5_bfs_teps_edges(g5_bfs *b, int64_t *nedge);

/* Graph500 validation of the last search on the device: parent range, root
 * is its own parent, no other self parent, every tree edge exists in the CSR,
 * level(parent) = level(child) - 1, every edge spans at most one level, and
 * every vertex adjacent to a visited vertex is visited (validate.h:248-491).
 * *valid = 1 if all hold.  If min_parent_out is not NULL it is set to 1 when
 * each parent is also the smallest previous-level neighbour (the reference
 * CPU BFS's choice). */
g5_status g5_bfs_validate(g5_bfs *b, int64_t root, int *valid, int *min_parent_out);

/* ------------------------------------------------------------------------ */
/* Batched BFS: up to 64 roots per graph with bit-sliced frontier words      */
/* ------------------------------------------------------------------------ */

typedef struct g5_batch g5_batch;

/* Workspace for batched searches over a set of graphs (one per slot). */
g5_status g5_batch_create(g5_graph *const *graphs, int ngraphs, g5_batch **out);
g5_status g5_batch_destroy(g5_batch *bt);

/* The same search as g5_batch_run with a host-driven level loop and CUDA
 * events around every launch (for profiling): kernel_ms[5] receives the
 * total ms of the count, scan, write, expand and fix-up kernels;
 * level_active, level_expand_ms, level_examined and level_dirs (nullable,
 * max_levels entries) the active vertices, the expansion ms, the adjacency
 * entries examined so far (cumulative) and the directions (bit 0 some graph
 * top-down, bit 1 some graph bottom-up) of each level;
 * *levels the levels run. */
g5_status g5_batch_profile(g5_batch *bt, const int64_t *roots_host, const int *nroots,
                           uint32_t *pred_out_dev, double *kernel_ms, int64_t *level_active,
                           double *level_expand_ms, int64_t *level_examined, int32_t *level_dirs,
                           int max_levels, int *levels);

/* Direction-switch thresholds of the batched search (defaults 14 and 24),
 * applied to each graph's union frontier. */
g5_status g5_batch_set_direction(g5_batch *bt, double alpha, double beta);

/* Runs nroots[i] (<= 64) roots on graph i, all graphs in one level loop.
 * roots holds the roots of graph 0, then graph 1, ...  Parents are written
 * as uint32 (0xFFFFFFFF unvisited, root -> root) to pred_out (device),
 * vertex-major per graph: graph 0 occupies n0 x nroots[0] entries, the
 * parent of vertex v for root j at [v * nroots[0] + j]; graph 1 follows.
 * (Each vertex's parents are contiguous, so a level's writes are
 * contiguous per warp.)  g5_batch_root_parents extracts one root's array.
 * Same parent choice as g5_bfs_run. */
g5_status g5_batch_run(g5_batch *bt, const int64_t *roots_host, const int *nroots,
                       uint32_t *pred_out_dev, double *device_ms);

/* Asynchronous form of g5_batch_run: launches the batch on the workspace's
 * stream and returns.  g5_batch_poll sets *done once it has finished (wait =
 * 1 blocks until then) and gives its device time and status.  The roots are
 * copied during the launch; pred_out_dev must stay valid until done. */
g5_status g5_batch_launch(g5_batch *bt, const int64_t *roots_host, const int *nroots, uint32_t *pred_out_dev);
g5_status g5_batch_poll(g5_batch *bt, int wait, int *done, double *device_ms);

/* One root's parents out of a vertex-major batch array of n vertices and
 * nroots parents per vertex: dst[v] = pred[v * nroots + r] (device arrays,
 * stream may be NULL). */
g5_status g5_batch_root_parents(const uint32_t *pred_dev, int64_t n, int nroots, int r, uint32_t *dst_dev,
                                void *stream);

/* Continuous batching on a batch workspace (used by the server below).
 * serve_begin gives graph g `slots[g]` (<= 64) root slots whose uint32
 * parents live in pred_dev, vertex-major per graph (slots[g] per vertex).  Each serve_step clears the
 * visited bits of the slots in retire_mask[g], starts the admitted roots
 * (adm_graph/adm_slot/adm_root, nadm entries) in their slots and runs one
 * level of every graph; active_mask[g] receives the slots whose frontier was
 * not empty in that level (a slot that was running and is not active has
 * finished: its parents are complete). */
g5_status g5_batch_serve_begin(g5_batch *bt, uint32_t *pred_dev, const int *slots);
g5_status g5_batch_serve_step(g5_batch *bt, const int32_t *adm_graph, const int32_t *adm_slot,
                              const int64_t *adm_root, int nadm, const uint64_t *retire_mask,
                              uint64_t *active_mask, double *device_ms);

/* ------------------------------------------------------------------------ */
/* Serving: resident graphs, single-root queries, continuous batching        */
/* ------------------------------------------------------------------------ */

/* The reference answers one root at a time (cpu_2d/main.cpp:419-462); the
 * server answers queries as they arrive, on graphs that stay resident.  A
 * worker thread admits queued queries into free slots and retires finished
 * ones while others run, so queries that arrive while others are on the GPU
 * start as soon as a slot is free and their work overlaps on the device.
 *   mode G5_SERVE_STREAMS: a slot is a one-root search workspace with its
 *     own stream; slots per graph = the graph's equal share of mem_budget
 *     divided by the workspace size (at most 64).
 *   mode G5_SERVE_LEVELS: a slot is a root bit of the graph's bit-sliced
 *     level loop, which is stepped one level at a time; queries join at the
 *     next level boundary; slots = share / (4 bytes x vertices), at most 64.
 *   mode G5_SERVE_AUTO: graphs of 2^25 vertices or more are served by level
 *     slots (their one-root searches would saturate the GPU first: a slot
 *     there shares every adjacency read with up to 63 other queries), the
 *     smaller ones by stream workspaces; each kind has its own worker.
 *   mode G5_SERVE_COHORTS: graphs of 2^21 vertices or more are served by
 *     cohorts, the smaller ones by stream workspaces.  A cohort graph holds
 *     two one-root workspaces and up to two batch workspaces (g5_batch,
 *     sharing one degree-ordered copy of the graph).  While fewer than four
 *     of its queries wait and none of its cohorts runs, they run alone on
 *     the one-root workspaces (a lone query finishes sooner alone); otherwise
 *     they gather, and when a batch workspace is free and 64 queries wait
 *     (or the oldest has waited 30 ms; g5_server_cohort_policy sets both),
 *     the queued queries, up to its root slots (at most 64), start together
 *     as one batched search, so under heavy load each adjacency read is
 *     shared by up to 64 queries.  Cohort graphs get the
 *     budget the other graphs leave, in proportion to their vertex counts
 *     (4 bytes per vertex and root slot, plus the workspaces and the copy).
 *     With keep_results a workspace is reused once every query on it has
 *     been released by g5_server_result.
 * Queries beyond the free slots wait in a FIFO per graph (memory-based
 * admission).  keep_results = 0 frees a slot as soon as its query finishes
 * (results are discarded). */
typedef struct g5_server g5_server;

enum { G5_SERVE_STREAMS = 0, G5_SERVE_LEVELS = 1, G5_SERVE_AUTO = 2, G5_SERVE_COHORTS = 3 };

g5_status g5_server_create(g5_graph *const *graphs, int ngraphs, size_t mem_budget,
                           int keep_results, int mode, g5_server **out);
/* As g5_server_create with the slot kind given per graph (modes[i] =
 * G5_SERVE_STREAMS, G5_SERVE_LEVELS or G5_SERVE_COHORTS). */
g5_status g5_server_create_modes(g5_graph *const *graphs, int ngraphs, size_t mem_budget,
                                 int keep_results, const int *modes, g5_server **out);
/* Cohort graphs: a cohort starts when min_roots (1..64) queries wait or
 * the oldest has waited max_wait_ms (defaults 64 and 30 ms). */
g5_status g5_server_cohort_policy(g5_server *sv, int min_roots, double max_wait_ms);
/* Slots per graph chosen by the admission rule. */
g5_status g5_server_slots(g5_server *sv, int *slots);
/* Thread safe: queues one query; *ticket identifies it. */
g5_status g5_server_submit(g5_server *sv, int graph, int64_t root, uint64_t *ticket);
/* Waits up to timeout_s seconds; *done = 1 when the query has finished. */
g5_status g5_server_wait(g5_server *sv, uint64_t ticket, double timeout_s, int *done);
/* Finished query: copies its parents (int64, -1 unvisited, root -> root;
 * pred_host may be NULL), its latency from submission to completion and its
 * queueing time, and forgets the query (frees its slot). */
g5_status g5_server_result(g5_server *sv, uint64_t ticket, int64_t *pred_host, double *latency_ms,
                           double *queue_ms);
g5_status g5_server_stats(g5_server *sv, uint64_t *steps, uint64_t *completed, double *device_ms);
g5_status g5_server_destroy(g5_server *sv);

/* ------------------------------------------------------------------------ */
/* s4-bp128 frontier codec on the device                                     */
/* ------------------------------------------------------------------------ */

typedef struct g5_codec g5_codec;

/* Upper bound on encoded words for n values. */
size_t g5_codec_bound(size_t n);

/* Workspace for values up to max_n per call. */
g5_status g5_codec_create(size_t max_n, g5_codec **out);
g5_status g5_codec_destroy(g5_codec *c);

/* IntegerCODEC::encodeArray of the named composite codec
 * (compression/cpusimd/include/compositecodec.h:31-51) on device buffers:
 * in_dev n uint32 values, out_dev >= g5_codec_bound(n) words (16-byte
 * aligned).  *out_words (host) = words written.  mode = G5_CODEC_D4 or
 * G5_CODEC_DM.  stream may be NULL (default stream). */
g5_status g5_codec_encode(g5_codec *c, const uint32_t *in_dev, size_t n, uint32_t *out_dev,
                          size_t *out_words, int mode, void *stream);

/* IntegerCODEC::decodeArray (compositecodec.h:52-71): decodes a stream of
 * `words` words into out_dev (capacity out_cap values); *out_n = values.
 * Streams that fail validation give G5_ERR_CORRUPT_STREAM. */
g5_status g5_codec_decode(g5_codec *c, const uint32_t *in_dev, size_t words, uint32_t *out_dev,
                          size_t out_cap, size_t *out_n, int mode, void *stream);

/* Asynchronous forms with the lengths in device memory, for callers that
 * keep a queue's length on the device (a level loop does) and for capture
 * in a CUDA graph: nothing is read back and the call returns after
 * enqueueing.  encode_async: n_dev (device, one uint64, at most the
 * workspace's max_n, else nothing is written and the workspace status is
 * G5_ERR_CAPACITY); the stream's words go to out_words_dev (device, one
 * uint64).  decode_async: words_dev (device) gives the stream's length;
 * the decoded count goes to out_n_dev (device).  g5_codec_status (a
 * synchronous read) gives the status of the last call on the workspace. */
g5_status g5_codec_encode_async(g5_codec *c, const uint32_t *in_dev, const uint64_t *n_dev, uint32_t *out_dev,
                                uint64_t *out_words_dev, int mode, void *stream);
g5_status g5_codec_decode_async(g5_codec *c, const uint32_t *in_dev, const uint64_t *words_dev, uint32_t *out_dev,
                                size_t out_cap, uint64_t *out_n_dev, int mode, void *stream);
g5_status g5_codec_status(g5_codec *c);

/* Many queues per call, one launch set for all of them (the reference's
 * compress/decompress run once per queue, vreduce.hpp:192-528,
 * globalbfs.hh:853-938; a level's queues or a microbench's queue set go
 * through the GPU together).  The streams are byte for byte those of
 * g5_codec_encode / g5_plugin_compress on each queue.
 *
 * encode_batch: queue q is in_dev[in_off[q] .. in_off[q+1]) (in_off on the
 * host, k+1 entries, in_off[0] = 0, total at most 2^31 values); stream q is
 * written at out_dev + out_off[q] (out_off filled by the call, k+1 entries:
 * the exclusive prefix of g5_codec_bound rounded up to 4 words, so every
 * stream starts 16-byte aligned; out_dev needs g5_codec_batch_bound words);
 * out_words[q] receives its length.  raw_threshold > 0 gives the plugin's
 * raw copy for queues of at most that many values (cpusimd.hh:102-117).
 *
 * decode_batch: stream q is in_dev[in_off[q] .. + words[q]) (in_off multiples
 * of 4) and holds n[q] values (the caller passes n out of band, as the
 * reference plugin does); value i of queue q goes to out_dev[out_off[q] + i]
 * (out_off filled: the exclusive prefix of n).  stream_ok (nullable, k
 * entries) gets 1 per stream that decoded to exactly n[q] values, 0 per
 * malformed stream; the call returns G5_ERR_CORRUPT_STREAM if any failed. */
size_t g5_codec_batch_bound(const uint64_t *in_off, int k);
g5_status g5_codec_encode_batch(g5_codec *c, const uint32_t *in_dev, const uint64_t *in_off, int k,
                                uint32_t *out_dev, uint64_t *out_off, uint64_t *out_words,
                                uint32_t raw_threshold, int mode, void *stream);
g5_status g5_codec_decode_batch(g5_codec *c, const uint32_t *in_dev, const uint64_t *in_off,
                                const uint64_t *words, const uint64_t *n, int k, uint32_t *out_dev,
                                uint64_t *out_off, int *stream_ok, uint32_t raw_threshold, int mode,
                                void *stream);

/* Same stream as g5_codec_encode, for callers that cannot allocate device
 * memory: a serving loop that must never block on or fragment the CUDA
 * allocator between requests, or a process whose device memory belongs to
 * another allocator (a framework's caching pool) with nothing left for
 * cudaMalloc.  It needs no g5_codec: its scratch is a fixed array of 12,608
 * bytes (about 12 KiB) in the library's device image, held on every GPU that
 * loads the library until the process exits, and it calls no allocating
 * function.  At most 1,048,576 values per call (more gives
 * G5_ERR_CAPACITY).  The first call on a device looks up that device's copy
 * of the array (cudaGetSymbolAddress) and keeps the address for the life of
 * the process, so make that call before any stream capture, and do not call
 * this entry point on a device again after cudaDeviceReset in the same
 * process.  All calls share the one array: calls that overlap on the GPU
 * (other streams, other host threads) race and must be serialised by the
 * caller.  This entry point has no counterpart in the reference. */
g5_status g5_codec_encode_noalloc(const uint32_t *in_dev, size_t n, uint32_t *out_dev,
                                  size_t *out_words, int mode, void *stream);

/* The CpuSimd plugin (cpu_2d/compression/cpusimd.hh:70-118): int64 host
 * queue -> *compressed (malloc'd by this call, caller frees, as the reference
 * caller does at cpu_2d/globalbfs.hh:903), raw uint32 when size <= threshold.
 * mode selects the stream; the reference plugin, whatever name it is given,
 * encodes with s4-bp128-dm because its codec member is a reference bound at
 * construction (cpusimd.hh:26,52-53), so G5_CODEC_DM matches it byte for byte. */
g5_status g5_plugin_compress(const int64_t *fq_host, size_t size, uint32_t **compressed,
                             size_t *compressedsize, uint32_t threshold, int mode);

/* cpusimd.hh:120-157: *uncompressedsize is the original length in and the
 * decoded length out; *uncompressed is malloc'd (int64). */
g5_status g5_plugin_decompress(const uint32_t *compressed_host, size_t compressedsize,
                               int64_t **uncompressed, size_t *uncompressedsize,
                               uint32_t threshold, int mode);

/* ------------------------------------------------------------------------ */
/* Frontier-bitmap OR                                                        */
/* ------------------------------------------------------------------------ */

/* dst[i] |= srcs[0][i] | ... | srcs[k-1][i] over `words` uint64 words, all
 * device pointers (srcs itself is a host array of k <= 64 device pointers):
 * the reduce callback of vreduce (cpu_2d/vreduce.hpp:112,257-259,359-361)
 * bound to CPUBFS_bin::reduce_fq_out (cpu_2d/cpubfs_bin.cpp:55-65). */
g5_status g5_bitmap_or(uint64_t *dst, const uint64_t *const *srcs, int k, size_t words,
                       void *stream);

#ifdef __cplusplus
}
#endif
#endif
