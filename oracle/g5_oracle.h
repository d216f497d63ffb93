/*
 * g5_oracle.h -- CPU restatement of the gpugraph500 BFS hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA path:
 * only the test suite, the smoke check and the CPU-baseline leg of the
 * benchmark load it.  The product library (gpugraph500_gb300/libg5bfs.so)
 * never links, loads or calls it.
 *
 * Every function restates the reference algorithm from its source and cites
 * the reference file:line it follows (paths relative to the gpugraph500
 * project root).  Parity of this restatement is pinned against the reference
 * itself, compiled from its own sources into oracle/_ref (see oracle/Makefile
 * and tests/golden/make_golden.py).
 */
#ifndef G5_ORACLE_H
#define G5_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- Graph500 Kronecker generator ------------------------------------ */

/* Writes edges [start, end) of the scale-`scale` Kronecker graph as (v0, v1)
 * int64 pairs.  cpu_2d/generator/graph_generator.c:157-187 with the seed
 * spreading of cpu_2d/generator/utils.c:60-67 and the per-edge MRG skip of
 * cpu_2d/generator/splittable_mrg.c:96-119. */
void g5o_generate_kronecker(int scale, uint64_t seed1, uint64_t seed2,
                            int64_t start, int64_t end, int64_t *edges);

/* The same edges generated on `threads` host threads (edge ranges split
 * evenly; every edge is independent of the others through the MRG skip). */
void g5o_generate_kronecker_mt(int scale, uint64_t seed1, uint64_t seed2,
                               int64_t start, int64_t end, int64_t *edges, int threads);

/* Per-edge MRG state skip table entry: A^(val * 2^(8*byte_index)), 5x5 mod
 * 2^31-1, row-major.  Exposed so the GPU generator can be checked entry-wise. */
void g5o_mrg_skip_matrix(int byte_index, int val, uint32_t out[25]);

/* ---- CSR construction -------------------------------------------------- */

/* Symmetrise, sort by (v0, v1), drop self loops and duplicates:
 * cpu_2d/distmatrix2d.hh:745-784 (symmetrise), 838-840 (sort),
 * 842-1166 (row counts, prefix, columns).  row_off has n+1 entries; col
 * must hold 2*nedges entries.  Returns nnz. */
int64_t g5o_build_csr(int64_t n, const int64_t *edges, int64_t nedges,
                      int64_t *row_off, uint32_t *col);

/* The same CSR (identical arrays) built on `threads` host threads by a
 * counting sort into per-row buckets, each row then sorted and deduplicated.
 * Returns nnz, or -1 if host memory runs out. */
int64_t g5o_build_csr_mt(int64_t n, const int64_t *edges, int64_t nedges,
                         int64_t *row_off, uint32_t *col, int threads);

/* end_deg[v] = occurrences of v as an endpoint of the generated edges
 * (duplicates included, a self loop twice). */
void g5o_endpoint_counts(int64_t n, const int64_t *edges, int64_t nedges, uint32_t *end_deg,
                         int threads);

/* TEPS edge count of a search (validate.h:440-443,485) from the endpoint
 * counts: the sum of end_deg over vertices with a parent, halved -- equal to
 * the nedge_out of g5o_validate. */
int64_t g5o_teps_edges(int64_t n, const uint32_t *end_deg, const int64_t *pred);

/* ---- CPU BFS (the reference's CPUBFS_bin driven in runBFS order) ------- */

/* cpu_2d/cpubfs_bin.cpp:116-180 (setStartVertex, runLocalBFS),
 * :74-87 (setModOutgoingFQ), cpu_2d/globalbfs.hh:657-1128 (level loop).
 * pred: -1 unvisited, root -> root, else the smallest frontier neighbour.
 * level: -1 unvisited (nullable).  Returns the number of levels run. */
int g5o_bfs(int64_t n, const int64_t *row_off, const uint32_t *col,
            int64_t root, int64_t *pred, int32_t *level);

/* ---- Graph500 validator --------------------------------------------------- */

/* cpu_2d/validate/validate.h:248-491 with 64-bit bit marks.  edges is the
 * generated (un-doubled) list; both orientations are swept.  Returns 1 if
 * valid.  *nedge_out = TEPS edge count (validate.h:440-443,485).
 * depth_out (nullable) receives the depth map (-1 unvisited). */
int g5o_validate(int64_t n, const int64_t *edges, int64_t nedges,
                 int64_t root, const int64_t *pred, int64_t *nedge_out,
                 int32_t *depth_out);

/* ---- s4-bp128 frontier codec ------------------------------------------------ */

enum { G5O_DELTA4 = 0, G5O_DELTAM = 1 };

/* Upper bound on the encoded words for n values. */
size_t g5o_codec_bound(size_t n);

/* CompositeCodec<SIMDBinaryPacking<SIMDIntegratedBlockPacker<D,true>>,
 * VariableByte<true>>::encodeArray, D = CoarseDelta4SIMD (mode 0, the
 * "s4-bp128-d4" codec) or Max4DeltaSIMD (mode 1, "s4-bp128-dm").
 * compression/cpusimd/include/compositecodec.h:31-51,
 * include/simdbinarypacking.h:104-235, include/deltatemplates.h:67-120,
 * include/variablebyte.h:30-161.  Returns the number of words written. */
size_t g5o_codec_encode(const uint32_t *in, size_t n, uint32_t *out, int mode);

/* Inverse of g5o_codec_encode.  Returns the number of values decoded, or
 * (size_t)-1 on a malformed stream. */
size_t g5o_codec_decode(const uint32_t *in, size_t words, uint32_t *out,
                        size_t out_cap, int mode);

/* The CpuSimd plugin layer: raw copy when n <= thr, else the codec.
 * cpu_2d/compression/cpusimd.hh:70-118.  Returns words written. */
size_t g5o_plugin_compress(const int64_t *in, size_t n, uint32_t *out,
                           size_t thr, int mode);
/* cpu_2d/compression/cpusimd.hh:120-173.  Returns values written. */
size_t g5o_plugin_decompress(const uint32_t *in, size_t words, size_t n,
                             int64_t *out, size_t thr, int mode);

/* ---- frontier bitmap OR ------------------------------------------------------- */

/* dst[i] |= srcs[k][i] for all k: cpu_2d/cpubfs_bin.cpp:55-65. */
void g5o_bitmap_or(uint64_t *dst, const uint64_t *const *srcs, int k,
                   size_t words);

/* ---- root selection (oracle/roots.cpp) --------------------------------------- */

/* cpu_2d/main.cpp:351-392: std::knuth_b (default seed) with
 * uniform_int_distribution<int64_t>(0, n-1), skipping repeats and vertices of
 * CSR degree 0, at most nroots * maxgen tries.  Returns roots found. */
int g5o_select_roots(int64_t n, const int64_t *row_off, int nroots,
                     int64_t maxgen, int64_t *roots);

#ifdef __cplusplus
}
#endif
#endif
