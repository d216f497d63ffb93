/*
 * g5_oracle.c -- CPU restatement of the gpugraph500 BFS hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA path, never linked into
 * the product library.  Each function cites the reference file:line it
 * restates (paths relative to the gpugraph500 project root).  The parity of
 * this file is pinned against the reference compiled from its own sources
 * (oracle/_ref, built by oracle/Makefile) through tests/golden.
 */
#define _POSIX_C_SOURCE 200809L
#include "g5_oracle.h"

#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ======================================================================= */
/* Graph500 Kronecker generator                                            */
/* ======================================================================= */

/* L'Ecuyer-Blouin-Couture MRG, m = 2^31-1, k = 5, multipliers x = 107374182
 * on z1 and y = 104480 on z5 (cpu_2d/generator/splittable_mrg.c:15-34,
 * mrg_orig_step at :79-87). */
#define MRG_P 0x7FFFFFFFu
#define MRG_X 107374182u
#define MRG_Y 104480u

typedef struct { uint32_t z[5]; } mrg_t;
typedef struct { uint32_t m[25]; } mat5_t;

static mat5_t g_skip[24][256];
static int g_skip_ready = 0;

static void mat5_mul(const mat5_t *a, const mat5_t *b, mat5_t *r)
{
    mat5_t t;
    for (int i = 0; i < 5; ++i)
        for (int j = 0; j < 5; ++j) {
            uint64_t s = 0;
            for (int k = 0; k < 5; ++k)
                s = (s + (uint64_t)a->m[i * 5 + k] * b->m[k * 5 + j]) % MRG_P;
            t.m[i * 5 + j] = (uint32_t)s;
        }
    *r = t;
}

/* The skip table holds A^(v * 256^k); the reference ships it precomputed
 * (cpu_2d/generator/mrg_transitions.c, produced by dump_mrg_powers); here it
 * is recomputed from the one-step matrix A. */
static void skip_fill(void);
static pthread_once_t g_skip_once = PTHREAD_ONCE_INIT;

static void skip_init(void)
{
    if (!g_skip_ready) pthread_once(&g_skip_once, skip_fill);
}

static void skip_fill(void)
{
    mat5_t a;
    memset(&a, 0, sizeof a);
    a.m[0] = MRG_X; a.m[4] = MRG_Y;
    a.m[5] = 1; a.m[11] = 1; a.m[17] = 1; a.m[23] = 1;
    mat5_t base = a; /* A^(256^k) */
    for (int k = 0; k < 24; ++k) {
        mat5_t id;
        memset(&id, 0, sizeof id);
        for (int i = 0; i < 5; ++i) id.m[i * 6] = 1;
        g_skip[k][0] = id;
        for (int v = 1; v < 256; ++v) mat5_mul(&g_skip[k][v - 1], &base, &g_skip[k][v]);
        mat5_t nb;
        mat5_mul(&g_skip[k][255], &base, &nb);
        base = nb;
    }
    g_skip_ready = 1;
}

void g5o_mrg_skip_matrix(int byte_index, int val, uint32_t out[25])
{
    skip_init();
    memcpy(out, g_skip[byte_index][val].m, 25 * sizeof(uint32_t));
}

/* x mod 2^31-1 for any 64-bit x (2^31 = 1 mod p, so fold the high bits in
 * twice); the same residue as the reference's `%`, computed without a
 * division. */
static inline uint32_t fold31(uint64_t x)
{
    x = (x & MRG_P) + (x >> 31);
    x = (x & MRG_P) + (x >> 31);
    return (uint32_t)(x >= MRG_P ? x - MRG_P : x);
}

static void mrg_apply(const mat5_t *m, mrg_t *s)
{
    uint32_t o[5];
    for (int i = 0; i < 5; ++i) {
        /* each product < 2^62 folds below 2^32, so five of them sum below 2^35 */
        uint64_t acc = 0;
        for (int k = 0; k < 5; ++k) {
            const uint64_t p = (uint64_t)m->m[i * 5 + k] * s->z[k];
            acc += (p & MRG_P) + (p >> 31);
        }
        o[i] = fold31(acc);
    }
    memcpy(s->z, o, sizeof o);
}

/* splittable_mrg.c:96-119: the exponent is a 192-bit word split in 3x64. */
static void mrg_skip(mrg_t *s, uint64_t hi, uint64_t mid, uint64_t lo)
{
    for (int b = 0; lo; ++b, lo >>= 8) if (lo & 0xFF) mrg_apply(&g_skip[b][lo & 0xFF], s);
    for (int b = 8; mid; ++b, mid >>= 8) if (mid & 0xFF) mrg_apply(&g_skip[b][mid & 0xFF], s);
    for (int b = 16; hi; ++b, hi >>= 8) if (hi & 0xFF) mrg_apply(&g_skip[b][hi & 0xFF], s);
}

/* splittable_mrg.c:79-87,123-127 */
static uint32_t mrg_next(mrg_t *s)
{
    uint32_t nz = fold31((uint64_t)MRG_X * s->z[0] + (uint64_t)MRG_Y * s->z[4]);
    s->z[4] = s->z[3]; s->z[3] = s->z[2]; s->z[2] = s->z[1]; s->z[1] = s->z[0];
    s->z[0] = nz;
    return nz;
}

/* graph_generator.c:45-80 with SPK_NOISE_LEVEL 0: a = .57, b = c = .19. */
static int bernoulli4(mrg_t *s)
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

static uint64_t bitrev64(uint64_t x)
{
    x = ((x >> 1) & 0x5555555555555555ull) | ((x & 0x5555555555555555ull) << 1);
    x = ((x >> 2) & 0x3333333333333333ull) | ((x & 0x3333333333333333ull) << 2);
    x = ((x >> 4) & 0x0F0F0F0F0F0F0F0Full) | ((x & 0x0F0F0F0F0F0F0F0Full) << 4);
    x = ((x >> 8) & 0x00FF00FF00FF00FFull) | ((x & 0x00FF00FF00FF00FFull) << 8);
    x = ((x >> 16) & 0x0000FFFF0000FFFFull) | ((x & 0x0000FFFF0000FFFFull) << 16);
    return (x >> 32) | (x << 32);
}

/* graph_generator.c:106-119 (hash scramble of the vertex labels). */
static int64_t scramble(int64_t v0, int lg, uint64_t val0, uint64_t val1)
{
    uint64_t v = (uint64_t)v0;
    v += val0 + val1;
    v *= (val0 | 0x4519840211493211ull);
    v = bitrev64(v) >> (64 - lg);
    v *= (val1 | 0x3050852102C843A5ull);
    v = bitrev64(v) >> (64 - lg);
    return (int64_t)v;
}

typedef struct {
    mrg_t seed;
    uint64_t val0, val1;
    int scale;
} gen_ctx_t;

/* utils.c:60-67 make_mrg_seed and graph_generator.c:168-178 scrambling values */
static void gen_setup(gen_ctx_t *c, int scale, uint64_t seed1, uint64_t seed2)
{
    skip_init();
    c->scale = scale;
    c->seed.z[0] = (uint32_t)((seed1 & 0x3FFFFFFF) + 1);
    c->seed.z[1] = (uint32_t)(((seed1 >> 30) & 0x3FFFFFFF) + 1);
    c->seed.z[2] = (uint32_t)((seed2 & 0x3FFFFFFF) + 1);
    c->seed.z[3] = (uint32_t)(((seed2 >> 30) & 0x3FFFFFFF) + 1);
    c->seed.z[4] = (uint32_t)(((seed2 >> 60) << 4) + (seed1 >> 60) + 1);
    mrg_t t = c->seed;
    mrg_skip(&t, 50, 7, 0);
    uint64_t v0 = mrg_next(&t);
    v0 *= 0xFFFFFFFFull;
    v0 += mrg_next(&t);
    uint64_t v1 = mrg_next(&t);
    v1 *= 0xFFFFFFFFull;
    v1 += mrg_next(&t);
    c->val0 = v0;
    c->val1 = v1;
}

/* Edges [start, end).  Edge ei draws from the seed skipped by ei * 2^64
 * steps (graph_generator.c:157-187 calls mrg_skip(&state, 0, ei, 0)).  The
 * skip is a product of commuting powers of the step matrix, one per byte of
 * ei, so the state after the bytes above the lowest is shared by 256
 * consecutive edges and is computed once for them; each edge then applies
 * only its lowest byte.  Same states, same edges as skipping every edge from
 * the seed. */
static void gen_range(const gen_ctx_t *c, int64_t start, int64_t end, int64_t *edges)
{
    const int64_t nverts = (int64_t)1 << c->scale;
    mrg_t base = c->seed;
    int64_t base_hi = -1;
    for (int64_t ei = start; ei < end; ++ei) {
        if ((ei >> 8) != base_hi) {
            base_hi = ei >> 8;
            base = c->seed;
            uint64_t hi = (uint64_t)ei >> 8;
            for (int b = 9; hi; ++b, hi >>= 8) if (hi & 0xFF) mrg_apply(&g_skip[b][hi & 0xFF], &base);
        }
        mrg_t s = base;
        if (ei & 0xFF) mrg_apply(&g_skip[8][ei & 0xFF], &s);
        /* graph_generator.c:122-151 make_one_edge with clip-and-flip */
        int64_t bs = 0, bt = 0, nv = nverts;
        while (nv > 1) {
            int sq = bernoulli4(&s);
            int so = sq / 2, to = sq % 2;
            if (bs == bt && so > to) { int tmp = so; so = to; to = tmp; }
            nv /= 2;
            bs += nv * so;
            bt += nv * to;
        }
        edges[2 * (ei - start)] = scramble(bs, c->scale, c->val0, c->val1);
        edges[2 * (ei - start) + 1] = scramble(bt, c->scale, c->val0, c->val1);
    }
}

void g5o_generate_kronecker(int scale, uint64_t seed1, uint64_t seed2,
                            int64_t start, int64_t end, int64_t *edges)
{
    gen_ctx_t c;
    gen_setup(&c, scale, seed1, seed2);
    gen_range(&c, start, end, edges);
}

/* ---- host threads ---------------------------------------------------------- */

typedef void (*par_fn)(void *ctx, int tid, int nthreads);
typedef struct { par_fn fn; void *ctx; int tid, n; } par_arg_t;

static void *par_tramp(void *p)
{
    par_arg_t *a = (par_arg_t *)p;
    a->fn(a->ctx, a->tid, a->n);
    return NULL;
}

/* Runs fn(ctx, t, T) for t = 0..T-1 on T host threads (the caller's is t = 0). */
static void run_parallel(int T, par_fn fn, void *ctx)
{
    if (T < 1) T = 1;
    if (T > 256) T = 256;
    pthread_t th[256];
    par_arg_t arg[256];
    int started = 1;
    for (int t = 1; t < T; ++t) {
        arg[t].fn = fn; arg[t].ctx = ctx; arg[t].tid = t; arg[t].n = T;
        if (pthread_create(&th[t], NULL, par_tramp, &arg[t]) != 0) break;
        started = t + 1;
    }
    /* threads that could not be started: their shares run here */
    for (int t = started; t < T; ++t) fn(ctx, t, T);
    fn(ctx, 0, T);
    for (int t = 1; t < started; ++t) pthread_join(th[t], NULL);
}

static void split(int64_t n, int tid, int T, int64_t *lo, int64_t *hi)
{
    *lo = n * tid / T;
    *hi = n * (tid + 1) / T;
}

typedef struct { gen_ctx_t g; int64_t start, end; int64_t *edges; } gen_job_t;

static void gen_worker(void *p, int tid, int T)
{
    gen_job_t *j = (gen_job_t *)p;
    int64_t lo, hi;
    split(j->end - j->start, tid, T, &lo, &hi);
    gen_range(&j->g, j->start + lo, j->start + hi, j->edges + 2 * lo);
}

void g5o_generate_kronecker_mt(int scale, uint64_t seed1, uint64_t seed2,
                               int64_t start, int64_t end, int64_t *edges, int threads)
{
    gen_job_t j;
    gen_setup(&j.g, scale, seed1, seed2);
    j.start = start;
    j.end = end;
    j.edges = edges;
    run_parallel(threads, gen_worker, &j);
}

/* ======================================================================= */
/* CSR build                                                               */
/* ======================================================================= */

static int cmp_u64(const void *a, const void *b)
{
    uint64_t x = *(const uint64_t *)a, y = *(const uint64_t *)b;
    return (x > y) - (x < y);
}

/* distmatrix2d.hh:752-784 appends the reversed copy of every edge; :838-840
 * sorts by (v0, v1); :856-903 counts per row the entries that are neither a
 * self loop nor equal to the previous column; :905-910 prefix sums; :966-1010
 * writes the columns. */
int64_t g5o_build_csr(int64_t n, const int64_t *edges, int64_t nedges,
                      int64_t *row_off, uint32_t *col)
{
    int64_t m2 = 2 * nedges;
    uint64_t *keys = (uint64_t *)malloc((size_t)(m2 > 0 ? m2 : 1) * sizeof(uint64_t));
    for (int64_t i = 0; i < nedges; ++i) {
        uint64_t a = (uint64_t)edges[2 * i], b = (uint64_t)edges[2 * i + 1];
        keys[i] = (a << 32) | b;
        keys[nedges + i] = (b << 32) | a;
    }
    qsort(keys, (size_t)m2, sizeof(uint64_t), cmp_u64);
    int64_t nnz = 0, j = 0;
    row_off[0] = 0;
    for (int64_t v = 0; v < n; ++v) {
        int64_t last = -1;
        while (j < m2 && (int64_t)(keys[j] >> 32) == v) {
            int64_t w = (int64_t)(keys[j] & 0xFFFFFFFFu);
            if (w != v && w != last) col[nnz++] = (uint32_t)w;
            last = w;
            ++j;
        }
        row_off[v + 1] = nnz;
    }
    free(keys);
    return nnz;
}

/* The same CSR on host threads, by counting instead of one global sort:
 * count each vertex's non-loop endpoints, scatter the neighbours into per-row
 * buckets, then sort each row and drop duplicates.  Row v ends up as the
 * ascending distinct neighbours of v other than v itself, which is exactly
 * what the sort-based build above (the reference's order of work) leaves, so
 * the arrays are identical; only the work is divided differently. */
typedef struct {
    int64_t n, nedges;
    const int64_t *edges;
    uint64_t *cur;   /* n + 1: bucket starts, then scatter cursors */
    uint64_t *start; /* n + 1: bucket starts (kept) */
    uint32_t *tmp;   /* 2 * nedges bucket entries */
    int64_t *row_off;
    uint32_t *col;
    int phase;
} csr_job_t;

static int cmp_u32(const void *a, const void *b)
{
    uint32_t x = *(const uint32_t *)a, y = *(const uint32_t *)b;
    return (x > y) - (x < y);
}

static void sort_u32(uint32_t *x, int64_t n)
{
    if (n <= 24) {
        for (int64_t i = 1; i < n; ++i) {
            uint32_t v = x[i];
            int64_t j = i;
            while (j > 0 && x[j - 1] > v) { x[j] = x[j - 1]; --j; }
            x[j] = v;
        }
    } else {
        qsort(x, (size_t)n, sizeof(uint32_t), cmp_u32);
    }
}

static void csr_worker(void *p, int tid, int T)
{
    csr_job_t *j = (csr_job_t *)p;
    int64_t lo, hi;
    if (j->phase == 0) { /* endpoint counts */
        split(j->nedges, tid, T, &lo, &hi);
        for (int64_t i = lo; i < hi; ++i) {
            int64_t a = j->edges[2 * i], b = j->edges[2 * i + 1];
            if (a == b) continue;
            __atomic_fetch_add(&j->cur[a + 1], 1, __ATOMIC_RELAXED);
            __atomic_fetch_add(&j->cur[b + 1], 1, __ATOMIC_RELAXED);
        }
    } else if (j->phase == 1) { /* scatter */
        split(j->nedges, tid, T, &lo, &hi);
        for (int64_t i = lo; i < hi; ++i) {
            int64_t a = j->edges[2 * i], b = j->edges[2 * i + 1];
            if (a == b) continue;
            j->tmp[__atomic_fetch_add(&j->cur[a], 1, __ATOMIC_RELAXED)] = (uint32_t)b;
            j->tmp[__atomic_fetch_add(&j->cur[b], 1, __ATOMIC_RELAXED)] = (uint32_t)a;
        }
    } else if (j->phase == 2) { /* sort and dedup each row in place; count */
        /* rows interleaved in blocks of 4096 so the heavy low rows spread */
        for (int64_t b0 = (int64_t)tid * 4096; b0 < j->n; b0 += (int64_t)T * 4096) {
            int64_t b1 = b0 + 4096 < j->n ? b0 + 4096 : j->n;
            for (int64_t v = b0; v < b1; ++v) {
                uint32_t *r = j->tmp + j->start[v];
                int64_t len = (int64_t)(j->start[v + 1] - j->start[v]);
                sort_u32(r, len);
                int64_t k = 0;
                for (int64_t i = 0; i < len; ++i)
                    if (k == 0 || r[i] != r[k - 1]) r[k++] = r[i];
                j->cur[v] = (uint64_t)k;
            }
        }
    } else { /* copy the distinct entries to their final place */
        for (int64_t b0 = (int64_t)tid * 4096; b0 < j->n; b0 += (int64_t)T * 4096) {
            int64_t b1 = b0 + 4096 < j->n ? b0 + 4096 : j->n;
            for (int64_t v = b0; v < b1; ++v)
                memcpy(j->col + j->row_off[v], j->tmp + j->start[v],
                       (size_t)(j->row_off[v + 1] - j->row_off[v]) * sizeof(uint32_t));
        }
    }
}

int64_t g5o_build_csr_mt(int64_t n, const int64_t *edges, int64_t nedges,
                         int64_t *row_off, uint32_t *col, int threads)
{
    csr_job_t j;
    j.n = n;
    j.nedges = nedges;
    j.edges = edges;
    j.row_off = row_off;
    j.col = col;
    j.cur = (uint64_t *)calloc((size_t)n + 2, sizeof(uint64_t));
    j.start = (uint64_t *)malloc(((size_t)n + 2) * sizeof(uint64_t));
    j.tmp = NULL;
    if (!j.cur || !j.start) { free(j.cur); free(j.start); return -1; }
    j.phase = 0;
    run_parallel(threads, csr_worker, &j);
    for (int64_t v = 0; v < n; ++v) j.cur[v + 1] += j.cur[v];
    memcpy(j.start, j.cur, ((size_t)n + 1) * sizeof(uint64_t));
    j.tmp = (uint32_t *)malloc((size_t)(j.start[n] ? j.start[n] : 1) * sizeof(uint32_t));
    if (!j.tmp) { free(j.cur); free(j.start); return -1; }
    j.phase = 1;
    run_parallel(threads, csr_worker, &j);
    j.phase = 2;
    run_parallel(threads, csr_worker, &j);
    row_off[0] = 0;
    for (int64_t v = 0; v < n; ++v) row_off[v + 1] = row_off[v] + (int64_t)j.cur[v];
    j.phase = 3;
    run_parallel(threads, csr_worker, &j);
    free(j.tmp);
    free(j.cur);
    free(j.start);
    return row_off[n];
}

/* Generated endpoints per vertex: end_deg[v] = occurrences of v in the edge
 * list (a self loop counts twice), duplicates included. */
typedef struct { const int64_t *edges; int64_t nedges; uint32_t *deg; } ecount_job_t;

static void ecount_worker(void *p, int tid, int T)
{
    ecount_job_t *j = (ecount_job_t *)p;
    int64_t lo, hi;
    split(j->nedges, tid, T, &lo, &hi);
    for (int64_t i = lo; i < hi; ++i) {
        __atomic_fetch_add(&j->deg[j->edges[2 * i]], 1, __ATOMIC_RELAXED);
        __atomic_fetch_add(&j->deg[j->edges[2 * i + 1]], 1, __ATOMIC_RELAXED);
    }
}

void g5o_endpoint_counts(int64_t n, const int64_t *edges, int64_t nedges, uint32_t *end_deg,
                         int threads)
{
    memset(end_deg, 0, (size_t)n * sizeof(uint32_t));
    ecount_job_t j = {edges, nedges, end_deg};
    run_parallel(threads, ecount_worker, &j);
}

/* validate.h:440-443,485: the TEPS edge count is the number of generated
 * edge orientations (a, b), both orientations of every edge swept, whose
 * first endpoint has a parent, halved.  Each vertex v is the first endpoint
 * of end_deg[v] orientations, so the count is the sum of end_deg over the
 * visited vertices, halved: the figure g5o_validate returns, without the
 * edge sweep. */
int64_t g5o_teps_edges(int64_t n, const uint32_t *end_deg, const int64_t *pred)
{
    uint64_t s = 0;
    for (int64_t v = 0; v < n; ++v)
        if (pred[v] != -1) s += end_deg[v];
    return (int64_t)(s / 2);
}

/* ======================================================================= */
/* CPU BFS                                                                 */
/* ======================================================================= */

int g5o_bfs(int64_t n, const int64_t *row_off, const uint32_t *col,
            int64_t root, int64_t *pred, int32_t *level)
{
    int64_t w64 = (n + 63) / 64;
    uint64_t *visited = (uint64_t *)calloc((size_t)w64 + 1, 8);
    uint64_t *fq_in = (uint64_t *)calloc((size_t)w64 + 1, 8);
    uint64_t *fq_out = (uint64_t *)calloc((size_t)w64 + 1, 8);
    /* cpubfs_bin.cpp:116-141 setStartVertex */
    for (int64_t v = 0; v < n; ++v) pred[v] = -1;
    if (level) for (int64_t v = 0; v < n; ++v) level[v] = -1;
    fq_in[root >> 6] = 1ull << (root & 63);
    visited[root >> 6] = 1ull << (root & 63);
    pred[root] = root;
    if (level) level[root] = 0;
    int depth = 0;
    for (;;) {
        /* cpubfs_bin.cpp:143-180 runLocalBFS: sources in ascending order,
         * first writer wins */
        memset(fq_out, 0, (size_t)w64 * 8);
        for (int64_t i = 0; i < w64; ++i) {
            uint64_t w = fq_in[i];
            while (w) {
                int ii = __builtin_ctzll(w);
                w &= w - 1;
                int64_t u = i * 64 + ii;
                for (int64_t e = row_off[u]; e < row_off[u + 1]; ++e) {
                    uint32_t v = col[e];
                    uint64_t bit = 1ull << (v & 63);
                    if (!(visited[v >> 6] & bit) && !(fq_out[v >> 6] & bit)) {
                        fq_out[v >> 6] |= bit;
                        pred[v] = u;
                    }
                }
            }
        }
        /* cpubfs_bin.cpp:119-129 istheresomethingnew; globalbfs.hh:708-740 */
        int any = 0;
        for (int64_t i = 0; i < w64; ++i) if (fq_out[i]) { any = 1; break; }
        if (!any) break;
        ++depth;
        /* cpubfs_bin.cpp:74-87 setModOutgoingFQ, :109-114 setIncommingFQ */
        for (int64_t i = 0; i < w64; ++i) {
            visited[i] |= fq_out[i];
            fq_in[i] = fq_out[i];
            if (level) {
                uint64_t w = fq_out[i];
                while (w) {
                    int ii = __builtin_ctzll(w);
                    w &= w - 1;
                    level[i * 64 + ii] = depth;
                }
            }
        }
    }
    free(visited); free(fq_in); free(fq_out);
    return depth + 1;
}

/* ======================================================================= */
/* Validator                                                               */
/* ======================================================================= */

int g5o_validate(int64_t n, const int64_t *edges, int64_t nedges,
                 int64_t root, const int64_t *pred, int64_t *nedge_out,
                 int32_t *depth_out)
{
    int ok = 1;
    *nedge_out = 0;
    /* validate.h:69-105 value ranges; :258-270 root range */
    for (int64_t v = 0; v < n; ++v)
        if (pred[v] < -1 || pred[v] >= n) return 0;
    if (root < 0 || root >= n) return 0;
    /* validate.h:284-295 root is its own parent */
    if (pred[root] != root) ok = 0;
    /* validate.h:299-342 nobody else is its own parent */
    for (int64_t v = 0; v < n; ++v)
        if (v != root && pred[v] == v) ok = 0;
    /* validate.h:110-242 depth map: depth[v] = depth[pred[v]] + 1, iterated
     * until stable; a mismatch with an existing depth fails. */
    int32_t *depth = (int32_t *)malloc((size_t)(n > 0 ? n : 1) * sizeof(int32_t));
    for (int64_t v = 0; v < n; ++v) depth[v] = -1;
    depth[root] = 0;
    for (int64_t iter = 0;; ++iter) {
        int changed = 0;
        for (int64_t v = 0; v < n; ++v) {
            if (v == root || pred[v] == -1) continue;
            int32_t pd = depth[pred[v]];
            if (pd < 0) continue;
            if (depth[v] >= 0 && depth[v] != pd + 1) ok = 0;
            else if (depth[v] < 0) { depth[v] = pd + 1; changed = 1; }
        }
        if (!changed || iter > n) break;
    }
    /* every vertex with a parent must have reached a depth (no cycles) */
    for (int64_t v = 0; v < n; ++v)
        if (pred[v] != -1 && depth[v] < 0) ok = 0;
    /* validate.h:401-486 edge sweep over both orientations: levels differ by
     * at most one, tree edges exist, visited edge count. */
    uint64_t *mark = (uint64_t *)calloc((size_t)(n / 64 + 2), 8);
    int64_t visit_count = 0;
    for (int64_t i = 0; i < 2 * nedges; ++i) {
        int64_t a, b;
        if (i < nedges) { a = edges[2 * i]; b = edges[2 * i + 1]; }
        else { a = edges[2 * (i - nedges) + 1]; b = edges[2 * (i - nedges)]; }
        int32_t da = depth[a], db = depth[b];
        if ((da < 0) != (db < 0)) ok = 0;
        else if (da >= 0 && (da - db > 1 || db - da > 1)) ok = 0;
        if (pred[b] == a) mark[b >> 6] |= 1ull << (b & 63);
        if (pred[a] != -1) ++visit_count;
    }
    /* validate.h:456-471 coverage: each visited non-root has its tree edge */
    for (int64_t v = 0; v < n; ++v)
        if (pred[v] != -1 && v != root && !(mark[v >> 6] & (1ull << (v & 63)))) ok = 0;
    *nedge_out = visit_count / 2;
    if (depth_out) memcpy(depth_out, depth, (size_t)n * sizeof(int32_t));
    free(mark);
    free(depth);
    return ok;
}

/* ======================================================================= */
/* s4-bp128 codec                                                          */
/* ======================================================================= */

#define COOKIE 123456u

size_t g5o_codec_bound(size_t n)
{
    /* 4 header words + per 2048 values 4 header words + 128 words per
     * miniblock at b = 32 + 5 bytes per tail value */
    size_t mb = n / 128;
    return 4 + 4 * (mb / 16 + 1) + mb * 128 + ((n % 128) * 5 + 3) / 4 + 4;
}

static uint32_t bits_of(uint32_t v) { return v ? 32u - (uint32_t)__builtin_clz(v) : 0u; }

/* The 4-lane delta of deltatemplates.h: CoarseDelta4SIMD (:67-84) subtracts
 * the previous vector lane-wise; Max4DeltaSIMD (:103-120) subtracts lane 3
 * of the previous vector from every lane. */
static inline uint32_t delta_of(const uint32_t *cur, const uint32_t *prev, int l, int mode)
{
    return cur[l] - (mode == G5O_DELTAM ? prev[3] : prev[l]);
}

/* simdbinarypacking.h:118-132 maxbits: OR of all 128 deltas, gccbits. */
static uint32_t mb_bits(const uint32_t *x, const uint32_t *prev, int mode)
{
    uint32_t acc = 0;
    for (int j = 0; j < 32; ++j) {
        const uint32_t *p = j ? x + 4 * (j - 1) : prev;
        for (int l = 0; l < 4; ++l) acc |= delta_of(x + 4 * j, p, l, mode);
    }
    return bits_of(acc);
}

/* ipackwithoutmask<b>: each lane packs its 32 values LSB-first in b-bit
 * fields; word w of lane l lands at out[4w + l].  b = 32 stores the raw
 * values (simdintegratedbitpacking.cpp:16381), b = 0 stores nothing. */
static void mb_pack(const uint32_t *x, const uint32_t *prev, uint32_t b, uint32_t *out, int mode)
{
    if (b == 0) return;
    if (b == 32) { memcpy(out, x, 128 * sizeof(uint32_t)); return; }
    memset(out, 0, 4 * b * sizeof(uint32_t));
    for (int l = 0; l < 4; ++l) {
        uint32_t bitpos = 0;
        for (int j = 0; j < 32; ++j) {
            const uint32_t *p = j ? x + 4 * (j - 1) : prev;
            uint32_t d = delta_of(x + 4 * j, p, l, mode);
            uint32_t w = bitpos >> 5, s = bitpos & 31;
            out[4 * w + l] |= d << s;
            if (s + b > 32) out[4 * (w + 1) + l] |= d >> (32 - s);
            bitpos += b;
        }
    }
}

static void mb_unpack(const uint32_t *in, uint32_t b, uint32_t *prev /* in/out, 4 */,
                      uint32_t *x, int mode)
{
    if (b == 32) {
        memcpy(x, in, 128 * sizeof(uint32_t));
        memcpy(prev, x + 124, 4 * sizeof(uint32_t));
        return;
    }
    uint32_t mask = b ? (uint32_t)((1ull << b) - 1) : 0u;
    for (int j = 0; j < 32; ++j) {
        uint32_t base[4];
        memcpy(base, prev, sizeof base);
        for (int l = 0; l < 4; ++l) {
            uint32_t d = 0;
            if (b) {
                uint32_t bitpos = (uint32_t)j * b, w = bitpos >> 5, s = bitpos & 31;
                uint64_t lo = in[4 * w + l];
                if (s + b > 32) lo |= (uint64_t)in[4 * (w + 1) + l] << 32;
                d = (uint32_t)(lo >> s) & mask;
            }
            x[4 * j + l] = d + (mode == G5O_DELTAM ? base[3] : base[l]);
        }
        memcpy(prev, x + 4 * j, 4 * sizeof(uint32_t));
    }
}

/* variablebyte.h:100-161: delta from 0, 7-bit groups little endian, the high
 * bit marks the last byte, zero padding to a word boundary. */
static size_t vbyte_encode(const uint32_t *in, size_t n, uint32_t *out)
{
    uint8_t *b = (uint8_t *)out, *b0 = b;
    uint32_t prev = 0;
    for (size_t k = 0; k < n; ++k) {
        uint32_t v = in[k] - prev;
        prev = in[k];
        while (v >= 128u) { *b++ = (uint8_t)(v & 127u); v >>= 7; }
        *b++ = (uint8_t)(v | 128u);
    }
    while ((size_t)(b - b0) & 3) *b++ = 0;
    return (size_t)(b - b0) / 4;
}

size_t g5o_codec_encode(const uint32_t *in, size_t n, uint32_t *out, int mode)
{
    /* compositecodec.h:31-51 */
    size_t n1 = n / 128 * 128;
    size_t o = 0;
    /* simdbinarypacking.h:174-235 */
    out[o++] = (uint32_t)n1;
    out[o++] = COOKIE; out[o++] = COOKIE; out[o++] = COOKIE;
    uint32_t zero[4] = {0, 0, 0, 0};
    size_t nmb = n1 / 128;
    for (size_t g = 0; g < nmb; g += 16) {
        uint32_t bs[16] = {0};
        size_t cnt = nmb - g < 16 ? nmb - g : 16;
        for (size_t i = 0; i < cnt; ++i) {
            size_t k = g + i;
            bs[i] = mb_bits(in + 128 * k, k ? in + 128 * k - 4 : zero, mode);
        }
        for (int h = 0; h < 4; ++h)
            out[o++] = (bs[4 * h] << 24) | (bs[4 * h + 1] << 16) | (bs[4 * h + 2] << 8) | bs[4 * h + 3];
        for (size_t i = 0; i < cnt; ++i) {
            size_t k = g + i;
            mb_pack(in + 128 * k, k ? in + 128 * k - 4 : zero, bs[i], out + o, mode);
            o += 4 * bs[i];
        }
    }
    if (n1 < n) o += vbyte_encode(in + n1, n - n1, out + o);
    return o;
}

size_t g5o_codec_decode(const uint32_t *in, size_t words, uint32_t *out,
                        size_t out_cap, int mode)
{
    if (words < 4) return (size_t)-1;
    size_t n1 = in[0];
    if (n1 % 128 || n1 > out_cap) return (size_t)-1;
    if (in[1] != COOKIE || in[2] != COOKIE || in[3] != COOKIE) return (size_t)-1;
    size_t p = 4;
    uint32_t prev[4] = {0, 0, 0, 0};
    size_t nmb = n1 / 128;
    for (size_t g = 0; g < nmb; g += 16) {
        if (p + 4 > words) return (size_t)-1;
        uint32_t bs[16];
        for (int h = 0; h < 4; ++h) {
            uint32_t w = in[p++];
            bs[4 * h] = w >> 24; bs[4 * h + 1] = (w >> 16) & 0xFF;
            bs[4 * h + 2] = (w >> 8) & 0xFF; bs[4 * h + 3] = w & 0xFF;
        }
        size_t cnt = nmb - g < 16 ? nmb - g : 16;
        for (size_t i = 0; i < cnt; ++i) {
            if (bs[i] > 32 || p + 4 * bs[i] > words) return (size_t)-1;
            mb_unpack(in + p, bs[i], prev, out + 128 * (g + i), mode);
            p += 4 * bs[i];
        }
    }
    /* variablebyte.h:217-: the tail up to the end of the stream */
    size_t o = n1;
    const uint8_t *b = (const uint8_t *)(in + p), *e = (const uint8_t *)(in + words);
    uint32_t prevv = 0, v = 0;
    int shift = 0;
    for (; b < e; ++b) {
        v |= (uint32_t)(*b & 127u) << shift;
        if (*b & 128u) {
            if (o >= out_cap) return (size_t)-1;
            prevv += v;
            out[o++] = prevv;
            v = 0; shift = 0;
        } else {
            shift += 7;
            if (shift > 28) return (size_t)-1; /* more than 5 bytes */
        }
    }
    return o;
}

size_t g5o_plugin_compress(const int64_t *in, size_t n, uint32_t *out,
                           size_t thr, int mode)
{
    uint32_t *tmp = (uint32_t *)malloc((n ? n : 1) * sizeof(uint32_t));
    for (size_t i = 0; i < n; ++i) tmp[i] = (uint32_t)in[i];
    size_t w;
    if (n > thr) w = g5o_codec_encode(tmp, n, out, mode);
    else { memcpy(out, tmp, n * sizeof(uint32_t)); w = n; }
    free(tmp);
    return w;
}

size_t g5o_plugin_decompress(const uint32_t *in, size_t words, size_t n,
                             int64_t *out, size_t thr, int mode)
{
    /* cpusimd.hh:169-173 isCompressed */
    if (n > thr && n != words) {
        uint32_t *tmp = (uint32_t *)malloc((n ? n : 1) * sizeof(uint32_t));
        size_t got = g5o_codec_decode(in, words, tmp, n, mode);
        if (got != (size_t)-1) for (size_t i = 0; i < got; ++i) out[i] = tmp[i];
        free(tmp);
        return got;
    }
    for (size_t i = 0; i < words; ++i) out[i] = in[i];
    return words;
}

void g5o_bitmap_or(uint64_t *dst, const uint64_t *const *srcs, int k, size_t words)
{
    for (int s = 0; s < k; ++s)
        for (size_t i = 0; i < words; ++i) dst[i] |= srcs[s][i];
}
