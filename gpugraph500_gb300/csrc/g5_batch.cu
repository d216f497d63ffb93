// g5_batch.cu -- batched BFS: up to 64 roots per graph, any number of graphs
// of uneven scale, all in one device-resident level loop.
//
// Each vertex carries three 64-bit words (one bit per root of its graph):
// visited, frontier and next-frontier.  One read of a vertex's adjacency
// serves every root whose frontier touches it, which is where the batched
// form beats 64 one-root searches.  The reference has no batched search (it
// runs runBFS once per root, cpu_2d/main.cpp:419-462); this is the
// multi-source form of the same level-synchronous BFS.
//
// Per level and per graph the direction is chosen as in the plain search
// (Beamer's alpha/beta on the union frontier):
//   top-down   edge-balanced tiles over the active-vertex queue; for an edge
//              (u, v) the roots new to v, front[u] & ~visited[v], are OR-ed
//              into next[v] and each such root's parent slot takes an
//              atomicMin with u (skipped when the slot is already <= u)
//   bottom-up  each vertex not yet visited by every root scans its ascending
//              adjacency: hit = front[u] & still-needed roots; the first hit
//              of a root is its parent; the scan stops once no root is needed
// Both give every root the smallest previous-level neighbour as parent, the
// same parent as the plain search and the reference CPU BFS.
//
// The search runs on a copy of each graph whose vertices are numbered by
// descending degree: the few high-degree vertices, which most adjacency
// entries point at, then share a small range of the frontier array that stays
// in L2 while the bottom-up levels probe it at random.  Each row keeps its
// neighbours in original-id order, so the first hit along a row is still the
// smallest original id; parents and roots are translated at the boundary and
// the output is indexed by original ids.  The bottom-up sweep itself walks
// the vertices in original-id order, which spreads the long rows over the
// warps.
//
// Vertex ranges of the graphs are padded to whole compaction chunks so every
// chunk belongs to one graph; the level loop is one CUDA graph (conditional
// while node) like the plain search.
#include <cub/cub.cuh>

#include <algorithm>
#include <cstring>
#include <vector>

#include "g5_common.cuh"
#include "g5_internal.h"

namespace {

constexpr int kB = 256;
constexpr int kW = kB / 32;
constexpr int kChunk = 2048;           // vertices per compaction chunk
constexpr uint64_t kTile = 256;        // edges per top-down warp tile
constexpr int kSerial = 4;             // bottom-up entries scanned per lane first
constexpr int kMaxGraphs = 64;
constexpr uint64_t kBuMinFrac = 16;    // bottom-up only when frontier entries > n / kBuMinFrac
constexpr int kMaxLevels = 1024;

enum : int32_t { TD = 0, BU = 1 };

struct GraphDesc {
    const int64_t *row_off;  // degree-ordered copy: rows by new id
    const uint32_t *col;     // new ids, each row in original-id order
    const uint32_t *orig;    // new id -> original id
    const uint32_t *perm;    // original id -> new id
    const int64_t *ostart;   // by original id: start of the vertex's row in col
    const uint32_t *odeg;    // by original id: its degree
    const uint32_t *blist;   // original ids of the vertices with edges, ascending
    uint64_t nblist;         // their count
    uint64_t step0;          // first bottom-up warp step of this graph
    int64_t n;
    int64_t nnz;
    uint64_t vbase;      // first global vertex id
    uint64_t pred_base;  // offset of vertex 0's parents in pred_out (nroots per vertex)
    uint64_t mask;       // one bit per root
    int32_t nroots;
    int32_t dir;         // direction for the current level
    uint64_t nf, mf;     // active vertices and their adjacency entries
    uint64_t mu;         // adjacency entries of not fully visited vertices
    uint64_t examined;
    uint64_t amask;      // roots whose frontier is not empty (this level)
    uint64_t amask_next; // being collected by k_bcount for the next level
};

struct BState {
    int32_t level;
    uint32_t err;
    uint64_t active;     // active vertices over all graphs (this level)
    uint64_t qlen;       // queue length (top-down graphs only)
    uint64_t qedges;     // its adjacency entries
    uint64_t examined;   // adjacency entries examined, all levels
    uint32_t dirs;       // this level: bit 0 a graph expands top-down, bit 1 bottom-up
};

struct BArgs {
    GraphDesc *gd;
    int ngraphs;
    const uint8_t *chunk_graph;
    uint32_t nchunks;
    uint64_t ntot;          // padded global vertex count
    const uint32_t *deg;    // per global vertex
    const uint32_t *iso;    // one bit per global vertex of degree 0
    uint64_t *vis, *front, *next;
    uint32_t *pred;         // output parents, vertex-major per graph: [v][nroots]
    uint32_t *queue;
    uint64_t *qoff;
    int64_t *qbase;
    uint32_t *tile_start;
    uint64_t max_tiles;
    uint64_t *chunk_n, *chunk_m;
    uint8_t *chunk_live;    // per chunk: bit 0 next frontier not empty, bit 1 nothing for k_bwrite
    const uint8_t *step_graph; // graph of each bottom-up warp step (32 list entries)
    uint64_t nsteps;
    BState *st;
    const int64_t *roots;   // device copy of the roots (graph-major)
    const int32_t *root_off;
    double alpha, beta;
    cudaGraphConditionalHandle cond;
    int use_cond;
    uint64_t *level_log;    // per level: active vertices
    int serving;            // continuous batching: no level cap, fixed m_u
};

__device__ __forceinline__ uint64_t wsum(uint64_t v)
{
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
    return v;
}

__device__ __forceinline__ int graph_of(const BArgs &a, uint64_t v) { return a.chunk_graph[v / kChunk]; }

// 4-byte asynchronous copy global -> shared (cp.async): the issuing thread
// goes on at once; cp_async_wait_all() waits for all of its copies.
__device__ __forceinline__ void cp_async4(void *smem, const void *gmem)
{
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    const size_t ga = __cvta_generic_to_global(gmem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(ga) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// ---- init: roots into next, parents of roots -------------------------------------

__global__ void k_binit(BArgs a)
{
    for (int g = blockIdx.x; g < a.ngraphs; g += gridDim.x) {
        GraphDesc &d = a.gd[g];
        for (int r = threadIdx.x; r < d.nroots; r += blockDim.x) {
            const int64_t root = a.roots[a.root_off[g] + r];
            if (root < 0 || root >= d.n) {
                atomicOr(&a.st->err, 1u);
                continue;
            }
            atomicOr((unsigned long long *)&a.next[d.vbase + d.perm[root]], 1ull << r);
            a.pred[d.pred_base + (uint64_t)root * d.nroots + r] = (uint32_t)root;
        }
        if (threadIdx.x == 0) {
            d.dir = TD;
            d.mu = (uint64_t)d.nnz;
            d.examined = 0;
            d.amask = 0;
            d.amask_next = 0;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.st->level = -1;
        a.st->err = 0;
        a.st->examined = 0;
    }
}

// ---- expansion ------------------------------------------------------------------------

__device__ void bexp_td(const BArgs &a, uint64_t &examined)
{
    __shared__ uint64_t s_q[kW][32];
    const int lane = g5_lane(), wib = threadIdx.x >> 5;
    const uint64_t gw = (uint64_t)blockIdx.x * kW + wib, nw = (uint64_t)gridDim.x * kW;
    const uint64_t mf = a.st->qedges, nf = a.st->qlen;
    const uint64_t ntiles = (mf + kTile - 1) / kTile;
    if (ntiles > a.max_tiles) {
        if (threadIdx.x == 0) atomicOr(&a.st->err, 2u);
        return;
    }
    for (uint64_t t = gw; t < ntiles; t += nw) {
        const uint64_t e0 = t * kTile, e1 = min(e0 + kTile, mf);
        uint64_t cur = a.tile_start[t];
        for (uint64_t gb = e0; gb < e1; gb += 32) {
            const uint64_t idx = cur + 1 + lane;
            s_q[wib][lane] = idx <= nf ? a.qoff[idx] : ~0ull;
            __syncwarp();
            const uint64_t e = gb + lane;
            int lo = 0, hi = 32;
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (s_q[wib][mid] <= e) lo = mid + 1;
                else hi = mid;
            }
            const uint64_t i = cur + lo;
            bool in_range = true;
            if (lo == 32 && e < e1) in_range = (i + 1 > nf) ? false : (a.qoff[i + 1] > e);
            if (e < e1) {
                if (!in_range) {
                    atomicOr(&a.st->err, 4u);
                } else {
                    const uint32_t ug = a.queue[i];
                    const GraphDesc &d = a.gd[graph_of(a, ug)];
                    const uint32_t vl = __ldg(d.col + (a.qbase[i] + (int64_t)e));
                    const uint64_t vg = d.vbase + vl;
                    // roots new to v: the smallest frontier neighbour is the
                    // parent (atomicMin, after a plain read to skip most)
                    const uint64_t nb = a.front[ug] & ~a.vis[vg];
                    if (nb) {
                        const uint32_t ul = __ldg(d.orig + (ug - d.vbase));
                        uint32_t *pv = a.pred + d.pred_base + (uint64_t)__ldg(d.orig + vl) * d.nroots;
                        uint64_t x = nb;
                        while (x) {
                            const int r = __ffsll((long long)x) - 1;
                            x &= x - 1;
                            uint32_t *slot = pv + r;
                            if (*slot > ul) atomicMin(slot, ul);
                        }
                        if (nb & ~a.next[vg]) atomicOr((unsigned long long *)&a.next[vg], (unsigned long long)nb);
                    }
                }
            }
            cur = __shfl_sync(0xFFFFFFFFu, i, 31);
            __syncwarp();
        }
        if (lane == 0) examined += e1 - e0;
    }
}

// Bottom-up: the candidates of v are the roots that have not visited it;
// the first frontier hit of each root along v's ascending adjacency is its
// parent.  A warp takes 32 consecutive vertices (never two graphs: graphs
// are chunk aligned).  Each lane first probes v's first kSerial entries with
// independent loads and keeps the hits as (parent, roots) events in shared
// memory; vertices still missing roots are then scanned by the whole warp,
// 64 entries per step, whose first hits per root (an exclusive prefix OR over
// the lanes) are written at once.  The serial hits are written last, lane r
// taking root r of each vertex: each vertex's parents are one contiguous run
// of nroots words, so those stores are contiguous.
__global__ void __launch_bounds__(kB, 4) k_bbu(BArgs a)
{
    __shared__ uint64_t s_evm[kW][kSerial][32];
    __shared__ uint32_t s_evu[kW][kSerial][32];
    // no graph expands bottom-up this level
    if (a.st->err || a.st->level < 0 || a.st->active == 0 || !(a.st->dirs & 2u)) return;
    const int lane = g5_lane(), wib = threadIdx.x >> 5;
    const uint64_t gw = ((uint64_t)blockIdx.x * kB + threadIdx.x) >> 5;
    const uint64_t nw = ((uint64_t)gridDim.x * kB) >> 5;
    uint64_t examined = 0;
    for (uint64_t w = gw; w < a.nsteps; w += nw) {
        // the graph's vertices with edges in original-id order, 32 per warp
        // step (vertices without edges are never reached, and half the
        // vertices of a Kronecker graph have none): high-degree vertices,
        // which have the lowest new ids, spread over the warps
        const GraphDesc &d = a.gd[a.step_graph[w]];
        if (d.dir != BU || d.nf == 0) continue;
        const uint64_t li = (w - d.step0) * 32 + lane;
        const uint64_t ol = li < d.nblist ? __ldg(d.blist + li) : 0u;
        const uint32_t R = (uint32_t)d.nroots;
        // new id and row bounds, indexed by original id: three loads issued
        // together (nearly coalesced: the list is ascending)
        uint32_t vl = 0, dg = 0;
        int64_t s = 0;
        if (li < d.nblist) {
            vl = __ldg(d.perm + ol);
            s = __ldg(d.ostart + ol);
            dg = __ldg(d.odeg + ol);
        }
        const int64_t e = s + dg;
        const uint64_t v = d.vbase + vl;
        // roots with an empty frontier cannot reach v
        uint64_t need = dg ? (~a.vis[v] & d.amask) : 0;
        // serial probes: all loads first, then the hits in adjacency order
        uint32_t u[kSerial];
        uint64_t f[kSerial];
#pragma unroll
        for (int k = 0; k < kSerial; ++k) u[k] = (need && s + k < e) ? __ldg(d.col + s + k) : 0xFFFFFFFFu;
#pragma unroll
        for (int k = 0; k < kSerial; ++k) f[k] = u[k] != 0xFFFFFFFFu ? a.front[d.vbase + u[k]] : 0ull;
        uint64_t found = 0, sfound = 0;
        int64_t j = s;
#pragma unroll
        for (int k = 0; k < kSerial; ++k) {
            const uint64_t hit = f[k] & need;
            s_evm[wib][k][lane] = hit;
            // the parent's original id lands in shared memory while the
            // rest of the row is scanned (read at the write-out below)
            if (hit) cp_async4(&s_evu[wib][k][lane], d.orig + u[k]);
            need &= ~hit;
            sfound |= hit;
            if (u[k] != 0xFFFFFFFFu && (need | hit)) j = s + k + 1;
        }
        found = sfound;
        const uint32_t vo = (uint32_t)ol;  // original id of v: its parents' row
        uint64_t ex = (uint64_t)(j - s);
        // short rows: pending vertices with at most 64 entries left are
        // packed whole, in lane order, into windows of 64 slots (slots lane
        // and lane + 32); each root's first hit in a row is found with a
        // segmented prefix OR over the slots
        while (true) {
            const bool sh = need && j < e && e - j <= 64;
            if (!__ballot_sync(0xFFFFFFFFu, sh)) break;
            const uint32_t r = sh ? (uint32_t)(e - j) : 0u;
            uint32_t inc = r;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, inc, o);
                if (lane >= o) inc += y;
            }
            const uint32_t start = inc - r;
            const bool in = sh && inc <= 64;  // row fits in this window
            uint32_t uq[2], s0q[2];
            uint64_t hq[2], vq[2];
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                const uint32_t k = (uint32_t)lane + 32u * q;
                // owner of slot k: the last lane whose row starts at or before k
                int ow = 0;
#pragma unroll
                for (int step = 16; step; step >>= 1) {
                    const uint32_t sv = __shfl_sync(0xFFFFFFFFu, start, ow + step);
                    if (sv <= k) ow += step;
                }
                const uint32_t s0 = __shfl_sync(0xFFFFFFFFu, start, ow);
                const uint32_t ro = __shfl_sync(0xFFFFFFFFu, in ? r : 0u, ow);
                const int64_t jo = __shfl_sync(0xFFFFFFFFu, j, ow);
                const uint64_t no = __shfl_sync(0xFFFFFFFFu, need, ow);
                vq[q] = __shfl_sync(0xFFFFFFFFu, (uint64_t)vo, ow);
                s0q[q] = s0;
                const bool live = k < s0 + ro;
                uq[q] = live ? __ldg(d.col + jo + (int64_t)(k - s0)) : 0xFFFFFFFFu;
                hq[q] = no;
            }
#pragma unroll
            for (int q = 0; q < 2; ++q) hq[q] = uq[q] != 0xFFFFFFFFu ? (a.front[d.vbase + uq[q]] & hq[q]) : 0ull;
            // the parent's original id, loaded for every hit before the scans
            // below, so its latency overlaps them
            uint32_t oq[2];
#pragma unroll
            for (int q = 0; q < 2; ++q) oq[q] = hq[q] ? __ldg(d.orig + uq[q]) : 0u;
            // segmented inclusive prefix OR: slots 0..31, then 32..63 with
            // the carry of a row that crosses slot 32
            uint64_t ia = hq[0], ib = hq[1];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint64_t ya = __shfl_up_sync(0xFFFFFFFFu, ia, o);
                const uint64_t yb = __shfl_up_sync(0xFFFFFFFFu, ib, o);
                if (lane >= o && (uint32_t)lane - o >= s0q[0]) ia |= ya;
                if (lane >= o && (uint32_t)lane + 32u - o >= s0q[1]) ib |= yb;
            }
            const uint64_t ca = __shfl_sync(0xFFFFFFFFu, ia, 31);
            if (s0q[1] < 32) ib |= ca;
            const uint64_t pa = __shfl_up_sync(0xFFFFFFFFu, ia, 1);
            const uint64_t pb = __shfl_up_sync(0xFFFFFFFFu, ib, 1);
            const uint64_t ea = (uint32_t)lane > s0q[0] ? pa : 0ull;
            const uint64_t eb = (uint32_t)lane + 32u > s0q[1] ? (lane ? pb : ca) : 0ull;
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                uint64_t x = hq[q] & ~(q ? eb : ea);
                if (x) {
                    uint32_t *pv = a.pred + d.pred_base + vq[q] * R;
                    const uint32_t uo = oq[q];
                    while (x) {
                        const int rr = __ffsll((long long)x) - 1;
                        x &= x - 1;
                        pv[rr] = uo;
                    }
                }
            }
            // each packed row takes its total from its last slot
            const uint32_t lk = in ? start + r - 1 : 0u;
            const uint64_t ta = __shfl_sync(0xFFFFFFFFu, ia, (int)(lk & 31));
            const uint64_t tb = __shfl_sync(0xFFFFFFFFu, ib, (int)(lk & 31));
            if (in) {
                const uint64_t seg = lk < 32 ? ta : tb;
                need &= ~seg;
                found |= seg;
                ex += r;
                j = e;
            }
        }
        // long rows: one vertex at a time, four windows of 32 entries per step
        unsigned pend = __ballot_sync(0xFFFFFFFFu, need && j < e);
        while (pend) {
            const int l = __ffs(pend) - 1;
            pend &= pend - 1;
            int64_t jj = __shfl_sync(0xFFFFFFFFu, j, l);
            const int64_t ee = __shfl_sync(0xFFFFFFFFu, e, l);
            uint64_t nd = __shfl_sync(0xFFFFFFFFu, need, l);
            uint32_t *pv = a.pred + d.pred_base + (uint64_t)__shfl_sync(0xFFFFFFFFu, vo, l) * R;
            const int64_t st = jj;
            uint64_t fnd = 0;
            while (jj < ee && nd) {
                uint32_t uw[4];
                uint64_t hw[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int64_t i = jj + 32 * q + lane;
                    uw[q] = i < ee ? __ldg(d.col + i) : 0xFFFFFFFFu;
                }
#pragma unroll
                for (int q = 0; q < 4; ++q) hw[q] = uw[q] != 0xFFFFFFFFu ? a.front[d.vbase + uw[q]] : 0ull;
                // one OR over the four windows; the first hits are located
                // only when the step holds a root not found before
                uint64_t lo = (hw[0] | hw[1] | hw[2] | hw[3]) & nd;
#pragma unroll
                for (int o = 16; o; o >>= 1) lo |= __shfl_xor_sync(0xFFFFFFFFu, lo, o);
                if (!lo) {
                    jj += 128;
                    continue;
                }
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    if (!nd) break;
                    const uint64_t hit = hw[q] & nd;
                    if (!__ballot_sync(0xFFFFFFFFu, hit != 0)) {
                        jj += 32;
                        continue;
                    }
                    const uint32_t uo = hit ? __ldg(d.orig + uw[q]) : 0u;  // overlaps the scan
                    // first lane of each root: exclusive prefix OR over the lanes
                    uint64_t incl = hit;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const uint64_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
                        if (lane >= o) incl |= y;
                    }
                    uint64_t excl = __shfl_up_sync(0xFFFFFFFFu, incl, 1);
                    if (lane == 0) excl = 0;
                    uint64_t x = hit & ~excl;
                    if (x) {
                        while (x) {
                            const int rr = __ffsll((long long)x) - 1;
                            x &= x - 1;
                            pv[rr] = uo;
                        }
                    }
                    const uint64_t all = __shfl_sync(0xFFFFFFFFu, incl, 31);
                    const unsigned cov = __ballot_sync(0xFFFFFFFFu, (incl & nd) == nd);
                    fnd |= all;
                    nd &= ~all;
                    jj += nd ? 32 : __ffs(cov);
                }
            }
            jj = min(jj, ee);
            if (lane == l) {
                found |= fnd;
                need = nd;
                ex += (uint64_t)(jj - st);
            }
        }
        cp_async_wait_all();
        __syncwarp();
        // serial hits, one (vertex, parent, roots) event at a time over the
        // warp: lane k writes roots k and k + 32.  Empty events cost nothing,
        // and the events' root sets are disjoint, so each parent is written
        // once.
#pragma unroll
        for (int k = 0; k < kSerial; ++k) {
            unsigned em = __ballot_sync(0xFFFFFFFFu, s_evm[wib][k][lane] != 0ull);
            while (em) {
                const int vi = __ffs(em) - 1;
                em &= em - 1;
                const uint64_t m = s_evm[wib][k][vi];
                const uint32_t u = s_evu[wib][k][vi];
                uint32_t *pv = a.pred + d.pred_base + (uint64_t)__shfl_sync(0xFFFFFFFFu, vo, vi) * R;
                if ((m >> lane) & 1ull) pv[lane] = u;
                if ((m >> (lane + 32)) & 1ull) pv[lane + 32] = u;
            }
        }
        __syncwarp();
        if (found) a.next[v] |= found;  // only this lane writes v in a bottom-up level
        examined += ex;
    }
    examined = wsum(examined);
    if (lane == 0 && examined) atomicAdd((unsigned long long *)&a.st->examined, (unsigned long long)examined);
}

// Top-down part of a level (graphs expanding top-down).
__global__ void __launch_bounds__(kB, 8) k_btd(BArgs a)
{
    if (a.st->err || a.st->level < 0 || a.st->active == 0 || a.st->qedges == 0) return;
    uint64_t ex = 0;
    bexp_td(a, ex);
    ex = wsum(ex);
    if (g5_lane() == 0 && ex) atomicAdd((unsigned long long *)&a.st->examined, (unsigned long long)ex);
}

// ---- compaction ---------------------------------------------------------------------------

// One warp per chunk over a persistent grid: the chunk's 2048 next words in
// coalesced 256-byte loads, 16 in flight per lane, then the degrees of the
// non-empty ones (no per-chunk block, barrier or serial tail).
__global__ void __launch_bounds__(kB) k_bcount(BArgs a)
{
    constexpr int kBatch = 16;
    const int lane = g5_lane();
    const uint64_t gw = ((uint64_t)blockIdx.x * kB + threadIdx.x) >> 5;
    const uint64_t nw = ((uint64_t)gridDim.x * kB) >> 5;
    for (uint64_t c = gw; c < a.nchunks; c += nw) {
        const uint64_t v0 = c * kChunk;
        const uint8_t live = a.chunk_live[c];
        uint64_t cn = 0, cm = 0, act = 0;
        for (int i0 = 0; i0 < kChunk / 32; i0 += kBatch) {
            uint64_t x[kBatch];
#pragma unroll
            for (int k = 0; k < kBatch; ++k) x[k] = __ldg(a.next + v0 + (uint64_t)(i0 + k) * 32 + lane);
#pragma unroll
            for (int k = 0; k < kBatch; ++k) {
                if (x[k]) {
                    ++cn;
                    cm += __ldg(a.deg + v0 + (uint64_t)(i0 + k) * 32 + lane);
                    act |= x[k];
                }
            }
        }
        cn = wsum(cn);
        cm = wsum(cm);
        // roots present in the next frontier of this chunk's graph
#pragma unroll
        for (int o = 16; o; o >>= 1) act |= __shfl_xor_sync(0xFFFFFFFFu, act, o);
        if (lane == 0) {
            a.chunk_n[c] = cn;
            a.chunk_m[c] = cm;
            // all chunks of a graph OR into one word: an atomic only for
            // roots not already recorded
            if (act) {
                unsigned long long *am = (unsigned long long *)&a.gd[a.chunk_graph[c]].amask_next;
                if (act & ~*(volatile unsigned long long *)am) atomicOr(am, (unsigned long long)act);
            }
            // no frontier this level nor the last: visited, front and next of
            // the chunk stay as they are, so the write pass skips it
            const bool prev = live & 1u, cur = cn != 0;
            a.chunk_live[c] = (uint8_t)(cur ? 1u : (prev ? 0u : 2u));
        }
    }
}

// Single block: per-graph totals and directions, then prefix sums over the
// chunks of top-down graphs (their vertices form the next queue).
__global__ void __launch_bounds__(1024) k_bscan(BArgs a)
{
    __shared__ uint64_t s_gn[kMaxGraphs], s_gm[kMaxGraphs];
    __shared__ int s_gdir[kMaxGraphs];
    for (int g = threadIdx.x; g < a.ngraphs; g += blockDim.x) {
        s_gn[g] = 0;
        s_gm[g] = 0;
    }
    if (threadIdx.x == 0) a.st->dirs = 0;
    __syncthreads();
    const uint32_t C = a.nchunks;
    // each warp owns a contiguous range of chunks and reads it 32 chunks at a
    // time (coalesced); a step inside one graph is summed with a warp
    // reduction and kept in registers until the graph changes
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const uint32_t per_w = (C + 31) / 32;
    const uint32_t w0 = min(C, wid * per_w), w1 = min(C, w0 + per_w);
    {
        int cur = -1;
        uint64_t an = 0, am = 0;
        for (uint32_t c0 = w0; c0 < w1; c0 += 32) {
            const uint32_t c = c0 + lane;
            const bool ok = c < w1;
            const uint64_t xn = ok ? a.chunk_n[c] : 0, xm = ok ? a.chunk_m[c] : 0;
            const int g = ok ? a.chunk_graph[c] : -1;
            const int g0 = __shfl_sync(0xFFFFFFFFu, g, 0);
            if (__all_sync(0xFFFFFFFFu, !ok || g == g0)) {
                const uint64_t sn = wsum(xn), sm = wsum(xm);
                if (g0 != cur) {
                    if (lane == 0 && cur >= 0 && (an | am)) {
                        atomicAdd((unsigned long long *)&s_gn[cur], (unsigned long long)an);
                        atomicAdd((unsigned long long *)&s_gm[cur], (unsigned long long)am);
                    }
                    cur = g0;
                    an = am = 0;
                }
                an += sn;
                am += sm;
            } else if (ok && (xn | xm)) {  // a graph boundary inside the step
                atomicAdd((unsigned long long *)&s_gn[g], (unsigned long long)xn);
                atomicAdd((unsigned long long *)&s_gm[g], (unsigned long long)xm);
            }
        }
        if (lane == 0 && cur >= 0 && (an | am)) {
            atomicAdd((unsigned long long *)&s_gn[cur], (unsigned long long)an);
            atomicAdd((unsigned long long *)&s_gm[cur], (unsigned long long)am);
        }
    }
    __syncthreads();
    if (threadIdx.x < a.ngraphs) {
        GraphDesc &d = a.gd[threadIdx.x];
        const uint64_t tn = s_gn[threadIdx.x], tm = s_gm[threadIdx.x];
        int nd = d.dir;
        // Beamer's switch on the union frontier of the graph's roots (when
        // serving, roots come and go, so m_u stays the whole graph)
        const uint64_t mu_after = a.serving ? (uint64_t)d.nnz : (d.mu >= tm ? d.mu - tm : 0);
        if (a.st->level >= 0) {
            if (d.dir == TD) {
                // Beamer's test, and a frontier large enough to pay for a
                // sweep over all of the graph's vertices
                if ((double)tm > (double)mu_after / a.alpha && tm > (uint64_t)d.n / kBuMinFrac) nd = BU;
            } else if ((double)tn < (double)d.n / a.beta && tn < d.nf) {
                nd = TD;
            }
        }
        d.mu = mu_after;
        d.dir = nd;
        d.nf = tn;
        d.mf = tm;
        d.amask = d.amask_next & d.mask;
        d.amask_next = 0;
        s_gdir[threadIdx.x] = nd;
        if (tn) atomicOr(&a.st->dirs, nd == TD ? 1u : 2u);
    }
    __syncthreads();
    // exclusive prefix over the chunks of top-down graphs: warp totals, a
    // scan of the 32 totals, then each warp writes its range's offsets
    uint64_t tn_w = 0, tm_w = 0;
    for (uint32_t c0 = w0; c0 < w1; c0 += 32) {
        const uint32_t c = c0 + lane;
        if (c < w1 && s_gdir[a.chunk_graph[c]] == TD) {
            tn_w += a.chunk_n[c];
            tm_w += a.chunk_m[c];
        }
    }
    tn_w = wsum(tn_w);
    tm_w = wsum(tm_w);
    __shared__ uint64_t s_wn[32], s_wm[32];
    if (lane == 0) {
        s_wn[wid] = tn_w;
        s_wm[wid] = tm_w;
    }
    __syncthreads();
    uint64_t tot_n = 0, tot_m = 0, on = 0, om = 0;
    for (int i = 0; i < 32; ++i) {
        if (i == wid) {
            on = tot_n;
            om = tot_m;
        }
        tot_n += s_wn[i];
        tot_m += s_wm[i];
    }
    for (uint32_t c0 = w0; c0 < w1; c0 += 32) {
        const uint32_t c = c0 + lane;
        const bool ok = c < w1;
        const bool td = ok && s_gdir[a.chunk_graph[c]] == TD;
        const uint64_t xn = td ? a.chunk_n[c] : 0, xm = td ? a.chunk_m[c] : 0;
        uint64_t in = xn, im = xm;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint64_t yn = __shfl_up_sync(0xFFFFFFFFu, in, o), ym = __shfl_up_sync(0xFFFFFFFFu, im, o);
            if (lane >= o) {
                in += yn;
                im += ym;
            }
        }
        if (ok) {
            a.chunk_n[c] = td ? on + in - xn : ~0ull;  // ~0: chunk not queued
            a.chunk_m[c] = om + im - xm;
        }
        on += __shfl_sync(0xFFFFFFFFu, in, 31);
        om += __shfl_sync(0xFFFFFFFFu, im, 31);
    }
    if (threadIdx.x == 0) {
        uint64_t act = 0;
        for (int g = 0; g < a.ngraphs; ++g) act += s_gn[g];
        BState *st = a.st;
        st->level += 1;
        st->active = act;
        st->qlen = tot_n;
        st->qedges = tot_m;
        a.qoff[tot_n] = tot_m;
        if (st->level < kMaxLevels) a.level_log[st->level] = act;
        bool cont = act > 0 && st->err == 0;
        if (cont && !a.serving && st->level + 1 >= kMaxLevels) {
            st->err |= 8u;
            cont = false;
        }
        if (a.use_cond) cudaGraphSetConditional(a.cond, cont ? 1u : 0u);
    }
}

// One warp per live chunk over a persistent grid: visited |= next, next ->
// front, and for chunks of top-down graphs the queue entries in ascending
// vertex order (a ballot per 32 words gives the positions, a warp scan the
// edge offsets).  All loads of a step come before its stores.
__global__ void __launch_bounds__(kB, 4) k_bwrite(BArgs a)
{
    constexpr int kBatch = 8;
    const int lane = g5_lane();
    const uint64_t gw = ((uint64_t)blockIdx.x * kB + threadIdx.x) >> 5;
    const uint64_t nw = ((uint64_t)gridDim.x * kB) >> 5;
    for (uint64_t c = gw; c < a.nchunks; c += nw) {
        if (a.chunk_live[c] & 2u) continue;
        const uint64_t v0 = c * kChunk;
        uint64_t pos = a.chunk_n[c], mpos = a.chunk_m[c];
        const bool queued = pos != ~0ull;
        const GraphDesc &d = a.gd[a.chunk_graph[c]];
        for (int i0 = 0; i0 < kChunk / 32; i0 += kBatch) {
            uint64_t nx[kBatch], vs[kBatch];
            uint32_t dg[kBatch];
#pragma unroll
            for (int k = 0; k < kBatch; ++k) nx[k] = a.next[v0 + (uint64_t)(i0 + k) * 32 + lane];
#pragma unroll
            for (int k = 0; k < kBatch; ++k) {
                const uint64_t v = v0 + (uint64_t)(i0 + k) * 32 + lane;
                vs[k] = nx[k] ? a.vis[v] : 0ull;
                dg[k] = (nx[k] && queued) ? a.deg[v] : 0u;
            }
#pragma unroll
            for (int k = 0; k < kBatch; ++k) {
                const uint64_t v = v0 + (uint64_t)(i0 + k) * 32 + lane;
                if (nx[k]) {
                    a.vis[v] = vs[k] | nx[k];
                    a.next[v] = 0;
                }
                a.front[v] = nx[k];
            }
            if (!queued) continue;
#pragma unroll
            for (int k = 0; k < kBatch; ++k) {
                const unsigned bal = __ballot_sync(0xFFFFFFFFu, nx[k] != 0ull);
                if (!bal) continue;
                const uint64_t v = v0 + (uint64_t)(i0 + k) * 32 + lane;
                const uint64_t dv = dg[k];
                uint64_t incl = dv;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const uint64_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
                    if (lane >= o) incl += y;
                }
                if (nx[k]) {
                    const uint64_t p = pos + __popc(bal & g5_lanemask_lt());
                    const uint64_t mp = mpos + incl - dv;
                    a.queue[p] = (uint32_t)v;
                    a.qoff[p] = mp;
                    a.qbase[p] = d.row_off[v - d.vbase] - (int64_t)mp;
                    uint64_t t = (mp + kTile - 1) / kTile;
                    const uint64_t tend = (mp + dv + kTile - 1) / kTile;
                    for (; t < tend && t < a.max_tiles; ++t) a.tile_start[t] = (uint32_t)p;
                }
                pos += __popc(bal);
                mpos += __shfl_sync(0xFFFFFFFFu, incl, 31);
            }
        }
    }
}

// Continuous batching: roots admitted into free slots (bit r of their
// graph) join the next level as its frontier; retired roots' visited bits are
// cleared so the slot can be reused.
struct Admit {
    int32_t graph;
    int32_t slot;
    int64_t root;
};

__global__ void k_sadmit(BArgs a, const Admit *adm, int nadm)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nadm; i += gridDim.x * blockDim.x) {
        const Admit x = adm[i];
        const GraphDesc &d = a.gd[x.graph];
        atomicOr((unsigned long long *)&a.next[d.vbase + d.perm[x.root]], 1ull << x.slot);
        a.pred[d.pred_base + (uint64_t)x.root * d.nroots + x.slot] = (uint32_t)x.root;
    }
}

__global__ void k_sclear(BArgs a, const uint64_t *clear_mask)
{
    // a retired slot's visited vertices get their parent entry back to
    // 0xFFFFFFFF: every entry of a free slot is unvisited again
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < a.ntot;
         v += (uint64_t)gridDim.x * blockDim.x) {
        const int g = graph_of(a, v);
        const uint64_t m = clear_mask[g];
        if (m) {
            const uint64_t x = a.vis[v];
            if (x & m) {
                a.vis[v] = x & ~m;
                const GraphDesc &d = a.gd[g];
                uint32_t *p = a.pred + d.pred_base + (uint64_t)d.orig[v - d.vbase] * d.nroots;
                uint64_t y = x & m;
                while (y) {
                    const int r = __ffsll((long long)y) - 1;
                    y &= y - 1;
                    p[r] = 0xFFFFFFFFu;
                }
            }
        }
    }
}

// One root's parents out of the vertex-major array: dst[v] = pred[v * R + r].
__global__ void k_gather_root(const uint32_t *pred, uint32_t R, uint32_t r, int64_t n, uint32_t *dst)
{
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x)
        dst[v] = pred[(uint64_t)v * R + r];
}

__global__ void k_bdeg(const GraphDesc *gd, const uint8_t *chunk_graph, uint64_t ntot, uint32_t *deg,
                       uint32_t *iso)
{
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < ntot;
         v += (uint64_t)gridDim.x * blockDim.x) {
        const GraphDesc &d = gd[chunk_graph[v / kChunk]];
        const int64_t vl = (int64_t)(v - d.vbase);
        const uint32_t dv = vl < d.n ? (uint32_t)(d.row_off[vl + 1] - d.row_off[vl]) : 0u;
        deg[v] = dv;
        const unsigned z = __ballot_sync(0xFFFFFFFFu, dv == 0u);
        if ((threadIdx.x & 31) == 0) iso[v >> 5] = z;
    }
}

// ---- degree-ordered copy of a graph ----------------------------------------------------

__global__ void k_rl_deg(const int64_t *row_off, int64_t n, uint32_t *deg, uint32_t *ids)
{
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
        deg[v] = (uint32_t)(row_off[v + 1] - row_off[v]);
        ids[v] = (uint32_t)v;
    }
}

// perm[orig[p]] = p; row2[p] = degree of new vertex p (scanned into offsets)
__global__ void k_rl_perm(const uint32_t *orig, const uint32_t *deg_sorted, int64_t n, uint32_t *perm, int64_t *row2)
{
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p <= n; p += (int64_t)gridDim.x * blockDim.x) {
        if (p < n) {
            perm[orig[p]] = (uint32_t)p;
            row2[p] = deg_sorted[p];
        } else {
            row2[n] = 0;
        }
    }
}

// by original id: where the vertex's row starts in the copy, and its degree
// (the bottom-up sweep walks original ids and reads these coalesced)
__global__ void k_rl_orig(const uint32_t *perm, const int64_t *row2, int64_t n, int64_t *ostart, uint32_t *odeg)
{
    for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < n; o += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t p = perm[o];
        const int64_t s = row2[p];
        ostart[o] = s;
        odeg[o] = (uint32_t)(row2[p + 1] - s);
    }
}

// one warp per new row: the original row, neighbours renamed, order kept
__global__ void k_rl_cols(const int64_t *row_off, const uint32_t *col, const uint32_t *orig, const uint32_t *perm,
                          const int64_t *row2, int64_t n, uint32_t *col2)
{
    const int lane = g5_lane();
    for (int64_t p = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; p < n;
         p += ((int64_t)gridDim.x * blockDim.x) >> 5) {
        const uint32_t o = orig[p];
        const int64_t s = row_off[o], len = row_off[o + 1] - s, d0 = row2[p];
        for (int64_t k = lane; k < len; k += 32) col2[d0 + k] = perm[col[s + k]];
    }
}

}  // namespace

struct g5_batch {
    std::vector<g5_graph *> graphs;
    std::vector<GraphDesc> hgd;
    BArgs args;
    cudaStream_t stream = nullptr;
    GraphDesc *gd = nullptr;
    uint8_t *chunk_graph = nullptr;
    uint8_t *step_graph = nullptr;  // graph of each bottom-up warp step
    uint32_t *deg = nullptr;
    uint32_t *iso = nullptr;
    uint64_t *words = nullptr;  // vis | front | next
    uint32_t *queue = nullptr;
    uint64_t *qoff = nullptr;
    int64_t *qbase = nullptr;
    uint32_t *tile_start = nullptr;
    uint64_t *chunks = nullptr;
    BState *st = nullptr;
    int64_t *roots = nullptr;
    int32_t *root_off = nullptr;
    uint64_t *level_log = nullptr;
    int64_t *h_roots = nullptr;
    int32_t *h_root_off = nullptr;
    BState *h_st = nullptr;
    uint32_t *bound_pred = nullptr;  // pred pointer the graph was built for
    void *adm_dev = nullptr;          // serving: admissions + retire masks
    void *adm_host = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaGraph_t graph = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::vector<void *> owned;        // degree-ordered graph copies
};

namespace {

void enqueue_batch(g5_batch *b, const BArgs &a, cudaStream_t s, bool body, std::vector<cudaEvent_t> *ev = nullptr)
{
    auto mark = [&]() {
        if (ev) {
            cudaEvent_t e;
            cudaEventCreate(&e);
            cudaEventRecord(e, s);
            ev->push_back(e);
        }
    };
    if (!body) {
        cudaMemsetAsync(b->words, 0, sizeof(uint64_t) * 3 * a.ntot, s);
        cudaMemsetAsync(a.chunk_live, 0, a.nchunks, s);
        k_binit<<<std::max(1, a.ngraphs), kB, 0, s>>>(a);
        return;
    }
    mark();
    k_bcount<<<g5::grid_for(8), kB, 0, s>>>(a);
    mark();
    k_bscan<<<1, 1024, 0, s>>>(a);
    mark();
    k_bwrite<<<g5::grid_for(4), kB, 0, s>>>(a);
    mark();
    k_btd<<<g5::grid_for(8), kB, 0, s>>>(a);
    k_bbu<<<g5::grid_for(4), kB, 0, s>>>(a);
    mark();
    mark();
}

g5_status build_batch_graph(g5_batch *b)
{
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
    cudaStream_t s = b->stream;
    cudaGraph_t pro = nullptr;
    G5_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    enqueue_batch(b, b->args, s, false);
    G5_CUDA(cudaStreamEndCapture(s, &pro));
    cudaGraph_t g = nullptr;
    G5_CUDA(cudaGraphCreate(&g, 0));
    cudaGraphNode_t pn;
    G5_CUDA(cudaGraphAddChildGraphNode(&pn, g, nullptr, 0, pro));
    cudaGraphDestroy(pro);
    cudaGraphConditionalHandle h;
    G5_CUDA(cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t cn;
    G5_CUDA(cudaGraphAddNode(&cn, g, &pn, nullptr, 1, &cp));
    BArgs a = b->args;
    a.cond = h;
    a.use_cond = 1;
    G5_CUDA(cudaStreamBeginCaptureToGraph(s, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                          cudaStreamCaptureModeThreadLocal));
    enqueue_batch(b, a, s, true);
    cudaGraph_t body = nullptr;
    G5_CUDA(cudaStreamEndCapture(s, &body));
    G5_CUDA(cudaGraphInstantiate(&b->exec, g, 0));
    b->graph = g;
    return G5_OK;
}

void free_batch(g5_batch *b)
{
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    cudaFree(b->gd);
    cudaFree(b->chunk_graph);
    cudaFree(b->deg);
    cudaFree(b->iso);
    cudaFree(b->words);
    cudaFree(b->queue);
    cudaFree(b->qoff);
    cudaFree(b->qbase);
    cudaFree(b->tile_start);
    cudaFree(b->chunks);
    cudaFree(b->step_graph);
    cudaFree(b->st);
    cudaFree(b->roots);
    cudaFree(b->root_off);
    cudaFree(b->level_log);
    cudaFree(b->adm_dev);
    cudaFreeHost(b->adm_host);
    cudaFreeHost(b->h_roots);
    cudaFreeHost(b->h_root_off);
    cudaFreeHost(b->h_st);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    for (void *p : b->owned) cudaFree(p);
    b->owned.clear();
    if (b->stream) cudaStreamDestroy(b->stream);
}

struct HasEdges {
    const uint32_t *deg;
    __device__ bool operator()(const uint32_t &v) const { return deg[v] > 0; }
};

// Degree-ordered copy of g on b's stream: new ids by descending degree (ties
// by original id), rows in new-id order, each row's neighbours renamed but in
// their original order.
g5_status build_relabel(g5_batch *b, const g5_graph *g, GraphDesc &d)
{
    const int64_t n = g->n, nnz = g->nnz;
    cudaStream_t s = b->stream;
    auto alloc = [&](void **p, size_t bytes) -> bool {
        if (cudaMalloc(p, bytes ? bytes : 16) != cudaSuccess) return false;
        b->owned.push_back(*p);
        return true;
    };
    uint32_t *orig = nullptr, *perm = nullptr, *col2 = nullptr, *odeg = nullptr;
    int64_t *row2 = nullptr, *ostart = nullptr;
    if (!alloc((void **)&orig, sizeof(uint32_t) * n) || !alloc((void **)&perm, sizeof(uint32_t) * n) ||
        !alloc((void **)&row2, sizeof(int64_t) * (n + 1)) || !alloc((void **)&col2, sizeof(uint32_t) * nnz) ||
        !alloc((void **)&ostart, sizeof(int64_t) * n) || !alloc((void **)&odeg, sizeof(uint32_t) * n))
        return G5_ERR_OOM;
    d.orig = orig;
    d.perm = perm;
    d.ostart = ostart;
    d.odeg = odeg;
    d.row_off = row2;
    d.col = col2;
    if (n == 0) {
        G5_CUDA(cudaMemsetAsync(row2, 0, sizeof(int64_t), s));
        return G5_OK;
    }
    g5::DevBuf<uint32_t> deg, ids, deg_sorted;
    if (deg.alloc(n) != G5_OK || ids.alloc(n) != G5_OK || deg_sorted.alloc(n) != G5_OK) return G5_ERR_OOM;
    const int blocks = g5::grid_for(8);
    k_rl_deg<<<blocks, 256, 0, s>>>(g->row_off, n, deg.p, ids.p);
    size_t t1 = 0, t2 = 0;
    G5_CUDA(cub::DeviceRadixSort::SortPairsDescending(nullptr, t1, deg.p, deg_sorted.p, ids.p, orig, n, 0, 32, s));
    G5_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, t2, row2, row2, n + 1, s));
    g5::DevBuf<uint8_t> tmp;
    if (tmp.alloc(std::max(t1, t2)) != G5_OK) return G5_ERR_OOM;
    G5_CUDA(cub::DeviceRadixSort::SortPairsDescending(tmp.p, t1, deg.p, deg_sorted.p, ids.p, orig, n, 0, 32, s));
    k_rl_perm<<<blocks, 256, 0, s>>>(orig, deg_sorted.p, n, perm, row2);
    G5_CUDA(cub::DeviceScan::ExclusiveSum(tmp.p, t2, row2, row2, n + 1, s));
    k_rl_cols<<<blocks, 256, 0, s>>>(g->row_off, g->col, orig, perm, row2, n, col2);
    k_rl_orig<<<blocks, 256, 0, s>>>(perm, row2, n, ostart, odeg);
    // the bottom-up sweep's vertex list: original ids with edges, ascending
    // (ids still holds 0..n-1: the sort wrote its values elsewhere)
    uint32_t *blist = nullptr;
    if (!alloc((void **)&blist, sizeof(uint32_t) * n)) return G5_ERR_OOM;
    g5::DevBuf<int64_t> nsel;
    if (nsel.alloc(1) != G5_OK) return G5_ERR_OOM;
    size_t t3 = 0;
    const HasEdges pred{odeg};
    G5_CUDA(cub::DeviceSelect::If(nullptr, t3, ids.p, blist, nsel.p, (int64_t)n, pred, s));
    g5::DevBuf<uint8_t> tmp3;
    if (tmp3.alloc(t3) != G5_OK) return G5_ERR_OOM;
    G5_CUDA(cub::DeviceSelect::If(tmp3.p, t3, ids.p, blist, nsel.p, (int64_t)n, pred, s));
    int64_t nl = 0;
    G5_CUDA(cudaMemcpyAsync(&nl, nsel.p, sizeof nl, cudaMemcpyDeviceToHost, s));
    G5_CUDA(cudaStreamSynchronize(s));
    d.blist = blist;
    d.nblist = (uint64_t)nl;
    return G5_OK;
}

}  // namespace

extern "C" {

}  // extern "C"

namespace {

// A batch workspace over `graphs`; with `share` (a workspace over the same
// graphs), its degree-ordered graph copies are borrowed instead of built, so
// several workspaces on one graph hold one copy (the owner must outlive the
// borrowers).
g5_status batch_create_impl(g5_graph *const *graphs, int ngraphs, const g5_batch *share, g5_batch **out)
{
    if (!graphs || !out || ngraphs < 1 || ngraphs > kMaxGraphs) return G5_ERR_INVALID_ARG;
    *out = nullptr;
    g5_batch *b = new g5_batch();
    auto fail = [&](g5_status s) {
        free_batch(b);
        delete b;
        return s;
    };
    uint64_t vb = 0, nnz_max = 0;
    std::vector<uint8_t> cg;
    for (int i = 0; i < ngraphs; ++i) {
        if (!graphs[i]) return fail(G5_ERR_INVALID_ARG);
        b->graphs.push_back(graphs[i]);
        GraphDesc d;
        memset(&d, 0, sizeof d);
        d.n = graphs[i]->n;
        d.nnz = graphs[i]->nnz;
        d.vbase = vb;
        const uint64_t chunks = ((uint64_t)d.n + kChunk - 1) / kChunk;
        for (uint64_t c = 0; c < chunks; ++c) cg.push_back((uint8_t)i);
        vb += chunks * kChunk;
        nnz_max += (uint64_t)d.nnz;
        b->hgd.push_back(d);
    }
    if (vb >= (1ull << 32)) return fail(G5_ERR_CAPACITY);
    BArgs &a = b->args;
    memset(&a, 0, sizeof a);
    a.ngraphs = ngraphs;
    a.nchunks = (uint32_t)cg.size();
    a.ntot = vb;
    a.max_tiles = nnz_max / kTile + 2 + (uint64_t)ngraphs;
    a.alpha = 14.0;
    a.beta = 24.0;
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) return fail(G5_ERR_CUDA);
    cudaEventCreate(&b->ev0);
    cudaEventCreate(&b->ev1);
    for (int i = 0; i < ngraphs; ++i) {
        if (share) {
            if ((int)share->graphs.size() != ngraphs || share->graphs[i] != graphs[i]) return fail(G5_ERR_INVALID_ARG);
            GraphDesc &d = b->hgd[i];
            const GraphDesc &o = share->hgd[i];
            d.row_off = o.row_off;
            d.col = o.col;
            d.orig = o.orig;
            d.perm = o.perm;
            d.ostart = o.ostart;
            d.odeg = o.odeg;
            d.blist = o.blist;
            d.nblist = o.nblist;
            continue;
        }
        const g5_status rs = build_relabel(b, graphs[i], b->hgd[i]);
        if (rs != G5_OK) return fail(rs);
    }
    // bottom-up warp steps: each graph's list in 32-entry steps, graphs one
    // after another
    std::vector<uint8_t> sg;
    for (int i = 0; i < ngraphs; ++i) {
        GraphDesc &d = b->hgd[i];
        d.step0 = sg.size();
        const uint64_t steps = (d.nblist + 31) / 32;
        sg.insert(sg.end(), steps, (uint8_t)i);
    }
    a.nsteps = sg.size();
#define B_ALLOC(ptr, bytes) \
    if (cudaMalloc(&(ptr), (bytes)) != cudaSuccess) return fail(G5_ERR_OOM)
    B_ALLOC(b->gd, sizeof(GraphDesc) * ngraphs);
    B_ALLOC(b->step_graph, sg.size() + 1);
    B_ALLOC(b->chunk_graph, cg.size());
    B_ALLOC(b->deg, sizeof(uint32_t) * vb);
    B_ALLOC(b->iso, sizeof(uint32_t) * (vb / 32));
    B_ALLOC(b->words, sizeof(uint64_t) * 3 * vb);
    B_ALLOC(b->queue, sizeof(uint32_t) * vb);
    B_ALLOC(b->qoff, sizeof(uint64_t) * (vb + 1));
    B_ALLOC(b->qbase, sizeof(int64_t) * vb);
    B_ALLOC(b->tile_start, sizeof(uint32_t) * a.max_tiles);
    B_ALLOC(b->chunks, sizeof(uint64_t) * 2 * a.nchunks + a.nchunks);
    B_ALLOC(b->st, sizeof(BState));
    B_ALLOC(b->roots, sizeof(int64_t) * 64 * ngraphs);
    B_ALLOC(b->root_off, sizeof(int32_t) * (ngraphs + 1));
    B_ALLOC(b->level_log, sizeof(uint64_t) * kMaxLevels);
#undef B_ALLOC
    if (cudaMallocHost(&b->h_roots, sizeof(int64_t) * 64 * ngraphs) != cudaSuccess ||
        cudaMallocHost(&b->h_root_off, sizeof(int32_t) * (ngraphs + 1)) != cudaSuccess ||
        cudaMallocHost(&b->h_st, sizeof(BState)) != cudaSuccess)
        return fail(G5_ERR_OOM);
    if ((!sg.empty() && cudaMemcpy(b->step_graph, sg.data(), sg.size(), cudaMemcpyHostToDevice) != cudaSuccess) ||
        cudaMemcpy(b->chunk_graph, cg.data(), cg.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(b->gd, b->hgd.data(), sizeof(GraphDesc) * ngraphs, cudaMemcpyHostToDevice) != cudaSuccess)
        return fail(G5_ERR_CUDA);
    a.gd = b->gd;
    a.chunk_graph = b->chunk_graph;
    a.deg = b->deg;
    a.iso = b->iso;
    a.vis = b->words;
    a.front = b->words + vb;
    a.next = b->words + 2 * vb;
    a.queue = b->queue;
    a.qoff = b->qoff;
    a.qbase = b->qbase;
    a.tile_start = b->tile_start;
    a.chunk_n = b->chunks;
    a.chunk_m = b->chunks + a.nchunks;
    a.chunk_live = reinterpret_cast<uint8_t *>(b->chunks + 2 * (uint64_t)a.nchunks);
    a.step_graph = b->step_graph;
    a.st = b->st;
    a.roots = b->roots;
    a.root_off = b->root_off;
    a.level_log = b->level_log;
    k_bdeg<<<g5::grid_for(8), kB, 0, b->stream>>>(b->gd, b->chunk_graph, vb, b->deg, b->iso);
    if (cudaStreamSynchronize(b->stream) != cudaSuccess) return fail(G5_ERR_CUDA);
    *out = b;
    return G5_OK;
}

}  // namespace

namespace g5 {

g5_status batch_create_sharing(g5_batch *owner, g5_batch **out)
{
    if (!owner || !out) return G5_ERR_INVALID_ARG;
    return batch_create_impl(owner->graphs.data(), (int)owner->graphs.size(), owner, out);
}

size_t batch_workspace_bytes(const g5_graph *g)
{
    // per vertex: 3 x 8 B words, degree, queue, edge offset, row base;
    // per 256 edges a tile start; the fixed parts rounded up
    return (size_t)g->n * (24 + 4 + 4 + 8 + 8) + (size_t)g->nnz / 64 + ((size_t)1 << 20);
}

size_t batch_copy_bytes(const g5_graph *g)
{
    // degree-ordered copy: two id maps, offsets, per-vertex row start and degree, columns
    return (size_t)g->n * (4 + 4 + 8 + 8 + 4) + (size_t)g->nnz * 4 + ((size_t)1 << 20);
}

}  // namespace g5

extern "C" {

g5_status g5_batch_create(g5_graph *const *graphs, int ngraphs, g5_batch **out)
{
    return batch_create_impl(graphs, ngraphs, nullptr, out);
}

g5_status g5_batch_set_direction(g5_batch *b, double alpha, double beta)
{
    if (!b || !(alpha > 0) || !(beta > 0)) return G5_ERR_INVALID_ARG;
    b->args.alpha = alpha;
    b->args.beta = beta;
    b->bound_pred = nullptr;  // rebuild the graph with the new kernel arguments
    return G5_OK;
}

g5_status g5_batch_profile(g5_batch *b, const int64_t *roots_host, const int *nroots, uint32_t *pred_out_dev,
                           double *kernel_ms, int64_t *level_active, double *level_expand_ms, int64_t *level_examined, int32_t *level_dirs,
                           int max_levels,
                           int *levels)
{
    // host-driven level loop with CUDA events around every launch: kernel_ms
    // gets count, scan, write, expand, fixup totals (ms); level_active the
    // active vertices of each level
    if (!b || !roots_host || !nroots || !pred_out_dev || !kernel_ms || !levels) return G5_ERR_INVALID_ARG;
    const int ng = (int)b->graphs.size();
    uint64_t pb = 0;
    int off = 0;
    for (int i = 0; i < ng; ++i) {
        if (nroots[i] < 0 || nroots[i] > 64) return G5_ERR_INVALID_ARG;
        GraphDesc &d = b->hgd[i];
        d.nroots = nroots[i];
        d.mask = nroots[i] == 64 ? ~0ull : ((1ull << nroots[i]) - 1);
        d.pred_base = pb;
        pb += (uint64_t)nroots[i] * (uint64_t)d.n;
        b->h_root_off[i] = off;
        for (int r = 0; r < nroots[i]; ++r) b->h_roots[off + r] = roots_host[off + r];
        off += nroots[i];
    }
    b->h_root_off[ng] = off;
    cudaStream_t s = b->stream;
    BArgs a = b->args;
    a.pred = pred_out_dev;
    a.use_cond = 0;
    G5_CUDA(cudaMemcpyAsync(b->gd, b->hgd.data(), sizeof(GraphDesc) * ng, cudaMemcpyHostToDevice, s));
    G5_CUDA(cudaMemcpyAsync(b->roots, b->h_roots, sizeof(int64_t) * (off ? off : 1), cudaMemcpyHostToDevice, s));
    G5_CUDA(cudaMemcpyAsync(b->root_off, b->h_root_off, sizeof(int32_t) * (ng + 1), cudaMemcpyHostToDevice, s));
    if (pb) G5_CUDA(cudaMemsetAsync(pred_out_dev, 0xFF, sizeof(uint32_t) * pb, s));
    enqueue_batch(b, a, s, false);
    for (int k = 0; k < 5; ++k) kernel_ms[k] = 0;
    int L = 0;
    for (; L < kMaxLevels; ++L) {
        std::vector<cudaEvent_t> ev;
        enqueue_batch(b, a, s, true, &ev);
        G5_CUDA(cudaMemcpyAsync(b->h_st, b->st, sizeof(BState), cudaMemcpyDeviceToHost, s));
        G5_CUDA(cudaStreamSynchronize(s));
        for (size_t k = 0; k + 1 < ev.size(); ++k) {
            float t = 0;
            cudaEventElapsedTime(&t, ev[k], ev[k + 1]);
            kernel_ms[k] += t;
            if (k == 3 && level_expand_ms && L < max_levels) level_expand_ms[L] = t;
        }
        if (level_examined && L < max_levels) level_examined[L] = (int64_t)b->h_st->examined;
        if (level_dirs && L < max_levels) level_dirs[L] = (int32_t)b->h_st->dirs;
        for (cudaEvent_t e : ev) cudaEventDestroy(e);
        if (level_active && L < max_levels) level_active[L] = (int64_t)b->h_st->active;
        if (b->h_st->active == 0 || b->h_st->err) break;
    }
    *levels = L + 1;
    return b->h_st->err ? G5_ERR_CAPACITY : G5_OK;
}

g5_status g5_batch_serve_begin(g5_batch *b, uint32_t *pred_dev, const int *slots)
{
    // every graph gets `slots[g]` root slots whose parents live in pred_dev,
    // root-major per graph (graph 0 slot 0, slot 1, ..., graph 1 ...)
    if (!b || !pred_dev || !slots) return G5_ERR_INVALID_ARG;
    const int ng = (int)b->graphs.size();
    uint64_t pb = 0;
    for (int i = 0; i < ng; ++i) {
        if (slots[i] < 0 || slots[i] > 64) return G5_ERR_INVALID_ARG;
        GraphDesc &d = b->hgd[i];
        d.nroots = slots[i];
        d.mask = slots[i] == 64 ? ~0ull : ((1ull << slots[i]) - 1);
        d.pred_base = pb;
        d.dir = TD;
        d.mu = (uint64_t)d.nnz;
        d.nf = d.mf = d.examined = d.amask = d.amask_next = 0;
        pb += (uint64_t)slots[i] * (uint64_t)d.n;
    }
    cudaStream_t s = b->stream;
    b->args.pred = pred_dev;
    b->args.serving = 1;
    b->args.use_cond = 0;
    if (!b->adm_dev) G5_CUDA(cudaMalloc(&b->adm_dev, sizeof(Admit) * 64 * ng + sizeof(uint64_t) * ng));
    if (!b->adm_host) G5_CUDA(cudaMallocHost(&b->adm_host, sizeof(Admit) * 64 * ng + sizeof(uint64_t) * ng));
    G5_CUDA(cudaMemcpyAsync(b->gd, b->hgd.data(), sizeof(GraphDesc) * ng, cudaMemcpyHostToDevice, s));
    G5_CUDA(cudaMemsetAsync(b->words, 0, sizeof(uint64_t) * 3 * b->args.ntot, s));
    G5_CUDA(cudaMemsetAsync(b->args.chunk_live, 0, b->args.nchunks, s));
    // every entry starts unvisited; a retired slot's entries are reset by
    // k_sclear, so an admitted root always starts from a clean column
    if (pb) G5_CUDA(cudaMemsetAsync(pred_dev, 0xFF, sizeof(uint32_t) * pb, s));
    BState z;
    memset(&z, 0, sizeof z);
    z.level = 0;
    *b->h_st = z;
    G5_CUDA(cudaMemcpyAsync(b->st, b->h_st, sizeof(BState), cudaMemcpyHostToDevice, s));
    G5_CUDA(cudaStreamSynchronize(s));
    return G5_OK;
}

g5_status g5_batch_serve_step(g5_batch *b, const int32_t *adm_graph, const int32_t *adm_slot,
                              const int64_t *adm_root, int nadm, const uint64_t *retire_mask,
                              uint64_t *active_mask, double *device_ms)
{
    // one level of continuous batching: clear the visited bits of retired
    // slots, start the admitted roots, run one level; active_mask[g] gets the
    // slots whose frontier is still non-empty
    if (!b || (nadm && (!adm_graph || !adm_slot || !adm_root)) || !active_mask || !b->args.serving)
        return G5_ERR_INVALID_ARG;
    const int ng = (int)b->graphs.size();
    if (nadm > 64 * ng) return G5_ERR_CAPACITY;
    cudaStream_t s = b->stream;
    Admit *ah = reinterpret_cast<Admit *>(b->adm_host);
    uint64_t *rh = reinterpret_cast<uint64_t *>(ah + 64 * ng);
    bool any_retire = false;
    for (int g = 0; g < ng; ++g) {
        rh[g] = retire_mask ? retire_mask[g] : 0;
        any_retire |= rh[g] != 0;
    }
    for (int i = 0; i < nadm; ++i) {
        const int g = adm_graph[i];
        if (g < 0 || g >= ng || adm_slot[i] < 0 || adm_slot[i] >= b->hgd[g].nroots || adm_root[i] < 0 ||
            adm_root[i] >= b->hgd[g].n)
            return G5_ERR_INVALID_ARG;
        ah[i].graph = g;
        ah[i].slot = adm_slot[i];
        ah[i].root = adm_root[i];
    }
    Admit *ad = reinterpret_cast<Admit *>(b->adm_dev);
    uint64_t *rd = reinterpret_cast<uint64_t *>(ad + 64 * ng);
    G5_CUDA(cudaEventRecord(b->ev0, s));
    if (any_retire || nadm) {
        G5_CUDA(cudaMemcpyAsync(b->adm_dev, b->adm_host, sizeof(Admit) * 64 * ng + sizeof(uint64_t) * ng,
                                cudaMemcpyHostToDevice, s));
    }
    if (any_retire) k_sclear<<<g5::grid_for(8), kB, 0, s>>>(b->args, rd);
    if (nadm) k_sadmit<<<1, 128, 0, s>>>(b->args, ad, nadm);
    enqueue_batch(b, b->args, s, true);
    G5_CUDA(cudaEventRecord(b->ev1, s));
    G5_CUDA(cudaMemcpyAsync(b->hgd.data(), b->gd, sizeof(GraphDesc) * ng, cudaMemcpyDeviceToHost, s));
    G5_CUDA(cudaMemcpyAsync(b->h_st, b->st, sizeof(BState), cudaMemcpyDeviceToHost, s));
    G5_CUDA(cudaStreamSynchronize(s));
    // active slots: in the frontier the step just wrote (collected by the
    // count kernel) plus anything the expansion put into the next frontier
    for (int g = 0; g < ng; ++g) active_mask[g] = b->hgd[g].amask;
    if (device_ms) {
        float ms = 0;
        cudaEventElapsedTime(&ms, b->ev0, b->ev1);
        *device_ms = ms;
    }
    return b->h_st->err ? G5_ERR_CAPACITY : G5_OK;
}

g5_status g5_batch_root_parents(const uint32_t *pred_dev, int64_t n, int nroots, int r, uint32_t *dst_dev,
                                void *stream)
{
    if (!pred_dev || !dst_dev || n < 0 || nroots < 1 || nroots > 64 || r < 0 || r >= nroots)
        return G5_ERR_INVALID_ARG;
    if (n == 0) return G5_OK;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const int blocks = (int)std::min<int64_t>((n + 255) / 256, (int64_t)g5::grid_for(8));
    k_gather_root<<<blocks, 256, 0, s>>>(pred_dev, (uint32_t)nroots, (uint32_t)r, n, dst_dev);
    return cudaGetLastError() == cudaSuccess ? G5_OK : G5_ERR_CUDA;
}

g5_status g5_batch_destroy(g5_batch *b)
{
    if (!b) return G5_ERR_INVALID_ARG;
    cudaStreamSynchronize(b->stream);
    free_batch(b);
    delete b;
    return G5_OK;
}

g5_status g5_batch_launch(g5_batch *b, const int64_t *roots_host, const int *nroots, uint32_t *pred_out_dev)
{
    if (!b || !roots_host || !nroots || !pred_out_dev) return G5_ERR_INVALID_ARG;
    const int ng = (int)b->graphs.size();
    uint64_t pb = 0;
    int off = 0;
    for (int i = 0; i < ng; ++i) {
        if (nroots[i] < 0 || nroots[i] > 64) return G5_ERR_INVALID_ARG;
        GraphDesc &d = b->hgd[i];
        d.nroots = nroots[i];
        d.mask = nroots[i] == 64 ? ~0ull : ((1ull << nroots[i]) - 1);
        d.pred_base = pb;
        pb += (uint64_t)nroots[i] * (uint64_t)d.n;
        b->h_root_off[i] = off;
        for (int r = 0; r < nroots[i]; ++r) {
            const int64_t v = roots_host[off + r];
            if (v < 0 || v >= d.n) return G5_ERR_INVALID_ARG;
            b->h_roots[off + r] = v;
        }
        off += nroots[i];
    }
    b->h_root_off[ng] = off;
    cudaStream_t s = b->stream;
    b->args.pred = pred_out_dev;
    b->args.serving = 0;
    if (!b->exec || b->bound_pred != pred_out_dev) {
        G5_TRY(build_batch_graph(b));
        b->bound_pred = pred_out_dev;
    }
    G5_CUDA(cudaMemcpyAsync(b->gd, b->hgd.data(), sizeof(GraphDesc) * ng, cudaMemcpyHostToDevice, s));
    G5_CUDA(cudaMemcpyAsync(b->roots, b->h_roots, sizeof(int64_t) * (off ? off : 1), cudaMemcpyHostToDevice, s));
    G5_CUDA(cudaMemcpyAsync(b->root_off, b->h_root_off, sizeof(int32_t) * (ng + 1), cudaMemcpyHostToDevice, s));
    G5_CUDA(cudaEventRecord(b->ev0, s));
    if (pb) G5_CUDA(cudaMemsetAsync(pred_out_dev, 0xFF, sizeof(uint32_t) * pb, s));
    G5_CUDA(cudaGraphLaunch(b->exec, s));
    G5_CUDA(cudaEventRecord(b->ev1, s));
    G5_CUDA(cudaMemcpyAsync(b->h_st, b->st, sizeof(BState), cudaMemcpyDeviceToHost, s));
    return G5_OK;
}

g5_status g5_batch_poll(g5_batch *b, int wait, int *done, double *device_ms)
{
    if (!b || !done) return G5_ERR_INVALID_ARG;
    if (wait) {
        G5_CUDA(cudaStreamSynchronize(b->stream));
    } else {
        const cudaError_t e = cudaStreamQuery(b->stream);
        if (e == cudaErrorNotReady) {
            *done = 0;
            return G5_OK;
        }
        G5_CUDA(e);
    }
    *done = 1;
    if (device_ms) {
        float ms = 0;
        cudaEventElapsedTime(&ms, b->ev0, b->ev1);
        *device_ms = ms;
    }
    if (b->h_st->err & 8u) return G5_ERR_TIMEOUT;
    if (b->h_st->err) return G5_ERR_CAPACITY;
    return G5_OK;
}

g5_status g5_batch_run(g5_batch *b, const int64_t *roots_host, const int *nroots, uint32_t *pred_out_dev,
                       double *device_ms)
{
    G5_TRY(g5_batch_launch(b, roots_host, nroots, pred_out_dev));
    int done = 0;
    return g5_batch_poll(b, 1, &done, device_ms);
}

}  // extern "C"
