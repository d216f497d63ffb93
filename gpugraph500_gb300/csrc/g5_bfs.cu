// g5_bfs.cu -- plain (one root per search) direction-optimising BFS.
//
// Replaces the reference's CUDA_BFS backend (cpu_2d/cuda/cuda_bfs.cu) and
// the b40c enactor it drives (b40c/graph/bfs/enactor_multi_gpu_2d.cuh:741-1101)
// for a 1x1 process grid.  Per level, all on the device:
//
//   expand   top-down (queue, edge-balanced tiles, next-bit atomicOr) or
//            bottom-up (bitmap sweep, first hit in the sorted adjacency)
//   fixup    after top-down: parents of the new vertices (first frontier hit)
//   count    popcount + degree sum of the next-frontier bitmap per chunk; the
//            last block to finish does the chunk prefix sums, the Beamer
//            direction switch and the loop condition
//   write    visited |= next, next -> front, sorted queue + edge offsets
//   codec    optional s4-bp128 encode + decode of the sorted queue; the
//            decoded queue feeds the next top-down level
//
// The level loop is one CUDA graph with a conditional while node, so a
// search costs one graph launch and one small read-back at the end (the
// reference copies the visited mask and the queue across PCIe every level,
// cuda_bfs.cu:252-269,397-450,524-529).
//
// Parent choice: a vertex discovered at level L+1 gets the smallest adjacent
// vertex of level L: the first frontier hit of its ascending adjacency, found
// by the bottom-up sweep itself, or on a top-down level by a 64-bit atomicMin
// per discovered edge (parent_mode 0, the default).  parent_mode 1 and 2 keep
// the atomicMin for vertices of degree > 64 only (1) or not at all (2) and
// find the other parents with a fix-up sweep of the new vertices' adjacency;
// all three give the same parents.  This is the parent
// CPUBFS_bin's ascending first-writer sweep picks (cpu_2d/cpubfs_bin.cpp:
// 143-180), so parents equal the reference CPU path's, not only valid ones.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "g5_codec_dev.cuh"
#include "g5_common.cuh"
#include "g5_internal.h"

namespace {

constexpr int kBlock = 256;
constexpr int kWarps = kBlock / 32;
// Bitmap words per compaction chunk (one block of k_count / k_write each):
// per graph the smallest of 256, 512, 1024 and 2048 that gives at most
// kMaxChunks chunks, so small graphs still get many blocks and large ones a
// short chunk scan (per search, against 2048 everywhere: scale 16 -18 %,
// scale 20 -15 % with 512, each about 3 % more with 256; scale 24 -3 % with
// 1024).
constexpr int kMaxChunks = 512;
// Graphs of at least this many vertices sweep the unvisited list from their
// first bottom-up level on (scale 22: 1.7 % faster per search; scale 20: 3 %
// slower).
constexpr int64_t kListFirst = (int64_t)1 << 21;
constexpr uint32_t kTileDefault = 256;  // frontier edges per top-down warp tile
constexpr int kBuSerialDefault = 8;     // entries a lane scans alone before the warp helps
constexpr uint32_t kHeavy = 64;    // degree above which top-down sets the parent itself
// Sparse levels: a top-down level whose frontier has at most kSparseCap
// adjacency entries, or a bottom-up level sweeping an unvisited list of at
// most kSparseCap vertices, adds at most kSparseCap vertices; it also
// appends them to a list and sums their degrees.  If their degrees sum to at
// most kSparseEdges and the next level is top-down, k_count returns at once
// and block 0 of k_write turns the list into the next queue, instead of two
// passes over the whole bitmaps.
constexpr uint32_t kSparseCap = 4096;
constexpr uint64_t kSparseEdges = 65536;
constexpr int kSparseRound = 4;  // list entries per thread per round of the finish

enum : int32_t { DIR_TD = 0, DIR_BU = 1 };

struct LevelRec {
    int32_t dir;        // direction used to expand this level's frontier
    int32_t pad;
    uint64_t nf;        // frontier vertices
    uint64_t mf;        // their adjacency entries
    uint64_t examined;  // adjacency entries read while expanding
};

struct BfsState {
    int32_t level;      // index L of the frontier currently held
    int32_t dir;        // direction for expanding F_L
    uint64_t nf, mf;    // |F_L| and its adjacency entries
    uint64_t mu;        // adjacency entries of still-unvisited vertices
    uint64_t nvisited;
    uint64_t examined;  // accumulator of the running expansion
    uint32_t err;
    int32_t want_queue; // 1 if F_L is also held as a sorted queue
    int32_t bu_levels;
    int32_t list_mode;  // 1: this bottom-up level sweeps the unvisited list
    uint64_t codec_acc[2]; // encoded words, values through the codec
    uint64_t ulen;      // unvisited list length
    uint64_t slen;      // vertices appended to the sparse list by this level
    uint64_t stm;       // their adjacency entries (degree sum)
    int32_t sparse;     // 1: this top-down level appends what it discovers
    int32_t sdone;      // 1: the sparse path took this level (set by k_count)
};

// Where the in-loop codec's streams are copied when a caller asks for them
// (g5_bfs_codec_capture); buf == nullptr leaves the copy off.
struct CodecCapture {
    uint32_t *buf;         // streams, each starting at a multiple of 4 words
    uint64_t cap;          // words in buf
    uint64_t *rec;         // per captured level: level, values, words, offset
    uint32_t max_rec;
    uint32_t count;        // levels captured by the current search
    uint64_t off;          // next free word of buf
    uint32_t overflow;     // a stream or record did not fit
    uint32_t blocks_done;  // blocks of k_codec_capture finished
};

struct BfsArgs {
    const int64_t *row_off;
    const uint32_t *col;
    const uint32_t *deg;
    int64_t n;
    int64_t nnz;
    uint64_t nwords;
    uint32_t nchunks;
    int chunk_words;      // bitmap words per compaction chunk: 256, 512, 1024 or 2048
    int list_first;       // 1: the first bottom-up level of a run sweeps the unvisited list too
    uint32_t *visited;
    uint32_t *front;
    uint32_t *next;
    int64_t *pred;
    int32_t *level;       // may be null
    uint32_t *queue;      // sorted next-frontier queue
    const uint32_t *qsrc; // queue the top-down expansion reads (decoded if codec)
    uint64_t *qoff;       // edge offset of each queue entry (+ sentinel)
    int64_t *qbase;       // row_off[u] - qoff[i]
    uint32_t *tile_start; // first queue index of each top-down tile
    const uint32_t *heavy; // one bit per vertex of degree > kHeavy
    const uint32_t *ro32;  // row offsets as uint32 when nnz < 2^32, else null
    uint32_t *multi;       // vertices a top-down level reached more than once
    uint32_t *wdeg;        // per word: degree sum of the vertices bottom-up added
    unsigned *done;        // blocks of k_count finished (reset by the last one)
    uint32_t *ulist;       // sorted unvisited vertices for a bottom-up level
    uint64_t *chunk_u;     // per chunk: unvisited vertices after the level
    uint32_t *slist;       // vertices a sparse top-down level discovered (unordered)
    int parent_mode;       // 0 atomicMin, 1 heavy atomicMin + fix-up, 2 first writer + fix-up
    const uint32_t *first; // first (smallest) neighbour of each vertex, 0 for isolated ones
    uint64_t tile;         // frontier edges per top-down warp tile (a power of two >= 32)
    int tile_shift;        // log2(tile)
    int bu_serial;         // entries a bottom-up lane scans alone before the warp helps
    uint64_t max_tiles;
    uint64_t *chunk_n;
    uint64_t *chunk_m;
    BfsState *st;
    LevelRec *log;
    int max_levels;
    const int64_t *root_dev;
    double alpha, beta;
    int codec;
    const uint64_t *codec_scal; // CS_* scalars of the codec work
    CodecCapture *ccap;         // stream capture descriptor (codec searches), or null
    cudaGraphConditionalHandle cond;
    int use_cond;
};

__device__ __forceinline__ uint64_t warp_sum_u64(uint64_t v)
{
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
    return v;
}

// Whether the next top-down level, whose frontier has tm adjacency entries,
// appends its discoveries to the sparse list (it discovers at most tm
// vertices, so the list always holds them).  The list is unordered, so
// searches that encode each level's sorted queue, and the fix-up parent
// modes, keep the full passes.
__device__ __forceinline__ int32_t sparse_next(const BfsArgs &a, uint64_t tm)
{
    return (a.slist && a.codec == 0 && a.parent_mode == 0 && tm <= kSparseCap) ? 1 : 0;
}

// Whether a bottom-up level that sweeps an unvisited list of ulen vertices
// appends what it finds (at most ulen vertices).
__device__ __forceinline__ int32_t sparse_next_list(const BfsArgs &a, uint64_t ulen)
{
    return (a.slist && a.codec == 0 && a.parent_mode == 0 && ulen <= kSparseCap) ? 1 : 0;
}

// ---- init -----------------------------------------------------------------

__global__ void k_init(BfsArgs a)
{
    __shared__ int64_t s_root, s_deg, s_base;
    __shared__ int s_ok;
    if (threadIdx.x == 0) {
        int64_t r = *a.root_dev;
        s_ok = (r >= 0 && r < a.n);
        s_root = s_ok ? r : 0;
        s_base = s_ok ? a.row_off[r] : 0;
        s_deg = s_ok ? a.row_off[r + 1] - s_base : 0;
        BfsState *st = a.st;
        st->level = 0;
        st->dir = DIR_TD;
        st->nf = s_ok ? 1 : 0;
        st->mf = (uint64_t)s_deg;
        st->mu = (uint64_t)(a.nnz - s_deg);
        st->nvisited = s_ok ? 1 : 0;
        st->examined = 0;
        st->err = s_ok ? 0u : G5_DEVERR_CAPACITY;
        st->want_queue = 1;
        st->bu_levels = 0;
        st->codec_acc[0] = st->codec_acc[1] = 0;
        st->list_mode = 0;
        st->ulen = 0;
        st->slen = 0;
        st->stm = 0;
        st->sparse = s_ok ? sparse_next(a, (uint64_t)s_deg) : 0;
        st->sdone = 0;
        a.log[0].dir = DIR_TD;
        a.log[0].nf = st->nf;
        a.log[0].mf = st->mf;
        a.log[0].examined = 0;
        if (a.ccap) {
            a.ccap->count = 0;
            a.ccap->off = 0;
            a.ccap->overflow = 0;
        }
        if (s_ok) {
            const int64_t r = s_root;
            a.pred[r] = r;
            a.visited[r >> 5] |= 1u << (r & 31);
            a.front[r >> 5] |= 1u << (r & 31);
            if (a.level) a.level[r] = 0;
            a.queue[0] = (uint32_t)r;
            if (a.qsrc != a.queue) const_cast<uint32_t *>(a.qsrc)[0] = (uint32_t)r;
            a.qoff[0] = 0;
            a.qoff[1] = (uint64_t)s_deg;
            a.qbase[0] = s_base;
        }
        // vertices past n in the last word count as visited
        const int tail = (int)(a.n & 31);
        if (tail) a.visited[a.nwords - 1] |= ~((1u << tail) - 1u);
    }
    __syncthreads();
    if (!s_ok) return;
    const uint64_t tiles = ((uint64_t)s_deg + a.tile - 1) >> a.tile_shift;
    for (uint64_t t = threadIdx.x; t < tiles; t += blockDim.x) a.tile_start[t] = 0;
}

// ---- expansion ----------------------------------------------------------------

__device__ void expand_td(const BfsArgs &a, uint64_t &examined)
{
    __shared__ uint64_t s_q[kWarps][32];
    const int lane = g5_lane();
    const int wib = threadIdx.x >> 5;
    const uint64_t gw = (uint64_t)blockIdx.x * kWarps + wib;
    const uint64_t nw = (uint64_t)gridDim.x * kWarps;
    const uint64_t mf = a.st->mf, nf = a.st->nf;
    const bool sparse = a.st->sparse != 0;  // the same for the whole grid
    const uint64_t ntiles = (mf + a.tile - 1) >> a.tile_shift;
    if (ntiles > a.max_tiles) {
        if (threadIdx.x == 0 && blockIdx.x == 0) atomicOr(&a.st->err, G5_DEVERR_CAPACITY);
        return;
    }
    for (uint64_t t = gw; t < ntiles; t += nw) {
        const uint64_t e0 = t << a.tile_shift;
        const uint64_t e1 = min(e0 + a.tile, mf);
        uint64_t cur = a.tile_start[t];
        for (uint64_t gb = e0; gb < e1; gb += 32) {
            const uint64_t idx = cur + 1 + lane;
            s_q[wib][lane] = idx <= nf ? a.qoff[idx] : ~0ull;
            __syncwarp();
            const uint64_t e = gb + lane;
            int lo = 0, hi = 32;
            while (lo < hi) {
                int mid = (lo + hi) >> 1;
                if (s_q[wib][mid] <= e) lo = mid + 1;
                else hi = mid;
            }
            const uint64_t i = cur + lo;
            // i(e) <= cur + 32 when every queued vertex has an edge (cur is
            // the vertex of the previous group's last edge); lo == 32 is then
            // exact, and the next boundary confirms it
            bool claimed = false;  // this lane set v's next bit first (sparse levels)
            uint32_t cv = 0;
            bool in_range = true;
            if (lo == 32 && e < e1) in_range = (i + 1 > nf) ? false : (a.qoff[i + 1] > e);
            if (e < e1) {
                if (!in_range) {
                    // a queued vertex without edges: only a non-symmetric CSR
                    atomicOr(&a.st->err, G5_DEVERR_CAPACITY);
                } else {
                    // light vertices: only the next-frontier bit is set here
                    // (an L2-resident atomic) and k_fixup finds the parent in
                    // the vertex's short adjacency; heavy vertices, whose scan
                    // could be long, take the smallest parent by atomicMin
                    const uint32_t v = __ldg(a.col + (a.qbase[i] + (int64_t)e));
                    const uint32_t bit = 1u << (v & 31);
                    if (!(a.visited[v >> 5] & bit)) {
                        const unsigned long long u = a.qsrc[i];
                        if (a.parent_mode == 0 || (__ldg(a.heavy + (v >> 5)) & bit)) {
                            // parents only decrease during a level, so a read
                            // value <= u (even a stale one) makes the atomic moot
                            if ((unsigned long long)a.pred[v] > u)
                                atomicMin((unsigned long long *)(a.pred + v), u);
                            if (!(a.next[v >> 5] & bit)) {
                                if (sparse) {
                                    claimed = !(atomicOr(a.next + (v >> 5), bit) & bit);
                                    cv = v;
                                } else {
                                    atomicOr(a.next + (v >> 5), bit);
                                }
                            }
                        } else if (a.parent_mode == 1) {
                            if (!(a.next[v >> 5] & bit)) atomicOr(a.next + (v >> 5), bit);
                        } else {
                            // first discoverer writes its parent; a vertex
                            // reached again is left to the fix-up sweep
                            const uint32_t old = (a.next[v >> 5] & bit) ? bit : atomicOr(a.next + (v >> 5), bit);
                            if (!(old & bit)) atomicMin((unsigned long long *)(a.pred + v), u);
                            else if (!(a.multi[v >> 5] & bit)) atomicOr(a.multi + (v >> 5), bit);
                        }
                    }
                }
            }
            if (sparse) {
                // the warp's new vertices go to the list with one atomic, and
                // their degree sum to the level's with another
                const unsigned cm = __ballot_sync(0xFFFFFFFFu, claimed);
                if (cm) {
                    const int lead = __ffs(cm) - 1;
                    const uint64_t dsum = warp_sum_u64(claimed ? (uint64_t)__ldg(a.deg + cv) : 0ull);
                    unsigned long long base = 0;
                    if (lane == lead) {
                        base = atomicAdd((unsigned long long *)&a.st->slen, (unsigned long long)__popc(cm));
                        atomicAdd((unsigned long long *)&a.st->stm, (unsigned long long)dsum);
                    }
                    base = __shfl_sync(0xFFFFFFFFu, base, lead);
                    const uint64_t p = base + __popc(cm & g5_lanemask_lt());
                    if (claimed && p < kSparseCap) a.slist[p] = cv;
                }
            }
            cur = __shfl_sync(0xFFFFFFFFu, i, 31);
            __syncwarp();
        }
        if (lane == 0) examined += e1 - e0;
    }
}

// One warp per 32-vertex word.  BOTTOM_UP: the candidates are the unvisited
// vertices; a candidate with a neighbour in the frontier joins the next
// frontier with the first such neighbour of its ascending adjacency as parent.
// FIXUP (after a top-down level): the candidates are the vertices top-down
// just discovered; each takes the first frontier neighbour of its adjacency.
// Either way the parent is the smallest neighbour in the frontier.
// Warp-collective search of each active lane's adjacency [s, e) for its
// first vertex in the frontier: every lane scans its first bu_serial entries
// alone (four independent loads at a time), then the warp finishes the longer
// lists one at a time, 32 entries per step (the first set ballot bit is the
// smallest index).  Returns found / par per lane and the entries read.
template <typename Off>
__device__ __forceinline__ void first_hit(const BfsArgs &a, bool mine, Off s, Off e, uint32_t u0, bool &found,
                                          uint32_t &par, uint64_t &ex)
{
    const int lane = g5_lane();
    const uint32_t *__restrict__ front = a.front;
    const uint32_t *__restrict__ col = a.col;
    found = false;
    par = 0;
    Off j = s;
    // the first neighbour comes from the dense copy (loaded with the offsets,
    // coalesced), so a vertex whose first neighbour is in the frontier never
    // touches its row
    if (mine && s < e) {
        if ((__ldg(front + (u0 >> 5)) >> (u0 & 31)) & 1u) {
            found = true;
            par = u0;
        }
        j = s + 1;
    }
    // (callers pass s = e = 0 on lanes without a candidate, so those lanes
    // scan nothing here)
    const Off lim = min(e, (Off)(s + a.bu_serial));
    while (j < lim && !found) {
        uint32_t u[4];
        bool h[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) u[k] = (j + k < lim) ? __ldg(col + j + k) : 0u;
#pragma unroll
        for (int k = 0; k < 4; ++k)
            h[k] = (j + k < lim) && ((__ldg(front + (u[k] >> 5)) >> (u[k] & 31)) & 1u);
        int k = 0;
        while (k < 4 && j + k < lim && !h[k]) ++k;
        if (k < 4 && j + k < lim) {
            found = true;
            par = u[k];
            j += k + 1;
        } else {
            j = min((Off)(j + 4), lim);
        }
    }
    ex = mine ? (uint64_t)(j - s) : 0;
    unsigned pend = __ballot_sync(0xFFFFFFFFu, mine && !found && j < e);
    while (pend) {
        const int l = __ffs(pend) - 1;
        pend &= pend - 1;
        Off jj = __shfl_sync(0xFFFFFFFFu, j, l);
        const Off ee = __shfl_sync(0xFFFFFFFFu, e, l);
        const Off st = jj;
        bool got = false;
        uint32_t gpar = 0;
        while (jj < ee) {
            const Off idx = jj + (Off)lane;
            uint32_t u = 0;
            bool hit = false;
            if (idx < ee) {
                u = __ldg(col + idx);
                hit = (__ldg(front + (u >> 5)) >> (u & 31)) & 1u;
            }
            const unsigned m = __ballot_sync(0xFFFFFFFFu, hit);
            if (m) {
                const int f = __ffs(m) - 1;
                gpar = __shfl_sync(0xFFFFFFFFu, u, f);
                got = true;
                jj += f + 1;
                break;
            }
            jj += 32;
        }
        jj = min(jj, ee);
        if (lane == l) {
            found = got;
            par = gpar;
            ex += (uint64_t)(jj - st);
        }
    }
}

// Row offsets of v: the uint32 copy when nnz < 2^32 (half the bytes, and
// 32-bit loop indices), else the int64 array.
__device__ __forceinline__ void load_offsets(const BfsArgs &a, uint64_t v, uint32_t &s, uint32_t &e)
{
    s = a.ro32[v];
    e = a.ro32[v + 1];
}
__device__ __forceinline__ void load_offsets(const BfsArgs &a, uint64_t v, int64_t &s, int64_t &e)
{
    s = a.row_off[v];
    e = a.row_off[v + 1];
}

// One warp per 32-vertex word.  BOTTOM-UP: the candidates are the unvisited
// vertices; a candidate with a neighbour in the frontier joins the next
// frontier with the first such neighbour of its ascending adjacency as
// parent (kept for reference; bottom-up levels normally sweep the unvisited
// list, bottom_up_list).  FIXUP (after a top-down level, parent modes 1 and
// 2): the candidates are vertices top-down just discovered; each takes the
// first frontier neighbour of its adjacency.
template <bool FIXUP, typename Off>
__device__ void sweep(const BfsArgs &a, uint64_t &examined)
{
    const int lane = g5_lane();
    const uint64_t gw = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    // FIXUP candidates are sparse: a warp loads 32 words at once (one per
    // lane, coalesced) and visits only the non-empty ones.  Bottom-up
    // candidates are dense: one word per warp step keeps more words in flight.
    const uint64_t step = FIXUP ? 32 : 1;
    for (uint64_t w0 = gw * step; w0 < a.nwords; w0 += nw * step) {
      uint32_t cw = 0;
      unsigned act;
      if (FIXUP) {
          const uint64_t wl = w0 + lane;
          if (wl < a.nwords) {
              if (a.parent_mode == 2) {
                  cw = a.multi[wl] & ~__ldg(a.heavy + wl);
                  if (cw) a.multi[wl] = 0;
              } else {
                  cw = a.parent_mode == 1 ? (a.next[wl] & ~__ldg(a.heavy + wl)) : 0u;
              }
          }
          act = __ballot_sync(0xFFFFFFFFu, cw != 0u);
      } else {
          cw = ~a.visited[w0];
          act = cw ? 1u : 0u;
      }
      while (act) {
        const int jw = __ffs(act) - 1;
        act &= act - 1;
        const uint64_t w = w0 + jw;
        const uint32_t cand_word = FIXUP ? __shfl_sync(0xFFFFFFFFu, cw, jw) : cw;
        const uint64_t v = w * 32 + lane;
        const bool mine = (cand_word >> lane) & 1u;
        Off s = 0, e = 0;
        uint32_t u0 = 0;
        if (mine) {
            load_offsets(a, v, s, e);
            u0 = a.first[v];
        }
        bool found;
        uint32_t par;
        uint64_t ex;
        first_hit<Off>(a, mine, s, e, u0, found, par, ex);
        if (found) a.pred[v] = (int64_t)par;
        if (FIXUP) {
            if (mine && !found) atomicOr(&a.st->err, G5_DEVERR_CAPACITY);  // cannot happen on a symmetric CSR
        } else {
            const unsigned fm = __ballot_sync(0xFFFFFFFFu, found);
            if (fm) {
                // degree sum of the added vertices: the counting pass after a
                // bottom-up level then reads one word per 32 vertices
                uint32_t dsum = found ? (uint32_t)(e - s) : 0u;
#pragma unroll
                for (int o = 16; o; o >>= 1) dsum += __shfl_xor_sync(0xFFFFFFFFu, dsum, o);
                if (lane == 0) {
                    a.next[w] = fm;
                    a.wdeg[w] = dsum;
                }
            }
        }
        examined += ex;
      }
    }
}

// First bottom-up level on graphs of fewer than kListFirst vertices: one warp
// per 32-vertex word, software-pipelined so that a word's visited bits are
// loaded two steps and its candidates' row offsets one step before the word
// is scanned; the scan of one word then overlaps the loads of the next two
// instead of waiting on each in turn.
template <typename Off>
__device__ void sweep_bu(const BfsArgs &a, uint64_t &examined)
{
    const int lane = g5_lane();
    const uint64_t gw = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const uint64_t nwords = a.nwords;
    // stage 2: candidates of the word after next; stage 1: next word's offsets
    uint32_t c1 = gw < nwords ? ~a.visited[gw] : 0u;
    uint32_t c2 = gw + nw < nwords ? ~a.visited[gw + nw] : 0u;
    Off s1 = 0, e1 = 0;
    uint32_t f1 = 0;
    if ((c1 >> lane) & 1u) {
        load_offsets(a, gw * 32 + lane, s1, e1);
        f1 = a.first[gw * 32 + lane];
    }
    for (uint64_t w = gw; w < nwords; w += nw) {
        const uint32_t cw = c1;
        const Off s = s1, e = e1;
        const uint32_t u0 = f1;
        c1 = c2;
        const uint64_t w2 = w + 2 * nw;
        c2 = w2 < nwords ? ~a.visited[w2] : 0u;
        s1 = e1 = 0;
        if ((c1 >> lane) & 1u) {
            load_offsets(a, (w + nw) * 32 + lane, s1, e1);
            f1 = a.first[(w + nw) * 32 + lane];
        }
        if (!cw) continue;
        const uint64_t v = w * 32 + lane;
        const bool mine = (cw >> lane) & 1u;
        bool found;
        uint32_t par;
        uint64_t ex;
        first_hit<Off>(a, mine, s, e, u0, found, par, ex);
        if (found) a.pred[v] = (int64_t)par;
        const unsigned fm = __ballot_sync(0xFFFFFFFFu, found);
        if (fm) {
            // degree sum of the added vertices: the counting pass after a
            // bottom-up level then reads one word per 32 vertices
            uint32_t dsum = found ? (uint32_t)(e - s) : 0u;
#pragma unroll
            for (int o = 16; o; o >>= 1) dsum += __shfl_xor_sync(0xFFFFFFFFu, dsum, o);
            if (lane == 0) {
                a.next[w] = fm;
                a.wdeg[w] = dsum;
            }
        }
        examined += ex;
    }
}

// Bottom-up level over the sorted list of unvisited vertices (written by the
// previous level's compaction): 32 candidates per warp step, every lane
// busy, instead of sweeping all words of which many hold no candidate.  The
// list entries are loaded two steps and their row offsets one step ahead.
template <typename Off>
__device__ void bottom_up_list(const BfsArgs &a, uint64_t &examined)
{
    const int lane = g5_lane();
    const uint64_t gw = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const uint64_t len = a.st->ulen;
    const uint32_t *__restrict__ list = a.ulist;
    const uint64_t stride = nw * 32;
    uint64_t p1 = gw * 32 + lane, p2 = p1 + stride;
    uint32_t v1 = p1 < len ? list[p1] : 0u;
    uint32_t v2 = p2 < len ? list[p2] : 0u;
    Off s1 = 0, e1 = 0;
    uint32_t f1 = 0;
    if (p1 < len) {
        load_offsets(a, v1, s1, e1);
        f1 = a.first[v1];
    }
    for (uint64_t b0 = gw * 32; b0 < len; b0 += stride) {
        const bool mine = b0 + lane < len;
        const uint32_t v = v1;
        const Off s = s1, e = e1;
        const uint32_t u0 = f1;
        v1 = v2;
        p1 = p2;
        p2 += stride;
        v2 = p2 < len ? list[p2] : 0u;
        s1 = e1 = 0;
        if (p1 < len) {
            load_offsets(a, v1, s1, e1);
            f1 = a.first[v1];
        }
        bool found;
        uint32_t par;
        uint64_t ex;
        first_hit<Off>(a, mine, s, e, u0, found, par, ex);
        if (found) a.pred[v] = (int64_t)par;
        // the list is sorted, so lanes holding vertices of one bitmap word
        // are adjacent: a segmented scan gives the last lane of each word
        // the word's new bits and their degree sum, and that lane alone
        // updates next and wdeg (one atomic pair per word, not per vertex)
        const unsigned fm = __ballot_sync(0xFFFFFFFFu, found);
        if (fm && a.st->sparse) {
            // the warp's new vertices go to the sparse list with one atomic,
            // their degree sum to the level's with another (the flag is read
            // here, not kept in a register across the loop)
            const int lead = __ffs(fm) - 1;
            const uint64_t dsum = warp_sum_u64(found ? (uint64_t)(e - s) : 0ull);
            unsigned long long base = 0;
            if (lane == lead) {
                base = atomicAdd((unsigned long long *)&a.st->slen, (unsigned long long)__popc(fm));
                atomicAdd((unsigned long long *)&a.st->stm, (unsigned long long)dsum);
            }
            base = __shfl_sync(0xFFFFFFFFu, base, lead);
            const uint64_t p = base + __popc(fm & g5_lanemask_lt());
            if (found && p < kSparseCap) a.slist[p] = v;
        }
        if (fm) {
            const uint32_t wv = mine ? (v >> 5) : 0xFFFFFFFFu;
            const uint32_t wprev = __shfl_up_sync(0xFFFFFFFFu, wv, 1);
            const unsigned heads = __ballot_sync(0xFFFFFFFFu, lane == 0 || wprev != wv);
            const int head = 31 - __clz(heads & (0xFFFFFFFFu >> (31 - lane)));
            uint32_t bits = found ? 1u << (v & 31) : 0u;
            uint32_t dsum = found ? (uint32_t)(e - s) : 0u;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t b2 = __shfl_up_sync(0xFFFFFFFFu, bits, o);
                const uint32_t d2 = __shfl_up_sync(0xFFFFFFFFu, dsum, o);
                if (lane - o >= head) {
                    bits |= b2;
                    dsum += d2;
                }
            }
            const uint32_t wnext = __shfl_down_sync(0xFFFFFFFFu, wv, 1);
            if (bits && (lane == 31 || wnext != wv)) {
                atomicOr(a.next + wv, bits);
                atomicAdd(a.wdeg + wv, dsum);
            }
        }
        examined += ex;
    }
}

__device__ __forceinline__ void add_examined(const BfsArgs &a, uint64_t examined)
{
    examined = warp_sum_u64(examined);
    __shared__ uint64_t s_ex[kWarps];
    if (g5_lane() == 0) s_ex[threadIdx.x >> 5] = examined;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint64_t t = 0;
        for (int i = 0; i < kWarps; ++i) t += s_ex[i];
        if (t) atomicAdd((unsigned long long *)&a.st->examined, (unsigned long long)t);
    }
}

// Top-down expansion of the level (no-op when the level is bottom-up).
__global__ void __launch_bounds__(kBlock, 8) k_td(BfsArgs a)
{
    if (a.st->err || a.st->dir != DIR_TD) return;
    uint64_t examined = 0;
    expand_td(a, examined);
    add_examined(a, examined);
}

// Bottom-up expansion of the level (no-op when the level is top-down): the
// list of unvisited vertices, or on small graphs the bitmap words for the
// first bottom-up level of a run.
template <typename Off>
__global__ void __launch_bounds__(kBlock, 8) k_bu(BfsArgs a)
{
    if (a.st->err || a.st->dir != DIR_BU) return;
    uint64_t examined = 0;
    if (a.st->list_mode) bottom_up_list<Off>(a, examined);
    else sweep_bu<Off>(a, examined);
    add_examined(a, examined);
}

// Parents of the vertices a top-down level discovered (no-op after bottom-up).
__global__ void __launch_bounds__(kBlock) k_fixup(BfsArgs a)
{
    if (a.st->err || a.st->dir != DIR_TD || a.parent_mode == 0) return;
    uint64_t examined = 0;
    if (a.ro32) sweep<true, uint32_t>(a, examined);
    else sweep<true, int64_t>(a, examined);
    examined = warp_sum_u64(examined);
    __shared__ uint64_t s_ex[kWarps];
    if (g5_lane() == 0) s_ex[threadIdx.x >> 5] = examined;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint64_t t = 0;
        for (int i = 0; i < kWarps; ++i) t += s_ex[i];
        if (t) atomicAdd((unsigned long long *)&a.st->examined, (unsigned long long)t);
    }
}

// ---- compaction: count, scan, write ----------------------------------------------

// A compaction chunk is CW bitmap words; each of the 8 warps of a
// block owns 256 consecutive words and walks them 32 at a time: lane l loads
// word l (coalesced), then for every non-empty word the lanes read the
// degrees of its set vertices in one coalesced 128-byte load.
template <int CW>
__device__ __forceinline__ void warp_chunk_counts(const BfsArgs &a, uint64_t wbeg, const uint32_t (&xs)[CW / kWarps / 32],
                                                  uint64_t &cn, uint64_t &cm)
{
    const int lane = g5_lane();
    cn = 0;
    cm = 0;
#pragma unroll
    for (int i = 0; i < CW / kWarps / 32; ++i) {
        const uint32_t x = xs[i];
        cn += __popc(x);
        unsigned act = __ballot_sync(0xFFFFFFFFu, x != 0u);
        while (act) {
            const int j = __ffs(act) - 1;
            act &= act - 1;
            const uint32_t wj = __shfl_sync(0xFFFFFFFFu, x, j);
            if ((wj >> lane) & 1u) cm += __ldg(a.deg + (wbeg + i * 32 + j) * 32 + lane);
        }
    }
    cn = warp_sum_u64(cn);
    cm = warp_sum_u64(cm);
}

// Counting: each thread owns CW / kBlock consecutive words and sums
// popcounts and the degrees of their set vertices (independent loads per
// thread; faster here than the lane-parallel walk of k_write).

__device__ void scan_and_decide(const BfsArgs &a);
__device__ bool sparse_take(const BfsArgs &a);

template <int CW>
__global__ void __launch_bounds__(kBlock, 6) k_count(BfsArgs a)
{
    constexpr int kWordsPerThread = CW / kBlock;
    // a level the sparse path takes needs no counts: block 0 of k_write
    // builds its queue from the list
    __shared__ int s_take;
    if (threadIdx.x == 0) {
        s_take = sparse_take(a) ? 1 : 0;
        if (blockIdx.x == 0) a.st->sdone = s_take;
    }
    __syncthreads();
    if (s_take) return;
    const uint32_t c = blockIdx.x;
    const uint64_t w0 = (uint64_t)c * CW + (uint64_t)threadIdx.x * kWordsPerThread;
    const bool bu = a.st->dir == DIR_BU;  // bottom-up levels leave per-word degree sums
    // unvisited vertices (the list length for a following bottom-up level)
    const bool count_u = bu || a.list_first;
    uint64_t cn = 0, cm = 0, cu = 0;
#pragma unroll
    for (int k = 0; k < kWordsPerThread; ++k) {
        uint32_t x = (w0 + k < a.nwords) ? a.next[w0 + k] : 0u;
        if (count_u && w0 + k < a.nwords) cu += __popc(~(a.visited[w0 + k] | x));
        cn += __popc(x);
        if (bu) {
            if (x) cm += a.wdeg[w0 + k];
            continue;
        }
        // top-down levels: the degrees of the new vertices (the expansion's
        // next-bit atomics stay fire-and-forget; a returning atomic per
        // discovered edge, to add degrees there, cost 5 % of the search)
        while (x) {
            const int b = __ffs(x) - 1;
            x &= x - 1;
            cm += __ldg(a.deg + (w0 + k) * 32 + b);
        }
    }
    cn = warp_sum_u64(cn);
    cm = warp_sum_u64(cm);
    cu = warp_sum_u64(cu);
    __shared__ uint64_t s_n[kWarps], s_m[kWarps], s_u[kWarps];
    if (g5_lane() == 0) {
        s_n[threadIdx.x >> 5] = cn;
        s_m[threadIdx.x >> 5] = cm;
        s_u[threadIdx.x >> 5] = cu;
    }
    __syncthreads();
    __shared__ unsigned s_last;
    if (threadIdx.x == 0) {
        uint64_t tn = 0, tm = 0, tu = 0;
        for (int i = 0; i < kWarps; ++i) {
            tn += s_n[i];
            tm += s_m[i];
            tu += s_u[i];
        }
        a.chunk_n[c] = tn;
        a.chunk_m[c] = tm;
        a.chunk_u[c] = tu;
        __threadfence();
        s_last = atomicAdd(a.done, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (s_last) {
        // every other block has published its counts
        __threadfence();
        scan_and_decide(a);
        if (threadIdx.x == 0) *a.done = 0;
    }
}

// Block-wide exclusive scan of one u64 per thread (blockDim.x a multiple of
// 32, at most 1024); s_warp holds 33 entries.
__device__ uint64_t block_excl_scan_1024(uint64_t v, uint64_t *s_warp, uint64_t &total)
{
    const int lane = g5_lane(), wid = threadIdx.x >> 5;
    const int nwarps = blockDim.x >> 5;
    uint64_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint64_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[wid] = x;
    __syncthreads();
    if (wid == 0) {
        uint64_t y = lane < nwarps ? s_warp[lane] : 0;
        uint64_t z = y;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint64_t t = __shfl_up_sync(0xFFFFFFFFu, z, o);
            if (lane >= o) z += t;
        }
        s_warp[lane] = z - y;
        if (lane == 31) s_warp[32] = z;
    }
    __syncthreads();
    const uint64_t r = x - v + s_warp[wid];
    total = s_warp[32];
    __syncthreads();
    return r;
}

// Chunk prefix sums, the direction switch and the loop condition; run by
// the last block of k_count to finish (it sees every chunk's count).
__device__ void scan_and_decide(const BfsArgs &a)
{
    __shared__ uint64_t s_w[33];
    const uint32_t C = a.nchunks;
    const uint32_t per = (C + blockDim.x - 1) / blockDim.x;
    const uint32_t b0 = threadIdx.x * per;
    uint64_t ln = 0, lm = 0, lu = 0;
    for (uint32_t i = 0; i < per && b0 + i < C; ++i) {
        ln += __ldcg(a.chunk_n + b0 + i);
        lm += __ldcg(a.chunk_m + b0 + i);
        lu += __ldcg(a.chunk_u + b0 + i);
    }
    uint64_t tn, tm, tu;
    uint64_t on = block_excl_scan_1024(ln, s_w, tn);
    uint64_t om = block_excl_scan_1024(lm, s_w, tm);
    uint64_t ou = block_excl_scan_1024(lu, s_w, tu);
    for (uint32_t i = 0; i < per && b0 + i < C; ++i) {
        const uint64_t xn = __ldcg(a.chunk_n + b0 + i), xm = __ldcg(a.chunk_m + b0 + i);
        const uint64_t xu = __ldcg(a.chunk_u + b0 + i);
        a.chunk_n[b0 + i] = on;
        a.chunk_m[b0 + i] = om;
        a.chunk_u[b0 + i] = ou;
        on += xn;
        om += xm;
        ou += xu;
    }
    if (threadIdx.x == 0) {
        BfsState *st = a.st;
        const int32_t L = st->level;
        a.log[L].examined = st->examined;
        const uint64_t mu_after = st->mu >= tm ? st->mu - tm : 0;
        int32_t nd = st->dir;
        if (st->dir == DIR_TD) {
            if ((double)tm > (double)mu_after / a.alpha) nd = DIR_BU;
        } else {
            if ((double)tn < (double)a.n / a.beta && tn < st->nf) nd = DIR_TD;
        }
        const bool want_q = (nd == DIR_TD) || a.codec != 0;
        // a bottom-up level sweeps the list of unvisited vertices that
        // k_write is about to write; on graphs of fewer than kListFirst
        // vertices the first one of a run sweeps the bitmap words instead
        // (there the list costs more to build than it saves; on large graphs
        // the word sweep leaves the lanes of visited vertices idle: the list
        // is 7 % faster per search at scale 26, 4 % at 24)
        st->list_mode = (nd == DIR_BU && (st->dir == DIR_BU || a.list_first)) ? 1 : 0;
        st->ulen = tu;
        st->level = L + 1;
        st->dir = nd;
        st->nf = tn;
        st->mf = tm;
        st->mu = mu_after;
        st->nvisited += tn;
        st->examined = 0;
        st->want_queue = want_q ? 1 : 0;
        // (list_mode: the next level sweeps the unvisited list of tu vertices)
        st->sparse = nd == DIR_TD ? sparse_next(a, tm) : (st->list_mode ? sparse_next_list(a, tu) : 0);
        st->slen = 0;
        st->stm = 0;
        if (tn && nd == DIR_BU) st->bu_levels += 1;
        if (want_q) a.qoff[tn] = tm;
        if (L + 1 < a.max_levels) {
            a.log[L + 1].dir = nd;
            a.log[L + 1].nf = tn;
            a.log[L + 1].mf = tm;
            a.log[L + 1].examined = 0;
        }
        bool cont = tn > 0 && st->err == 0;
        if (cont && L + 2 >= a.max_levels) {
            st->err |= G5_DEVERR_LEVELS;
            cont = false;
        }
        if (a.codec_scal && a.codec_scal[g5::CS_ERR]) cont = false;
        if (a.use_cond) cudaGraphSetConditional(a.cond, cont ? 1u : 0u);
    }
}

// Whether the sparse path takes the level that just expanded.  The
// expansion appended every vertex it added to the list and summed their
// degrees; the path takes the level when the new vertices have at most
// kSparseEdges adjacency entries (a larger next level wants the sorted queue
// the full passes build) and the next level is top-down (a bottom-up one
// needs the frontier bitmap or the unvisited list k_write builds).  Every
// block of k_count evaluates it before any block changes the state.
__device__ bool sparse_take(const BfsArgs &a)
{
    const BfsState *st = a.st;
    if (!st->sparse || st->err || st->slen > kSparseCap || st->stm > kSparseEdges) return false;
    const uint64_t tn = st->slen, tm = st->stm;
    const uint64_t mu_after = st->mu >= tm ? st->mu - tm : 0;
    // the direction rule of scan_and_decide
    const bool next_bu = st->dir == DIR_BU ? !((double)tn < (double)a.n / a.beta && tn < st->nf)
                                           : (double)tm > (double)mu_after / a.alpha;
    return !next_bu;
}

// Block 0 of k_write on a level the sparse path took: the list becomes the
// next queue (edge offsets by block scans of the degrees in list order, row
// bases, tile starts, levels), the new vertices join the visited bitmap,
// their next words (after a bottom-up level also their per-word degree
// sums) are cleared, and the level state and the loop condition are set as
// in scan_and_decide.  Entries are taken kSparseRound per thread per round,
// all of a round's loads issued before any is used.  The queue is not
// sorted: the top-down expansion needs only the edge offsets to follow queue
// order, and parents come from atomicMin whatever the order.
__device__ void sparse_finish(const BfsArgs &a)
{
    __shared__ uint64_t s_w[33];
    BfsState *st = a.st;
    const uint32_t len = (uint32_t)st->slen;
    const int32_t L = st->level;
    const bool bu = st->dir == DIR_BU;
    const uint32_t tid = threadIdx.x;
    uint64_t carry = 0;
    for (uint32_t base = 0; base < len; base += kSparseRound * kBlock) {
        uint32_t vv[kSparseRound], dd[kSparseRound];
        int64_t rs[kSparseRound];
        uint64_t mps[kSparseRound];
#pragma unroll
        for (int k = 0; k < kSparseRound; ++k) {
            const uint32_t i = base + k * kBlock + tid;
            vv[k] = i < len ? a.slist[i] : 0u;
        }
#pragma unroll
        for (int k = 0; k < kSparseRound; ++k) {
            const uint32_t i = base + k * kBlock + tid;
            dd[k] = i < len ? __ldg(a.deg + vv[k]) : 0u;
            rs[k] = i < len ? __ldg(a.row_off + vv[k]) : 0;
        }
#pragma unroll
        for (int k = 0; k < kSparseRound; ++k) {
            mps[k] = 0;
            if (base + k * kBlock < len) {  // the same for every thread
                uint64_t tot = 0;
                mps[k] = carry + block_excl_scan_1024(dd[k], s_w, tot);
                carry += tot;
            }
        }
#pragma unroll
        for (int k = 0; k < kSparseRound; ++k) {
            const uint32_t p = base + k * kBlock + tid;
            if (p < len) {
                const uint32_t v = vv[k];
                const uint64_t mp = mps[k];
                a.queue[p] = v;
                a.qoff[p] = mp;
                a.qbase[p] = rs[k] - (int64_t)mp;
                uint64_t t = (mp + a.tile - 1) >> a.tile_shift;
                const uint64_t tend = (mp + dd[k] + a.tile - 1) >> a.tile_shift;
                for (; t < tend && t < a.max_tiles; ++t) a.tile_start[t] = p;
                if (a.level) a.level[v] = L + 1;
                atomicOr(a.visited + (v >> 5), 1u << (v & 31));
                a.next[v >> 5] = 0;  // every next bit of this level is a list entry
                if (bu) a.wdeg[v >> 5] = 0;
            }
        }
    }
    __syncthreads();  // every thread has read the level state
    if (tid == 0) {
        const uint64_t tn = len, tm = carry;
        a.log[L].examined = st->examined;
        const uint64_t mu_after = st->mu >= tm ? st->mu - tm : 0;
        st->level = L + 1;
        st->dir = DIR_TD;
        st->nf = tn;
        st->mf = tm;
        st->mu = mu_after;
        st->nvisited += tn;
        st->examined = 0;
        st->want_queue = 1;
        st->list_mode = 0;
        st->ulen = 0;
        st->sparse = sparse_next(a, tm);
        st->slen = 0;
        st->stm = 0;
        a.qoff[tn] = tm;
        if (L + 1 < a.max_levels) {
            a.log[L + 1].dir = DIR_TD;
            a.log[L + 1].nf = tn;
            a.log[L + 1].mf = tm;
            a.log[L + 1].examined = 0;
        }
        bool cont = tn > 0 && st->err == 0;
        if (cont && L + 2 >= a.max_levels) {
            st->err |= G5_DEVERR_LEVELS;
            cont = false;
        }
        if (a.use_cond) cudaGraphSetConditional(a.cond, cont ? 1u : 0u);
    }
}

// (at most 48 registers: the sparse finish must not cost the full pass its
// fifth block per SM)
template <int CW>
__global__ void __launch_bounds__(kBlock, 5) k_write(BfsArgs a)
{
    constexpr int kWordsPerWarp = CW / kWarps;
    constexpr int kWordIters = kWordsPerWarp / 32;  // words per lane
    if (a.st->sdone) {  // the sparse path took the level
        if (blockIdx.x == 0) sparse_finish(a);
        return;
    }
    const uint32_t c = blockIdx.x;
    const int lane = g5_lane(), wid = threadIdx.x >> 5;
    const uint64_t wbeg = (uint64_t)c * CW + (uint64_t)wid * kWordsPerWarp;
    const int32_t L = a.st->level;  // index of the new frontier
    const bool want_q = a.st->want_queue != 0;
    const bool want_u = a.st->list_mode != 0;  // next level is bottom-up
    uint64_t pos = a.chunk_n[c], mpos = a.chunk_m[c], upos = a.chunk_u[c];
    // every word of the warp's range up front (one load per lane and word,
    // all in flight at once): xs = next, vs = visited (all ones past the
    // end, so those words hold no unvisited vertex)
    uint32_t xs[kWordIters], vs[kWordIters];
#pragma unroll
    for (int i = 0; i < kWordIters; ++i) {
        const uint64_t wl = wbeg + i * 32 + lane;
        xs[i] = wl < a.nwords ? a.next[wl] : 0u;
        vs[i] = wl < a.nwords ? a.visited[wl] : ~0u;
    }
    // per-warp totals, then the warp's offsets inside the chunk
    uint64_t cn = 0, cm = 0, cu = 0;
    if (want_q || a.level) warp_chunk_counts<CW>(a, wbeg, xs, cn, cm);
    if (want_u) {
#pragma unroll
        for (int i = 0; i < kWordIters; ++i) cu += __popc(~(vs[i] | xs[i]));
        cu = warp_sum_u64(cu);
    }
    __shared__ uint64_t s_n[kWarps], s_m[kWarps], s_u[kWarps];
    if (lane == 0) {
        s_n[wid] = cn;
        s_m[wid] = cm;
        s_u[wid] = cu;
    }
    __syncthreads();
    for (int i = 0; i < wid; ++i) {
        pos += s_n[i];
        mpos += s_m[i];
        upos += s_u[i];
    }
#pragma unroll
    for (int i = 0; i < kWordIters; ++i) {
        const uint64_t wl = wbeg + i * 32 + lane;
        const uint32_t x = xs[i];
        const uint32_t vis = vs[i] | x;
        const uint32_t unv = ~vis;
        if (wl < a.nwords) {
            if (x) {
                a.visited[wl] = vis;
                a.next[wl] = 0;
                a.wdeg[wl] = 0;  // a bottom-up list sweep adds into it
            }
            a.front[wl] = x;
        }
        if (want_u) {
            // unvisited vertices of these 32 words, in order: one word at a
            // time across the warp so the list writes are coalesced
            unsigned uact = __ballot_sync(0xFFFFFFFFu, unv != 0u);
            while (uact) {
                const int j = __ffs(uact) - 1;
                uact &= uact - 1;
                const uint32_t uj = __shfl_sync(0xFFFFFFFFu, unv, j);
                if ((uj >> lane) & 1u)
                    a.ulist[upos + __popc(uj & g5_lanemask_lt())] = (uint32_t)((wbeg + i * 32 + j) * 32 + lane);
                upos += __popc(uj);
            }
        }
        if (!want_q && !a.level) continue;
        unsigned act = __ballot_sync(0xFFFFFFFFu, x != 0u);
        while (act) {
            const int j = __ffs(act) - 1;
            act &= act - 1;
            const uint32_t wj = __shfl_sync(0xFFFFFFFFu, x, j);
            const bool mine = (wj >> lane) & 1u;
            const uint64_t v = (wbeg + i * 32 + j) * 32 + lane;
            uint64_t d = mine ? (uint64_t)__ldg(a.deg + v) : 0;
            // inclusive scan of the degrees of this word's vertices
            uint64_t incl = d;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint64_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
                if (lane >= o) incl += y;
            }
            if (mine) {
                const uint64_t p = pos + __popc(wj & g5_lanemask_lt());
                const uint64_t mp = mpos + incl - d;
                if (a.level) a.level[v] = L;
                if (want_q) {
                    a.queue[p] = (uint32_t)v;
                    a.qoff[p] = mp;
                    a.qbase[p] = a.row_off[v] - (int64_t)mp;
                    uint64_t t = (mp + a.tile - 1) >> a.tile_shift;
                    const uint64_t tend = (mp + d + a.tile - 1) >> a.tile_shift;
                    for (; t < tend && t < a.max_tiles; ++t) a.tile_start[t] = (uint32_t)p;
                }
            }
            pos += __popc(wj);
            mpos += __shfl_sync(0xFFFFFFFFu, incl, 31);
        }
    }
}

// Copies the level's encoded stream (scal[CS_WORDS] words) to the capture
// buffer and records (level, values, words, offset); a no-op unless a caller
// set a buffer.  All blocks read the same starting offset; the last block to
// finish advances it.
__global__ void __launch_bounds__(kBlock) k_codec_capture(CodecCapture *cc, const uint32_t *stream,
                                                          const uint64_t *scal, const BfsState *st)
{
    if (!cc->buf) return;
    const uint64_t words = scal[g5::CS_WORDS], off = cc->off;
    const uint32_t count = cc->count;
    const bool fits = count < cc->max_rec && off + words <= cc->cap;
    if (fits)
        for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < words;
             i += (uint64_t)gridDim.x * blockDim.x)
            cc->buf[off + i] = stream[i];
    __syncthreads();
    __shared__ bool s_last;
    if (threadIdx.x == 0) {
        __threadfence();
        s_last = atomicAdd(&cc->blocks_done, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (s_last && threadIdx.x == 0) {
        if (fits) {
            uint64_t *r = cc->rec + 4 * (uint64_t)count;
            r[0] = (uint64_t)st->level;
            r[1] = st->nf;
            r[2] = words;
            r[3] = off;
            cc->off = off + ((words + 3) & ~(uint64_t)3);
            cc->count = count + 1;
        } else {
            cc->overflow = 1;
        }
        cc->blocks_done = 0;
    }
}

// ---- TEPS edge count and validation -----------------------------------------------

__global__ void k_teps(const int64_t *__restrict__ pred, const uint32_t *__restrict__ end_deg, int64_t n,
                       unsigned long long *out)
{
    uint64_t s = 0;
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n;
         v += (int64_t)gridDim.x * blockDim.x)
        if (pred[v] != -1) s += end_deg[v];
    s = warp_sum_u64(s);
    if (g5_lane() == 0 && s) atomicAdd(out, (unsigned long long)s);
}

enum : unsigned {
    VAL_RANGE = 1u, VAL_ROOT = 2u, VAL_SELF = 4u, VAL_CYCLE = 8u, VAL_TREE_EDGE = 16u,
    VAL_LEVEL = 32u, VAL_COVER = 64u, VAL_MINPAR = 128u
};

__global__ void k_val_init(const int64_t *__restrict__ pred, int64_t n, int64_t root,
                           int64_t *__restrict__ anc, int32_t *__restrict__ dist, unsigned *flags)
{
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n;
         v += (int64_t)gridDim.x * blockDim.x) {
        const int64_t p = pred[v];
        if (p < -1 || p >= n) {
            atomicOr(flags, VAL_RANGE);
            anc[v] = -1;
            dist[v] = -1;
            continue;
        }
        if (v == root) {
            if (p != root) atomicOr(flags, VAL_ROOT);
            anc[v] = root;
            dist[v] = 0;
        } else if (p == -1) {
            anc[v] = -1;
            dist[v] = -1;
        } else {
            if (p == v) atomicOr(flags, VAL_SELF);
            anc[v] = p;
            dist[v] = 1;
        }
    }
}

// One pointer-jumping round: dist += dist[anc], anc = anc[anc].
__global__ void k_val_jump(const int64_t *__restrict__ anc_in, const int32_t *__restrict__ dist_in,
                           int64_t *__restrict__ anc_out, int32_t *__restrict__ dist_out, int64_t n,
                           int64_t root, unsigned *changed)
{
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n;
         v += (int64_t)gridDim.x * blockDim.x) {
        const int64_t p = anc_in[v];
        int32_t d = dist_in[v];
        int64_t np = p;
        if (p >= 0 && p != root) {
            const int64_t pp = anc_in[p];
            const int32_t pd = dist_in[p];
            if (pp < 0 || pd < 0) {
                np = -2;  // chain leaves the tree: pred points at an unvisited vertex
                d = -1;
            } else {
                np = pp;
                d = d + pd;
                if (d > (int32_t)(1 << 30)) d = (int32_t)(1 << 30);
                *changed = 1u;
            }
        }
        anc_out[v] = np;
        dist_out[v] = d;
    }
}

// lev[v] = BFS level of v if its parent chain reaches the root, else -1:
// one 4-byte word per vertex, so the edge check below reads one random word
// per adjacency entry instead of the parent, ancestor and depth arrays.
__global__ void k_val_level(const int64_t *__restrict__ pred, const int64_t *__restrict__ anc,
                            const int32_t *__restrict__ dist, int64_t n, int64_t root, int32_t *__restrict__ lev)
{
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n;
         v += (int64_t)gridDim.x * blockDim.x)
        lev[v] = (pred[v] == -1 || anc[v] != root || dist[v] < 0) ? -1 : dist[v];
}

__global__ void k_val_edges(const int64_t *__restrict__ row_off, const uint32_t *__restrict__ col,
                            const int64_t *__restrict__ pred, const int32_t *__restrict__ lev, int64_t n,
                            int64_t root, unsigned *flags)
{
    const int lane = g5_lane();
    const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t v = gw; v < n; v += nw) {
        const int64_t p = pred[v];
        if (p == -1) continue;
        const int32_t d = lev[v];
        if (d < 0) {
            // visited but its parent chain does not reach the root
            if (lane == 0) atomicOr(flags, VAL_CYCLE);
            continue;
        }
        const int64_t s = row_off[v], e = row_off[v + 1];
        bool tree = (v == root);
        int64_t first_prev = -1;  // smallest neighbour one level up
        unsigned bad = 0;
        for (int64_t j0 = s; j0 < e; j0 += 32) {
            const int64_t j = j0 + lane;
            bool is_par = false, is_prev = false;
            uint32_t u = 0;
            if (j < e) {
                u = __ldg(col + j);
                const int32_t du = __ldg(lev + u);
                if (du < 0) bad |= VAL_COVER;
                else if (du > d + 1 || du < d - 1) bad |= VAL_LEVEL;
                is_par = ((int64_t)u == p);
                is_prev = (du == d - 1);
            }
            if (__any_sync(0xFFFFFFFFu, is_par)) tree = true;
            const unsigned pm = __ballot_sync(0xFFFFFFFFu, is_prev);
            if (pm && first_prev < 0) first_prev = __shfl_sync(0xFFFFFFFFu, (int64_t)u, __ffs(pm) - 1);
        }
        if (v != root) {
            if (!tree) bad |= VAL_TREE_EDGE;
            if (first_prev != p) bad |= VAL_MINPAR;
            if (d != 0 && first_prev < 0) bad |= VAL_LEVEL;
        }
        if (bad) atomicOr(flags, bad);
    }
}

// Kernel kinds timed in profile mode.
// profile-mode buckets; KP_HOST is the host loop's gap after a level (its
// state read-back and synchronise) up to the next level's first launch
enum { KP_PRO = 0, KP_EXPAND, KP_FIXUP, KP_COUNT, KP_SCAN, KP_WRITE, KP_CODEC, KP_HOST, KP_N };

struct Prof {
    bool on = false;
    std::vector<cudaEvent_t> ev;
    std::vector<int> kind;
    size_t used = 0;
    void mark(int k, cudaStream_t s)
    {
        if (!on) return;
        if (used + 1 > ev.size()) {
            cudaEvent_t e;
            cudaEventCreate(&e);
            ev.push_back(e);
            kind.push_back(0);
        }
        kind[used] = k;
        cudaEventRecord(ev[used++], s);
    }
};

}  // namespace

// ---- workspace --------------------------------------------------------------------

struct g5_bfs {
    g5_graph *g = nullptr;
    g5_bfs_config cfg;
    cudaStream_t stream = nullptr;
    BfsArgs args;
    uint32_t *deg = nullptr;
    uint32_t *bitmaps = nullptr;  // visited | front | next
    uint32_t *isolated = nullptr; // one bit per vertex of degree 0
    uint32_t *heavy = nullptr;    // one bit per vertex of degree > kHeavy
    uint32_t *ro32 = nullptr;     // uint32 copy of the row offsets (nnz < 2^32)
    uint32_t *first = nullptr;    // first neighbour of each vertex (dense, coalesced)
    uint32_t *multi = nullptr;    // reached more than once in a top-down level
    uint32_t *wdeg = nullptr;     // per-word degree sums written by bottom-up
    uint32_t *ulist = nullptr;    // sorted unvisited vertices (n entries)
    unsigned *done = nullptr;     // k_count's finished-block counter
    int64_t *pred = nullptr;
    int32_t *level = nullptr;
    uint32_t *queue = nullptr;
    uint32_t *dqueue = nullptr;
    uint64_t *qoff = nullptr;
    int64_t *qbase = nullptr;
    uint32_t *tile_start = nullptr;
    uint64_t *chunks = nullptr;
    uint32_t *slist = nullptr;    // sparse top-down list (kSparseCap entries)
    BfsState *st = nullptr;
    LevelRec *log = nullptr;
    int64_t *root_dev = nullptr;
    uint32_t *codec_stream = nullptr;
    CodecCapture *ccap = nullptr;  // device descriptor (codec searches)
    bool capture_on = false;       // the level loop launches the stream copy (k_codec_capture)
    g5::CodecWork cw;
    // host mirrors
    int64_t *h_root = nullptr;  // pinned
    BfsState *h_st = nullptr;   // pinned
    LevelRec *h_log = nullptr;  // pinned
    cudaGraphExec_t exec = nullptr;
    cudaGraph_t graph = nullptr;
    // g5_bfs_run_many: a second parent buffer with its own graph, a copy
    // stream, and events (created on first use)
    int64_t *pred2 = nullptr;
    cudaGraphExec_t exec2 = nullptr;
    cudaGraph_t graph2 = nullptr;
    cudaStream_t cstream = nullptr;
    cudaEvent_t searched[2] = {nullptr, nullptr}, copied[2] = {nullptr, nullptr};
    std::vector<cudaEvent_t> tev;   // start/end of each search of a run_many call
    int64_t *h_roots = nullptr;     // pinned roots of a run_many call
    uint32_t *h_errs = nullptr;     // pinned error flags, one per search
    int roots_cap = 0;
    int64_t *cur_pred = nullptr;    // parent array of the last search
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    Prof prof;
    int64_t with_edges = 0;  // vertices of degree > 0
    bool ran = false;
    int64_t last_root = -1;
};

namespace {

void enqueue_prologue(g5_bfs *b, const BfsArgs &a, cudaStream_t s)
{
    // vertices without edges can never be reached: they start out visited, so
    // bottom-up sweeps skip them (the root is set again by k_init)
    cudaMemcpyAsync(b->bitmaps, b->isolated, sizeof(uint32_t) * a.nwords, cudaMemcpyDeviceToDevice, s);
    cudaMemsetAsync(b->bitmaps + a.nwords, 0, sizeof(uint32_t) * 2 * a.nwords, s);
    // per-word degree sums start at zero (a search stopped by an error can
    // leave some behind)
    cudaMemsetAsync(b->wdeg, 0, sizeof(uint32_t) * a.nwords, s);
    cudaMemsetAsync(a.pred, 0xFF, sizeof(int64_t) * (size_t)a.n, s);
    if (b->level) cudaMemsetAsync(b->level, 0xFF, sizeof(int32_t) * (size_t)a.n, s);
    k_init<<<1, kBlock, 0, s>>>(a);
}

void enqueue_level(g5_bfs *b, const BfsArgs &a, cudaStream_t s, Prof *pf = nullptr)
{
    Prof dummy;
    Prof &p = pf ? *pf : dummy;
    // (programmatic dependent launches here measured no faster: 605 against
    // 603 GTEPS at scale 26, 508 against 516 at scale 24)
    p.mark(KP_EXPAND, s);
    k_td<<<g5::grid_for(8), kBlock, 0, s>>>(a);
    if (a.ro32) k_bu<uint32_t><<<g5::grid_for(8), kBlock, 0, s>>>(a);
    else k_bu<int64_t><<<g5::grid_for(8), kBlock, 0, s>>>(a);
    p.mark(KP_FIXUP, s);
    if (a.parent_mode != 0) k_fixup<<<g5::grid_for(8), kBlock, 0, s>>>(a);
    p.mark(KP_COUNT, s);
    switch (a.chunk_words) {
    case 256: k_count<256><<<a.nchunks, kBlock, 0, s>>>(a); break;
    case 512: k_count<512><<<a.nchunks, kBlock, 0, s>>>(a); break;
    case 1024: k_count<1024><<<a.nchunks, kBlock, 0, s>>>(a); break;
    default: k_count<2048><<<a.nchunks, kBlock, 0, s>>>(a); break;
    }
    p.mark(KP_WRITE, s);
    switch (a.chunk_words) {
    case 256: k_write<256><<<a.nchunks, kBlock, 0, s>>>(a); break;
    case 512: k_write<512><<<a.nchunks, kBlock, 0, s>>>(a); break;
    case 1024: k_write<1024><<<a.nchunks, kBlock, 0, s>>>(a); break;
    default: k_write<2048><<<a.nchunks, kBlock, 0, s>>>(a); break;
    }
    p.mark(KP_CODEC, s);
    if (a.codec) {
        g5::codec_encode_launch(b->cw, b->queue, &b->st->nf, b->codec_stream, a.codec,
                                b->cfg.codec_threshold, s);
        // the stream copy is launched only while a caller has a buffer set
        if (b->capture_on) k_codec_capture<<<g5::grid_for(1), kBlock, 0, s>>>(a.ccap, b->codec_stream, b->cw.scal, b->st);
        g5::decode_launch_acc(b->cw, b->codec_stream, b->cw.scal + g5::CS_WORDS, b->dqueue, (size_t)a.n,
                              a.codec, b->cfg.codec_threshold, &b->st->nf, b->queue, b->st->codec_acc, s);
    }
    p.mark(KP_HOST, s);
}

// The search as one CUDA graph writing its parents to `pred`: the prologue,
// then the level loop under a conditional while node.
g5_status build_graph(g5_bfs *b, int64_t *pred, cudaGraphExec_t *exec_out, cudaGraph_t *graph_out)
{
    cudaStream_t s = b->stream;
    BfsArgs a = b->args;
    a.pred = pred;
    // prologue captured as a child graph
    cudaGraph_t pro = nullptr;
    G5_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    enqueue_prologue(b, a, s);
    G5_CUDA(cudaStreamEndCapture(s, &pro));
    cudaGraph_t g = nullptr;
    G5_CUDA(cudaGraphCreate(&g, 0));
    cudaGraphNode_t pro_node;
    G5_CUDA(cudaGraphAddChildGraphNode(&pro_node, g, nullptr, 0, pro));
    cudaGraphDestroy(pro);
    cudaGraphConditionalHandle h;
    G5_CUDA(cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t cnode;
    G5_CUDA(cudaGraphAddNode(&cnode, g, &pro_node, nullptr, 1, &cp));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    a.cond = h;
    a.use_cond = 1;
    G5_CUDA(cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    enqueue_level(b, a, s);
    cudaGraph_t body_out = nullptr;
    G5_CUDA(cudaStreamEndCapture(s, &body_out));
    G5_CUDA(cudaGraphInstantiate(exec_out, g, 0));
    *graph_out = g;
    return G5_OK;
}

g5_status alloc_ws(g5_bfs *b)
{
    g5_graph *g = b->g;
    const int64_t n = g->n;
    BfsArgs &a = b->args;
    memset(&a, 0, sizeof a);
    a.n = n;
    a.nnz = g->nnz;
    a.nwords = (uint64_t)((n + 31) / 32);
    a.chunk_words = 2048;
    for (int cw = 256; cw < 2048; cw *= 2)
        if ((a.nwords + cw - 1) / cw <= (uint64_t)kMaxChunks) {
            a.chunk_words = cw;
            break;
        }
    a.nchunks = (uint32_t)((a.nwords + a.chunk_words - 1) / a.chunk_words);
    a.list_first = n >= kListFirst ? 1 : 0;
    a.tile = b->cfg.tile_edges;
    a.tile_shift = __builtin_ctz(b->cfg.tile_edges);
    a.bu_serial = b->cfg.bu_serial;
    a.max_tiles = (uint64_t)g->nnz / a.tile + 2;
    a.max_levels = b->cfg.max_levels;
    G5_CUDA(cudaMalloc(&b->deg, sizeof(uint32_t) * (size_t)n));
    G5_CUDA(cudaMalloc(&b->bitmaps, sizeof(uint32_t) * 3 * a.nwords));
    G5_CUDA(cudaMalloc(&b->isolated, sizeof(uint32_t) * a.nwords));
    G5_CUDA(cudaMalloc(&b->heavy, sizeof(uint32_t) * a.nwords));
    // 32-bit offsets while every scan position (row end + one 32-entry step) fits
    if (g->nnz < ((int64_t)1 << 32) - 64) G5_CUDA(cudaMalloc(&b->ro32, sizeof(uint32_t) * (size_t)(n + 1)));
    G5_CUDA(cudaMalloc(&b->first, sizeof(uint32_t) * (size_t)n));
    G5_CUDA(cudaMalloc(&b->multi, sizeof(uint32_t) * a.nwords));
    G5_CUDA(cudaMalloc(&b->wdeg, sizeof(uint32_t) * a.nwords));
    G5_CUDA(cudaMemset(b->wdeg, 0, sizeof(uint32_t) * a.nwords));
    G5_CUDA(cudaMalloc(&b->ulist, sizeof(uint32_t) * (size_t)n + 16));
    G5_CUDA(cudaMalloc(&b->done, sizeof(unsigned)));
    G5_CUDA(cudaMemset(b->done, 0, sizeof(unsigned)));
    G5_CUDA(cudaMemset(b->multi, 0, sizeof(uint32_t) * a.nwords));
    G5_CUDA(cudaMalloc(&b->pred, sizeof(int64_t) * (size_t)n));
    if (b->cfg.want_levels) G5_CUDA(cudaMalloc(&b->level, sizeof(int32_t) * (size_t)n));
    G5_CUDA(cudaMalloc(&b->queue, sizeof(uint32_t) * (size_t)n + 16));
    G5_CUDA(cudaMalloc(&b->qoff, sizeof(uint64_t) * (size_t)(n + 1)));
    G5_CUDA(cudaMalloc(&b->qbase, sizeof(int64_t) * (size_t)n));
    G5_CUDA(cudaMalloc(&b->tile_start, sizeof(uint32_t) * a.max_tiles));
    G5_CUDA(cudaMalloc(&b->chunks, sizeof(uint64_t) * 3 * a.nchunks));
    G5_CUDA(cudaMalloc(&b->slist, sizeof(uint32_t) * kSparseCap));
    G5_CUDA(cudaMalloc(&b->st, sizeof(BfsState)));
    G5_CUDA(cudaMalloc(&b->log, sizeof(LevelRec) * (size_t)b->cfg.max_levels));
    G5_CUDA(cudaMalloc(&b->root_dev, sizeof(int64_t)));
    G5_CUDA(cudaMallocHost(&b->h_root, sizeof(int64_t)));
    G5_CUDA(cudaMallocHost(&b->h_st, sizeof(BfsState)));
    G5_CUDA(cudaMallocHost(&b->h_log, sizeof(LevelRec) * (size_t)b->cfg.max_levels));
    if (b->cfg.codec) {
        G5_CUDA(cudaMalloc(&b->dqueue, sizeof(uint32_t) * (size_t)n + 16));
        G5_CUDA(cudaMalloc(&b->codec_stream, sizeof(uint32_t) * g5::codec_bound((size_t)n)));
        G5_TRY(g5::codec_work_alloc(b->cw, (size_t)n));
        G5_CUDA(cudaMalloc(&b->ccap, sizeof(CodecCapture)));
        G5_CUDA(cudaMemset(b->ccap, 0, sizeof(CodecCapture)));
    }
    a.row_off = g->row_off;
    a.col = g->col;
    a.deg = b->deg;
    a.visited = b->bitmaps;
    a.front = b->bitmaps + a.nwords;
    a.next = b->bitmaps + 2 * a.nwords;
    a.pred = b->pred;
    a.level = b->level;
    a.queue = b->queue;
    a.qsrc = b->cfg.codec ? b->dqueue : b->queue;
    a.qoff = b->qoff;
    a.qbase = b->qbase;
    a.tile_start = b->tile_start;
    a.heavy = b->heavy;
    a.ro32 = b->ro32;
    a.first = b->first;
    a.multi = b->multi;
    a.wdeg = b->wdeg;
    a.ulist = b->ulist;
    a.done = b->done;
    a.parent_mode = b->cfg.parent_mode;
    a.chunk_n = b->chunks;
    a.chunk_m = b->chunks + a.nchunks;
    a.chunk_u = b->chunks + 2 * a.nchunks;
    a.slist = b->slist;
    a.st = b->st;
    a.log = b->log;
    a.root_dev = b->root_dev;
    a.alpha = b->cfg.alpha;
    a.beta = b->cfg.beta;
    a.codec = b->cfg.codec;
    a.codec_scal = b->cfg.codec ? b->cw.scal : nullptr;
    a.ccap = b->ccap;
    a.use_cond = 0;
    return G5_OK;
}

__global__ void k_degrees(const int64_t *__restrict__ ro, const uint32_t *__restrict__ col, int64_t n,
                          uint32_t *__restrict__ d, uint32_t *__restrict__ iso, uint32_t *__restrict__ heavy,
                          uint32_t *__restrict__ ro32, uint32_t *__restrict__ first)
{
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < ((n + 31) & ~(int64_t)31);
         v += (int64_t)gridDim.x * blockDim.x) {
        if (ro32 && v < n) {
            ro32[v] = (uint32_t)ro[v];  // ro32[n] is written by thread 0
            if (v == 0) ro32[n] = (uint32_t)ro[n];
        }
        const uint32_t dv = v < n ? (uint32_t)(ro[v + 1] - ro[v]) : 0u;
        if (v < n) {
            d[v] = dv;
            first[v] = dv ? col[ro[v]] : 0u;
        }
        const unsigned m = __ballot_sync(0xFFFFFFFFu, dv == 0 && v < n);
        const unsigned h = __ballot_sync(0xFFFFFFFFu, dv > kHeavy);
        if ((threadIdx.x & 31) == 0) {
            iso[v >> 5] = m;
            heavy[v >> 5] = h;
        }
    }
}

void free_ws(g5_bfs *b)
{
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    if (b->exec2) cudaGraphExecDestroy(b->exec2);
    if (b->graph2) cudaGraphDestroy(b->graph2);
    cudaFree(b->pred2);
    if (b->cstream) cudaStreamDestroy(b->cstream);
    for (int i = 0; i < 2; ++i) {
        if (b->searched[i]) cudaEventDestroy(b->searched[i]);
        if (b->copied[i]) cudaEventDestroy(b->copied[i]);
    }
    for (cudaEvent_t e : b->tev) cudaEventDestroy(e);
    cudaFreeHost(b->h_roots);
    cudaFreeHost(b->h_errs);
    cudaFree(b->deg);
    cudaFree(b->bitmaps);
    cudaFree(b->isolated);
    cudaFree(b->heavy);
    cudaFree(b->ro32);
    cudaFree(b->first);
    cudaFree(b->multi);
    cudaFree(b->wdeg);
    cudaFree(b->ulist);
    cudaFree(b->done);
    cudaFree(b->pred);
    cudaFree(b->level);
    cudaFree(b->queue);
    cudaFree(b->dqueue);
    cudaFree(b->qoff);
    cudaFree(b->qbase);
    cudaFree(b->tile_start);
    cudaFree(b->chunks);
    cudaFree(b->slist);
    cudaFree(b->st);
    cudaFree(b->log);
    cudaFree(b->root_dev);
    cudaFree(b->codec_stream);
    cudaFree(b->ccap);
    cudaFreeHost(b->h_root);
    cudaFreeHost(b->h_st);
    cudaFreeHost(b->h_log);
    if (b->cfg.codec) g5::codec_work_free(b->cw);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    for (cudaEvent_t e : b->prof.ev) cudaEventDestroy(e);
    if (b->stream) cudaStreamDestroy(b->stream);
}

// Algorithmic HBM bytes of one search from the level log.  With C the
// candidates of a bottom-up level (vertices with edges not yet visited) and
// off the bytes of a row offset, per level: top-down 20|F| + 4 E_td + N/8
// (queue entry, edge offset and row base per frontier vertex, adjacency,
// visited bitmap); a bottom-up sweep of the unvisited list (2 off + 8) C +
// 4 E_bu + N/8 (the list, row bounds and first neighbour of each listed
// vertex, adjacency until the first hit, frontier); a sweep of the bitmap
// words (the first bottom-up level on small graphs) 3N/8 + (off + 4) C +
// 4 E_bu (visited, frontier and next bitmaps, each candidate's row start and
// dense first neighbour, adjacency); plus 4 + 9 bytes per vertex the level
// adds (queue, parent, level) after top-down and 9 after bottom-up.
int64_t alg_bytes(const LevelRec *log, int nlev, int64_t n, int64_t with_edges, int off, bool list_first)
{
    double B = 0, seen = 0;
    for (int L = 0; L < nlev; ++L) {
        const double nf = (double)log[L].nf;
        const double nf1 = (L + 1 < nlev) ? (double)log[L + 1].nf : 0.0;
        seen += nf;
        const double cand = std::max(0.0, (double)with_edges - seen);
        const double E = 4.0 * (double)log[L].examined;
        if (log[L].dir == DIR_TD)
            B += 20.0 * nf + E + (double)n / 8.0 + 13.0 * nf1;
        else if (!list_first && (L == 0 || log[L - 1].dir != DIR_BU))
            B += 3.0 * (double)n / 8.0 + (off + 4.0) * cand + E + 9.0 * nf1;
        else
            B += (2.0 * off + 8.0) * cand + E + (double)n / 8.0 + 9.0 * nf1;
    }
    return (int64_t)B;
}

}  // namespace

extern "C" {

void g5_bfs_config_default(g5_bfs_config *cfg)
{
    if (!cfg) return;
    cfg->alpha = 14.0;
    cfg->beta = 24.0;
    cfg->codec = G5_CODEC_NONE;
    cfg->codec_threshold = 64;
    cfg->use_graph = 1;
    cfg->max_levels = 4096;
    cfg->want_levels = 0;
    cfg->profile = 0;
    cfg->parent_mode = 0;
    cfg->tile_edges = kTileDefault;
    cfg->bu_serial = kBuSerialDefault;
}

g5_status g5_bfs_create(g5_graph *g, const g5_bfs_config *cfg, g5_bfs **out)
{
    if (!g || !out) return G5_ERR_INVALID_ARG;
    *out = nullptr;
    g5_bfs *b = new g5_bfs();
    b->g = g;
    if (cfg) b->cfg = *cfg;
    else g5_bfs_config_default(&b->cfg);
    if (b->cfg.max_levels < 2) b->cfg.max_levels = 2;
    if (b->cfg.codec < 0 || b->cfg.codec > 2 || b->cfg.alpha <= 0 || b->cfg.beta <= 0 ||
        b->cfg.parent_mode < 0 || b->cfg.parent_mode > 2 || b->cfg.tile_edges < 32 ||
        b->cfg.tile_edges > 4096 || (b->cfg.tile_edges & (b->cfg.tile_edges - 1)) != 0 || b->cfg.bu_serial < 1 || b->cfg.bu_serial > 64) {
        delete b;
        return G5_ERR_INVALID_ARG;
    }
    g5_status st = G5_OK;
    auto fail = [&](g5_status s) {
        free_ws(b);
        delete b;
        return s;
    };
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) return fail(G5_ERR_CUDA);
    cudaEventCreate(&b->ev0);
    cudaEventCreate(&b->ev1);
    if ((st = alloc_ws(b)) != G5_OK) return fail(st);
    k_degrees<<<g5::grid_for(8), kBlock, 0, b->stream>>>(g->row_off, g->col, g->n, b->deg, b->isolated,
                                                          b->heavy, b->ro32, b->first);
    if (cudaStreamSynchronize(b->stream) != cudaSuccess) return fail(G5_ERR_CUDA);
    {
        // vertices with edges (for the algorithmic byte count): n minus the
        // isolated bits
        std::vector<uint32_t> iso((size_t)b->args.nwords);
        if (cudaMemcpy(iso.data(), b->isolated, sizeof(uint32_t) * iso.size(), cudaMemcpyDeviceToHost) != cudaSuccess)
            return fail(G5_ERR_CUDA);
        int64_t isolated = 0;
        for (uint32_t w : iso) isolated += __builtin_popcount(w);
        b->with_edges = g->n - isolated;
    }
    if (b->cfg.use_graph && (st = build_graph(b, b->pred, &b->exec, &b->graph)) != G5_OK) return fail(st);
    b->cur_pred = b->pred;
    *out = b;
    return G5_OK;
}

g5_status g5_bfs_destroy(g5_bfs *b)
{
    if (!b) return G5_ERR_INVALID_ARG;
    cudaStreamSynchronize(b->stream);
    free_ws(b);
    delete b;
    return G5_OK;
}

g5_status g5_bfs_run(g5_bfs *b, int64_t root, int64_t *pred_out, int32_t *level_out, g5_bfs_stats *stats)
{
    if (!b || root < 0 || root >= b->g->n) return G5_ERR_INVALID_ARG;
    if (level_out && !b->level) return G5_ERR_INVALID_ARG;
    cudaStream_t s = b->stream;
    *b->h_root = root;
    G5_CUDA(cudaMemcpyAsync(b->root_dev, b->h_root, sizeof(int64_t), cudaMemcpyHostToDevice, s));
    G5_CUDA(cudaEventRecord(b->ev0, s));
    b->prof.on = b->cfg.profile && !b->exec;
    b->prof.used = 0;
    if (b->exec) {
        G5_CUDA(cudaGraphLaunch(b->exec, s));
    } else {
        b->prof.mark(KP_PRO, s);
        enqueue_prologue(b, b->args, s);
        for (int L = 0; L < b->cfg.max_levels; ++L) {
            enqueue_level(b, b->args, s, &b->prof);
            G5_CUDA(cudaMemcpyAsync(b->h_st, b->st, sizeof(BfsState), cudaMemcpyDeviceToHost, s));
            G5_CUDA(cudaStreamSynchronize(s));
            if (b->h_st->nf == 0 || b->h_st->err) break;
        }
    }
    G5_CUDA(cudaEventRecord(b->ev1, s));
    G5_CUDA(cudaMemcpyAsync(b->h_st, b->st, sizeof(BfsState), cudaMemcpyDeviceToHost, s));
    if (pred_out)
        G5_CUDA(cudaMemcpyAsync(pred_out, b->pred, sizeof(int64_t) * (size_t)b->g->n, cudaMemcpyDefault, s));
    if (level_out)
        G5_CUDA(cudaMemcpyAsync(level_out, b->level, sizeof(int32_t) * (size_t)b->g->n, cudaMemcpyDefault, s));
    uint64_t cscal[g5::CS_COUNT] = {0};
    if (b->cfg.codec)
        G5_CUDA(cudaMemcpyAsync(cscal, b->cw.scal, sizeof cscal, cudaMemcpyDeviceToHost, s));
    G5_CUDA(cudaStreamSynchronize(s));
    b->ran = true;
    b->last_root = root;
    b->cur_pred = b->pred;
    const BfsState &hs = *b->h_st;
    g5_status rc = G5_OK;
    if (hs.err & G5_DEVERR_LEVELS) rc = G5_ERR_TIMEOUT;
    else if (hs.err) rc = G5_ERR_CAPACITY;
    else if (b->cfg.codec && (cscal[g5::CS_ERR] & G5_DEVERR_WAIT)) rc = G5_ERR_TIMEOUT;
    else if (b->cfg.codec && (cscal[g5::CS_ERR] & G5_DEVERR_MISMATCH)) rc = G5_ERR_MISMATCH;
    else if (b->cfg.codec && cscal[g5::CS_ERR]) rc = G5_ERR_CORRUPT_STREAM;
    if (stats) {
        const int nlev = std::min(hs.level + 1, b->cfg.max_levels);
        G5_CUDA(cudaMemcpy(b->h_log, b->log, sizeof(LevelRec) * (size_t)nlev, cudaMemcpyDeviceToHost));
        memset(stats, 0, sizeof *stats);
        stats->levels = nlev;
        stats->visited = (int64_t)hs.nvisited;
        for (int L = 0; L < nlev; ++L) {
            const LevelRec &r = b->h_log[L];
            if (r.dir == DIR_TD) stats->edges_td += (int64_t)r.examined;
            else {
                stats->edges_bu += (int64_t)r.examined;
                stats->bottom_up_levels += 1;
            }
            stats->queue_total += (int64_t)r.nf;
        }
        stats->codec_words = (int64_t)hs.codec_acc[0];
        stats->codec_values = (int64_t)hs.codec_acc[1];
        stats->alg_bytes = alg_bytes(b->h_log, nlev, b->g->n, b->with_edges, b->ro32 ? 4 : 8, b->args.list_first != 0);
        float ms = 0;
        cudaEventElapsedTime(&ms, b->ev0, b->ev1);
        stats->device_ms = ms;
        if (b->prof.on && b->prof.used) {
            // each mark closes the previous interval; the last one ends at ev1
            for (size_t i = 0; i < b->prof.used; ++i) {
                float t = 0;
                cudaEventElapsedTime(&t, b->prof.ev[i], i + 1 < b->prof.used ? b->prof.ev[i + 1] : b->ev1);
                const int k = b->prof.kind[i];
                if (k >= 0 && k < 8) stats->kernel_ms[k] += t;
            }
        }
    }
    return rc;
}

g5_status g5_bfs_level_log(g5_bfs *b, int64_t *out, int max_rows, int *rows)
{
    if (!b || !out || !rows || max_rows < 1 || !b->ran) return G5_ERR_INVALID_ARG;
    const int nlev = std::min(std::min(b->h_st->level + 1, b->cfg.max_levels), max_rows);
    G5_CUDA(cudaMemcpy(b->h_log, b->log, sizeof(LevelRec) * (size_t)nlev, cudaMemcpyDeviceToHost));
    for (int L = 0; L < nlev; ++L) {
        out[4 * L + 0] = b->h_log[L].dir;
        out[4 * L + 1] = (int64_t)b->h_log[L].nf;
        out[4 * L + 2] = (int64_t)b->h_log[L].mf;
        out[4 * L + 3] = (int64_t)b->h_log[L].examined;
    }
    *rows = nlev;
    return G5_OK;
}

g5_status g5_bfs_profile_log(g5_bfs *b, int32_t *kinds, double *ms, int max_rows, int *rows)
{
    if (!b || !kinds || !ms || !rows || max_rows < 1) return G5_ERR_INVALID_ARG;
    int k = 0;
    for (size_t i = 0; i < b->prof.used && k < max_rows; ++i, ++k) {
        float t = 0;
        cudaEventElapsedTime(&t, b->prof.ev[i], i + 1 < b->prof.used ? b->prof.ev[i + 1] : b->ev1);
        kinds[k] = b->prof.kind[i];
        ms[k] = t;
    }
    *rows = k;
    return G5_OK;
}

g5_status g5_bfs_launch(g5_bfs *b, int64_t root)
{
    // asynchronous search on the workspace's stream (CUDA-graph workspaces
    // only): completion is polled with g5_bfs_poll
    if (!b || root < 0 || root >= b->g->n || !b->exec) return G5_ERR_INVALID_ARG;
    cudaStream_t s = b->stream;
    *b->h_root = root;
    G5_CUDA(cudaMemcpyAsync(b->root_dev, b->h_root, sizeof(int64_t), cudaMemcpyHostToDevice, s));
    G5_CUDA(cudaEventRecord(b->ev0, s));
    G5_CUDA(cudaGraphLaunch(b->exec, s));
    G5_CUDA(cudaEventRecord(b->ev1, s));
    G5_CUDA(cudaMemcpyAsync(b->h_st, b->st, sizeof(BfsState), cudaMemcpyDeviceToHost, s));
    b->ran = true;
    b->last_root = root;
    b->cur_pred = b->pred;
    return G5_OK;
}

g5_status g5_bfs_poll(g5_bfs *b, int *done, double *device_ms)
{
    if (!b || !done) return G5_ERR_INVALID_ARG;
    const cudaError_t e = cudaStreamQuery(b->stream);
    if (e == cudaErrorNotReady) {
        *done = 0;
        return G5_OK;
    }
    G5_CUDA(e);
    *done = 1;
    if (device_ms) {
        float ms = 0;
        cudaEventElapsedTime(&ms, b->ev0, b->ev1);
        *device_ms = ms;
    }
    const BfsState &hs = *b->h_st;
    if (hs.err & G5_DEVERR_LEVELS) return G5_ERR_TIMEOUT;
    if (hs.err) return G5_ERR_CAPACITY;
    return G5_OK;
}

g5_status g5_bfs_run_many(g5_bfs *b, const int64_t *roots, int k, int64_t *const *pred_out, double *device_ms)
{
    if (!b || k < 0 || (k && !roots)) return G5_ERR_INVALID_ARG;
    for (int i = 0; i < k; ++i)
        if (roots[i] < 0 || roots[i] >= b->g->n) return G5_ERR_INVALID_ARG;
    if (!b->exec) {
        // host-driven workspaces: one search after the other
        for (int i = 0; i < k; ++i) {
            g5_bfs_stats st;
            G5_TRY(g5_bfs_run(b, roots[i], pred_out ? pred_out[i] : nullptr, nullptr, device_ms ? &st : nullptr));
            if (device_ms) device_ms[i] = st.device_ms;
        }
        return G5_OK;
    }
    const int64_t n = b->g->n;
    cudaStream_t s = b->stream;
    // first use: the second parent buffer, its graph, the copy stream, events
    if (!b->exec2) {
        G5_CUDA(cudaMalloc(&b->pred2, sizeof(int64_t) * (size_t)n));
        G5_TRY(build_graph(b, b->pred2, &b->exec2, &b->graph2));
        G5_CUDA(cudaStreamCreateWithFlags(&b->cstream, cudaStreamNonBlocking));
        for (int i = 0; i < 2; ++i) {
            G5_CUDA(cudaEventCreateWithFlags(&b->searched[i], cudaEventDisableTiming));
            G5_CUDA(cudaEventCreateWithFlags(&b->copied[i], cudaEventDisableTiming));
        }
    }
    if (k > b->roots_cap) {
        cudaFreeHost(b->h_roots);
        cudaFreeHost(b->h_errs);
        b->h_roots = nullptr;
        b->h_errs = nullptr;
        b->roots_cap = 0;
        G5_CUDA(cudaMallocHost(&b->h_roots, sizeof(int64_t) * (size_t)k));
        G5_CUDA(cudaMallocHost(&b->h_errs, sizeof(uint32_t) * (size_t)k));
        b->roots_cap = k;
    }
    while (device_ms && b->tev.size() < 2 * (size_t)k) {
        cudaEvent_t e;
        G5_CUDA(cudaEventCreate(&e));
        b->tev.push_back(e);
    }
    int64_t *buf[2] = {b->pred, b->pred2};
    cudaGraphExec_t ex[2] = {b->exec, b->exec2};
    for (int i = 0; i < k; ++i) {
        b->h_roots[i] = roots[i];
        b->h_errs[i] = 0;
    }
    // search i writes buffer i % 2 on the search stream while the copy stream
    // moves search i - 1's parents out; search i + 2 waits for that copy
    for (int i = 0; i < k; ++i) {
        const int slot = i & 1;
        if (i >= 2) G5_CUDA(cudaStreamWaitEvent(s, b->copied[slot], 0));
        G5_CUDA(cudaMemcpyAsync(b->root_dev, b->h_roots + i, sizeof(int64_t), cudaMemcpyHostToDevice, s));
        if (device_ms) G5_CUDA(cudaEventRecord(b->tev[2 * i], s));
        G5_CUDA(cudaGraphLaunch(ex[slot], s));
        if (device_ms) G5_CUDA(cudaEventRecord(b->tev[2 * i + 1], s));
        G5_CUDA(cudaMemcpyAsync(b->h_errs + i, &b->st->err, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
        G5_CUDA(cudaEventRecord(b->searched[slot], s));
        G5_CUDA(cudaStreamWaitEvent(b->cstream, b->searched[slot], 0));
        if (pred_out && pred_out[i])
            G5_CUDA(cudaMemcpyAsync(pred_out[i], buf[slot], sizeof(int64_t) * (size_t)n, cudaMemcpyDefault,
                                    b->cstream));
        G5_CUDA(cudaEventRecord(b->copied[slot], b->cstream));
    }
    G5_CUDA(cudaStreamSynchronize(s));
    G5_CUDA(cudaStreamSynchronize(b->cstream));
    if (k) {
        b->ran = true;
        b->last_root = roots[k - 1];
        b->cur_pred = buf[(k - 1) & 1];
        G5_CUDA(cudaMemcpy(b->h_st, b->st, sizeof(BfsState), cudaMemcpyDeviceToHost));
    }
    g5_status rc = G5_OK;
    for (int i = 0; i < k; ++i) {
        if (device_ms) {
            float ms = 0;
            cudaEventElapsedTime(&ms, b->tev[2 * i], b->tev[2 * i + 1]);
            device_ms[i] = ms;
        }
        if (rc == G5_OK && b->h_errs[i]) rc = (b->h_errs[i] & G5_DEVERR_LEVELS) ? G5_ERR_TIMEOUT : G5_ERR_CAPACITY;
    }
    return rc;
}

g5_status g5_bfs_codec_capture(g5_bfs *b, uint32_t *buf_dev, uint64_t cap_words, uint64_t *rec_dev,
                               int max_levels)
{
    if (!b || !b->ccap) return G5_ERR_INVALID_ARG;
    if (buf_dev && (!rec_dev || max_levels < 1 || !g5::is_device_ptr(buf_dev) || !g5::is_device_ptr(rec_dev)))
        return G5_ERR_INVALID_ARG;
    CodecCapture h = {};
    h.buf = buf_dev;
    h.cap = buf_dev ? cap_words : 0;
    h.rec = buf_dev ? rec_dev : nullptr;
    h.max_rec = buf_dev ? (uint32_t)max_levels : 0;
    G5_CUDA(cudaStreamSynchronize(b->stream));
    G5_CUDA(cudaMemcpy(b->ccap, &h, sizeof h, cudaMemcpyHostToDevice));
    const bool on = buf_dev != nullptr;
    if (on != b->capture_on) {
        // the level loop's graphs launch the copy only while it is on
        b->capture_on = on;
        if (b->exec) {
            cudaGraphExecDestroy(b->exec);
            cudaGraphDestroy(b->graph);
            b->exec = nullptr;
            b->graph = nullptr;
            G5_TRY(build_graph(b, b->pred, &b->exec, &b->graph));
        }
        if (b->exec2) {
            cudaGraphExecDestroy(b->exec2);
            cudaGraphDestroy(b->graph2);
            b->exec2 = nullptr;
            b->graph2 = nullptr;
            G5_TRY(build_graph(b, b->pred2, &b->exec2, &b->graph2));
        }
    }
    return G5_OK;
}

g5_status g5_bfs_codec_captured(g5_bfs *b, int *levels, int *overflow)
{
    if (!b || !b->ccap || !levels) return G5_ERR_INVALID_ARG;
    CodecCapture h;
    G5_CUDA(cudaStreamSynchronize(b->stream));
    G5_CUDA(cudaMemcpy(&h, b->ccap, sizeof h, cudaMemcpyDeviceToHost));
    *levels = (int)h.count;
    if (overflow) *overflow = (int)h.overflow;
    return G5_OK;
}

g5_status g5_bfs_device_pred(g5_bfs *b, const int64_t **pred)
{
    if (!b || !pred) return G5_ERR_INVALID_ARG;
    *pred = b->cur_pred;
    return G5_OK;
}

g5_status g5_bfs_teps_edges(g5_bfs *b, int64_t *nedge)
{
    if (!b || !nedge || !b->ran || !b->g->end_deg) return G5_ERR_INVALID_ARG;
    unsigned long long *d = nullptr;
    G5_CUDA(cudaMalloc(&d, sizeof *d));
    cudaMemsetAsync(d, 0, sizeof *d, b->stream);
    k_teps<<<g5::grid_for(8), kBlock, 0, b->stream>>>(b->cur_pred, b->g->end_deg, b->g->n, d);
    unsigned long long h = 0;
    cudaMemcpyAsync(&h, d, sizeof h, cudaMemcpyDeviceToHost, b->stream);
    cudaError_t e = cudaStreamSynchronize(b->stream);
    cudaFree(d);
    G5_CUDA(e);
    *nedge = (int64_t)(h / 2);
    return G5_OK;
}

g5_status g5_bfs_validate(g5_bfs *b, int64_t root, int *valid, int *min_parent_out)
{
    if (!b || !valid || root < 0 || root >= b->g->n || !b->ran) return G5_ERR_INVALID_ARG;
    const int64_t n = b->g->n;
    cudaStream_t s = b->stream;
    int64_t *anc[2] = {nullptr, nullptr};
    int32_t *dist[2] = {nullptr, nullptr};
    unsigned *flags = nullptr;
    g5_status rc = G5_OK;
    auto cleanup = [&]() {
        cudaFree(anc[0]);
        cudaFree(anc[1]);
        cudaFree(dist[0]);
        cudaFree(dist[1]);
        cudaFree(flags);
    };
    if (cudaMalloc(&anc[0], sizeof(int64_t) * n) != cudaSuccess ||
        cudaMalloc(&anc[1], sizeof(int64_t) * n) != cudaSuccess ||
        cudaMalloc(&dist[0], sizeof(int32_t) * n) != cudaSuccess ||
        cudaMalloc(&dist[1], sizeof(int32_t) * n) != cudaSuccess ||
        cudaMalloc(&flags, sizeof(unsigned) * 2) != cudaSuccess) {
        cleanup();
        return G5_ERR_OOM;
    }
    cudaMemsetAsync(flags, 0, sizeof(unsigned) * 2, s);
    const int64_t *pred = b->cur_pred;
    k_val_init<<<g5::grid_for(8), kBlock, 0, s>>>(pred, n, root, anc[0], dist[0], flags);
    int cur = 0;
    for (int r = 0; r < 64; ++r) {
        cudaMemsetAsync(flags + 1, 0, sizeof(unsigned), s);
        k_val_jump<<<g5::grid_for(8), kBlock, 0, s>>>(anc[cur], dist[cur], anc[1 - cur], dist[1 - cur], n, root,
                                                       flags + 1);
        cur = 1 - cur;
        unsigned ch = 0;
        cudaMemcpyAsync(&ch, flags + 1, sizeof ch, cudaMemcpyDeviceToHost, s);
        if (cudaStreamSynchronize(s) != cudaSuccess) {
            rc = G5_ERR_CUDA;
            break;
        }
        if (!ch) break;
    }
    if (rc == G5_OK) {
        int32_t *lev = dist[1 - cur];  // free after the last jump round
        k_val_level<<<g5::grid_for(8), kBlock, 0, s>>>(pred, anc[cur], dist[cur], n, root, lev);
        k_val_edges<<<g5::grid_for(8), kBlock, 0, s>>>(b->g->row_off, b->g->col, pred, lev, n, root, flags);
        unsigned f = 0;
        cudaMemcpyAsync(&f, flags, sizeof f, cudaMemcpyDeviceToHost, s);
        if (cudaStreamSynchronize(s) != cudaSuccess) rc = G5_ERR_CUDA;
        *valid = (f & ~VAL_MINPAR) == 0;
        if (min_parent_out) *min_parent_out = (f & VAL_MINPAR) == 0;
    }
    cleanup();
    return rc;
}

}  // extern "C"
