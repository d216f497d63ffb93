// g5_codec.cu -- the s4-bp128 frontier-queue codec on the device.
//
// Wire format (identical, word for word, to the reference's vendored
// SIMDCompressionAndIntersection library as configured by the reference,
// cpu_2d/compression/cpusimd/include/codecfactory.h:103-108):
//
//   CompositeCodec (compositecodec.h:31-71): the first floor(n/128)*128 values
//   go to SIMDBinaryPacking, the rest to VariableByte<true>.
//   SIMDBinaryPacking (simdbinarypacking.h:174-289): word 0 = n1, three
//   cookie words 123456, then groups of 16 miniblocks of 128 values: four
//   header words with the 16 bit widths (big-endian bytes), then each
//   miniblock's 4*b payload words.  A partial last group still writes the
//   four header words.
//   Miniblock (SIMDIntegratedBlockPacker, deltatemplates.h:67-120): 32
//   vectors of 4 lanes; d4 subtracts the previous vector lane-wise, dm
//   subtracts lane 3 of the previous vector; the previous vector of the
//   first miniblock is zero; b = bit length of the OR of all deltas; each lane
//   packs its 32 deltas LSB-first, word w of lane l at 4w+l; b = 32 stores the
//   raw values.
//   VariableByte<true> (variablebyte.h:100-161): delta from 0, 7-bit groups
//   little-endian, high bit on the last byte, zero-padded to a word.
//
// GPU design, one stream per call: every miniblock is independent for
// encoding (its deltas only need the input), so one warp packs one
// miniblock; a first launch stores every miniblock's bit width and the word
// count of each block's range of groups, a second one places each range
// after the ranges before it and packs (two launches, no device waits).
// Decoding needs each group's position, which the
// stream only gives as a chain (each header says how long its group is): a
// first pass follows the chain inside chunks of the stream from every
// possible entry and carries the real entries across chunks by look-back;
// a second pass unpacks one group per block, with the running values
// carried across groups by look-back (two launches).  The many-streams
// calls (one launch set for k queues) resolve the chains by binary lifting
// over all 16-byte positions (group starts are always 16-byte aligned) and
// use separate scan passes.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "g5_codec_dev.cuh"
#include "g5_common.cuh"

namespace g5 {

namespace {

constexpr uint32_t kCookie = 123456u;
constexpr int kB = 256;
constexpr int kTailMaxBytes = 4096;  // largest VariableByte tail decoded

// extra scalar slots (beyond CodecScalar)
enum { CS_NMB = 5, CS_RAW = 6, CS_NG = 7 };
// the scalar block holds CS_COUNT entries; decode uses a few more

__device__ __forceinline__ uint32_t bits_of(uint32_t v) { return v ? 32u - __clz(v) : 0u; }

// ---- generic device-count scans -------------------------------------------------

struct AddU32 {
    typedef uint32_t T;
    __device__ static T id() { return 0u; }
    __device__ static T op(T a, T b) { return a + b; }
    __device__ static T shfl_up(T v, int o) { return __shfl_up_sync(0xFFFFFFFFu, v, o); }
};

struct ResetAdd {
    typedef VecFlag T;
    __device__ static T id()
    {
        T t;
        t.v = make_uint4(0, 0, 0, 0);
        t.f = 0;
        return t;
    }
    __device__ static T op(T a, T b)
    {
        if (b.f) return b;
        T r;
        r.v = make_uint4(a.v.x + b.v.x, a.v.y + b.v.y, a.v.z + b.v.z, a.v.w + b.v.w);
        r.f = a.f;
        return r;
    }
    __device__ static T shfl_up(T v, int o)
    {
        T r;
        r.v.x = __shfl_up_sync(0xFFFFFFFFu, v.v.x, o);
        r.v.y = __shfl_up_sync(0xFFFFFFFFu, v.v.y, o);
        r.v.z = __shfl_up_sync(0xFFFFFFFFu, v.v.z, o);
        r.v.w = __shfl_up_sync(0xFFFFFFFFu, v.v.w, o);
        r.f = __shfl_up_sync(0xFFFFFFFFu, v.f, o);
        return r;
    }
};

// Inclusive block scan (blockDim.x == kB); returns inclusive value, total in *tot.
template <class Op>
__device__ typename Op::T block_scan_incl(typename Op::T x, typename Op::T *s_w, typename Op::T &tot)
{
    typedef typename Op::T T;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T y = Op::shfl_up(x, o);
        if (lane >= o) x = Op::op(y, x);
    }
    if (lane == 31) s_w[wid] = x;
    __syncthreads();
    if (threadIdx.x == 0) {
        T acc = Op::id();
        for (int i = 0; i < kB / 32; ++i) {
            T t = s_w[i];
            s_w[i] = acc;
            acc = Op::op(acc, t);
        }
        s_w[kB / 32] = acc;
    }
    __syncthreads();
    T r = Op::op(s_w[wid], x);
    tot = s_w[kB / 32];
    __syncthreads();
    return r;
}

__device__ __forceinline__ void range_of(uint64_t n, uint64_t &b0, uint64_t &b1)
{
    const uint64_t per = (n + gridDim.x - 1) / gridDim.x;
    b0 = min(n, (uint64_t)blockIdx.x * per);
    b1 = min(n, b0 + per);
}

template <class Op>
__global__ void __launch_bounds__(kB) k_scan_red(const typename Op::T *in, const uint64_t *cnt,
                                                 typename Op::T *part)
{
    typedef typename Op::T T;
    __shared__ T s_w[kB / 32 + 1];
    uint64_t b0, b1;
    range_of(*cnt, b0, b1);
    T carry = Op::id();
    for (uint64_t t0 = b0; t0 < b1; t0 += kB) {
        const uint64_t i = t0 + threadIdx.x;
        T x = i < b1 ? in[i] : Op::id();
        T tt;
        block_scan_incl<Op>(x, s_w, tt);
        carry = Op::op(carry, tt);
    }
    if (threadIdx.x == 0) part[blockIdx.x] = carry;
}

// Exclusive scan of the partials in place (single block); total -> *total.
template <class Op>
__global__ void __launch_bounds__(kB) k_scan_top(typename Op::T *part, int np, typename Op::T *total)
{
    typedef typename Op::T T;
    __shared__ T s_w[kB / 32 + 1];
    T carry = Op::id();
    for (int t0 = 0; t0 < np; t0 += kB) {
        const int i = t0 + threadIdx.x;
        T x = i < np ? part[i] : Op::id();
        T tt;
        T inc = block_scan_incl<Op>(x, s_w, tt);
        // exclusive = carry op (inclusive without x): recompute from shuffle
        T exc_local = Op::shfl_up(inc, 1);
        if ((threadIdx.x & 31) == 0) exc_local = Op::id();
        __shared__ T s_prev[kB / 32];
        if ((threadIdx.x & 31) == 31) s_prev[threadIdx.x >> 5] = inc;
        __syncthreads();
        T ex = ((threadIdx.x & 31) == 0) ? (threadIdx.x == 0 ? Op::id() : s_prev[(threadIdx.x >> 5) - 1])
                                          : exc_local;
        if (i < np) part[i] = Op::op(carry, ex);
        __syncthreads();
        carry = Op::op(carry, tt);
    }
    if (threadIdx.x == 0 && total) *total = carry;
}

// Exclusive scan of in[] into out[] (may alias) seeded by part[block].
template <class Op>
__global__ void __launch_bounds__(kB) k_scan_down(const typename Op::T *in, typename Op::T *out,
                                                  const uint64_t *cnt, const typename Op::T *part)
{
    typedef typename Op::T T;
    __shared__ T s_w[kB / 32 + 1];
    __shared__ T s_prev[kB / 32];
    uint64_t b0, b1;
    range_of(*cnt, b0, b1);
    T carry = part[blockIdx.x];
    for (uint64_t t0 = b0; t0 < b1; t0 += kB) {
        const uint64_t i = t0 + threadIdx.x;
        T x = i < b1 ? in[i] : Op::id();
        T tt;
        T inc = block_scan_incl<Op>(x, s_w, tt);
        T exc_local = Op::shfl_up(inc, 1);
        if ((threadIdx.x & 31) == 31) s_prev[threadIdx.x >> 5] = inc;
        __syncthreads();
        T ex = ((threadIdx.x & 31) == 0) ? (threadIdx.x == 0 ? Op::id() : s_prev[(threadIdx.x >> 5) - 1])
                                          : exc_local;
        if (i < b1) out[i] = Op::op(carry, ex);
        __syncthreads();
        carry = Op::op(carry, tt);
    }
}

// ---- encoder ---------------------------------------------------------------------------

__device__ __forceinline__ uint4 deltas(uint4 cur, uint4 prev, int mode)
{
    if (mode == G5_CODEC_DM)
        return make_uint4(cur.x - prev.w, cur.y - prev.w, cur.z - prev.w, cur.w - prev.w);
    return make_uint4(cur.x - prev.x, cur.y - prev.y, cur.z - prev.z, cur.w - prev.w);
}

__device__ __forceinline__ uint32_t comp(const uint4 &v, int l)
{
    return l == 0 ? v.x : l == 1 ? v.y : l == 2 ? v.z : v.w;
}

// ---- decoder ---------------------------------------------------------------------------

// Unpacks lane j's 4 deltas of miniblock k (b < 32) or raw values (b == 32).
__device__ __forceinline__ uint4 unpack_vec(const uint32_t *in, uint64_t off_vec, uint32_t b)
{
    const int j = g5_lane();
    const uint4 *v = reinterpret_cast<const uint4 *>(in) + off_vec;
    if (b == 32) return v[j];
    if (b == 0) return make_uint4(0, 0, 0, 0);
    const uint32_t bit = (uint32_t)j * b, w = bit >> 5, s = bit & 31;
    const uint4 a = v[w];
    uint4 r;
    const uint32_t mask = (b == 32) ? 0xFFFFFFFFu : ((1u << b) - 1u);
    if (s + b > 32) {
        const uint4 c = v[w + 1];
        r.x = ((a.x >> s) | (c.x << (32 - s))) & mask;
        r.y = ((a.y >> s) | (c.y << (32 - s))) & mask;
        r.z = ((a.z >> s) | (c.z << (32 - s))) & mask;
        r.w = ((a.w >> s) | (c.w << (32 - s))) & mask;
    } else {
        r.x = (a.x >> s) & mask;
        r.y = (a.y >> s) & mask;
        r.z = (a.z >> s) & mask;
        r.w = (a.w >> s) & mask;
    }
    return r;
}

__device__ __forceinline__ void mb_locate(const uint32_t *in, const uint32_t *gpos, uint64_t k,
                                          uint64_t &off_vec, uint32_t &b)
{
    const uint64_t g = k / 16, i = k % 16;
    const uint32_t p = gpos[g];
    const uint4 h = reinterpret_cast<const uint4 *>(in)[p];
    const uint32_t hw[4] = {h.x, h.y, h.z, h.w};
    uint64_t s = 0;
    for (uint64_t q = 0; q < i; ++q) s += (hw[q / 4] >> (24 - 8 * (q % 4))) & 0xFF;
    b = (hw[i / 4] >> (24 - 8 * (i % 4))) & 0xFF;
    off_vec = (uint64_t)p + 1 + s;
}

// ---- one-pass kernels: decoupled look-back -----------------------------------------------
//
// The single-stream decoder's passes run over the stream's tiles (a group of
// 16 miniblocks for unpacking, a range of stream vectors for locating
// groups).  Blocks claim tiles in launch order
// from a counter, so a tile only ever waits on tiles claimed before it, whose
// blocks are already running.  Each tile publishes its own aggregate, then
// its inclusive prefix once known; a tile combines the nearest inclusive
// prefix before it with the aggregates in between.  Payloads are written
// before their status word (with a fence between); a status word holds the
// call's epoch, so what earlier calls left reads as "not published" and
// nothing is cleared between calls.  The last block to finish resets the
// counter and advances the epoch.  Every wait is bounded: past kSpinLimit
// polls the kernel records G5_DEVERR_WAIT and goes on with what it has, so
// no launch can spin forever.

constexpr int kOB = 512;                 // one-pass blocks: 16 warps, one per miniblock of a group
constexpr uint32_t kSpinLimit = 1u << 21;
constexpr int kEntries = 513;            // a group spans at most 1 + 16 * 32 vectors
constexpr uint32_t kDead = 0xFFFFu;
enum : uint32_t { ST_NONE = 0, ST_AGG = 1, ST_INC = 2 };

// scalar slots of the one-pass kernels (the scalar block holds kScalars)
enum {
    CS_L_CTR = 20, CS_L_DONE = 21,
    CS_U_CTR = 25, CS_U_DONE = 26, CS_U_EPOCH = 27
};

__device__ __forceinline__ uint64_t vload64(const uint64_t *p) { return *reinterpret_cast<const volatile uint64_t *>(p); }
__device__ __forceinline__ void vstore64(uint64_t *p, uint64_t v) { *reinterpret_cast<volatile uint64_t *>(p) = v; }

__device__ __forceinline__ uint32_t status_flag(uint64_t s, uint64_t epoch)
{
    return (s >> 2) == epoch ? (uint32_t)(s & 3u) : ST_NONE;
}

// Running lane sums with resets (decoder: a raw miniblock restarts the sums).
struct ResetAddV {
    typedef VecFlag T;
    __device__ static T id() { return ResetAdd::id(); }
    __device__ static T op(T a, T b) { return ResetAdd::op(a, b); }
    __device__ static T shfl_down(T v, int o)
    {
        T r;
        r.v.x = __shfl_down_sync(0xFFFFFFFFu, v.v.x, o);
        r.v.y = __shfl_down_sync(0xFFFFFFFFu, v.v.y, o);
        r.v.z = __shfl_down_sync(0xFFFFFFFFu, v.v.z, o);
        r.v.w = __shfl_down_sync(0xFFFFFFFFu, v.v.w, o);
        r.f = __shfl_down_sync(0xFFFFFFFFu, v.f, o);
        return r;
    }
    __device__ static T bcast0(const T &v)
    {
        T r;
        r.v.x = __shfl_sync(0xFFFFFFFFu, v.v.x, 0);
        r.v.y = __shfl_sync(0xFFFFFFFFu, v.v.y, 0);
        r.v.z = __shfl_sync(0xFFFFFFFFu, v.v.z, 0);
        r.v.w = __shfl_sync(0xFFFFFFFFu, v.v.w, 0);
        r.f = __shfl_sync(0xFFFFFFFFu, v.f, 0);
        return r;
    }
    __device__ static T load(const T *p)
    {
        const volatile uint32_t *q = reinterpret_cast<const volatile uint32_t *>(p);
        T r;
        r.v = make_uint4(q[0], q[1], q[2], q[3]);
        r.f = q[4];
        return r;
    }
    __device__ static void store(T *p, const T &v)
    {
        volatile uint32_t *q = reinterpret_cast<volatile uint32_t *>(p);
        q[0] = v.v.x;
        q[1] = v.v.y;
        q[2] = v.v.z;
        q[3] = v.v.w;
        q[4] = v.f;
    }
};

// Decoupled look-back of tile t, run by one whole warp: publishes `mine` as
// the tile's aggregate (tile 0: as its inclusive prefix), combines the tiles
// before it in order and publishes the inclusive prefix; returns the
// exclusive prefix.  agg[t] / inc[t] hold the payloads, st[t] the status.
template <class Op>
__device__ typename Op::T lookback(uint64_t *st, typename Op::T *agg, typename Op::T *inc, uint64_t t,
                                   uint64_t epoch, const typename Op::T &mine, uint64_t *err)
{
    typedef typename Op::T T;
    const int lane = g5_lane();
    if (t == 0) {
        if (lane == 0) {
            Op::store(inc, mine);
            __threadfence();
            vstore64(st, (epoch << 2) | ST_INC);
        }
        return Op::id();
    }
    if (lane == 0) {
        Op::store(agg + t, mine);
        __threadfence();
        vstore64(st + t, (epoch << 2) | ST_AGG);
    }
    T acc = Op::id();  // combination of the tiles after the current window, in order
    int64_t j = (int64_t)t - 1;
    uint32_t spins = 0;
    for (;;) {
        const int64_t idx = j - lane;  // lane 0 is the nearest tile
        const uint32_t flag = idx >= 0 ? status_flag(vload64(st + idx), epoch) : ST_INC;
        const unsigned incm = __ballot_sync(0xFFFFFFFFu, flag == ST_INC);
        const unsigned ready = __ballot_sync(0xFFFFFFFFu, flag != ST_NONE);
        const int first = incm ? __ffs(incm) - 1 : 32;
        const unsigned need = first == 32 ? 0xFFFFFFFFu : (2u << first) - 1u;
        if ((ready & need) != need) {
            if (++spins > kSpinLimit) {
                if (lane == 0) atomicOr((unsigned long long *)err, (unsigned long long)G5_DEVERR_WAIT);
                break;
            }
            __nanosleep(32);
            continue;
        }
        __threadfence();
        T v = Op::id();
        if (lane <= first && idx >= 0) v = flag == ST_INC ? Op::load(inc + idx) : Op::load(agg + idx);
        // in-order reduction: a higher lane is an earlier tile, so each step
        // puts the value from the higher lane first; lane 0 ends with the
        // window's tiles combined from the earliest to the latest
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const T y = Op::shfl_down(v, o);
            if (lane + o < 32) v = Op::op(y, v);
        }
        acc = Op::op(Op::bcast0(v), acc);
        if (first < 32) break;
        j -= 32;
    }
    if (lane == 0) {
        Op::store(inc + t, Op::op(acc, mine));
        __threadfence();
        vstore64(st + t, (epoch << 2) | ST_INC);
    }
    return acc;
}

// Claims the next tile for the whole block (thread 0 draws, all read).
__device__ __forceinline__ uint64_t claim_tile(uint64_t *ctr, uint64_t *s_t)
{
    __syncthreads();  // the previous tile's shared state is no longer read
    if (threadIdx.x == 0) *s_t = atomicAdd((unsigned long long *)ctr, 1ull);
    __syncthreads();
    return *s_t;
}

// True in the block that finishes last (thread 0 only); it may then reset the
// call's counters: every other block has passed its last read of them.
__device__ __forceinline__ bool last_block(uint64_t *done)
{
    __syncthreads();
    if (threadIdx.x != 0) return false;
    __threadfence();
    return atomicAdd((unsigned long long *)done, 1ull) == gridDim.x - 1;
}

// Stream header words and the VariableByte tail of n - n1 (< 128) values,
// written by one warp; blkend = word after the block part.  Total words ->
// scal[CS_WORDS] and, if given, *words_out.  (compositecodec.h:31-51,
// variablebyte.h:100-161: each value's delta from the one before, 0 before
// the first, in 7-bit groups from the low end, the high bit on the last
// byte, zero-padded to a word.)  One lane per value: its byte count, their
// exclusive prefix over the warp (its place), then its bytes.
__device__ void enc_tail_warp(const uint32_t *in, uint64_t n, uint64_t n1, uint64_t blkend, uint32_t *out,
                              uint64_t *scal, uint64_t *words_out, uint32_t *s_bytes)
{
    const int lane = g5_lane();
    const uint32_t nt = (uint32_t)(n - n1);
    for (uint32_t i = lane; i < (128 * 5 + 3) / 4 + 1; i += 32) s_bytes[i] = 0;
    __syncwarp();
    uint8_t *bb = reinterpret_cast<uint8_t *>(s_bytes);
    uint32_t p = 0, last = 0;  // bytes so far and the value before this round (warp-uniform)
    for (uint32_t i0 = 0; i0 < nt; i0 += 32) {
        const uint32_t i = i0 + lane;
        const bool have = i < nt;
        const uint32_t x = have ? in[n1 + i] : 0u;
        uint32_t px = __shfl_up_sync(0xFFFFFFFFu, x, 1);
        if (lane == 0) px = last;
        const uint32_t d = x - px;
        const uint32_t len = have ? 1u + (d >= (1u << 7)) + (d >= (1u << 14)) + (d >= (1u << 21)) + (d >= (1u << 28)) : 0u;
        uint32_t inc = len;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, inc, o);
            if (lane >= o) inc += y;
        }
        const uint32_t at = p + inc - len;
        for (uint32_t k = 0; k < len; ++k)
            bb[at + k] = (uint8_t)(((d >> (7 * k)) & 127u) | (k + 1 == len ? 128u : 0u));
        p += __shfl_sync(0xFFFFFFFFu, inc, 31);
        last = __shfl_sync(0xFFFFFFFFu, x, 31);
    }
    __syncwarp();
    const uint32_t tw = (p + 3) / 4;
    if (lane == 0) {
        out[0] = (uint32_t)n1;
        out[1] = kCookie;
        out[2] = kCookie;
        out[3] = kCookie;
        scal[CS_WORDS] = blkend + tw;
        if (words_out) *words_out = blkend + tw;
        scal[CS_BLKEND] = blkend;
    }
    for (uint32_t i = lane; i < tw; i += 32) out[blkend + i] = s_bytes[i];
}

// ---- encoder: two passes ----------------------------------------------------------------
//
// A miniblock's bit width depends only on its own 128 values and the vector
// before them, so the stream's layout is fixed once every width is known.
// Block b of the B launched blocks takes the groups [b NG / B, (b + 1) NG / B)
// in both passes (NG groups of 16 miniblocks):
//   k_enc_widths  a warp per miniblock ORs the deltas and stores the width
//                 (one byte per miniblock); the block stores its range's
//                 word count (4 header words per group + 4 b per miniblock)
//   k_enc_pack    the block adds up the counts of the blocks before it (its
//                 range's place in the stream), scans its groups' sizes, and
//                 a warp per miniblock packs the deltas at their place from a
//                 second read of the input (mostly still in L2); the block
//                 with the last group writes the stream header and the
//                 VariableByte tail
// No block waits on another: the launch boundary orders the passes.  n comes
// from device memory, so both launches can sit in a CUDA graph with a fixed
// grid.
constexpr int kEB = 512;  // encoder threads per block: 16 warps
constexpr int kEU = 4;    // miniblocks whose loads a warp has in flight together (widths)
constexpr int kPU = 2;    // the same when packing (two blocks of 512 fit an SM at 64 registers)
constexpr int kPC = 256;  // groups per packing chunk (each miniblock's place held in shared memory)

struct EncLen {
    uint64_t n, n1, nmb, ng;
    bool raw, too_long;
};

__device__ __forceinline__ EncLen enc_len(const uint64_t *n_dev, uint64_t max_n, uint64_t raw_thr)
{
    EncLen e;
    const uint64_t n_in = *n_dev;
    e.too_long = n_in > max_n;  // a device-side length past the workspace: nothing is written
    e.n = e.too_long ? 0 : n_in;
    e.n1 = e.n / 128 * 128;
    e.nmb = e.n / 128;
    e.ng = (e.nmb + 15) / 16;
    e.raw = raw_thr && e.n <= raw_thr;
    return e;
}

__device__ __forceinline__ void enc_range(uint64_t ng, uint32_t nb, uint64_t &g0, uint64_t &g1)
{
    g0 = ng * blockIdx.x / nb;
    g1 = ng * (blockIdx.x + 1) / nb;
}

// Lane j's vector j of miniblock k; lane 0 also the vector before the
// miniblock (zero before the first).  Loads only: prev_of() shuffles later.
__device__ __forceinline__ void load_cur(const uint32_t *in, uint64_t k, uint4 &cur, uint4 &pl)
{
    const uint4 *v = reinterpret_cast<const uint4 *>(in) + k * 32;
    cur = v[g5_lane()];
    pl = (g5_lane() == 0 && k) ? v[-1] : make_uint4(0, 0, 0, 0);
}

__device__ __forceinline__ uint4 prev_of(const uint4 &cur, const uint4 &pl)
{
    uint4 p;
    p.x = __shfl_up_sync(0xFFFFFFFFu, cur.x, 1);
    p.y = __shfl_up_sync(0xFFFFFFFFu, cur.y, 1);
    p.z = __shfl_up_sync(0xFFFFFFFFu, cur.z, 1);
    p.w = __shfl_up_sync(0xFFFFFFFFu, cur.w, 1);
    return g5_lane() == 0 ? pl : p;
}

// The widths of group g (16 bytes, byte q = miniblock 16 g + q) with the
// bytes of miniblocks past nmb cleared (a partial last group's header
// carries width 0 there, simdbinarypacking.h:200-214).
__device__ __forceinline__ uint4 group_widths(const uint8_t *wb, uint64_t g, uint64_t nmb)
{
    uint4 w = *reinterpret_cast<const uint4 *>(wb + 16 * g);
    const uint64_t c = nmb - 16 * g;  // miniblocks in the group
    if (c < 16) {
        uint32_t x[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int keep = (int)c - 4 * j;  // bytes of word j that stay
            x[j] = keep >= 4 ? x[j] : keep <= 0 ? 0u : x[j] & ((1u << (8 * keep)) - 1u);
        }
        w = make_uint4(x[0], x[1], x[2], x[3]);
    }
    return w;
}

// Sum of the first i widths of a group (bytes 0 .. i-1 of w).
__device__ __forceinline__ uint32_t widths_before(const uint4 &w, uint32_t i)
{
    const uint32_t x[4] = {w.x, w.y, w.z, w.w};
    uint32_t s = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int keep = (int)i - 4 * j;
        const uint32_t m = keep >= 4 ? 0xFFFFFFFFu : keep <= 0 ? 0u : (1u << (8 * keep)) - 1u;
        s = __dp4a(x[j] & m, 0x01010101u, s);
    }
    return s;
}

__global__ void __launch_bounds__(kEB, 2) k_enc_widths(const uint32_t *__restrict__ in, const uint64_t *n_dev,
                                                    uint64_t max_n, uint64_t raw_thr, uint8_t *__restrict__ wb,
                                                    uint64_t *__restrict__ btot, uint32_t nb, int mode)
{
    __shared__ uint32_t s_sum;
    g5_pdl_sync();
    const EncLen e = enc_len(n_dev, max_n, raw_thr);
    if (e.raw || e.too_long) return;
    const int lane = g5_lane(), wid = threadIdx.x >> 5;
    uint64_t g0, g1;
    enc_range(e.ng, nb, g0, g1);
    const uint64_t k1 = min(16 * g1, e.nmb);
    if (threadIdx.x == 0) s_sum = 0;
    __syncthreads();
    uint32_t sum = 0;  // warp-uniform
    for (uint64_t kb = 16 * g0 + wid; kb < k1; kb += 16 * kEU) {
        uint4 cur[kEU], pl[kEU];
#pragma unroll
        for (int i = 0; i < kEU; ++i) {
            cur[i] = pl[i] = make_uint4(0, 0, 0, 0);
            if (kb + 16 * i < k1) load_cur(in, kb + 16 * i, cur[i], pl[i]);
        }
#pragma unroll
        for (int i = 0; i < kEU; ++i) {
            const uint64_t k = kb + 16 * i;
            if (k >= k1) break;
            const uint4 d = deltas(cur[i], prev_of(cur[i], pl[i]), mode);
            const uint32_t b = bits_of(__reduce_or_sync(0xFFFFFFFFu, d.x | d.y | d.z | d.w));
            if (lane == 0) wb[k] = (uint8_t)b;
            sum += b;
        }
    }
    if (lane == 0 && sum) atomicAdd(&s_sum, sum);
    __syncthreads();
    if (threadIdx.x == 0) btot[blockIdx.x] = 4 * (g1 - g0) + 4 * (uint64_t)s_sum;
}

// Sum over the block (kEB threads) of a 64-bit value, returned to all.
__device__ __forceinline__ uint64_t block_sum_u64(uint64_t x, uint64_t *s_red)
{
    const int lane = g5_lane(), wid = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o; o >>= 1) x += __shfl_down_sync(0xFFFFFFFFu, x, o);
    if (lane == 0) s_red[wid] = x;
    __syncthreads();
    uint64_t t = 0;
#pragma unroll
    for (int i = 0; i < kEB / 32; ++i) t += s_red[i];
    __syncthreads();
    return t;
}

// Exclusive scan over the block (kEB threads) of a 32-bit value; total -> tot.
__device__ __forceinline__ uint32_t block_excl_u32(uint32_t x, uint32_t *s_w, uint32_t &tot)
{
    const int lane = g5_lane(), wid = threadIdx.x >> 5;
    uint32_t inc = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, inc, o);
        if (lane >= o) inc += y;
    }
    if (lane == 31) s_w[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        const uint32_t v = lane < kEB / 32 ? s_w[lane] : 0u;
        uint32_t vi = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, vi, o);
            if (lane >= o) vi += y;
        }
        if (lane < kEB / 32) s_w[lane] = vi - v;
        if (lane == kEB / 32 - 1) s_w[kEB / 32] = vi;
    }
    __syncthreads();
    const uint32_t r = s_w[wid] + inc - x;
    tot = s_w[kEB / 32];
    __syncthreads();
    return r;
}

// Packs a miniblock's deltas (lane j holds vector j) with width b (1..31)
// into shared memory at s: value j of lane l occupies bits j b .. of lane
// l's bit stream, whose word w is s[4 w + l]
// (ipackwithoutmask<b>, simdintegratedbitpacking.cpp:875).  Each lane ORs
// its four values into place (a value that straddles two words into both)
// after the words are cleared: no division, no loop over values.
__device__ __forceinline__ void pack_mb_smem(const uint4 &d, uint32_t b, uint32_t *s)
{
    const int lane = g5_lane();
    if (lane < (int)b) reinterpret_cast<uint4 *>(s)[lane] = make_uint4(0, 0, 0, 0);  // 4 b words
    __syncwarp();
    const uint32_t bit = (uint32_t)lane * b, w = bit >> 5, sh = bit & 31;
    const bool spill = sh + b > 32;
    uint32_t *p = s + 4 * w;
    const uint32_t v[4] = {d.x, d.y, d.z, d.w};
#pragma unroll
    for (int l = 0; l < 4; ++l) {
        atomicOr(p + l, v[l] << sh);
        if (spill) atomicOr(p + 4 + l, v[l] >> (32 - sh));
    }
}

__global__ void __launch_bounds__(kEB, 2) k_enc_pack(const uint32_t *__restrict__ in, const uint64_t *n_dev,
                                                  uint64_t max_n, uint64_t raw_thr, uint32_t *__restrict__ out,
                                                  uint64_t *scal, const uint8_t *__restrict__ wb,
                                                  const uint64_t *__restrict__ btot, uint32_t nb,
                                                  uint64_t *words_out, int mode)
{
    __shared__ __align__(16) uint32_t s_stage[kEB / 32][128];  // one miniblock's payload per warp
    __shared__ __align__(16) uint32_t s_moff[kPC * 16];  // words from the chunk's first header to each miniblock
    __shared__ __align__(16) uint8_t s_mb[kPC * 16];     // each miniblock's width
    __shared__ uint64_t s_red[kEB / 32];
    __shared__ uint32_t s_w[kEB / 32 + 1];
    __shared__ uint32_t s_bytes[(128 * 5 + 3) / 4 + 1];
    g5_pdl_sync();
    const EncLen e = enc_len(n_dev, max_n, raw_thr);
    const int lane = g5_lane(), wid = threadIdx.x >> 5;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        scal[CS_N] = e.n;
        scal[CS_N1] = e.n1;
        scal[CS_NMB] = e.nmb;
        scal[CS_RAW] = e.raw ? 1 : 0;
        scal[CS_ERR] = e.too_long ? G5_DEVERR_CAPACITY : 0;
    }
    if (e.too_long) return;
    if (e.raw) {
        for (uint64_t i = (uint64_t)blockIdx.x * kEB + threadIdx.x; i < e.n; i += (uint64_t)gridDim.x * kEB)
            out[i] = in[i];
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            scal[CS_WORDS] = e.n;
            if (words_out) *words_out = e.n;
        }
        return;
    }
    if (e.ng == 0) {
        if (blockIdx.x == 0 && wid == 0) enc_tail_warp(in, e.n, e.n1, 4, out, scal, words_out, s_bytes);
        return;
    }
    uint64_t g0, g1;
    enc_range(e.ng, nb, g0, g1);
    if (g0 == g1) return;
    uint64_t x = 0;
    for (uint32_t i = threadIdx.x; i < blockIdx.x; i += kEB) x += btot[i];
    uint64_t cbase = 4 + block_sum_u64(x, s_red);  // word of the chunk's first group header
    uint32_t *stage = s_stage[wid];
    for (uint64_t c0 = g0; c0 < g1; c0 += kPC) {
        // thread t < kPC takes group c0 + t: its size into the chunk's scan,
        // then its header, and its miniblocks' places and widths into
        // shared memory
        const uint64_t g = c0 + threadIdx.x;
        const bool mine = threadIdx.x < kPC && g < g1;
        uint4 wv = make_uint4(0, 0, 0, 0);
        if (mine) wv = group_widths(wb, g, e.nmb);
        uint32_t ctot;
        const uint32_t goff = block_excl_u32(mine ? 4 + 4 * widths_before(wv, 16) : 0u, s_w, ctot);
        if (mine) {
            // the 16 widths, big-endian bytes in each word (simdbinarypacking.h:200-214)
            reinterpret_cast<uint4 *>(out + cbase + goff)[0] =
                make_uint4(__byte_perm(wv.x, 0, 0x0123), __byte_perm(wv.y, 0, 0x0123),
                           __byte_perm(wv.z, 0, 0x0123), __byte_perm(wv.w, 0, 0x0123));
            reinterpret_cast<uint4 *>(s_mb)[threadIdx.x] = wv;
            uint32_t o = goff + 4;
            const uint32_t x[4] = {wv.x, wv.y, wv.z, wv.w};
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                uint4 r;
                r.x = o;
                o += 4 * (x[j] & 0xFFu);
                r.y = o;
                o += 4 * ((x[j] >> 8) & 0xFFu);
                r.z = o;
                o += 4 * ((x[j] >> 16) & 0xFFu);
                r.w = o;
                o += 4 * (x[j] >> 24);
                reinterpret_cast<uint4 *>(s_moff)[4 * threadIdx.x + j] = r;
            }
        }
        __syncthreads();
        const uint64_t kc = 16 * c0;  // the chunk's first miniblock
        const uint32_t mk = (uint32_t)(min(16 * min(c0 + kPC, g1), e.nmb) - kc);  // its miniblocks
        for (uint32_t mb = wid; mb < mk; mb += 16 * kPU) {
            uint4 cur[kPU], pl[kPU];
#pragma unroll
            for (int i = 0; i < kPU; ++i) {
                cur[i] = pl[i] = make_uint4(0, 0, 0, 0);
                if (mb + 16 * i < mk) load_cur(in, kc + mb + 16 * i, cur[i], pl[i]);
            }
#pragma unroll
            for (int i = 0; i < kPU; ++i) {
                const uint32_t m = mb + 16 * i;
                if (m >= mk) break;
                const uint32_t b = s_mb[m];
                uint4 *dst = reinterpret_cast<uint4 *>(out + cbase + s_moff[m]);
                if (b == 32) {
                    dst[lane] = cur[i];
                } else if (b) {
                    pack_mb_smem(deltas(cur[i], prev_of(cur[i], pl[i]), mode), b, stage);
                    __syncwarp();
                    if (lane < (int)b) dst[lane] = reinterpret_cast<const uint4 *>(stage)[lane];
                    __syncwarp();
                }
            }
        }
        cbase += ctot;
        __syncthreads();
    }
    if (g1 == e.ng && wid == 0) enc_tail_warp(in, e.n, e.n1, cbase, out, scal, words_out, s_bytes);
}

// ---- decoder: locate groups ----------------------------------------------------------
//
// A group's position is only given by the chain of group headers before it
// (each says how long its group is).  The stream's vectors are cut into
// chunks of S (a power of two from kLocMin to kLocMax, chosen so that there
// are at most kLocFit chunks); a chunk's first group starts somewhere in its
// first kEntries vectors (a group spans at most that many).
//   k_loc_tables  (one block per chunk) follows the chain inside the chunk
//                 from every possible entry and writes, per entry, where the
//                 chain leaves the chunk and how many groups it started (the
//                 chunk's transfer table), and each vector's jump
//   k_loc_walk    (one block) carries the real entry from chunk to chunk
//                 through the tables, held in shared memory
//   k_loc_pos     (one block per chunk) follows the chain from the chunk's
//                 real entry and writes its groups' positions
// Chains through vectors that cannot be headers (a width above 32, a group
// running past the stream) are marked dead; a real chain that reaches one
// before the last group makes the stream corrupt.

// Header checks every block makes alike; false if the stream is raw or bad.
struct DecHead {
    uint64_t words, nv, n1, nmb, ng;
    bool raw, bad;
};

__device__ __forceinline__ DecHead dec_head(const uint32_t *in, const uint64_t *words_dev, uint64_t cap,
                                            uint64_t raw_thr, const uint64_t *n_expect, uint64_t max_vec,
                                            uint64_t max_mb)
{
    DecHead h;
    h.words = *words_dev;
    h.nv = h.words / 4;
    h.n1 = h.nmb = h.ng = 0;
    h.bad = false;
    // plugin semantics: raw when n <= thr or the stream is as long as n
    // (cpu_2d/compression/cpusimd.hh:169-173)
    h.raw = raw_thr && n_expect && (*n_expect <= raw_thr || h.words == *n_expect);
    if (h.raw) {
        h.bad = h.words > cap;
        return h;
    }
    if (h.words < 4) {
        h.bad = true;
    } else {
        h.n1 = in[0];
        if (in[1] != kCookie || in[2] != kCookie || in[3] != kCookie) h.bad = true;
        if (h.n1 % 128 || h.n1 > cap || h.n1 / 128 >= max_mb) h.bad = true;
    }
    if (h.nv > max_vec) h.bad = true;
    if (h.bad) h.n1 = 0;
    h.nmb = h.n1 / 128;
    h.ng = (h.nmb + 15) / 16;
    return h;
}

__device__ __forceinline__ uint32_t width_of(uint4 h, int i)
{
    const uint32_t w = i < 4 ? h.x : i < 8 ? h.y : i < 12 ? h.z : h.w;
    return (w >> (24 - 8 * (i & 3))) & 0xFFu;
}

constexpr int kLocMin = 2048, kLocMax = 16384;  // chunk sizes in vectors
constexpr int kLocBatch = 4;                    // candidate vectors a thread loads together
// a chunk's candidates are read in whole rounds of kOB * kLocBatch, none past its end
static_assert(kLocMin % (kOB * kLocBatch) == 0, "chunk sizes must be whole load rounds");
constexpr int kLocFit = 96;                     // chunks whose tables the walk holds in shared memory
constexpr int kWalkThreads = 1024;

// Chunk size for a stream of nv vectors (the same in all three kernels).
__device__ __forceinline__ uint32_t loc_chunk(uint64_t nv)
{
    uint32_t S = kLocMin;
    while (S < kLocMax && (nv + S - 1) / S > (uint64_t)kLocFit) S <<= 1;
    return S;
}

__global__ void __launch_bounds__(kOB) k_loc_tables(const uint32_t *__restrict__ in, const uint64_t *words_dev,
                                                    uint64_t cap, uint64_t raw_thr, const uint64_t *n_expect,
                                                    uint64_t *scal, uint64_t max_vec, uint64_t max_mb,
                                                    uint32_t *ltab, uint16_t *ljump)
{
    __shared__ uint16_t s_j[kLocMax];
    __shared__ uint64_t s_t;
    g5_pdl_sync();
    const DecHead h = dec_head(in, words_dev, cap, raw_thr, n_expect, max_vec, max_mb);
    const uint32_t S = loc_chunk(h.nv);
    const uint64_t nchunks = (h.raw || h.bad || h.ng == 0) ? 0 : (h.nv - 1 + S - 1) / S;
    for (;;) {
        const uint64_t c = claim_tile(&scal[CS_L_CTR], &s_t);
        if (c >= nchunks) break;
        const uint64_t a = 1 + c * S;  // first vector of the chunk
        const uint4 *v = reinterpret_cast<const uint4 *>(in);
        // kLocBatch of the thread's candidate vectors loaded together, then
        // their jumps (S is a multiple of kOB * kLocBatch)
        for (uint32_t p0 = threadIdx.x; p0 < S; p0 += kOB * kLocBatch) {
            uint4 hv[kLocBatch];
#pragma unroll
            for (int i = 0; i < kLocBatch; ++i) {
                const uint32_t p = p0 + i * kOB;
                hv[i] = a + p < h.nv ? v[a + p] : make_uint4(0, 0, 0, 0);
            }
#pragma unroll
            for (int i = 0; i < kLocBatch; ++i) {
                const uint32_t p = p0 + i * kOB;
                uint32_t r = kDead;
                if (a + p < h.nv) {
                    // the 16 widths (bytes) added four at a time; a byte
                    // above 32 rules the vector out as a header
                    const uint32_t x[4] = {hv[i].x, hv[i].y, hv[i].z, hv[i].w};
                    uint32_t sum = 0, over = 0;
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        sum = __dp4a(x[j], 0x01010101u, sum);
                        over |= __vcmpgtu4(x[j], 0x20202020u);
                    }
                    if (!over && a + p + 1 + sum <= h.nv) r = p + 1 + sum;  // <= S + 512 < kDead
                    ljump[a + p] = (uint16_t)r;
                }
                s_j[p] = (uint16_t)r;
            }
        }
        __syncthreads();
        // transfer table: entry e -> (exit offset in the next chunk, groups started)
        for (uint32_t e = threadIdx.x; e < kEntries; e += kOB) {
            uint32_t p = e, cnt = 0, exit = kDead;
            if (a + e < h.nv) {
                while (p < S) {
                    const uint32_t r = s_j[p];
                    ++cnt;  // a group starts at p
                    if (r == kDead) break;
                    p = r;
                }
                if (p >= S) exit = p - S;
                else --cnt;  // the dead header starts no group
            }
            ltab[c * kEntries + e] = (exit << 16) | cnt;
        }
    }
    if (last_block(&scal[CS_L_DONE])) {
        scal[CS_L_CTR] = 0;
        scal[CS_L_DONE] = 0;
        __threadfence();
    }
}

// One block: the real entry E_c and groups before it G_c of every chunk,
// chained through the tables (in shared memory when they fit); writes
// lent[c] = E_c | G_c << 32 and the stream's scalars.
__global__ void __launch_bounds__(kWalkThreads) k_loc_walk(const uint32_t *__restrict__ in, const uint64_t *words_dev,
                                                           uint64_t cap, uint64_t raw_thr, const uint64_t *n_expect,
                                                           uint64_t *scal, uint64_t max_vec, uint64_t max_mb,
                                                           const uint32_t *ltab, uint64_t *lent)
{
    extern __shared__ uint32_t s_tab[];
    g5_pdl_sync();
    const DecHead h = dec_head(in, words_dev, cap, raw_thr, n_expect, max_vec, max_mb);
    const uint32_t S = loc_chunk(h.nv);
    const uint64_t nchunks = (h.raw || h.bad || h.ng == 0) ? 0 : (h.nv - 1 + S - 1) / S;
    const bool fit = nchunks <= (uint64_t)kLocFit;
    if (fit) {
        // eight loads per thread in flight at a time
        const uint64_t tot = nchunks * kEntries;
        for (uint64_t i0 = threadIdx.x; i0 < tot; i0 += 8ull * blockDim.x) {
            uint32_t r[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const uint64_t i = i0 + (uint64_t)k * blockDim.x;
                r[k] = i < tot ? ltab[i] : 0u;
            }
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const uint64_t i = i0 + (uint64_t)k * blockDim.x;
                if (i < tot) s_tab[i] = r[k];
            }
        }
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    uint64_t err = h.bad ? G5_DEVERR_CORRUPT : 0;
    uint64_t E = 1, G = 0;
    for (uint64_t c = 0; c < nchunks; ++c) {
        const uint64_t a = 1 + c * S;
        lent[c] = (E & 0xFFFFFFFFull) | (G << 32);
        if (G >= h.ng) continue;  // the chain has ended: this chunk owns nothing
        if (E < a || E - a >= kEntries) {
            err |= G5_DEVERR_CORRUPT;
            G = h.ng;
            continue;
        }
        const uint32_t tv = fit ? s_tab[c * kEntries + (E - a)] : ltab[c * kEntries + (E - a)];
        G += tv & 0xFFFFu;
        if (G >= h.ng) {
            G = h.ng;
            continue;
        }
        if ((tv >> 16) == kDead) {  // the chain dies before the last group
            err |= G5_DEVERR_CORRUPT;
            G = h.ng;
            continue;
        }
        E = a + S + (tv >> 16);
    }
    if (!h.raw && !h.bad && h.ng > 0 && G < h.ng) err |= G5_DEVERR_CORRUPT;
    if (!h.raw && h.ng == 0) scal[CS_BLKEND] = 4;
    scal[CS_ERR] = err;
    scal[CS_WORDS] = h.words;
    scal[CS_RAW] = h.raw ? 1 : 0;
    scal[CS_N1] = h.n1;
    scal[CS_NMB] = h.nmb;
    scal[CS_NG] = h.ng;
    scal[CS_N] = h.raw ? h.words : 0;
}

// One block per chunk: the positions of the chunk's own groups, from its
// real entry along the jumps (staged in shared memory); the block with the
// last group also checks it and sets the end of the block part.
__global__ void __launch_bounds__(kOB) k_loc_pos(const uint32_t *__restrict__ in, uint64_t *scal,
                                                 const uint16_t *ljump, const uint64_t *lent, uint32_t *gpos)
{
    __shared__ uint16_t s_j[kLocMax];
    g5_pdl_sync();
    if (scal[CS_RAW] || scal[CS_ERR]) return;
    const uint64_t ng = scal[CS_NG], nmb = scal[CS_NMB];
    const uint64_t nv = scal[CS_WORDS] / 4;
    const uint32_t S = loc_chunk(nv);
    const uint64_t nchunks = ng == 0 ? 0 : (nv - 1 + S - 1) / S;
    const uint4 *v = reinterpret_cast<const uint4 *>(in);
    for (uint64_t c = blockIdx.x; c < nchunks; c += gridDim.x) {
        const uint64_t a = 1 + c * S;
        const uint64_t en = lent[c];
        const uint64_t g0 = en >> 32;
        const uint64_t gnext = c + 1 < nchunks ? (lent[c + 1] >> 32) : ng;
        if (g0 >= gnext) continue;  // uniform over the block
        __syncthreads();            // the previous chunk's jumps are no longer read
        for (uint32_t p0 = threadIdx.x; p0 < S; p0 += kOB * kLocBatch) {
            uint16_t jv[kLocBatch];
#pragma unroll
            for (int i = 0; i < kLocBatch; ++i) {
                const uint32_t p = p0 + i * kOB;
                jv[i] = a + p < nv ? ljump[a + p] : (uint16_t)0;
            }
#pragma unroll
            for (int i = 0; i < kLocBatch; ++i) {
                const uint32_t p = p0 + i * kOB;
                if (a + p < nv) s_j[p] = jv[i];
            }
        }
        __syncthreads();
        if (threadIdx.x != 0) continue;
        uint64_t p = en & 0xFFFFFFFFull;
        for (uint64_t g = g0; g < gnext; ++g) {
            gpos[g] = (uint32_t)p;
            if (g == ng - 1) {
                // the last group holds only the remaining miniblocks
                const uint4 hv = v[p];
                const uint64_t howmany = nmb - 16 * g;
                uint64_t sum = 0;
                bool ok = true;
                for (uint64_t q = 0; q < howmany; ++q) {
                    const uint32_t b = width_of(hv, (int)q);
                    ok &= b <= 32;
                    sum += b;
                }
                const uint64_t end = p + 1 + sum;
                if (!ok || end > nv) atomicOr((unsigned long long *)&scal[CS_ERR], (unsigned long long)G5_DEVERR_CORRUPT);
                else scal[CS_BLKEND] = 4 * end;
                break;
            }
            if (g + 1 == gnext) break;  // the next group starts in the next chunk
            const uint32_t r = s_j[p - a];
            if (r == kDead) {  // the walk's tables rule this out; kept as a guard
                atomicOr((unsigned long long *)&scal[CS_ERR], (unsigned long long)G5_DEVERR_CORRUPT);
                break;
            }
            p = a + r;
        }
    }
}

// ---- decoder: unpack (one pass) --------------------------------------------------------
//
// Tiles of 4 or 8 groups (8 when tiles of 4 would need more than one wave
// of the grid: fewer tiles make a shorter look-back chain), warp w taking
// miniblocks w, w + 16, w + 32, ... of the tile, four at a time, at the
// positions the locator found: one lane scan per miniblock gives its values
// from the miniblock's start (staged in shared memory) and, in lane 31, its
// aggregate (the lane sums, or for a raw b = 32 miniblock its last vector
// with a reset flag); warp 0 scans the tile's aggregates, finds the tile's
// prefix by look-back and each miniblock's base, which is added as the
// values are written.  Block 0 first decodes the VariableByte tail, which
// starts from 0 whatever the block part holds.  With `expect` every value
// is compared with the expected one (the level loop's round-trip check);
// `acc` accumulates words and values.
constexpr int kTG = 8;          // groups per unpacker tile, at most (4 or 8, see k_dec_unpack)
constexpr int kTM = 16 * kTG;   // miniblocks per tile, at most (each warp takes four at a time)
// dynamic shared memory of the unpacker: each miniblock's values relative
// to its start (kTM x 32 vectors), aggregates, in-tile prefixes, bases, raw flags
constexpr size_t kUValBytes = sizeof(uint4) * kTM * 32;
constexpr size_t kUSmem = kUValBytes + 2 * sizeof(VecFlag) * kTM + sizeof(uint4) * kTM + kTM;

// Stream position (16-byte vectors) and width of miniblock i of the group
// whose header is at vector p.
__device__ __forceinline__ void mb_at(const uint32_t *in, uint32_t p, int i, uint64_t &off, uint32_t &b)
{
    const uint4 hv = reinterpret_cast<const uint4 *>(in)[p];
    // the widths before i: the leading (big-endian) bytes of the header
    // words, each word's bytes added by one dp4a
    const uint32_t x[4] = {hv.x, hv.y, hv.z, hv.w};
    uint32_t sum = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int keep = i - 4 * j;
        const uint32_t m = keep >= 4 ? 0xFFFFFFFFu : keep <= 0 ? 0u : ~(0xFFFFFFFFu >> (8 * keep));
        sum = __dp4a(x[j] & m, 0x01010101u, sum);
    }
    off = (uint64_t)p + 1 + sum;
    b = width_of(hv, i);
}

// A miniblock's deltas (lane j: vector j) turned into its running sums from
// the miniblock's start, in place, and the miniblock's aggregate in lane 31
// (its lane sums, or for a raw b = 32 miniblock its last vector with a reset
// flag).  d4 sums each lane component over the vectors; dm sums component 3
// (every component of a vector is relative to component 3 of the vector
// before), so components 0-2 keep their deltas.  One scan serves both the
// aggregate and the values from the miniblock's start.
__device__ __forceinline__ VecFlag mb_scan(uint4 &d, uint32_t b, int mode)
{
    const int lane = g5_lane();
    VecFlag r;
    if (b == 32) {
        r.v = d;
        r.f = 1;
        return r;
    }
    if (mode == G5_CODEC_DM) {
        uint32_t c = d.w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, c, o);
            if (lane >= o) c += y;
        }
        d.w = c;
        r.v = make_uint4(c, c, c, c);
    } else {
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t yx = __shfl_up_sync(0xFFFFFFFFu, d.x, o);
            const uint32_t yy = __shfl_up_sync(0xFFFFFFFFu, d.y, o);
            const uint32_t yz = __shfl_up_sync(0xFFFFFFFFu, d.z, o);
            const uint32_t yw = __shfl_up_sync(0xFFFFFFFFu, d.w, o);
            if (lane >= o) {
                d.x += yx;
                d.y += yy;
                d.z += yz;
                d.w += yw;
            }
        }
        r.v = d;
    }
    r.f = 0;
    return r;
}

// VariableByte tail decoded by one warp (variablebyte.h:217-): nbytes bytes
// in bb (shared memory), values from out[o] on, each the running sum of the
// decoded deltas from 0; o (warp-uniform) ends past the last value.  A byte
// with the high bit ends a value; a sixth byte of one value (a fifth byte
// without the high bit) or an output index at cap makes the stream corrupt
// and ends the decode there, as the sequential decoder does.  32 bytes per
// round: a ballot marks the values' last bytes, the lane holding one
// gathers its value's bytes from the previous last byte on, and a warp scan
// of the values gives the running sums.
__device__ void dec_tail_warp(const uint8_t *bb, uint32_t nbytes, uint64_t cap, uint32_t *out,
                              const uint32_t *expect, uint64_t &o, uint64_t &e)
{
    const int lane = g5_lane();
    const unsigned lt = g5_lanemask_lt();
    uint32_t run = 0;    // the last value so far
    int last_end = -1;   // byte index of the last value's last byte
    for (uint32_t b0 = 0; b0 < nbytes; b0 += 32) {
        const uint32_t pb = b0 + lane;
        const bool in_range = pb < nbytes;
        const bool term = in_range && (bb[pb] & 128u);
        const unsigned tm = __ballot_sync(0xFFFFFFFFu, term);
        const unsigned below = tm & lt;
        const int prev_end = below ? (int)(b0 + 31 - __clz(below)) : last_end;
        // the fifth byte of a value without the high bit
        const unsigned em = __ballot_sync(0xFFFFFFFFu, in_range && !term && (int)pb - prev_end >= 5);
        unsigned ok = em ? tm & ((1u << (__ffs(em) - 1)) - 1u) : tm;  // values ending before it
        // output capacity, checked value by value
        const uint64_t room = cap > o ? cap - o : 0;
        if ((uint64_t)__popc(ok) > room) {
            unsigned keep = ok;
            for (uint64_t k = 0; k < room; ++k) keep &= keep - 1;  // drop the first `room` values
            ok &= ~keep;
            e |= G5_DEVERR_CORRUPT;
        }
        if (em) e |= G5_DEVERR_CORRUPT;
        const bool mine = (ok >> lane) & 1u;
        uint32_t v = 0;
        if (mine)
            for (int k = prev_end + 1, sh = 0; k <= (int)pb; ++k, sh += 7) v |= (uint32_t)(bb[k] & 127u) << sh;
        uint32_t inc = v;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, inc, d);
            if (lane >= d) inc += y;
        }
        if (mine) {
            const uint64_t idx = o + __popc(ok & lt);
            const uint32_t val = run + inc;
            out[idx] = val;
            if (expect && expect[idx] != val) e |= G5_DEVERR_MISMATCH;
        }
        o += __popc(ok);
        run += __shfl_sync(0xFFFFFFFFu, inc, 31);
        if (tm) last_end = (int)(b0 + 31 - __clz(tm));
        if (e & G5_DEVERR_CORRUPT) break;
    }
    // the lanes' mismatch flags into one
    e |= __reduce_or_sync(0xFFFFFFFFu, (unsigned)(e & G5_DEVERR_MISMATCH)) ? G5_DEVERR_MISMATCH : 0;
}

__global__ void __launch_bounds__(kOB) k_dec_unpack(const uint32_t *__restrict__ in, uint64_t *scal,
                                                    const uint32_t *__restrict__ gpos, uint32_t *__restrict__ out,
                                                    uint64_t cap, const uint64_t *n_expect,
                                                    const uint32_t *__restrict__ expect, uint64_t *acc,
                                                    uint64_t *ust, VecFlag *uagg, VecFlag *uinc, uint64_t *n_out,
                                                    int mode)
{
    extern __shared__ __align__(16) unsigned char s_dyn_u[];
    uint4 *s_val = reinterpret_cast<uint4 *>(s_dyn_u);                        // values from each miniblock's start
    VecFlag *s_vf = reinterpret_cast<VecFlag *>(s_dyn_u + kUValBytes);        // miniblock aggregates
    VecFlag *s_base = s_vf + kTM;                                              // prefixes from the tile's start
    uint4 *s_full = reinterpret_cast<uint4 *>(s_base + kTM);                   // each miniblock's base
    uint8_t *s_raw = reinterpret_cast<uint8_t *>(s_full + kTM);                // 1: a raw miniblock
    __shared__ VecFlag s_ex;            // the tile's aggregate, then its exclusive prefix (look-back)
    __shared__ uint64_t s_t;
    __shared__ uint32_t s_b[kTailMaxBytes / 4];
    const int lane = g5_lane(), wid = threadIdx.x >> 5;
    g5_pdl_sync();
    const uint64_t epoch = scal[CS_U_EPOCH];
    const uint64_t err0 = scal[CS_ERR];
    const uint64_t words = scal[CS_WORDS];
    bool bad = false;
    // the value count: final here for a raw stream or one the locator
    // rejected, else the tail's writer below sets it
    if (n_out && blockIdx.x == 0 && threadIdx.x == 0 && (scal[CS_RAW] || err0)) *n_out = scal[CS_N];
    if (scal[CS_RAW]) {
        const uint64_t n = scal[CS_N];
        if (!err0)
            for (uint64_t i = (uint64_t)blockIdx.x * kOB + threadIdx.x; i < n; i += (uint64_t)gridDim.x * kOB) {
                out[i] = in[i];
                bad |= expect && expect[i] != in[i];
            }
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            if (n_expect && n != *n_expect)
                atomicOr((unsigned long long *)&scal[CS_ERR], (unsigned long long)G5_DEVERR_MISMATCH);
            if (acc) {
                acc[0] += words;
                acc[1] += n;
            }
        }
    } else if (!err0) {
        const uint64_t nmb = scal[CS_NMB], ng = scal[CS_NG], n1 = scal[CS_N1];
        // tiles of 8 groups when tiles of 4 would not all fit in one wave of
        // the grid (fewer tiles, so a shorter look-back chain), else of 4 (more
        // blocks at work on mid-size streams); every block decides alike
        const int R = (ng + 3) / 4 > (uint64_t)gridDim.x ? 2 : 1;  // rounds of four miniblocks per warp
        const uint64_t tm = 64ull * R;                              // miniblocks per tile
        const uint64_t ntiles = (nmb + tm - 1) / tm;
        if (blockIdx.x == 0 && wid == 0) {
            // VariableByte tail (variablebyte.h:217-): words after the block part
            const uint64_t blkend = scal[CS_BLKEND];
            const uint64_t tw = words > blkend ? words - blkend : 0;
            if (tw * 4 > kTailMaxBytes) {
                if (lane == 0) {
                    atomicOr((unsigned long long *)&scal[CS_ERR], (unsigned long long)G5_DEVERR_CORRUPT);
                    if (n_out) *n_out = 0;
                }
            } else {
                for (uint64_t i = lane; i < tw; i += 32) s_b[i] = in[blkend + i];
                __syncwarp();
                uint64_t o = n1, e = 0;
                dec_tail_warp(reinterpret_cast<const uint8_t *>(s_b), (uint32_t)(tw * 4), cap, out, expect, o, e);
                if (lane == 0) {
                    scal[CS_N] = o;
                    if (n_out) *n_out = o;
                    if (n_expect && o != *n_expect) e |= G5_DEVERR_MISMATCH;
                    if (e) atomicOr((unsigned long long *)&scal[CS_ERR], (unsigned long long)e);
                    if (acc) {
                        acc[0] += words;
                        acc[1] += o;
                    }
                }
            }
        }
        for (;;) {
            const uint64_t t = claim_tile(&scal[CS_U_CTR], &s_t);
            if (t >= ntiles) break;
            const uint64_t k0 = tm * t;
            // each warp's miniblocks wid, wid + 16, ..., four at a time: the
            // positions and loads first, then one lane scan per miniblock,
            // whose running sums are the values from the miniblock's start
            // (for dm, components 0-2 take the running component 3 of the
            // vector before) and whose lane 31 holds the aggregate
#pragma unroll 1
            for (int r = 0; r < R; ++r) {
                uint4 d[4];
                uint32_t b[4];
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const uint64_t k = k0 + wid + 16 * (4 * r + i);
                    d[i] = make_uint4(0, 0, 0, 0);
                    b[i] = 0;
                    if (k < nmb) {
                        uint64_t off;
                        mb_at(in, gpos[k / 16], wid, off, b[i]);
                        d[i] = unpack_vec(in, off, b[i]);
                    }
                }
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const int m = wid + 16 * (4 * r + i);
                    if (k0 + m < nmb) {
                        const VecFlag agg = mb_scan(d[i], b[i], mode);
                        uint4 rel = d[i];
                        if (b[i] != 32 && mode == G5_CODEC_DM) {
                            uint32_t cp = __shfl_up_sync(0xFFFFFFFFu, d[i].w, 1);
                            if (lane == 0) cp = 0;
                            rel = make_uint4(d[i].x + cp, d[i].y + cp, d[i].z + cp, d[i].w);
                        }
                        s_val[m * 32 + lane] = rel;
                        if (lane == 31) s_vf[m] = agg;
                        if (lane == 0) s_raw[m] = b[i] == 32 ? 1 : 0;
                    } else if (lane == 31) {
                        s_vf[m] = ResetAdd::id();
                    }
                }
            }
            __syncthreads();
            if (wid == 0) {
                // prefixes from the tile's start, 2 R miniblocks per lane in
                // order (a reset inside the tile makes the rest absolute)
                const int kPer = 2 * R;
                VecFlag c = s_vf[kPer * lane];
                for (int j = 1; j < kPer; ++j) c = ResetAdd::op(c, s_vf[kPer * lane + j]);
                VecFlag inc = c;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const VecFlag y = ResetAdd::shfl_up(inc, o);
                    if (lane >= o) inc = ResetAdd::op(y, inc);
                }
                VecFlag ex = ResetAdd::shfl_up(inc, 1);
                if (lane == 0) ex = ResetAdd::id();
                for (int j = 0; j < kPer; ++j) {
                    s_base[kPer * lane + j] = ex;
                    ex = ResetAdd::op(ex, s_vf[kPer * lane + j]);
                }
                if (lane == 31) s_ex = inc;  // the tile's aggregate, until the look-back replaces it
            }
            __syncthreads();
            // warp 0 finds the tile's prefix (look-back), then every
            // miniblock's base: the tile's prefix combined with the
            // miniblock's prefix inside the tile
            if (wid == 0) {
                const VecFlag pre = lookback<ResetAddV>(ust, uagg, uinc, t, epoch, s_ex, &scal[CS_ERR]);
                for (int m = lane; m < (int)tm; m += 32) s_full[m] = ResetAdd::op(pre, s_base[m]).v;
            }
            __syncthreads();
            {
                const uint64_t kn = min(tm, nmb - k0);  // miniblocks in this tile
                for (uint32_t q = threadIdx.x; q < kn * 32; q += kOB) {
                    const uint32_t m = q >> 5;  // miniblock of this 16-byte vector
                    uint4 x = s_val[q];
                    if (!s_raw[m]) {
                        const uint4 bm = s_full[m];
                        if (mode == G5_CODEC_DM) {
                            x.x += bm.w;
                            x.y += bm.w;
                            x.z += bm.w;
                            x.w += bm.w;
                        } else {
                            x.x += bm.x;
                            x.y += bm.y;
                            x.z += bm.z;
                            x.w += bm.w;
                        }
                    }
                    reinterpret_cast<uint4 *>(out)[k0 * 32 + q] = x;
                    if (expect) {
                        const uint4 e = reinterpret_cast<const uint4 *>(expect)[k0 * 32 + q];
                        bad |= (e.x != x.x) | (e.y != x.y) | (e.z != x.z) | (e.w != x.w);
                    }
                }
            }
        }
    }
    if (bad) atomicOr((unsigned long long *)&scal[CS_ERR], (unsigned long long)G5_DEVERR_MISMATCH);
    if (last_block(&scal[CS_U_DONE])) {
        scal[CS_U_CTR] = 0;
        scal[CS_U_DONE] = 0;
        scal[CS_U_EPOCH] = epoch + 1;
        __threadfence();
    }
}

// ---- many streams in one launch set -------------------------------------------------------
//
// k queues (or k streams) are concatenated; each kernel below walks the global
// index space of all streams' miniblocks, groups or vectors and finds the
// stream of an index by a binary search over the per-stream first indices, so
// the k streams cost one launch set instead of k.  Each stream's bytes are
// exactly those of a single-stream call.

struct BStream {
    uint64_t in_off;   // encode: first input value; decode: first stream word (multiple of 4)
    uint64_t out_off;  // encode: first output word (multiple of 4); decode: first output value
    uint64_t n;        // values
    uint64_t words;    // decode: stream length; encode: written by k_benc_tail
    uint64_t nmb;      // miniblocks of the block part (0 for a raw stream)
    uint64_t nv;       // decode: whole 16-byte vectors of the stream
    uint64_t blkend;   // decode: word after the block part
    uint32_t raw;      // raw copy (plugin threshold semantics)
    uint32_t err;      // G5_DEVERR_* bits
};

// The last stream s < k with first[s] <= x (empty streams share a first
// index with the next one, so x always lands in a stream that holds it).
__device__ __forceinline__ int find_stream(const uint64_t *first, int k, uint64_t x)
{
    int lo = 0, hi = k - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (first[mid] <= x) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// load_vectors for an input of any alignment (queues start anywhere).
__device__ __forceinline__ void load_vectors_any(const uint32_t *in, uint64_t k, uint4 &cur, uint4 &prev)
{
    const int lane = g5_lane();
    const uint32_t *p = in + k * 128 + 4 * (uint64_t)lane;
    cur = make_uint4(p[0], p[1], p[2], p[3]);
    uint4 q;
    q.x = __shfl_up_sync(0xFFFFFFFFu, cur.x, 1);
    q.y = __shfl_up_sync(0xFFFFFFFFu, cur.y, 1);
    q.z = __shfl_up_sync(0xFFFFFFFFu, cur.z, 1);
    q.w = __shfl_up_sync(0xFFFFFFFFu, cur.w, 1);
    if (lane == 0) q = k ? make_uint4(p[-4], p[-3], p[-2], p[-1]) : make_uint4(0, 0, 0, 0);
    prev = q;
}

__global__ void __launch_bounds__(kB) k_benc_bits(const uint32_t *in, const BStream *bs, const uint64_t *mb0,
                                                  int k, uint64_t total_mb, uint8_t *mb_bits, uint32_t *mb_len,
                                                  int mode)
{
    const uint64_t gw = ((uint64_t)blockIdx.x * kB + threadIdx.x) >> 5;
    const uint64_t nw = ((uint64_t)gridDim.x * kB) >> 5;
    for (uint64_t kg = gw; kg < total_mb; kg += nw) {
        const int s = find_stream(mb0, k, kg);
        uint4 cur, prev;
        load_vectors_any(in + bs[s].in_off, kg - mb0[s], cur, prev);
        const uint4 d = deltas(cur, prev, mode);
        uint32_t acc = d.x | d.y | d.z | d.w;
#pragma unroll
        for (int o = 16; o; o >>= 1) acc |= __shfl_xor_sync(0xFFFFFFFFu, acc, o);
        if (g5_lane() == 0) {
            const uint32_t b = bits_of(acc);
            mb_bits[kg] = (uint8_t)b;
            mb_len[kg] = 4 * b;
        }
    }
}

// mb_off: exclusive prefix of the payload words over all miniblocks.
__global__ void __launch_bounds__(kB) k_benc_pack(const uint32_t *in, const BStream *bs, const uint64_t *mb0,
                                                  int k, uint64_t total_mb, const uint8_t *mb_bits,
                                                  const uint32_t *mb_off, uint32_t *out, int mode)
{
    __shared__ uint4 s_d[kB / 32][32];
    const int lane = g5_lane(), wib = threadIdx.x >> 5;
    const uint64_t gw = ((uint64_t)blockIdx.x * kB + threadIdx.x) >> 5;
    const uint64_t nw = ((uint64_t)gridDim.x * kB) >> 5;
    for (uint64_t kg = gw; kg < total_mb; kg += nw) {
        const int s = find_stream(mb0, k, kg);
        const BStream &st = bs[s];
        const uint64_t kl = kg - mb0[s];
        const uint32_t base = mb_off[mb0[s]];
        uint32_t *o = out + st.out_off;
        const uint32_t b = mb_bits[kg];
        const uint64_t off = 4 + 4 * (kl / 16 + 1) + (uint64_t)(mb_off[kg] - base);
        if ((kl & 15) == 0 && lane < 4) {
            uint32_t h = 0;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const uint64_t kk = kl + 4 * lane + q;
                const uint32_t bb = kk < st.nmb ? mb_bits[mb0[s] + kk] : 0u;
                h |= bb << (24 - 8 * q);
            }
            o[4 + 4 * (kl / 16) + (uint64_t)(mb_off[kg] - base) + lane] = h;
        }
        uint4 cur, prev;
        load_vectors_any(in + st.in_off, kl, cur, prev);
        if (b == 32) {
            reinterpret_cast<uint4 *>(o + off)[lane] = cur;
            continue;
        }
        if (b == 0) continue;
        s_d[wib][lane] = deltas(cur, prev, mode);
        __syncwarp();
        for (uint32_t idx = lane; idx < 4 * b; idx += 32) {
            const uint32_t w = idx >> 2, l = idx & 3;
            const uint32_t bit0 = 32 * w;
            const uint32_t j0 = bit0 / b, j1 = (bit0 + 31) / b;
            uint32_t word = 0;
            for (uint32_t j = j0; j <= j1 && j < 32; ++j) {
                const uint32_t dd = comp(s_d[wib][j], l);
                const int sh = (int)(j * b) - (int)bit0;
                word |= sh >= 0 ? (dd << sh) : (dd >> (-sh));
            }
            o[off + idx] = word;
        }
        __syncwarp();
    }
}

// One warp per stream: raw copies, header words and the VariableByte tail;
// the stream's length -> bs[s].words.  payload_total: sum of all payloads.
__global__ void k_benc_tail(const uint32_t *in, BStream *bs, const uint64_t *mb0, int k, uint64_t total_mb,
                            const uint32_t *mb_off, const uint32_t *payload_total, uint32_t *out)
{
    __shared__ uint32_t s_val[128];
    __shared__ uint32_t s_bytes[(128 * 5 + 3) / 4 + 1];
    const int lane = threadIdx.x;
    for (int s = blockIdx.x; s < k; s += gridDim.x) {
        BStream &st = bs[s];
        const uint32_t *x = in + st.in_off;
        uint32_t *o = out + st.out_off;
        if (st.raw) {
            for (uint64_t i = lane; i < st.n; i += 32) o[i] = x[i];
            if (lane == 0) st.words = st.n;
            continue;
        }
        const uint64_t nmb = st.nmb, n1 = nmb * 128, ngroups = (nmb + 15) / 16;
        uint64_t payload = 0;
        if (nmb) {
            const uint64_t e = mb0[s] + nmb;
            payload = (uint64_t)((e < total_mb ? mb_off[e] : *payload_total) - mb_off[mb0[s]]);
        }
        const uint64_t blkend = 4 + 4 * ngroups + payload;
        const uint32_t nt = (uint32_t)(st.n - n1);
        __syncwarp();
        for (uint32_t i = lane; i < nt; i += 32) s_val[i] = x[n1 + i];
        for (uint32_t i = lane; i < sizeof(s_bytes) / 4; i += 32) s_bytes[i] = 0;
        __syncwarp();
        if (lane == 0) {
            o[0] = (uint32_t)n1;
            o[1] = kCookie;
            o[2] = kCookie;
            o[3] = kCookie;
            uint8_t *bb = reinterpret_cast<uint8_t *>(s_bytes);
            uint32_t p = 0, prevv = 0;
            for (uint32_t i = 0; i < nt; ++i) {
                uint32_t v = s_val[i] - prevv;
                prevv = s_val[i];
                while (v >= 128u) {
                    bb[p++] = (uint8_t)(v & 127u);
                    v >>= 7;
                }
                bb[p++] = (uint8_t)(v | 128u);
            }
            const uint32_t tw = (p + 3) / 4;
            s_val[0] = tw;
            st.words = blkend + tw;
        }
        __syncwarp();
        const uint32_t tw = s_val[0];
        for (uint32_t i = lane; i < tw; i += 32) o[blkend + i] = s_bytes[i];
    }
}

// Stream headers (one thread per stream): cookies and the block-part length.
__global__ void k_bdec_prep(const uint32_t *in, BStream *bs, int k)
{
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < k; s += gridDim.x * blockDim.x) {
        BStream &st = bs[s];
        st.err = 0;
        st.blkend = 4;
        if (st.raw) {
            if (st.words != st.n) st.err |= G5_DEVERR_CORRUPT;
            continue;
        }
        const uint32_t *x = in + st.in_off;
        if (st.words < 4 || x[0] != st.nmb * 128 || x[1] != kCookie || x[2] != kCookie || x[3] != kCookie)
            st.err |= G5_DEVERR_CORRUPT;
    }
}

// jump[vg] = global vector after the group whose header is global vector vg,
// or the sink (total_v) when that leaves the stream.
__global__ void __launch_bounds__(kB) k_bdec_jump(const uint32_t *in, const BStream *bs, const uint64_t *v0,
                                                  int k, uint64_t total_v, uint32_t *jump)
{
    for (uint64_t vg = (uint64_t)blockIdx.x * kB + threadIdx.x; vg <= total_v; vg += (uint64_t)gridDim.x * kB) {
        uint32_t j = (uint32_t)total_v;
        if (vg < total_v) {
            const int s = find_stream(v0, k, vg);
            const BStream &st = bs[s];
            const uint64_t lv = vg - v0[s];
            const uint4 h = reinterpret_cast<const uint4 *>(in + st.in_off)[lv];
            const uint32_t hw[4] = {h.x, h.y, h.z, h.w};
            uint32_t sum = 0;
            bool ok = true;
#pragma unroll
            for (int q = 0; q < 4; ++q)
#pragma unroll
                for (int by = 0; by < 4; ++by) {
                    const uint32_t b = (hw[q] >> (8 * by)) & 0xFF;
                    ok &= b <= 32;
                    sum += b;
                }
            if (ok && lv + 1 + sum < st.nv) j = (uint32_t)(vg + 1 + sum);
        }
        jump[vg] = j;
    }
}

__global__ void __launch_bounds__(kB) k_bdec_lift(uint32_t *jump, uint64_t total_v, uint64_t stride, int r)
{
    const uint32_t *t = jump + stride * r;
    uint32_t *t1 = jump + stride * (r + 1);
    for (uint64_t i = (uint64_t)blockIdx.x * kB + threadIdx.x; i <= total_v; i += (uint64_t)gridDim.x * kB)
        t1[i] = t[t[i]];
}

// Group positions (local vector index of each group header); the last group
// of a stream gives the end of its block part.
__global__ void __launch_bounds__(kB) k_bdec_pos(const uint32_t *in, BStream *bs, const uint64_t *g0,
                                                 const uint64_t *v0, int k, uint64_t total_g, uint64_t total_v,
                                                 const uint32_t *jump, uint64_t stride, int R, uint32_t *gpos)
{
    for (uint64_t gg = (uint64_t)blockIdx.x * kB + threadIdx.x; gg < total_g; gg += (uint64_t)gridDim.x * kB) {
        const int s = find_stream(g0, k, gg);
        BStream &st = bs[s];
        const uint64_t g = gg - g0[s], ng = (st.nmb + 15) / 16;
        uint64_t pos = v0[s] + 1;
        for (int r = 0; r < R && pos < total_v; ++r)
            if ((g >> r) & 1) pos = jump[stride * r + pos];
        uint64_t lp = 0;
        if (st.err || pos >= v0[s] + st.nv) {
            atomicOr(&st.err, (uint32_t)G5_DEVERR_CORRUPT);
        } else {
            lp = pos - v0[s];
            if (g == ng - 1) {
                const uint64_t howmany = st.nmb - 16 * g;
                const uint4 h = reinterpret_cast<const uint4 *>(in + st.in_off)[lp];
                const uint32_t hw[4] = {h.x, h.y, h.z, h.w};
                uint64_t sum = 0;
                bool ok = true;
                for (uint64_t i = 0; i < howmany; ++i) {
                    const uint32_t b = (hw[i / 4] >> (24 - 8 * (i % 4))) & 0xFF;
                    ok &= b <= 32;
                    sum += b;
                }
                const uint64_t end = lp + 1 + sum;
                if (!ok || end > st.nv) atomicOr(&st.err, (uint32_t)G5_DEVERR_CORRUPT);
                else st.blkend = 4 * end;
            }
        }
        gpos[gg] = (uint32_t)lp;
    }
}

// Per miniblock lane sums (the first miniblock of a stream starts from zero,
// so its sums are absolute and reset the scan).
__global__ void __launch_bounds__(kB) k_bdec_sum(const uint32_t *in, const BStream *bs, const uint64_t *mb0,
                                                 const uint64_t *g0, int k, uint64_t total_mb,
                                                 const uint32_t *gpos, VecFlag *mb_sf, int mode)
{
    const uint64_t gw = ((uint64_t)blockIdx.x * kB + threadIdx.x) >> 5;
    const uint64_t nw = ((uint64_t)gridDim.x * kB) >> 5;
    for (uint64_t kg = gw; kg < total_mb; kg += nw) {
        const int s = find_stream(mb0, k, kg);
        const BStream &st = bs[s];
        const uint64_t kl = kg - mb0[s];
        VecFlag r;
        r.v = make_uint4(0, 0, 0, 0);
        r.f = 1;
        if (!st.err) {
            const uint32_t *x = in + st.in_off;
            uint64_t off;
            uint32_t b;
            mb_locate(x, gpos + g0[s], kl, off, b);
            const uint4 d = unpack_vec(x, off, b);
            if (b == 32) {
                r.v.x = __shfl_sync(0xFFFFFFFFu, d.x, 31);
                r.v.y = __shfl_sync(0xFFFFFFFFu, d.y, 31);
                r.v.z = __shfl_sync(0xFFFFFFFFu, d.z, 31);
                r.v.w = __shfl_sync(0xFFFFFFFFu, d.w, 31);
            } else {
                uint32_t sx = d.x, sy = d.y, sz = d.z, sw = d.w;
#pragma unroll
                for (int o = 16; o; o >>= 1) {
                    sx += __shfl_xor_sync(0xFFFFFFFFu, sx, o);
                    sy += __shfl_xor_sync(0xFFFFFFFFu, sy, o);
                    sz += __shfl_xor_sync(0xFFFFFFFFu, sz, o);
                    sw += __shfl_xor_sync(0xFFFFFFFFu, sw, o);
                }
                if (mode == G5_CODEC_DM) r.v = make_uint4(sw, sw, sw, sw);
                else r.v = make_uint4(sx, sy, sz, sw);
                r.f = kl == 0 ? 1u : 0u;
            }
        }
        if (g5_lane() == 0) mb_sf[kg] = r;
    }
}

__global__ void __launch_bounds__(kB) k_bdec_out(const uint32_t *in, const BStream *bs, const uint64_t *mb0,
                                                 const uint64_t *g0, int k, uint64_t total_mb,
                                                 const uint32_t *gpos, const VecFlag *mb_base, uint32_t *out,
                                                 int mode)
{
    const int lane = g5_lane();
    const uint64_t gw = ((uint64_t)blockIdx.x * kB + threadIdx.x) >> 5;
    const uint64_t nw = ((uint64_t)gridDim.x * kB) >> 5;
    for (uint64_t kg = gw; kg < total_mb; kg += nw) {
        const int s = find_stream(mb0, k, kg);
        const BStream &st = bs[s];
        if (st.err) continue;
        const uint64_t kl = kg - mb0[s];
        const uint32_t *x = in + st.in_off;
        uint64_t off;
        uint32_t b;
        mb_locate(x, gpos + g0[s], kl, off, b);
        const uint4 d = unpack_vec(x, off, b);
        const uint4 base = kl == 0 ? make_uint4(0, 0, 0, 0) : mb_base[kg].v;
        uint4 v;
        if (b == 32) {
            v = d;
        } else if (mode == G5_CODEC_DM) {
            uint32_t c = d.w;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, c, o);
                if (lane >= o) c += y;
            }
            c += base.w;
            uint32_t pc = __shfl_up_sync(0xFFFFFFFFu, c, 1);
            if (lane == 0) pc = base.w;
            v = make_uint4(d.x + pc, d.y + pc, d.z + pc, c);
        } else {
            uint32_t cx = d.x, cy = d.y, cz = d.z, cw = d.w;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t yx = __shfl_up_sync(0xFFFFFFFFu, cx, o);
                const uint32_t yy = __shfl_up_sync(0xFFFFFFFFu, cy, o);
                const uint32_t yz = __shfl_up_sync(0xFFFFFFFFu, cz, o);
                const uint32_t yw = __shfl_up_sync(0xFFFFFFFFu, cw, o);
                if (lane >= o) {
                    cx += yx;
                    cy += yy;
                    cz += yz;
                    cw += yw;
                }
            }
            v = make_uint4(cx + base.x, cy + base.y, cz + base.z, cw + base.w);
        }
        uint32_t *o = out + st.out_off + kl * 128 + 4 * (uint64_t)lane;  // any alignment
        o[0] = v.x;
        o[1] = v.y;
        o[2] = v.z;
        o[3] = v.w;
    }
}

// One warp per stream: raw copies and the VariableByte tail; every stream
// must decode to exactly its n values.
__global__ void k_bdec_tail(const uint32_t *in, BStream *bs, int k, uint32_t *out)
{
    __shared__ uint32_t s_b[kTailMaxBytes / 4];
    const int lane = threadIdx.x;
    for (int s = blockIdx.x; s < k; s += gridDim.x) {
        BStream &st = bs[s];
        const uint32_t *x = in + st.in_off;
        uint32_t *o = out + st.out_off;
        if (st.err) continue;
        if (st.raw) {
            for (uint64_t i = lane; i < st.n; i += 32) o[i] = x[i];
            continue;
        }
        const uint64_t n1 = st.nmb * 128;
        const uint64_t tw = st.words > st.blkend ? st.words - st.blkend : 0;
        if (tw * 4 > kTailMaxBytes) {
            if (lane == 0) st.err |= G5_DEVERR_CORRUPT;
            continue;
        }
        __syncwarp();
        for (uint64_t i = lane; i < tw; i += 32) s_b[i] = x[st.blkend + i];
        __syncwarp();
        if (lane == 0) {
            const uint8_t *bb = reinterpret_cast<const uint8_t *>(s_b);
            uint64_t c = n1;
            uint32_t prevv = 0, v = 0;
            int shift = 0;
            uint32_t err = 0;
            for (uint64_t p = 0; p < tw * 4; ++p) {
                const uint32_t ch = bb[p];
                v |= (ch & 127u) << shift;
                if (ch & 128u) {
                    if (c >= st.n) {
                        err |= G5_DEVERR_CORRUPT;
                        break;
                    }
                    prevv += v;
                    o[c++] = prevv;
                    v = 0;
                    shift = 0;
                } else {
                    shift += 7;
                    if (shift > 28) {
                        err |= G5_DEVERR_CORRUPT;
                        break;
                    }
                }
            }
            if (c != st.n) err |= G5_DEVERR_CORRUPT;
            st.err |= err;
        }
    }
}

}  // namespace

size_t codec_bound(size_t n)
{
    const size_t mb = n / 128;
    return 4 + 4 * (mb / 16 + 1) + mb * 128 + ((n % 128) * 5 + 3) / 4 + 8;
}

size_t codec_tiles(size_t max_n) { return (max_n / 128 + 1) / 16 + 2; }

size_t codec_chunks(size_t max_n) { return (codec_bound(max_n) / 4 + 2) / kLocMin + 2; }

int codec_grid() { return num_sms() * 2; }

g5_status codec_work_alloc(CodecWork &w, size_t max_n)
{
    w.max_n = max_n;
    w.max_mb = max_n / 128 + 1;
    w.max_vec = codec_bound(max_n) / 4 + 2;
    w.grid = codec_grid();
    const size_t T = codec_tiles(max_n), C = codec_chunks(max_n);
    G5_CUDA(cudaMalloc(&w.scal, sizeof(uint64_t) * kScalars));
    G5_CUDA(cudaMalloc(&w.gpos, sizeof(uint32_t) * T));
    w.enc_blocks = w.grid;
    G5_CUDA(cudaMalloc(&w.ewb, 16 * T));
    G5_CUDA(cudaMalloc(&w.etot, sizeof(uint64_t) * w.enc_blocks));
    G5_CUDA(cudaMalloc(&w.ltab, sizeof(uint32_t) * kEntries * C));
    G5_CUDA(cudaMalloc(&w.lent, sizeof(uint64_t) * C));
    G5_CUDA(cudaMalloc(&w.ljump, sizeof(uint16_t) * (w.max_vec + 2)));
    // the walk's table cache needs more than 48 KB of shared memory (set per device)
    G5_CUDA(cudaFuncSetAttribute(k_loc_walk, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(sizeof(uint32_t) * kEntries * kLocFit)));
    G5_CUDA(cudaFuncSetAttribute(k_dec_unpack, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kUSmem));
    G5_CUDA(cudaMalloc(&w.ust, sizeof(uint64_t) * T));
    G5_CUDA(cudaMalloc(&w.uagg, sizeof(VecFlag) * 2 * T));
    w.uinc = w.uagg + T;
    // epochs start at 1, so zeroed status words read as "not published"
    G5_CUDA(cudaMemset(w.scal, 0, sizeof(uint64_t) * kScalars));
    G5_CUDA(cudaMemset(w.ust, 0, sizeof(uint64_t) * T));
    const uint64_t one = 1;
    for (int e : {CS_U_EPOCH})
        G5_CUDA(cudaMemcpy(w.scal + e, &one, sizeof one, cudaMemcpyHostToDevice));
    return G5_OK;
}

void codec_work_free(CodecWork &w)
{
    cudaFree(w.scal);
    cudaFree(w.gpos);
    cudaFree(w.ewb);
    cudaFree(w.etot);
    cudaFree(w.ltab);
    cudaFree(w.lent);
    cudaFree(w.ljump);
    cudaFree(w.ust);
    cudaFree(w.uagg);
    w = CodecWork();
}

void codec_encode_launch(CodecWork &w, const uint32_t *in, const uint64_t *n_dev, uint32_t *out, int mode,
                         uint64_t raw_threshold, cudaStream_t s, uint64_t *words_out)
{
    // programmatic dependent launches: each kernel's first instruction waits
    // for the kernel before it, so only the launch latency is overlapped
    const uint32_t nb = (uint32_t)std::min(w.grid, w.enc_blocks);
    launch(true, k_enc_widths, nb, kEB, s, in, n_dev, (uint64_t)w.max_n, raw_threshold, w.ewb, w.etot, nb, mode);
    launch(true, k_enc_pack, nb, kEB, s, in, n_dev, (uint64_t)w.max_n, raw_threshold, out, w.scal,
           (const uint8_t *)w.ewb, (const uint64_t *)w.etot, nb, words_out, mode);
}

void codec_decode_launch(CodecWork &w, const uint32_t *in, const uint64_t *words_dev, uint32_t *out, size_t cap,
                         int mode, uint64_t raw_threshold, const uint64_t *n_expect_dev, const uint32_t *expect,
                         cudaStream_t s, uint64_t *n_out)
{
    decode_launch_acc(w, in, words_dev, out, cap, mode, raw_threshold, n_expect_dev, expect, nullptr, s, n_out);
}

void decode_launch_acc(CodecWork &w, const uint32_t *in, const uint64_t *words_dev, uint32_t *out, size_t cap,
                       int mode, uint64_t raw_threshold, const uint64_t *n_expect_dev, const uint32_t *expect,
                       uint64_t *acc, cudaStream_t s, uint64_t *n_out)
{
    // programmatic dependent launches: each kernel's first instruction waits
    // for the kernel before it, so only the launch latency is overlapped
    const uint64_t mv = w.max_vec, mm = w.max_mb, c = cap, rt = raw_threshold;
    launch(true, k_loc_tables, w.grid, kOB, s, in, words_dev, c, rt, n_expect_dev, w.scal, mv, mm, w.ltab, w.ljump);
    launch_dyn(true, k_loc_walk, 1, kWalkThreads, sizeof(uint32_t) * kEntries * kLocFit, s, in, words_dev, c, rt,
               n_expect_dev, w.scal, mv, mm, (const uint32_t *)w.ltab, w.lent);
    launch(true, k_loc_pos, w.grid, kOB, s, in, w.scal, (const uint16_t *)w.ljump, (const uint64_t *)w.lent, w.gpos);
    launch_dyn(true, k_dec_unpack, w.grid, kOB, kUSmem, s, in, w.scal, (const uint32_t *)w.gpos, out, c,
               n_expect_dev, expect, acc, w.ust, w.uagg, w.uinc, n_out, mode);
}

}  // namespace g5

// ---- C ABI ----------------------------------------------------------------------------

namespace {

// Device buffers of the batched calls, grown on demand (contents not kept).
struct BatchWs {
    void *p[10] = {nullptr};
    size_t cap[10] = {0};
    enum { BS, IDX, BITS, LEN, JUMP, GPOS, SF, BASE, PART, CNT };
    g5_status grow(int i, size_t bytes)
    {
        if (p[i] && cap[i] >= bytes) return G5_OK;
        cudaFree(p[i]);
        p[i] = nullptr;
        cap[i] = 0;
        if (cudaMalloc(&p[i], bytes ? bytes : 16) != cudaSuccess) return G5_ERR_OOM;
        cap[i] = bytes;
        return G5_OK;
    }
    void release()
    {
        for (int i = 0; i < 10; ++i) cudaFree(p[i]);
        *this = BatchWs();
    }
};

size_t round4(size_t w) { return (w + 3) & ~(size_t)3; }

}  // namespace

struct g5_codec {
    g5::CodecWork w;
    uint64_t *n_dev = nullptr;
    uint64_t *h_scal = nullptr;  // pinned
    BatchWs bw;
};

extern "C" {

size_t g5_codec_bound(size_t n) { return g5::codec_bound(n); }

g5_status g5_codec_create(size_t max_n, g5_codec **out)
{
    if (!out || max_n == 0 || max_n > ((size_t)1 << 31)) return G5_ERR_INVALID_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return G5_ERR_NO_DEVICE;
    }
    g5_codec *c = new g5_codec();
    g5_status s = g5::codec_work_alloc(c->w, max_n);
    if (s == G5_OK && cudaMalloc(&c->n_dev, sizeof(uint64_t) * 2) != cudaSuccess) s = G5_ERR_OOM;
    if (s == G5_OK && cudaMallocHost(&c->h_scal, sizeof(uint64_t) * 16) != cudaSuccess) s = G5_ERR_OOM;
    if (s != G5_OK) {
        g5::codec_work_free(c->w);
        cudaFree(c->n_dev);
        delete c;
        return s;
    }
    *out = c;
    return G5_OK;
}

g5_status g5_codec_destroy(g5_codec *c)
{
    if (!c) return G5_ERR_INVALID_ARG;
    cudaDeviceSynchronize();
    g5::codec_work_free(c->w);
    cudaFree(c->n_dev);
    cudaFreeHost(c->h_scal);
    c->bw.release();
    delete c;
    return G5_OK;
}

g5_status g5_codec_encode(g5_codec *c, const uint32_t *in_dev, size_t n, uint32_t *out_dev, size_t *out_words,
                          int mode, void *stream)
{
    if (!c || (n && !in_dev) || !out_dev || !out_words || n > c->w.max_n) return G5_ERR_INVALID_ARG;
    if (mode != G5_CODEC_D4 && mode != G5_CODEC_DM) return G5_ERR_INVALID_ARG;
    if (((uintptr_t)in_dev | (uintptr_t)out_dev) & 15) return G5_ERR_INVALID_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    c->h_scal[15] = n;
    G5_CUDA(cudaMemcpyAsync(c->n_dev, &c->h_scal[15], sizeof(uint64_t), cudaMemcpyHostToDevice, s));
    g5::codec_encode_launch(c->w, in_dev, c->n_dev, out_dev, mode, 0, s);
    G5_CUDA(cudaGetLastError());
    G5_CUDA(cudaMemcpyAsync(c->h_scal, c->w.scal, sizeof(uint64_t) * 8, cudaMemcpyDeviceToHost, s));
    G5_CUDA(cudaStreamSynchronize(s));
    if (c->h_scal[g5::CS_ERR]) return G5_ERR_CAPACITY;  // the encoder has no device waits
    *out_words = (size_t)c->h_scal[g5::CS_WORDS];
    return G5_OK;
}

g5_status g5_codec_decode(g5_codec *c, const uint32_t *in_dev, size_t words, uint32_t *out_dev, size_t out_cap,
                          size_t *out_n, int mode, void *stream)
{
    if (!c || !in_dev || !out_dev || !out_n) return G5_ERR_INVALID_ARG;
    if (mode != G5_CODEC_D4 && mode != G5_CODEC_DM) return G5_ERR_INVALID_ARG;
    if (((uintptr_t)in_dev | (uintptr_t)out_dev) & 15) return G5_ERR_INVALID_ARG;
    if (words / 4 > c->w.max_vec) return G5_ERR_CAPACITY;
    cudaStream_t s = (cudaStream_t)stream;
    c->h_scal[15] = words;
    G5_CUDA(cudaMemcpyAsync(c->n_dev + 1, &c->h_scal[15], sizeof(uint64_t), cudaMemcpyHostToDevice, s));
    g5::codec_decode_launch(c->w, in_dev, c->n_dev + 1, out_dev, out_cap, mode, 0, nullptr, nullptr, s);
    G5_CUDA(cudaGetLastError());
    G5_CUDA(cudaMemcpyAsync(c->h_scal, c->w.scal, sizeof(uint64_t) * 8, cudaMemcpyDeviceToHost, s));
    G5_CUDA(cudaStreamSynchronize(s));
    if (c->h_scal[g5::CS_ERR] & G5_DEVERR_WAIT) return G5_ERR_TIMEOUT;
    if (c->h_scal[g5::CS_ERR]) return G5_ERR_CORRUPT_STREAM;
    *out_n = (size_t)c->h_scal[g5::CS_N];
    return G5_OK;
}

g5_status g5_codec_encode_async(g5_codec *c, const uint32_t *in_dev, const uint64_t *n_dev, uint32_t *out_dev,
                                uint64_t *out_words_dev, int mode, void *stream)
{
    if (!c || !in_dev || !n_dev || !out_dev || !out_words_dev) return G5_ERR_INVALID_ARG;
    if (mode != G5_CODEC_D4 && mode != G5_CODEC_DM) return G5_ERR_INVALID_ARG;
    if (((uintptr_t)in_dev | (uintptr_t)out_dev) & 15) return G5_ERR_INVALID_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    g5::codec_encode_launch(c->w, in_dev, n_dev, out_dev, mode, 0, s, out_words_dev);
    G5_CUDA(cudaGetLastError());
    return G5_OK;
}

g5_status g5_codec_decode_async(g5_codec *c, const uint32_t *in_dev, const uint64_t *words_dev, uint32_t *out_dev,
                                size_t out_cap, uint64_t *out_n_dev, int mode, void *stream)
{
    if (!c || !in_dev || !words_dev || !out_dev || !out_n_dev) return G5_ERR_INVALID_ARG;
    if (mode != G5_CODEC_D4 && mode != G5_CODEC_DM) return G5_ERR_INVALID_ARG;
    if (((uintptr_t)in_dev | (uintptr_t)out_dev) & 15) return G5_ERR_INVALID_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    g5::codec_decode_launch(c->w, in_dev, words_dev, out_dev, out_cap, mode, 0, nullptr, nullptr, s, out_n_dev);
    G5_CUDA(cudaGetLastError());
    return G5_OK;
}

g5_status g5_codec_status(g5_codec *c)
{
    if (!c) return G5_ERR_INVALID_ARG;
    uint64_t err = 0;
    G5_CUDA(cudaMemcpy(&err, c->w.scal + g5::CS_ERR, sizeof err, cudaMemcpyDeviceToHost));
    if (err & G5_DEVERR_WAIT) return G5_ERR_TIMEOUT;
    if (err & G5_DEVERR_CAPACITY) return G5_ERR_CAPACITY;
    if (err) return G5_ERR_CORRUPT_STREAM;
    return G5_OK;
}

size_t g5_codec_batch_bound(const uint64_t *in_off, int k)
{
    if (!in_off || k < 0) return 0;
    size_t w = 0;
    for (int q = 0; q < k; ++q) w += round4(g5::codec_bound((size_t)(in_off[q + 1] - in_off[q])));
    return w;
}

g5_status g5_codec_encode_batch(g5_codec *c, const uint32_t *in_dev, const uint64_t *in_off, int k,
                                uint32_t *out_dev, uint64_t *out_off, uint64_t *out_words,
                                uint32_t raw_threshold, int mode, void *stream)
{
    if (!c || !in_off || !out_off || !out_words || k < 0 || !out_dev) return G5_ERR_INVALID_ARG;
    if (mode != G5_CODEC_D4 && mode != G5_CODEC_DM) return G5_ERR_INVALID_ARG;
    if ((uintptr_t)out_dev & 15) return G5_ERR_INVALID_ARG;
    out_off[0] = 0;
    if (k == 0) return G5_OK;
    if (!in_dev || in_off[0] != 0) return G5_ERR_INVALID_ARG;
    for (int q = 0; q < k; ++q)
        if (in_off[q + 1] < in_off[q]) return G5_ERR_INVALID_ARG;
    if (in_off[k] > ((uint64_t)1 << 31)) return G5_ERR_CAPACITY;  // payload offsets are 32-bit
    std::vector<g5::BStream> hb((size_t)k);
    std::vector<uint64_t> mb0((size_t)k + 1);
    uint64_t total_mb = 0;
    for (int q = 0; q < k; ++q) {
        g5::BStream &b = hb[q];
        memset(&b, 0, sizeof b);
        b.in_off = in_off[q];
        b.out_off = out_off[q];
        b.n = in_off[q + 1] - in_off[q];
        b.raw = raw_threshold && b.n <= raw_threshold;
        b.nmb = b.raw ? 0 : b.n / 128;
        out_off[q + 1] = out_off[q] + round4(g5::codec_bound((size_t)b.n));
        mb0[q] = total_mb;
        total_mb += b.nmb;
    }
    mb0[k] = total_mb;
    BatchWs &w = c->bw;
    const int grid = g5::num_sms() * 4;
    G5_TRY(w.grow(BatchWs::BS, sizeof(g5::BStream) * (size_t)k));
    G5_TRY(w.grow(BatchWs::IDX, sizeof(uint64_t) * ((size_t)k + 1)));
    G5_TRY(w.grow(BatchWs::BITS, total_mb + 1));
    G5_TRY(w.grow(BatchWs::LEN, sizeof(uint32_t) * (total_mb + 1)));
    G5_TRY(w.grow(BatchWs::PART, sizeof(uint32_t) * ((size_t)grid + 1)));
    G5_TRY(w.grow(BatchWs::CNT, sizeof(uint64_t)));
    g5::BStream *bs = (g5::BStream *)w.p[BatchWs::BS];
    uint64_t *idx = (uint64_t *)w.p[BatchWs::IDX], *cnt = (uint64_t *)w.p[BatchWs::CNT];
    uint8_t *bits = (uint8_t *)w.p[BatchWs::BITS];
    uint32_t *len = (uint32_t *)w.p[BatchWs::LEN], *part = (uint32_t *)w.p[BatchWs::PART];
    cudaStream_t s = (cudaStream_t)stream;
    G5_CUDA(cudaMemcpyAsync(bs, hb.data(), sizeof(g5::BStream) * (size_t)k, cudaMemcpyHostToDevice, s));
    G5_CUDA(cudaMemcpyAsync(idx, mb0.data(), sizeof(uint64_t) * ((size_t)k + 1), cudaMemcpyHostToDevice, s));
    G5_CUDA(cudaMemcpyAsync(cnt, &mb0[k], sizeof(uint64_t), cudaMemcpyHostToDevice, s));
    G5_CUDA(cudaMemsetAsync(part + grid, 0, sizeof(uint32_t), s));
    if (total_mb) {
        g5::k_benc_bits<<<grid, g5::kB, 0, s>>>(in_dev, bs, idx, k, total_mb, bits, len, mode);
        g5::k_scan_red<g5::AddU32><<<grid, g5::kB, 0, s>>>(len, cnt, part);
        g5::k_scan_top<g5::AddU32><<<1, g5::kB, 0, s>>>(part, grid, part + grid);
        g5::k_scan_down<g5::AddU32><<<grid, g5::kB, 0, s>>>(len, len, cnt, part);
        g5::k_benc_pack<<<grid, g5::kB, 0, s>>>(in_dev, bs, idx, k, total_mb, bits, len, out_dev, mode);
    }
    g5::k_benc_tail<<<std::min(k, 65535), 32, 0, s>>>(in_dev, bs, idx, k, total_mb, len, part + grid, out_dev);
    G5_CUDA(cudaGetLastError());
    G5_CUDA(cudaMemcpyAsync(hb.data(), bs, sizeof(g5::BStream) * (size_t)k, cudaMemcpyDeviceToHost, s));
    G5_CUDA(cudaStreamSynchronize(s));
    for (int q = 0; q < k; ++q) out_words[q] = hb[q].words;
    return G5_OK;
}

g5_status g5_codec_decode_batch(g5_codec *c, const uint32_t *in_dev, const uint64_t *in_off,
                                const uint64_t *words, const uint64_t *n, int k, uint32_t *out_dev,
                                uint64_t *out_off, int *stream_ok, uint32_t raw_threshold, int mode,
                                void *stream)
{
    if (!c || !in_off || !words || !n || !out_off || k < 0) return G5_ERR_INVALID_ARG;
    if (mode != G5_CODEC_D4 && mode != G5_CODEC_DM) return G5_ERR_INVALID_ARG;
    out_off[0] = 0;
    if (k == 0) return G5_OK;
    if (!in_dev || !out_dev || ((uintptr_t)in_dev & 15)) return G5_ERR_INVALID_ARG;
    std::vector<g5::BStream> hb((size_t)k);
    std::vector<uint64_t> mb0((size_t)k + 1), g0((size_t)k + 1), v0((size_t)k + 1);
    uint64_t total_mb = 0, total_g = 0, total_v = 0;
    int max_ng = 0;
    for (int q = 0; q < k; ++q) {
        if (in_off[q] % 4) return G5_ERR_INVALID_ARG;  // streams start 16-byte aligned
        g5::BStream &b = hb[q];
        memset(&b, 0, sizeof b);
        b.in_off = in_off[q];
        b.out_off = out_off[q];
        b.n = n[q];
        b.words = words[q];
        // plugin semantics: raw when n <= thr or the stream is as long as n
        b.raw = raw_threshold && (b.n <= raw_threshold || b.words == b.n);
        b.nmb = b.raw ? 0 : b.n / 128;
        b.nv = b.raw ? 0 : b.words / 4;
        out_off[q + 1] = out_off[q] + b.n;
        mb0[q] = total_mb;
        g0[q] = total_g;
        v0[q] = total_v;
        const uint64_t ng = (b.nmb + 15) / 16;
        total_mb += b.nmb;
        total_g += ng;
        total_v += b.nv;
        max_ng = std::max<int>(max_ng, (int)std::min<uint64_t>(ng, 1u << 30));
    }
    mb0[k] = total_mb;
    g0[k] = total_g;
    v0[k] = total_v;
    if (total_v >= ((uint64_t)1 << 32) - 2 || out_off[k] > ((uint64_t)1 << 40)) return G5_ERR_CAPACITY;
    int R = 1;
    while (((uint64_t)1 << R) < (uint64_t)max_ng + 1) ++R;
    const uint64_t stride = total_v + 1;
    BatchWs &w = c->bw;
    const int grid = g5::num_sms() * 4;
    G5_TRY(w.grow(BatchWs::BS, sizeof(g5::BStream) * (size_t)k));
    G5_TRY(w.grow(BatchWs::IDX, sizeof(uint64_t) * 3 * ((size_t)k + 1)));
    G5_TRY(w.grow(BatchWs::JUMP, sizeof(uint32_t) * stride * (size_t)R));
    G5_TRY(w.grow(BatchWs::GPOS, sizeof(uint32_t) * (total_g + 1)));
    G5_TRY(w.grow(BatchWs::SF, sizeof(g5::VecFlag) * (total_mb + 1)));
    G5_TRY(w.grow(BatchWs::BASE, sizeof(g5::VecFlag) * (total_mb + 1)));
    G5_TRY(w.grow(BatchWs::PART, sizeof(g5::VecFlag) * ((size_t)grid + 1)));
    G5_TRY(w.grow(BatchWs::CNT, sizeof(uint64_t)));
    g5::BStream *bs = (g5::BStream *)w.p[BatchWs::BS];
    uint64_t *idx = (uint64_t *)w.p[BatchWs::IDX], *cnt = (uint64_t *)w.p[BatchWs::CNT];
    uint64_t *dmb0 = idx, *dg0 = idx + (k + 1), *dv0 = idx + 2 * (k + 1);
    uint32_t *jump = (uint32_t *)w.p[BatchWs::JUMP], *gpos = (uint32_t *)w.p[BatchWs::GPOS];
    g5::VecFlag *sf = (g5::VecFlag *)w.p[BatchWs::SF], *base = (g5::VecFlag *)w.p[BatchWs::BASE];
    g5::VecFlag *part = (g5::VecFlag *)w.p[BatchWs::PART];
    cudaStream_t s = (cudaStream_t)stream;
    std::vector<uint64_t> allidx;
    allidx.reserve(3 * ((size_t)k + 1));
    allidx.insert(allidx.end(), mb0.begin(), mb0.end());
    allidx.insert(allidx.end(), g0.begin(), g0.end());
    allidx.insert(allidx.end(), v0.begin(), v0.end());
    G5_CUDA(cudaMemcpyAsync(bs, hb.data(), sizeof(g5::BStream) * (size_t)k, cudaMemcpyHostToDevice, s));
    G5_CUDA(cudaMemcpyAsync(idx, allidx.data(), sizeof(uint64_t) * allidx.size(), cudaMemcpyHostToDevice, s));
    G5_CUDA(cudaMemcpyAsync(cnt, &mb0[k], sizeof(uint64_t), cudaMemcpyHostToDevice, s));
    const int pgrid = std::max(1, std::min(grid, (k + g5::kB - 1) / g5::kB));
    g5::k_bdec_prep<<<pgrid, g5::kB, 0, s>>>(in_dev, bs, k);
    if (total_g) {
        g5::k_bdec_jump<<<grid, g5::kB, 0, s>>>(in_dev, bs, dv0, k, total_v, jump);
        for (int r = 0; r + 1 < R; ++r) g5::k_bdec_lift<<<grid, g5::kB, 0, s>>>(jump, total_v, stride, r);
        g5::k_bdec_pos<<<grid, g5::kB, 0, s>>>(in_dev, bs, dg0, dv0, k, total_g, total_v, jump, stride, R, gpos);
    }
    if (total_mb) {
        g5::k_bdec_sum<<<grid, g5::kB, 0, s>>>(in_dev, bs, dmb0, dg0, k, total_mb, gpos, sf, mode);
        g5::k_scan_red<g5::ResetAdd><<<grid, g5::kB, 0, s>>>(sf, cnt, part);
        g5::k_scan_top<g5::ResetAdd><<<1, g5::kB, 0, s>>>(part, grid, nullptr);
        g5::k_scan_down<g5::ResetAdd><<<grid, g5::kB, 0, s>>>(sf, base, cnt, part);
        g5::k_bdec_out<<<grid, g5::kB, 0, s>>>(in_dev, bs, dmb0, dg0, k, total_mb, gpos, base, out_dev, mode);
    }
    g5::k_bdec_tail<<<std::min(k, 65535), 32, 0, s>>>(in_dev, bs, k, out_dev);
    G5_CUDA(cudaGetLastError());
    G5_CUDA(cudaMemcpyAsync(hb.data(), bs, sizeof(g5::BStream) * (size_t)k, cudaMemcpyDeviceToHost, s));
    G5_CUDA(cudaStreamSynchronize(s));
    bool all = true;
    for (int q = 0; q < k; ++q) {
        const bool ok = hb[q].err == 0;
        if (stream_ok) stream_ok[q] = ok ? 1 : 0;
        all &= ok;
    }
    return all ? G5_OK : G5_ERR_CORRUPT_STREAM;
}

}  // extern "C"

// ---- encode without allocation ---------------------------------------------------------
//
// For callers that must not touch the CUDA allocator at all: a serving loop
// that may not block on (or fragment) device memory between requests, or a
// host process whose device memory is owned by another allocator (a
// framework's caching pool) with no headroom for cudaMalloc.  The encoder's
// scratch (its scalars, the length, the bit width of every miniblock and the
// word count of every encoder block) lives in the file-scope array below
// instead of a g5_codec workspace: 12,608 bytes (about 12 KiB,
// kNoAllocBytes) that every GPU which loads the library holds until the
// process exits.  Nothing in it needs clearing between calls: each call
// writes every width and count it reads.  The array's device address is looked up
// once per device and cached for the life of the process, so the entry point
// must not be used again on a device after cudaDeviceReset in the same
// process (the reset frees the module that holds the array).

namespace {

constexpr size_t kNoAllocMaxValues = (size_t)1 << 20;             // values per call
constexpr size_t kNoAllocMb = kNoAllocMaxValues / 128 + 1;          // miniblocks
constexpr size_t kNoAllocWb = (kNoAllocMb / 16 + 1) * 16;          // miniblock widths, whole groups
constexpr size_t kNoAllocBlocks = 516;                              // encoder blocks at most
constexpr size_t kNoAllocScal = sizeof(uint64_t) * g5::kScalars;    // scalars
constexpr size_t kNoAllocBytes = kNoAllocScal + 16 + kNoAllocWb + sizeof(uint64_t) * kNoAllocBlocks;
static_assert(kNoAllocBytes == 12608, "the documented size of the scratch array");

// In host code this name is only a host-side stand-in for the device array;
// kernels receive the device address fetched with cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g5_noalloc_scratch[kNoAllocBytes];

std::mutex g_noalloc_mu;
void *g_noalloc_addr[256] = {nullptr};  // per device ordinal

}  // namespace

extern "C" g5_status g5_codec_encode_noalloc(const uint32_t *in_dev, size_t n, uint32_t *out_dev,
                                             size_t *out_words, int mode, void *stream)
{
    if ((n && !in_dev) || !out_dev || !out_words) return G5_ERR_INVALID_ARG;
    if (mode != G5_CODEC_D4 && mode != G5_CODEC_DM) return G5_ERR_INVALID_ARG;
    if (((uintptr_t)in_dev | (uintptr_t)out_dev) & 15) return G5_ERR_INVALID_ARG;
    if (n > kNoAllocMaxValues) {
        if (getenv("G5_VERBOSE"))
            fprintf(stderr, "g5_codec_encode_noalloc: %zu values exceed the limit of %zu\n", n, kNoAllocMaxValues);
        return G5_ERR_CAPACITY;
    }
    int dev = 0;
    G5_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 256) return G5_ERR_INVALID_ARG;
    void *base = nullptr;
    {
        // set-up, once per device, with that device current
        std::lock_guard<std::mutex> lk(g_noalloc_mu);
        if (!g_noalloc_addr[dev]) {
            void *p = nullptr;
            G5_CUDA(cudaGetSymbolAddress(&p, g5_noalloc_scratch));
            g_noalloc_addr[dev] = p;
        }
        base = g_noalloc_addr[dev];
    }
    unsigned char *b = static_cast<unsigned char *>(base);
    g5::CodecWork w;
    w.max_n = kNoAllocMaxValues;
    w.max_mb = kNoAllocMb;
    w.grid = g5::codec_grid();
    w.scal = reinterpret_cast<uint64_t *>(b);
    uint64_t *n_dev = reinterpret_cast<uint64_t *>(b + kNoAllocScal);
    w.ewb = b + kNoAllocScal + 16;
    w.etot = reinterpret_cast<uint64_t *>(b + kNoAllocScal + 16 + kNoAllocWb);
    w.enc_blocks = (int)kNoAllocBlocks;
    static_assert((kNoAllocScal + 16 + kNoAllocWb) % 16 == 0, "the widths are read as 16-byte vectors");
    cudaStream_t s = (cudaStream_t)stream;
    uint64_t hn = n;
    G5_CUDA(cudaMemcpyAsync(n_dev, &hn, sizeof hn, cudaMemcpyHostToDevice, s));
    g5::codec_encode_launch(w, in_dev, n_dev, out_dev, mode, 0, s);
    G5_CUDA(cudaGetLastError());
    uint64_t sc[3] = {0, 0, 0};  // CS_N, CS_WORDS, CS_ERR
    G5_CUDA(cudaMemcpyAsync(sc, w.scal, sizeof sc, cudaMemcpyDeviceToHost, s));
    G5_CUDA(cudaStreamSynchronize(s));
    if (sc[g5::CS_ERR]) return G5_ERR_CAPACITY;
    *out_words = (size_t)sc[g5::CS_WORDS];
    return G5_OK;
}
