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
// GPU design: every miniblock is independent for encoding (its deltas only
// need the input), so one warp packs one miniblock; offsets come from a
// prefix sum of the bit widths.  Decoding needs each group's position, which
// the stream only gives as a chain (each header says how long its group is):
// the chain is resolved with binary lifting over all 16-byte positions
// (group starts are always 16-byte aligned), then one warp unpacks each
// miniblock and a prefix sum over miniblocks restores absolute values.
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
enum { CS_NV = 8, CS_LIFT = 9, CS_TOTAL = 12 };

__device__ __forceinline__ uint32_t bits_of(uint32_t v) { return v ? 32u - __clz(v) : 0u; }

// ---- generic device-count scans -------------------------------------------------

struct AddU32 {
    typedef uint32_t T;
    __device__ static T id() { return 0u; }
    __device__ static T op(T a, T b) { return a + b; }
    __device__ static T shfl_up(T v, int o) { return __shfl_up_sync(0xFFFFFFFFu, v, o); }
};

struct VecFlag {
    uint4 v;
    uint32_t f;
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

__global__ void k_enc_prep(const uint64_t *n_dev, uint64_t raw_thr, uint64_t *scal)
{
    if (threadIdx.x) return;
    const uint64_t n = *n_dev;
    scal[CS_N] = n;
    scal[CS_N1] = n / 128 * 128;
    scal[CS_NMB] = n / 128;
    scal[CS_RAW] = (raw_thr && n <= raw_thr) ? 1 : 0;
    scal[CS_ERR] = 0;
}

// Lane j of a warp loads vector j of miniblock k and its predecessor vector.
__device__ __forceinline__ void load_vectors(const uint32_t *in, uint64_t k, uint4 &cur, uint4 &prev)
{
    const int lane = g5_lane();
    const uint4 *v = reinterpret_cast<const uint4 *>(in) + k * 32;
    cur = v[lane];
    uint4 p;
    p.x = __shfl_up_sync(0xFFFFFFFFu, cur.x, 1);
    p.y = __shfl_up_sync(0xFFFFFFFFu, cur.y, 1);
    p.z = __shfl_up_sync(0xFFFFFFFFu, cur.z, 1);
    p.w = __shfl_up_sync(0xFFFFFFFFu, cur.w, 1);
    if (lane == 0) p = k ? v[-1] : make_uint4(0, 0, 0, 0);
    prev = p;
}

__device__ __forceinline__ uint4 deltas(uint4 cur, uint4 prev, int mode)
{
    if (mode == G5_CODEC_DM)
        return make_uint4(cur.x - prev.w, cur.y - prev.w, cur.z - prev.w, cur.w - prev.w);
    return make_uint4(cur.x - prev.x, cur.y - prev.y, cur.z - prev.z, cur.w - prev.w);
}

__global__ void __launch_bounds__(kB) k_enc_bits(const uint32_t *in, uint64_t *scal, uint8_t *mb_bits,
                                                 uint32_t *mb_len, int mode)
{
    if (scal[CS_RAW]) return;
    const uint64_t nmb = scal[CS_NMB];
    const uint64_t gw = ((uint64_t)blockIdx.x * kB + threadIdx.x) >> 5;
    const uint64_t nw = ((uint64_t)gridDim.x * kB) >> 5;
    for (uint64_t k = gw; k < nmb; k += nw) {
        uint4 cur, prev;
        load_vectors(in, k, cur, prev);
        uint4 d = deltas(cur, prev, mode);
        uint32_t acc = d.x | d.y | d.z | d.w;
#pragma unroll
        for (int o = 16; o; o >>= 1) acc |= __shfl_xor_sync(0xFFFFFFFFu, acc, o);
        if (g5_lane() == 0) {
            const uint32_t b = bits_of(acc);
            mb_bits[k] = (uint8_t)b;
            mb_len[k] = 4 * b;
        }
    }
}

__device__ __forceinline__ uint32_t comp(const uint4 &v, int l)
{
    return l == 0 ? v.x : l == 1 ? v.y : l == 2 ? v.z : v.w;
}

__global__ void __launch_bounds__(kB) k_enc_pack(const uint32_t *in, uint64_t *scal, const uint8_t *mb_bits,
                                                 const uint32_t *mb_off, uint32_t *out, int mode)
{
    __shared__ uint4 s_d[kB / 32][32];
    if (scal[CS_RAW]) {
        const uint64_t n = scal[CS_N];
        for (uint64_t i = (uint64_t)blockIdx.x * kB + threadIdx.x; i < n; i += (uint64_t)gridDim.x * kB)
            out[i] = in[i];
        if (blockIdx.x == 0 && threadIdx.x == 0) scal[CS_WORDS] = n;
        return;
    }
    const uint64_t nmb = scal[CS_NMB];
    const int lane = g5_lane(), wib = threadIdx.x >> 5;
    const uint64_t gw = ((uint64_t)blockIdx.x * kB + threadIdx.x) >> 5;
    const uint64_t nw = ((uint64_t)gridDim.x * kB) >> 5;
    for (uint64_t k = gw; k < nmb; k += nw) {
        const uint32_t b = mb_bits[k];
        const uint64_t off = 4 + 4 * (k / 16 + 1) + (uint64_t)mb_off[k];
        if ((k & 15) == 0 && lane < 4) {
            uint32_t h = 0;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const uint64_t kk = k + 4 * lane + q;
                const uint32_t bb = kk < nmb ? mb_bits[kk] : 0u;
                h |= bb << (24 - 8 * q);
            }
            out[4 + 4 * (k / 16) + (uint64_t)(k == 0 ? 0 : mb_off[k]) + lane] = h;
        }
        uint4 cur, prev;
        load_vectors(in, k, cur, prev);
        if (b == 32) {
            reinterpret_cast<uint4 *>(out + off)[lane] = cur;
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
                const uint32_t d = comp(s_d[wib][j], l);
                const int sh = (int)(j * b) - (int)bit0;
                word |= sh >= 0 ? (d << sh) : (d >> (-sh));
            }
            out[off + idx] = word;
        }
        __syncwarp();
    }
}

// Header words and the VariableByte tail; total words -> scal[CS_WORDS].
__global__ void k_enc_tail(const uint32_t *in, uint64_t *scal, const uint32_t *payload_total, uint32_t *out)
{
    __shared__ uint32_t s_val[128];
    __shared__ uint32_t s_bytes[(128 * 5 + 3) / 4 + 1];
    if (scal[CS_RAW]) return;
    const uint64_t n = scal[CS_N], n1 = scal[CS_N1], nmb = scal[CS_NMB];
    const uint64_t ngroups = (nmb + 15) / 16;
    const uint64_t blkend = 4 + 4 * ngroups + (nmb ? (uint64_t)*payload_total : 0);
    const int lane = threadIdx.x;
    const uint32_t nt = (uint32_t)(n - n1);
    for (uint32_t i = lane; i < nt; i += 32) s_val[i] = in[n1 + i];
    for (uint32_t i = lane; i < sizeof(s_bytes) / 4; i += 32) s_bytes[i] = 0;
    __syncwarp();
    if (lane == 0) {
        out[0] = (uint32_t)n1;
        out[1] = kCookie;
        out[2] = kCookie;
        out[3] = kCookie;
        uint8_t *bb = reinterpret_cast<uint8_t *>(s_bytes);
        uint32_t p = 0, prev = 0;
        for (uint32_t i = 0; i < nt; ++i) {
            uint32_t v = s_val[i] - prev;
            prev = s_val[i];
            while (v >= 128u) {
                bb[p++] = (uint8_t)(v & 127u);
                v >>= 7;
            }
            bb[p++] = (uint8_t)(v | 128u);
        }
        const uint32_t tw = (p + 3) / 4;
        s_val[0] = tw;
        scal[CS_WORDS] = blkend + tw;
        scal[CS_BLKEND] = blkend;
    }
    __syncwarp();
    const uint32_t tw = s_val[0];
    for (uint32_t i = lane; i < tw; i += 32) out[blkend + i] = s_bytes[i];
}

// ---- decoder ---------------------------------------------------------------------------

__global__ void k_dec_prep(const uint32_t *in, const uint64_t *words_dev, uint64_t cap, uint64_t raw_thr,
                           const uint64_t *n_expect, uint64_t *scal, int lift_levels, uint64_t max_vec,
                           uint64_t max_mb)
{
    if (threadIdx.x) return;
    const uint64_t words = *words_dev;
    scal[CS_ERR] = 0;
    scal[CS_WORDS] = words;
    // plugin semantics: raw when n <= thr or the stream is as long as n
    // (cpu_2d/compression/cpusimd.hh:169-173)
    if (raw_thr && n_expect) {
        const uint64_t ne = *n_expect;
        if (ne <= raw_thr || words == ne) {
            scal[CS_RAW] = 1;
            scal[CS_N] = words;
            if (words > cap) scal[CS_ERR] |= G5_DEVERR_CORRUPT;
            return;
        }
    }
    scal[CS_RAW] = 0;
    uint64_t err = 0;
    uint64_t n1 = 0;
    if (words < 4) err = 1;
    else {
        n1 = in[0];
        if (in[1] != kCookie || in[2] != kCookie || in[3] != kCookie) err = 1;
        if (n1 % 128 || n1 > cap || n1 / 128 >= max_mb) err = 1;
    }
    const uint64_t nmb = err ? 0 : n1 / 128;
    const uint64_t ng = (nmb + 15) / 16;
    const uint64_t nv = words / 4;
    if (nv > max_vec) err = 1;
    int R = 0;
    while (((uint64_t)1 << R) < ng + 1) ++R;
    if (R > lift_levels) err = 1;
    scal[CS_N1] = err ? 0 : n1;
    scal[CS_NMB] = err ? 0 : nmb;
    scal[CS_NG] = err ? 0 : ng;
    scal[CS_NV] = nv;
    scal[CS_LIFT] = R;
    scal[CS_N] = 0;
    if (err) scal[CS_ERR] |= G5_DEVERR_CORRUPT;
}

// jump[i] = vector index after a group whose header is vector i (16 widths).
__global__ void __launch_bounds__(kB) k_dec_jump(const uint32_t *in, const uint64_t *scal, uint32_t *jump)
{
    if (scal[CS_RAW] || scal[CS_ERR] || scal[CS_NG] < 2) return;
    const uint64_t nv = scal[CS_NV];
    const uint32_t sink = (uint32_t)nv + 1;
    const uint4 *v = reinterpret_cast<const uint4 *>(in);
    for (uint64_t i = (uint64_t)blockIdx.x * kB + threadIdx.x; i <= nv + 1; i += (uint64_t)gridDim.x * kB) {
        uint32_t j = sink;
        if (i < nv) {
            const uint4 h = v[i];
            const uint32_t hw[4] = {h.x, h.y, h.z, h.w};
            uint32_t s = 0;
            bool ok = true;
#pragma unroll
            for (int q = 0; q < 4; ++q)
#pragma unroll
                for (int by = 0; by < 4; ++by) {
                    const uint32_t b = (hw[q] >> (8 * by)) & 0xFF;
                    ok &= b <= 32;
                    s += b;
                }
            if (ok && i + 1 + s <= nv) j = (uint32_t)(i + 1 + s);
        }
        jump[i] = j;
    }
}

__global__ void __launch_bounds__(kB) k_dec_lift(const uint64_t *scal, uint32_t *jump, uint64_t stride, int r)
{
    if (scal[CS_RAW] || scal[CS_ERR] || scal[CS_NG] < 2 || (uint64_t)r + 1 >= scal[CS_LIFT]) return;
    const uint64_t nv = scal[CS_NV];
    const uint32_t *t = jump + stride * r;
    uint32_t *t1 = jump + stride * (r + 1);
    for (uint64_t i = (uint64_t)blockIdx.x * kB + threadIdx.x; i <= nv + 1; i += (uint64_t)gridDim.x * kB)
        t1[i] = t[t[i]];
}

__global__ void __launch_bounds__(kB) k_dec_pos(const uint32_t *in, uint64_t *scal, const uint32_t *jump,
                                                uint64_t stride, uint32_t *gpos)
{
    if (scal[CS_RAW] || scal[CS_ERR]) return;
    const uint64_t ng = scal[CS_NG], nv = scal[CS_NV], nmb = scal[CS_NMB];
    const int R = (int)scal[CS_LIFT];
    for (uint64_t g = (uint64_t)blockIdx.x * kB + threadIdx.x; g < ng; g += (uint64_t)gridDim.x * kB) {
        uint64_t pos = 1;
        for (int r = 0; r < R && pos < nv; ++r)
            if ((g >> r) & 1) pos = jump[stride * r + pos];
        if (ng < 2) pos = 1;
        if (pos >= nv) {
            atomicOr((unsigned long long *)&scal[CS_ERR], (unsigned long long)G5_DEVERR_CORRUPT);
            pos = 0;
        }
        gpos[g] = (uint32_t)pos;
        if (g == ng - 1 && pos) {
            // the last group only holds `howmany` miniblocks
            const uint64_t howmany = nmb - 16 * g;
            const uint4 h = reinterpret_cast<const uint4 *>(in)[pos];
            const uint32_t hw[4] = {h.x, h.y, h.z, h.w};
            uint64_t s = 0;
            bool ok = true;
            for (uint64_t i = 0; i < howmany; ++i) {
                const uint32_t b = (hw[i / 4] >> (24 - 8 * (i % 4))) & 0xFF;
                ok &= b <= 32;
                s += b;
            }
            const uint64_t end = pos + 1 + s;
            if (!ok || end > nv)
                atomicOr((unsigned long long *)&scal[CS_ERR], (unsigned long long)G5_DEVERR_CORRUPT);
            else
                scal[CS_BLKEND] = 4 * end;
        }
    }
    if (ng == 0 && blockIdx.x == 0 && threadIdx.x == 0) scal[CS_BLKEND] = 4;
}

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

__global__ void __launch_bounds__(kB) k_dec_sum(const uint32_t *in, const uint64_t *scal, const uint32_t *gpos,
                                                VecFlag *mb_sf, int mode)
{
    if (scal[CS_RAW] || scal[CS_ERR]) return;
    const uint64_t nmb = scal[CS_NMB];
    const uint64_t gw = ((uint64_t)blockIdx.x * kB + threadIdx.x) >> 5;
    const uint64_t nw = ((uint64_t)gridDim.x * kB) >> 5;
    for (uint64_t k = gw; k < nmb; k += nw) {
        uint64_t off;
        uint32_t b;
        mb_locate(in, gpos, k, off, b);
        uint4 d = unpack_vec(in, off, b);
        VecFlag r;
        if (b == 32) {
            r.v.x = __shfl_sync(0xFFFFFFFFu, d.x, 31);
            r.v.y = __shfl_sync(0xFFFFFFFFu, d.y, 31);
            r.v.z = __shfl_sync(0xFFFFFFFFu, d.z, 31);
            r.v.w = __shfl_sync(0xFFFFFFFFu, d.w, 31);
            r.f = 1;
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
            r.f = 0;
        }
        if (g5_lane() == 0) mb_sf[k] = r;
    }
}

__global__ void __launch_bounds__(kB) k_dec_out(const uint32_t *in, uint64_t *scal, const uint32_t *gpos,
                                                const VecFlag *mb_base, uint32_t *out, const uint32_t *expect,
                                                int mode)
{
    if (scal[CS_RAW]) {
        const uint64_t n = scal[CS_N];
        if (scal[CS_ERR]) return;
        for (uint64_t i = (uint64_t)blockIdx.x * kB + threadIdx.x; i < n; i += (uint64_t)gridDim.x * kB) {
            out[i] = in[i];
            if (expect && expect[i] != in[i])
                atomicOr((unsigned long long *)&scal[CS_ERR], (unsigned long long)G5_DEVERR_MISMATCH);
        }
        return;
    }
    if (scal[CS_ERR]) return;
    const uint64_t nmb = scal[CS_NMB];
    const int lane = g5_lane();
    const uint64_t gw = ((uint64_t)blockIdx.x * kB + threadIdx.x) >> 5;
    const uint64_t nw = ((uint64_t)gridDim.x * kB) >> 5;
    bool bad = false;
    for (uint64_t k = gw; k < nmb; k += nw) {
        uint64_t off;
        uint32_t b;
        mb_locate(in, gpos, k, off, b);
        uint4 d = unpack_vec(in, off, b);
        const uint4 base = mb_base[k].v;
        uint4 x;
        if (b == 32) {
            x = d;
        } else if (mode == G5_CODEC_DM) {
            uint32_t c = d.w;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                uint32_t y = __shfl_up_sync(0xFFFFFFFFu, c, o);
                if (lane >= o) c += y;
            }
            c += base.w;
            uint32_t pc = __shfl_up_sync(0xFFFFFFFFu, c, 1);
            if (lane == 0) pc = base.w;
            x = make_uint4(d.x + pc, d.y + pc, d.z + pc, c);
        } else {
            uint32_t cx = d.x, cy = d.y, cz = d.z, cw = d.w;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                uint32_t yx = __shfl_up_sync(0xFFFFFFFFu, cx, o);
                uint32_t yy = __shfl_up_sync(0xFFFFFFFFu, cy, o);
                uint32_t yz = __shfl_up_sync(0xFFFFFFFFu, cz, o);
                uint32_t yw = __shfl_up_sync(0xFFFFFFFFu, cw, o);
                if (lane >= o) {
                    cx += yx;
                    cy += yy;
                    cz += yz;
                    cw += yw;
                }
            }
            x = make_uint4(cx + base.x, cy + base.y, cz + base.z, cw + base.w);
        }
        reinterpret_cast<uint4 *>(out)[k * 32 + lane] = x;
        if (expect) {
            const uint4 e = reinterpret_cast<const uint4 *>(expect)[k * 32 + lane];
            bad |= (e.x != x.x) | (e.y != x.y) | (e.z != x.z) | (e.w != x.w);
        }
    }
    if (bad) atomicOr((unsigned long long *)&scal[CS_ERR], (unsigned long long)G5_DEVERR_MISMATCH);
}

__global__ void k_dec_tail(const uint32_t *in, uint64_t *scal, uint64_t cap, uint32_t *out,
                           const uint64_t *n_expect, const uint32_t *expect, uint64_t *acc)
{
    __shared__ uint32_t s_b[kTailMaxBytes / 4];
    const int lane = threadIdx.x;
    if (scal[CS_RAW]) {
        if (lane == 0) {
            if (n_expect && scal[CS_N] != *n_expect) scal[CS_ERR] |= G5_DEVERR_MISMATCH;
            if (acc) {
                acc[0] += scal[CS_WORDS];
                acc[1] += scal[CS_N];
            }
        }
        return;
    }
    if (scal[CS_ERR]) return;
    const uint64_t words = scal[CS_WORDS], blkend = scal[CS_BLKEND], n1 = scal[CS_N1];
    const uint64_t tw = words > blkend ? words - blkend : 0;
    if (tw * 4 > kTailMaxBytes) {
        if (lane == 0) scal[CS_ERR] |= G5_DEVERR_CORRUPT;
        return;
    }
    for (uint64_t i = lane; i < tw; i += 32) s_b[i] = in[blkend + i];
    __syncwarp();
    if (lane == 0) {
        const uint8_t *bb = reinterpret_cast<const uint8_t *>(s_b);
        uint64_t o = n1;
        uint32_t prev = 0, v = 0;
        int shift = 0;
        uint64_t err = 0;
        for (uint64_t p = 0; p < tw * 4; ++p) {
            const uint32_t c = bb[p];
            v |= (c & 127u) << shift;
            if (c & 128u) {
                if (o >= cap) {
                    err |= G5_DEVERR_CORRUPT;
                    break;
                }
                prev += v;
                out[o] = prev;
                if (expect && expect[o] != prev) err |= G5_DEVERR_MISMATCH;
                ++o;
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
        scal[CS_N] = o;
        if (n_expect && o != *n_expect) err |= G5_DEVERR_MISMATCH;
        scal[CS_ERR] |= err;
        if (acc) {
            acc[0] += words;
            acc[1] += o;
        }
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

int lift_levels_for(size_t max_n)
{
    const size_t ng = (max_n / 128 + 15) / 16;
    int R = 0;
    while (((size_t)1 << R) < ng + 1) ++R;
    return R < 1 ? 1 : R;
}

}  // namespace

size_t codec_bound(size_t n)
{
    const size_t mb = n / 128;
    return 4 + 4 * (mb / 16 + 1) + mb * 128 + ((n % 128) * 5 + 3) / 4 + 8;
}

g5_status codec_work_alloc(CodecWork &w, size_t max_n)
{
    w.max_n = max_n;
    w.max_mb = max_n / 128 + 1;
    w.max_vec = codec_bound(max_n) / 4 + 2;
    w.lift_levels = lift_levels_for(max_n);
    w.grid = num_sms() * 4;
    G5_CUDA(cudaMalloc(&w.mb_len, sizeof(uint32_t) * w.max_mb));
    G5_CUDA(cudaMalloc(&w.mb_bits, w.max_mb));
    G5_CUDA(cudaMalloc(&w.jump, sizeof(uint32_t) * (w.max_vec + 2) * (size_t)w.lift_levels));
    G5_CUDA(cudaMalloc(&w.gpos, sizeof(uint32_t) * (w.max_mb / 16 + 2)));
    G5_CUDA(cudaMalloc(&w.mb_sum, sizeof(VecFlag) * w.max_mb));
    G5_CUDA(cudaMalloc(&w.mb_base, sizeof(VecFlag) * w.max_mb));
    w.mb_flag = nullptr;
    G5_CUDA(cudaMalloc(&w.part, sizeof(VecFlag) * (size_t)(w.grid + 1)));
    G5_CUDA(cudaMalloc(&w.scal, sizeof(uint64_t) * 16));
    G5_CUDA(cudaMemset(w.scal, 0, sizeof(uint64_t) * 16));
    return G5_OK;
}

void codec_work_free(CodecWork &w)
{
    cudaFree(w.mb_len);
    cudaFree(w.mb_bits);
    cudaFree(w.jump);
    cudaFree(w.gpos);
    cudaFree(w.mb_sum);
    cudaFree(w.mb_base);
    cudaFree(w.part);
    cudaFree(w.scal);
    w = CodecWork();
}

void codec_encode_launch(CodecWork &w, const uint32_t *in, const uint64_t *n_dev, uint32_t *out, int mode,
                         uint64_t raw_threshold, cudaStream_t s)
{
    k_enc_prep<<<1, 32, 0, s>>>(n_dev, raw_threshold, w.scal);
    k_enc_bits<<<w.grid, kB, 0, s>>>(in, w.scal, w.mb_bits, w.mb_len, mode);
    uint32_t *part = reinterpret_cast<uint32_t *>(w.part);
    k_scan_red<AddU32><<<w.grid, kB, 0, s>>>(w.mb_len, w.scal + CS_NMB, part);
    k_scan_top<AddU32><<<1, kB, 0, s>>>(part, w.grid, part + w.grid);
    k_scan_down<AddU32><<<w.grid, kB, 0, s>>>(w.mb_len, w.mb_len, w.scal + CS_NMB, part);
    k_enc_pack<<<w.grid, kB, 0, s>>>(in, w.scal, w.mb_bits, w.mb_len, out, mode);
    k_enc_tail<<<1, 32, 0, s>>>(in, w.scal, part + w.grid, out);
}

void codec_decode_launch(CodecWork &w, const uint32_t *in, const uint64_t *words_dev, uint32_t *out, size_t cap,
                         int mode, uint64_t raw_threshold, const uint64_t *n_expect_dev, const uint32_t *expect,
                         cudaStream_t s)
{
    decode_launch_acc(w, in, words_dev, out, cap, mode, raw_threshold, n_expect_dev, expect, nullptr, s);
}

void decode_launch_acc(CodecWork &w, const uint32_t *in, const uint64_t *words_dev, uint32_t *out, size_t cap,
                       int mode, uint64_t raw_threshold, const uint64_t *n_expect_dev, const uint32_t *expect,
                       uint64_t *acc, cudaStream_t s)
{
    const uint64_t stride = w.max_vec + 2;
    k_dec_prep<<<1, 32, 0, s>>>(in, words_dev, cap, raw_threshold, n_expect_dev, w.scal, w.lift_levels,
                                 w.max_vec, w.max_mb);
    k_dec_jump<<<w.grid, kB, 0, s>>>(in, w.scal, w.jump);
    for (int r = 0; r + 1 < w.lift_levels; ++r) k_dec_lift<<<w.grid, kB, 0, s>>>(w.scal, w.jump, stride, r);
    k_dec_pos<<<w.grid, kB, 0, s>>>(in, w.scal, w.jump, stride, w.gpos);
    VecFlag *sf = reinterpret_cast<VecFlag *>(w.mb_sum);
    VecFlag *base = reinterpret_cast<VecFlag *>(w.mb_base);
    VecFlag *part = reinterpret_cast<VecFlag *>(w.part);
    k_dec_sum<<<w.grid, kB, 0, s>>>(in, w.scal, w.gpos, sf, mode);
    k_scan_red<ResetAdd><<<w.grid, kB, 0, s>>>(sf, w.scal + CS_NMB, part);
    k_scan_top<ResetAdd><<<1, kB, 0, s>>>(part, w.grid, nullptr);
    k_scan_down<ResetAdd><<<w.grid, kB, 0, s>>>(sf, base, w.scal + CS_NMB, part);
    k_dec_out<<<w.grid, kB, 0, s>>>(in, w.scal, w.gpos, base, out, expect, mode);
    k_dec_tail<<<1, 32, 0, s>>>(in, w.scal, cap, out, n_expect_dev, expect, acc);
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
    if (c->h_scal[g5::CS_ERR]) return G5_ERR_CORRUPT_STREAM;
    *out_n = (size_t)c->h_scal[g5::CS_N];
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
    const int grid = c->w.grid;
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
    const int grid = c->w.grid;
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
// scratch (bit widths, payload offsets, scan partials, length scalars) lives
// in the file-scope array below instead of a g5_codec workspace: 57,741
// bytes (about 56 KiB, kNoAllocBytes) that every GPU which loads the library
// holds until the process exits.  The array's device address is looked up
// once per device and cached for the life of the process, so the entry point
// must not be used again on a device after cudaDeviceReset in the same
// process (the reset frees the module that holds the array).

namespace {

constexpr size_t kNoAllocMaxValues = (size_t)1 << 20;          // values per call
constexpr size_t kNoAllocMb = kNoAllocMaxValues / 128 + 1;       // miniblocks
constexpr size_t kNoAllocParts = 4096;                           // scan partials
constexpr size_t kNoAllocBytes = 128 + 8 + kNoAllocMb * 4 + kNoAllocMb + kNoAllocParts * 4 + 256;
static_assert(kNoAllocBytes == 57741, "the documented size of the scratch array");

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
    w.grid = std::min(g5::num_sms() * 4, (int)kNoAllocParts - 1);
    w.scal = reinterpret_cast<uint64_t *>(b);                        // 16 scalars
    uint64_t *n_dev = reinterpret_cast<uint64_t *>(b + 128);
    w.mb_len = reinterpret_cast<uint32_t *>(b + 136);
    w.mb_bits = reinterpret_cast<uint8_t *>(b + 136 + kNoAllocMb * 4);
    const size_t off_part = (136 + 5 * kNoAllocMb + 7) & ~(size_t)7;
    static_assert(((136 + 5 * kNoAllocMb + 7) & ~(size_t)7) + kNoAllocParts * 4 <= kNoAllocBytes,
                  "scratch layout exceeds the static array");
    w.part = reinterpret_cast<uint64_t *>(b + off_part);
    cudaStream_t s = (cudaStream_t)stream;
    uint64_t hn = n;
    // every scratch word the encoder reads is written earlier in the same
    // call (k_enc_prep resets the scalars), so nothing needs clearing here
    G5_CUDA(cudaMemcpyAsync(n_dev, &hn, sizeof hn, cudaMemcpyHostToDevice, s));
    g5::codec_encode_launch(w, in_dev, n_dev, out_dev, mode, 0, s);
    G5_CUDA(cudaGetLastError());
    uint64_t words = 0;
    G5_CUDA(cudaMemcpyAsync(&words, w.scal + g5::CS_WORDS, sizeof words, cudaMemcpyDeviceToHost, s));
    G5_CUDA(cudaStreamSynchronize(s));
    *out_words = (size_t)words;
    return G5_OK;
}
