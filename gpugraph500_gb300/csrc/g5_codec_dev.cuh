// g5_codec_dev.cuh -- device-resident s4-bp128 codec pipeline, callable from
// a BFS level loop (lengths live in device memory, grids are fixed, so the
// launches can be captured in a CUDA graph).
#pragma once

#include <cstdint>

#include "g5_common.cuh"

namespace g5 {

struct CodecWork {
    size_t max_n = 0;        // capacity in values
    size_t max_mb = 0;       // miniblocks
    size_t max_vec = 0;      // 16-byte vectors of the largest stream
    int lift_levels = 0;     // binary-lifting tables
    int grid = 0;            // blocks of the fixed grid
    // encoder
    uint32_t *mb_len = nullptr;    // 4*b per miniblock, then exclusive prefix
    uint8_t *mb_bits = nullptr;    // b per miniblock
    // decoder
    uint32_t *jump = nullptr;      // lift_levels tables of max_vec + 1 entries
    uint32_t *gpos = nullptr;      // vector index of each group header
    uint4 *mb_sum = nullptr;       // per miniblock lane sums (or raw last vector)
    uint32_t *mb_flag = nullptr;   // 1 if the miniblock is raw (b == 32)
    uint4 *mb_base = nullptr;      // scanned base vector of each miniblock
    // scan partials and device scalars
    uint64_t *part = nullptr;      // grid * 8 words
    uint64_t *scal = nullptr;      // device scalars, see CodecScalar
};

enum CodecScalar {
    CS_N = 0,       // values to encode / decoded value count
    CS_WORDS = 1,   // encoded words
    CS_ERR = 2,     // error bits (G5_DEVERR_*)
    CS_N1 = 3,      // values in the block part
    CS_BLKEND = 4,  // word index where the block part ends
    CS_COUNT = 8
};

size_t codec_bound(size_t n);
g5_status codec_work_alloc(CodecWork &w, size_t max_n);
void codec_work_free(CodecWork &w);

// Encode in[0 .. *n_dev) to out; words written -> w.scal[CS_WORDS].
// raw_threshold: if *n_dev <= raw_threshold, a raw copy (plugin semantics);
// pass 0 for pure IntegerCODEC semantics.
void codec_encode_launch(CodecWork &w, const uint32_t *in, const uint64_t *n_dev, uint32_t *out,
                         int mode, uint64_t raw_threshold, cudaStream_t s);

// Decode in[0 .. *words_dev) to out (capacity cap); values -> w.scal[CS_N].
// If expect != nullptr, each decoded value is compared with expect[i] and
// *n_expect_dev with the decoded count; a difference sets G5_DEVERR_MISMATCH.
// raw_threshold as for encode (raw when n <= thr or words == n), with
// *n_expect_dev giving the original length.
void codec_decode_launch(CodecWork &w, const uint32_t *in, const uint64_t *words_dev, uint32_t *out,
                         size_t cap, int mode, uint64_t raw_threshold, const uint64_t *n_expect_dev,
                         const uint32_t *expect, cudaStream_t s);

// As codec_decode_launch; if acc != nullptr, acc[0] += words and
// acc[1] += decoded values (running totals kept on the device).
void decode_launch_acc(CodecWork &w, const uint32_t *in, const uint64_t *words_dev, uint32_t *out, size_t cap,
                       int mode, uint64_t raw_threshold, const uint64_t *n_expect_dev, const uint32_t *expect,
                       uint64_t *acc, cudaStream_t s);

}  // namespace g5
