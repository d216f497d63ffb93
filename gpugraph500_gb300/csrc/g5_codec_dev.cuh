// g5_codec_dev.cuh -- device-resident s4-bp128 codec pipeline, callable from
// a BFS level loop (lengths live in device memory, grids are fixed, so the
// launches can be captured in a CUDA graph).
#pragma once

#include <cstdint>

#include "g5_common.cuh"

namespace g5 {

// Four running lane sums and a reset flag (a raw miniblock restarts the sums).
struct VecFlag {
    uint4 v;
    uint32_t f;
};

struct CodecWork {
    size_t max_n = 0;        // capacity in values
    size_t max_mb = 0;       // miniblocks
    size_t max_vec = 0;      // 16-byte vectors of the largest stream
    int grid = 0;            // blocks of the fixed grid
    uint64_t *scal = nullptr;  // device scalars (kScalars), see CodecScalar
    uint32_t *gpos = nullptr;  // decoder: vector index of each group header
    // encoder: bit width of every miniblock (16-byte aligned, a group's 16
    // widths one vector) and the word count of each encoder block's range
    uint8_t *ewb = nullptr;
    uint64_t *etot = nullptr;
    int enc_blocks = 0;        // encoder blocks (entries of etot)
    // decoder group locator: per chunk a transfer table and the real entry,
    // per stream vector its jump
    uint32_t *ltab = nullptr;
    uint64_t *lent = nullptr;
    uint16_t *ljump = nullptr;
    // decoder unpacker look-back: status, aggregate and inclusive lane sums per group
    uint64_t *ust = nullptr;
    VecFlag *uagg = nullptr, *uinc = nullptr;
};

enum CodecScalar {
    CS_N = 0,       // values to encode / decoded value count
    CS_WORDS = 1,   // encoded words
    CS_ERR = 2,     // error bits (G5_DEVERR_*)
    CS_N1 = 3,      // values in the block part
    CS_BLKEND = 4,  // word index where the block part ends
    CS_COUNT = 8
};

constexpr int kScalars = 32;  // scalar slots of a CodecWork

// Groups (look-back tiles of the unpacker) and locate chunks a workspace
// for max_n values needs, and the fixed grid of the codec kernels.
size_t codec_tiles(size_t max_n);
size_t codec_chunks(size_t max_n);
int codec_grid();

size_t codec_bound(size_t n);
g5_status codec_work_alloc(CodecWork &w, size_t max_n);
void codec_work_free(CodecWork &w);

// Encode in[0 .. *n_dev) to out; words written -> w.scal[CS_WORDS] and, if
// words_out is given, *words_out.  raw_threshold: if *n_dev <= raw_threshold,
// a raw copy (plugin semantics); pass 0 for pure IntegerCODEC semantics.
void codec_encode_launch(CodecWork &w, const uint32_t *in, const uint64_t *n_dev, uint32_t *out,
                         int mode, uint64_t raw_threshold, cudaStream_t s, uint64_t *words_out = nullptr);

// Decode in[0 .. *words_dev) to out (capacity cap); values -> w.scal[CS_N].
// If expect != nullptr, each decoded value is compared with expect[i] and
// *n_expect_dev with the decoded count; a difference sets G5_DEVERR_MISMATCH.
// raw_threshold as for encode (raw when n <= thr or words == n), with
// *n_expect_dev giving the original length.  If n_out is given, the value
// count is also written there.
void codec_decode_launch(CodecWork &w, const uint32_t *in, const uint64_t *words_dev, uint32_t *out,
                         size_t cap, int mode, uint64_t raw_threshold, const uint64_t *n_expect_dev,
                         const uint32_t *expect, cudaStream_t s, uint64_t *n_out = nullptr);

// As codec_decode_launch; if acc != nullptr, acc[0] += words and
// acc[1] += decoded values (running totals kept on the device).
void decode_launch_acc(CodecWork &w, const uint32_t *in, const uint64_t *words_dev, uint32_t *out, size_t cap,
                       int mode, uint64_t raw_threshold, const uint64_t *n_expect_dev, const uint32_t *expect,
                       uint64_t *acc, cudaStream_t s, uint64_t *n_out = nullptr);

}  // namespace g5
