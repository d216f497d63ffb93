// ref_codec.cpp -- exposes the reference's vendored SIMD codec library and its
// CpuSimd plugin (compiled unmodified from the gpugraph500 tree) to the
// golden-vector script.
//
// TEST INFRASTRUCTURE ONLY (built into oracle/_ref, never into the product).
// cpu_2d/compression/cpusimd.hh:70-173 (plugin),
// cpu_2d/compression/cpusimd/include/codecfactory.h:103-108 (codecs).
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <string>

#include "codecfactory.h"
#include "compression/cpusimd.hh"

using namespace SIMDCompressionLib;

namespace {
uint32_t *aligned_words(size_t n)
{
    void *p = nullptr;
    if (posix_memalign(&p, 16, (n + 4) * sizeof(uint32_t))) return nullptr;
    std::memset(p, 0, (n + 4) * sizeof(uint32_t));
    return (uint32_t *)p;
}
}  // namespace

extern "C" {

// IntegerCODEC::encodeArray of the named codec; returns words written.
size_t ref_codec_encode(const char *name, const uint32_t *in, size_t n, uint32_t *out, size_t cap)
{
    IntegerCODEC &c = *CODECFactory::getFromName(name);
    uint32_t *a = aligned_words(n);
    uint32_t *o = aligned_words(cap);
    std::memcpy(a, in, n * sizeof(uint32_t));
    size_t nv = cap;
    c.encodeArray(a, n, o, nv);
    std::memcpy(out, o, nv * sizeof(uint32_t));
    free(a);
    free(o);
    return nv;
}

// IntegerCODEC::decodeArray of the named codec; returns values written.
size_t ref_codec_decode(const char *name, const uint32_t *in, size_t words, uint32_t *out, size_t n)
{
    IntegerCODEC &c = *CODECFactory::getFromName(name);
    uint32_t *a = aligned_words(words);
    uint32_t *o = aligned_words(n + 256);
    std::memcpy(a, in, words * sizeof(uint32_t));
    size_t nv = n;
    c.decodeArray(a, words, o, nv);
    std::memcpy(out, o, nv * sizeof(uint32_t));
    free(a);
    free(o);
    return nv;
}

// The plugin exactly as the reference driver configures it: construct,
// reconfigure(thr, codec) (cpu_2d/main.cpp:300-301), compress.  The output
// buffer the plugin allocates holds only n words (cpusimd.hh:80), so callers
// pass inputs that compress.  Returns compressedsize.
size_t ref_plugin_compress(int thr, const char *codec, const int64_t *in, size_t n, uint32_t *out)
{
    CpuSimd<int64_t, uint32_t> p;
    p.reconfigure(thr, codec);
    int64_t *a = nullptr;
    if (posix_memalign((void **)&a, 16, (n + 2) * sizeof(int64_t))) return 0;
    std::memcpy(a, in, n * sizeof(int64_t));
    uint32_t *c = nullptr;
    size_t cs = 0;
    p.compress(a, n, &c, cs);
    std::memcpy(out, c, cs * sizeof(uint32_t));
    free(c);
    free(a);
    return cs;
}

size_t ref_plugin_decompress(int thr, const char *codec, const uint32_t *in, size_t words, size_t n, int64_t *out)
{
    CpuSimd<int64_t, uint32_t> p;
    p.reconfigure(thr, codec);
    uint32_t *a = nullptr;
    if (posix_memalign((void **)&a, 16, (words + 4) * sizeof(uint32_t))) return 0;
    std::memcpy(a, in, words * sizeof(uint32_t));
    int64_t *u = nullptr;
    size_t us = n;
    p.decompress(a, (int)words, &u, us);
    std::memcpy(out, u, us * sizeof(int64_t));
    free(u);
    free(a);
    return us;
}

}  // extern "C"
