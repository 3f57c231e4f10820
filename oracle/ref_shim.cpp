// ref_shim.cpp -- TEST INFRASTRUCTURE: exposes the reference encoder itself
// (goofy::compressDXT1 / goofy::compressETC1 from GoofyTC/goofy_tc.h, included
// from the reference tree by oracle/build.py via -I; nothing is copied) with C
// linkage so tests and the golden-vector script can call it through ctypes,
// together with the harness's block decoders and its PNG loader (lodepng,
// ThirdParty/lodepng, also compiled from where it lies).
// It is compiled in the Release configuration (-DNDEBUG) the reference harness
// ships with; a debug build asserts 64-byte aligned strips (goofy_tc.h:1072).
// goofy_tc.h defines its functions non-inline (goofy_tc.h:34), so it is
// included in this one translation unit only.
// Built a second time with GOOFY_REF_ENCODER_ONLY from the header copy that
// oracle/build.py generates without goofy_tc.h:16 (the reference's scalar
// path, for hosts without SSE2): the encoder entry points only.
#include "goofy_tc.h"

#ifndef GOOFY_REF_ENCODER_ONLY
#include "decoder.h"
#include "lodepng.h"
#endif

#include <thread>
#include <vector>

extern "C" int ref_compress(int codec, unsigned char* result, const unsigned char* input,
                            unsigned width, unsigned height, unsigned stride)
{
    return codec == 0 ? goofy::compressDXT1(result, input, width, height, stride)
                      : goofy::compressETC1(result, input, width, height, stride);
}

// The reference striped by block rows over `threads` std::threads, each calling
// the reference entry point on its slice of rows (the %16 / %4 rules hold per
// slice).  Returns the thread count used or the reference's error code.
extern "C" int ref_compress_mt(int codec, unsigned char* result, const unsigned char* input,
                               unsigned width, unsigned height, unsigned stride, int threads)
{
    if (width % 16 != 0) return -1;
    if (height % 4 != 0) return -2;
    if (threads <= 0) threads = (int)std::thread::hardware_concurrency();
    const unsigned bh = height / 4;
    if (threads < 1) threads = 1;
    if ((unsigned)threads > bh) threads = bh ? (int)bh : 1;
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t) {
        const unsigned b0 = (unsigned)((unsigned long long)bh * t / threads);
        const unsigned b1 = (unsigned)((unsigned long long)bh * (t + 1) / threads);
        pool.emplace_back([=] {
            ref_compress(codec, result + (size_t)b0 * (width / 4) * 8, input + (size_t)b0 * 4 * stride,
                         width, (b1 - b0) * 4, stride);
        });
    }
    for (auto& th : pool) th.join();
    return threads;
}

#ifndef GOOFY_REF_ENCODER_ONLY
// The reference harness's block decoders (Src/decoder.cpp:933-971): one
// block into 16 RGBA8 pixels, 16-byte rows.
extern "C" void ref_decode_block(int codec, const unsigned char* blk, unsigned char* out64)
{
    if (codec == 0) DecoderBC::decodeBlockDXT1(blk, out64, 16);
    else DecoderBC::decodeBlockETC1(blk, out64, 16);
}

// The harness's PNG loader core (Src/main.cpp:270: lodepng::decode to 8-bit
// RGBA, from memory here).  Returns lodepng's error code; on success `out`
// (caller-sized by ref_png_size) receives width*height*4 bytes.
extern "C" unsigned ref_png_decode(const unsigned char* png, size_t n, unsigned char* out, size_t out_bytes,
                                   unsigned* w, unsigned* h)
{
    std::vector<unsigned char> img;
    const unsigned err = lodepng::decode(img, *w, *h, png, n);
    if (err) return err;
    if (img.size() > out_bytes) return 1000;
    std::copy(img.begin(), img.end(), out);
    return 0;
}
#endif  // GOOFY_REF_ENCODER_ONLY
