// block_codec_host.cpp -- TEST ONLY.  Compiles goofy_gb300/csrc/block_codec.cuh
// and block_decode.cuh for the CPU (through host_emulation.h) and exposes the
// per-block encoders and decoders over a whole image, so tests can compare the
// kernels' arithmetic with the oracle without a GPU.  Not linked into the
// library.
#include <cstring>

#include "block_codec.cuh"
#include "block_decode.cuh"

// codec 0: BC1, 1: ETC1s, 2: both from encode_both (BC1 blocks at `out`, the
// ETC1s blocks right after them).
extern "C" int host_emu_encode(int codec, uint8_t* out, const uint8_t* src, unsigned width, unsigned height,
                               unsigned stride)
{
    if (width % 4 || height % 4) return -1;
    uint8_t lut[128];
    for (uint32_t i = 0; i < 128; ++i) lut[i] = (uint8_t)goofy_gpu::etc_control_byte(2 * i);
    const unsigned bw = width / 4, bh = height / 4;
    for (unsigned by = 0; by < bh; ++by)
        for (unsigned bx = 0; bx < bw; ++bx) {
            uint32_t w[16];
            for (int y = 0; y < 4; ++y)
                std::memcpy(&w[4 * y], src + (size_t)(4 * by + y) * stride + 16 * (size_t)bx, 16);
            uint8_t* o = out + 8 * ((size_t)by * bw + bx);
            if (codec == 2) {
                const uint4 r = goofy_gpu::encode_both(w, lut);
                uint8_t* o2 = o + 8 * (size_t)bw * bh;
                std::memcpy(o, &r.x, 4);
                std::memcpy(o + 4, &r.y, 4);
                std::memcpy(o2, &r.z, 4);
                std::memcpy(o2 + 4, &r.w, 4);
                continue;
            }
            const uint2 r = codec == 0 ? goofy_gpu::encode_bc1(w) : goofy_gpu::encode_etc1s(w, lut);
            std::memcpy(o, &r.x, 4);
            std::memcpy(o + 4, &r.y, 4);
        }
    return 0;
}

// Decodes (width/4)*(height/4) blocks into RGBA rows of `stride` bytes; returns
// the number of unsupported blocks.
extern "C" long host_emu_decode(int codec, const uint8_t* blocks, unsigned width, unsigned height, uint8_t* rgba,
                                unsigned stride)
{
    const unsigned bw = width / 4, bh = height / 4;
    long bad = 0;
    uint32_t store[8];
    for (unsigned by = 0; by < bh; ++by)
        for (unsigned bx = 0; bx < bw; ++bx) {
            uint2 blk;
            std::memcpy(&blk.x, blocks + 8 * ((size_t)by * bw + bx), 4);
            std::memcpy(&blk.y, blocks + 8 * ((size_t)by * bw + bx) + 4, 4);
            uint32_t px[16];
            const bool ok = codec == 0 ? goofy_gpu::decode_block<goofy_gpu::kBC1>(blk, store, 1, px)
                                       : goofy_gpu::decode_block<goofy_gpu::kETC1S>(blk, store, 1, px);
            bad += ok ? 0 : 1;
            for (int y = 0; y < 4; ++y)
                std::memcpy(rgba + (size_t)(4 * by + y) * stride + 16 * (size_t)bx, &px[4 * y], 16);
        }
    return bad;
}
