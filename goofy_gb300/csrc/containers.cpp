// containers.cpp -- DDS (BC1) and KTX 1.1 (ETC1) containers for encoded
// blocks.  The reference harness writes one-level files with saveDds /
// saveKtx (Src/main.cpp:154-220); for one level these functions produce the
// same bytes, including the reference's header field choices (DDS flags
// 0x000A1007, caps left 0; KTX glTypeSize 1, GL_RGB base format).  More than
// one level (a mip chain) sets the level count and appends the levels in
// order, each KTX level preceded by its byte size.  The harness's TGA images
// (saveTga, Src/main.cpp:222-255: an 18-byte header, type 2, 32 bits per
// pixel, top-left origin, then BGRA pixels) hold its original, baseline and
// decoded images.
#include <cstring>

#include "../../include/goofy_gpu.h"
#include "host_util.h"

namespace {

constexpr size_t kDdsHeader = 128, kKtxHeader = 64;

void put32(uint8_t* p, uint32_t v)
{
    p[0] = (uint8_t)v;
    p[1] = (uint8_t)(v >> 8);
    p[2] = (uint8_t)(v >> 16);
    p[3] = (uint8_t)(v >> 24);
}

uint64_t level_bytes(uint32_t w, uint32_t h) { return (uint64_t)(w / 4) * (h / 4) * 8; }

}  // namespace

extern "C" {

GOOFY_EXPORT size_t goofy_gpu_container_size(int codec, const uint32_t* widths, const uint32_t* heights,
                                             uint32_t levels)
{
    if ((codec != GOOFY_CODEC_BC1 && codec != GOOFY_CODEC_ETC1S) || !widths || !heights || levels == 0) return 0;
    uint64_t n = codec == GOOFY_CODEC_BC1 ? kDdsHeader : kKtxHeader;
    for (uint32_t i = 0; i < levels; ++i) {
        if (widths[i] % 4 || heights[i] % 4) return 0;
        n += level_bytes(widths[i], heights[i]) + (codec == GOOFY_CODEC_ETC1S ? 4 : 0);
    }
    return (size_t)n;
}

GOOFY_EXPORT int goofy_gpu_write_container(int codec, const uint8_t* const* level_blocks, const uint32_t* widths,
                                           const uint32_t* heights, uint32_t levels, uint8_t* out, size_t out_size)
{
    const size_t need = goofy_gpu_container_size(codec, widths, heights, levels);
    if (need == 0 || !level_blocks || !out) return GOOFY_ERR_INVALID;
    if (out_size < need) return goofy_gpu::fail(GOOFY_ERR_TOO_LARGE, "container: output buffer too small");
    for (uint32_t i = 0; i < levels; ++i)
        if (!level_blocks[i] && level_bytes(widths[i], heights[i])) return GOOFY_ERR_INVALID;
    uint8_t* p = out;
    if (codec == GOOFY_CODEC_BC1) {
        std::memset(p, 0, kDdsHeader);
        put32(p + 0, 0x20534444u);                                   // "DDS "
        put32(p + 4, 124);                                           // header size
        put32(p + 8, 0x000A1007u);                                   // caps | height | width | pixelformat | mipmapcount | linearsize
        put32(p + 12, heights[0]);
        put32(p + 16, widths[0]);
        put32(p + 20, (uint32_t)level_bytes(widths[0], heights[0]));  // linear size of the top level
        put32(p + 24, 1);                                            // depth
        put32(p + 28, levels);                                       // mip map count
        put32(p + 76, 32);                                           // pixel format size
        put32(p + 80, 0x4);                                          // FOURCC
        put32(p + 84, 0x31545844u);                                  // "DXT1"
        p += kDdsHeader;
        for (uint32_t i = 0; i < levels; ++i) {
            const size_t n = (size_t)level_bytes(widths[i], heights[i]);
            if (n) std::memcpy(p, level_blocks[i], n);
            p += n;
        }
    } else {
        static const uint8_t ident[12] = {0xAB, 0x4B, 0x54, 0x58, 0x20, 0x31, 0x31, 0xBB, 0x0D, 0x0A, 0x1A, 0x0A};
        std::memset(p, 0, kKtxHeader);
        std::memcpy(p, ident, 12);
        put32(p + 12, 0x04030201u);  // endianness
        put32(p + 20, 1);            // glTypeSize
        put32(p + 28, 0x8D64u);      // GL_ETC1_RGB8_OES
        put32(p + 32, 0x1907u);      // GL_RGB
        put32(p + 36, widths[0]);
        put32(p + 40, heights[0]);
        put32(p + 52, 1);            // faces
        put32(p + 56, levels);       // mip levels
        p += kKtxHeader;
        for (uint32_t i = 0; i < levels; ++i) {
            const size_t n = (size_t)level_bytes(widths[i], heights[i]);
            put32(p, (uint32_t)n);
            p += 4;
            if (n) std::memcpy(p, level_blocks[i], n);
            p += n;  // n is a multiple of 8: no mip padding
        }
    }
    return GOOFY_OK;
}

GOOFY_EXPORT size_t goofy_gpu_tga_size(uint32_t width, uint32_t height)
{
    if (width == 0 || height == 0 || width > 65535 || height > 65535) return 0;
    return 18 + (size_t)width * height * 4;
}

GOOFY_EXPORT int goofy_gpu_write_tga(const uint8_t* rgba, uint32_t stride, uint32_t width, uint32_t height,
                                     uint8_t* out, size_t out_size)
{
    const size_t need = goofy_gpu_tga_size(width, height);
    if (need == 0 || !rgba || !out || (uint64_t)stride < 4ull * width) return GOOFY_ERR_INVALID;
    if (out_size < need) return goofy_gpu::fail(GOOFY_ERR_TOO_LARGE, "tga: output buffer too small");
    std::memset(out, 0, 18);
    out[2] = 2;  // uncompressed true colour
    out[12] = (uint8_t)width;
    out[13] = (uint8_t)(width >> 8);
    out[14] = (uint8_t)height;
    out[15] = (uint8_t)(height >> 8);
    out[16] = 32;    // bits per pixel
    out[17] = 0x20;  // rows stored top first
    uint8_t* p = out + 18;
    for (uint32_t y = 0; y < height; ++y) {
        const uint8_t* row = rgba + (size_t)y * stride;
        for (uint32_t x = 0; x < width; ++x, p += 4) {
            p[0] = row[4 * x + 2];
            p[1] = row[4 * x + 1];
            p[2] = row[4 * x + 0];
            p[3] = row[4 * x + 3];
        }
    }
    return GOOFY_OK;
}

}  // extern "C"
