// block_decode.cuh -- per-block BC1 / ETC1 decoding, branch-free.
//
// The reference harness's decoders (Src/decoder.cpp: DecompressColour
// :799-871 with decodeBlockDXT1 :933-943; decompressBlockDiffFlipC :388-678
// with decodeBlockETC1 :958-971) restated as a palette per block -- 4 RGBA
// words for BC1, 4 per sub-block (8) for ETC1 -- and a palette slot per
// pixel.  The palette goes to a per-thread column of a store (shared memory
// on the device: entry k of thread t at store[k * stride + t], bank-conflict
// free), and each pixel is one indexed load from it instead of a chain of
// selects.
//
// ETC1 differential blocks whose second colour leaves 0..31 are ETC2 modes the
// harness does not decode (decoder.cpp:740-760); they decode to zeros and are
// reported as unsupported.
#pragma once
#include <cstdint>

#include "block_codec.cuh"

namespace goofy_gpu {

// 5/6/5-bit endpoint to an RGBA word by bit replication, alpha 255.
GOOFY_FN uint32_t expand565(uint32_t v)
{
    const uint32_t r = (v >> 11) & 31u, g = (v >> 5) & 63u, b = v & 31u;
    return (r << 3 | r >> 2) | (g << 2 | g >> 4) << 8 | (b << 3 | b >> 2) << 16 | 0xff000000u;
}

// DecompressColour: c0 > c1 gives the 1/3 and 2/3 points as colours 2 and 3,
// otherwise colour 2 is the midpoint and colour 3 transparent black.  Division
// by 3 of n <= 765 is (n * 21846) >> 16.
GOOFY_FN void bc1_palette(uint32_t ends, uint32_t* pal)
{
    const uint32_t a = ends & 0xffffu, b = ends >> 16;
    const bool four = a > b;
    const uint32_t p = expand565(a), q = expand565(b);
    uint32_t p2 = 0xff000000u, p3 = 0xff000000u;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const uint32_t x = (p >> (8 * c)) & 0xffu, y = (q >> (8 * c)) & 0xffu;
        const uint32_t third = ((2u * x + y) * 21846u) >> 16, two_thirds = ((x + 2u * y) * 21846u) >> 16;
        p2 |= (four ? third : (x + y) >> 1) << (8 * c);
        p3 |= two_thirds << (8 * c);
    }
    pal[0] = p;
    pal[1] = q;
    pal[2] = p2;
    pal[3] = four ? p3 : 0u;
}

// Base colours (bytes R, G, B) of the two sub-blocks of the big-endian word
// w0: 4+4-bit individual colours, or a 5-bit colour and a 3-bit signed delta.
// False for a differential second colour outside 0..31.
GOOFY_FN bool etc1_bases(uint32_t w0, uint32_t& base0, uint32_t& base1)
{
    const bool diff = (w0 >> 1) & 1u;
    bool ok = true;
    base0 = base1 = 0;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const uint32_t h = (w0 >> (24 - 8 * c)) & 0xffu;
        const uint32_t i0 = (h >> 4) * 17u, i1 = (h & 15u) * 17u;
        const int c5 = (int)(h >> 3), d = (int)(h & 3u) - (int)(h & 4u);  // 3-bit two's complement
        const int c52 = c5 + d;
        ok = ok && (!diff || (c52 >= 0 && c52 <= 31));
        const int cl = min(max(c52, 0), 31);
        const uint32_t d0 = (uint32_t)(c5 << 3 | c5 >> 2), d1 = (uint32_t)(cl << 3 | cl >> 2);
        base0 |= (diff ? d0 : i0) << (8 * c);
        base1 |= (diff ? d1 : i1) << (8 * c);
    }
    return ok;
}

// Intensity modifier tables (compressParams, decoder.cpp:391-408): the small and large
// magnitude of each of the 8 tables, one byte each, picked with a byte permute.
GOOFY_FN int etc1_small(uint32_t table) { return (int)(perm(0x0D090502u, 0x2F211812u, table) & 0xffu); }
GOOFY_FN int etc1_large(uint32_t table) { return (int)(perm(0x2A1D1108u, 0xB76A503Cu, table) & 0xffu); }

// The 4 colours of a sub-block, slot = pixel index (msb << 1 | lsb):
// base + {small, large, -small, -large}, each channel clamped to 0..255.
// R and B are clamped together in 16-bit lanes biased by 256.
GOOFY_FN void etc1_subpalette(uint32_t base, uint32_t table, uint32_t* pal)
{
    const int s = etc1_small(table), l = etc1_large(table);
    const int mod[4] = {s, l, -s, -l};
    const uint32_t rb = base & 0x00ff00ffu;
    const int g = (int)((base >> 8) & 0xffu);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const uint32_t v = vmin2(vmax2(rb + (uint32_t)(256 + mod[k]) * 0x00010001u, 0x01000100u), 0x01ff01ffu) -
                           0x01000100u;
        pal[k] = v | (uint32_t)min(max(g + mod[k], 0), 255) << 8 | 0xff000000u;
    }
}

// 2-bit palette index of every pixel, pixel k = 4x + y at bits 2k..2k+1, from
// the lsb plane (bits 0..15) and msb plane (bits 16..31) of the index word.
GOOFY_FN uint32_t spread_bits16(uint32_t x)
{
    x = (x | x << 8) & 0x00ff00ffu;
    x = (x | x << 4) & 0x0f0f0f0fu;
    x = (x | x << 2) & 0x33333333u;
    return (x | x << 1) & 0x55555555u;
}

GOOFY_FN uint32_t etc1_codes(uint32_t w1) { return spread_bits16(w1 & 0xffffu) | spread_bits16(w1 >> 16) << 1; }

// Decodes one block into 16 row-major RGBA words, using store[k * stride]
// (k < 8) for the palette.  Returns false for an unsupported ETC1 block.
template <int CODEC>
GOOFY_FN bool decode_block(uint2 blk, uint32_t* store, uint32_t stride, uint32_t (&px)[16])
{
    if constexpr (CODEC == kBC1) {
        uint32_t pal[4];
        bc1_palette(blk.x, pal);
#pragma unroll
        for (int k = 0; k < 4; ++k) store[k * stride] = pal[k];
#pragma unroll
        for (int i = 0; i < 16; ++i) px[i] = store[((blk.y >> (2 * i)) & 3u) * stride];
        return true;
    } else {
        // the block is big-endian: bytes 0..3 of blk.x are bits 63..32
        const uint32_t w0 = perm(blk.x, 0u, 0x0123u), w1 = perm(blk.y, 0u, 0x0123u);
        if ((w0 & 0x07070702u) == 0x00000002u && ((w0 >> 5) & 7u) == ((w0 >> 2) & 7u)) {
            // ETC1s shape (every block this encoder writes): differential, zero deltas, one
            // table.  Both sub-blocks have the 5-bit colour (bits 31..27, 23..19, 15..11)
            // expanded by bit replication as base: one palette, no sub-block offsets.
            const uint32_t c5 = (w0 >> 3) & 0x1f1f1f00u;  // R5, G5, B5 in bytes 3, 2, 1
            const uint32_t e = ((c5 << 3) & 0xf8f8f800u) | ((c5 >> 2) & 0x07070700u);
            uint32_t pal[4];
            etc1_subpalette(perm(e, 0u, 0x4123u), (w0 >> 5) & 7u, pal);  // bytes R, G, B, 0
#pragma unroll
            for (int k = 0; k < 4; ++k) store[k * stride] = pal[k];
            const uint32_t codes = etc1_codes(w1);
#pragma unroll
            for (int y = 0; y < 4; ++y)
#pragma unroll
                for (int x = 0; x < 4; ++x) px[4 * y + x] = store[((codes >> (2 * (4 * x + y))) & 3u) * stride];
            return true;
        }
        const bool flip = w0 & 1u;
        uint32_t b0, b1, pal[4];
        const bool ok = etc1_bases(w0, b0, b1);
        // ETC1s blocks (zero deltas, one table) have one palette for both
        // sub-blocks: it is built and stored once
        const bool one = b0 == b1 && ((w0 >> 5) & 7u) == ((w0 >> 2) & 7u);
        etc1_subpalette(b0, (w0 >> 5) & 7u, pal);
#pragma unroll
        for (int k = 0; k < 4; ++k) store[k * stride] = ok ? pal[k] : 0u;
        if (!one) {
            etc1_subpalette(b1, (w0 >> 2) & 7u, pal);
#pragma unroll
            for (int k = 0; k < 4; ++k) store[(4 + k) * stride] = ok ? pal[k] : 0u;
        }
        const uint32_t codes = etc1_codes(w1);
        if (one) {  // every block this encoder writes: one palette, no sub-block offsets
#pragma unroll
            for (int y = 0; y < 4; ++y)
#pragma unroll
                for (int x = 0; x < 4; ++x) px[4 * y + x] = store[((codes >> (2 * (4 * x + y))) & 3u) * stride];
            return ok;
        }
        // sub-block 1: right half (x >= 2) without flip, bottom half (y >= 2) with flip
        const uint32_t s1 = 4u * stride;
        const uint32_t lower_right = s1, upper_right = flip ? 0u : s1, lower_left = flip ? s1 : 0u;
#pragma unroll
        for (int y = 0; y < 4; ++y)
#pragma unroll
            for (int x = 0; x < 4; ++x) {
                const uint32_t sub = x < 2 ? (y < 2 ? 0u : lower_left) : (y < 2 ? upper_right : lower_right);
                px[4 * y + x] = store[sub + ((codes >> (2 * (4 * x + y))) & 3u) * stride];
            }
        return ok;
    }
}

}  // namespace goofy_gpu
