// block_codec.cuh -- per-4x4-block Goofy encoder for sm_103a, integer SIMT.
//
// One thread encodes one block from its 16 RGBA8 pixel words (row-major,
// byte 0 = R).  The arithmetic is the reference heuristic
// (GoofyTC/goofy_tc.h:1066-1494, goofySimdEncode) restated for 32-bit
// registers instead of 16-byte SSE2 vectors; results are bit-identical.
//
// Identities the formulation relies on (all exact on 0..255 inputs):
//  * luma  Y(c) = avg(avg(R, B), G)  with avg(a,b) = (a+b+1)>>1
//          (goofy_tc.h:1159-1166) equals ceil((R + 2G + B) / 4).  Writing
//          S = R + 2G + B (one dp4a against bytes 1,2,1,0):
//             Y >= c   <=>   S >= 4c - 3      for every integer c,
//          so every per-pixel brightness test is one add of a per-block
//          constant followed by a look at one bit.
//  * gez = (Y >= mid); lqt = |Y - mid| < qt <=> (Y >= mid-qt+1) && !(Y >= mid+qt)
//          (qt <= 96 < 127, so the clamp to 127 at goofy_tc.h:1207-1208 and
//          the signed compare at :1224 never change the outcome).
//  * to5(x) = avg(avg(avg(subsat(x,8),0),0),0)  (goofy_tc.h:1309)
//           = (max(x,1) - 1) >> 3.
//  * the ETC1 mean tree of rounding averages (goofy_tc.h:1402-1414) is kept
//    exact in 16-bit lanes by carrying each level scaled by 2^k:
//           2^k * avg(x, y) = (2^(k-1) x + 2^(k-1) y + 2^(k-1)) & ~(2^k - 1).
#pragma once
#include <cstdint>

#if defined(GOOFY_HOST_EMULATION)
// Test-only: lets tests/host_emu compile this header for the CPU to check the
// block arithmetic against the oracle without a GPU.  Never part of the
// shipped library, which is built for sm_103a only.
#include "host_emulation.h"
#else
#define GOOFY_FN __device__ __forceinline__
#endif

namespace goofy_gpu {

enum Codec : int { kBC1 = 0, kETC1S = 1, kBoth = 2 };  // kBoth: one pass writing both codecs' blocks

#if !defined(GOOFY_HOST_EMULATION)
GOOFY_FN uint32_t perm(uint32_t a, uint32_t b, uint32_t sel) { return __byte_perm(a, b, sel); }

GOOFY_FN uint32_t vmin2(uint32_t a, uint32_t b)
{
    uint32_t d;
    asm("min.u16x2 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b));
    return d;
}

GOOFY_FN uint32_t vmax2(uint32_t a, uint32_t b)
{
    uint32_t d;
    asm("max.u16x2 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b));
    return d;
}
#endif

// S = R + 2G + B + acc
GOOFY_FN uint32_t luma_sum(uint32_t px, uint32_t acc) { return __dp4a(px, 0x00010201u, acc); }

// Y = avg(avg(R,B),G) of an RGB word
GOOFY_FN uint32_t luma(uint32_t px) { return luma_sum(px, 3u) >> 2; }

// The same from an R/B lane word (R in byte 0, B in byte 2) and a word with G
// in byte 0: two byte dot products, no repacking.
GOOFY_FN uint32_t luma_lanes(uint32_t rb, uint32_t g) { return __dp4a(rb, 0x00010001u, __dp4a(g, 0x00000002u, 3u)) >> 2; }

// to5 on both 16-bit lanes
GOOFY_FN uint32_t to5x2(uint32_t lanes) { return ((vmax2(lanes, 0x00010001u) - 0x00010001u) >> 3) & 0x001f001fu; }

// Lane-wise min / max of N words, reduced three words at a time
// (min(min(a, b), c) is one three-input lane min / max instruction): 16 words
// take 8 instructions, 8 words 4.
template <int N, bool MAX>
GOOFY_FN uint32_t tree_reduce(const uint32_t* v)
{
    if constexpr (N == 1) return v[0];
    else if constexpr (N == 2) return MAX ? vmax2(v[0], v[1]) : vmin2(v[0], v[1]);
    else {
        constexpr int M = (N + 2) / 3;
        uint32_t r[M];
#pragma unroll
        for (int i = 0; i < M; ++i) {
            const int n = N - 3 * i < 3 ? N - 3 * i : 3;
            const uint32_t* p = v + 3 * i;
            r[i] = n == 1 ? p[0] : n == 2 ? (MAX ? vmax2(p[0], p[1]) : vmin2(p[0], p[1]))
                                          : (MAX ? vmax2(vmax2(p[0], p[1]), p[2]) : vmin2(vmin2(p[0], p[1]), p[2]));
        }
        return tree_reduce<M, MAX>(r);
    }
}

template <int N>
GOOFY_FN uint32_t tree_min(const uint32_t* v) { return tree_reduce<N, false>(v); }

template <int N>
GOOFY_FN uint32_t tree_max(const uint32_t* v) { return tree_reduce<N, true>(v); }

// Run starts of etc1BrighnessRangeTocontrolByte (goofy_tc.h:1040-1057); all
// are even, so a 128-entry table indexed by range>>1 reproduces it.
GOOFY_FN uint32_t etc_control_byte(uint32_t range)
{
    const uint32_t t = (range >= 22) + (range >= 44) + (range >= 74) + (range >= 106) + (range >= 152) +
                       (range >= 182) + (range >= 254);
    return t * 0x24u + 3u;  // (t<<5)|(t<<2)|diff|flip
}

struct BlockRange {
    uint32_t range, mid, qt;
};

// Brightness statistics of the block from its channel min / max (R/B lane
// words and G in byte 0), goofy_tc.h:1151-1190.
GOOFY_FN BlockRange block_range(uint32_t mn_rb, uint32_t mn_g, uint32_t mx_rb, uint32_t mx_g)
{
    const uint32_t ymin = luma_lanes(mn_rb, mn_g), ymax = luma_lanes(mx_rb, mx_g);
    BlockRange r;
    r.range = max(ymax - ymin, 8u);
    r.mid = (ymin + ymax + 1u) >> 1;
    const uint32_t quarter = (r.range + 3u) >> 2;  // avg(avg(range, 0), 0)
    r.qt = quarter + ((quarter + 1u) >> 1);
    return r;
}

// 4 * avg(avg(a, b), avg(c, d)) on both 16-bit lanes (a..d <= 255), two
// rounding averages in one step.  With s = a + b + 1 and t = c + d + 1,
//     avg(avg(a, b), avg(c, d)) = (s + t + 2 - (s & t & 1)) >> 2:
// (s >> 1) + (t >> 1) = (s + t - (s & 1) - (t & 1)) / 2, and of the two
// parities only the case of both set moves the quotient by 4.  The result
// depends on a, b, c, d only through a + b and c + d, and the identity holds
// for every pair of sums in 0..510.  The +2 rides in s, where it leaves s's
// parity alone.
GOOFY_FN uint32_t avg4_x4(uint32_t a, uint32_t b, uint32_t c, uint32_t d)
{
    const uint32_t s = a + b + 0x00030003u, t = c + d + 0x00010001u;
    return (s + t - (s & t & 0x00010001u)) & 0xfffcfffcu;
}

// Channel extents of a block: R/B lane words (R in bits 0-7, B in bits
// 16-23) and words whose byte 0 is the minimum / maximum G.
struct Extents {
    uint32_t mn_rb, mx_rb, mn_g, mx_g;
};

// Lane words of one block shared by the extents and the ETC1s mean tree:
// rb[i] = R, B of pixel i; gp[2y + x] = G(y, x), G(y, x + 2).
struct BlockLanes {
    uint32_t rb[16], gp[8];
};

GOOFY_FN void block_lanes(const uint32_t (&w)[16], BlockLanes& l)
{
#pragma unroll
    for (int i = 0; i < 16; ++i) l.rb[i] = w[i] & 0x00ff00ffu;
#pragma unroll
    for (int y = 0; y < 4; ++y)
#pragma unroll
        for (int x = 0; x < 2; ++x)  // lanes G(y, x), G(y, x+2): byte dot products and a multiply-add (FMA pipe)
            l.gp[2 * y + x] = __dp4a(w[4 * y + x + 2], 0x00000100u, 0u) * 0x10000u + __dp4a(w[4 * y + x], 0x00000100u, 0u);
}

GOOFY_FN Extents lane_extents(const BlockLanes& l)
{
    Extents e;
    e.mn_rb = tree_min<16>(l.rb);
    e.mx_rb = tree_max<16>(l.rb);
    const uint32_t mn_g = tree_min<8>(l.gp), mx_g = tree_max<8>(l.gp);
    e.mn_g = vmin2(mn_g, mn_g >> 16);
    e.mx_g = vmax2(mx_g, mx_g >> 16);
    return e;
}

// ---------------------------------------------------------------------------
// BC1: returns {c0 | c1 << 16, indices}; pixel i (row-major) at bits 2i..2i+1.
// goofy_tc.h:1276-1357.
// ---------------------------------------------------------------------------
GOOFY_FN uint2 bc1_from_extents(const uint32_t (&w)[16], const Extents& e)
{
    const uint32_t mn_rb = e.mn_rb, mx_rb = e.mx_rb, mn_g = e.mn_g, mx_g = e.mx_g;
    const BlockRange br = block_range(mn_rb, mn_g, mx_rb, mx_g);

    // thresholds on S of two pixels at once (16-bit lanes): flag bits 14 / 15
    const uint32_t k_gez = (0x4003u - 4u * br.mid) * 0x10001u;                // bit 14: Y >= mid
    const uint32_t k_lo = (0x8003u - 4u * (br.mid - br.qt + 1u)) * 0x10001u;  // bit 15: Y >= mid-qt+1
    const uint32_t k_hi = (0x8003u - 4u * (br.mid + br.qt)) * 0x10001u;       // bit 15: Y >= mid+qt
    uint32_t idx = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) {  // pixels i and i+8 share a register
        const uint32_t s = luma_sum(w[i + 8], 0u) * 0x10000u + luma_sum(w[i], 0u);
        const uint32_t f_gez = s + k_gez, f_lo = s + k_lo, f_hi = s + k_hi;
        // bit 14: not gez, bit 15: lqt (and 30 / 31 for pixel i+8)
        const uint32_t z = (f_lo & ~f_hi & 0x80008000u) | (~f_gez & 0x40004000u);
        idx = (idx >> 2) + z;  // after the last pair, pair i sits at bits 2i (and 16 + 2i)
    }

    // endpoints: lanes {max, min} for each channel, c0 in the low half
    const uint32_t r5 = to5x2(perm(mx_rb, mn_rb, 0x5410u));
    const uint32_t b5 = to5x2(perm(mx_rb, mn_rb, 0x7632u));
    const uint32_t g5 = to5x2(perm(mx_g, mn_g, 0x0400u) & 0x00ff00ffu);
    const uint32_t ends = (r5 << 11) | (g5 << 6) | b5 | 0x20u;
    return make_uint2(ends, idx);
}

GOOFY_FN uint2 encode_bc1(const uint32_t (&w)[16])
{
    uint32_t rb[16], gg[8];
#pragma unroll
    for (int i = 0; i < 16; ++i) rb[i] = w[i] & 0x00ff00ffu;           // lanes R, B
#pragma unroll
    for (int k = 0; k < 8; ++k) gg[k] = perm(w[k], w[k + 8], 0x5511u);  // lanes 257*G of two pixels
    Extents e;
    e.mn_rb = tree_min<16>(rb);
    e.mx_rb = tree_max<16>(rb);
    const uint32_t mn_g = tree_min<8>(gg), mx_g = tree_max<8>(gg);
    e.mn_g = vmin2(mn_g, mn_g >> 16);  // byte 0 = min G
    e.mx_g = vmax2(mx_g, mx_g >> 16);
    return bc1_from_extents(w, e);
}

// ---------------------------------------------------------------------------
// ETC1s: returns {word0, word1} as the reference stores them (little-endian
// u32s of the big-endian ETC1 block).  goofy_tc.h:1358-1493.
// `ctrl_lut` holds etc_control_byte(2*i) for i < 128.  With FROM_BC1 the
// index word is not computed here: word1 returns 0 and the caller derives it
// from the BC1 indices of the block (etc1s_indices_from_bc1).
// ---------------------------------------------------------------------------
template <bool FROM_BC1 = false>
GOOFY_FN uint2 etc1s_from_extents(const uint32_t (&w)[16], const BlockLanes& l, const Extents& e,
                                  const uint8_t* ctrl_lut)
{
    const uint32_t(&rb)[16] = l.rb;
    const uint32_t(&gp)[8] = l.gp;
    const BlockRange br = block_range(e.mn_rb, e.mn_g, e.mx_rb, e.mx_g);

    // block mean, rounding-average tree kept exact at scale 2^level; the
    // column averages and the two top levels of R / B go two levels at a
    // time (avg4_x4, and the same identity at scale 4 below)
    uint32_t col_rb[4];
#pragma unroll
    for (int x = 0; x < 4; ++x) col_rb[x] = avg4_x4(rb[x], rb[4 + x], rb[8 + x], rb[12 + x]);
    // 16 * avg(avg(c0, c1), avg(c2, c3)) for c multiples of 4, plus a bias of
    // 256 after the shift (0x1000 in s, clear of the parity bit 2): lanes
    // 256 + mean R, 256 + mean B
    const uint32_t s_rb = col_rb[0] + col_rb[1] + 0x100c100cu, t_rb = col_rb[2] + col_rb[3] + 0x00040004u;
    const uint32_t m_rb = ((s_rb + t_rb - (s_rb & t_rb & 0x00040004u)) & 0xfff0fff0u) >> 4;
    uint32_t col_g[2];
#pragma unroll
    for (int x = 0; x < 2; ++x) col_g[x] = avg4_x4(gp[x], gp[2 + x], gp[4 + x], gp[6 + x]);  // 4*col(x), 4*col(x+2)
    const uint32_t uv_g = (col_g[0] + col_g[1] + 0x00040004u) & 0xfff8fff8u;
    const uint32_t m_g = ((uv_g + (uv_g >> 16) + 0x1008u) & 0xfff0u) >> 4;  // 256 + mean G

    // Move the mean's brightness onto mid (goofy_tc.h:1416-1449): with
    // corr = min(|mid - Y(mean)|, 127) the base is min(mean + corr, 255) when
    // Y(mean) <= mid and max(mean - corr, 0) otherwise, i.e.
    //     base = clamp(mean + d, 0, 255),   d = mid - Y(mean),
    // the clamp of corr to 127 never acting: every channel of the mean lies in
    // [(max + 15 min) / 16, (15 max + min) / 16 + 2] (one bright pixel moves it
    // by at least a sixteenth; each level of rounding averages adds at most
    // 1/2), which keeps Y(mean) within 7/16 * 255 + 3 < 115 of mid.  Then
    // to5(base) = (clamp(mean + d, 1, 255) - 1) >> 3.  On the biased lanes
    // (the bias sits in bytes 1 / 3, which the luma dot products skip) that is
    // (clamp(lane + d, 257, 511) - 257) >> 3, so to5(base) << 3 is
    // (clamp(lane + d, 257, 511) - 257) & 0xf8, one mask for R, G and B
    // together once the three clamped lanes minus 257 sit in bytes 0, 1, 2.
    const int d = (int)br.mid - (int)luma_lanes(m_rb, m_g);
    const uint32_t c_rb = vmin2(vmax2(m_rb + (uint32_t)d * 0x00010001u, 0x01010101u), 0x01ff01ffu);
    const uint32_t c_g = min(max(m_g + (uint32_t)d, 257u), 511u);
    const uint32_t rgb = c_rb + c_g * 256u - 257u * 0x00010101u;  // bytes 0, 1, 2: clamped R, G, B - 257
    const uint32_t word0 = (uint32_t)ctrl_lut[br.range >> 1] << 24 | (rgb & 0x00f8f8f8u);
    if constexpr (FROM_BC1) return make_uint2(word0, 0u);

    // indices: bit j = not gez, bit 16+j = not lqt of the pixel with
    // j = 4*(x^2) + y (transposeAs4x4x4 order, goofy_tc.h:1366-1395).
    // Per pixel, one register holds S + k in both 16-bit lanes (low lane: the
    // gez test, high lane: the Y >= mid-qt+1 test) scaled by 2^m, so the flag
    // bits land at 11+m / 27+m.  Pixels are grouped by the shift that still
    // separates them from their final bit: j = 11..15 (m = j-11, no shift),
    // j = 6..10 (m = j-6, >> 5), j = 1..5 (m = j-1, >> 10), j = 0 (>> 11);
    // flags within a group are distinct bits, so groups are summed and
    // shifted once.  A test S >= t is bit 11 of S + 2048 - t; with S <= 1020,
    // mid <= 255 and qt <= 96 the thresholds t_gez = 4 mid - 3,
    // t_lo = 4 (mid - qt) + 1 and t_hi = 4 (mid + qt) - 3 keep every lane
    // value in [0, 4096), so bit 11 is the test and the lanes, even scaled by
    // 2^4, never carry into each other.
    const uint32_t k_q = 0x07ff0803u + br.qt * 0x00040000u - br.mid * 0x00040004u;  // 2048 - t_gez | 2048 - t_lo
    const uint32_t k_h = (0x0803u - 4u * (br.mid + br.qt)) << 16;                    // h: S | S + 2048 - t_hi
    uint32_t group[4] = {0, 0, 0, 0};
#pragma unroll
    for (int y = 0; y < 4; ++y)
#pragma unroll
        for (int x = 0; x < 4; ++x) {
            const int j = 4 * (x ^ 2) + y;
            const int gi = j >= 11 ? 0 : j >= 6 ? 1 : j >= 1 ? 2 : 3;
            const int m = j >= 11 ? j - 11 : j >= 6 ? j - 6 : j >= 1 ? j - 1 : 0;
            const uint32_t s = luma_sum(w[4 * y + x], 0u);
            const uint32_t q = s * (0x00010001u << m) + (k_q << m);  // bit 11+m: Y >= mid, 27+m: Y >= mid-qt+1
            const uint32_t h = q + ((k_h - k_q) << m);                // bit 27+m: Y >= mid+qt; bit 11+m clear
            group[gi] += (~q | h) & (0x08000800u << m);
        }
    const uint32_t word1 = group[0] + (group[1] >> 5) + (group[2] >> 10) + (group[3] >> 11);
    return make_uint2(word0, word1);
}

// ETC1s word 1 from the BC1 index word of the same block.  Both codecs take
// the same two tests per pixel from the same brightness statistics (gez:
// Y >= mid; lqt: |Y - mid| < qt), so their index words hold the same 32 bits
// in another order: BC1 keeps pixel i = 4y + x at bits 2i (not gez) and
// 2i + 1 (lqt), ETC1s keeps not gez at bit j and not lqt at bit 16 + j, with
// j = 4(x ^ 2) + y.  Fixed bit permutation, by delta swaps (each swaps the
// bit pairs (p, p + s) selected by a mask):
//  1. three rounds of the inverse perfect shuffle: byte 0 / 2 then hold the
//     not-gez bits of pixels 0-7 / 8-15, byte 1 / 3 the lqt bits;
//  2. the 4x4 transpose (y, x) -> (x, y) of both bit planes at once: 2x2
//     blocks (pairs 3 apart), then the off-diagonal 2x2 blocks, which lie in
//     different bytes here (pairs 14 apart);
//  3. one byte permute for x -> x ^ 2 (pixels 0-7 and 8-15 trade places) and
//     the order of the two halves; lqt inverted on the way in.
GOOFY_FN uint32_t etc1s_indices_from_bc1(uint32_t idx)
{
    uint32_t x = idx ^ 0xaaaaaaaau, t;  // lqt -> not lqt
    t = (x ^ (x >> 1)) & 0x22222222u;
    x ^= t ^ (t << 1);
    t = (x ^ (x >> 2)) & 0x0c0c0c0cu;
    x ^= t ^ (t << 2);
    t = (x ^ (x >> 4)) & 0x00f000f0u;
    x ^= t ^ (t << 4);
    t = (x ^ (x >> 3)) & 0x0a0a0a0au;
    x ^= t ^ (t << 3);
    t = (x ^ (x >> 14)) & 0x0000ccccu;
    x ^= t ^ (t << 14);
    return perm(x, 0u, 0x1302u);
}

GOOFY_FN uint2 encode_etc1s(const uint32_t (&w)[16], const uint8_t* ctrl_lut)
{
    BlockLanes l;
    block_lanes(w, l);
    return etc1s_from_extents(w, l, lane_extents(l), ctrl_lut);
}

// Both codecs from one set of lanes and extents: the R/B masks, the min / max
// trees and the brightness statistics are computed once, and the ETC1s index
// word is a bit permutation of the BC1 one.  {BC1 block, ETC1s block}, each
// bit-identical to its own encoder's.
GOOFY_FN uint4 encode_both(const uint32_t (&w)[16], const uint8_t* ctrl_lut)
{
    BlockLanes l;
    block_lanes(w, l);
    const Extents e = lane_extents(l);
    const uint2 a = bc1_from_extents(w, e), b = etc1s_from_extents<true>(w, l, e, ctrl_lut);
    return make_uint4(a.x, a.y, b.x, etc1s_indices_from_bc1(a.y));
}

template <int CODEC>
GOOFY_FN uint2 encode_block(const uint32_t (&w)[16], const uint8_t* ctrl_lut)
{
    if constexpr (CODEC == kBC1) return encode_bc1(w);
    else return encode_etc1s(w, ctrl_lut);
}

}  // namespace goofy_gpu
