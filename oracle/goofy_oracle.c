/*
 * goofy_oracle.c -- TEST INFRASTRUCTURE: CPU restatement of the Goofy encoder.
 *
 * Restates, block by block and in the reference's own byte arithmetic, what
 * goofySimdEncode<GOOFY_DXT1/GOOFY_ETC1> (GoofyTC/goofy_tc.h:1066-1494) does
 * for 4 blocks at once with SSE2.  Every SSE2 primitive is replaced by its
 * scalar per-byte meaning (goofy_tc.h:165-396, and the portable restatement
 * the reference itself carries at :398-1027):
 *   avg(a,b)     = (a+b+1)>>1                 _mm_avg_epu8     :218-221
 *   subsat(a,b)  = max(a-b, 0)                _mm_subs_epu8    :258-261
 *   addsat(a,b)  = min(a+b, 255)              _mm_adds_epu8    :253-256
 *   lt_s8(a,b)   = (int8)a < (int8)b          _mm_cmplt_epi8   :248-251
 *   movemask     = MSB of each byte -> bit    _mm_movemask_epi8:380-383
 * Used only by tests/, __graft_entry__.smoke() and bench.py's CPU legs.
 */
#include "goofy_oracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

static inline uint8_t avg_u8(uint8_t a, uint8_t b) { return (uint8_t)((a + b + 1) >> 1); }
static inline uint8_t subsat_u8(uint8_t a, uint8_t b) { return (uint8_t)(a > b ? a - b : 0); }
static inline uint8_t addsat_u8(uint8_t a, uint8_t b) { int s = a + b; return (uint8_t)(s > 255 ? 255 : s); }
static inline uint8_t min_u8(uint8_t a, uint8_t b) { return a < b ? a : b; }
static inline uint8_t max_u8(uint8_t a, uint8_t b) { return a > b ? a : b; }
static inline int lt_s8(uint8_t a, uint8_t b) { return (int8_t)a < (int8_t)b; }

/* YCoCg luma Y = ((R+B)/2 + G)/2 with rounding averages, goofy_tc.h:1151-1166, :1205 */
static inline uint8_t luma(const uint8_t* c) { return avg_u8(avg_u8(c[0], c[2]), c[1]); }

/* rgb888 -> 5 bits: avg(avg(avg(subsat(x, 8), 0), 0), 0), goofy_tc.h:1309-1311, :1456 */
static inline uint32_t to5(uint8_t x)
{
    return avg_u8(avg_u8(avg_u8(subsat_u8(x, 8), 0), 0), 0);
}

/* etc1BrighnessRangeTocontrolByte (goofy_tc.h:1040-1057) restated as the
 * interval boundaries of its eight runs.  Run t holds (t<<29)|(t<<26)|(3<<24):
 * both 3-bit codeword-table indices = t, diff bit = 1, flip bit = 1. */
static uint32_t etc_control_word(uint8_t range)
{
    static const uint8_t run_start[7] = {22, 44, 74, 106, 152, 182, 254};
    uint32_t t = 0;
    for (int k = 0; k < 7; ++k) t += range >= run_start[k];
    return (t << 29) | (t << 26) | (3u << 24);
}

/* Order in which transposeAs4x4x4 (goofy_tc.h:297-366) and the movemasks of
 * :1378-1395 put the 16 pixels into the index bits of an ETC1 block: bit j
 * comes from row-major pixel etc_bit_pixel[j] (the C G K O / D H L P / A E I M /
 * B F J N diagram at :1366-1373). */
static const uint8_t etc_bit_pixel[16] = {2, 6, 10, 14, 3, 7, 11, 15, 0, 4, 8, 12, 1, 5, 9, 13};

static inline void put_le32(uint8_t* o, uint32_t v)
{
    o[0] = (uint8_t)v; o[1] = (uint8_t)(v >> 8); o[2] = (uint8_t)(v >> 16); o[3] = (uint8_t)(v >> 24);
}

void oracle_encode_block(int codec, const uint8_t* p, size_t stride, uint8_t out[8])
{
    uint8_t px[16][4];
    for (int y = 0; y < 4; ++y) memcpy(px[4 * y], p + (size_t)y * stride, 16); /* :1077-1099 */

    /* per-block channel min / max (all four channels, alpha unused later), :1103-1140 */
    uint8_t mn[4], mx[4];
    for (int c = 0; c < 4; ++c) {
        mn[c] = mx[c] = px[0][c];
        for (int i = 1; i < 16; ++i) { mn[c] = min_u8(mn[c], px[i][c]); mx[c] = max_u8(mx[c], px[i][c]); }
    }

    /* brightness range, mid point and quantisation threshold, :1151-1190 */
    const uint8_t ymin = luma(mn), ymax = luma(mx);
    const uint8_t range = max_u8(subsat_u8(ymax, ymin), 8);
    const uint8_t mid = avg_u8(ymin, ymax);
    const uint8_t half = avg_u8(range, 0), quarter = avg_u8(half, 0), eighth = avg_u8(quarter, 0);
    const uint8_t qt = addsat_u8(quarter, eighth);

    /* per-pixel masks, :1196-1272 */
    int gez[16], lqt[16];
    for (int i = 0; i < 16; ++i) {
        const uint8_t yv = luma(px[i]);
        const uint8_t pos = min_u8(subsat_u8(yv, mid), 0x7f);
        const uint8_t neg = min_u8(subsat_u8(mid, yv), 0x7f);
        gez[i] = neg == 0;
        lqt[i] = lt_s8((uint8_t)(pos | neg), qt);
    }

    if (codec == ORACLE_BC1) {
        /* zip(~gez, lqt) + movemask: pixel i -> bits 2i (not gez), 2i+1 (lqt), :1276-1301 */
        uint32_t idx = 0;
        for (int i = 0; i < 16; ++i) idx |= ((uint32_t)!gez[i] << (2 * i)) | ((uint32_t)lqt[i] << (2 * i + 1));
        /* 565 endpoints from the 5-bit channel values; green LSB of c0 forced to 1, :1303-1356 */
        const uint32_t c0 = 0x20u | to5(mx[0]) << 11 | to5(mx[1]) << 6 | to5(mx[2]);
        const uint32_t c1 = to5(mn[0]) << 11 | to5(mn[1]) << 6 | to5(mn[2]);
        put_le32(out, c0 | c1 << 16);
        put_le32(out + 4, idx);
        return;
    }

    /* ETC1s.  Block mean by the rounding-average tree, :1400-1414 */
    uint8_t col[4][4], m[4];
    for (int x = 0; x < 4; ++x)
        for (int c = 0; c < 4; ++c)
            col[x][c] = avg_u8(avg_u8(px[x][c], px[4 + x][c]), avg_u8(px[8 + x][c], px[12 + x][c]));
    for (int c = 0; c < 4; ++c) m[c] = avg_u8(avg_u8(col[0][c], col[1][c]), avg_u8(col[2][c], col[3][c]));

    /* move the mean's brightness onto `mid`, :1416-1449 */
    const uint8_t ya = luma(m);
    const uint8_t pc = min_u8(subsat_u8(mid, ya), 0x7f);
    const uint8_t nc = min_u8(subsat_u8(ya, mid), 0x7f);
    const int up = nc == 0;
    const uint8_t corr = (uint8_t)(pc | nc);
    uint32_t base5[3];
    for (int c = 0; c < 3; ++c) base5[c] = to5(up ? addsat_u8(m[c], corr) : subsat_u8(m[c], corr));

    /* word 0: 5-bit base colour, zero deltas, control byte; word 1: inverted masks, :1451-1493 */
    const uint32_t w0 = etc_control_word(range) | base5[0] << 3 | base5[1] << 11 | base5[2] << 19;
    uint32_t pos_or_zero = 0, less_qt = 0;
    for (int j = 0; j < 16; ++j) {
        pos_or_zero |= (uint32_t)gez[etc_bit_pixel[j]] << j;
        less_qt |= (uint32_t)lqt[etc_bit_pixel[j]] << j;
    }
    put_le32(out, w0);
    put_le32(out + 4, ~(pos_or_zero | less_qt << 16));
}

static void encode_rows(int codec, uint8_t* result, const uint8_t* input, unsigned bw,
                        unsigned by0, unsigned by1, unsigned stride)
{
    for (unsigned by = by0; by < by1; ++by) {
        const uint8_t* row = input + (size_t)by * 4 * stride;
        uint8_t* out = result + (size_t)by * bw * 8;
        for (unsigned bx = 0; bx < bw; ++bx) oracle_encode_block(codec, row + 16 * (size_t)bx, stride, out + 8 * (size_t)bx);
    }
}

int oracle_compress(int codec, uint8_t* result, const uint8_t* input,
                    unsigned width, unsigned height, unsigned stride)
{
    if (width % 16 != 0) return -1; /* :1500-1503 */
    if (height % 4 != 0) return -2; /* :1505-1508 */
    encode_rows(codec, result, input, width / 4, 0, height / 4, stride);
    return 0;
}

int oracle_compress_any(int codec, uint8_t* result, const uint8_t* input,
                        unsigned width, unsigned height, unsigned stride)
{
    if (width % 4 != 0) return -1;
    if (height % 4 != 0) return -2;
    encode_rows(codec, result, input, width / 4, 0, height / 4, stride);
    return 0;
}

typedef struct {
    int codec;
    uint8_t* result;
    const uint8_t* input;
    unsigned bw, by0, by1, stride;
} stripe_job;

static void* stripe_main(void* arg)
{
    const stripe_job* j = (const stripe_job*)arg;
    encode_rows(j->codec, j->result, j->input, j->bw, j->by0, j->by1, j->stride);
    return NULL;
}

int oracle_compress_mt(int codec, uint8_t* result, const uint8_t* input,
                       unsigned width, unsigned height, unsigned stride, int threads)
{
    if (width % 4 != 0) return -1;
    if (height % 4 != 0) return -2;
    if (threads <= 0) {
        long n = sysconf(_SC_NPROCESSORS_ONLN);
        threads = n > 0 ? (int)n : 1;
    }
    const unsigned bh = height / 4;
    if ((unsigned)threads > bh) threads = bh ? (int)bh : 1;
    if (threads <= 1) {
        encode_rows(codec, result, input, width / 4, 0, bh, stride);
        return 1;
    }
    pthread_t* tid = (pthread_t*)calloc((size_t)threads, sizeof(pthread_t));
    stripe_job* job = (stripe_job*)calloc((size_t)threads, sizeof(stripe_job));
    char* started = (char*)calloc((size_t)threads, 1);
    if (!tid || !job || !started) { free(tid); free(job); free(started); return -5; }
    for (int t = 0; t < threads; ++t) {
        job[t] = (stripe_job){codec, result, input, width / 4,
                              (unsigned)((uint64_t)bh * t / threads),
                              (unsigned)((uint64_t)bh * (t + 1) / threads), stride};
        if (pthread_create(&tid[t], NULL, stripe_main, &job[t]) == 0) started[t] = 1;
        else stripe_main(&job[t]);
    }
    for (int t = 0; t < threads; ++t)
        if (started[t]) pthread_join(tid[t], NULL);
    free(tid);
    free(job);
    free(started);
    return threads;
}

/* ------------------------------------------------------------------------- */
/* Decoding (test infrastructure: the quality check of the reference harness) */

static void expand565(uint32_t v, uint8_t c[4])
{
    const uint32_t r = (v >> 11) & 31, g = (v >> 5) & 63, b = v & 31; /* Unpack565, decoder.cpp:799-816 */
    c[0] = (uint8_t)(r << 3 | r >> 2);
    c[1] = (uint8_t)(g << 2 | g >> 4);
    c[2] = (uint8_t)(b << 3 | b >> 2);
    c[3] = 255;
}

static void decode_bc1(const uint8_t blk[8], uint8_t out[64])
{
    uint8_t pal[4][4];
    const uint32_t a = blk[0] | (uint32_t)blk[1] << 8, b = blk[2] | (uint32_t)blk[3] << 8;
    expand565(a, pal[0]);
    expand565(b, pal[1]);
    for (int c = 0; c < 3; ++c) { /* decoder.cpp:828-843 */
        const int p = pal[0][c], q = pal[1][c];
        if (a <= b) {
            pal[2][c] = (uint8_t)((p + q) / 2);
            pal[3][c] = 0;
        } else {
            pal[2][c] = (uint8_t)((2 * p + q) / 3);
            pal[3][c] = (uint8_t)((p + 2 * q) / 3);
        }
    }
    pal[2][3] = 255;
    pal[3][3] = a <= b ? 0 : 255;
    for (int i = 0; i < 16; ++i) { /* row y in byte 4+y, pixel x at bits 2x, decoder.cpp:849-868 */
        const int idx = (blk[4 + i / 4] >> (2 * (i % 4))) & 3;
        memcpy(out + 4 * i, pal[idx], 4);
    }
}

static const int etc1_modifiers[8][2] = {{2, 8}, {5, 17}, {9, 29}, {13, 42}, {18, 60}, {24, 80}, {33, 106}, {47, 183}};

static int decode_etc1(const uint8_t blk[8], uint8_t out[64])
{
    const uint32_t w0 = (uint32_t)blk[0] << 24 | (uint32_t)blk[1] << 16 | (uint32_t)blk[2] << 8 | blk[3];
    const uint32_t w1 = (uint32_t)blk[4] << 24 | (uint32_t)blk[5] << 16 | (uint32_t)blk[6] << 8 | blk[7];
    const int diff = (w0 >> 1) & 1, flip = w0 & 1;
    int base[2][3];
    if (diff) { /* 5-bit colour + signed 3-bit delta, decoder.cpp:554-631 */
        for (int c = 0; c < 3; ++c) {
            const int c5 = (w0 >> (27 - 8 * c)) & 31;
            int d = (w0 >> (24 - 8 * c)) & 7;
            d = d >= 4 ? d - 8 : d;
            const int c52 = c5 + d;
            if (c52 < 0 || c52 > 31) {  /* an ETC2 mode: not decoded here, zeros */
                memset(out, 0, 64);
                return -1;
            }
            base[0][c] = c5 << 3 | c5 >> 2;
            base[1][c] = c52 << 3 | c52 >> 2;
        }
    } else { /* two 4-bit colours, decoder.cpp:412-424 */
        for (int c = 0; c < 3; ++c) {
            const int a = (w0 >> (28 - 8 * c)) & 15, b = (w0 >> (24 - 8 * c)) & 15;
            base[0][c] = a << 4 | a;
            base[1][c] = b << 4 | b;
        }
    }
    const int table[2] = {(int)(w0 >> 5) & 7, (int)(w0 >> 2) & 7};
    for (int y = 0; y < 4; ++y)
        for (int x = 0; x < 4; ++x) {
            const int k = 4 * x + y; /* column-major pixel bit */
            const int idx = (int)((w1 >> (16 + k)) & 1) << 1 | (int)((w1 >> k) & 1);
            const int sub = flip ? (y >= 2) : (x >= 2);
            const int m = etc1_modifiers[table[sub]][idx & 1] * ((idx & 2) ? -1 : 1);
            uint8_t* px = out + 4 * (4 * y + x);
            for (int c = 0; c < 3; ++c) {
                const int v = base[sub][c] + m;
                px[c] = (uint8_t)(v < 0 ? 0 : (v > 255 ? 255 : v));
            }
            px[3] = 255;
        }
    return 0;
}

int oracle_decode_block(int codec, const uint8_t blk[8], uint8_t out[64])
{
    if (codec == ORACLE_BC1) {
        decode_bc1(blk, out);
        return 0;
    }
    return decode_etc1(blk, out);
}

long oracle_decode_image(int codec, const uint8_t* blocks, unsigned width, unsigned height, uint8_t* rgba,
                         unsigned stride)
{
    long bad = 0;
    uint8_t px[64];
    const unsigned bw = width / 4, bh = height / 4;
    for (unsigned by = 0; by < bh; ++by)
        for (unsigned bx = 0; bx < bw; ++bx) {
            bad += oracle_decode_block(codec, blocks + 8 * ((size_t)by * bw + bx), px) != 0;
            for (int y = 0; y < 4; ++y) memcpy(rgba + (size_t)(4 * by + y) * stride + 16 * (size_t)bx, px + 16 * y, 16);
        }
    return bad;
}

void oracle_sq_error(const uint8_t* a, unsigned a_stride, const uint8_t* b, unsigned b_stride, unsigned width,
                     unsigned height, uint64_t sums[4])
{
    for (int c = 0; c < 4; ++c) sums[c] = 0;
    for (unsigned y = 0; y < height; ++y) {
        const uint8_t* pa = a + (size_t)y * a_stride;
        const uint8_t* pb = b + (size_t)y * b_stride;
        for (unsigned x = 0; x < 4 * width; ++x) {
            const int d = (int)pa[x] - (int)pb[x];
            sums[x & 3] += (uint64_t)(d * d);
        }
    }
}

static double psnr_of(double mse, double peak)
{
    /* getPSNR, Src/main.cpp:386-395 */
    if (mse < 0.0000001) return DBL_MAX;
    return 10.0 * log10((peak * peak) / mse);
}

void oracle_mse_psnr(const uint8_t* a, unsigned a_stride, const uint8_t* b, unsigned b_stride, unsigned width,
                     unsigned height, double out[14])
{
    /* getMsePsnr, Src/main.cpp:403-469, in its own double arithmetic and
     * order.  Each pixel is read as a little-endian u32, so its "R" is byte 2
     * and its "B" byte 0 (:423-431); luminosity 0.21 R + 0.72 G + 0.07 B
     * (:398-401). */
    double mr = 0, mg = 0, mb = 0, ma = 0, mrgb = 0, my = 0;
    for (unsigned y = 0; y < height; ++y) {
        const uint8_t* pa = a + (size_t)y * a_stride;
        const uint8_t* pb = b + (size_t)y * b_stride;
        for (unsigned x = 0; x < width; ++x) {
            const double r1 = pa[4 * x + 2], g1 = pa[4 * x + 1], b1 = pa[4 * x], a1 = pa[4 * x + 3];
            const double r2 = pb[4 * x + 2], g2 = pb[4 * x + 1], b2 = pb[4 * x], a2 = pb[4 * x + 3];
            const double y1 = 0.21 * r1 + 0.72 * g1 + 0.07 * b1;
            const double y2 = 0.21 * r2 + 0.72 * g2 + 0.07 * b2;
            const double dy = y2 - y1;
            my += dy * dy;
            const double dr = r1 - r2, dg = g1 - g2, db = b1 - b2, da = a1 - a2;
            mrgb += (dr * dr) + (dg * dg) + (db * db);
            mr += dr * dr;
            mg += dg * dg;
            mb += db * db;
            ma += da * da;
        }
    }
    const double n = (double)(uint32_t)(width * height); /* the harness multiplies in 32 bits */
    out[0] = mr / n;
    out[1] = mg / n;
    out[2] = mb / n;
    out[3] = ma / n;
    out[5] = mrgb / n;
    out[6] = my / n;
    out[4] = fmax(fmax(out[0], out[1]), fmax(out[2], out[3]));
    for (int c = 0; c < 4; ++c) out[7 + c] = psnr_of(out[c], 255.0);
    out[11] = fmin(fmin(out[7], out[8]), fmin(out[9], out[10]));
    out[12] = psnr_of(out[5], 768.0);
    out[13] = psnr_of(out[6], 255.0);
}

double oracle_psnr_rgb(const uint64_t sums[4], unsigned width, unsigned height)
{
    /* mseRGB = sum(dR^2 + dG^2 + dB^2) / pixels; psnr = 10 log10(768^2 / mse), DBL_MAX below 1e-7 */
    const double mse = (double)(sums[0] + sums[1] + sums[2]) / ((double)width * (double)height);
    if (mse < 0.0000001) return DBL_MAX;
    return 10.0 * log10((768.0 * 768.0) / mse);
}
