/*
 * synth.c -- deterministic synthetic RGBA8 workloads for the encoder's tests
 * and benchmarks (the reference measures on PNG photographs that are not
 * redistributable here; these stand in with the stated shapes and
 * distributions).  Pure C, double arithmetic without contraction, so x86-64
 * and aarch64 hosts produce identical bytes.
 *
 *  scene    gradient (R = x, G = y, B = (x+y)/2, scaled to 0..255)
 *           + 4-octave value noise (periods 64/32/16/8 px times `period_scale`,
 *             amplitudes 48/24/12/6, smoothstep, lattice values uniform in
 *             [-1, 1] from PCG32, one lattice per octave and channel)
 *           + `rects` axis-aligned rectangles (8..96 px, uniform RGB fill)
 *  stress   four vertical quarters: i.i.d. RGBA noise / one colour per 4x4
 *           block / two colours per block / greyscale noise with random alpha
 *  mips     2x2 box filter with rounding, sizes halving down to 4
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#define EXPORT __attribute__((visibility("default")))

/* ---- PCG32 (O'Neill, pcg32_random_r / pcg32_srandom_r) ---- */
typedef struct { uint64_t state, inc; } pcg32;

static uint32_t pcg32_next(pcg32* r)
{
    uint64_t old = r->state;
    r->state = old * 6364136223846793005ULL + r->inc;
    uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    uint32_t rot = (uint32_t)(old >> 59u);
    return (xs >> rot) | (xs << ((-rot) & 31u));
}

static void pcg32_seed(pcg32* r, uint64_t initstate, uint64_t initseq)
{
    r->state = 0u;
    r->inc = (initseq << 1u) | 1u;
    pcg32_next(r);
    r->state += initstate;
    pcg32_next(r);
}

static double unit_pm1(pcg32* r) { return (double)pcg32_next(r) * (2.0 / 4294967296.0) - 1.0; }

EXPORT uint32_t goofy_synth_pcg32(uint64_t seed, uint64_t seq, uint32_t skip)
{
    pcg32 r;
    pcg32_seed(&r, seed, seq);
    for (uint32_t i = 0; i < skip; ++i) pcg32_next(&r);
    return pcg32_next(&r);
}

/* ---- value noise ---- */
typedef struct {
    int period, gw, gh;
    double amp;
    double* lattice; /* [3][gh][gw] */
} octave;

typedef struct {
    octave oct[4];
    int channels;
} noise_field;

static int noise_init(noise_field* nf, pcg32* rng, unsigned w, unsigned h, unsigned period_scale, int channels)
{
    static const int base_period[4] = {64, 32, 16, 8};
    static const double base_amp[4] = {48.0, 24.0, 12.0, 6.0};
    nf->channels = channels;
    for (int o = 0; o < 4; ++o) {
        octave* oc = &nf->oct[o];
        oc->period = base_period[o] * (int)(period_scale ? period_scale : 1);
        oc->amp = base_amp[o];
        oc->gw = (int)((w + (unsigned)oc->period - 1) / (unsigned)oc->period) + 1;
        oc->gh = (int)((h + (unsigned)oc->period - 1) / (unsigned)oc->period) + 1;
        size_t n = (size_t)channels * (size_t)oc->gw * (size_t)oc->gh;
        oc->lattice = (double*)malloc(n * sizeof(double));
        if (!oc->lattice) return -1;
        for (size_t i = 0; i < n; ++i) oc->lattice[i] = unit_pm1(rng);
    }
    return 0;
}

static void noise_free(noise_field* nf)
{
    for (int o = 0; o < 4; ++o) free(nf->oct[o].lattice);
}

static inline double smooth(double t) { return t * t * (3.0 - 2.0 * t); }

static double noise_at(const noise_field* nf, int c, unsigned x, unsigned y)
{
    double v = 0.0;
    for (int o = 0; o < 4; ++o) {
        const octave* oc = &nf->oct[o];
        const unsigned i = x / (unsigned)oc->period, j = y / (unsigned)oc->period;
        const double tx = smooth((double)(x % (unsigned)oc->period) / (double)oc->period);
        const double ty = smooth((double)(y % (unsigned)oc->period) / (double)oc->period);
        const double* L = oc->lattice + (size_t)c * oc->gw * oc->gh;
        const double a = L[(size_t)j * oc->gw + i], b = L[(size_t)j * oc->gw + i + 1];
        const double d = L[(size_t)(j + 1) * oc->gw + i], e = L[(size_t)(j + 1) * oc->gw + i + 1];
        const double top = a + (b - a) * tx, bot = d + (e - d) * tx;
        v += oc->amp * (top + (bot - top) * ty);
    }
    return v;
}

static inline uint8_t clamp_round(double v)
{
    double r = floor(v + 0.5);
    return (uint8_t)(r < 0.0 ? 0.0 : (r > 255.0 ? 255.0 : r));
}

typedef struct {
    uint8_t* dst;
    unsigned w, h, stride, y0, y1;
    const noise_field* nf;
} scene_rows;

/* Per-column lattice index and smoothed weight of each octave: the same
 * expressions noise_at() evaluates, computed once per column. */
typedef struct {
    unsigned* i;
    double* t;
} axis_weights;

static int axis_init(axis_weights* a, const noise_field* nf, unsigned n)
{
    a->i = (unsigned*)malloc(sizeof(unsigned) * 4 * (size_t)n);
    a->t = (double*)malloc(sizeof(double) * 4 * (size_t)n);
    if (!a->i || !a->t) return -1;
    for (int o = 0; o < 4; ++o) {
        const unsigned p = (unsigned)nf->oct[o].period;
        for (unsigned x = 0; x < n; ++x) {
            a->i[(size_t)o * n + x] = x / p;
            a->t[(size_t)o * n + x] = smooth((double)(x % p) / (double)p);
        }
    }
    return 0;
}

static void axis_free(axis_weights* a)
{
    free(a->i);
    free(a->t);
}

static void* scene_rows_main(void* arg)
{
    const scene_rows* s = (const scene_rows*)arg;
    const double sx = s->w > 1 ? 255.0 / (double)(s->w - 1) : 0.0;
    const double sy = s->h > 1 ? 255.0 / (double)(s->h - 1) : 0.0;
    const double sb = (s->w + s->h) > 2 ? 255.0 / (double)(s->w + s->h - 2) : 0.0;
    axis_weights ax;
    if (axis_init(&ax, s->nf, s->w) != 0) {
        axis_free(&ax);
        /* fall back to the direct evaluation */
        for (unsigned y = s->y0; y < s->y1; ++y) {
            uint8_t* row = s->dst + (size_t)y * s->stride;
            for (unsigned x = 0; x < s->w; ++x) {
                const double base[3] = {(double)x * sx, (double)y * sy, (double)(x + y) * sb};
                for (int c = 0; c < 3; ++c) row[4 * x + c] = clamp_round(base[c] + noise_at(s->nf, c, x, y));
                row[4 * x + 3] = 255;
            }
        }
        return NULL;
    }
    for (unsigned y = s->y0; y < s->y1; ++y) {
        uint8_t* row = s->dst + (size_t)y * s->stride;
        unsigned jy[4];
        double ty[4];
        for (int o = 0; o < 4; ++o) {
            const unsigned p = (unsigned)s->nf->oct[o].period;
            jy[o] = y / p;
            ty[o] = smooth((double)(y % p) / (double)p);
        }
        for (unsigned x = 0; x < s->w; ++x) {
            const double base[3] = {(double)x * sx, (double)y * sy, (double)(x + y) * sb};
            for (int c = 0; c < 3; ++c) {
                double v = 0.0;
                for (int o = 0; o < 4; ++o) {
                    const octave* oc = &s->nf->oct[o];
                    const unsigned i = ax.i[(size_t)o * s->w + x];
                    const double tx = ax.t[(size_t)o * s->w + x];
                    const double* L = oc->lattice + (size_t)c * oc->gw * oc->gh;
                    const double a = L[(size_t)jy[o] * oc->gw + i], b = L[(size_t)jy[o] * oc->gw + i + 1];
                    const double d = L[(size_t)(jy[o] + 1) * oc->gw + i], e = L[(size_t)(jy[o] + 1) * oc->gw + i + 1];
                    const double top = a + (b - a) * tx, bot = d + (e - d) * tx;
                    v += oc->amp * (top + (bot - top) * ty[o]);
                }
                row[4 * x + c] = clamp_round(base[c] + v);
            }
            row[4 * x + 3] = 255;
        }
    }
    axis_free(&ax);
    return NULL;
}

static void run_rows(scene_rows* proto, int threads)
{
    if (threads < 1) {  /* 0: one per online CPU */
        long n = sysconf(_SC_NPROCESSORS_ONLN);
        threads = n > 0 ? (int)n : 1;
    }
    if ((unsigned)threads > proto->h) threads = proto->h ? (int)proto->h : 1;
    pthread_t tid[64];
    scene_rows part[64];
    char started[64] = {0};
    if (threads > 64) threads = 64;
    for (int t = 0; t < threads; ++t) {
        part[t] = *proto;
        part[t].y0 = (unsigned)((uint64_t)proto->h * t / threads);
        part[t].y1 = (unsigned)((uint64_t)proto->h * (t + 1) / threads);
        if (threads > 1 && pthread_create(&tid[t], NULL, scene_rows_main, &part[t]) == 0) started[t] = 1;
        else scene_rows_main(&part[t]);
    }
    for (int t = 0; t < threads; ++t)
        if (started[t]) pthread_join(tid[t], NULL);
}

/* Gradient + noise + rectangles.  Returns 0, or -1 on bad arguments / OOM. */
EXPORT int goofy_synth_scene(uint8_t* dst, unsigned w, unsigned h, unsigned stride, uint64_t seed,
                             unsigned period_scale, unsigned rects, int threads)
{
    if (!dst || stride < 4u * w) return -1;
    pcg32 rng;
    pcg32_seed(&rng, seed, 0x5eedu);
    noise_field nf;
    memset(&nf, 0, sizeof nf);
    if (noise_init(&nf, &rng, w, h, period_scale, 3) != 0) { noise_free(&nf); return -1; }
    scene_rows proto = {dst, w, h, stride, 0, h, &nf};
    run_rows(&proto, threads);
    noise_free(&nf);
    for (unsigned r = 0; r < rects; ++r) {
        const unsigned x0 = pcg32_next(&rng) % w, y0 = pcg32_next(&rng) % h;
        const unsigned rw = 8 + pcg32_next(&rng) % 89, rh = 8 + pcg32_next(&rng) % 89;
        const uint32_t col = pcg32_next(&rng);
        const unsigned x1 = x0 + rw < w ? x0 + rw : w, y1 = y0 + rh < h ? y0 + rh : h;
        for (unsigned y = y0; y < y1; ++y) {
            uint8_t* row = dst + (size_t)y * stride;
            for (unsigned x = x0; x < x1; ++x) {
                row[4 * x + 0] = (uint8_t)col;
                row[4 * x + 1] = (uint8_t)(col >> 8);
                row[4 * x + 2] = (uint8_t)(col >> 16);
            }
        }
    }
    return 0;
}

/* Degenerate / stress distributions as four vertical quarters (w % 16 == 0,
 * h % 4 == 0): (a) i.i.d. RGBA; (b) one random colour per 4x4 block;
 * (c) two random colours per block, chosen per pixel; (d) greyscale value
 * noise with uniformly random alpha. */
EXPORT int goofy_synth_stress(uint8_t* dst, unsigned w, unsigned h, unsigned stride, uint64_t seed)
{
    if (!dst || stride < 4u * w || w % 16 || h % 4) return -1;
    const unsigned qw = w / 4;
    pcg32 rng;
    /* (a) */
    pcg32_seed(&rng, seed, 1);
    for (unsigned y = 0; y < h; ++y)
        for (unsigned x = 0; x < qw; ++x) {
            uint32_t v = pcg32_next(&rng);
            memcpy(dst + (size_t)y * stride + 4 * (size_t)x, &v, 4);
        }
    /* (b), (c) */
    for (int q = 1; q <= 2; ++q) {
        pcg32_seed(&rng, seed, (uint64_t)q + 1);
        for (unsigned by = 0; by < h / 4; ++by)
            for (unsigned bx = 0; bx < qw / 4; ++bx) {
                uint32_t c0 = pcg32_next(&rng) | 0xff000000u;
                uint32_t c1 = q == 2 ? (pcg32_next(&rng) | 0xff000000u) : c0;
                uint32_t pick = q == 2 ? pcg32_next(&rng) : 0;
                for (unsigned y = 0; y < 4; ++y)
                    for (unsigned x = 0; x < 4; ++x) {
                        uint32_t v = (pick >> (4 * y + x)) & 1u ? c1 : c0;
                        memcpy(dst + (size_t)(4 * by + y) * stride + 4 * (size_t)(q * qw + 4 * bx + x), &v, 4);
                    }
            }
    }
    /* (d) */
    pcg32_seed(&rng, seed, 4);
    noise_field nf;
    memset(&nf, 0, sizeof nf);
    if (noise_init(&nf, &rng, qw, h, 1, 1) != 0) { noise_free(&nf); return -1; }
    for (unsigned y = 0; y < h; ++y)
        for (unsigned x = 0; x < qw; ++x) {
            uint8_t* p = dst + (size_t)y * stride + 4 * (size_t)(3 * qw + x);
            p[0] = p[1] = p[2] = clamp_round(128.0 + noise_at(&nf, 0, x, y));
            p[3] = (uint8_t)pcg32_next(&rng);
        }
    noise_free(&nf);
    return 0;
}

/* One mip level from the level above: 2x2 box filter, (a+b+c+d+2)>>2 per
 * channel; sizes halve and are clamped at 4 (a clamped axis is copied). */
EXPORT int goofy_synth_downsample(uint8_t* dst, unsigned dst_stride, const uint8_t* src, unsigned w,
                                  unsigned h, unsigned src_stride)
{
    if (!dst || !src) return -1;
    const unsigned dw = w / 2 >= 4 ? w / 2 : 4, dh = h / 2 >= 4 ? h / 2 : 4;
    const unsigned fx = w > dw ? 2 : 1, fy = h > dh ? 2 : 1;
    for (unsigned y = 0; y < dh; ++y)
        for (unsigned x = 0; x < dw; ++x)
            for (int c = 0; c < 4; ++c) {
                const uint8_t* p = src + (size_t)(y * fy) * src_stride + 4 * (size_t)(x * fx) + c;
                unsigned a = p[0], b = p[4 * (fx - 1)], d = p[(size_t)src_stride * (fy - 1)],
                         e = p[(size_t)src_stride * (fy - 1) + 4 * (fx - 1)];
                dst[(size_t)y * dst_stride + 4 * (size_t)x + c] = (uint8_t)((a + b + d + e + 2) >> 2);
            }
    return 0;
}

/* Shape of texture `index` of the mixed batch workload: width and height drawn
 * independently from {64,...,2048} (log-uniform), 20% with a full mip chain,
 * codec 0 (BC1) or 1 (ETC1s) 50/50. */
EXPORT void goofy_synth_texture_spec(uint64_t index, unsigned* w, unsigned* h, int* mips, int* codec)
{
    pcg32 rng;
    pcg32_seed(&rng, index, 0xba7c4u);
    *w = 64u << (pcg32_next(&rng) % 6u);
    *h = 64u << (pcg32_next(&rng) % 6u);
    *mips = (pcg32_next(&rng) % 5u) == 0u;
    *codec = (int)(pcg32_next(&rng) & 1u);
}
