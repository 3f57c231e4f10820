// mips.cu -- mip-chain generation on the device, feeding the batch encoder.
//
// The reference has no mip generator (its harness only builds an RGB565 x2
// downsample as a quality baseline, Src/main.cpp:501-557); textures with mip
// chains are encoded level by level from levels the caller made.  Here each
// level is produced from the one above by a 2x2 box filter with rounding,
// (a + b + c + d + 2) >> 2 per channel, an axis that is already 4 pixels
// being copied instead of halved -- the rule of the workload generator's
// goofy_synth_downsample, so device and host chains are bit-identical.  While
// both axes halve, one launch makes up to 6 levels from shared-memory tiles
// (mip_fused_kernel); the rest take one launch per level, a thread per output
// pixel.  Channel pairs are summed in 16-bit lanes.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/goofy_gpu.h"
#include "host_util.h"
#include "pdl.cuh"

namespace {

__device__ __forceinline__ uint32_t box4(uint32_t a, uint32_t b, uint32_t c, uint32_t d)
{
    const uint32_t m = 0x00ff00ffu;
    const uint32_t rb = (a & m) + (b & m) + (c & m) + (d & m) + 0x00020002u;
    const uint32_t ga = ((a >> 8) & m) + ((b >> 8) & m) + ((c >> 8) & m) + ((d >> 8) & m) + 0x00020002u;
    return ((rb >> 2) & m) | (((ga >> 2) & m) << 8);
}

// One output pixel per thread.  FX = 2 (the level halves horizontally) with
// 8-byte aligned rows reads the two source pixels of each row with one 8-byte
// load; otherwise four 4-byte loads.
template <bool PAIR>
__global__ void __launch_bounds__(256) mip_level_kernel(const uint8_t* __restrict__ src, size_t src_stride,
                                                        uint8_t* __restrict__ dst, size_t dst_stride, uint32_t dw,
                                                        uint32_t dh, uint32_t fx, uint32_t fy)
{
    goofy_gpu::pdl_launch_dependents();
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= dw || y >= dh) return;
    goofy_gpu::pdl_wait();
    const uint8_t* r0 = src + (size_t)(y * fy) * src_stride + 4u * (size_t)(x * fx);
    const uint8_t* r1 = r0 + src_stride * (fy - 1);
    uint32_t a, b, c, d;
    if constexpr (PAIR) {
        const uint2 p = __ldg(reinterpret_cast<const uint2*>(r0)), q = __ldg(reinterpret_cast<const uint2*>(r1));
        a = p.x;
        b = p.y;
        c = q.x;
        d = q.y;
    } else {
        a = __ldg(reinterpret_cast<const uint32_t*>(r0));
        b = __ldg(reinterpret_cast<const uint32_t*>(r0 + 4 * (fx - 1)));
        c = __ldg(reinterpret_cast<const uint32_t*>(r1));
        d = __ldg(reinterpret_cast<const uint32_t*>(r1 + 4 * (fx - 1)));
    }
    *reinterpret_cast<uint32_t*>(dst + (size_t)y * dst_stride + 4u * (size_t)x) = box4(a, b, c, d);
}

// Up to 6 levels per launch: a CTA takes a tile of up to 64x64 pixels of the
// level above.  Each thread reads a 4x4 patch (four 16-byte row loads), makes
// the 2x2 quad of the first new level and the one pixel of the second from it
// in registers, the third level comes from the 2x2 neighbourhood of second-
// level pixels held by lanes t^1, t^w, t^w^1 of the same warp (shuffles), and
// the remaining levels (at most 8x8 pixels per tile) go through shared
// memory.  Used while both axes halve; every level is the same box4 of the
// level above as in the one-level kernel, so the results are identical.
struct MipOut {
    uint8_t* data[6];
    uint32_t pitch[6];
};

__device__ __forceinline__ void store_px(const MipOut& o, int l, uint32_t row, uint32_t col, uint32_t v)
{
    *reinterpret_cast<uint32_t*>(o.data[l] + (size_t)row * o.pitch[l] + 4u * col) = v;
}

// One tile's levels from its thread's 4x4 patch `r` (already loaded).
__device__ __forceinline__ void mip_tile(const uint4 (&r)[4], bool act, uint32_t tx, uint32_t ty, uint32_t tw_log2,
                                         uint32_t th_log2, uint32_t nlev, const MipOut& out, uint32_t (*buf)[64])
{
    const uint32_t t = threadIdx.x;
    const uint32_t w2_log2 = tw_log2 - 2, h2_log2 = th_log2 - 2, w2 = 1u << w2_log2;
    const uint32_t x2 = t & (w2 - 1u), y2 = t >> w2_log2;
    uint32_t v2 = 0;
    if (act) {
        const uint32_t q00 = box4(r[0].x, r[0].y, r[1].x, r[1].y), q01 = box4(r[0].z, r[0].w, r[1].z, r[1].w);
        const uint32_t q10 = box4(r[2].x, r[2].y, r[3].x, r[3].y), q11 = box4(r[2].z, r[2].w, r[3].z, r[3].w);
        const uint32_t row1 = (ty << (th_log2 - 1)) + 2u * y2, col1 = (tx << (tw_log2 - 1)) + 2u * x2;
        *reinterpret_cast<uint2*>(out.data[0] + (size_t)row1 * out.pitch[0] + 4u * col1) = make_uint2(q00, q01);
        *reinterpret_cast<uint2*>(out.data[0] + (size_t)(row1 + 1) * out.pitch[0] + 4u * col1) = make_uint2(q10, q11);
        v2 = box4(q00, q01, q10, q11);
        if (nlev > 1) store_px(out, 1, (ty << h2_log2) + y2, (tx << w2_log2) + x2, v2);
    }
    if (nlev <= 2) return;
    // third level: lanes with even x2 and y2 combine their 2x2 neighbourhood
    const uint32_t b = __shfl_xor_sync(0xffffffffu, v2, 1), c = __shfl_xor_sync(0xffffffffu, v2, w2),
                   d = __shfl_xor_sync(0xffffffffu, v2, w2 ^ 1u);
    const uint32_t w3_log2 = w2_log2 - 1, h3_log2 = h2_log2 - 1;
    if (act && !(x2 & 1u) && !(y2 & 1u)) {
        const uint32_t v3 = box4(v2, b, c, d), x3 = x2 >> 1, y3 = y2 >> 1;
        store_px(out, 2, (ty << h3_log2) + y3, (tx << w3_log2) + x3, v3);
        buf[0][(y3 << w3_log2) + x3] = v3;
    }
    uint32_t cw_log2 = w3_log2, ch_log2 = h3_log2;
#pragma unroll
    for (uint32_t l = 3; l < 6; ++l) {  // unrolled: the level indexes `out` as a constant (no stack copy)
        if (l >= nlev) break;
        __syncthreads();
        const uint32_t* in = buf[(l - 3) & 1];
        uint32_t* next = buf[(l - 2) & 1];
        const uint32_t nw_log2 = cw_log2 - 1, nh_log2 = ch_log2 - 1, cw = 1u << cw_log2;
        if (t < (1u << (nw_log2 + nh_log2))) {
            const uint32_t ox = t & ((1u << nw_log2) - 1u), oy = t >> nw_log2;
            const uint32_t* r0 = in + (2u * oy) * cw + 2u * ox;
            const uint32_t v = box4(r0[0], r0[1], r0[cw], r0[cw + 1]);
            next[t] = v;
            store_px(out, (int)l, (ty << nh_log2) + oy, (tx << nw_log2) + ox, v);
        }
        cw_log2 = nw_log2;
        ch_log2 = nh_log2;
    }
    __syncthreads();  // the next tile of this CTA reuses buf
}

// TILES horizontally adjacent tiles per CTA: every patch load of all of them
// is issued before the first tile is reduced, so more bytes are in flight.
template <int TILES>
__global__ void __launch_bounds__(256) mip_fused_kernel(const uint8_t* __restrict__ src, size_t src_stride,
                                                        uint32_t tw_log2, uint32_t th_log2, uint32_t nlev, MipOut out)
{
    goofy_gpu::pdl_launch_dependents();
    __shared__ uint32_t buf[2][64];
    const uint32_t t = threadIdx.x, ty = blockIdx.y;
    const uint32_t w2_log2 = tw_log2 - 2, h2_log2 = th_log2 - 2, w2 = 1u << w2_log2;
    const bool act = t < (1u << (w2_log2 + h2_log2));
    const uint32_t x2 = t & (w2 - 1u), y2 = t >> w2_log2;
    uint4 r[TILES][4];
    goofy_gpu::pdl_wait();  // the level above may come from the previous launch
#pragma unroll
    for (int k = 0; k < TILES; ++k) {
        if (act) {
            const uint32_t tx = blockIdx.x * TILES + k;
            const uint8_t* patch = src + (((size_t)ty << th_log2) + 4u * y2) * src_stride +
                                   (((size_t)tx << tw_log2) + 4u * x2) * 4u;
#pragma unroll
            for (int j = 0; j < 4; ++j) r[k][j] = __ldg(reinterpret_cast<const uint4*>(patch + (size_t)j * src_stride));
        }
    }
#pragma unroll
    for (int k = 0; k < TILES; ++k) mip_tile(r[k], act, blockIdx.x * TILES + k, ty, tw_log2, th_log2, nlev, out, buf);
}

bool pow2(uint32_t v) { return v && !(v & (v - 1)); }

uint32_t log2u(uint32_t v)
{
    uint32_t l = 0;
    while (v > 1) {
        v >>= 1;
        ++l;
    }
    return l;
}

size_t pitch_of(uint32_t w) { return ((size_t)4 * w + 255) & ~(size_t)255; }

}  // namespace

extern "C" {

GOOFY_EXPORT uint32_t goofy_gpu_mip_count(uint32_t width, uint32_t height)
{
    if (!pow2(width) || !pow2(height) || width < 4 || height < 4) return 0;
    uint32_t n = 1;
    while (width > 4 || height > 4) {
        width = width / 2 >= 4 ? width / 2 : 4;
        height = height / 2 >= 4 ? height / 2 : 4;
        ++n;
    }
    return n;
}

GOOFY_EXPORT size_t goofy_gpu_mip_arena_bytes(uint32_t width, uint32_t height)
{
    const uint32_t n = goofy_gpu_mip_count(width, height);
    size_t bytes = 0;
    for (uint32_t i = 1; i < n; ++i) {
        width = width / 2 >= 4 ? width / 2 : 4;
        height = height / 2 >= 4 ? height / 2 : 4;
        bytes += pitch_of(width) * height;
    }
    return bytes;
}

GOOFY_EXPORT int goofy_gpu_generate_mips(const void* src, uint32_t width, uint32_t height, uint32_t stride,
                                         void* arena, size_t arena_bytes, goofy_gpu_level* levels,
                                         uint32_t max_levels, uint32_t* nlevels, void* stream)
{
    const uint32_t n = goofy_gpu_mip_count(width, height);
    if (n == 0) return goofy_gpu::fail(GOOFY_ERR_WIDTH, "mips: sizes must be powers of two >= 4");
    if (!src || !levels || !nlevels || (n > 1 && !arena)) return GOOFY_ERR_INVALID;
    if ((uint64_t)stride < 4ull * width || stride % 4 || reinterpret_cast<uintptr_t>(src) % 4)
        return GOOFY_ERR_ALIGNMENT;
    if (max_levels < n) return goofy_gpu::fail(GOOFY_ERR_TOO_LARGE, "mips: level array too small");
    if (arena_bytes < goofy_gpu_mip_arena_bytes(width, height) || reinterpret_cast<uintptr_t>(arena) % 256)
        return goofy_gpu::fail(GOOFY_ERR_TOO_LARGE, "mips: arena too small or not 256-byte aligned");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    levels[0] = goofy_gpu_level{const_cast<void*>(src), width, height, stride};
    uint8_t* out = static_cast<uint8_t*>(arena);
    for (uint32_t i = 1; i < n; ++i) {  // the arena layout: levels 1.. back to back, 256-byte rows
        const goofy_gpu_level& up = levels[i - 1];
        const uint32_t dw = up.width / 2 >= 4 ? up.width / 2 : 4, dh = up.height / 2 >= 4 ? up.height / 2 : 4;
        const size_t pitch = pitch_of(dw);
        levels[i] = goofy_gpu_level{out, dw, dh, (uint32_t)pitch};
        out += pitch * dh;
    }
    for (uint32_t i = 1; i < n;) {
        const goofy_gpu_level& up = levels[i - 1];
        // levels from here on that halve both axes (an axis at 4 stays 4)
        uint32_t both = 0;
        for (uint32_t w = up.width, h = up.height; i + both < n && w > 4 && h > 4; w /= 2, h /= 2) ++both;
        uint32_t f = log2u(up.width < up.height ? up.width : up.height);
        f = f < both ? f : both;
        f = f < 6 ? f : 6;
        // square tiles of 2^f pixels make exactly f levels (one pixel of the last);
        // the tail of a chain thus gets many small tiles instead of a few large ones
        const uint32_t tw = 1u << f, th = 1u << f;
        if (f >= 2 && reinterpret_cast<uintptr_t>(up.data) % 16 == 0 && up.stride % 16 == 0) {
            MipOut mo{};
            for (uint32_t l = 0; l < f; ++l) {
                mo.data[l] = static_cast<uint8_t*>(levels[i + l].data);
                mo.pitch[l] = levels[i + l].stride;
            }
            const uint32_t gx = up.width / tw, gy = up.height / th;
            const uint8_t* up_data = static_cast<const uint8_t*>(up.data);
            const size_t up_stride = up.stride;
            if (gx % 2 == 0 && (uint64_t)gx * gy >= 2048)  // two tiles a CTA (faster than one or four) on large grids
                GOOFY_CUDA_TRY(goofy_gpu::launch_pdl(mip_fused_kernel<2>, dim3(gx / 2, gy), dim3(256), 0, st, up_data,
                                                     up_stride, log2u(tw), log2u(th), f, mo));
            else
                GOOFY_CUDA_TRY(goofy_gpu::launch_pdl(mip_fused_kernel<1>, dim3(gx, gy), dim3(256), 0, st, up_data,
                                                     up_stride, log2u(tw), log2u(th), f, mo));
            i += f;
            continue;
        }
        const goofy_gpu_level& lv = levels[i];
        const uint32_t fx = up.width > lv.width ? 2 : 1, fy = up.height > lv.height ? 2 : 1;
        const bool pair = fx == 2 && reinterpret_cast<uintptr_t>(up.data) % 8 == 0 && up.stride % 8 == 0;
        const dim3 grid((lv.width + 255) / 256, lv.height);
        const uint8_t* up_data = static_cast<const uint8_t*>(up.data);
        uint8_t* lv_data = static_cast<uint8_t*>(lv.data);
        const size_t up_stride = up.stride, lv_stride = lv.stride;
        if (pair)
            GOOFY_CUDA_TRY(goofy_gpu::launch_pdl(mip_level_kernel<true>, grid, dim3(256), 0, st, up_data, up_stride,
                                                 lv_data, lv_stride, lv.width, lv.height, fx, fy));
        else
            GOOFY_CUDA_TRY(goofy_gpu::launch_pdl(mip_level_kernel<false>, grid, dim3(256), 0, st, up_data, up_stride,
                                                 lv_data, lv_stride, lv.width, lv.height, fx, fy));
        ++i;
    }
    *nlevels = n;
    return GOOFY_OK;
}

}  // extern "C"
