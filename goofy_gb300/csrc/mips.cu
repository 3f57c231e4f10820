// mips.cu -- mip-chain generation on the device, feeding the batch encoder.
//
// The reference has no mip generator (its harness only builds an RGB565 x2
// downsample as a quality baseline, Src/main.cpp:501-557); textures with mip
// chains are encoded level by level from levels the caller made.  Here each
// level is produced from the one above by a 2x2 box filter with rounding,
// (a + b + c + d + 2) >> 2 per channel, an axis that is already 4 pixels
// being copied instead of halved -- the rule of the workload generator's
// goofy_synth_downsample, so device and host chains are bit-identical.  One
// launch per level (each level depends on the previous one); a thread makes
// one output pixel, channel pairs summed in 16-bit lanes.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/goofy_gpu.h"
#include "host_util.h"

namespace {

__device__ __forceinline__ uint32_t box4(uint32_t a, uint32_t b, uint32_t c, uint32_t d)
{
    const uint32_t m = 0x00ff00ffu;
    const uint32_t rb = (a & m) + (b & m) + (c & m) + (d & m) + 0x00020002u;
    const uint32_t ga = ((a >> 8) & m) + ((b >> 8) & m) + ((c >> 8) & m) + ((d >> 8) & m) + 0x00020002u;
    return ((rb >> 2) & m) | (((ga >> 2) & m) << 8);
}

__global__ void __launch_bounds__(256) mip_level_kernel(const uint8_t* __restrict__ src, size_t src_stride,
                                                        uint8_t* __restrict__ dst, size_t dst_stride, uint32_t dw,
                                                        uint32_t dh, uint32_t fx, uint32_t fy)
{
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= dw || y >= dh) return;
    const uint8_t* r0 = src + (size_t)(y * fy) * src_stride + 4u * (size_t)(x * fx);
    const uint8_t* r1 = r0 + src_stride * (fy - 1);
    const uint32_t a = __ldg(reinterpret_cast<const uint32_t*>(r0));
    const uint32_t b = __ldg(reinterpret_cast<const uint32_t*>(r0 + 4 * (fx - 1)));
    const uint32_t c = __ldg(reinterpret_cast<const uint32_t*>(r1));
    const uint32_t d = __ldg(reinterpret_cast<const uint32_t*>(r1 + 4 * (fx - 1)));
    *reinterpret_cast<uint32_t*>(dst + (size_t)y * dst_stride + 4u * (size_t)x) = box4(a, b, c, d);
}

bool pow2(uint32_t v) { return v && !(v & (v - 1)); }

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
    for (uint32_t i = 1; i < n; ++i) {
        const goofy_gpu_level& up = levels[i - 1];
        const uint32_t dw = up.width / 2 >= 4 ? up.width / 2 : 4, dh = up.height / 2 >= 4 ? up.height / 2 : 4;
        const uint32_t fx = up.width > dw ? 2 : 1, fy = up.height > dh ? 2 : 1;
        const size_t pitch = pitch_of(dw);
        mip_level_kernel<<<dim3((dw + 255) / 256, dh), 256, 0, st>>>(static_cast<const uint8_t*>(up.data), up.stride,
                                                                      out, pitch, dw, dh, fx, fy);
        GOOFY_CUDA_TRY(cudaGetLastError());
        levels[i] = goofy_gpu_level{out, dw, dh, (uint32_t)pitch};
        out += pitch * dh;
    }
    *nlevels = n;
    return GOOFY_OK;
}

}  // extern "C"
