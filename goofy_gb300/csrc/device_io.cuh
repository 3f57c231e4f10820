// device_io.cuh -- global-memory access helpers shared by the encoder kernels.
#pragma once
#include <cstdint>

#include "block_codec.cuh"

namespace goofy_gpu {

// Source pixels are read exactly once: 128-bit loads that skip L1.
__device__ __forceinline__ uint4 ld_once16(const uint8_t* p)
{
    uint4 v;
    asm("ld.global.nc.L1::no_allocate.v4.u32 {%0, %1, %2, %3}, [%4];"
        : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
        : "l"(p));
    return v;
}

__device__ __forceinline__ uint32_t ld_once4(const uint8_t* p)
{
    uint32_t v;
    asm("ld.global.nc.L1::no_allocate.u32 %0, [%1];" : "=r"(v) : "l"(p));
    return v;
}

// Encoded blocks are written once and not read back by the kernel: streaming store.
__device__ __forceinline__ void st_stream8(uint8_t* p, uint2 v)
{
    asm volatile("st.global.cs.v2.u32 [%0], {%1, %2};" ::"l"(p), "r"(v.x), "r"(v.y) : "memory");
}

// 16 pixel words of the block at `p`: 16-byte aligned rows use one vector load
// each, 4-byte aligned rows four word loads.
__device__ __forceinline__ void load_block_rows(const uint8_t* p, size_t stride, bool vec16, uint32_t (&w)[16])
{
    if (vec16) {
#pragma unroll
        for (int y = 0; y < 4; ++y) {
            const uint4 v = ld_once16(p + (size_t)y * stride);
            w[4 * y + 0] = v.x;
            w[4 * y + 1] = v.y;
            w[4 * y + 2] = v.z;
            w[4 * y + 3] = v.w;
        }
    } else {
#pragma unroll
        for (int y = 0; y < 4; ++y)
#pragma unroll
            for (int x = 0; x < 4; ++x) w[4 * y + x] = ld_once4(p + (size_t)y * stride + 4 * x);
    }
}

// n / d for n < 2^32 with magic = floor((2^32 - 1) / d): the estimate is low by
// at most one, so a single correction makes it exact.
__device__ __forceinline__ uint32_t div_magic(uint32_t n, uint32_t d, uint32_t magic, uint32_t& rem)
{
    uint32_t q = __umulhi(n, magic);
    uint32_t r = n - q * d;
    if (r >= d) {
        ++q;
        r -= d;
    }
    rem = r;
    return q;
}

// Largest i < n with first_unit[i] <= u (first_unit[0] == 0, ascending): the
// image a work unit of a batch belongs to.
__device__ __forceinline__ uint32_t find_image(const uint32_t* first_unit, uint32_t n, uint32_t u)
{
    uint32_t lo = 0, hi = n;  // invariant: first_unit[lo] <= u < first_unit[hi] (first_unit[n] = inf)
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (first_unit[mid] <= u) lo = mid;
        else hi = mid;
    }
    return lo;
}

// etc1BrighnessRangeTocontrolByte (goofy_tc.h:1040-1057) as 128 bytes indexed by range >> 1.
__device__ __forceinline__ void fill_ctrl_lut(uint8_t* lut)
{
    for (uint32_t i = threadIdx.x; i < 128; i += blockDim.x) lut[i] = (uint8_t)etc_control_byte(2 * i);
}

}  // namespace goofy_gpu
