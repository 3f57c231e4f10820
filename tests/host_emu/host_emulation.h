// host_emulation.h -- TEST ONLY.  CPU definitions of the few CUDA device
// intrinsics block_codec.cuh uses, so that its per-block arithmetic can be
// compiled with g++ and compared with the oracle on the CPU.  Each follows the
// CUDA documentation of the intrinsic / PTX instruction it stands in for.
#pragma once
#include <algorithm>
#include <cstdint>

#define GOOFY_FN static inline

struct uint2 {
    uint32_t x, y;
};
static inline uint2 make_uint2(uint32_t x, uint32_t y) { return uint2{x, y}; }
struct uint4 {
    uint32_t x, y, z, w;
};
static inline uint4 make_uint4(uint32_t x, uint32_t y, uint32_t z, uint32_t w) { return uint4{x, y, z, w}; }

using std::max;
using std::min;

// __byte_perm(x, y, s): byte n of the result is byte (s >> 4n) & 7 of {y:x}
static inline uint32_t __byte_perm(uint32_t x, uint32_t y, uint32_t s)
{
    const uint64_t v = (uint64_t)y << 32 | x;
    uint32_t r = 0;
    for (int n = 0; n < 4; ++n) r |= (uint32_t)((v >> (8 * ((s >> (4 * n)) & 7u))) & 0xffu) << (8 * n);
    return r;
}

// __dp4a(unsigned, unsigned, unsigned): sum of the four byte products plus c
static inline uint32_t __dp4a(uint32_t a, uint32_t b, uint32_t c)
{
    uint32_t s = c;
    for (int n = 0; n < 4; ++n) s += ((a >> (8 * n)) & 0xffu) * ((b >> (8 * n)) & 0xffu);
    return s;
}

static inline uint32_t __umulhi(uint32_t a, uint32_t b) { return (uint32_t)(((uint64_t)a * b) >> 32); }

namespace goofy_gpu {
// min.u16x2 / max.u16x2: lane-wise unsigned 16-bit min / max
static inline uint32_t perm(uint32_t a, uint32_t b, uint32_t sel) { return __byte_perm(a, b, sel); }
static inline uint32_t vmin2(uint32_t a, uint32_t b)
{
    return std::min(a & 0xffffu, b & 0xffffu) | std::min(a >> 16, b >> 16) << 16;
}
static inline uint32_t vmax2(uint32_t a, uint32_t b)
{
    return std::max(a & 0xffffu, b & 0xffffu) | std::max(a >> 16, b >> 16) << 16;
}
}  // namespace goofy_gpu
