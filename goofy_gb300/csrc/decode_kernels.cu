// decode_kernels.cu -- BC1 / ETC1 block decoding and the encode-quality error
// reduction on sm_103a.
//
// The reference checks quality on the CPU: it decodes every block with its
// harness decoders (Src/decoder.cpp: DecompressColour :819-871 for BC1,
// decompressBlockDiffFlipC :388-678 for ETC1) and sums squared channel
// differences in getMsePsnr (Src/main.cpp:403-469).  Here one thread decodes
// one block (BC1: both endpoint orders; ETC1: individual and differential
// modes, both flips; ETC2-only differential overflows are counted as
// unsupported and decoded as black) and either stores the 16 pixels or
// compares them with the source pixels, summing squared differences per
// channel exactly in integers (64-bit per thread over a grid stride, then
// shuffles and shared memory, one 64-bit atomic per CTA and channel).
#include <cuda_runtime.h>

#include <atomic>

#include "batch.h"
#include "block_codec.cuh"
#include "block_decode.cuh"
#include "decode.h"
#include "device_io.cuh"
#include "pdl.cuh"

namespace goofy_gpu {

// Threads per CTA of every decoding kernel: the palette column stride, a
// constant so that a pixel's palette address is a shift and an add.
constexpr uint32_t kDecodeThreads = 256;

__device__ __forceinline__ uint2 load_block8(const uint8_t* p)
{
    uint2 v;
    asm("ld.global.nc.L1::no_allocate.v2.u32 {%0, %1}, [%2];" : "=r"(v.x), "=r"(v.y) : "l"(p));
    return v;
}

template <int CODEC>
__global__ void __launch_bounds__(kDecodeThreads) decode_image_kernel(const uint8_t* __restrict__ blocks, uint32_t bw,
                                                           uint32_t nblk, uint8_t* __restrict__ rgba, size_t stride,
                                                           unsigned long long* __restrict__ unsupported)
{
    pdl_launch_dependents();
    __shared__ uint32_t pal[8 * kDecodeThreads];
    const uint32_t i = blockIdx.x * kDecodeThreads + threadIdx.x;
    bool ok = true;
    pdl_wait();
    if (i < nblk) {
        const uint32_t by = i / bw, bx = i - by * bw;
        uint32_t px[16];
        ok = decode_block<CODEC>(load_block8(blocks + 8u * (size_t)i), pal + threadIdx.x, kDecodeThreads, px);
        uint8_t* row = rgba + (size_t)by * 4u * stride + 16u * (size_t)bx;
#pragma unroll
        for (int y = 0; y < 4; ++y)
            *reinterpret_cast<uint4*>(row + (size_t)y * stride) = make_uint4(px[4 * y], px[4 * y + 1], px[4 * y + 2],
                                                                             px[4 * y + 3]);
    }
    const unsigned bad = __ballot_sync(0xffffffffu, !ok);
    if (bad && (threadIdx.x & 31u) == 0) atomicAdd(unsupported, (unsigned long long)__popc(bad));
}

// Sums of squared channel differences of one 4-pixel row: |a-b| per byte,
// bytes regrouped so each word holds one channel of the 4 pixels, then a
// dot product of each channel word with itself.
__device__ __forceinline__ void accumulate_row(const uint32_t (&a)[4], const uint32_t (&b)[4], uint32_t (&acc)[4])
{
    uint32_t d[4];
#pragma unroll
    for (int x = 0; x < 4; ++x) d[x] = __vabsdiffu4(a[x], b[x]);
    const uint32_t t0 = __byte_perm(d[0], d[1], 0x5140), t1 = __byte_perm(d[2], d[3], 0x5140);
    const uint32_t t2 = __byte_perm(d[0], d[1], 0x7362), t3 = __byte_perm(d[2], d[3], 0x7362);
    const uint32_t ch[4] = {__byte_perm(t0, t1, 0x5410), __byte_perm(t0, t1, 0x7632), __byte_perm(t2, t3, 0x5410),
                            __byte_perm(t2, t3, 0x7632)};
#pragma unroll
    for (int c = 0; c < 4; ++c) acc[c] = __dp4a(ch[c], ch[c], acc[c]);
}

// The harness's luminosity difference (0.21 R + 0.72 G + 0.07 B of a pixel
// read as a little-endian u32, R = byte 2) in hundredths, which is exact in
// integers: 21 * d(byte 2) + 72 * d(byte 1) + 7 * d(byte 0).  Two byte dot
// products: the second multiplies b's unsigned bytes by the negated weights
// (signed bytes) and adds the first, so no subtraction is needed.
__device__ __forceinline__ int luma_diff(uint32_t a, uint32_t b)
{
    constexpr uint32_t kWeights = 0x00154807u;     // bytes 0..3: 7, 72, 21, 0
    constexpr uint32_t kNegWeights = 0x00ebb8f9u;  // bytes 0..3: -7, -72, -21, 0
    int d;
    asm("dp4a.u32.s32 %0, %1, %2, %3;" : "=r"(d) : "r"(b), "r"(kNegWeights), "r"((int)__dp4a(a, kWeights, 0u)));
    return d;
}

// Squared luminosity differences summed over a row of 4 pixels (at most
// 4 * 25500^2 < 2^32).
__device__ __forceinline__ uint32_t luma_row(const uint32_t (&a)[4], const uint32_t (&b)[4])
{
    uint32_t acc = 0;
#pragma unroll
    for (int x = 0; x < 4; ++x) {
        const int d = luma_diff(a[x], b[x]);
        acc += (uint32_t)(d * d);
    }
    return acc;
}

// Resident grid: each thread walks blocks with a grid stride, keeps 64-bit
// sums, then the CTA reduces (shuffles, shared memory) and adds its six
// totals with one atomic each.  Register caps for 4 (BC1, 64 registers) /
// 3 (ETC1, 80) CTAs per SM, no spills: uncapped, ETC1 took 94 registers and
// 2 CTAs per SM (51.3 against 47.4 us at 8192^2); capped at 4 CTAs it
// spilled (50.9 us).
template <int CODEC>
__global__ void __launch_bounds__(kDecodeThreads, CODEC == kBC1 ? 4 : 3)
    block_error_kernel(const uint8_t* __restrict__ blocks, uint32_t bw, uint32_t nblk, const uint8_t* __restrict__ src,
                       size_t stride, bool vec16, unsigned long long* __restrict__ sums)
{
    pdl_launch_dependents();
    __shared__ uint32_t pal[8 * kDecodeThreads];
    unsigned long long s[6] = {0, 0, 0, 0, 0, 0};
    const uint32_t bw_magic = 0xffffffffu / bw;
    pdl_wait();
    // software pipeline: the next block's source rows and code are loaded
    // before this block is decoded and compared
    const uint32_t step = gridDim.x * kDecodeThreads;
    uint32_t i = blockIdx.x * kDecodeThreads + threadIdx.x;
    uint32_t w[16];
    uint2 blk = make_uint2(0, 0);
    if (i < nblk) {
        uint32_t bx;
        const uint32_t by = div_magic(i, bw, bw_magic, bx);
        load_block_rows(src + (size_t)by * 4u * stride + 16u * (size_t)bx, stride, vec16, w);
        blk = load_block8(blocks + 8u * (size_t)i);
    }
    for (; i < nblk; i += step) {
        uint32_t px[16], cur[16];
#pragma unroll
        for (int k = 0; k < 16; ++k) cur[k] = w[k];
        const uint2 cur_blk = blk;
        if (i + step < nblk) {
            uint32_t bx;
            const uint32_t by = div_magic(i + step, bw, bw_magic, bx);
            load_block_rows(src + (size_t)by * 4u * stride + 16u * (size_t)bx, stride, vec16, w);
            blk = load_block8(blocks + 8u * (size_t)(i + step));
        }
        const bool ok = decode_block<CODEC>(cur_blk, pal + threadIdx.x, kDecodeThreads, px);
        uint32_t acc[4] = {0, 0, 0, 0};  // one block: at most 16 * 255^2 per channel
#pragma unroll
        for (int y = 0; y < 4; ++y) {
            const uint32_t a[4] = {cur[4 * y], cur[4 * y + 1], cur[4 * y + 2], cur[4 * y + 3]};
            const uint32_t b[4] = {px[4 * y], px[4 * y + 1], px[4 * y + 2], px[4 * y + 3]};
            accumulate_row(a, b, acc);
            s[5] += luma_row(a, b);
        }
#pragma unroll
        for (int c = 0; c < 4; ++c) s[c] += acc[c];
        s[4] += ok ? 0u : 1u;
    }
    __shared__ unsigned long long part[6][8];
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
#pragma unroll
    for (int c = 0; c < 6; ++c) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s[c] += __shfl_xor_sync(0xffffffffu, s[c], o);
        if (lane == 0) part[c][warp] = s[c];
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        unsigned long long t = 0;
        for (uint32_t k = 0; k < (kDecodeThreads >> 5); ++k) t += part[threadIdx.x][k];
        if (t) atomicAdd(&sums[threadIdx.x], t);
    }
}

// The error sums of every image of a batch (the request server's quality
// measurement): the batch's work units, pulled from a counter as in the
// encoder's batch kernel, decode the image's blocks (`dst`) and compare them
// with its source; a warp sums its unit and adds six totals to the image's
// sums[6 * image + c].
__global__ void __launch_bounds__(kDecodeThreads) quality_batch_kernel(const BatchImage* __restrict__ images, uint32_t n_images,
                                                            const uint32_t* __restrict__ first_unit,
                                                            uint32_t total_units, uint32_t unit_blocks,
                                                            uint32_t* __restrict__ work_counter,
                                                            unsigned long long* __restrict__ sums)
{
    __shared__ uint32_t pal[8 * kDecodeThreads];
    const uint32_t lane = threadIdx.x & 31u;
    for (;;) {
        uint32_t u = 0;
        if (lane == 0) u = atomicAdd(work_counter, 1u);
        u = __shfl_sync(0xffffffffu, u, 0);
        if (u >= total_units) return;
        const uint32_t ii = find_image(first_unit, n_images, u);
        const BatchImage im = images[ii];
        const uint32_t first = (u - im.first_unit) * unit_blocks, last = min(first + unit_blocks, im.bw * im.bh);
        // per lane at most 2048 blocks of a unit: 2048 * 16 * 255^2 < 2^32 per channel
        uint32_t acc[4] = {0, 0, 0, 0}, bad = 0;
        unsigned long long ys = 0;
        for (uint32_t b = first + lane; b < last; b += 32u) {
            uint32_t bx;
            const uint32_t by = div_magic(b, im.bw, im.bw_magic, bx);
            uint32_t px[16], w[16];
            const uint2 blk = load_block8(im.dst + 8u * (size_t)b);
            const bool ok = im.codec == kBC1 ? decode_block<kBC1>(blk, pal + threadIdx.x, kDecodeThreads, px)
                                             : decode_block<kETC1S>(blk, pal + threadIdx.x, kDecodeThreads, px);
            load_block_rows(im.src + (size_t)by * 4u * im.stride + 16u * (size_t)bx, im.stride, im.vec16 != 0, w);
#pragma unroll
            for (int y = 0; y < 4; ++y) {
                const uint32_t a[4] = {w[4 * y], w[4 * y + 1], w[4 * y + 2], w[4 * y + 3]};
                const uint32_t d[4] = {px[4 * y], px[4 * y + 1], px[4 * y + 2], px[4 * y + 3]};
                accumulate_row(a, d, acc);
                ys += luma_row(a, d);
            }
            bad += ok ? 0u : 1u;
        }
        unsigned long long t[6] = {acc[0], acc[1], acc[2], acc[3], bad, ys};
#pragma unroll
        for (int c = 0; c < 6; ++c) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) t[c] += __shfl_xor_sync(0xffffffffu, t[c], o);
        }
        if (lane == 0)
#pragma unroll
            for (int c = 0; c < 6; ++c)
                if (t[c]) atomicAdd(&sums[6u * ii + c], t[c]);
    }
}

cudaError_t launch_quality_batch(const BatchImage* images, uint32_t n_images, const uint32_t* first_unit,
                                 uint32_t total_units, uint32_t unit_blocks, uint32_t* work_counter,
                                 unsigned long long* sums, cudaStream_t stream)
{
    if (total_units == 0) return cudaSuccess;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const uint64_t warps = total_units, ctas = (warps + 7) / 8;
    const uint32_t grid = (uint32_t)(ctas < (uint64_t)sms * 8u ? ctas : (uint64_t)sms * 8u);
    quality_batch_kernel<<<grid, kDecodeThreads, 0, stream>>>(images, n_images, first_unit, total_units, unit_blocks,
                                                   work_counter, sums);
    return cudaGetLastError();
}

cudaError_t launch_decode(int codec, const uint8_t* blocks, uint32_t width, uint32_t height, uint8_t* rgba,
                          size_t stride, unsigned long long* unsupported, cudaStream_t stream)
{
    const uint32_t bw = width / 4, nblk = bw * (height / 4);
    if (nblk == 0) return cudaSuccess;
    const uint32_t grid = (nblk + kDecodeThreads - 1) / kDecodeThreads;
    if (codec == kBC1)
        return launch_pdl(decode_image_kernel<kBC1>, dim3(grid), dim3(kDecodeThreads), 0, stream, blocks, bw, nblk, rgba, stride,
                          unsupported);
    return launch_pdl(decode_image_kernel<kETC1S>, dim3(grid), dim3(kDecodeThreads), 0, stream, blocks, bw, nblk, rgba, stride,
                      unsupported);
}

namespace {

// Resident CTAs of `kernel` per SM on device `dev` (cached per device and
// slot), at least 1.
template <typename K>
uint32_t resident_per_sm(K kernel, int dev, int slot)
{
    static std::atomic<uint32_t> cache[64][2];
    if (dev < 0 || dev >= 64) dev = 0;
    uint32_t n = cache[dev][slot].load(std::memory_order_relaxed);
    if (n == 0) {
        int per_sm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kDecodeThreads, 0) != cudaSuccess) {
            cudaGetLastError();
            per_sm = 0;
        }
        n = per_sm > 0 ? (uint32_t)per_sm : 1u;
        cache[dev][slot].store(n, std::memory_order_relaxed);
    }
    return n;
}

}  // namespace

cudaError_t launch_block_error(int codec, const uint8_t* blocks, const uint8_t* src, uint32_t width, uint32_t height,
                               size_t stride, bool vec16, unsigned long long* sums, cudaStream_t stream)
{
    const uint32_t bw = width / 4, nblk = bw * (height / 4);
    if (nblk == 0) return cudaSuccess;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    // One wave: as many CTAs as fit on the GPU at once, each thread striding
    // over its share of the blocks.  A grid of 8 CTAs per SM ran in 2.7
    // waves for BC1 and left SMs part-empty in the last one (50.6 against
    // 47.2 us at 8192^2).
    const uint32_t per_sm = codec == kBC1 ? resident_per_sm(block_error_kernel<kBC1>, dev, 0)
                                          : resident_per_sm(block_error_kernel<kETC1S>, dev, 1);
    const uint32_t grid = min((nblk + kDecodeThreads - 1) / kDecodeThreads, (uint32_t)(sms > 0 ? sms : 1) * per_sm);
    if (codec == kBC1)
        return launch_pdl(block_error_kernel<kBC1>, dim3(grid), dim3(kDecodeThreads), 0, stream, blocks, bw, nblk, src, stride,
                          vec16, sums);
    return launch_pdl(block_error_kernel<kETC1S>, dim3(grid), dim3(kDecodeThreads), 0, stream, blocks, bw, nblk, src, stride,
                      vec16, sums);
}

}  // namespace goofy_gpu
