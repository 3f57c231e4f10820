// encode_kernels.cu -- image encoder kernels for sm_103a.
//
// Replaces the reference's image driver loops (goofy::compressDXT1 /
// compressETC1, GoofyTC/goofy_tc.h:1497-1557: block rows x 16-pixel strips,
// 4 blocks per goofySimdEncode call) with a grid over 4x4 blocks.
//
// Mapping: one warp owns a segment of 32*BPT consecutive blocks of one block
// row; lane l encodes blocks l, l+32, ..., l+32*(BPT-1) of the segment.  For
// each of the 4 pixel rows a warp-wide 128-bit load instruction therefore
// reads 512 contiguous bytes (every 32-byte sector fully used), and each
// 8-byte block store of the warp writes 256 contiguous bytes.  Source rows are
// read once (L1 no-allocate) and blocks are written with streaming stores:
// the kernel moves 4 B/px in and 0.5 B/px out and is meant to sit on the HBM
// roofline.  Launched with programmatic dependent launch (pdl.cuh): CTAs may
// start while the previous kernel in the stream drains and wait for it before
// their first load.
#include <cuda_runtime.h>

#include <atomic>

#include "block_codec.cuh"
#include "device_io.cuh"
#include "kernels.h"
#include "pdl.cuh"

namespace goofy_gpu {

template <SrcAccess ACCESS>
__device__ __forceinline__ void load_block(const uint8_t* p, size_t stride, uint32_t (&w)[16])
{
    load_block_rows(p, stride, ACCESS == SrcAccess::kVec16, w);
}

struct Segment {
    uint32_t by, bx0;  // block row, first block of this lane
};

template <int BPT, SrcAccess ACCESS>
__device__ __forceinline__ Segment load_segment(const uint8_t* __restrict__ src, size_t stride, uint32_t bw,
                                                uint32_t seg, uint32_t segs_per_row, uint32_t seg_magic,
                                                uint32_t lane, uint32_t (&w)[BPT][16])
{
    uint32_t sx;
    Segment sg;
    sg.by = div_magic(seg, segs_per_row, seg_magic, sx);
    sg.bx0 = sx * (32u * BPT) + lane;
    const uint8_t* row = src + (size_t)sg.by * 4u * stride;
#pragma unroll
    for (int j = 0; j < BPT; ++j) {
        const uint32_t bx = sg.bx0 + 32u * j;
        if (bx < bw) load_block<ACCESS>(row + 16u * (size_t)bx, stride, w[j]);
    }
    return sg;
}

template <int CODEC, int BPT>
__device__ __forceinline__ void encode_segment(uint8_t* __restrict__ dst, uint8_t* __restrict__ dst2, uint32_t bw,
                                               Segment sg, const uint32_t (&w)[BPT][16], const uint8_t* ctrl_lut)
{
    const size_t row = (size_t)sg.by * bw * 8u;
#pragma unroll
    for (int j = 0; j < BPT; ++j) {
        const uint32_t bx = sg.bx0 + 32u * j;
        if (bx < bw) {
            if constexpr (CODEC == kBoth) {
                const uint4 e = encode_both(w[j], ctrl_lut);
                st_stream8(dst + row + 8u * (size_t)bx, make_uint2(e.x, e.y));
                st_stream8(dst2 + row + 8u * (size_t)bx, make_uint2(e.z, e.w));
            } else {
                st_stream8(dst + row + 8u * (size_t)bx, encode_block<CODEC>(w[j], ctrl_lut));
            }
        }
    }
}

// Persistent grid: warp-segments are dealt round-robin to the resident warps;
// each warp loads its next segment before encoding the current one, so the
// 64*BPT bytes per lane of the next segment are in flight during the math.
// One segment per warp: every lane issues its 4*BPT row loads up front.
template <int CODEC, int BPT, SrcAccess ACCESS>
__global__ void __launch_bounds__(512) encode_image_kernel(const uint8_t* __restrict__ src, size_t stride,
                                                           uint8_t* __restrict__ dst, uint8_t* __restrict__ dst2,
                                                           uint32_t bw, uint32_t total_segs, uint32_t segs_per_row,
                                                           uint32_t seg_magic)
{
    pdl_launch_dependents();
    __shared__ uint8_t ctrl_lut[128];
    if constexpr (CODEC != kBC1) {
        fill_ctrl_lut(ctrl_lut);
        __syncthreads();
    }
    const uint32_t seg = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (seg >= total_segs) return;
    pdl_wait();
    uint32_t w[BPT][16];
    const Segment sg = load_segment<BPT, ACCESS>(src, stride, bw, seg, segs_per_row, seg_magic, threadIdx.x & 31u, w);
    encode_segment<CODEC, BPT>(dst, dst2, bw, sg, w, ctrl_lut);
}

template <int CODEC, int BPT, SrcAccess ACCESS>
__global__ void __launch_bounds__(512) encode_image_persistent(const uint8_t* __restrict__ src, size_t stride,
                                                               uint8_t* __restrict__ dst, uint32_t bw,
                                                               uint32_t total_segs, uint32_t segs_per_row,
                                                               uint32_t seg_magic)
{
    pdl_launch_dependents();
    __shared__ uint8_t ctrl_lut[128];
    if constexpr (CODEC == kETC1S) {
        fill_ctrl_lut(ctrl_lut);
        __syncthreads();
    }
    pdl_wait();
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t warp_stride = gridDim.x * (blockDim.x >> 5);
    uint32_t seg = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    uint32_t a[BPT][16], b[BPT][16];
    Segment sa{}, sb{};
    if (seg < total_segs) sa = load_segment<BPT, ACCESS>(src, stride, bw, seg, segs_per_row, seg_magic, lane, a);
    while (seg < total_segs) {
        uint32_t next = seg + warp_stride;
        if (next < total_segs) sb = load_segment<BPT, ACCESS>(src, stride, bw, next, segs_per_row, seg_magic, lane, b);
        encode_segment<CODEC, BPT>(dst, nullptr, bw, sa, a, ctrl_lut);
        seg = next;
        if (seg >= total_segs) break;
        next = seg + warp_stride;
        if (next < total_segs) sa = load_segment<BPT, ACCESS>(src, stride, bw, next, segs_per_row, seg_magic, lane, a);
        encode_segment<CODEC, BPT>(dst, nullptr, bw, sb, b, ctrl_lut);
        seg = next;
    }
}

template <int CODEC, int BPT, SrcAccess ACCESS>
static int resident_ctas(uint32_t threads)
{
    // cached per instantiation, device and block size
    static std::atomic<int> cached[64][3];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 1;
    const int slot = threads == 128 ? 0 : threads == 256 ? 1 : 2;
    int n = cached[dev][slot].load(std::memory_order_relaxed);
    if (n == 0) {
        int sms = 0, per_sm = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, encode_image_persistent<CODEC, BPT, ACCESS>, threads, 0);
        n = (sms > 0 ? sms : 1) * (per_sm > 0 ? per_sm : 1);
        cached[dev][slot].store(n, std::memory_order_relaxed);
    }
    return n;
}

// The image kernels run with the shared-memory-heavy carveout of the
// bulk-copy kernel (their loads bypass L1 anyway), so alternating the two
// does not reconfigure the SMs between launches.
template <typename K>
static void prefer_shared(K kernel, int slot)
{
    static std::atomic<bool> done[64][2];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64 || done[dev][slot].load(std::memory_order_relaxed))
        return;
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared) !=
        cudaSuccess)
        cudaGetLastError();
    done[dev][slot].store(true, std::memory_order_relaxed);
}

template <int CODEC, int BPT, SrcAccess ACCESS>
static cudaError_t launch_t(const uint8_t* src, size_t stride, uint8_t* dst, uint8_t* dst2, uint32_t bw, uint32_t bh,
                            uint32_t threads, bool persistent, cudaStream_t stream)
{
    constexpr bool kHasPersistent = BPT <= 2 && CODEC != kBoth;
    prefer_shared(encode_image_kernel<CODEC, BPT, ACCESS>, 0);
    if constexpr (kHasPersistent) prefer_shared(encode_image_persistent<CODEC, BPT, ACCESS>, 1);
    const uint32_t segs = (bw + 32u * BPT - 1) / (32u * BPT);
    const uint64_t total = (uint64_t)segs * bh;
    if (total > 0x7fffffffull) return cudaErrorInvalidValue;
    const uint32_t wpc = threads / 32u;
    uint64_t ctas = (total + wpc - 1) / wpc;
    const uint32_t magic = 0xffffffffu / segs;
    if constexpr (kHasPersistent) {
        if (persistent) {
            const uint64_t resident = (uint64_t)resident_ctas<CODEC, BPT, ACCESS>(threads);
            if (ctas > resident) ctas = resident;
            return launch_pdl(encode_image_persistent<CODEC, BPT, ACCESS>, dim3((unsigned)ctas), dim3(threads), 0,
                              stream, src, stride, dst, bw, (uint32_t)total, segs, magic);
        }
    }
    return launch_pdl(encode_image_kernel<CODEC, BPT, ACCESS>, dim3((unsigned)ctas), dim3(threads), 0, stream, src,
                      stride, dst, dst2, bw, (uint32_t)total, segs, magic);
}

template <int CODEC, SrcAccess ACCESS>
static cudaError_t launch_bpt(const uint8_t* src, size_t stride, uint8_t* dst, uint8_t* dst2, uint32_t bw,
                              uint32_t bh, Tile tile, cudaStream_t stream)
{
    switch (tile.bpt) {
    case 1: return launch_t<CODEC, 1, ACCESS>(src, stride, dst, dst2, bw, bh, tile.threads, tile.persistent, stream);
    case 2: return launch_t<CODEC, 2, ACCESS>(src, stride, dst, dst2, bw, bh, tile.threads, tile.persistent, stream);
    case 4:
        if constexpr (CODEC != kBoth) return launch_t<CODEC, 4, ACCESS>(src, stride, dst, dst2, bw, bh, tile.threads, false, stream);
        return cudaErrorInvalidValue;
    default: return cudaErrorInvalidValue;
    }
}

template <int CODEC>
static cudaError_t launch_access(const uint8_t* src, size_t stride, uint8_t* dst, uint8_t* dst2, uint32_t bw,
                                 uint32_t bh, Tile tile, SrcAccess access, cudaStream_t stream)
{
    if (access == SrcAccess::kVec16)
        return launch_bpt<CODEC, SrcAccess::kVec16>(src, stride, dst, dst2, bw, bh, tile, stream);
    return launch_bpt<CODEC, SrcAccess::kWord4>(src, stride, dst, dst2, bw, bh, tile, stream);
}

cudaError_t launch_image(int codec, const uint8_t* src, size_t stride, uint8_t* dst, uint32_t width,
                         uint32_t height, Tile tile, SrcAccess access, cudaStream_t stream, uint8_t* dst2)
{
    if (!tile_valid(tile)) return cudaErrorInvalidValue;
    if (codec != kBC1 && codec != kETC1S && (codec != kBoth || !dst2)) return cudaErrorInvalidValue;
    const uint32_t bw = width / 4, bh = height / 4;
    if (bw == 0 || bh == 0) return cudaSuccess;
    if (tile.persistent == 2) {
        if (access == SrcAccess::kVec16)
            return launch_image_tma(codec, src, stride, dst, width, height, tile, stream, dst2);
        tile.persistent = 0;  // word-aligned rows: the register-loading kernel with the same shape
    }
    if (codec == kBC1) return launch_access<kBC1>(src, stride, dst, nullptr, bw, bh, tile, access, stream);
    if (codec == kETC1S) return launch_access<kETC1S>(src, stride, dst, nullptr, bw, bh, tile, access, stream);
    return launch_access<kBoth>(src, stride, dst, dst2, bw, bh, tile, access, stream);
}

}  // namespace goofy_gpu
