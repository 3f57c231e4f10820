// encode_tma.cu -- the image encoder fed by bulk asynchronous copies.
//
// A resident grid of CTAs, each with one producer warp and C compute warps
// (C = threads / 32).  Work is cut into tiles of 4 pixel rows x (32 * C * BPT)
// blocks; CTA b takes tiles b, b + grid, ...  The producer's elected lane
// copies each tile's four row segments (16 bytes per block, contiguous in the
// source) into the next free stage of a shared-memory ring with
// cp.async.bulk, counted on that stage's "full" mbarrier; compute warps wait
// for it, pull their blocks into registers with conflict-free 128-bit shared
// loads (lane l of a warp reads 16 contiguous bytes, the warp 512), run the
// same block codec as every other kernel, store 8 bytes per block with
// streaming stores and release the stage on its "empty" mbarrier.  Global
// loads never sit in the compute warps' registers, so the integer math of one
// tile overlaps the HBM reads of the next stages.
//
// Launched with programmatic dependent launch (pdl.cuh): the prologue
// (barriers, control-byte table) runs while the previous kernel in the stream
// drains, and no copy is issued before that kernel has completed.
//
// Needs 16-byte aligned source rows (base and stride); other images take the
// register-loading kernels.  Every wait is bounded (async_copy.cuh): a stuck
// barrier ends the kernel with a counted time-out instead of a hang, and the
// producer then waits (bounded) for the copies it issued before its CTA exits.
#include <cuda_runtime.h>

#include <atomic>

#include "async_copy.cuh"
#include "batch.h"
#include "block_codec.cuh"
#include "device_io.cuh"
#include "kernels.h"
#include "pdl.cuh"

namespace goofy_gpu {

__device__ unsigned int g_pipeline_timeouts;

// CTAs per SM each instantiation is compiled for (register caps that keep
// that many resident; every ring fits that many times in shared memory).  With
// two blocks a thread the ETC1s codec wants about 80 registers, so the
// 512-thread CTA runs alone on its SM; the 256-thread one is capped at 72 to
// fit 3.  The 128-thread CTA stays at 4: 5 would put 7 warps on one scheduler,
// whose quarter of the register file then caps them at 72 with spills.
__host__ __device__ constexpr int tma_min_ctas(uint32_t bpt, uint32_t compute_threads)
{
    return bpt == 1 ? (compute_threads == 512 ? 2 : compute_threads == 256 ? 4 : 7)
                    : (compute_threads == 512 ? 1 : compute_threads == 256 ? 3 : 4);
}

struct TmaLayout {
    uint32_t tile_blocks, row_bytes, stage_bytes, stages;
};

__host__ __device__ constexpr TmaLayout tma_layout(uint32_t compute_threads, uint32_t bpt)
{
    TmaLayout l{};
    l.tile_blocks = compute_threads * bpt;
    l.row_bytes = 16u * l.tile_blocks;
    l.stage_bytes = 4u * l.row_bytes;
    // ring budget scaled with the CTA (112 KB at 512 compute threads), so the
    // CTAs the registers allow per SM also fit in shared memory; at least 3
    // stages for a CTA alone on its SM (a stage is released only once it has
    // been encoded, so 2 would leave that SM a single stage of lookahead)
    const uint32_t s = (114688u / 512u * compute_threads) / l.stage_bytes;
    const uint32_t lo = tma_min_ctas(bpt, compute_threads) == 1 ? 3u : 2u;
    l.stages = s < lo ? lo : s > 6u ? 6u : s;
    return l;
}

constexpr size_t tma_smem_bytes(const TmaLayout& l) { return (size_t)l.stages * (l.stage_bytes + 16u) + 128u; }

// Tiles (batch: units) of a CTA whose rows its producer asks L2 for before
// the dependency wait, while the previous kernel drains.  Two of the three
// stages measured best: with all three the launch starts later (8192^2
// ETC1s 45.3 against 44.8 us, 4096^2 13.9 against 13.2 us), with one the
// first copies find less in L2.
#ifndef GOOFY_L2_PREFETCH_TILES
#define GOOFY_L2_PREFETCH_TILES 2
#endif
__host__ __device__ constexpr uint32_t l2_prefetch_tiles(const TmaLayout& l)
{
    return (uint32_t)GOOFY_L2_PREFETCH_TILES < l.stages ? (uint32_t)GOOFY_L2_PREFETCH_TILES : l.stages;
}

// Encodes the blocks of one stage held in shared memory (4 rows of
// row_bytes, block b at 16 * b in each) and stores those below nb at
// out + 8 * b (and out2, for both codecs).  Thread `lane` of compute warp
// `warp` takes blocks (warp * BPT + j) * 32 + lane.  Every thread loads and
// encodes all its slots, also past nb (a narrower tile at the right edge):
// such a slot holds whatever an earlier tile left in the stage, which
// nothing writes while the stage is held, and its result is dropped.  Only
// the stores are conditional, so the loads and the codec run without
// branches.
template <int CODEC, int BPT>
__device__ __forceinline__ void encode_stage(const uint8_t* buf, uint32_t row_bytes, uint32_t warp, uint32_t lane,
                                             uint32_t nb, uint8_t* out, uint8_t* out2, const uint8_t* ctrl_lut)
{
    uint32_t w[BPT][16];
#pragma unroll
    for (int j = 0; j < BPT; ++j) {
        const uint32_t b = (warp * BPT + j) * 32u + lane;
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const uint4 v = *reinterpret_cast<const uint4*>(buf + r * row_bytes + 16u * b);
            w[j][4 * r + 0] = v.x;
            w[j][4 * r + 1] = v.y;
            w[j][4 * r + 2] = v.z;
            w[j][4 * r + 3] = v.w;
        }
    }
#pragma unroll
    for (int j = 0; j < BPT; ++j) {
        const uint32_t b = (warp * BPT + j) * 32u + lane;
        if constexpr (CODEC == kBoth) {
            const uint4 e = encode_both(w[j], ctrl_lut);
            if (b < nb) {
                st_stream8(out + 8u * (size_t)b, make_uint2(e.x, e.y));
                st_stream8(out2 + 8u * (size_t)b, make_uint2(e.z, e.w));
            }
        } else {
            const uint2 e = encode_block<CODEC>(w[j], ctrl_lut);
            if (b < nb) st_stream8(out + 8u * (size_t)b, e);
        }
    }
}

template <int CODEC, int BPT, int COMPUTE>
__global__ void __launch_bounds__(COMPUTE + 32, tma_min_ctas(BPT, COMPUTE))
    encode_image_tma(const uint8_t* __restrict__ src, size_t stride, uint8_t* __restrict__ dst,
                     uint8_t* __restrict__ dst2, uint32_t bw, uint32_t tiles_per_row, uint32_t total_tiles,
                     uint32_t tile_magic)
{
    pdl_launch_dependents();
    extern __shared__ __align__(128) uint8_t smem[];
    __shared__ uint32_t abort_flag;
    constexpr uint32_t compute_warps = COMPUTE / 32;
    constexpr TmaLayout L = tma_layout(COMPUTE, BPT);
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + L.stages * L.stage_bytes);
    uint64_t* empty = full + L.stages;
    uint8_t* ctrl_lut = reinterpret_cast<uint8_t*>(empty + L.stages);
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;

    if (threadIdx.x == 0) {
        for (uint32_t s = 0; s < L.stages; ++s) {
            mbar_init(&full[s], 1u);
            mbar_init(&empty[s], compute_warps);
        }
        abort_flag = 0u;
        mbar_init_fence();
    }
    if constexpr (CODEC != kBC1) fill_ctrl_lut(ctrl_lut);
    __syncthreads();
    if (warp == compute_warps && lane == 0) {
        // While the previous kernel in the stream drains, ask L2 for the rows
        // of this CTA's first tiles.  Only a hint: no data enters the CTA
        // before pdl_wait(), and L2 is coherent with the previous kernel's
        // writes, so the copies after the wait still read what it wrote.
        uint32_t n = 0;
        for (uint32_t t = blockIdx.x; t < total_tiles && n < l2_prefetch_tiles(L); t += gridDim.x, ++n) {
            uint32_t tx;
            const uint32_t by = div_magic(t, tiles_per_row, tile_magic, tx);
            const uint32_t bx0 = tx * L.tile_blocks;
            const uint32_t bytes = 16u * min(L.tile_blocks, bw - bx0);
            const uint8_t* row = src + (size_t)by * 4u * stride + 16u * (size_t)bx0;
#pragma unroll
            for (int r = 0; r < 4; ++r) bulk_prefetch_l2(row + r * stride, bytes);
        }
    }
    pdl_wait();  // no global memory access before the previous kernel in the stream is done

    if (warp == compute_warps) {  // producer
        if (lane != 0) return;
        // Rows are read once: evict-first in L2 (single-codec launches back to
        // back: 4096^2 ETC1s 12.3 against 13.2 us, BC1 11.2 against 12.4 us).
        // The two-codec pass marks half of them: with all it measured 0.9 us
        // slower at 8192^2; with half, as fast there and 0.4 us faster at 4096^2.
        const uint64_t policy = CODEC == kBoth ? l2_evict_first_half_policy() : l2_evict_first_policy();
        uint32_t issued = 0, slot = 0, phase = 0;
        for (uint32_t t = blockIdx.x; t < total_tiles; t += gridDim.x) {
            if (issued >= L.stages && !mbar_wait(&empty[slot], phase ^ 1u, &abort_flag, &g_pipeline_timeouts))
                break;
            uint32_t tx;
            const uint32_t by = div_magic(t, tiles_per_row, tile_magic, tx);
            const uint32_t bx0 = tx * L.tile_blocks;
            const uint32_t nb = min(L.tile_blocks, bw - bx0);
            const uint32_t bytes = 16u * nb;
            mbar_arrive_expect_tx(&full[slot], 4u * bytes);
            const uint8_t* row = src + (size_t)by * 4u * stride + 16u * (size_t)bx0;
            uint8_t* buf = smem + slot * L.stage_bytes;
#pragma unroll
            for (int r = 0; r < 4; ++r)
                bulk_copy_g2s_hint(buf + r * L.row_bytes, row + r * stride, bytes, &full[slot], policy);
            ++issued;
            if (++slot == L.stages) {
                slot = 0;
                phase ^= 1u;
            }
        }
        if (*static_cast<volatile uint32_t*>(&abort_flag)) {
            // the copies of the last stages may still be landing: wait for them (bounded) before exiting
            const uint32_t n = issued < L.stages ? issued : L.stages;
            for (uint32_t i = issued - n; i < issued; ++i)
                mbar_wait(&full[i % L.stages], (i / L.stages) & 1u, nullptr, &g_pipeline_timeouts);
        }
        return;
    }

    uint32_t slot = 0, phase = 0;
    for (uint32_t t = blockIdx.x; t < total_tiles; t += gridDim.x) {
        if (!mbar_wait(&full[slot], phase, &abort_flag, &g_pipeline_timeouts)) break;
        uint32_t tx;
        const uint32_t by = div_magic(t, tiles_per_row, tile_magic, tx);
        const uint32_t bx0 = tx * L.tile_blocks;
        const uint32_t nb = min(L.tile_blocks, bw - bx0);
        const uint8_t* buf = smem + slot * L.stage_bytes;
        const size_t o = ((size_t)by * bw + bx0) * 8u;
        if (warp * (BPT * 32u) < nb)  // warps wholly past a narrower tile's last block skip it
            encode_stage<CODEC, BPT>(buf, L.row_bytes, warp, lane, nb, dst + o,
                                     CODEC == kBoth ? dst2 + o : nullptr, ctrl_lut);
        // Release the stage only now.  An arrival right after the shared loads
        // can overtake them: the loads wait in the load/store queue (behind
        // other kernels' global loads when SMs are shared) while the arrival
        // completes at once, and the producer's next copy into the stage then
        // lands before they read it (seen with a concurrent register-loading
        // kernel: rows of the stage's next tile inside this tile's blocks).
        // The stores cannot issue before the blocks they write are encoded
        // from every loaded word, and the arrival (a release) stays after them.
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[slot]);
        if (++slot == L.stages) {
            slot = 0;
            phase ^= 1u;
        }
    }
}


// ---------------------------------------------------------------------------
// The batch kernel on the same pipeline (tile `pipeline` = 1).  A work unit is
// one stage: up to COMPUTE * BPT consecutive blocks of one image (they may
// span several block rows).  CTA b takes units b, b + grid, ... (equal units
// balance like the image kernel's tiles, and no work counter is needed); its
// producer finds each unit's image, writes the stage's unit record and copies
// the unit's rows: for each block row segment of nb blocks, its 4 pixel rows
// (16 * nb bytes each) land one after another, so block k of a segment that
// starts at unit block ks sits at 64 * ks + 16 * (k - ks) + r * 16 * nb.
// Units of images with 4-byte aligned rows, or narrower than an eighth of a
// unit, are not copied: their record says so and the compute warps load those
// blocks themselves.  A record with no blocks ends the CTA's work.
// ---------------------------------------------------------------------------
struct UnitRec {
    const uint8_t* src;
    uint8_t* dst;
    uint32_t stride, bw, bw_magic, codec;
    uint32_t first, n;  // first block of the unit in its image, blocks in the unit (0: no more units)
    uint32_t direct;    // 1: rows not copied (4-byte aligned source), blocks read from global memory
    uint32_t reserved;
};
static_assert(sizeof(UnitRec) == 48, "UnitRec layout");

constexpr size_t batch_tma_smem_bytes(const TmaLayout& l)
{
    return (size_t)l.stages * (l.stage_bytes + 16u + sizeof(UnitRec)) + 128u;
}

// PARAM_TABLES: the descriptor and first-unit tables are the kernel's
// parameter (readable before the dependency wait); otherwise they are device
// memory the stream wrote before this launch.
template <int BPT, int COMPUTE, bool PARAM_TABLES>
__device__ __forceinline__ void batch_tma_body(const BatchImage* __restrict__ images, uint32_t n_images,
                                               const uint32_t* __restrict__ first_unit, uint32_t total_units)
{
    pdl_launch_dependents();
    extern __shared__ __align__(128) uint8_t smem[];
    __shared__ uint32_t abort_flag;
    constexpr uint32_t compute_warps = COMPUTE / 32;
    constexpr TmaLayout L = tma_layout(COMPUTE, BPT);
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + L.stages * L.stage_bytes);
    uint64_t* empty = full + L.stages;
    UnitRec* rec = reinterpret_cast<UnitRec*>(empty + L.stages);
    uint8_t* ctrl_lut = reinterpret_cast<uint8_t*>(rec + L.stages);
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;

    if (threadIdx.x == 0) {
        for (uint32_t s = 0; s < L.stages; ++s) {
            mbar_init(&full[s], 1u);
            mbar_init(&empty[s], compute_warps);
        }
        abort_flag = 0u;
        mbar_init_fence();
    }
    fill_ctrl_lut(ctrl_lut);
    __syncthreads();
    if constexpr (PARAM_TABLES) {
        if (warp == compute_warps && lane == 0) {
            // While the previous kernel in the stream drains, ask L2 for the rows
            // of this CTA's first units (a hint, as in encode_image_tma: nothing
            // enters the CTA and nothing is written before pdl_wait()).
            uint32_t ii = 0;
            for (uint32_t u = blockIdx.x, k = 0; u < total_units && k < l2_prefetch_tiles(L); u += gridDim.x, ++k) {
                ii += find_image(first_unit + ii, n_images - ii, u);
                const BatchImage& im = images[ii];
                if (!im.vec16 || im.bw * 8u < L.tile_blocks) continue;  // units the compute warps load themselves
                const uint32_t first = (u - im.first_unit) * L.tile_blocks;
                const uint32_t n = min(L.tile_blocks, im.bw * im.bh - first);
                for (uint32_t gb = first; gb < first + n;) {
                    uint32_t bx;
                    const uint32_t by = div_magic(gb, im.bw, im.bw_magic, bx);
                    const uint32_t nb = min(im.bw - bx, first + n - gb);
                    const uint8_t* row = im.src + (size_t)by * 4u * im.stride + 16u * (size_t)bx;
#pragma unroll
                    for (int rr = 0; rr < 4; ++rr) bulk_prefetch_l2(row + (size_t)rr * im.stride, 16u * nb);
                    gb += nb;
                }
            }
        }
    }
    pdl_wait();  // no copy and no store before the previous kernel in the stream is done

    if (warp == compute_warps) {  // producer
        if (lane != 0) return;
        // Units u = blockIdx.x, + gridDim.x, ...: the image of the next unit and
        // its descriptor are looked up right after the current unit's copies are
        // issued, while the compute warps work; the search starts at the current
        // image (units only grow), so a batch of large images rarely searches.
        // Rows are read once: evict-first in L2, as in encode_image_tma.
        const uint64_t policy = l2_evict_first_policy();
        uint32_t issued = 0, slot = 0, phase = 0;
        uint32_t u = blockIdx.x, ii = 0;
        BatchImage im{};
        if (u < total_units) {
            ii = find_image(first_unit, n_images, u);
            im = images[ii];
        }
        for (;;) {
            if (issued >= L.stages && !mbar_wait(&empty[slot], phase ^ 1u, &abort_flag, &g_pipeline_timeouts))
                break;
            UnitRec& r = rec[slot];
            if (u >= total_units) {
                r.n = 0;  // published by the arrival (release), read after the wait (acquire)
                mbar_arrive(&full[slot]);
                ++issued;
                break;
            }
            const uint32_t first = (u - im.first_unit) * L.tile_blocks;
            const uint32_t n = min(L.tile_blocks, im.bw * im.bh - first);
            r.src = im.src;
            r.dst = im.dst;
            r.stride = im.stride;
            r.bw = im.bw;
            r.bw_magic = im.bw_magic;
            r.codec = im.codec;
            r.first = first;
            r.n = n;
            // narrow images would take many small copies per unit (one per pixel row of every
            // block row): a unit is copied only when it spans at most about 9 block rows
            const bool copy = im.vec16 && im.bw * 8u >= L.tile_blocks;
            r.direct = copy ? 0u : 1u;
            if (copy) {
                mbar_arrive_expect_tx(&full[slot], 64u * n);
                uint8_t* buf = smem + slot * L.stage_bytes;
                for (uint32_t g = first; g < first + n;) {
                    uint32_t bx;
                    const uint32_t by = div_magic(g, im.bw, im.bw_magic, bx);
                    const uint32_t nb = min(im.bw - bx, first + n - g);
                    const uint8_t* row = im.src + (size_t)by * 4u * im.stride + 16u * (size_t)bx;
                    uint8_t* d = buf + 64u * (g - first);
#pragma unroll
                    for (int rr = 0; rr < 4; ++rr)
                        bulk_copy_g2s_hint(d + rr * 16u * nb, row + (size_t)rr * im.stride, 16u * nb, &full[slot],
                                           policy);
                    g += nb;
                }
            } else {
                mbar_arrive(&full[slot]);
            }
            ++issued;
            if (++slot == L.stages) {
                slot = 0;
                phase ^= 1u;
            }
            u += gridDim.x;
            if (u < total_units && ii + 1 < n_images && first_unit[ii + 1] <= u) {
                ii += find_image(first_unit + ii, n_images - ii, u);
                im = images[ii];
            }
        }
        if (*static_cast<volatile uint32_t*>(&abort_flag)) {
            const uint32_t n = issued < L.stages ? issued : L.stages;
            for (uint32_t i = issued - n; i < issued; ++i)
                mbar_wait(&full[i % L.stages], (i / L.stages) & 1u, nullptr, &g_pipeline_timeouts);
        }
        return;
    }

    uint32_t slot = 0, phase = 0;
    for (;;) {
        if (!mbar_wait(&full[slot], phase, &abort_flag, &g_pipeline_timeouts)) break;
        const UnitRec r = rec[slot];
        if (r.n == 0) break;
        const uint8_t* buf = smem + slot * L.stage_bytes;
        uint32_t w[BPT][16];
#pragma unroll
        for (int j = 0; j < BPT; ++j) {
            const uint32_t k = (warp * BPT + j) * 32u + lane;
            if (k < r.n) {
                uint32_t bx;
                const uint32_t by = div_magic(r.first + k, r.bw, r.bw_magic, bx);
                if (r.direct) {
                    load_block_rows(r.src + (size_t)by * 4u * r.stride + 16u * (size_t)bx, r.stride, false, w[j]);
                } else {
                    const uint32_t row0 = by * r.bw;  // first block of this block row
                    const uint32_t ks = row0 > r.first ? row0 - r.first : 0u;
                    const uint32_t nb = min(row0 + r.bw, r.first + r.n) - max(row0, r.first);
                    const uint8_t* p = buf + 64u * ks + 16u * (k - ks);
#pragma unroll
                    for (int rr = 0; rr < 4; ++rr) {
                        const uint4 v = *reinterpret_cast<const uint4*>(p + rr * 16u * nb);
                        w[j][4 * rr + 0] = v.x;
                        w[j][4 * rr + 1] = v.y;
                        w[j][4 * rr + 2] = v.z;
                        w[j][4 * rr + 3] = v.w;
                    }
                }
            }
        }
#pragma unroll
        for (int j = 0; j < BPT; ++j) {
            const uint32_t k = (warp * BPT + j) * 32u + lane;
            if (k < r.n) {
                const uint2 e = r.codec == kBC1 ? encode_bc1(w[j]) : encode_etc1s(w[j], ctrl_lut);
                st_stream8(r.dst + 8u * (size_t)(r.first + k), e);
            }
        }
        // released only after the stores, which wait for every loaded word (see encode_image_tma)
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[slot]);
        if (++slot == L.stages) {
            slot = 0;
            phase ^= 1u;
        }
    }
}

// Descriptor and first-unit tables in device memory (uploaded per call).
template <int BPT, int COMPUTE>
__global__ void __launch_bounds__(COMPUTE + 32, tma_min_ctas(BPT, COMPUTE))
    encode_batch_tma(const BatchImage* __restrict__ images, uint32_t n_images, const uint32_t* __restrict__ first_unit,
                     uint32_t total_units)
{
    batch_tma_body<BPT, COMPUTE, false>(images, n_images, first_unit, total_units);
}

// The same tables in the kernel's parameter space (small batches).
template <int BPT, int COMPUTE>
__global__ void __launch_bounds__(COMPUTE + 32, tma_min_ctas(BPT, COMPUTE))
    encode_batch_tma_inline(const __grid_constant__ InlineBatch batch, uint32_t n_images, uint32_t total_units)
{
    batch_tma_body<BPT, COMPUTE, true>(batch.images, n_images, batch.first_unit, total_units);
}

namespace {

template <int CODEC, int BPT, int COMPUTE>
cudaError_t launch_tma_t(const uint8_t* src, size_t stride, uint8_t* dst, uint8_t* dst2, uint32_t bw, uint32_t bh,
                         cudaStream_t stream)
{
    constexpr TmaLayout L = tma_layout(COMPUTE, BPT);
    const size_t smem = tma_smem_bytes(L);
    constexpr uint32_t block = COMPUTE + 32u;
    // per device: dynamic shared memory opt-in and resident CTAs per SM
    static std::atomic<int> resident[64];
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    int ctas = resident[dev].load(std::memory_order_relaxed);
    if (ctas == 0) {
        e = cudaFuncSetAttribute(encode_image_tma<CODEC, BPT, COMPUTE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem);
        if (e != cudaSuccess) return e;
        e = cudaFuncSetAttribute(encode_image_tma<CODEC, BPT, COMPUTE>,
                                 cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
        if (e != cudaSuccess) return e;
        int sms = 0, per_sm = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, encode_image_tma<CODEC, BPT, COMPUTE>, (int)block,
                                                          smem);
        if (e != cudaSuccess) return e;
        ctas = (sms > 0 ? sms : 1) * (per_sm > 0 ? per_sm : 1);
        resident[dev].store(ctas, std::memory_order_relaxed);
    }
    const uint32_t tiles_per_row = (bw + L.tile_blocks - 1) / L.tile_blocks;
    const uint64_t total = (uint64_t)tiles_per_row * bh;
    if (total > 0x7fffffffull) return cudaErrorInvalidValue;
    const uint32_t grid = (uint32_t)(total < (uint64_t)ctas ? total : (uint64_t)ctas);
    return launch_pdl(encode_image_tma<CODEC, BPT, COMPUTE>, dim3(grid), dim3(block), smem, stream, src, stride, dst,
                      dst2, bw, tiles_per_row, (uint32_t)total, 0xffffffffu / tiles_per_row);
}

template <int CODEC, int BPT>
cudaError_t launch_tma_bpt(const uint8_t* src, size_t stride, uint8_t* dst, uint8_t* dst2, uint32_t bw, uint32_t bh,
                           uint32_t threads, cudaStream_t stream)
{
    switch (threads) {
    case 128: return launch_tma_t<CODEC, BPT, 128>(src, stride, dst, dst2, bw, bh, stream);
    case 256: return launch_tma_t<CODEC, BPT, 256>(src, stride, dst, dst2, bw, bh, stream);
    case 512: return launch_tma_t<CODEC, BPT, 512>(src, stride, dst, dst2, bw, bh, stream);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace

cudaError_t launch_image_tma(int codec, const uint8_t* src, size_t stride, uint8_t* dst, uint32_t width,
                             uint32_t height, Tile tile, cudaStream_t stream, uint8_t* dst2)
{
    const uint32_t bw = width / 4, bh = height / 4;
    if (bw == 0 || bh == 0) return cudaSuccess;
    if (reinterpret_cast<uintptr_t>(src) % 16 || stride % 16) return cudaErrorInvalidValue;
    if (codec == kBC1) {
        if (tile.bpt == 1) return launch_tma_bpt<kBC1, 1>(src, stride, dst, nullptr, bw, bh, tile.threads, stream);
        if (tile.bpt == 2) return launch_tma_bpt<kBC1, 2>(src, stride, dst, nullptr, bw, bh, tile.threads, stream);
    } else if (codec == kETC1S) {
        if (tile.bpt == 1) return launch_tma_bpt<kETC1S, 1>(src, stride, dst, nullptr, bw, bh, tile.threads, stream);
        if (tile.bpt == 2) return launch_tma_bpt<kETC1S, 2>(src, stride, dst, nullptr, bw, bh, tile.threads, stream);
    } else if (codec == kBoth && dst2) {
        if (tile.bpt == 1) return launch_tma_bpt<kBoth, 1>(src, stride, dst, dst2, bw, bh, tile.threads, stream);
        if (tile.bpt == 2) return launch_tma_bpt<kBoth, 2>(src, stride, dst, dst2, bw, bh, tile.threads, stream);
    }
    return cudaErrorInvalidValue;
}

namespace {

template <int BPT, int COMPUTE>
int batch_tma_ctas_t(int dev)
{
    constexpr TmaLayout L = tma_layout(COMPUTE, BPT);
    constexpr size_t smem = batch_tma_smem_bytes(L);
    static std::atomic<int> resident[64];
    if (dev < 0 || dev >= 64) return 0;
    int ctas = resident[dev].load(std::memory_order_relaxed);
    if (ctas == 0) {
        if (cudaFuncSetAttribute(encode_batch_tma<BPT, COMPUTE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem) != cudaSuccess ||
            cudaFuncSetAttribute(encode_batch_tma<BPT, COMPUTE>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 cudaSharedmemCarveoutMaxShared) != cudaSuccess)
            return 0;
        int sms = 0, per_sm = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, encode_batch_tma<BPT, COMPUTE>, COMPUTE + 32,
                                                          smem) != cudaSuccess)
            return 0;
        ctas = (sms > 0 ? sms : 1) * (per_sm > 0 ? per_sm : 1);
        resident[dev].store(ctas, std::memory_order_relaxed);
    }
    return ctas;
}

template <int BPT, int COMPUTE>
cudaError_t launch_batch_tma_t(const BatchImage* images, uint32_t n_images, const uint32_t* first_unit,
                               uint32_t total_units, uint32_t* work_counter, uint32_t ctas, cudaStream_t stream)
{
    (void)work_counter;  // units are dealt to CTAs statically
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const int resident = batch_tma_ctas_t<BPT, COMPUTE>(dev);
    if (resident == 0) return cudaErrorInvalidValue;
    if (ctas > (uint32_t)resident) ctas = (uint32_t)resident;
    constexpr size_t smem = batch_tma_smem_bytes(tma_layout(COMPUTE, BPT));
    return launch_pdl(encode_batch_tma<BPT, COMPUTE>, dim3(ctas ? ctas : 1u), dim3(COMPUTE + 32), smem, stream,
                      images, n_images, first_unit, total_units);
}

template <int BPT, int COMPUTE>
cudaError_t launch_batch_tma_inline_t(const InlineBatch& batch, uint32_t n_images, uint32_t total_units, uint32_t ctas,
                                      cudaStream_t stream)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const int resident = batch_tma_ctas_t<BPT, COMPUTE>(dev);
    if (resident == 0 || dev < 0 || dev >= 64) return cudaErrorInvalidValue;
    constexpr size_t smem = batch_tma_smem_bytes(tma_layout(COMPUTE, BPT));
    static std::atomic<bool> ready[64];
    if (!ready[dev].load(std::memory_order_relaxed)) {
        e = cudaFuncSetAttribute(encode_batch_tma_inline<BPT, COMPUTE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(encode_batch_tma_inline<BPT, COMPUTE>,
                                     cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
        if (e != cudaSuccess) return e;
        ready[dev].store(true, std::memory_order_relaxed);
    }
    if (ctas > (uint32_t)resident) ctas = (uint32_t)resident;
    return launch_pdl(encode_batch_tma_inline<BPT, COMPUTE>, dim3(ctas ? ctas : 1u), dim3(COMPUTE + 32), smem,
                      stream, batch, n_images, total_units);
}

}  // namespace

cudaError_t launch_batch_tma_inline(const InlineBatch& batch, uint32_t n_images, uint32_t total_units,
                                    const BatchTile& tile, uint32_t ctas, cudaStream_t stream)
{
    if (total_units == 0) return cudaSuccess;
    if (n_images > kInlineImages || tile.unit_blocks != tile.threads * tile.bpt) return cudaErrorInvalidValue;
    const uint32_t t = tile.threads;
    if (tile.bpt == 1) {
        if (t == 128) return launch_batch_tma_inline_t<1, 128>(batch, n_images, total_units, ctas, stream);
        if (t == 256) return launch_batch_tma_inline_t<1, 256>(batch, n_images, total_units, ctas, stream);
        if (t == 512) return launch_batch_tma_inline_t<1, 512>(batch, n_images, total_units, ctas, stream);
    } else if (tile.bpt == 2) {
        if (t == 128) return launch_batch_tma_inline_t<2, 128>(batch, n_images, total_units, ctas, stream);
        if (t == 256) return launch_batch_tma_inline_t<2, 256>(batch, n_images, total_units, ctas, stream);
        if (t == 512) return launch_batch_tma_inline_t<2, 512>(batch, n_images, total_units, ctas, stream);
    }
    return cudaErrorInvalidValue;
}

int batch_tma_resident_ctas(uint32_t threads, uint32_t bpt)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 1;
    int n = 0;
    if (bpt == 1) n = threads == 128 ? batch_tma_ctas_t<1, 128>(dev) : threads == 256 ? batch_tma_ctas_t<1, 256>(dev)
                                                                                      : batch_tma_ctas_t<1, 512>(dev);
    else n = threads == 128 ? batch_tma_ctas_t<2, 128>(dev) : threads == 256 ? batch_tma_ctas_t<2, 256>(dev)
                                                                             : batch_tma_ctas_t<2, 512>(dev);
    return n > 0 ? n : 1;
}

cudaError_t launch_batch_tma(const BatchImage* images, uint32_t n_images, const uint32_t* first_unit,
                             uint32_t total_units, uint32_t* work_counter, const BatchTile& tile, uint32_t ctas,
                             cudaStream_t stream)
{
    if (total_units == 0) return cudaSuccess;
    if (tile.unit_blocks != tile.threads * tile.bpt) return cudaErrorInvalidValue;
    const uint32_t t = tile.threads;
    if (tile.bpt == 1) {
        if (t == 128) return launch_batch_tma_t<1, 128>(images, n_images, first_unit, total_units, work_counter, ctas, stream);
        if (t == 256) return launch_batch_tma_t<1, 256>(images, n_images, first_unit, total_units, work_counter, ctas, stream);
        if (t == 512) return launch_batch_tma_t<1, 512>(images, n_images, first_unit, total_units, work_counter, ctas, stream);
    } else if (tile.bpt == 2) {
        if (t == 128) return launch_batch_tma_t<2, 128>(images, n_images, first_unit, total_units, work_counter, ctas, stream);
        if (t == 256) return launch_batch_tma_t<2, 256>(images, n_images, first_unit, total_units, work_counter, ctas, stream);
        if (t == 512) return launch_batch_tma_t<2, 512>(images, n_images, first_unit, total_units, work_counter, ctas, stream);
    }
    return cudaErrorInvalidValue;
}

// Thread 0 waits on an mbarrier that expects one arrival and gets none.
// Nothing is copied into the CTA, so nothing is in flight when it returns.
__global__ void bounded_wait_selftest_kernel(unsigned int* counter, uint32_t* out)
{
    __shared__ uint64_t bar;
    __shared__ uint32_t abort_flag;
    if (threadIdx.x != 0) return;
    mbar_init(&bar, 1u);
    abort_flag = 0u;
    mbar_init_fence();
    const bool completed = mbar_wait(&bar, 0u, &abort_flag, counter);
    out[0] = completed ? 1u : 0u;
    out[1] = abort_flag;
}

cudaError_t bounded_wait_selftest(bool* completed, bool* aborted, unsigned int* counted)
{
    uint32_t* d = nullptr;  // {counter, wait result, abort flag}
    cudaError_t e = cudaMalloc(&d, 3 * sizeof(uint32_t));
    if (e != cudaSuccess) return e;
    uint32_t h[3] = {0, 0, 0};
    e = cudaMemset(d, 0, 3 * sizeof(uint32_t));
    if (e == cudaSuccess) {
        bounded_wait_selftest_kernel<<<1, 32>>>(d, d + 1);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(h, d, sizeof h, cudaMemcpyDeviceToHost);
    cudaFree(d);
    *counted = h[0];
    *completed = h[1] != 0;
    *aborted = h[2] != 0;
    return e;
}

cudaError_t pipeline_timeouts(unsigned int* count, bool reset)
{
    cudaError_t e = cudaMemcpyFromSymbol(count, g_pipeline_timeouts, sizeof(unsigned int));
    if (e == cudaSuccess && reset) {
        const unsigned int zero = 0;
        e = cudaMemcpyToSymbol(g_pipeline_timeouts, &zero, sizeof(unsigned int));
    }
    return e;
}

}  // namespace goofy_gpu
