// batch.cpp -- host side of the batched encoder: many device images of uneven
// sizes (textures and their mip levels, either codec) in one persistent launch.
//
// No reference counterpart: the reference encodes one image per call
// (goofy::compressDXT1/ETC1, GoofyTC/goofy_tc.h:1497-1557).  A batch object
// owns two descriptor slots (pinned host staging + device table + work
// counter).  Slots alternate between calls, so the descriptors of the next
// batch are written while the previous batch still runs; a slot is refilled
// only after the launch that used it completed.  Each encode is one H2D copy
// (descriptors, first-unit table and a zeroed work counter, one buffer) and
// the persistent kernel, enqueued on the caller's stream (a pipelined batch
// of at most kInlineImages images instead passes its descriptors as the
// kernel's parameter: one launch, no upload).  With graphs enabled
// the two are captured once per slot (on the library's own idle stream) and
// the graph is launched on the caller's stream while the batch shape (image
// count, work units, tile) stays the same; the pointers inside the
// descriptors may change freely.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "../../include/goofy_gpu.h"
#include "batch.h"
#include "host_util.h"

using goofy_gpu::BatchImage;
using goofy_gpu::BatchTile;
using goofy_gpu::cuda_fail;
using goofy_gpu::DeviceGuard;

namespace {

// A call's upload, one contiguous buffer: `count` descriptors (48 B each),
// the first-unit table (4 B each) and the work counter (4 B, uploaded as 0),
// so one copy sets up a launch.
size_t upload_bytes(uint32_t count) { return (size_t)count * (sizeof(BatchImage) + sizeof(uint32_t)) + sizeof(uint32_t); }

struct Slot {
    uint8_t* h_buf = nullptr;  // pinned
    uint8_t* d_buf = nullptr;
    cudaEvent_t done = nullptr;
    bool in_flight = false;
    cudaGraphExec_t exec = nullptr;
    uint32_t g_count = 0, g_units = 0, g_ctas = 0;
    BatchTile g_tile{0, 0, 0, 0};
};

}  // namespace

struct goofy_gpu_batch {
    std::mutex mu;
    int device = 0;
    uint32_t max_images = 0;
    BatchTile tile{128, 1, 256, 0};
    bool graphs = true;
    cudaStream_t stream = nullptr;
    Slot slot[2];
    int next = 0;
    std::vector<uint32_t> units_scratch;
};

int goofy_gpu::validate_and_fill(const goofy_gpu_image* images, uint32_t count, uint32_t unit_blocks,
                                 BatchImage* desc, uint32_t* first, uint32_t* total_units)
{
    uint64_t units = 0;
    for (uint32_t i = 0; i < count; ++i) {
        const goofy_gpu_image& im = images[i];
        if (im.codec != GOOFY_CODEC_BC1 && im.codec != GOOFY_CODEC_ETC1S)
            return goofy_gpu::fail(GOOFY_ERR_INVALID, "batch: bad codec");
        if (im.width % 4) return goofy_gpu::fail(GOOFY_ERR_WIDTH, "batch: width % 4 != 0");
        if (im.height % 4) return goofy_gpu::fail(GOOFY_ERR_HEIGHT, "batch: height % 4 != 0");
        const uint64_t bw = im.width / 4, bh = im.height / 4;
        if (bw * bh > 0x7fffffffull) return goofy_gpu::fail(GOOFY_ERR_TOO_LARGE, "batch: image too large");
        BatchImage& d = desc[i];
        std::memset(&d, 0, sizeof d);
        d.first_unit = (uint32_t)units;
        first[i] = (uint32_t)units;
        if (bw == 0 || bh == 0) continue;  // empty image: no units
        if (!im.src || !im.dst) return goofy_gpu::fail(GOOFY_ERR_INVALID, "batch: null pointer");
        if ((uint64_t)im.stride < 4ull * im.width) return goofy_gpu::fail(GOOFY_ERR_INVALID, "batch: stride");
        const uintptr_t s = reinterpret_cast<uintptr_t>(im.src);
        if (reinterpret_cast<uintptr_t>(im.dst) % 8 || s % 4 || im.stride % 4)
            return goofy_gpu::fail(GOOFY_ERR_ALIGNMENT, "batch: alignment");
        d.src = static_cast<const uint8_t*>(im.src);
        d.dst = static_cast<uint8_t*>(im.dst);
        d.stride = im.stride;
        d.bw = (uint32_t)bw;
        d.bh = (uint32_t)bh;
        d.bw_magic = 0xffffffffu / (uint32_t)bw;
        d.codec = (uint32_t)im.codec;
        d.vec16 = (s % 16 == 0 && im.stride % 16 == 0) ? 1u : 0u;
        units += (bw * bh + unit_blocks - 1) / unit_blocks;
        if (units > 0x7fffffffull) return goofy_gpu::fail(GOOFY_ERR_TOO_LARGE, "batch: too many work units");
    }
    *total_units = (uint32_t)units;
    return GOOFY_OK;
}

namespace {

using goofy_gpu::validate_and_fill;

void free_slot(Slot& s)
{
    if (s.done) cudaEventSynchronize(s.done);
    if (s.exec) cudaGraphExecDestroy(s.exec);
    if (s.h_buf) cudaFreeHost(s.h_buf);
    if (s.d_buf) cudaFree(s.d_buf);
    if (s.done) cudaEventDestroy(s.done);
    s = Slot{};
}

// Enqueue the upload (descriptors, first-unit table, zeroed counter) and the kernel on `st`.
cudaError_t enqueue(const Slot& s, uint32_t count, uint32_t units, const BatchTile& tile, uint32_t ctas,
                    cudaStream_t st)
{
    cudaError_t e = cudaMemcpyAsync(s.d_buf, s.h_buf, upload_bytes(count), cudaMemcpyHostToDevice, st);
    const BatchImage* d_desc = reinterpret_cast<const BatchImage*>(s.d_buf);
    const uint32_t* d_first = reinterpret_cast<const uint32_t*>(s.d_buf + sizeof(BatchImage) * count);
    uint32_t* d_counter = reinterpret_cast<uint32_t*>(s.d_buf + upload_bytes(count) - sizeof(uint32_t));
    if (e == cudaSuccess) e = goofy_gpu::launch_batch(d_desc, count, d_first, units, d_counter, tile, ctas, st);
    return e;
}

int encode_locked(goofy_gpu_batch* b, const goofy_gpu_image* images, uint32_t count, cudaStream_t caller,
                  const BatchTile& tile)
{
    if (count > b->max_images) return goofy_gpu::fail(GOOFY_ERR_TOO_LARGE, "batch: more images than max_images");
    if (count == 0) return GOOFY_OK;
    DeviceGuard g(b->device);
    GOOFY_CUDA_TRY(g.err);
    if (tile.pipeline && count <= goofy_gpu::kInlineImages) {
        // a small pipelined batch: its descriptors travel as the kernel's parameter (no upload, no graph)
        goofy_gpu::InlineBatch ib{};
        uint32_t units = 0;
        const int rc = validate_and_fill(images, count, tile.unit_blocks, ib.images, ib.first_unit, &units);
        if (rc != GOOFY_OK) return rc;
        if (units == 0) return GOOFY_OK;
        const uint32_t ctas = (uint32_t)std::min<uint64_t>(
            (uint64_t)goofy_gpu::batch_resident_ctas(tile.threads, tile.bpt, tile.pipeline), units);
        const cudaError_t e = goofy_gpu::launch_batch_tma_inline(ib, count, units, tile, ctas, caller);
        if (e != cudaSuccess) return cuda_fail(e, "batch launch");
        return GOOFY_OK;
    }
    Slot& s = b->slot[b->next];
    b->next ^= 1;
    if (s.in_flight) {
        GOOFY_CUDA_TRY(cudaEventSynchronize(s.done));  // staging of this slot is free again
        s.in_flight = false;
    }
    uint32_t units = 0;
    BatchImage* h_desc = reinterpret_cast<BatchImage*>(s.h_buf);
    uint32_t* h_first = reinterpret_cast<uint32_t*>(s.h_buf + sizeof(BatchImage) * count);
    *reinterpret_cast<uint32_t*>(s.h_buf + upload_bytes(count) - sizeof(uint32_t)) = 0;  // the work counter
    const int rc = validate_and_fill(images, count, tile.unit_blocks, h_desc, h_first, &units);
    if (rc != GOOFY_OK) return rc;
    if (units == 0) return GOOFY_OK;
    // warps a unit (plain) or one unit per stage of a CTA (pipeline): no more CTAs than have work
    const uint64_t useful = tile.pipeline ? (uint64_t)units : ((uint64_t)units * 32 + tile.threads - 1) / tile.threads;
    const uint32_t ctas = (uint32_t)std::min<uint64_t>(
        (uint64_t)goofy_gpu::batch_resident_ctas(tile.threads, tile.bpt, tile.pipeline), useful);

    if (b->graphs) {
        const bool match = s.exec && s.g_count == count && s.g_units == units && s.g_ctas == ctas &&
                           s.g_tile.threads == tile.threads && s.g_tile.bpt == tile.bpt &&
                           s.g_tile.unit_blocks == tile.unit_blocks && s.g_tile.pipeline == tile.pipeline;
        if (!match) {
            if (s.exec) {
                cudaGraphExecDestroy(s.exec);
                s.exec = nullptr;
            }
            cudaGraph_t graph = nullptr;
            GOOFY_CUDA_TRY(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
            cudaError_t e = enqueue(s, count, units, tile, ctas, b->stream);
            cudaError_t e2 = cudaStreamEndCapture(b->stream, &graph);
            if (e != cudaSuccess || e2 != cudaSuccess) {
                if (graph) cudaGraphDestroy(graph);
                return cuda_fail(e != cudaSuccess ? e : e2, "batch graph capture");
            }
            e = cudaGraphInstantiate(&s.exec, graph, 0);
            cudaGraphDestroy(graph);
            if (e != cudaSuccess) {
                s.exec = nullptr;
                return cuda_fail(e, "cudaGraphInstantiate");
            }
            s.g_count = count;
            s.g_units = units;
            s.g_ctas = ctas;
            s.g_tile = tile;
        }
        GOOFY_CUDA_TRY(cudaGraphLaunch(s.exec, caller));  // (captured on the idle library stream)
    } else {
        const cudaError_t e = enqueue(s, count, units, tile, ctas, caller);
        if (e != cudaSuccess) return cuda_fail(e, "batch enqueue");
    }
    GOOFY_CUDA_TRY(cudaEventRecord(s.done, caller));
    s.in_flight = true;
    return GOOFY_OK;
}

}  // namespace

extern "C" {

GOOFY_EXPORT int goofy_gpu_batch_create(goofy_gpu_batch** out, uint32_t max_images, int device)
{
    if (!out || max_images == 0 || max_images > (1u << 24)) return GOOFY_ERR_INVALID;
    *out = nullptr;
    int n = 0;
    GOOFY_CUDA_TRY(cudaGetDeviceCount(&n));
    if (device < 0 || device >= n) return GOOFY_ERR_NO_DEVICE;
    DeviceGuard g(device);
    GOOFY_CUDA_TRY(g.err);
    goofy_gpu_batch* b = new (std::nothrow) goofy_gpu_batch();
    if (!b) return GOOFY_ERR_NOMEM;
    b->device = device;
    b->max_images = max_images;
    auto cleanup = [&](int rc) {
        for (auto& s : b->slot) free_slot(s);
        if (b->stream) cudaStreamDestroy(b->stream);
        delete b;
        return rc;
    };
    cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    for (auto& s : b->slot) {
        if (e == cudaSuccess) e = cudaHostAlloc(&s.h_buf, upload_bytes(max_images), cudaHostAllocDefault);
        if (e == cudaSuccess) e = cudaMalloc(&s.d_buf, upload_bytes(max_images));
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming);
    }
    if (e != cudaSuccess) return cleanup(cuda_fail(e, "goofy_gpu_batch_create"));
    *out = b;
    return GOOFY_OK;
}

GOOFY_EXPORT void goofy_gpu_batch_destroy(goofy_gpu_batch* b)
{
    if (!b) return;
    {
        std::lock_guard<std::mutex> lk(b->mu);
        DeviceGuard g(b->device);
        for (auto& s : b->slot) free_slot(s);
        if (b->stream) cudaStreamDestroy(b->stream);
    }
    delete b;
}

GOOFY_EXPORT int goofy_gpu_batch_encode(goofy_gpu_batch* b, const goofy_gpu_image* images, uint32_t count,
                                        void* stream)
{
    if (!b || (count && !images)) return GOOFY_ERR_INVALID;
    std::lock_guard<std::mutex> lk(b->mu);
    return encode_locked(b, images, count, static_cast<cudaStream_t>(stream), b->tile);
}

GOOFY_EXPORT int goofy_gpu_batch_set_graphs(goofy_gpu_batch* b, int enable)
{
    if (!b) return GOOFY_ERR_INVALID;
    std::lock_guard<std::mutex> lk(b->mu);
    b->graphs = enable != 0;
    return GOOFY_OK;
}

GOOFY_EXPORT int goofy_gpu_batch_get_tile(goofy_gpu_batch* b, goofy_gpu_batch_tile* tile)
{
    if (!b || !tile) return GOOFY_ERR_INVALID;
    std::lock_guard<std::mutex> lk(b->mu);
    tile->threads_per_cta = b->tile.threads;
    tile->blocks_per_thread = b->tile.bpt;
    tile->unit_blocks = b->tile.unit_blocks;
    tile->pipeline = b->tile.pipeline;
    return GOOFY_OK;
}

GOOFY_EXPORT int goofy_gpu_batch_set_tile(goofy_gpu_batch* b, const goofy_gpu_batch_tile* tile)
{
    if (!b || !tile) return GOOFY_ERR_INVALID;
    const BatchTile t{tile->threads_per_cta, tile->blocks_per_thread, tile->unit_blocks, tile->pipeline};
    if (!goofy_gpu::batch_tile_valid(t)) return GOOFY_ERR_INVALID;
    std::lock_guard<std::mutex> lk(b->mu);
    b->tile = t;
    return GOOFY_OK;
}

GOOFY_EXPORT int goofy_gpu_batch_autotune(goofy_gpu_batch* b, const goofy_gpu_image* images, uint32_t count,
                                          uint32_t reps, goofy_gpu_batch_tile* best, float* best_us)
{
    if (!b || !images || count == 0 || reps == 0 || reps > 100) return GOOFY_ERR_INVALID;
    std::lock_guard<std::mutex> lk(b->mu);
    DeviceGuard g(b->device);
    GOOFY_CUDA_TRY(g.err);
    cudaEvent_t ev[2] = {nullptr, nullptr};
    GOOFY_CUDA_TRY(cudaEventCreate(&ev[0]));
    if (cudaEventCreate(&ev[1]) != cudaSuccess) {
        cudaEventDestroy(ev[0]);
        return cuda_fail(cudaGetLastError(), "cudaEventCreate");
    }
    const bool graphs = b->graphs;
    b->graphs = false;  // time the launches themselves, not graph instantiation
    int rc = GOOFY_OK;
    BatchTile best_tile{0, 0, 0, 0};
    float best_time = 0.f;
    std::vector<BatchTile> candidates;
    for (uint32_t threads : {128u, 256u, 512u})
        for (uint32_t bpt : {1u, 2u}) {
            for (uint32_t unit : {64u, 128u, 256u, 512u, 1024u, 2048u})
                candidates.push_back(BatchTile{threads, bpt, unit, 0});
            candidates.push_back(BatchTile{threads, bpt, threads * bpt, 1});  // the pipelined kernel: a unit per stage
        }
    // Per tile: two warm-up launches, then three rounds of `reps` launches
    // back to back between two events (no event between launches, so each
    // can overlap the previous one's tail as a caller's stream of batches
    // does); the median round's mean per launch.
    for (const BatchTile& tile : candidates) {
        if (!goofy_gpu::batch_tile_valid(tile)) continue;
        for (uint32_t w = 0; w < 2 && rc == GOOFY_OK; ++w) rc = encode_locked(b, images, count, b->stream, tile);
        float t[3] = {0.f, 0.f, 0.f};
        for (int r = 0; r < 3 && rc == GOOFY_OK; ++r) {
            cudaError_t e = cudaEventRecord(ev[0], b->stream);
            if (e != cudaSuccess) {
                rc = cuda_fail(e, "cudaEventRecord");
                break;
            }
            for (uint32_t k = 0; k < reps && rc == GOOFY_OK; ++k) rc = encode_locked(b, images, count, b->stream, tile);
            if (rc != GOOFY_OK) break;
            e = cudaEventRecord(ev[1], b->stream);
            if (e == cudaSuccess) e = cudaEventSynchronize(ev[1]);
            float ms = 0.f;
            if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, ev[0], ev[1]);
            if (e != cudaSuccess) {
                rc = cuda_fail(e, "autotune timing");
                break;
            }
            t[r] = ms / (float)reps;
        }
        if (rc != GOOFY_OK) break;
        std::sort(t, t + 3);
        const float med = t[1];
        if (best_tile.threads == 0 || med < best_time) {
            best_time = med;
            best_tile = tile;
        }
    }
    b->graphs = graphs;
    cudaEventDestroy(ev[0]);
    cudaEventDestroy(ev[1]);
    if (rc != GOOFY_OK) return rc;
    b->tile = best_tile;
    if (best) {
        best->threads_per_cta = best_tile.threads;
        best->blocks_per_thread = best_tile.bpt;
        best->unit_blocks = best_tile.unit_blocks;
        best->pipeline = best_tile.pipeline;
    }
    if (best_us) *best_us = best_time * 1e3f;
    return GOOFY_OK;
}

}  // extern "C"
