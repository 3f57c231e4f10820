// capi.cpp -- C ABI, host-pointer pipeline and the C++ drop-in entry points.
//
// Reference interface replaced: goofy::compressDXT1 / goofy::compressETC1
// (GoofyTC/goofy_tc.h:10-13, :1497-1557), a synchronous CPU function over
// caller-owned host buffers.  Here the same call runs on the GPU.  Direct
// path: when the GPU can address both buffers (pinned, or any host memory
// where it walks the host page tables), one kernel reads the caller's rows
// and writes its blocks over the host link.  Staged path: the rows are split
// into bands, and for each band
//   host -> device copy, encode kernel, device -> host copy
// are queued on one of two streams, so the copy-in of band b+1 overlaps the
// encode and copy-out of band b.  Pinned caller buffers are copied by DMA
// directly; pageable ones go through library-owned pinned staging.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/goofy_gpu.h"
#include "../../include/goofy_tc_gpu.h"
#include "host_util.h"
#include "kernels.h"
#include "tile_cache.h"

namespace goofy_gpu {

namespace {
thread_local char g_last_error[256] = "";
}

int cuda_fail(cudaError_t e, const char* what)
{
    std::snprintf(g_last_error, sizeof g_last_error, "%s: %s", what, cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? GOOFY_ERR_NOMEM
           : (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) ? GOOFY_ERR_NO_DEVICE
                                                                           : GOOFY_ERR_CUDA;
}

int fail(int status, const char* what)
{
    std::snprintf(g_last_error, sizeof g_last_error, "%s", what);
    return status;
}

const char* last_error_text() { return g_last_error; }

}  // namespace goofy_gpu

namespace {

using goofy_gpu::cuda_fail;
using goofy_gpu::DeviceGuard;
using goofy_gpu::SrcAccess;
using goofy_gpu::Tile;

#define CUDA_TRY GOOFY_CUDA_TRY

// Every codec on the bulk-copy pipeline, 512 compute threads, 2 blocks a thread.  For BC1 alone the
// register-loading grid is as fast on some boxes (the autotuner picks per box), but the bulk-copy
// kernel lets a BC1 launch and an ETC1s launch follow each other without a gap: both use one CTA of
// the same size per SM, so the next launch's CTA takes an SM as soon as the last one leaves it.
constexpr Tile kDefaultTile[3] = {{512, 2, 2}, {512, 2, 2}, {512, 2, 2}};
Tile g_tile[3] = {kDefaultTile[0], kDefaultTile[1], kDefaultTile[2]};
bool g_tile_explicit[3] = {false, false, false};  // set by goofy_gpu_set_tile / the autotuner: the cache leaves it
std::mutex g_tile_mu;
constexpr int kMaxDevices = 64;
std::atomic<bool> g_cache_loaded[kMaxDevices];

Tile tile_for(int codec)
{
    std::lock_guard<std::mutex> lk(g_tile_mu);
    return g_tile[codec == GOOFY_CODEC_BOTH ? 2 : codec & 1];
}

// Name and SM count of a device: the key of its tile cache entries.
int device_key(int dev, std::string* name, uint32_t* sms)
{
    cudaDeviceProp p;
    CUDA_TRY(cudaGetDeviceProperties(&p, dev));
    *name = p.name;
    *sms = (uint32_t)p.multiProcessorCount;
    return GOOFY_OK;
}

// Installs the cached tiles of device `dev` for the codecs nobody set
// explicitly; returns how many were installed, or a negative status.
int load_tile_cache(int dev)
{
    std::string name;
    uint32_t sms = 0;
    const int rc = device_key(dev, &name, &sms);
    if (rc != GOOFY_OK) return rc;
    const std::string path = goofy_gpu::tile_cache_path();
    Tile found[3];
    bool have[3];
    for (int c = 0; c < 3; ++c) have[c] = goofy_gpu::tile_cache_lookup(path, name, sms, c, &found[c]);
    int applied = 0;
    std::lock_guard<std::mutex> lk(g_tile_mu);
    for (int c = 0; c < 3; ++c)
        if (have[c] && !g_tile_explicit[c]) {
            g_tile[c] = found[c];
            ++applied;
        }
    if (dev >= 0 && dev < kMaxDevices) g_cache_loaded[dev].store(true);
    return applied;
}

// Once per device and process (goofy_gpu_init, or the first encode call).
void ensure_tile_cache(int dev)
{
    if (dev < 0 || dev >= kMaxDevices || g_cache_loaded[dev].load(std::memory_order_relaxed)) return;
    if (load_tile_cache(dev) < 0) {
        cudaGetLastError();
        g_cache_loaded[dev].store(true);  // no usable entry: keep the compiled defaults
    }
}

void ensure_tile_cache_current()
{
    int dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess) ensure_tile_cache(dev);
    else cudaGetLastError();
}

struct Buffer {
    uint8_t* p = nullptr;
    size_t cap = 0;
};

// Per-process state of the host-pointer path.
struct HostPath {
    std::mutex mu;
    bool ready = false;
    bool pageable_ok = false;  // kernels may read / write pageable host memory
    int device = 0;
    cudaStream_t stream[2] = {nullptr, nullptr};
    cudaEvent_t done[2] = {nullptr, nullptr};
    Buffer d_src[2], d_dst[2], h_src[2], h_dst[2];

    int ensure_device(Buffer& b, size_t bytes)
    {
        if (b.cap >= bytes) return GOOFY_OK;
        if (b.p) cudaFree(b.p);
        b.p = nullptr;
        b.cap = 0;
        CUDA_TRY(cudaMalloc(&b.p, bytes));
        b.cap = bytes;
        return GOOFY_OK;
    }

    int ensure_pinned(Buffer& b, size_t bytes)
    {
        if (b.cap >= bytes) return GOOFY_OK;
        if (b.p) cudaFreeHost(b.p);
        b.p = nullptr;
        b.cap = 0;
        CUDA_TRY(cudaHostAlloc(&b.p, bytes, cudaHostAllocDefault));
        b.cap = bytes;
        return GOOFY_OK;
    }

    int init_locked(int dev)
    {
        if (ready && dev == device) return GOOFY_OK;
        release_locked();
        int n = 0;
        CUDA_TRY(cudaGetDeviceCount(&n));
        if (dev < 0 || dev >= n) return GOOFY_ERR_NO_DEVICE;
        DeviceGuard g(dev);
        CUDA_TRY(g.err);
        device = dev;
        int pageable = 0, ats = 0;
        CUDA_TRY(cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev));
        CUDA_TRY(cudaDeviceGetAttribute(&ats, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev));
        pageable_ok = pageable && ats;
        for (int i = 0; i < 2; ++i) {
            CUDA_TRY(cudaStreamCreateWithFlags(&stream[i], cudaStreamNonBlocking));
            CUDA_TRY(cudaEventCreateWithFlags(&done[i], cudaEventDisableTiming));
        }
        ready = true;
        return GOOFY_OK;
    }

    void release_locked()
    {
        if (!ready) return;
        DeviceGuard g(device);
        for (int i = 0; i < 2; ++i) {
            if (stream[i]) cudaStreamSynchronize(stream[i]);
            if (d_src[i].p) cudaFree(d_src[i].p);
            if (d_dst[i].p) cudaFree(d_dst[i].p);
            if (h_src[i].p) cudaFreeHost(h_src[i].p);
            if (h_dst[i].p) cudaFreeHost(h_dst[i].p);
            d_src[i] = d_dst[i] = h_src[i] = h_dst[i] = Buffer{};
            if (done[i]) cudaEventDestroy(done[i]);
            if (stream[i]) cudaStreamDestroy(stream[i]);
            done[i] = nullptr;
            stream[i] = nullptr;
        }
        ready = false;
    }
};

HostPath& host_path()
{
    static HostPath* hp = new HostPath();  // never destroyed: no CUDA calls at static teardown
    return *hp;
}

bool is_pinned(const void* p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

std::atomic<int> g_host_path{GOOFY_HOST_PATH_AUTO};

// Address under which the current device's kernels can use host buffer `p`
// directly, or nullptr: pinned memory (its mapped address), device or managed
// memory, or -- where the GPU walks the host page tables (NVLink-C2C
// address translation) -- ordinary pageable memory.
const void* device_view(const void* p, bool pageable_ok)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    switch (a.type) {
    case cudaMemoryTypeHost: return a.devicePointer;
    case cudaMemoryTypeDevice:
    case cudaMemoryTypeManaged: return p;
    default: return pageable_ok ? p : nullptr;
    }
}

int check_args(int codec, const void* dst, const void* src, uint32_t width, uint32_t height, uint32_t stride)
{
    if (codec != GOOFY_CODEC_BC1 && codec != GOOFY_CODEC_ETC1S) return GOOFY_ERR_INVALID;
    if (width % 4 != 0) return GOOFY_ERR_WIDTH;
    if (height % 4 != 0) return GOOFY_ERR_HEIGHT;
    if (width == 0 || height == 0) return GOOFY_OK;
    if (!dst || !src) return GOOFY_ERR_INVALID;
    if ((uint64_t)stride < 4ull * width) return GOOFY_ERR_INVALID;
    return 1;  // proceed
}

// The two outputs of the two-codec pass, (w/4)(h/4)*8 bytes each, must not overlap.
bool outputs_overlap(const void* a, const void* b, uint32_t width, uint32_t height)
{
    const uint64_t n = (uint64_t)(width / 4) * (height / 4) * 8;
    const uintptr_t x = reinterpret_cast<uintptr_t>(a), y = reinterpret_cast<uintptr_t>(b);
    return x < y + n && y < x + n;
}

constexpr size_t kBandBytes = 16u << 20;  // source bytes per band of the host path

// Either codec into `dst`, or (codec GOOFY_CODEC_BOTH) the BC1 blocks into
// `dst` and the ETC1s blocks into `dst2` from one pass.
int compress_host_impl(int codec, uint8_t* dst, const uint8_t* src, uint32_t width, uint32_t height, uint32_t stride,
                       uint8_t* dst2 = nullptr)
{
    const bool both = codec == GOOFY_CODEC_BOTH;
    int rc = check_args(both ? GOOFY_CODEC_BC1 : codec, dst, src, width, height, stride);
    if (rc <= 0) return rc;
    if (both && (!dst2 || outputs_overlap(dst, dst2, width, height))) return GOOFY_ERR_INVALID;
    HostPath& hp = host_path();
    std::lock_guard<std::mutex> lk(hp.mu);
    if (!hp.ready) {
        rc = hp.init_locked(hp.device);
        if (rc != GOOFY_OK) return rc;
    }
    DeviceGuard g(hp.device);
    CUDA_TRY(g.err);
    ensure_tile_cache(hp.device);

    // Direct path: one kernel reads the caller's rows and writes its blocks
    // over the host link, no staging copies.
    const int path = g_host_path.load();
    if (path != GOOFY_HOST_PATH_STAGED) {
        const void* dsrc = device_view(src, hp.pageable_ok);
        void* ddst = const_cast<void*>(device_view(dst, hp.pageable_ok));
        void* ddst2 = both ? const_cast<void*>(device_view(dst2, hp.pageable_ok)) : nullptr;
        const uintptr_t sa = reinterpret_cast<uintptr_t>(dsrc);
        const bool aligned = sa % 4 == 0 && stride % 4 == 0 && reinterpret_cast<uintptr_t>(ddst) % 8 == 0 &&
                             reinterpret_cast<uintptr_t>(ddst2) % 8 == 0;
        if (dsrc && ddst && (!both || ddst2) && aligned) {
            const SrcAccess access = (sa % 16 == 0 && stride % 16 == 0) ? SrcAccess::kVec16 : SrcAccess::kWord4;
            // bulk async copies only ever read device memory: host rows go through the register-loading
            // kernel, in CTAs of 128 threads, whose number spreads the host-link reads over every SM
            Tile t = tile_for(codec);
            if (t.persistent == 2) t = Tile{128, t.bpt, 0};
            CUDA_TRY(goofy_gpu::launch_image(codec, static_cast<const uint8_t*>(dsrc), stride,
                                             static_cast<uint8_t*>(ddst), width, height, t, access, hp.stream[0],
                                             static_cast<uint8_t*>(ddst2)));
            CUDA_TRY(cudaStreamSynchronize(hp.stream[0]));
            return GOOFY_OK;
        }
        if (path == GOOFY_HOST_PATH_DIRECT)
            return goofy_gpu::fail(GOOFY_ERR_INVALID, "direct host path: buffers not GPU-accessible or misaligned");
    }

    const uint32_t bw = width / 4, bh = height / 4;
    const size_t row_bytes = 4ull * width;
    const size_t dpitch = (row_bytes + 15) & ~size_t(15);  // device / staging pitch: 16-byte rows
    const uint32_t band_bh = (uint32_t)std::max<size_t>(1, std::min<size_t>(bh, kBandBytes / (4 * dpitch)));
    const uint32_t nbands = (bh + band_bh - 1) / band_bh;
    const bool src_pinned = is_pinned(src), dst_pinned = is_pinned(dst) && (!both || is_pinned(dst2));
    // output planes of a band slot: BC1 or ETC1s at 0, and the ETC1s blocks of the two-codec pass at band_out
    const size_t band_in = (size_t)band_bh * 4 * dpitch, band_out = (size_t)band_bh * bw * 8;
    const size_t slot_out = both ? 2 * band_out : band_out;
    const int slots = nbands > 1 ? 2 : 1;
    for (int s = 0; s < slots; ++s) {
        if ((rc = hp.ensure_device(hp.d_src[s], band_in)) != GOOFY_OK) return rc;
        if ((rc = hp.ensure_device(hp.d_dst[s], slot_out)) != GOOFY_OK) return rc;
        if (!src_pinned && (rc = hp.ensure_pinned(hp.h_src[s], band_in)) != GOOFY_OK) return rc;
        if (!dst_pinned && (rc = hp.ensure_pinned(hp.h_dst[s], slot_out)) != GOOFY_OK) return rc;
    }
    const Tile tile = tile_for(codec);
    uint8_t* const planes[2] = {dst, dst2};

    // band b: rows [b*band_bh, ...); slot b % slots.  A slot is reused only
    // after its previous band finished (and, for pageable dst, was copied out).
    auto finish_band = [&](uint32_t b) -> int {
        const int s = (int)(b % slots);
        CUDA_TRY(cudaEventSynchronize(hp.done[s]));
        if (!dst_pinned) {
            const uint32_t rows = std::min(band_bh, bh - b * band_bh);
            for (int k = 0; k < (both ? 2 : 1); ++k)
                std::memcpy(planes[k] + (size_t)b * band_bh * bw * 8, hp.h_dst[s].p + k * band_out,
                            (size_t)rows * bw * 8);
        }
        return GOOFY_OK;
    };
    for (uint32_t b = 0; b < nbands; ++b) {
        const int s = (int)(b % slots);
        if (b >= (uint32_t)slots && (rc = finish_band(b - slots)) != GOOFY_OK) return rc;
        const uint32_t rows = std::min(band_bh, bh - b * band_bh);
        const uint8_t* sb = src + (size_t)b * band_bh * 4 * stride;
        cudaStream_t st = hp.stream[s];
        if (src_pinned) {
            CUDA_TRY(cudaMemcpy2DAsync(hp.d_src[s].p, dpitch, sb, stride, row_bytes, (size_t)rows * 4,
                                       cudaMemcpyHostToDevice, st));
        } else {
            uint8_t* stage = hp.h_src[s].p;
            for (size_t y = 0; y < (size_t)rows * 4; ++y) std::memcpy(stage + y * dpitch, sb + y * stride, row_bytes);
            CUDA_TRY(cudaMemcpyAsync(hp.d_src[s].p, stage, (size_t)rows * 4 * dpitch, cudaMemcpyHostToDevice, st));
        }
        CUDA_TRY(goofy_gpu::launch_image(codec, hp.d_src[s].p, dpitch, hp.d_dst[s].p, width, rows * 4, tile,
                                         SrcAccess::kVec16, st, both ? hp.d_dst[s].p + band_out : nullptr));
        for (int k = 0; k < (both ? 2 : 1); ++k) {
            uint8_t* out = dst_pinned ? planes[k] + (size_t)b * band_bh * bw * 8 : hp.h_dst[s].p + k * band_out;
            CUDA_TRY(cudaMemcpyAsync(out, hp.d_dst[s].p + k * band_out, (size_t)rows * bw * 8,
                                     cudaMemcpyDeviceToHost, st));
        }
        CUDA_TRY(cudaEventRecord(hp.done[s], st));
    }
    for (uint32_t b = nbands > (uint32_t)slots ? nbands - slots : 0; b < nbands; ++b)
        if ((rc = finish_band(b)) != GOOFY_OK) return rc;
    return GOOFY_OK;
}

int compress_device_impl(int codec, void* dst, const void* src, uint32_t width, uint32_t height, uint32_t stride,
                         void* stream)
{
    int rc = check_args(codec, dst, src, width, height, stride);
    if (rc <= 0) return rc;
    if (reinterpret_cast<uintptr_t>(dst) % 8 != 0) return GOOFY_ERR_ALIGNMENT;
    const uintptr_t s = reinterpret_cast<uintptr_t>(src);
    SrcAccess access;
    if (s % 16 == 0 && stride % 16 == 0) access = SrcAccess::kVec16;
    else if (s % 4 == 0 && stride % 4 == 0) access = SrcAccess::kWord4;
    else return GOOFY_ERR_ALIGNMENT;
    ensure_tile_cache_current();
    CUDA_TRY(goofy_gpu::launch_image(codec, static_cast<const uint8_t*>(src), stride, static_cast<uint8_t*>(dst),
                                     width, height, tile_for(codec), access, static_cast<cudaStream_t>(stream)));
    return GOOFY_OK;
}

int compress_both_device_impl(void* dst_bc1, void* dst_etc1s, const void* src, uint32_t width, uint32_t height,
                              uint32_t stride, void* stream)
{
    int rc = check_args(GOOFY_CODEC_BC1, dst_bc1, src, width, height, stride);
    if (rc <= 0) return rc;
    if (!dst_etc1s || outputs_overlap(dst_bc1, dst_etc1s, width, height)) return GOOFY_ERR_INVALID;
    if (reinterpret_cast<uintptr_t>(dst_bc1) % 8 != 0 || reinterpret_cast<uintptr_t>(dst_etc1s) % 8 != 0)
        return GOOFY_ERR_ALIGNMENT;
    const uintptr_t s = reinterpret_cast<uintptr_t>(src);
    SrcAccess access;
    if (s % 16 == 0 && stride % 16 == 0) access = SrcAccess::kVec16;
    else if (s % 4 == 0 && stride % 4 == 0) access = SrcAccess::kWord4;
    else return GOOFY_ERR_ALIGNMENT;
    ensure_tile_cache_current();
    CUDA_TRY(goofy_gpu::launch_image(GOOFY_CODEC_BOTH, static_cast<const uint8_t*>(src), stride,
                                     static_cast<uint8_t*>(dst_bc1), width, height, tile_for(GOOFY_CODEC_BOTH), access,
                                     static_cast<cudaStream_t>(stream), static_cast<uint8_t*>(dst_etc1s)));
    return GOOFY_OK;
}

// Times launches for the autotuners on a stream of their own: after two
// warm-up launches, three rounds of `reps` launches back to back between two
// events (an event between two launches would delay the second one's start);
// `ms` is the median round's mean time of one launch(k).
struct Timer {
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[2] = {nullptr, nullptr};

    int init()
    {
        CUDA_TRY(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        for (auto& e : ev) CUDA_TRY(cudaEventCreate(&e));
        return GOOFY_OK;
    }

    ~Timer()
    {
        for (auto& e : ev)
            if (e) cudaEventDestroy(e);
        if (stream) cudaStreamDestroy(stream);
    }

    template <typename F>
    cudaError_t time(uint32_t reps, float& ms, F launch)
    {
        float t[3];
        cudaError_t e = cudaSuccess;
        for (uint32_t w = 0; w < 2 && e == cudaSuccess; ++w) e = launch(w);
        for (int r = 0; r < 3 && e == cudaSuccess; ++r) {
            e = cudaEventRecord(ev[0], stream);
            for (uint32_t k = 0; k < reps && e == cudaSuccess; ++k) e = launch(k);
            if (e == cudaSuccess) e = cudaEventRecord(ev[1], stream);
            if (e == cudaSuccess) e = cudaEventSynchronize(ev[1]);
            if (e == cudaSuccess) e = cudaEventElapsedTime(&t[r], ev[0], ev[1]);
            t[r] /= (float)reps;
        }
        std::sort(t, t + 3);
        ms = t[1];
        return e;
    }
};

// Every tile shape of `codec`, fastest first, as (mean ms a launch, tile).
int rank_tiles(Timer& tm, int codec, uint8_t* dst, uint8_t* dst2, const uint8_t* src, uint32_t stride,
               uint32_t width, uint32_t height, SrcAccess access, uint32_t reps,
               std::vector<std::pair<float, Tile>>* ranked)
{
    const bool both = codec == GOOFY_CODEC_BOTH;
    ranked->clear();
    for (uint32_t persistent : {0u, 1u, 2u})
        for (uint32_t threads : {128u, 256u, 512u})
            for (uint32_t bpt : {1u, 2u, 4u}) {
                const Tile t{threads, bpt, persistent};
                if (!goofy_gpu::tile_valid(t) || (both && (bpt > 2 || persistent == 1))) continue;
                float ms = 0.f;
                const cudaError_t e = tm.time(reps, ms, [&](uint32_t) {
                    return goofy_gpu::launch_image(codec, src, stride, dst, width, height, t, access, tm.stream, dst2);
                });
                if (e != cudaSuccess) return cuda_fail(e, "autotune launch");
                ranked->emplace_back(ms, t);
            }
    std::stable_sort(ranked->begin(), ranked->end(),
                     [](const std::pair<float, Tile>& a, const std::pair<float, Tile>& b) { return a.first < b.first; });
    return GOOFY_OK;
}

// Installs a tuned tile as the codec's (an explicit setting) and records it
// for this GPU model; a cache that cannot be written keeps the result valid
// for this process.
void install_and_record(int codec, const Tile& t, float ms)
{
    {
        std::lock_guard<std::mutex> lk(g_tile_mu);
        g_tile[codec] = t;
        g_tile_explicit[codec] = true;
    }
    int dev = 0;
    std::string name;
    uint32_t sms = 0;
    const std::string path = goofy_gpu::tile_cache_path();
    if (!path.empty() && cudaGetDevice(&dev) == cudaSuccess && device_key(dev, &name, &sms) == GOOFY_OK)
        goofy_gpu::tile_cache_store(path, name, sms, codec, t, ms > 0.f ? ms * 1e3f : 1.f);
    cudaGetLastError();
}

}  // namespace

extern "C" {

GOOFY_EXPORT int goofy_gpu_init(int device)
{
    HostPath& hp = host_path();
    std::lock_guard<std::mutex> lk(hp.mu);
    const int rc = hp.init_locked(device);
    if (rc == GOOFY_OK) ensure_tile_cache(device);
    return rc;
}

GOOFY_EXPORT void goofy_gpu_shutdown(void)
{
    HostPath& hp = host_path();
    std::lock_guard<std::mutex> lk(hp.mu);
    hp.release_locked();
}

GOOFY_EXPORT const char* goofy_gpu_status_string(int status)
{
    switch (status) {
    case GOOFY_OK: return "ok";
    case GOOFY_ERR_WIDTH: return "width is not a multiple of the block width";
    case GOOFY_ERR_HEIGHT: return "height is not a multiple of 4";
    case GOOFY_ERR_INVALID: return "invalid argument";
    case GOOFY_ERR_ALIGNMENT: return "misaligned pointer or stride";
    case GOOFY_ERR_CUDA: return "CUDA error";
    case GOOFY_ERR_NOMEM: return "out of memory";
    case GOOFY_ERR_TIMEOUT: return "timed out";
    case GOOFY_ERR_BUSY: return "busy";
    case GOOFY_ERR_NO_DEVICE: return "no CUDA device";
    case GOOFY_ERR_TOO_LARGE: return "request exceeds capacity";
    default: return "unknown status";
    }
}

GOOFY_EXPORT const char* goofy_gpu_last_error(void) { return goofy_gpu::last_error_text(); }

GOOFY_EXPORT int goofy_gpu_compress_device(int codec, void* dst, const void* src, uint32_t width, uint32_t height,
                                           uint32_t stride, void* stream)
{
    return compress_device_impl(codec, dst, src, width, height, stride, stream);
}

GOOFY_EXPORT int goofy_gpu_compress_bc1_device(void* dst, const void* src, uint32_t width, uint32_t height,
                                               uint32_t stride, void* stream)
{
    return compress_device_impl(GOOFY_CODEC_BC1, dst, src, width, height, stride, stream);
}

GOOFY_EXPORT int goofy_gpu_compress_etc1s_device(void* dst, const void* src, uint32_t width, uint32_t height,
                                                 uint32_t stride, void* stream)
{
    return compress_device_impl(GOOFY_CODEC_ETC1S, dst, src, width, height, stride, stream);
}

GOOFY_EXPORT int goofy_gpu_compress_host(int codec, uint8_t* dst, const uint8_t* src, uint32_t width,
                                         uint32_t height, uint32_t stride)
{
    return compress_host_impl(codec, dst, src, width, height, stride);
}

GOOFY_EXPORT int goofy_gpu_compress_both_device(void* dst_bc1, void* dst_etc1s, const void* src, uint32_t width,
                                                uint32_t height, uint32_t stride, void* stream)
{
    return compress_both_device_impl(dst_bc1, dst_etc1s, src, width, height, stride, stream);
}

GOOFY_EXPORT int goofy_gpu_compress_both_host(uint8_t* dst_bc1, uint8_t* dst_etc1s, const uint8_t* src,
                                              uint32_t width, uint32_t height, uint32_t stride)
{
    return compress_host_impl(GOOFY_CODEC_BOTH, dst_bc1, src, width, height, stride, dst_etc1s);
}

GOOFY_EXPORT int goofy_gpu_compress_bc1_host(uint8_t* dst, const uint8_t* src, uint32_t width, uint32_t height,
                                             uint32_t stride)
{
    return compress_host_impl(GOOFY_CODEC_BC1, dst, src, width, height, stride);
}

GOOFY_EXPORT int goofy_gpu_compress_etc1s_host(uint8_t* dst, const uint8_t* src, uint32_t width, uint32_t height,
                                               uint32_t stride)
{
    return compress_host_impl(GOOFY_CODEC_ETC1S, dst, src, width, height, stride);
}

GOOFY_EXPORT int goofy_gpu_set_host_path(int path)
{
    if (path != GOOFY_HOST_PATH_AUTO && path != GOOFY_HOST_PATH_STAGED && path != GOOFY_HOST_PATH_DIRECT)
        return GOOFY_ERR_INVALID;
    g_host_path.store(path);
    return GOOFY_OK;
}

GOOFY_EXPORT int goofy_gpu_get_host_path(void) { return g_host_path.load(); }

GOOFY_EXPORT void* goofy_gpu_host_alloc(size_t bytes)
{
    void* p = nullptr;
    if (cudaHostAlloc(&p, bytes, cudaHostAllocDefault) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return p;
}

GOOFY_EXPORT void goofy_gpu_host_free(void* p)
{
    if (p) cudaFreeHost(p);
}

GOOFY_EXPORT int goofy_gpu_get_tile(int codec, goofy_gpu_tile* tile)
{
    if (!tile || codec < GOOFY_CODEC_BC1 || codec > GOOFY_CODEC_BOTH) return GOOFY_ERR_INVALID;
    const Tile t = tile_for(codec);
    tile->threads_per_cta = t.threads;
    tile->blocks_per_thread = t.bpt;
    tile->persistent = t.persistent;
    return GOOFY_OK;
}

GOOFY_EXPORT int goofy_gpu_set_tile(int codec, const goofy_gpu_tile* tile)
{
    if (!tile || codec < GOOFY_CODEC_BC1 || codec > GOOFY_CODEC_BOTH) return GOOFY_ERR_INVALID;
    const Tile t{tile->threads_per_cta, tile->blocks_per_thread, tile->persistent};
    if (!goofy_gpu::tile_valid(t) || (codec == GOOFY_CODEC_BOTH && t.bpt > 2)) return GOOFY_ERR_INVALID;
    std::lock_guard<std::mutex> lk(g_tile_mu);
    g_tile[codec] = t;
    g_tile_explicit[codec] = true;
    return GOOFY_OK;
}

GOOFY_EXPORT int goofy_gpu_reset_tiles(void)
{
    std::lock_guard<std::mutex> lk(g_tile_mu);
    for (int c = 0; c < 3; ++c) {
        g_tile[c] = kDefaultTile[c];
        g_tile_explicit[c] = false;
    }
    for (auto& f : g_cache_loaded) f.store(false);
    return GOOFY_OK;
}

GOOFY_EXPORT int goofy_gpu_set_tile_cache_path(const char* path)
{
    goofy_gpu::set_tile_cache_path(path);
    return GOOFY_OK;
}

GOOFY_EXPORT size_t goofy_gpu_get_tile_cache_path(char* buf, size_t size)
{
    const std::string p = goofy_gpu::tile_cache_path();
    if (buf && size) {
        const size_t n = std::min(size - 1, p.size());
        std::memcpy(buf, p.data(), n);
        buf[n] = '\0';
    }
    return p.size();
}

GOOFY_EXPORT int goofy_gpu_device_key(int device, char* name, size_t size, uint32_t* sm_count)
{
    if (!name || size == 0 || !sm_count) return GOOFY_ERR_INVALID;
    std::string n;
    const int rc = device_key(device, &n, sm_count);
    if (rc != GOOFY_OK) return rc;
    const size_t k = std::min(size - 1, n.size());
    std::memcpy(name, n.data(), k);
    name[k] = '\0';
    return GOOFY_OK;
}

GOOFY_EXPORT int goofy_gpu_tile_cache_store(const char* path, const char* gpu_name, uint32_t sm_count, int codec,
                                            const goofy_gpu_tile* tile, float us)
{
    if (!gpu_name || !tile) return GOOFY_ERR_INVALID;
    const Tile t{tile->threads_per_cta, tile->blocks_per_thread, tile->persistent};
    return goofy_gpu::tile_cache_store(path ? std::string(path) : goofy_gpu::tile_cache_path(), gpu_name, sm_count,
                                       codec, t, us);
}

GOOFY_EXPORT int goofy_gpu_tile_cache_lookup(const char* path, const char* gpu_name, uint32_t sm_count, int codec,
                                             goofy_gpu_tile* tile)
{
    if (!gpu_name || !tile) return GOOFY_ERR_INVALID;
    Tile t{0, 0, 0};
    if (!goofy_gpu::tile_cache_lookup(path ? std::string(path) : goofy_gpu::tile_cache_path(), gpu_name, sm_count,
                                      codec, &t))
        return goofy_gpu::fail(GOOFY_ERR_INVALID, "tile cache: no entry");
    tile->threads_per_cta = t.threads;
    tile->blocks_per_thread = t.bpt;
    tile->persistent = t.persistent;
    return GOOFY_OK;
}

GOOFY_EXPORT int goofy_gpu_load_tile_cache(int device) { return load_tile_cache(device); }

GOOFY_EXPORT int goofy_gpu_autotune(int codec, void* dst, const void* src, uint32_t width, uint32_t height,
                                   uint32_t stride, uint32_t reps, goofy_gpu_tile* best, float* best_us)
{
    const bool both = codec == GOOFY_CODEC_BOTH;  // dst: the BC1 blocks, then the ETC1s blocks
    int rc = check_args(both ? GOOFY_CODEC_BC1 : codec, dst, src, width, height, stride);
    if (rc <= 0) return rc == GOOFY_OK ? GOOFY_ERR_INVALID : rc;
    if (reps == 0 || reps > 1000) return GOOFY_ERR_INVALID;
    const uintptr_t s = reinterpret_cast<uintptr_t>(src);
    if (reinterpret_cast<uintptr_t>(dst) % 8 != 0 || s % 4 != 0 || stride % 4 != 0) return GOOFY_ERR_ALIGNMENT;
    const SrcAccess access = (s % 16 == 0 && stride % 16 == 0) ? SrcAccess::kVec16 : SrcAccess::kWord4;
    Timer tm;
    if ((rc = tm.init()) != GOOFY_OK) return rc;
    uint8_t* const dst2 = both ? static_cast<uint8_t*>(dst) + (size_t)(width / 4) * (height / 4) * 8 : nullptr;
    std::vector<std::pair<float, Tile>> ranked;
    if ((rc = rank_tiles(tm, codec, static_cast<uint8_t*>(dst), dst2, static_cast<const uint8_t*>(src), stride,
                         width, height, access, reps, &ranked)) != GOOFY_OK)
        return rc;
    const Tile best_tile = ranked[0].second;
    const float best_time = ranked[0].first;
    install_and_record(codec, best_tile, best_time);
    if (best) {
        best->threads_per_cta = best_tile.threads;
        best->blocks_per_thread = best_tile.bpt;
        best->persistent = best_tile.persistent;
    }
    if (best_us) *best_us = best_time * 1e3f;
    return GOOFY_OK;
}

GOOFY_EXPORT int goofy_gpu_autotune_pair(void* dst_bc1, void* dst_etc1s, const void* src, uint32_t width,
                                        uint32_t height, uint32_t stride, uint32_t reps, goofy_gpu_tile* best_bc1,
                                        goofy_gpu_tile* best_etc1s, float* best_us)
{
    int rc = check_args(GOOFY_CODEC_BC1, dst_bc1, src, width, height, stride);
    if (rc <= 0) return rc == GOOFY_OK ? GOOFY_ERR_INVALID : rc;
    if (!dst_etc1s || outputs_overlap(dst_bc1, dst_etc1s, width, height)) return GOOFY_ERR_INVALID;
    if (reps == 0 || reps > 1000) return GOOFY_ERR_INVALID;
    const uintptr_t s = reinterpret_cast<uintptr_t>(src);
    if (reinterpret_cast<uintptr_t>(dst_bc1) % 8 || reinterpret_cast<uintptr_t>(dst_etc1s) % 8 || s % 4 ||
        stride % 4)
        return GOOFY_ERR_ALIGNMENT;
    const SrcAccess access = (s % 16 == 0 && stride % 16 == 0) ? SrcAccess::kVec16 : SrcAccess::kWord4;
    const uint8_t* in = static_cast<const uint8_t*>(src);
    uint8_t* out[2] = {static_cast<uint8_t*>(dst_bc1), static_cast<uint8_t*>(dst_etc1s)};
    Timer tm;
    if ((rc = tm.init()) != GOOFY_OK) return rc;
    // Each codec alone first.  Finalists per codec: its three fastest shapes and its three fastest
    // bulk-copy shapes (a bulk-copy BC1 launch hands the SMs to a bulk-copy ETC1s launch without a
    // gap, so it can win the pair while losing alone).  The finalists' pairs then run as the
    // alternating BC1 / ETC1s launches on one image that a caller encoding every image with both
    // codecs issues.
    std::vector<std::pair<float, Tile>> ranked[2];
    std::vector<Tile> finalists[2];
    for (int c = 0; c < 2; ++c) {
        if ((rc = rank_tiles(tm, c, out[c], nullptr, in, stride, width, height, access, reps, &ranked[c])) !=
            GOOFY_OK)
            return rc;
        size_t fast = 0, bulk = 0;
        for (const auto& r : ranked[c]) {
            const bool is_bulk = r.second.persistent == 2;
            if (fast < 3 || (is_bulk && bulk < 3)) finalists[c].push_back(r.second);
            ++fast;
            if (is_bulk) ++bulk;
        }
    }
    Tile best[2] = {ranked[0][0].second, ranked[1][0].second};
    float best_time = -1.f;
    for (const Tile& t0 : finalists[0])
        for (const Tile& t1 : finalists[1]) {
            const Tile t[2] = {t0, t1};
            float ms = 0.f;
            const cudaError_t e = tm.time(reps, ms, [&](uint32_t k) -> cudaError_t {
                cudaError_t r = goofy_gpu::launch_image(GOOFY_CODEC_BC1, in, stride, out[0], width, height, t[0],
                                                        access, tm.stream);
                (void)k;
                return r == cudaSuccess ? goofy_gpu::launch_image(GOOFY_CODEC_ETC1S, in, stride, out[1], width,
                                                                  height, t[1], access, tm.stream)
                                        : r;
            });
            if (e != cudaSuccess) return cuda_fail(e, "autotune pair launch");
            if (best_time < 0.f || ms < best_time) {
                best_time = ms;
                best[0] = t[0];
                best[1] = t[1];
            }
        }
    for (int c = 0; c < 2; ++c) {
        float alone = 0.f;
        for (const auto& r : ranked[c])
            if (r.second.threads == best[c].threads && r.second.bpt == best[c].bpt &&
                r.second.persistent == best[c].persistent)
                alone = r.first;
        install_and_record(c, best[c], alone);
    }
    goofy_gpu_tile* const want[2] = {best_bc1, best_etc1s};
    for (int c = 0; c < 2; ++c)
        if (want[c]) {
            want[c]->threads_per_cta = best[c].threads;
            want[c]->blocks_per_thread = best[c].bpt;
            want[c]->persistent = best[c].persistent;
        }
    if (best_us) *best_us = best_time * 1e3f;
    return GOOFY_OK;
}

GOOFY_EXPORT int goofy_gpu_selftest_bounded_wait(uint32_t* elapsed_ms)
{
    const auto t0 = std::chrono::steady_clock::now();
    bool completed = true, aborted = false;
    unsigned int counted = 0;
    CUDA_TRY(goofy_gpu::bounded_wait_selftest(&completed, &aborted, &counted));
    if (elapsed_ms)
        *elapsed_ms = (uint32_t)std::chrono::duration_cast<std::chrono::milliseconds>(
                          std::chrono::steady_clock::now() - t0).count();
    if (completed || !aborted || counted != 1) {
        char what[128];
        std::snprintf(what, sizeof what, "bounded wait self-test: completed %d, abort flag %d, time-outs counted %u",
                      (int)completed, (int)aborted, counted);
        return goofy_gpu::fail(GOOFY_ERR_CUDA, what);
    }
    return GOOFY_OK;
}

GOOFY_EXPORT int goofy_gpu_pipeline_timeouts(uint32_t* count, int reset)
{
    if (!count) return GOOFY_ERR_INVALID;
    unsigned int n = 0;
    CUDA_TRY(goofy_gpu::pipeline_timeouts(&n, reset != 0));
    *count = n;
    return GOOFY_OK;
}

}  // extern "C"

// ---- C++ drop-in: goofy::compressDXT1 / compressETC1 (goofy_tc.h:10-13) ----
namespace goofy {

GOOFY_EXPORT int compressDXT1(unsigned char* result, const unsigned char* input, unsigned int width,
                              unsigned int height, unsigned int stride)
{
    if (width % 16 != 0) return -1;  // goofy_tc.h:1500-1503
    if (height % 4 != 0) return -2;  // goofy_tc.h:1505-1508
    return compress_host_impl(GOOFY_CODEC_BC1, result, input, width, height, stride);
}

GOOFY_EXPORT int compressETC1(unsigned char* result, const unsigned char* input, unsigned int width,
                              unsigned int height, unsigned int stride)
{
    if (width % 16 != 0) return -1;  // goofy_tc.h:1531-1534
    if (height % 4 != 0) return -2;  // goofy_tc.h:1536-1539
    return compress_host_impl(GOOFY_CODEC_ETC1S, result, input, width, height, stride);
}

}  // namespace goofy
