// server_replay.cpp -- open-loop load replay for measuring the request server,
// and the plain one-request-per-launch loop it is compared with.  Both take a
// request list with arrival times (offsets from the start, e.g. a Poisson
// process) and report, per request, the latency from its scheduled arrival to
// its completion, so time a request waits because the system is behind is
// counted (open loop).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <thread>
#include <vector>

#include "../../include/goofy_gpu.h"
#include "host_util.h"
#include "kernels.h"

namespace {

void wait_until(int64_t t_ns)
{
    for (;;) {
        const int64_t now = goofy_gpu_now_ns();
        if (now >= t_ns) return;
        if (t_ns - now > 200000) std::this_thread::sleep_for(std::chrono::microseconds((t_ns - now) / 2000));
    }
}

}  // namespace

extern "C" {

GOOFY_EXPORT int goofy_gpu_server_replay(goofy_gpu_server* s, const goofy_gpu_request* reqs, const int64_t* arrival_ns,
                                         uint32_t n, int64_t* latency_ns, int64_t* wall_ns,
                                         goofy_gpu_request_times* times)
{
    if (!s || !reqs || !arrival_ns || !latency_ns || n == 0) return GOOFY_ERR_INVALID;
    std::vector<uint64_t> tickets(n, 0);
    std::vector<std::atomic<int>> ready(n);
    for (auto& r : ready) r.store(0, std::memory_order_relaxed);
    std::atomic<int> first_error{GOOFY_OK};
    const int64_t t0 = goofy_gpu_now_ns() + 2000000;  // 2 ms to get both threads going
    std::thread collector([&] {
        for (uint32_t i = 0; i < n; ++i) {
            int st;
            // the latency comes from the completion timestamp, so this thread
            // may lag; it sleeps rather than spin so it takes no core from the
            // submitting and scheduling threads
            while ((st = ready[i].load(std::memory_order_acquire)) == 0)
                std::this_thread::sleep_for(std::chrono::microseconds(50));
            if (st < 0) {
                latency_ns[i] = -1;
                continue;
            }
            goofy_gpu_request_times t{};
            const int rc = goofy_gpu_server_wait(s, tickets[i], 600000, &t);
            if (rc != GOOFY_OK) {
                int expected = GOOFY_OK;
                first_error.compare_exchange_strong(expected, rc);
                latency_ns[i] = -1;
                continue;
            }
            latency_ns[i] = t.done_ns - (t0 + arrival_ns[i]);
            if (times) times[i] = t;
        }
    });
    for (uint32_t i = 0; i < n; ++i) {
        wait_until(t0 + arrival_ns[i]);
        int rc;
        while ((rc = goofy_gpu_server_submit(s, &reqs[i], &tickets[i])) == GOOFY_ERR_BUSY)
            std::this_thread::sleep_for(std::chrono::microseconds(20));  // ticket ring full: the collector releases tickets
        if (rc != GOOFY_OK) {
            int expected = GOOFY_OK;
            first_error.compare_exchange_strong(expected, rc);
            ready[i].store(-1, std::memory_order_release);
        } else {
            ready[i].store(1, std::memory_order_release);
        }
    }
    collector.join();
    if (wall_ns) *wall_ns = goofy_gpu_now_ns() - t0;
    return first_error.load();
}

GOOFY_EXPORT int goofy_gpu_plain_replay(int device, const goofy_gpu_request* reqs, const int64_t* arrival_ns,
                                        uint32_t n, int64_t* latency_ns, int64_t* wall_ns)
{
    if (!reqs || !arrival_ns || !latency_ns || n == 0) return GOOFY_ERR_INVALID;
    goofy_gpu::DeviceGuard g(device);
    GOOFY_CUDA_TRY(g.err);
    size_t in_cap = 0, out_cap = 0;
    for (uint32_t i = 0; i < n; ++i) {
        in_cap = std::max<size_t>(in_cap, (size_t)((4ull * reqs[i].width + 15) & ~15ull) * reqs[i].height);
        out_cap = std::max<size_t>(out_cap, (size_t)(reqs[i].width / 4) * (reqs[i].height / 4) * 8);
    }
    uint8_t *d_in = nullptr, *d_out = nullptr;
    cudaStream_t st = nullptr;
    GOOFY_CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    int rc = GOOFY_OK;
    cudaError_t e = cudaMalloc(&d_in, in_cap ? in_cap : 16);
    if (e == cudaSuccess) e = cudaMalloc(&d_out, out_cap ? out_cap : 16);
    if (e != cudaSuccess) rc = goofy_gpu::cuda_fail(e, "plain replay buffers");
    goofy_gpu_tile tiles[2];
    goofy_gpu_get_tile(0, &tiles[0]);
    goofy_gpu_get_tile(1, &tiles[1]);
    const int64_t t0 = goofy_gpu_now_ns() + 1000000;
    for (uint32_t i = 0; i < n && rc == GOOFY_OK; ++i) {
        const goofy_gpu_request& q = reqs[i];
        wait_until(t0 + arrival_ns[i]);
        const size_t dpitch = (4ull * q.width + 15) & ~15ull;
        const goofy_gpu_tile& t = tiles[q.codec & 1];
        e = cudaMemcpy2DAsync(d_in, dpitch, q.src, q.stride, 4ull * q.width, q.height, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess)
            e = goofy_gpu::launch_image(q.codec, d_in, dpitch, d_out, q.width, q.height,
                                        goofy_gpu::Tile{t.threads_per_cta, t.blocks_per_thread, t.persistent},
                                        goofy_gpu::SrcAccess::kVec16, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(q.dst, d_out, (size_t)(q.width / 4) * (q.height / 4) * 8, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            rc = goofy_gpu::cuda_fail(e, "plain replay");
            break;
        }
        latency_ns[i] = goofy_gpu_now_ns() - (t0 + arrival_ns[i]);
    }
    if (wall_ns) *wall_ns = goofy_gpu_now_ns() - t0;
    if (d_in) cudaFree(d_in);
    if (d_out) cudaFree(d_out);
    cudaStreamDestroy(st);
    return rc;
}

}  // extern "C"
