// Large copies between pageable host memory and the device, through page-locked staging buffers
// with the host side split over threads.
//
// A cudaMemcpyAsync from or to pageable memory runs the host-side memcpy into the driver's
// staging (and, for a fresh destination, the first-touch page faults) on the calling thread
// alone: a few tens of GB/s.  Here a transfer of at least kMinStaged bytes is cut into one
// contiguous segment per thread; each thread pipelines its segment through two page-locked slots
// on its own stream, the memcpy of one chunk overlapping the DMA of the other.  Page-locked host
// buffers (cudaHostAlloc, cudaHostRegister) and small transfers take the plain copy.
#include <algorithm>
#include <cstring>
#include <thread>
#include <vector>

#include "astro_internal.h"

namespace {

constexpr size_t kSlot = 8u << 20;        // bytes per staging slot
constexpr int kMaxThreads = 8;            // host threads (and streams) per transfer
constexpr size_t kMinStaged = 64u << 20;  // smaller transfers: one plain copy

bool page_locked(const void *p) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

}  // namespace

struct HostStage {
    int threads = 0;
    void *pinned[kMaxThreads][2] = {};
    cudaStream_t stream[kMaxThreads] = {};
    cudaEvent_t ev[kMaxThreads][2] = {};
};

void host_stage_release(astro_ctx *ctx) {
    HostStage *S = ctx->stage;
    if (!S) return;
    for (int t = 0; t < kMaxThreads; ++t) {
        for (int k = 0; k < 2; ++k) {
            if (S->pinned[t][k]) cudaFreeHost(S->pinned[t][k]);
            if (S->ev[t][k]) cudaEventDestroy(S->ev[t][k]);
        }
        if (S->stream[t]) cudaStreamDestroy(S->stream[t]);
    }
    delete S;
    ctx->stage = nullptr;
}

static bool stage_ready(astro_ctx *ctx) {
    if (ctx->stage) return true;
    HostStage *S = new HostStage;
    const unsigned hc = std::thread::hardware_concurrency();
    S->threads = std::max(1, std::min(kMaxThreads, hc ? (int)hc / 2 : 4));
    bool ok = cudaSetDevice(ctx->device) == cudaSuccess;  // the streams belong to the context's device
    for (int t = 0; t < S->threads && ok; ++t) {
        for (int k = 0; k < 2 && ok; ++k)
            ok = cudaHostAlloc(&S->pinned[t][k], kSlot, cudaHostAllocDefault) == cudaSuccess &&
                 cudaEventCreateWithFlags(&S->ev[t][k], cudaEventDisableTiming) == cudaSuccess;
        ok = ok && cudaStreamCreateWithFlags(&S->stream[t], cudaStreamNonBlocking) == cudaSuccess;
    }
    ctx->stage = S;
    if (!ok) {  // no staging: the plain copy serves
        cudaGetLastError();
        host_stage_release(ctx);
    }
    return ok;
}

// Runs fn(t, b0, b1) on the stage's threads over byte segments of [0, bytes); first error wins.
template <class F> static cudaError_t stage_run(astro_ctx *ctx, size_t bytes, F fn) {
    HostStage *S = ctx->stage;
    const int T = S->threads;
    const size_t seg = ((bytes + T - 1) / T + 4095) / 4096 * 4096;
    std::vector<cudaError_t> err(T, cudaSuccess);
    std::vector<std::thread> th;
    for (int t = 0; t < T; ++t)
        th.emplace_back([&, t] {
            const size_t b0 = std::min(bytes, (size_t)t * seg), b1 = std::min(bytes, b0 + seg);
            cudaError_t e = cudaSetDevice(ctx->device);
            if (e == cudaSuccess && b1 > b0) e = fn(t, b0, b1);
            if (e == cudaSuccess) e = cudaStreamSynchronize(S->stream[t]);
            err[t] = e;
        });
    for (std::thread &x : th) x.join();
    for (cudaError_t e : err)
        if (e != cudaSuccess) return e;
    return cudaSuccess;
}

// dst (device) <- src (host); complete on return.
int copy_to_device(astro_ctx *ctx, void *dst, const void *src, size_t bytes, const char *what) {
    if (bytes < kMinStaged || page_locked(src) || !stage_ready(ctx)) {
        cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        return cuda_check(ctx, e, what);
    }
    // earlier work on the library stream may still use the destination
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_check(ctx, e, what);
    HostStage *S = ctx->stage;
    e = stage_run(ctx, bytes, [&](int t, size_t b0, size_t b1) {
        cudaError_t r = cudaSuccess;
        int i = 0;
        for (size_t o = b0; o < b1 && r == cudaSuccess; o += kSlot, ++i) {
            const int sl = i & 1;
            const size_t len = std::min(kSlot, b1 - o);
            if (i >= 2) r = cudaEventSynchronize(S->ev[t][sl]);  // the slot's previous DMA
            if (r != cudaSuccess) break;
            std::memcpy(S->pinned[t][sl], static_cast<const char *>(src) + o, len);
            r = cudaMemcpyAsync(static_cast<char *>(dst) + o, S->pinned[t][sl], len, cudaMemcpyHostToDevice,
                                S->stream[t]);
            if (r == cudaSuccess) r = cudaEventRecord(S->ev[t][sl], S->stream[t]);
        }
        return r;
    });
    return cuda_check(ctx, e, what);
}

// dst (host) <- src (device) after the work queued on the library stream; complete on return.
int copy_to_host(astro_ctx *ctx, void *dst, const void *src, size_t bytes, const char *what) {
    if (bytes < kMinStaged || page_locked(dst) || !stage_ready(ctx)) {
        cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        return cuda_check(ctx, e, what);
    }
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_check(ctx, e, what);
    HostStage *S = ctx->stage;
    e = stage_run(ctx, bytes, [&](int t, size_t b0, size_t b1) {
        const size_t n = (b1 - b0 + kSlot - 1) / kSlot;
        auto issue = [&](size_t i) {
            const size_t o = b0 + i * kSlot, len = std::min(kSlot, b1 - o);
            cudaError_t r = cudaMemcpyAsync(S->pinned[t][i & 1], static_cast<const char *>(src) + o, len,
                                            cudaMemcpyDeviceToHost, S->stream[t]);
            return r == cudaSuccess ? cudaEventRecord(S->ev[t][i & 1], S->stream[t]) : r;
        };
        cudaError_t r = issue(0);
        for (size_t i = 0; i < n && r == cudaSuccess; ++i) {
            // chunk i + 1 into the other slot (its previous chunk was copied out last trip)
            if (i + 1 < n && (r = issue(i + 1)) != cudaSuccess) break;
            if ((r = cudaEventSynchronize(S->ev[t][i & 1])) != cudaSuccess) break;
            const size_t o = b0 + i * kSlot;
            std::memcpy(static_cast<char *>(dst) + o, S->pinned[t][i & 1], std::min(kSlot, b1 - o));
        }
        return r;
    });
    return cuda_check(ctx, e, what);
}
