// Autotuner of the launch shapes (no counterpart in the reference).
//
// A few kernels have a launch shape whose best value depends on the model and the GPU: the
// zero-state brick kernel's warps per CTA (occupancy against colour tails), the band
// factorisation's CTAs per cluster (parallelism inside a panel against the number of panels
// that run at once), and the many-column band solve's CTAs per cluster (tiles per producer warp
// against the cluster barrier's cost).  astro_autotune times every candidate on the context's own
// model with CUDA events and keeps the fastest for the context; a cache file remembers the choice
// per GPU, tunable and model size, so a later run applies it without timing.
#include <cmath>
#include <cstdio>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "astro_internal.h"

int launch_hex8_assemble(astro_ctx *ctx, int precision, int store);  // elem_hex8.cu

namespace {

std::string gpu_name(astro_ctx *ctx) {
    cudaDeviceProp p{};
    if (cudaGetDeviceProperties(&p, ctx->device) != cudaSuccess) return "unknown";
    std::string s(p.name);
    for (char &c : s)
        if (c == ' ') c = '_';
    return s;
}

// cache lines: "<key> <choice> <seconds>"
bool cache_find(const char *path, const std::string &key, int *choice) {
    if (!path) return false;
    std::ifstream f(path);
    std::string line;
    bool hit = false;
    while (std::getline(f, line)) {
        std::istringstream is(line);
        std::string k;
        int c = 0;
        if (is >> k >> c && k == key) {
            *choice = c;  // the last entry for a key wins
            hit = true;
        }
    }
    return hit;
}

void cache_add(const char *path, const std::string &key, int choice, double seconds) {
    if (!path) return;
    std::ofstream f(path, std::ios::app);
    if (f) f << key << " " << choice << " " << seconds << "\n";
}

// seconds per call of fn (CUDA events on the context's stream, after one warm-up call)
template <class F> int time_it(astro_ctx *ctx, int reps, F fn, double *sec) {
    int rc;
    if ((rc = fn())) return rc;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaEventRecord(a, ctx->stream);
    for (int r = 0; r < reps && !rc; ++r) rc = fn();
    cudaEventRecord(b, ctx->stream);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    *sec = ms * 1e-3 / reps;
    return rc ? rc : cuda_check(ctx, cudaGetLastError(), "autotune");
}

}  // namespace

extern "C" int astro_autotune(astro_ctx *ctx, int32_t what, const char *cache_path, int32_t *choices) {
    if (!ctx || (what & ~(ASTRO_TUNE_BRICK_WARPS | ASTRO_TUNE_PANEL_CLUSTER | ASTRO_TUNE_CASES_CLUSTER)))
        return ASTRO_ERR_ARG;
    const AstroPrep &P = ctx->P;
    const std::string gpu = gpu_name(ctx);
    int rc;
    if (what & ASTRO_TUNE_BRICK_WARPS) {
        if (!ctx->hasSolid || ctx->has81 || ctx->hasShell)
            return set_err(ctx, ASTRO_ERR_UNSUPPORTED, "autotune: the zero-state brick kernel needs a brick8 mesh");
        const std::string key = gpu + "/brick_warps/E" + std::to_string(P.E) + "/colors" + std::to_string(P.ncolors);
        int best = 0;
        if (!cache_find(cache_path, key, &best)) {
            if ((rc = ensure_K(ctx, 1))) return rc;
            double bestS = 1e30;
            for (int fw : {1, 2, 4}) {
                ctx->tuneHex8Warps = fw;
                double sec = 0.0;
                if ((rc = time_it(ctx, 10, [&] { return launch_hex8_assemble(ctx, 32, 1); }, &sec))) return rc;
                if (sec < bestS) {
                    bestS = sec;
                    best = fw;
                }
            }
            cache_add(cache_path, key, best, bestS);
            ctx->haveK32 = 1;
            ctx->k32Version++;
        }
        ctx->tuneHex8Warps = best;
        // the captured assembly pass holds the old launch shape
        if (ctx->asmExec) cudaGraphExecDestroy(ctx->asmExec);
        if (ctx->asmGraph) cudaGraphDestroy(ctx->asmGraph);
        ctx->asmExec = nullptr;
        ctx->asmGraph = nullptr;
    }
    if (what & ASTRO_TUNE_PANEL_CLUSTER) {
        const std::string key = gpu + "/panel_cluster/N" + std::to_string(P.N) + "/nb" + std::to_string(P.nb);
        int best = 0;
        if (!cache_find(cache_path, key, &best)) {
            double bestS = 1e30;
            for (int cs : {2, 4, 8}) {
                astro_panels_info info{};
                if ((rc = astro_panels_factor(ctx, cs, &info))) return rc;
                if (info.factor_seconds < bestS) {
                    bestS = info.factor_seconds;
                    best = cs;
                }
            }
            cache_add(cache_path, key, best, bestS);
        }
        ctx->tunePanelCluster = best;
    }
    if (what & ASTRO_TUNE_CASES_CLUSTER) {
        int np = 0, bw = 0;
        long long bandBytes = 0;
        double fs = 0.0;
        panels_shape(ctx, &np, &bw, &bandBytes, &fs);
        const int cols = panels_cases_columns(ctx);
        if (!cols) return set_err(ctx, ASTRO_ERR_STATE, "autotune: no prepared many-column solve (astro_newmark_cases)");
        const std::string key = gpu + "/cases_cluster/n" + std::to_string(P.n) + "/bw" + std::to_string(bw) + "/cols" +
                                std::to_string(cols) + (panels_cases_launches(ctx) == 7 ? "/twisted" : "");
        int best = 0;
        if (!cache_find(cache_path, key, &best)) {
            DevBuf v;
            if ((rc = dev_alloc(ctx, v, sizeof(double) * (size_t)P.n * cols))) return rc;
            CK(cudaMemsetAsync(v.p, 0, sizeof(double) * (size_t)P.n * cols, ctx->stream));
            double bestS = 1e30;
            for (int cs : {2, 4, 8}) {
                ctx->tuneCasesCluster = cs;
                double sec = 0.0;
                // the solve's time does not depend on the values: zero right-hand sides
                rc = time_it(ctx, 3, [&] { return panels_cases_solve(ctx, dptr<double>(v), ctx->stream); }, &sec);
                if (rc) break;
                if (sec < bestS) {
                    bestS = sec;
                    best = cs;
                }
            }
            dev_free(v);
            if (rc) return rc;
            cache_add(cache_path, key, best, bestS);
        }
        ctx->tuneCasesCluster = best;
    }
    if (choices) {
        choices[0] = ctx->tuneHex8Warps;
        choices[1] = ctx->tunePanelCluster;
        choices[2] = ctx->tuneCasesCluster;
    }
    return ASTRO_OK;
}
