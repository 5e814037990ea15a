// Batched linear Newmark: many load cases of one model through one factorisation of K_eff.
//
// The reference's dynamic branch of solve (Working/AStrO_commandFunctions.f90:770-812) assembles
// K_eff = K + c1 c2 M at the initial state (getElasticSolnLoad(1) with the dynamic flag),
// scales the constraints, factors K_eff + C^T C once by getSparseLDLFact when nLGeom = 0, and
// then runs stepSolve and the Newmark update (:796-799) per step, one load history per job.
// Here the model's linear dynamics are stepped for num_cases load histories together:
//   setup     K (static, zero state) and K_eff (dynamic, zero state) assembled on the device,
//             both condensed over the internal DOF; scaleElasticMPC; the band LDL^T of
//             K_eff + C^T C (panels.cu: the tensor-core trailing updates) and its double-float
//             copies for the many-column solve;
//   step      r = amp_k(t) p_k + C^T rhs - K (u - w) - K_eff w - C^T C u with
//             w = -(dt v + (1 - 2 beta) a / c2), which is f - K u - M a_pred - C^T (C u - rhs)
//             with a_pred the acceleration at the start of the step (M = (K_eff - K) / (c1 c2));
//             du = (K_eff + C^T C)^-1 r for every case in one cluster launch
//             (k_band_solve_cases); u += du and the reference's acceleration / velocity update;
//   graph     the step's kernels are captured once into a CUDA graph, which is launched
//             num_steps times back to back: no host round trip per step (the step counter and
//             the load amplitudes live on the device).
// The element equations of the reference carry the Green-Lagrange strain and (shells) finite
// rotations at every state; this loop evaluates their linearisation at the zero state through the
// assembled matrices, which is what lets one factorisation serve every case and step.  For the
// brick8 element the two agree to the geometric nonlinearity of the displacement field; for the
// shell with the consistent tangent (ASTRO_OPT_SHELL_MEAN_ROT_TERM) likewise; with the
// reference's default shell tangent they differ (the default tangent is not the derivative of
// the residual).
#include <chrono>
#include <cmath>
#include <vector>

#include "astro_internal.h"
#include "dfloat.cuh"

namespace {

// residual of every case, thread per (block row, case); R in internal numbering, case-major
// r = amp p + C^T rhs - K (u - w) - K_eff w - C^T C u for every case: one warp per block row,
// lane = case (32 cases per pass), so the row's blocks of K and K_eff are read once for all
// cases (the lanes load the same entry: a broadcast) and only the vectors differ per lane; the
// products in double-float on the FP32 pipe from double-float copies of the matrices and of
// u - w and w.
template <int DPN>
__global__ void k_nmc_residual(int N, int nc, int steps, const int *__restrict__ bRowPtr, const int *__restrict__ bCol,
                               const float2 *__restrict__ KstF, const float2 *__restrict__ KeffF,
                               const int *__restrict__ penPtr, const int *__restrict__ penRow,
                               const int *__restrict__ penCol, const double *__restrict__ penVal,
                               const double *__restrict__ U, const float2 *__restrict__ UW,
                               const float2 *__restrict__ WW, const double *__restrict__ P,
                               const double *__restrict__ amp, const int *__restrict__ dStep,
                               const double *__restrict__ G, double *__restrict__ R) {
    const long long gw = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (gw >= N) return;
    const int r = (int)gw;
    const size_t n = (size_t)N * DPN;
    const int step = *dStep;
    const int b0 = bRowPtr[r], b1 = bRowPtr[r + 1];
    for (int c0 = 0; c0 < nc; c0 += 32) {
        const int c = c0 + lane;
        const bool on = c < nc;
        const size_t base = (size_t)(on ? c : 0) * n;
        const float2 *uwc = UW + base, *wc = WW + base;
        DF y[DPN];
#pragma unroll
        for (int i = 0; i < DPN; ++i) y[i] = DF{0.f, 0.f};
        for (int b = b0; b < b1; ++b) {
            const int col = bCol[b];
            float2 uw[DPN], wv[DPN];
#pragma unroll
            for (int j = 0; j < DPN; ++j) {
                uw[j] = uwc[(size_t)col * DPN + j];
                wv[j] = wc[(size_t)col * DPN + j];
            }
            const float2 *ks = KstF + (size_t)b * DPN * DPN, *ke = KeffF + (size_t)b * DPN * DPN;
#pragma unroll
            for (int i = 0; i < DPN; ++i) {
#pragma unroll
                for (int j = 0; j < DPN; ++j) {
                    const float2 kv = ks[i * DPN + j], ev = ke[i * DPN + j];
                    df_acc(y[i], kv.x, kv.y, uw[j].x, uw[j].y);
                    df_acc(y[i], ev.x, ev.y, wv[j].x, wv[j].y);
                }
                y[i] = df_norm(y[i]);
            }
        }
        if (!on) continue;
        const double a = amp[(size_t)c * steps + step];
        const double *Uc = U + base;
        double yp[DPN];
#pragma unroll
        for (int i = 0; i < DPN; ++i) yp[i] = df_to_double(y[i]);
        if (penPtr)
            for (int p = penPtr[r]; p < penPtr[r + 1]; ++p) {
                const double v = penVal[p] * Uc[penCol[p]];
                const int i = penRow[p];
#pragma unroll
                for (int k = 0; k < DPN; ++k) yp[k] += (k == i) ? v : 0.0;
            }
#pragma unroll
        for (int i = 0; i < DPN; ++i) {
            const size_t k = (size_t)r * DPN + i;
            R[base + k] = a * P[base + k] + G[k] - yp[i];
        }
    }
}

// double-float copies of a matrix's values
__global__ void k_nmc_df(long long cnt, const double *__restrict__ v, float2 *__restrict__ out) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= cnt) return;
    const DF d = df_from_double(v[t]);
    out[t] = make_float2(d.hi, d.lo);
}

// u - w and w (w = -(dt v + (1 - 2 beta) a / c2), the predictor's correction) in double-float for
// the next residual
__device__ __forceinline__ void nmc_uw(double u, double v, double a, double dt, double q, float2 *uw, float2 *ww) {
    const double w = -(dt * v + q * a);
    const DF dw = df_from_double(w), duw = df_from_double(u - w);
    *uw = make_float2(duw.hi, duw.lo);
    *ww = make_float2(dw.hi, dw.lo);
}

__global__ void k_nmc_uw(long long total, double dt, double q, const double *__restrict__ U,
                         const double *__restrict__ V, const double *__restrict__ A, float2 *__restrict__ UW,
                         float2 *__restrict__ WW) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t < total) nmc_uw(U[t], V[t], A[t], dt, q, UW + t, WW + t);
}

// u += du, then the reference's update (AStrO_commandFunctions.f90:796-799) with the previous
// values the current ones; the step's displacement into the history when there is one
__global__ void k_nmc_update(long long total, double c1, double c2, double dt, double beta, double gamma,
                             double *__restrict__ U, double *__restrict__ V, double *__restrict__ A,
                             const double *__restrict__ D, double *__restrict__ hist, const int *__restrict__ dStep,
                             float2 *__restrict__ UW, float2 *__restrict__ WW) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= total) return;
    const double du = D[t], vp = V[t], ap = A[t];
    const double u = U[t] + du;
    const double an = c1 * (c2 * (du - dt * vp) - (1.0 - 2.0 * beta) * ap);
    const double vn = vp + dt * ((1.0 - gamma) * ap + gamma * an);
    V[t] = vn;
    A[t] = an;
    U[t] = u;
    if (hist) hist[(size_t)(*dStep) * total + t] = u;
    nmc_uw(u, vn, an, dt, (1.0 - 2.0 * beta) / c2, UW + t, WW + t);
}

__global__ void k_nmc_tick(int *dStep) { *dStep += 1; }

__global__ void k_nmc_sub(long long total, double *__restrict__ D, const double *__restrict__ E) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t < total) D[t] -= E[t];
}

// y = (K_eff + C^T C) x - r for the last step's check, thread per (block row, case)
template <int DPN>
__global__ void k_nmc_check(int N, int nc, const int *__restrict__ bRowPtr, const int *__restrict__ bCol,
                            const double *__restrict__ Keff, const int *__restrict__ penPtr,
                            const int *__restrict__ penRow, const int *__restrict__ penCol,
                            const double *__restrict__ penVal, const double *__restrict__ X,
                            const double *__restrict__ R, double *__restrict__ E) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)N * nc) return;
    const int r = (int)(t % N), c = (int)(t / N);
    const size_t base = (size_t)c * N * DPN;
    double y[DPN];
#pragma unroll
    for (int i = 0; i < DPN; ++i) y[i] = 0.0;
    for (int b = bRowPtr[r]; b < bRowPtr[r + 1]; ++b) {
        const int col = bCol[b];
        const double *ke = Keff + (size_t)b * DPN * DPN;
#pragma unroll
        for (int i = 0; i < DPN; ++i)
#pragma unroll
            for (int j = 0; j < DPN; ++j) y[i] += ke[i * DPN + j] * X[base + (size_t)col * DPN + j];
    }
    if (penPtr)
        for (int p = penPtr[r]; p < penPtr[r + 1]; ++p) {
            const double v = penVal[p] * X[base + penCol[p]];
            const int i = penRow[p];
#pragma unroll
            for (int k = 0; k < DPN; ++k) y[k] += (k == i) ? v : 0.0;
        }
#pragma unroll
    for (int i = 0; i < DPN; ++i) {
        const size_t k = base + (size_t)r * DPN + i;
        E[k] = y[i] - R[k];
    }
}

struct NmcBufs {
    DevBuf U, V, A, P, amp, R, D, G, hist, Kst, zero, step, E, KstF, KeffF, UW, WW;
    ~NmcBufs() {
        DevBuf *b[] = {&U, &V, &A, &P, &amp, &R, &D, &G, &hist, &Kst, &zero, &step, &E, &KstF, &KeffF, &UW, &WW};
        for (auto *x : b) dev_free(*x);
    }
};

template <int DPN>
int enqueue_step(astro_ctx *ctx, NmcBufs &B, int nc, int steps, double dt, double beta, double gamma, int refine,
                 cudaStream_t s, int *launches) {
    const AstroPrep &P = ctx->P;
    const int N = P.N, n = P.n;
    const double c1 = 0.5 / beta, c2 = 2.0 / (dt * dt);
    const long long rows = (long long)N * nc, tot = (long long)n * nc;
    const int *penPtr = ctx->penRows ? dptr<int>(ctx->d_penPtr) : nullptr;
    k_nmc_residual<DPN><<<(unsigned)((N + 3) / 4), 128, 0, s>>>(
        N, nc, steps, dptr<int>(ctx->d_bRowPtr), dptr<int>(ctx->d_bCol), dptr<float2>(B.KstF), dptr<float2>(B.KeffF),
        penPtr, dptr<int>(ctx->d_penRow), dptr<int>(ctx->d_penCol), dptr<double>(ctx->d_penVal), dptr<double>(B.U),
        dptr<float2>(B.UW), dptr<float2>(B.WW), dptr<double>(B.P), dptr<double>(B.amp), dptr<int>(B.step),
        dptr<double>(B.G), dptr<double>(B.R));
    CK(cudaMemcpyAsync(B.D.p, B.R.p, sizeof(double) * (size_t)tot, cudaMemcpyDeviceToDevice, s));
    int rc = panels_cases_solve(ctx, dptr<double>(B.D), s);
    if (rc) return rc;
    // FP64 refinement: du -= A^-1 (A du - r), the residual in FP64 over the assembled values
    for (int q = 0; q < refine; ++q) {
        k_nmc_check<DPN><<<(unsigned)((rows + 127) / 128), 128, 0, s>>>(
            N, nc, dptr<int>(ctx->d_bRowPtr), dptr<int>(ctx->d_bCol), dptr<double>(ctx->d_K64), penPtr,
            dptr<int>(ctx->d_penRow), dptr<int>(ctx->d_penCol), dptr<double>(ctx->d_penVal), dptr<double>(B.D),
            dptr<double>(B.R), dptr<double>(B.E));
        if ((rc = panels_cases_solve(ctx, dptr<double>(B.E), s))) return rc;
        k_nmc_sub<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(tot, dptr<double>(B.D), dptr<double>(B.E));
    }
    k_nmc_update<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(tot, c1, c2, dt, beta, gamma, dptr<double>(B.U),
                                                               dptr<double>(B.V), dptr<double>(B.A), dptr<double>(B.D),
                                                               B.hist.p ? dptr<double>(B.hist) : nullptr,
                                                               dptr<int>(B.step), dptr<float2>(B.UW),
                                                               dptr<float2>(B.WW));
    k_nmc_tick<<<1, 1, 0, s>>>(dptr<int>(B.step));
    // residual, the solve's launches, update, tick; each refinement: check, the solve's, sub
    const int pl = panels_cases_launches(ctx);
    *launches = 3 + pl + (2 + pl) * refine;
    return cuda_check(ctx, cudaGetLastError(), "newmark cases step");
}

}  // namespace

extern "C" int astro_newmark_cases(astro_ctx *ctx, const astro_newmark_cases_opts *o, const double *patterns,
                                   const double *amplitudes, double *disp, double *vel, double *acc,
                                   double *disp_history, astro_newmark_cases_info *info) {
    if (!ctx || !o || !patterns || !amplitudes || !disp || !vel || !acc || o->num_steps < 0 || o->num_cases < 1 ||
        !(o->del_t > 0.0) || !(o->nm_beta > 0.0))
        return ASTRO_ERR_ARG;
    if (o->method != ASTRO_NMC_FACTORED) return set_err(ctx, ASTRO_ERR_ARG, "newmark cases: unknown method");
    if (o->refine < 0 || o->refine > 4) return set_err(ctx, ASTRO_ERR_ARG, "newmark cases: refine must be 0..4");
    const AstroPrep &P = ctx->P;
    const int n = P.n, nc = o->num_cases, steps = o->num_steps;
    const size_t cn = (size_t)n * nc;
    cudaStream_t s = ctx->stream;
    int rc;
    NmcBufs B;
    const auto t0 = std::chrono::steady_clock::now();
    if ((rc = ensure_io(ctx, false))) return rc;
    double *dRef = dptr<double>(ctx->d_ioRef);
    if ((rc = dev_alloc(ctx, B.U, sizeof(double) * cn)) || (rc = dev_alloc(ctx, B.V, sizeof(double) * cn)) ||
        (rc = dev_alloc(ctx, B.A, sizeof(double) * cn)) || (rc = dev_alloc(ctx, B.P, sizeof(double) * cn)) ||
        (rc = dev_alloc(ctx, B.R, sizeof(double) * cn)) || (rc = dev_alloc(ctx, B.D, sizeof(double) * cn)) ||
        (rc = dev_alloc(ctx, B.G, sizeof(double) * n)) || (rc = dev_alloc(ctx, B.zero, sizeof(double) * n)) ||
        (rc = dev_alloc(ctx, B.step, sizeof(int))) ||
        (rc = dev_alloc(ctx, B.amp, sizeof(double) * (size_t)nc * std::max(steps, 1))))
        return rc;
    if (disp_history && steps > 0 && (rc = dev_alloc(ctx, B.hist, sizeof(double) * cn * steps))) return rc;
    if ((rc = dev_alloc(ctx, B.E, sizeof(double) * cn))) return rc;
    // per-case vectors, global DOF numbering on the host -> internal numbering
    const double *src[4] = {disp, vel, acc, patterns};
    DevBuf *dst[4] = {&B.U, &B.V, &B.A, &B.P};
    for (int q = 0; q < 4; ++q)
        for (int c = 0; c < nc; ++c) {
            CK(cudaMemcpyAsync(dRef, src[q] + (size_t)c * n, sizeof(double) * n, cudaMemcpyHostToDevice, s));
            if ((rc = ref_to_int_vec(ctx, dRef, dptr<double>(*dst[q]) + (size_t)c * n, n))) return rc;
            CK(cudaStreamSynchronize(s));
        }
    CK(cudaMemcpyAsync(B.amp.p, amplitudes, sizeof(double) * (size_t)nc * steps, cudaMemcpyHostToDevice, s));
    CK(cudaMemsetAsync(B.zero.p, 0, sizeof(double) * n, s));
    CK(cudaMemsetAsync(B.G.p, 0, sizeof(double) * n, s));
    CK(cudaMemsetAsync(B.step.p, 0, sizeof(int), s));
    // K at the static zero state, then K_eff at the dynamic zero state (left in d_K64)
    ElemDevState ds;
    ds.disp = ds.pdisp = ds.pvel = ds.pacc = dptr<double>(B.zero);
    ds.dynamic = 0;
    ds.beta = o->nm_beta;
    ds.gamma = o->nm_gamma;
    ds.delT = o->del_t;
    DevBuf izero;
    if (P.intVecSize) {
        if ((rc = dev_alloc(ctx, izero, sizeof(double) * P.intVecSize))) return rc;
        CK(cudaMemsetAsync(izero.p, 0, sizeof(double) * P.intVecSize, s));
        ds.idisp = ds.pidisp = dptr<double>(izero);
    }
    const size_t kBytes = sizeof(double) * (size_t)P.nb * P.dpn * P.dpn;
    if ((rc = ensure_K(ctx, 2))) return rc;
    if ((rc = elem_soln_load_dev(ctx, ds, nullptr, nullptr, 1, true))) return rc;
    if ((rc = dev_alloc(ctx, B.Kst, kBytes))) return rc;
    CK(cudaMemcpyAsync(B.Kst.p, ctx->d_K64.p, kBytes, cudaMemcpyDeviceToDevice, s));
    ds.dynamic = 1;
    if ((rc = elem_soln_load_dev(ctx, ds, nullptr, nullptr, 1, true))) return rc;
    dev_free(izero);
    // double-float copies of K and K_eff, and u - w and w of the initial state, for the residual
    {
        const long long kv = (long long)P.nb * P.dpn * P.dpn, tot = (long long)cn;
        if ((rc = dev_alloc(ctx, B.KstF, sizeof(float2) * (size_t)kv)) ||
            (rc = dev_alloc(ctx, B.KeffF, sizeof(float2) * (size_t)kv)) ||
            (rc = dev_alloc(ctx, B.UW, sizeof(float2) * cn)) || (rc = dev_alloc(ctx, B.WW, sizeof(float2) * cn)))
            return rc;
        k_nmc_df<<<(unsigned)((kv + 255) / 256), 256, 0, s>>>(kv, dptr<double>(B.Kst), dptr<float2>(B.KstF));
        k_nmc_df<<<(unsigned)((kv + 255) / 256), 256, 0, s>>>(kv, dptr<double>(ctx->d_K64), dptr<float2>(B.KeffF));
        const double c2 = 2.0 / (o->del_t * o->del_t);
        k_nmc_uw<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(tot, o->del_t, (1.0 - 2.0 * o->nm_beta) / c2,
                                                               dptr<double>(B.U), dptr<double>(B.V), dptr<double>(B.A),
                                                               dptr<float2>(B.UW), dptr<float2>(B.WW));
        if ((rc = cuda_check(ctx, cudaGetLastError(), "newmark cases double-float copies"))) return rc;
    }
    ctx->haveK64 = 1;
    ctx->k64Version++;
    ctx->haveIntMat = P.intVecSize > 0;
    ctx->haveLT = 0;
    ctx->ltFactored = 0;
    if ((rc = astro_scale_mpc(ctx, nullptr, nullptr))) return rc;
    if ((rc = constraint_load_dev(ctx, nullptr, dptr<double>(B.G)))) return rc;  // C^T rhs
    // the plan (the autotuned cluster size, else 8); the whole band's factorisation unless the
    // many-column solve runs twisted, which factors its own halves
    astro_panels_info pinfo{};
    if ((rc = panels_factor_impl(ctx, 0, &pinfo, 0))) return rc;
    if (!panels_cases_would_twist(ctx) && (rc = astro_panels_factor(ctx, 0, &pinfo))) return rc;
    size_t dfBytes = 0;
    if ((rc = panels_cases_prepare(ctx, nc, &dfBytes))) return rc;
    if (o->autotune && !ctx->tuneCasesCluster && (rc = astro_autotune(ctx, ASTRO_TUNE_CASES_CLUSTER, nullptr, nullptr)))
        return rc;
    CK(cudaStreamSynchronize(s));
    const double prepSeconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    // the step as a graph, launched num_steps times
    int launches = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    const bool useGraph = o->no_graph == 0;
    auto enqueue = [&](cudaStream_t st) {
        return P.dpn == 3 ? enqueue_step<3>(ctx, B, nc, steps, o->del_t, o->nm_beta, o->nm_gamma, o->refine, st, &launches)
                          : enqueue_step<6>(ctx, B, nc, steps, o->del_t, o->nm_beta, o->nm_gamma, o->refine, st, &launches);
    };
    size_t graphNodes = 0;
    if (useGraph && steps > 0) {
        CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        rc = enqueue(s);
        cudaError_t e = cudaStreamEndCapture(s, &graph);
        if (rc) {
            if (graph) cudaGraphDestroy(graph);
            return rc;
        }
        CK(e);
        CK(cudaGraphInstantiate(&exec, graph, 0));
        cudaGraphGetNodes(graph, nullptr, &graphNodes);
        CK(cudaGraphUpload(exec, s));
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, s);
    for (int k = 0; k < steps && !rc; ++k) {
        if (exec) {
            cudaError_t e = cudaGraphLaunch(exec, s);
            if (e != cudaSuccess) rc = cuda_check(ctx, e, "newmark cases graph launch");
        } else {
            rc = enqueue(s);
        }
    }
    cudaEventRecord(e1, s);
    cudaError_t es = cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (rc) return rc;
    if ((rc = cuda_check(ctx, es, "newmark cases steps"))) return rc;
    // the last step's solve against its residual: max over cases of ||A du - r|| / ||r||
    double worst = 0.0;
    if (steps > 0) {
        const long long rows = (long long)P.N * nc;
        const int *penPtr = ctx->penRows ? dptr<int>(ctx->d_penPtr) : nullptr;
        if (P.dpn == 3)
            k_nmc_check<3><<<(unsigned)((rows + 127) / 128), 128, 0, s>>>(
                P.N, nc, dptr<int>(ctx->d_bRowPtr), dptr<int>(ctx->d_bCol), dptr<double>(ctx->d_K64), penPtr,
                dptr<int>(ctx->d_penRow), dptr<int>(ctx->d_penCol), dptr<double>(ctx->d_penVal), dptr<double>(B.D),
                dptr<double>(B.R), dptr<double>(B.E));
        else
            k_nmc_check<6><<<(unsigned)((rows + 127) / 128), 128, 0, s>>>(
                P.N, nc, dptr<int>(ctx->d_bRowPtr), dptr<int>(ctx->d_bCol), dptr<double>(ctx->d_K64), penPtr,
                dptr<int>(ctx->d_penRow), dptr<int>(ctx->d_penCol), dptr<double>(ctx->d_penVal), dptr<double>(B.D),
                dptr<double>(B.R), dptr<double>(B.E));
        std::vector<double> he(cn), hr(cn);
        CK(cudaMemcpyAsync(he.data(), B.E.p, sizeof(double) * cn, cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(hr.data(), B.R.p, sizeof(double) * cn, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        for (int c = 0; c < nc; ++c) {
            double en = 0.0, rn = 0.0;
            for (int i = 0; i < n; ++i) {
                en += he[(size_t)c * n + i] * he[(size_t)c * n + i];
                rn += hr[(size_t)c * n + i] * hr[(size_t)c * n + i];
            }
            if (rn > 0.0) worst = std::max(worst, std::sqrt(en / rn));
        }
    }
    // final states and the history back to global numbering
    double *hostDst[3] = {disp, vel, acc};
    DevBuf *devSrc[3] = {&B.U, &B.V, &B.A};
    for (int q = 0; q < 3; ++q)
        for (int c = 0; c < nc; ++c) {
            if ((rc = int_to_ref_vec(ctx, dptr<double>(*devSrc[q]) + (size_t)c * n, dRef, n))) return rc;
            CK(cudaMemcpyAsync(hostDst[q] + (size_t)c * n, dRef, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
            CK(cudaStreamSynchronize(s));
        }
    if (B.hist.p)
        for (size_t v = 0; v < (size_t)steps * nc; ++v) {
            if ((rc = int_to_ref_vec(ctx, dptr<double>(B.hist) + v * n, dRef, n))) return rc;
            CK(cudaMemcpyAsync(disp_history + v * n, dRef, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
            CK(cudaStreamSynchronize(s));
        }
    if (info) {
        int np = 0, bw = 0;
        long long bandBytes = 0;
        double fs = 0.0;
        panels_shape(ctx, &np, &bw, &bandBytes, &fs);
        info->factor_seconds = fs;
        info->prepare_seconds = prepSeconds;
        info->step_seconds = ms * 1e-3;
        info->last_rel_residual = worst;
        info->band_bytes = bandBytes;
        info->df_band_bytes = (int64_t)dfBytes;
        info->bandwidth = bw;
        info->panels = np;
        info->graph_nodes = (int32_t)graphNodes;
        info->kernels_per_step = launches;
        info->cluster_size = ctx->tuneCasesCluster ? ctx->tuneCasesCluster : 4;
    }
    return ASTRO_OK;
}
