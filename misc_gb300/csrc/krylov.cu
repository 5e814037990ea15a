// Restarted GMRES(m) on A = K + C^T C for the spec solvers.
//
//   * K is kept for the solvers as a slot-major block-ELL copy of the assembled block-CSR matrix:
//     the s-th block of every block row is contiguous across rows, so the SpMV runs one thread
//     per block row with every value load coalesced across the warp and no cross-lane reduction.
//     GB300 issues FP64 at 1/64 of its FP32 rate, so the products are accumulated in the
//     precision of the matrix (FP32 for the inner solver, FP64 for the comparator) and no FP64
//     warp reductions remain.  C^T C (the scaled penalty of scaleElasticMPC) stays in FP64 as a
//     per-block-row list and is added by the same thread;
//   * preconditioner: Jacobi on the right (A D^-1 y = b, x = D^-1 y), so the Arnoldi residual
//     estimate is the residual of the unpreconditioned system;
//   * orthogonalisation: classical Gram-Schmidt with one re-orthogonalisation (CGS2).  The Krylov
//     basis is stored vector-major (V[k*ld + i]); the dot products stage a chunk of w in shared
//     memory and let each warp stream whole basis vectors over that chunk, the updates run one
//     thread per row; both work in the precision of the basis.  Dot products are reduced
//     deterministically (per-CTA partials in FP64, then one reduction CTA).  Givens rotations
//     and the stopping test run on the device; one Arnoldi step is 7 launches and a restart
//     cycle is captured once as a CUDA graph and replayed, the host reading one status word per
//     cycle;
//   * precision: the plain solver runs in FP64 throughout (the comparator).  The mixed solver
//     runs the Krylov cycles in FP32 (FP32 matrix and basis) inside an FP64 iterative refinement
//     whose residual b - A x is formed in FP64 arithmetic.
#include <cuda_fp16.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "astro_internal.h"
#include "krylov_ops.cuh"

using namespace astro_kry;

namespace {

// Device-side control of a restart cycle captured as a chain of conditional IF nodes, each holding
// two Arnoldi steps: the kernel that finishes a step (and the cycle start) sets the next node's
// condition to "not done", and a node whose condition is zero skips its steps without launching
// them.  The chain has a fixed length, so the number of steps is bounded whatever the conditions.
struct LoopCond {
    cudaGraphConditionalHandle h;
    int use;
};
__device__ __forceinline__ void loop_cond_set(const LoopCond &lc, unsigned v) {
    if (lc.use) cudaGraphSetConditional(lc.h, v);
}

// Partial dot products of the staged tile sw (cnt vector rows from row0, at most ROWS) with
// V[0..j], and with itself when self is set (stored as vector kMaxM): part[k * nCh + cta].
// Warp-per-vector, ROWS/32 rows per lane, eight loads in flight; full tiles take the unguarded
// multiply-add path.  Lane 0 of each warp makes its partials visible device-wide.
template <class TV, int ROWS>
__device__ __forceinline__ void chunk_dots(const TV *__restrict__ V, size_t ld, const TV *sw, int row0, int cnt, int j,
                                           double *part, int nCh, bool self) {
    static_assert(ROWS % 256 == 0, "tile rows: a multiple of 32 lanes x 8 loads");
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int nv = j + 1 + (self ? 1 : 0);
    for (int kk = wid; kk < nv; kk += kGsWarps) {
        const bool isSelf = kk > j;
        const TV *__restrict__ vk = isSelf ? sw : V + (size_t)kk * ld + row0;
        TV s = TV(0);
        if (cnt == ROWS) {
#pragma unroll
            for (int u0 = 0; u0 < ROWS / 32; u0 += 8) {
                TV v[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) v[u] = vk[lane + 32 * (u0 + u)];
#pragma unroll
                for (int u = 0; u < 8; ++u) s = fma(v[u], sw[lane + 32 * (u0 + u)], s);
            }
        } else {
            for (int t = lane; t < cnt; t += 32) s = fma(vk[t], sw[t], s);
        }
        s = warp_sum(s);
        if (lane == 0) {
            part[(size_t)(isSelf ? kMaxM : kk) * nCh + blockIdx.x] = (double)s;
            __threadfence();
        }
    }
}

// h[k] = sum of the nCh CTA partials of vector k in a fixed order (one warp per vector, reads
// bypassing L1); recorded in h1 and in the Hessenberg column (mode 0) or added to it (mode 1).
// In mode 0 the partials also carry ||w||^2 (vector kMaxM), and the second pass is requested when
// the first removed more than half of it: ||w - V h||^2 = ||w||^2 - ||h||^2 < ||w||^2 / 2
// (the "twice is enough" test of Kahan and Parlett).
__device__ __forceinline__ void reduce_h(GmresCtl *ctl, const double *part, int nCh, int j, int mode) {
    __shared__ double shh[kGsWarps], sww;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    double *Hc = ctl->H + (size_t)j * (kMaxM + 1);
    double hh = 0.0;
    const int nv = j + 1 + (mode == 0 ? 1 : 0);
    for (int kk = wid; kk < nv; kk += kGsWarps) {
        const int k = kk > j ? kMaxM : kk;
        double s = 0.0;
        for (int q0 = lane; q0 < nCh; q0 += 256) {
            double v[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int q = q0 + 32 * u;
                v[u] = (q < nCh) ? __ldcg(part + (size_t)k * nCh + q) : 0.0;
            }
#pragma unroll
            for (int u = 0; u < 8; ++u) s += v[u];
        }
        s = warp_sum(s);
        if (lane == 0) {
            if (kk > j) {
                sww = s;
            } else {
                ctl->h1[k] = s;
                Hc[k] = (mode == 0) ? s : Hc[k] + s;
                hh += s * s;
            }
        }
    }
    if (mode != 0) return;
    if (lane == 0) shh[wid] = hh;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int q = 0; q < kGsWarps; ++q) t += shh[q];
        ctl->reorth = (sww - t < 0.5 * sww) ? 1 : 0;
        ctl->reorths += ctl->reorth;
    }
}

// Norm of w from the CTA partials, Hessenberg subdiagonal, Givens rotation, residual estimate
// and stopping test (thread 0 of the last CTA).
__device__ void step_control(GmresCtl *ctl, const double *part, int nCh, int m) {
    const int lane = threadIdx.x & 31;
    if (threadIdx.x >= 32) return;
    double s = 0.0;
    for (int q = lane; q < nCh; q += 32) s += __ldcg(part + q);
    s = warp_sum(s);
    if (lane != 0) return;
    const int j = ctl->j;
    const double nrm = sqrt(s);
    double *Hc = ctl->H + (size_t)j * (kMaxM + 1);
    Hc[j + 1] = nrm;
    for (int k = 0; k < j; ++k) {
        const double a = Hc[k], b = Hc[k + 1];
        Hc[k] = ctl->cs[k] * a + ctl->sn[k] * b;
        Hc[k + 1] = -ctl->sn[k] * a + ctl->cs[k] * b;
    }
    const double a = Hc[j], b = Hc[j + 1];
    const double rr = hypot(a, b);
    double c = 1.0, sn = 0.0;
    if (rr > 0.0) {
        c = a / rr;
        sn = b / rr;
    }
    ctl->cs[j] = c;
    ctl->sn[j] = sn;
    Hc[j] = rr;
    Hc[j + 1] = 0.0;
    const double gj = ctl->g[j];
    ctl->g[j] = c * gj;
    ctl->g[j + 1] = -sn * gj;
    ctl->resest = fabs(ctl->g[j + 1]);
    ctl->j = j + 1;
    if (!isfinite(nrm) || !isfinite(rr)) {
        ctl->nonfinite = 1;
        ctl->done = 1;
        return;
    }
    if (!(nrm > 1e-300)) {
        ctl->breakdown = 1;
        ctl->done = 1;
        ctl->inv = 0.0;
        return;
    }
    ctl->inv = 1.0 / nrm;
    if (ctl->resest <= ctl->target || ctl->j >= m) ctl->done = 1;
}

// v_j = wprev * inv (written to V[j]); w = A D^-1 v_j = inv * A zprev with zprev = D^-1 wprev.
// Warp-per-slot-group mapping (kRowThreads warps per 32 block rows, partials met in shared
// memory); the products accumulate in the precision of the basis.
template <class TM, class TV, int DPN>
__global__ void __launch_bounds__(kThreads) k_spmv_step(Op<TM> op, TV *__restrict__ V, size_t ld, const TV *__restrict__ wprev,
                                                        const TV *__restrict__ zprev, TV *__restrict__ w,
                                                        const GmresCtl *__restrict__ ctl) {
    if (ctl->done) return;
    const CtaRow c = cta_row(op.N);  // (the FP64 branch keeps the CTA's 64 rows, lane-grouped)
    const int j = ctl->j;
    const TV inv = (TV)ctl->inv;
    TV y[DPN] = {};
    if constexpr (sizeof(TM) == 8) {
        // FP64 comparator: kRowThreads adjacent lanes per block row, partials combined by shuffles
        // (the FP64 products bound this kernel, not its loads); same grid, rows renumbered
        const int r = blockIdx.x * kCtaRows + (int)threadIdx.x / kRowThreads, sub = threadIdx.x % kRowThreads;
        const int rr = r < op.N ? r : op.N - 1;
        ell_row_part<TV, TM, TV, DPN>(op, rr, sub, zprev, y);
        if (r >= op.N) return;
#pragma unroll
        for (int q = 0; q < DPN; ++q) {
            if (q % kRowThreads != sub) continue;
            const size_t i = (size_t)r * DPN + q;
            V[(size_t)j * ld + i] = wprev[i] * inv;
            w[i] = y[q] * inv;
        }
    } else {
        if (c.valid) ell_row_group<TV, TM, TV, DPN>(op, c.r, c.sub, zprev, y);
        if (!ell_cta_reduce<TV, DPN>(y, c) || !c.valid) return;
#pragma unroll
        for (int q = 0; q < DPN; ++q) {
            const size_t i = (size_t)c.r * DPN + q;
            V[(size_t)j * ld + i] = wprev[i] * inv;
            w[i] = y[q] * inv;
        }
    }
}

// One hop of the polynomial preconditioner P v = sum_k W_k T_k(xi(D^-1 A)) D^-1 v / lambda,
// evaluated in the symmetrically scaled space: with S = D^-1/2 and A^ = S A S (unit diagonal,
// entries in [-1, 1], kept in FP16), T_k(xi(D^-1 A)) D^-1 = S T_k(xi(A^)) S, so the hops run on
// y^_k = T_k(xi(A^)) S v and the node outputs are W_k (S y^_k).  With u = A^ y^_k,
// y^_{k+1} = c (u - theta y^_k) - [k > 0] y^_{k-1} (the Chebyshev three-term recurrence in the
// shifted and scaled variable) and z += W_{k+1} S y^_{k+1} per node (the first hop also adds
// W_0 S y^_0).  Same row mapping as the SpMV step; the slot-group-0 thread of a row then has the
// whole node's A^ y^_k and finishes the row.  The weights arrive already divided by lambda.
struct HopArgs {
    float w[36];   // W_{k+1} / lambda, row-major dpn x dpn
    float w0[36];  // W_0 / lambda (first hop)
    float theta, c;
    int first;
    const float *amod;  // per-node hop scales a_k(r) at amod[k * N + r] (null: all 1)
    int k1;             // k + 1, the hop whose output this launch adds
};

template <class OP, class TV, int DPN>
__global__ void __launch_bounds__(kThreads) k_poly_hop(OP op, const TV *__restrict__ dsq, const TV *__restrict__ yk,
                                                       const TV *__restrict__ ykm1, TV *__restrict__ ykp1,
                                                       TV *__restrict__ zacc, const HopArgs h,
                                                       const GmresCtl *__restrict__ ctl, int always) {
    if (!always && ctl->done) return;
    const CtaRow c = cta_row(op.N);
    TV t[DPN] = {};
    if (c.valid) row_group<TV, DPN>(op, c.r, c.sub, yk, t);
    if (!ell_cta_reduce<TV, DPN>(t, c) || !c.valid) return;
    const size_t base = (size_t)c.r * DPN;
    TV yc[DPN], yn[DPN], sc[DPN];
#pragma unroll
    for (int q = 0; q < DPN; ++q) {
        yc[q] = yk[base + q];
        sc[q] = dsq[base + q];
    }
#pragma unroll
    for (int q = 0; q < DPN; ++q) {
        yn[q] = (TV)h.c * (t[q] - (TV)h.theta * yc[q]);
        if (!h.first) yn[q] -= ykm1[base + q];
    }
    // the modulation network's scales of this hop (and of hop 0 on the first) at this node
    const TV a1 = h.amod ? (TV)h.amod[(size_t)h.k1 * op.N + c.r] : TV(1);
    const TV a0 = (h.amod && h.first) ? (TV)h.amod[c.r] : TV(1);
#pragma unroll
    for (int q = 0; q < DPN; ++q) {
        if (ykp1) ykp1[base + q] = yn[q];
        TV z = h.first ? TV(0) : zacc[base + q];
        if (h.first) {
            TV z0 = TV(0);
#pragma unroll
            for (int jj = 0; jj < DPN; ++jj) z0 += (TV)h.w0[q * DPN + jj] * (sc[jj] * yc[jj]);
            z += a0 * z0;
        }
        TV z1 = TV(0);
#pragma unroll
        for (int jj = 0; jj < DPN; ++jj) z1 += (TV)h.w[q * DPN + jj] * (sc[jj] * yn[jj]);
        zacc[base + q] = z + a1 * z1;
    }
}

// A^ = S A S in the FP16 block-vector layout of OpH (same slots and columns as the solver copy),
// S = diag(dsq): one thread per (row, slot); padding rows and slots get zero blocks.
template <int DPN>
__global__ void k_scaled_bv(const float *__restrict__ K, const int *__restrict__ col, int S, int ld, int N,
                            const float *__restrict__ dsq, uint4 *__restrict__ Kv, void *__restrict__ KrRaw) {
    using Sh = BvShape<DPN>;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)S * ld) return;
    const int s = (int)(t / ld), r = (int)(t - (long long)s * ld);
    unsigned short h[Sh::NV * 8 + 4] = {};
    if (r < N) {
        const int c = col[(size_t)s * ld + r];
#pragma unroll
        for (int i = 0; i < DPN; ++i)
#pragma unroll
            for (int j = 0; j < DPN; ++j) {
                const float v = K[((size_t)s * Sh::DD + i * DPN + j) * ld + r] * dsq[(size_t)r * DPN + i] *
                                dsq[(size_t)c * DPN + j];
                h[i * DPN + j] = __half_as_ushort(__float2half_rn(v));
            }
    }
#pragma unroll
    for (int p = 0; p < Sh::NV; ++p) {
        uint4 u;
        u.x = h[8 * p] | ((unsigned)h[8 * p + 1] << 16);
        u.y = h[8 * p + 2] | ((unsigned)h[8 * p + 3] << 16);
        u.z = h[8 * p + 4] | ((unsigned)h[8 * p + 5] << 16);
        u.w = h[8 * p + 6] | ((unsigned)h[8 * p + 7] << 16);
        Kv[((size_t)s * Sh::NV + p) * ld + r] = u;
    }
    const int b = 8 * Sh::NV;
    if constexpr (Sh::REM == 1) {
        static_cast<unsigned short *>(KrRaw)[(size_t)s * ld + r] = h[b];
    } else {
        uint2 u;
        u.x = h[b] | ((unsigned)h[b + 1] << 16);
        u.y = h[b + 2] | ((unsigned)h[b + 3] << 16);
        static_cast<uint2 *>(KrRaw)[(size_t)s * ld + r] = u;
    }
}

__global__ void k_scaled_pen(const int *__restrict__ penPtr, const int *__restrict__ penRow,
                             const int *__restrict__ penCol, const double *__restrict__ penVal, int N, int dpn,
                             const double *__restrict__ dinv, double *__restrict__ out) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= N) return;
    for (int t = penPtr[r]; t < penPtr[r + 1]; ++t)
        out[t] = penVal[t] * sqrt(dinv[(size_t)r * dpn + penRow[t]] * dinv[penCol[t]]);
}

__global__ void k_sqrt_f(const double *__restrict__ dinv, float *__restrict__ dsq, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dsq[i] = (float)sqrt(dinv[i]);
}

// Power iteration for the largest eigenvalue of D^-1 A: y = s D^-1 A x with s = scal[0] (the
// reciprocal norm of x from the previous step), SpMV-step row mapping; warp 0 of the last CTA
// sums the per-CTA ||y||^2 in a fixed order and sets scal[1] = ||y||, scal[0] = 1 / ||y||.  Every CTA reads
// scal[0] before it arrives, so the last one may overwrite it.  dinv null: the operator is
// already scaled (A^ = D^-1/2 A D^-1/2, the same spectrum as D^-1 A).
template <class OP, class TV, int DPN>
__global__ void __launch_bounds__(kThreads) k_power_step(OP op, const TV *__restrict__ dinv, const TV *__restrict__ x,
                                                         TV *__restrict__ y, double *part, unsigned *counter,
                                                         double *scal) {
    __shared__ double sp[kWarps];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const CtaRow c = cta_row(op.N);
    const TV s = (TV)scal[0];
    double yy = 0.0;
    TV t[DPN] = {};
    if (c.valid) row_group<TV, DPN>(op, c.r, c.sub, x, t);
    if (ell_cta_reduce<TV, DPN>(t, c) && c.valid) {
#pragma unroll
        for (int q = 0; q < DPN; ++q) {
            const size_t i = (size_t)c.r * DPN + q;
            const TV v = s * (dinv ? dinv[i] : TV(1)) * t[q];
            y[i] = v;
            yy += (double)v * (double)v;
        }
    }
    yy = warp_sum(yy);
    if (lane == 0) sp[wid] = yy;
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0;
        for (int q = 0; q < kWarps; ++q) a += sp[q];
        part[blockIdx.x] = a;
        __threadfence();
    }
    if (last_to_arrive(counter) && threadIdx.x < 32) {
        // warp 0 sums the CTA partials (lane-strided, then a fixed shuffle tree)
        double a = 0.0;
        for (unsigned q = threadIdx.x; q < gridDim.x; q += 32) a += __ldcg(part + q);
        a = warp_sum(a);
        if (threadIdx.x == 0) {
            const double nrm = sqrt(a);
            scal[1] = nrm;
            scal[0] = nrm > 0.0 ? 1.0 / nrm : 0.0;
        }
    }
}

// Start vector of the power iteration: a fixed pseudo-random pattern in [-1, 1) (an integer hash
// of the index), so that every eigenvector has a component and the estimate is reproducible.
template <class TV>
__global__ void k_power_init(TV *x, int n, double *scal) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) {
        scal[0] = 1.0;
        scal[1] = 0.0;
    }
    if (i >= n) return;
    unsigned h = (unsigned)i * 2654435761u + 0x9e3779b9u;
    h ^= h >> 16;
    h *= 0x85ebca6bu;
    h ^= h >> 13;
    h *= 0xc2b2ae35u;
    h ^= h >> 16;
    x[i] = (TV)((double)(h >> 8) * (2.0 / 16777216.0) - 1.0);
}

template <class TV>
__global__ void k_add(int n, TV *__restrict__ x, const TV *__restrict__ d) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] += d[i];
}

// First Gram-Schmidt pass: partial dots of w with V[0..j] and with itself over this CTA's rows;
// the last CTA reduces them into h1 and decides whether a second pass is needed.
template <class TV>
__global__ void __launch_bounds__(kGsThreads, 2) k_dots(int n, const TV *__restrict__ V, size_t ld, const TV *__restrict__ w,
                                                        GmresCtl *__restrict__ ctl, double *part, int nCh) {
    if (ctl->done) return;
    __shared__ TV sw[kChunk];
    const int row0 = blockIdx.x * kChunk;
    const int cnt = min(kChunk, n - row0);
    const int j = ctl->j;
    for (int t = threadIdx.x; t < cnt; t += kGsThreads) sw[t] = w[row0 + t];
    __syncthreads();
    chunk_dots<TV, kChunk>(V, ld, sw, row0, cnt, j, part, nCh, true);
    if (last_to_arrive(&ctl->arrive[0])) reduce_h(ctl, part, nCh, j, 0);
}

// One Gram-Schmidt update on this CTA's rows: w -= V[0..j] h1.  The first update (pass 0) is
// followed by the second pass's partial dots when the first pass asked for it (its last CTA then
// adds the correction to the Hessenberg column); otherwise, and after the second update
// (pass 1), the step finishes here: the partial ||w||^2, the Jacobi-scaled copy z = D^-1 w read
// by the next SpMV, and the step control in the last CTA.  The second update returns at once
// when no second pass was requested.
template <class TV>
__global__ void __launch_bounds__(kGsThreads, 2) k_update(int n, const TV *__restrict__ V, size_t ld, TV *__restrict__ w,
                                                          GmresCtl *__restrict__ ctl, double *__restrict__ partDots,
                                                          double *__restrict__ partNorm, int nCh, int pass,
                                                          const TV *__restrict__ dinv, TV *__restrict__ z, int m,
                                                          LoopCond lc) {
    constexpr int ROWS = kChunk;
    if (ctl->done) return;
    const bool second = ctl->reorth != 0;
    if (pass == 1 && !second) return;
    const bool finish = (pass == 1) || !second;
    __shared__ TV sw[ROWS];
    __shared__ TV sh[kMaxM + 1];
    __shared__ double sred[kGsWarps];
    const int j = ctl->j;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int k = threadIdx.x; k <= j; k += kGsThreads) sh[k] = (TV)ctl->h1[k];
    __syncthreads();
    const int row0 = blockIdx.x * ROWS;
    const int cnt = min(ROWS, n - row0);
    TV nrm = TV(0);
    for (int t = threadIdx.x; t < cnt; t += kGsThreads) {
        const int i = row0 + t;
        TV s = w[i];
        int k = 0;
        for (; k + 8 <= j + 1; k += 8) {
            TV v[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) v[u] = V[(size_t)(k + u) * ld + i];
#pragma unroll
            for (int u = 0; u < 8; ++u) s -= sh[k + u] * v[u];
        }
        for (; k <= j; ++k) s -= sh[k] * V[(size_t)k * ld + i];
        w[i] = s;
        if (!finish) {
            sw[t] = s;
        } else {
            z[i] = dinv[i] * s;
            nrm += s * s;
        }
    }
    if (!finish) {
        __syncthreads();
        chunk_dots<TV, ROWS>(V, ld, sw, row0, cnt, j, partDots, nCh, false);
        if (last_to_arrive(&ctl->arrive[1])) reduce_h(ctl, partDots, nCh, j, 1);
    } else {
        nrm = warp_sum(nrm);
        if (lane == 0) sred[wid] = (double)nrm;
        __syncthreads();
        if (threadIdx.x == 0) {
            double s = 0.0;
            for (int q = 0; q < kGsWarps; ++q) s += sred[q];
            partNorm[blockIdx.x] = s;
            __threadfence();
        }
        if (last_to_arrive(&ctl->arrive[2])) {
            step_control(ctl, partNorm, nCh, m);
            if (threadIdx.x == 0) loop_cond_set(lc, ctl->done ? 0u : 1u);
        }
    }
}

// sum of part[q*stride + off] over q = lane, lane+32, ... < nparts, eight loads in flight
__device__ __forceinline__ double lane_sum(const double *part, int nparts, size_t stride, int off, int lane) {
    double s = 0.0;
    for (int q0 = lane; q0 < nparts; q0 += 256) {
        double v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int q = q0 + 32 * u;
            v[u] = (q < nparts) ? part[(size_t)q * stride + off] : 0.0;
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) s += v[u];
    }
    return s;
}

// Least squares H y = g (upper triangular j x j), one thread.
__global__ void k_lsq(GmresCtl *ctl) {
    const int j = ctl->j;
    for (int i = j - 1; i >= 0; --i) {
        double s = ctl->g[i];
        for (int k = i + 1; k < j; ++k) s -= ctl->H[(size_t)k * (kMaxM + 1) + i] * ctl->y[k];
        ctl->y[i] = s / ctl->H[(size_t)i * (kMaxM + 1) + i];
    }
}

// x += D^-1 V[0..j-1] y, or with out the preconditioner input out = D^-1 V[0..j-1] y (the
// polynomial preconditioner then maps it to the update)
template <class TV, class TX>
__global__ void __launch_bounds__(kThreads) k_xupdate(int n, const TV *__restrict__ V, size_t ld, const TV *__restrict__ dinv,
                                                      const GmresCtl *__restrict__ ctl, TX *__restrict__ x,
                                                      TV *__restrict__ out = nullptr) {
    __shared__ TV sy[kMaxM];
    const int j = ctl->j;
    for (int k = threadIdx.x; k < j; k += kThreads) sy[k] = (TV)ctl->y[k];
    __syncthreads();
    for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
        TV s = TV(0);
        int k = 0;
        for (; k + 8 <= j; k += 8) {
            TV v[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) v[u] = V[(size_t)(k + u) * ld + i];
#pragma unroll
            for (int u = 0; u < 8; ++u) s += sy[k + u] * v[u];
        }
        for (; k < j; ++k) s += sy[k] * V[(size_t)k * ld + i];
        if (out) out[i] = dinv[i] * s;
        else x[i] = (TX)(x[i] + dinv[i] * s);
    }
}

// r = b - A x with the products accumulated in FP64, partial ||r||^2 and ||b||^2 per CTA; with
// z also the Jacobi-scaled copy z = D^-1 r.  One thread per block row.
template <class TM, class TX, class TR, int DPN>
__global__ void __launch_bounds__(kThreads) k_residual(Op<TM> op, const TX *__restrict__ x, const double *__restrict__ b,
                                                       TR *__restrict__ r, double *part, const TR *__restrict__ dinv = nullptr,
                                                       TR *__restrict__ z = nullptr) {
    __shared__ double sp[kWarps][2];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int row = blockIdx.x * kThreads + threadIdx.x;
    double rr = 0.0, bb = 0.0;
    if (row < op.N) {
        double y[DPN];
        if (x) {
            ell_row<double, TM, TX, DPN>(op, row, x, y);
        } else {
#pragma unroll
            for (int q = 0; q < DPN; ++q) y[q] = 0.0;
        }
#pragma unroll
        for (int q = 0; q < DPN; ++q) {
            const size_t i = (size_t)row * DPN + q;
            const double v = b[i] - y[q];
            const TR rv = (TR)v;
            r[i] = rv;
            if (z) z[i] = dinv[i] * rv;
            rr += v * v;
            bb += b[i] * b[i];
        }
    }
    rr = warp_sum(rr);
    bb = warp_sum(bb);
    if (lane == 0) {
        sp[wid][0] = rr;
        sp[wid][1] = bb;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, c = 0.0;
        for (int q = 0; q < kWarps; ++q) {
            a += sp[q][0];
            c += sp[q][1];
        }
        part[2 * blockIdx.x] = a;
        part[2 * blockIdx.x + 1] = c;
    }
}

// Start of a cycle: beta = ||r||, inv = 1/beta, g = [beta, 0...], j = 0.
__global__ void k_cycle_start(GmresCtl *ctl, const double *part, int nparts, const double *targetAbsPtr, LoopCond lc) {
    const double targetAbs = *targetAbsPtr;
    const int lane = threadIdx.x;
    double a = 0.0;
    a = lane_sum(part, nparts, 2, 0, lane);
    a = warp_sum(a);
    if (lane != 0) return;
    const double beta = sqrt(a);
    ctl->j = 0;
    ctl->reorth = 0;
    ctl->reorths = 0;
    ctl->breakdown = 0;
    ctl->nonfinite = !isfinite(beta);
    ctl->g[0] = beta;
    for (int k = 1; k <= kMaxM; ++k) ctl->g[k] = 0.0;
    ctl->resest = beta;
    ctl->inv = beta > 0.0 ? 1.0 / beta : 0.0;
    ctl->target = targetAbs;
    ctl->done = (beta <= targetAbs || beta == 0.0 || ctl->nonfinite) ? 1 : 0;
    loop_cond_set(lc, ctl->done ? 0u : 1u);
}

__global__ void k_zero_f(float *a, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = 0.f;
}
__global__ void k_axpy_f2d(double *x, const float *d, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] += (double)d[i];
}

// Jacobi inverse diagonal 1 / (K_ii + (C^T C)_ii) from the block-CSR values, in FP64 and in the
// precision of the Krylov basis.
template <class TM, class TV>
__global__ void k_dinv(const TM *__restrict__ K, const int *__restrict__ rowPtr, const int *__restrict__ bCol, int N,
                       int dpn, const int *penPtr, const int *penRow, const int *penCol, const double *penVal,
                       double *dinv, TV *dinvT) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= N) return;
    int kd = -1;
    for (int k = rowPtr[r]; k < rowPtr[r + 1]; ++k)
        if (bCol[k] == r) kd = k;
    for (int q = 0; q < dpn; ++q) {
        double d = (kd >= 0) ? (double)K[(size_t)kd * dpn * dpn + q * dpn + q] : 0.0;
        if (penPtr)
            for (int t = penPtr[r]; t < penPtr[r + 1]; ++t)
                if (penRow[t] == q && penCol[t] == r * dpn + q) d += penVal[t];
        const double v = (d != 0.0) ? 1.0 / d : 1.0;
        dinv[(size_t)r * dpn + q] = v;
        dinvT[(size_t)r * dpn + q] = (TV)v;
    }
}

// block-CSR (dd-value row-major blocks) -> slot-major block-ELL, one thread per (row, slot); the
// values are converted to the ELL's type (an FP32 solver copy of the FP64 matrix)
template <class TS, class T>
__global__ void k_to_ell(const TS *__restrict__ K, const int *__restrict__ rowPtr, const int *__restrict__ bCol, int N,
                         int S, int ld, int dd, T *__restrict__ Ke, int *__restrict__ colE) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)S * ld) return;
    const int s = (int)(t / ld), r = (int)(t - (long long)s * ld);
    const int k = (r < N) ? rowPtr[r] + s : -1;
    const bool has = r < N && k < rowPtr[r + 1];
    if (colE) colE[t] = has ? bCol[k] : (r < N ? r : 0);
    for (int q = 0; q < dd; ++q) Ke[((size_t)s * dd + q) * ld + r] = has ? (T)K[(size_t)k * dd + q] : T(0);
}

}  // namespace

// ---------------------------------------------------------------------------------------------

// Polynomial preconditioner of one solve: hop parameters with the weights already divided by
// the eigenvalue bound (host copy, passed to the hop kernels by value).
struct PolyHost {
    int deg = 0;
    float theta = 0.f, delta = 0.f;
    const float *amod = nullptr;  // per-node hop scales of the modulation network (device), or null
    double apwKey = 0.0;  // the L2 window the hop launches carry (part of the graph's key)
    float W[(ASTRO_PRECOND_MAX_DEGREE + 1) * 36] = {};
};

struct GmresWork {
    DevBuf V, w0, w1, z0, z1, part, ctl, dinv, dinvT, rres, xs, tgt;
    DevBuf x64, b64;  // FP64 solver: the solve's x and b live here, so its graph is reused across solves
    DevBuf yB0, yB1, zacc, pw;  // polynomial preconditioner: hop vectors, output, power-iteration scratch
    DevBuf Kh, Kr, penS, dsqT;  // its operator A^ = S A S (FP16 block-vector planes, scaled penalty) and S
    DevBuf nfF, nfL, nfPd, nfPart, mlpPrm, amod;  // node features and the modulation network's scales
    cudaStream_t bodyStream = nullptr;  // captures the bodies of the cycle's IF nodes
    bool condOk = true;                 // conditional graph nodes available
    OpH hop;
    int hopVersion = -1;  // version of the matrix the operator and lamEst were built from
    double lamEst = 0.0;  // power-iteration estimate of the largest eigenvalue of D^-1 A
    // L2 persistence window over the operator's block planes for the hop launches (a launch
    // attribute, so captured into the graph nodes); off when the device has no persisting L2
    cudaAccessPolicyWindow apw = {};
    bool apwOn = false;
    const PolyHost *poly = nullptr;
    // vector that scales a residual into the preconditioner's input: D^-1 (Jacobi) or S (poly)
    template <class TV> const TV *y0s() { return poly ? dptr<TV>(dsqT) : dptr<TV>(dinvT); }
    // restart cycle captured as a graph, reused while the matrix and vectors stay the same
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    const void *gK = nullptr, *gx = nullptr, *gb = nullptr;
    PolyHost gPoly;  // the hop parameters the graph was captured with
    int n = 0, m = 0;
    size_t ld = 0;
    int nChunks = 0, nRowCtas = 0;
    std::vector<double> hp;
};

// Version of the matrix the FP32 solver copy comes from: the FP32 assembly when there is one,
// else the FP64 matrix converted (the shell path has no FP32 element kernels).
static int k32_source_version(const astro_ctx *ctx) {
    return ctx->haveK32 ? ctx->k32Version : 1000000 + ctx->k64Version;
}

// Solver copy of the assembled matrix in slot-major block-ELL layout (rebuilt when the assembly
// changed).  The FP32 copy converts the FP64 matrix when no FP32 assembly exists.
template <class TM> static const TM *ell_of(astro_ctx *ctx, int *rc) {
    const bool f64 = sizeof(TM) == 8;
    const bool cvt = !f64 && !ctx->haveK32;
    DevBuf &dst = f64 ? ctx->d_K64p : ctx->d_K32p;
    int &ver = f64 ? ctx->k64PlanesVersion : ctx->k32PlanesVersion;
    const int cur = f64 ? ctx->k64Version : k32_source_version(ctx);
    const AstroPrep &P = ctx->P;
    const int dd = P.dpn * P.dpn;
    *rc = ASTRO_OK;
    if (!ctx->ellSlots) {
        int S = 0;
        for (int r = 0; r < P.N; ++r) S = std::max(S, P.bRowPtr[r + 1] - P.bRowPtr[r]);
        ctx->ellSlots = S;
        ctx->ellLd = (P.N + 31) / 32 * 32;
    }
    const int S = ctx->ellSlots, ld = ctx->ellLd;
    bool needCol = false;
    if (!ctx->d_ellCol.p) {
        if ((*rc = dev_alloc(ctx, ctx->d_ellCol, sizeof(int) * (size_t)S * ld))) return nullptr;
        needCol = true;
    }
    if (!dst.p && (*rc = dev_alloc(ctx, dst, sizeof(TM) * (size_t)S * dd * ld))) return nullptr;
    if (ver != cur || needCol) {
        const long long tot = (long long)S * ld;
        const unsigned g = (unsigned)((tot + 255) / 256);
        int *colOut = needCol ? dptr<int>(ctx->d_ellCol) : nullptr;
        if (f64 || cvt)
            k_to_ell<double, TM><<<g, 256, 0, ctx->stream>>>(dptr<double>(ctx->d_K64), dptr<int>(ctx->d_bRowPtr),
                                                             dptr<int>(ctx->d_bCol), P.N, S, ld, dd, dptr<TM>(dst), colOut);
        else
            k_to_ell<float, TM><<<g, 256, 0, ctx->stream>>>(dptr<float>(ctx->d_K32), dptr<int>(ctx->d_bRowPtr),
                                                            dptr<int>(ctx->d_bCol), P.N, S, ld, dd, dptr<TM>(dst), colOut);
        if ((*rc = cuda_check(ctx, cudaGetLastError(), "to_ell"))) return nullptr;
        ver = cur;
    }
    return dptr<TM>(dst);
}

template <class TM> static Op<TM> make_op(astro_ctx *ctx, const TM *Kell) {
    Op<TM> op;
    op.K = Kell;
    op.col = dptr<int>(ctx->d_ellCol);
    op.S = ctx->ellSlots;
    op.ld = ctx->ellLd;
    op.penPtr = ctx->penRows ? dptr<int>(ctx->d_penPtr) : nullptr;
    op.penRow = dptr<int>(ctx->d_penRow);
    op.penCol = dptr<int>(ctx->d_penCol);
    op.penVal = dptr<double>(ctx->d_penVal);
    op.N = ctx->P.N;
    op.dpn = ctx->P.dpn;
    return op;
}

// Enqueues the hops of the polynomial preconditioner on y0 = D^-1 v (overwritten: the three-term
// recurrence rotates through y0 and two scratch vectors) and returns the output vector P v.
// always: run even when the cycle has finished (the final update of x).
template <class TM, class TV, int DPN>
static TV *enqueue_poly(astro_ctx *ctx, GmresWork &W, TV *y0, int always, cudaStream_t s) {
    const PolyHost &P = *W.poly;
    const int dd = DPN * DPN;
    TV *buf[3] = {y0, dptr<TV>(W.yB0), dptr<TV>(W.yB1)};
    TV *z = dptr<TV>(W.zacc);
    const unsigned grid = (unsigned)((ctx->P.N + kCtaRows - 1) / kCtaRows);
    HopArgs h;
    std::memset(&h, 0, sizeof(h));
    for (int q = 0; q < dd; ++q) h.w0[q] = P.W[q];
    h.theta = P.theta;
    h.amod = P.amod;
    int cur = 0;
    for (int k = 0; k < P.deg; ++k) {
        const int nxt = (cur + 1) % 3, prv = (cur + 2) % 3;
        for (int q = 0; q < dd; ++q) h.w[q] = P.W[(k + 1) * dd + q];
        h.first = (k == 0);
        h.k1 = k + 1;
        h.c = (k == 0 ? 1.f : 2.f) / P.delta;
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(grid);
        cfg.blockDim = dim3(kThreads);
        cfg.stream = s;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeAccessPolicyWindow;
        at[0].val.accessPolicyWindow = W.apw;
        cfg.attrs = at;
        cfg.numAttrs = W.apwOn ? 1 : 0;
        cudaLaunchKernelEx(&cfg, k_poly_hop<OpH, TV, DPN>, W.hop, (const TV *)dptr<TV>(W.dsqT), (const TV *)buf[cur],
                           (const TV *)buf[prv], k + 1 < P.deg ? buf[nxt] : (TV *)nullptr, z, h,
                           (const GmresCtl *)dptr<GmresCtl>(W.ctl), always);
        cur = nxt;
    }
    return z;
}

// Enqueues Arnoldi steps first..first+nsteps-1 on s (the w/z buffers alternate with the step's
// parity); with lc.use each step's control sets the condition lc (of the next IF node).
template <class TM, class TV, int DPN>
static void enqueue_cycle(astro_ctx *ctx, GmresWork &W, const Op<TM> &op, int m, int first, int nsteps,
                          cudaStream_t s, LoopCond lc) {
    TV *V = dptr<TV>(W.V), *wa = dptr<TV>(W.w0), *wb = dptr<TV>(W.w1);
    TV *za = dptr<TV>(W.z0), *zb = dptr<TV>(W.z1);
    GmresCtl *ctl = dptr<GmresCtl>(W.ctl);
    double *part = dptr<double>(W.part);
    const TV *dinv = W.y0s<TV>();
    const int n = W.n;
    double *partB = part + (size_t)(kMaxM + 1) * W.nChunks;
    double *partN = partB + (size_t)(kMaxM + 1) * W.nChunks;  // per-CTA ||w||^2 of the step's last update
    const unsigned spmvGrid = (unsigned)((ctx->P.N + kCtaRows - 1) / kCtaRows);
    for (int step = first; step < first + nsteps; ++step) {
        TV *wprev = (step % 2 == 0) ? wa : wb, *zprev = (step % 2 == 0) ? za : zb;
        TV *wnew = (step % 2 == 0) ? wb : wa, *znew = (step % 2 == 0) ? zb : za;
        const TV *zin = W.poly ? enqueue_poly<TM, TV, DPN>(ctx, W, zprev, 0, s) : zprev;
        k_spmv_step<TM, TV, DPN><<<spmvGrid, kThreads, 0, s>>>(op, V, W.ld, wprev, zin, wnew, ctl);
        k_dots<TV><<<W.nChunks, kGsThreads, 0, s>>>(n, V, W.ld, wnew, ctl, part, W.nChunks);
        k_update<TV><<<W.nChunks, kGsThreads, 0, s>>>(n, V, W.ld, wnew, ctl, partB, partN, W.nChunks, 0, dinv, znew, m, lc);
        k_update<TV><<<W.nChunks, kGsThreads, 0, s>>>(n, V, W.ld, wnew, ctl, partB, partN, W.nChunks, 1, dinv, znew, m, lc);
    }
}

static double sum_parts(astro_ctx *ctx, GmresWork &W, int which, int *rc) {
    const int np = W.nRowCtas;
    W.hp.resize(2 * (size_t)np);
    cudaError_t e = cudaMemcpyAsync(W.hp.data(), W.part.p, sizeof(double) * 2 * np, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    *rc = cuda_check(ctx, e, "residual partials");
    double s = 0.0;
    for (int q = 0; q < np; ++q) s += W.hp[2 * q + which];
    return s;
}

// Restarted Jacobi-GMRES(m) on A x = b in precision TV with matrix values TM.  x (TV) in/out
// on the device, b (double) on the device.
template <class TM, class TV, int DPN>
static int gmres_solve(astro_ctx *ctx, GmresWork &W, const TM *K, TV *x, const double *b, double tgtAbs, int maxCycles,
                       int m, int *iters, int *cycles, double *finalRes) {
    cudaStream_t s = ctx->stream;
    Op<TM> op = make_op<TM>(ctx, K);
    GmresCtl *ctl = dptr<GmresCtl>(W.ctl);
    double *part = dptr<double>(W.part);
    // the absolute target is read by the graph from device memory
    CK(cudaMemcpyAsync(W.tgt.p, &tgtAbs, sizeof(double), cudaMemcpyHostToDevice, s));
    const bool samePoly = W.poly ? (W.gPoly.deg == W.poly->deg && std::memcmp(&W.gPoly, W.poly, sizeof(PolyHost)) == 0)
                                 : W.gPoly.deg == 0;
    if (!(W.exec && W.gK == K && W.gx == x && W.gb == b && samePoly)) {
        if (W.exec) cudaGraphExecDestroy(W.exec);
        if (W.graph) cudaGraphDestroy(W.graph);
        W.exec = nullptr;
        W.graph = nullptr;
        const LoopCond none{0, 0};
        // the Arnoldi steps of a cycle behind conditional IF nodes (two steps each), or, when the
        // driver does not take conditional nodes, unrolled to m steps that turn into no-ops once
        // the cycle has finished
        bool cond = W.condOk;
        for (int attempt = 0; attempt < 2 && !W.graph; ++attempt) {
            CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
            k_residual<TM, TV, TV, DPN><<<W.nRowCtas, kThreads, 0, s>>>(op, x, b, dptr<TV>(W.w0), part, W.y0s<TV>(),
                                                                         dptr<TV>(W.z0));
            // one handle per IF node (a handle belongs to one node): the cycle start sets the first,
            // the steps behind node i set the handle of node i + 1; every handle starts each
            // launch at 0, so the nodes after a skipped one are skipped too
            const int nIf = (m + 1) / 2;
            std::vector<cudaGraphConditionalHandle> hs(nIf, 0);
            cudaGraph_t cg = nullptr;
            cudaError_t ce = cudaSuccess;
            bool useCond = false;
            if (cond) {
                cudaStreamCaptureStatus cs;
                ce = cudaStreamGetCaptureInfo(s, &cs, nullptr, &cg);
                for (int i = 0; i < nIf && ce == cudaSuccess; ++i)
                    ce = cudaGraphConditionalHandleCreate(&hs[i], cg, 0, cudaGraphCondAssignDefault);
                useCond = ce == cudaSuccess;
            }
            k_cycle_start<<<1, 32, 0, s>>>(ctl, part, W.nRowCtas, dptr<double>(W.tgt),
                                           useCond ? LoopCond{hs[0], 1} : none);
            if (useCond) {
                // ceil(m/2) IF nodes in sequence, two steps in each
                for (int first = 0; first < m && ce == cudaSuccess; first += 2) {
                    const int i = first / 2;
                    const LoopCond next = (i + 1 < nIf) ? LoopCond{hs[i + 1], 1} : none;
                    cudaStreamCaptureStatus cs;
                    const cudaGraphNode_t *deps = nullptr;
                    const cudaGraphEdgeData *ed = nullptr;
                    size_t nd = 0;
                    ce = cudaStreamGetCaptureInfo(s, &cs, nullptr, &cg, &deps, &ed, &nd);
                    cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
                    cp.conditional.handle = hs[i];
                    cp.conditional.type = cudaGraphCondTypeIf;
                    cp.conditional.size = 1;
                    cudaGraphNode_t cn = nullptr;
                    if (ce == cudaSuccess) ce = cudaGraphAddNode(&cn, cg, deps, ed, nd, &cp);
                    if (ce == cudaSuccess)
                        ce = cudaStreamBeginCaptureToGraph(W.bodyStream, cp.conditional.phGraph_out[0], nullptr, nullptr,
                                                           0, cudaStreamCaptureModeRelaxed);
                    if (ce == cudaSuccess) {
                        enqueue_cycle<TM, TV, DPN>(ctx, W, op, m, first, std::min(2, m - first), W.bodyStream, next);
                        cudaGraph_t body = nullptr;
                        ce = cudaStreamEndCapture(W.bodyStream, &body);
                    }
                    if (ce == cudaSuccess)
                        ce = cudaStreamUpdateCaptureDependencies(s, &cn, nullptr, 1, cudaStreamSetCaptureDependencies);
                }
            } else {
                enqueue_cycle<TM, TV, DPN>(ctx, W, op, m, 0, m, s, none);
            }
            k_lsq<<<1, 1, 0, s>>>(ctl);
            if (W.poly) {
                TV *y0 = dptr<TV>(W.z0);
                k_xupdate<TV, TV><<<4 * 152, kThreads, 0, s>>>(W.n, dptr<TV>(W.V), W.ld, W.y0s<TV>(), ctl, x, y0);
                TV *dz = enqueue_poly<TM, TV, DPN>(ctx, W, y0, 1, s);
                k_add<TV><<<(W.n + 255) / 256, 256, 0, s>>>(W.n, x, dz);
            } else {
                k_xupdate<TV, TV><<<4 * 152, kThreads, 0, s>>>(W.n, dptr<TV>(W.V), W.ld, dptr<TV>(W.dinvT), ctl, x);
            }
            cudaGraph_t g = nullptr;
            cudaError_t ee = cudaStreamEndCapture(s, &g);
            if (cond && (ce != cudaSuccess || ee != cudaSuccess)) {
                // conditional nodes refused: clear the error state and capture the unrolled cycle
                if (g) cudaGraphDestroy(g);
                cudaGetLastError();
                cond = W.condOk = false;
                continue;
            }
            CK(ee);
            cudaError_t ie = cudaGraphInstantiate(&W.exec, g, 0);
            if (cond && ie != cudaSuccess) {
                cudaGraphDestroy(g);
                W.exec = nullptr;
                cudaGetLastError();
                cond = W.condOk = false;
                continue;
            }
            if (ie != cudaSuccess) cudaGraphDestroy(g);
            CK(ie);
            W.graph = g;
        }
        if (W.poly) W.gPoly = *W.poly;
        else W.gPoly.deg = 0;
        W.gK = K;
        W.gx = x;
        W.gb = b;
    }
    cudaGraphExec_t exec = W.exec;
    int status = ASTRO_OK;
    struct {
        double resest;
        int j, done, breakdown, nonfinite;
    } hc;
    for (int cyc = 0; cyc < maxCycles; ++cyc) {
        CK(cudaGraphLaunch(exec, s));
        CK(cudaMemcpyAsync(&hc, &ctl->resest, sizeof(hc), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        *iters += hc.j;
        *cycles += 1;
        *finalRes = hc.resest;
        if (hc.nonfinite) {
            status = ASTRO_ERR_NAN;
            break;
        }
        if (hc.resest <= tgtAbs || hc.breakdown) break;
        if (cyc == maxCycles - 1) status = ASTRO_ERR_MAXIT;
    }
    return status;
}

static int work_alloc(astro_ctx *ctx, GmresWork &W, int m, int tv) {
    const int n = ctx->P.n;
    W.n = n;
    W.m = m;
    W.ld = ((size_t)n + 31) / 32 * 32;
    W.nChunks = (n + kChunk - 1) / kChunk;
    W.nRowCtas = (ctx->P.N + kThreads - 1) / kThreads;
    const size_t nparts = std::max((size_t)3 * W.nChunks * (kMaxM + 1), (size_t)2 * W.nRowCtas);
    int rc;
    if ((rc = dev_alloc(ctx, W.V, W.ld * (m + 1) * tv))) return rc;
    if ((rc = dev_alloc(ctx, W.w0, (size_t)n * tv))) return rc;
    if ((rc = dev_alloc(ctx, W.w1, (size_t)n * tv))) return rc;
    if ((rc = dev_alloc(ctx, W.z0, (size_t)n * tv))) return rc;
    if ((rc = dev_alloc(ctx, W.z1, (size_t)n * tv))) return rc;
    if ((rc = dev_alloc(ctx, W.part, sizeof(double) * nparts))) return rc;
    if ((rc = dev_alloc(ctx, W.ctl, sizeof(GmresCtl)))) return rc;
    if ((rc = dev_alloc(ctx, W.dinv, sizeof(double) * (size_t)n))) return rc;
    if ((rc = dev_alloc(ctx, W.dinvT, (size_t)n * tv))) return rc;
    if ((rc = dev_alloc(ctx, W.rres, sizeof(double) * (size_t)n))) return rc;
    if ((rc = dev_alloc(ctx, W.xs, sizeof(float) * (size_t)n))) return rc;
    if ((rc = dev_alloc(ctx, W.tgt, sizeof(double)))) return rc;
    CK(cudaMemsetAsync(W.ctl.p, 0, sizeof(GmresCtl), ctx->stream));
    CK(cudaStreamCreateWithFlags(&W.bodyStream, cudaStreamNonBlocking));
    return ASTRO_OK;
}

static void work_free(GmresWork &W) {
    if (W.bodyStream) cudaStreamDestroy(W.bodyStream);
    W.bodyStream = nullptr;
    if (W.exec) cudaGraphExecDestroy(W.exec);
    if (W.graph) cudaGraphDestroy(W.graph);
    W.exec = nullptr;
    W.graph = nullptr;
    DevBuf *b[] = {&W.V,    &W.w0,   &W.w1,    &W.z0, &W.z1,  &W.part, &W.ctl, &W.dinv,
                   &W.dinvT, &W.rres, &W.xs,  &W.tgt, &W.yB0, &W.yB1,  &W.zacc, &W.pw,
                   &W.Kh,    &W.Kr,   &W.penS, &W.dsqT, &W.x64, &W.b64, &W.nfF, &W.nfL,
                   &W.nfPd,  &W.nfPart, &W.mlpPrm, &W.amod};
    for (auto *x : b) dev_free(*x);
}

// Solver workspace of one method kept on the context (slot 0 FP64, 1 mixed, 2 learned), with its
// captured restart-cycle graph; reallocated when the basis size changes.
static GmresWork *work_get(astro_ctx *ctx, int slot, int m, int tv, int *rc) {
    GmresWork *W = static_cast<GmresWork *>(ctx->solveWork[slot]);
    if (W && W->m == m && W->n == ctx->P.n) return W;
    if (W) {
        work_free(*W);
        delete W;
    }
    W = new GmresWork();
    W->condOk = !ctx->unrolledCycles;
    ctx->solveWork[slot] = W;
    if ((*rc = work_alloc(ctx, *W, m, tv))) {
        work_free(*W);
        delete W;
        ctx->solveWork[slot] = nullptr;
        return nullptr;
    }
    return W;
}

void krylov_release(astro_ctx *ctx) {
    for (void *&p : ctx->solveWork) {
        if (!p) continue;
        GmresWork *W = static_cast<GmresWork *>(p);
        work_free(*W);
        delete W;
        p = nullptr;
    }
}

// r = b - A x with A from K64 (kind 64) or K32 (kind 32); returns ||r||/||b|| (||r|| if b = 0).
template <int DPN>
static int true_residual(astro_ctx *ctx, GmresWork &W, int kind, const double *x, const double *b, double *rel,
                         double *r_out, double *rnorm = nullptr, double *bnorm = nullptr) {
    cudaStream_t s = ctx->stream;
    double *part = dptr<double>(W.part);
    int prc = ASTRO_OK;
    if (kind == 64) {
        const double *Kp = ell_of<double>(ctx, &prc);
        if (prc) return prc;
        Op<double> op = make_op<double>(ctx, Kp);
        k_residual<double, double, double, DPN><<<W.nRowCtas, kThreads, 0, s>>>(op, x, b, r_out, part);
    } else {
        const float *Kp = ell_of<float>(ctx, &prc);
        if (prc) return prc;
        Op<float> op = make_op<float>(ctx, Kp);
        k_residual<float, double, double, DPN><<<W.nRowCtas, kThreads, 0, s>>>(op, x, b, r_out, part);
    }
    int rc = ASTRO_OK;
    const double a = sum_parts(ctx, W, 0, &rc);
    if (rc) return rc;
    double c = 0.0;
    for (int q = 0; q < W.nRowCtas; ++q) c += W.hp[2 * q + 1];
    *rel = (c > 0.0) ? std::sqrt(a / c) : std::sqrt(a);
    if (rnorm) *rnorm = std::sqrt(a);
    if (bnorm) *bnorm = std::sqrt(c);
    return ASTRO_OK;
}

// 50 power iterations of D^-1 A (deterministic start vector and reductions); lam = the last
// norm ratio, which approaches the largest eigenvalue from below.
template <class OP, class TV, int DPN>
static int power_lambda(astro_ctx *ctx, const OP &op, const TV *dinv, double *lam) {
    const int n = ctx->P.n;
    const int nCta = (ctx->P.N + kCtaRows - 1) / kCtaRows;
    cudaStream_t s = ctx->stream;
    DevBuf a, b, part, cnt, scal;
    int rc;
    if ((rc = dev_alloc(ctx, a, sizeof(TV) * n)) || (rc = dev_alloc(ctx, b, sizeof(TV) * n)) ||
        (rc = dev_alloc(ctx, part, sizeof(double) * nCta)) || (rc = dev_alloc(ctx, cnt, sizeof(unsigned))) ||
        (rc = dev_alloc(ctx, scal, 2 * sizeof(double)))) {
        dev_free(a), dev_free(b), dev_free(part), dev_free(cnt), dev_free(scal);
        return rc;
    }
    cudaMemsetAsync(cnt.p, 0, sizeof(unsigned), s);
    k_power_init<TV><<<(n + 255) / 256, 256, 0, s>>>(dptr<TV>(a), n, dptr<double>(scal));
    for (int it = 0; it < 50; ++it) {
        TV *x = dptr<TV>(it % 2 ? b : a), *y = dptr<TV>(it % 2 ? a : b);
        k_power_step<OP, TV, DPN><<<nCta, kThreads, 0, s>>>(op, dinv, x, y, dptr<double>(part), dptr<unsigned>(cnt),
                                                            dptr<double>(scal));
    }
    double h[2] = {0.0, 0.0};
    cudaError_t e = cudaMemcpyAsync(h, scal.p, sizeof(h), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    rc = cuda_check(ctx, e, "power iteration");
    dev_free(a), dev_free(b), dev_free(part), dev_free(cnt), dev_free(scal);
    *lam = h[1];
    if (!rc && !(std::isfinite(h[1]) && h[1] > 0.0)) rc = set_err(ctx, ASTRO_ERR_NAN, "eigenvalue estimate is not positive");
    return rc;
}

// Persisting L2 for the hops: when the operator (plus the vectors) does not fit in L2, every hop
// streams it from HBM and LRU evicts each part before its reuse; a window that keeps a fixed share
// of the block planes resident (half of the persisting set-aside) cuts that traffic.  The
// set-aside is a limit of this CUDA context: persist_begin raises it to the device's maximum and
// fills the workspace's window; persist_end releases the persisting lines and restores the limit.
static bool persist_begin(astro_ctx *ctx, GmresWork &W, size_t *prev) {
    int maxPersist = 0, maxWin = 0;
    cudaDeviceGetAttribute(&maxPersist, cudaDevAttrMaxPersistingL2CacheSize, ctx->device);
    cudaDeviceGetAttribute(&maxWin, cudaDevAttrMaxAccessPolicyWindowSize, ctx->device);
    W.apwOn = false;
    if (!(maxPersist > 0 && maxWin > 0 && cudaDeviceGetLimit(prev, cudaLimitPersistingL2CacheSize) == cudaSuccess &&
          cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, (size_t)maxPersist) == cudaSuccess)) {
        cudaGetLastError();
        return false;
    }
    W.apw.base_ptr = W.Kh.p;
    W.apw.num_bytes = std::min(W.Kh.bytes, (size_t)maxWin);
    W.apw.hitRatio = (float)std::min(1.0, 0.5 * maxPersist / (double)W.apw.num_bytes);
    W.apw.hitProp = cudaAccessPropertyPersisting;
    W.apw.missProp = cudaAccessPropertyStreaming;
    W.apwOn = true;
    return true;
}
static void persist_end(size_t prev) {
    cudaCtxResetPersistingL2Cache();
    cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, prev);
    cudaGetLastError();
}

// Checks the network against the model (degree, DOF per node, interval, finite weights).
static int precond_check(astro_ctx *ctx, const astro_precond *p) {
    if (p->degree < 1 || p->degree > ASTRO_PRECOND_MAX_DEGREE) return set_err(ctx, ASTRO_ERR_ARG, "precond degree out of range");
    if (p->dpn != ctx->P.dpn) return set_err(ctx, ASTRO_ERR_ARG, "precond DOF per node differs from the model's");
    if (!(p->ratio > 1.0) || !(p->lambda_scale > 0.0) || !std::isfinite(p->ratio) || !std::isfinite(p->lambda_scale))
        return set_err(ctx, ASTRO_ERR_ARG, "precond ratio must be > 1 and lambda_scale > 0");
    for (int q = 0; q < (p->degree + 1) * p->dpn * p->dpn; ++q)
        if (!std::isfinite(p->weights[q])) return set_err(ctx, ASTRO_ERR_ARG, "non-finite precond weight");
    return ASTRO_OK;
}

template <int DPN>
static int solve_static_dev(astro_ctx *ctx, const double *d_b, double *d_x, const astro_solve_opts *o,
                            astro_solve_stats *st) {
    const int n = ctx->P.n;
    const int m = o->restart > 0 ? (o->restart > kMaxM ? kMaxM : o->restart) : 50;
    const int maxIters = o->max_iters > 0 ? o->max_iters : 200000;
    const int maxCycles = (maxIters + m - 1) / m;
    int rc = ASTRO_OK;
    int iters = 0, cycles = 0, refinements = 0;
    double rel = 0.0, est = 0.0, rn = 0.0, bn = 0.0;
    const bool fp64 = o->method == ASTRO_SOLVER_GMRES_JACOBI_FP64;
    const bool learned = o->method == ASTRO_SOLVER_FGMRES_LEARNED;
    // the matrix the true residual is formed with: the FP64 assembly whenever it is resident
    const int resKind = ctx->haveK64 ? 64 : 32;
    astro_precond pdef;
    const astro_precond *pc = o->precond;
    if (learned && !pc) {
        astro_precond_init(24, 3000.0, ctx->P.dpn, &pdef);
        pc = &pdef;
    }
    if (learned && (rc = precond_check(ctx, pc))) return rc;
    PolyHost ph;
    std::memset(&ph, 0, sizeof(ph));  // compared bytewise as the graph's key
    size_t persistPrev = 0;
    bool persistSet = false;
    if (fp64 && !ctx->haveK64) return set_err(ctx, ASTRO_ERR_STATE, "FP64 stiffness not assembled");
    if (!fp64 && !ctx->haveK32 && !ctx->haveK64) return set_err(ctx, ASTRO_ERR_STATE, "stiffness not assembled");
    GmresWork *Wp = work_get(ctx, fp64 ? 0 : (learned ? 2 : 1), m, fp64 ? sizeof(double) : sizeof(float), &rc);
    if (!Wp) return rc;
    GmresWork &W = *Wp;
    W.poly = nullptr;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, ctx->stream);
    double *r = dptr<double>(W.rres);
    if (fp64) {
        const double *K64p = ell_of<double>(ctx, &rc);
        if (rc) return rc;
        k_dinv<double, double><<<(ctx->P.N + 255) / 256, 256, 0, ctx->stream>>>(
            dptr<double>(ctx->d_K64), dptr<int>(ctx->d_bRowPtr), dptr<int>(ctx->d_bCol), ctx->P.N, ctx->P.dpn,
            ctx->penRows ? dptr<int>(ctx->d_penPtr) : nullptr, dptr<int>(ctx->d_penRow), dptr<int>(ctx->d_penCol),
            dptr<double>(ctx->d_penVal), dptr<double>(W.dinv), dptr<double>(W.dinvT));
        if (!W.x64.p && ((rc = dev_alloc(ctx, W.x64, sizeof(double) * n)) || (rc = dev_alloc(ctx, W.b64, sizeof(double) * n)))) {
            dev_free(W.x64);
            return rc;
        }
        double *x = dptr<double>(W.x64);
        const double *bb = dptr<double>(W.b64);
        CK(cudaMemcpyAsync(W.x64.p, d_x, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->stream));
        CK(cudaMemcpyAsync(W.b64.p, d_b, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->stream));
        rc = true_residual<DPN>(ctx, W, 64, nullptr, bb, &rel, r, &rn, &bn);
        const double tgt = o->rtol * bn;
        while (rc == ASTRO_OK) {
            int grc = gmres_solve<double, double, DPN>(ctx, W, K64p, x, bb, tgt, maxCycles - cycles, m,
                                                       &iters, &cycles, &est);
            if ((rc = true_residual<DPN>(ctx, W, 64, x, bb, &rel, r))) break;
            if (rel <= o->rtol) break;
            if (grc == ASTRO_ERR_NAN) {
                rc = set_err(ctx, ASTRO_ERR_NAN, "non-finite value in GMRES");
                break;
            }
            if (grc == ASTRO_ERR_MAXIT || cycles >= maxCycles) {
                rc = ASTRO_ERR_MAXIT;
                break;
            }
        }
        CK(cudaMemcpyAsync(d_x, W.x64.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->stream));
    } else {
        const float *K32p = ell_of<float>(ctx, &rc);
        if (rc) return rc;
        const int* pp = ctx->penRows ? dptr<int>(ctx->d_penPtr) : nullptr;
        if (ctx->haveK32)
            k_dinv<float, float><<<(ctx->P.N + 255) / 256, 256, 0, ctx->stream>>>(
                dptr<float>(ctx->d_K32), dptr<int>(ctx->d_bRowPtr), dptr<int>(ctx->d_bCol), ctx->P.N, ctx->P.dpn, pp,
                dptr<int>(ctx->d_penRow), dptr<int>(ctx->d_penCol), dptr<double>(ctx->d_penVal), dptr<double>(W.dinv),
                dptr<float>(W.dinvT));
        else
            k_dinv<double, float><<<(ctx->P.N + 255) / 256, 256, 0, ctx->stream>>>(
                dptr<double>(ctx->d_K64), dptr<int>(ctx->d_bRowPtr), dptr<int>(ctx->d_bCol), ctx->P.N, ctx->P.dpn, pp,
                dptr<int>(ctx->d_penRow), dptr<int>(ctx->d_penCol), dptr<double>(ctx->d_penVal), dptr<double>(W.dinv),
                dptr<float>(W.dinvT));
        if (learned) {
            // the network's hop vectors, its operator A^ = S A S in FP16 with S = D^-1/2, and the
            // interval [lambda/ratio, lambda] from the eigenvalue estimate on A^ (inside the timed
            // solve)
            double lam = 0.0;
            const int S = ctx->ellSlots, ld = ctx->ellLd, dd = DPN * DPN;
            // allocated once per workspace: the captured graph holds these pointers
            if (!W.Kh.p &&
                ((rc = dev_alloc(ctx, W.yB0, sizeof(float) * n)) || (rc = dev_alloc(ctx, W.yB1, sizeof(float) * n)) ||
                 (rc = dev_alloc(ctx, W.zacc, sizeof(float) * n)) || (rc = dev_alloc(ctx, W.dsqT, sizeof(float) * n)) ||
                 (rc = dev_alloc(ctx, W.penS, sizeof(double) * std::max(1, ctx->penRows))) ||  // penalty entries
                 (rc = dev_alloc(ctx, W.Kr, sizeof(uint16_t) * BvShape<DPN>::REM * (size_t)S * ld)) ||
                 (rc = dev_alloc(ctx, W.Kh, sizeof(uint4) * BvShape<DPN>::NV * (size_t)S * ld)))) {
                dev_free(W.Kh);
                return rc;
            }
            // the operator and its eigenvalue estimate depend only on the matrix: rebuilt when the
            // matrix (or its constraint scaling) changed, reused by repeated solves (time steps)
            const int opVer = k32_source_version(ctx) * 64 + (ctx->penVersion & 63);
            if (W.hopVersion != opVer) {
                k_sqrt_f<<<(n + 255) / 256, 256, 0, ctx->stream>>>(dptr<double>(W.dinv), dptr<float>(W.dsqT), n);
                const long long tot = (long long)S * ld;
                k_scaled_bv<DPN><<<(unsigned)((tot + 255) / 256), 256, 0, ctx->stream>>>(
                    K32p, dptr<int>(ctx->d_ellCol), S, ld, ctx->P.N, dptr<float>(W.dsqT), dptr<uint4>(W.Kh), W.Kr.p);
                const Op<float> o32 = make_op<float>(ctx, K32p);
                W.hop = OpH{dptr<uint4>(W.Kh), W.Kr.p, o32.col,    o32.S,      o32.ld,    o32.penPtr,
                            o32.penRow,         o32.penCol, o32.penVal, o32.N, o32.dpn};
                if (ctx->penRows) {
                    k_scaled_pen<<<(ctx->P.N + 255) / 256, 256, 0, ctx->stream>>>(
                        dptr<int>(ctx->d_penPtr), dptr<int>(ctx->d_penRow), dptr<int>(ctx->d_penCol),
                        dptr<double>(ctx->d_penVal), ctx->P.N, DPN, dptr<double>(W.dinv), dptr<double>(W.penS));
                    W.hop.penVal = dptr<double>(W.penS);
                }
                if ((rc = cuda_check(ctx, cudaGetLastError(), "preconditioner operator")) ||
                    (rc = power_lambda<OpH, float, DPN>(ctx, W.hop, (const float *)nullptr, &W.lamEst)))
                    return rc;
                W.hopVersion = opVer;
            }
            lam = W.lamEst * pc->lambda_scale;
            ph.deg = pc->degree;
            ph.theta = (float)(0.5 * lam * (1.0 + 1.0 / pc->ratio));
            ph.delta = (float)(0.5 * lam * (1.0 - 1.0 / pc->ratio));
            for (int q = 0; q < (pc->degree + 1) * DPN * DPN; ++q) ph.W[q] = (float)(pc->weights[q] / lam);
            if (o->mlp && o->mlp->hidden > 0) {
                // the modulation network's per-node hop scales from the node features of the
                // assembly (one pass over the matrix and one over the nodes per solve); the
                // buffer is allocated once for the largest degree, so the graph's pointer holds
                if ((rc = precond_mlp_check(ctx, o->mlp, pc->degree))) return rc;
                const int N = ctx->P.N;
                if (!W.amod.p && ((rc = dev_alloc(ctx, W.nfF, sizeof(double) * (size_t)N * ASTRO_NODE_FEATURES)) ||
                                  (rc = dev_alloc(ctx, W.amod, sizeof(float) * (size_t)N *
                                                                   (ASTRO_PRECOND_MAX_DEGREE + 1)))))
                    return rc;
                if ((rc = precond_node_features(ctx, ctx->haveK64 ? 64 : 32, dptr<double>(W.nfF), W.nfL, W.nfPd,
                                                W.nfPart, ctx->stream)) ||
                    (rc = precond_mlp_scales_f32(ctx, o->mlp, dptr<double>(W.nfF), W.mlpPrm, dptr<float>(W.amod),
                                                 ctx->stream)))
                    return rc;
                ph.amod = dptr<float>(W.amod);
            }
            W.poly = &ph;
            persistSet = persist_begin(ctx, W, &persistPrev);
            if (W.apwOn) ph.apwKey = (double)W.apw.hitRatio * 1e12 + (double)W.apw.num_bytes;
        }
        float *d32 = dptr<float>(W.xs);
        const double inner = o->inner_rtol > 0 ? o->inner_rtol : 1e-4;
        // the outer residual is formed with the FP64 matrix when it is resident (the system the
        // tolerance refers to), else with the FP32 assembly's values in FP64 arithmetic
        const int refKind = resKind;
        for (refinements = 0; refinements < 200; ++refinements) {
            if ((rc = true_residual<DPN>(ctx, W, refKind, d_x, d_b, &rel, r, &rn))) break;
            if (rel <= o->rtol) break;
            if (!std::isfinite(rel)) {
                rc = set_err(ctx, ASTRO_ERR_NAN, "non-finite residual in refinement");
                break;
            }
            if (cycles >= maxCycles) {
                rc = ASTRO_ERR_MAXIT;
                break;
            }
            k_zero_f<<<(n + 255) / 256, 256, 0, ctx->stream>>>(d32, n);
            // a refinement asks for the usual inner reduction, except when the reduction left to
            // reach rtol is within what one FP32 inner solve resolves (1e-6): then it asks for
            // just that, with a margin, so that it is the last one
            const double need = 0.3 * o->rtol / rel;
            const double innerK = need >= 1e-6 ? need : inner;
            int rci = gmres_solve<float, float, DPN>(ctx, W, K32p, d32, r, innerK * rn, maxCycles - cycles,
                                                     m, &iters, &cycles, &est);
            if (rci == ASTRO_ERR_NAN) {
                rc = set_err(ctx, ASTRO_ERR_NAN, "non-finite value in the FP32 inner solve");
                break;
            }
            k_axpy_f2d<<<(n + 255) / 256, 256, 0, ctx->stream>>>(d_x, d32, n);
        }
        if (rc == ASTRO_OK && rel > o->rtol) rc = ASTRO_ERR_MAXIT;
    }
    cudaEventRecord(e1, ctx->stream);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (persistSet) persist_end(persistPrev);
    if (st) {
        st->iterations = iters;
        st->restarts = cycles;
        st->refinements = refinements;
        st->status = rc;
        st->rel_residual = rel;
        st->seconds = ms * 1e-3;
        st->conditional_graph = W.condOk ? 1 : 0;
        st->residual_kind = resKind;
    }
    if (rc == ASTRO_ERR_MAXIT) set_err(ctx, rc, "iteration limit reached before the residual tolerance");
    return rc;
}

static int solve_static_dpn(astro_ctx *ctx, const double *d_b, double *d_x, const astro_solve_opts *o,
                            astro_solve_stats *st) {
    if (ctx->P.dpn == 3) return solve_static_dev<3>(ctx, d_b, d_x, o, st);
    return solve_static_dev<6>(ctx, d_b, d_x, o, st);
}

// The learned solver falls back to the FP32 Jacobi solver (from the caller's initial guess) when
// it ends in a non-finite value, a breakdown or the iteration cap; the statistics then add both
// runs and set fallback.
int krylov_solve_static(astro_ctx *ctx, const double *d_b, double *d_x, const astro_solve_opts *o,
                        astro_solve_stats *st) {
    if (o->method != ASTRO_SOLVER_FGMRES_LEARNED) {
        const int rc = solve_static_dpn(ctx, d_b, d_x, o, st);
        if (st) st->fallback = 0;
        return rc;
    }
    const size_t bytes = sizeof(double) * ctx->P.n;
    DevBuf x0;
    int rc = dev_alloc(ctx, x0, bytes);
    if (rc) return rc;
    CK(cudaMemcpyAsync(x0.p, d_x, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    astro_solve_stats s1{};
    rc = solve_static_dpn(ctx, d_b, d_x, o, &s1);
    s1.fallback = 0;
    if (rc == ASTRO_ERR_NAN || rc == ASTRO_ERR_MAXIT || rc == ASTRO_ERR_BREAKDOWN) {
        CK(cudaMemcpyAsync(d_x, x0.p, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
        astro_solve_opts o2 = *o;
        o2.method = ASTRO_SOLVER_FGMRES_MIXED;
        o2.precond = nullptr;
        astro_solve_stats s2{};
        rc = solve_static_dpn(ctx, d_b, d_x, &o2, &s2);
        s2.iterations += s1.iterations;
        s2.restarts += s1.restarts;
        s2.refinements += s1.refinements;
        s2.seconds += s1.seconds;
        s2.fallback = 1;
        s1 = s2;
    }
    dev_free(x0);
    if (st) *st = s1;
    return rc;
}

// Times reps launches of one preconditioner hop on the operator of the last learned solve (the
// hop of the Chebyshev recurrence with zero weights: same loads and stores, no accumulation).
template <int DPN>
static int time_hop(astro_ctx *ctx, GmresWork &W, int reps, double *us, double *bytes) {
    using Sh = BvShape<DPN>;
    cudaStream_t s = ctx->stream;
    HopArgs h;
    std::memset(&h, 0, sizeof(h));
    h.theta = 0.5f;
    h.c = 1.0f;
    const unsigned grid = (unsigned)((ctx->P.N + kCtaRows - 1) / kCtaRows);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    size_t prev = 0;
    const bool ps = persist_begin(ctx, W, &prev);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kThreads);
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeAccessPolicyWindow;
    at[0].val.accessPolicyWindow = W.apw;
    cfg.attrs = at;
    cfg.numAttrs = W.apwOn ? 1 : 0;
    auto launch = [&]() {
        cudaLaunchKernelEx(&cfg, k_poly_hop<OpH, float, DPN>, W.hop, (const float *)dptr<float>(W.dsqT),
                           (const float *)dptr<float>(W.z0), (const float *)dptr<float>(W.yB0), dptr<float>(W.yB1),
                           dptr<float>(W.zacc), h, (const GmresCtl *)dptr<GmresCtl>(W.ctl), 1);
    };
    for (int i = 0; i < 5; ++i) launch();
    cudaEventRecord(e0, s);
    for (int i = 0; i < reps; ++i) launch();
    cudaEventRecord(e1, s);
    cudaError_t e = cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    int rc = cuda_check(ctx, e == cudaSuccess ? cudaGetLastError() : e, "hop timing");
    if (ps) persist_end(prev);
    if (rc) return rc;
    *us = 1e3 * ms / reps;
    // matrix planes and columns of every slot, then per block row the loads of y_k, y_{k-1}, S and
    // z and the stores of y_{k+1} and z (the gathered y_k are counted once)
    const double sl = (double)W.hop.S * W.hop.ld;
    *bytes = sl * (16.0 * Sh::NV + 2.0 * Sh::REM + 4.0) + (double)ctx->P.n * 4.0 * 6.0;
    return ASTRO_OK;
}

extern "C" int astro_precond_time_hop(astro_ctx *ctx, int32_t reps, double *us_per_hop, double *bytes_per_hop) {
    if (!ctx || reps < 1 || !us_per_hop || !bytes_per_hop) return ASTRO_ERR_ARG;
    GmresWork *W = static_cast<GmresWork *>(ctx->solveWork[2]);
    if (!W || !W->Kh.p) return set_err(ctx, ASTRO_ERR_STATE, "no learned solve has run on this context");
    return ctx->P.dpn == 3 ? time_hop<3>(ctx, *W, reps, us_per_hop, bytes_per_hop)
                           : time_hop<6>(ctx, *W, reps, us_per_hop, bytes_per_hop);
}

int krylov_op64(astro_ctx *ctx, Op<double> *op) {
    if (!ctx->haveK64) return set_err(ctx, ASTRO_ERR_STATE, "FP64 stiffness not assembled");
    int rc = ASTRO_OK;
    const double *Kp = ell_of<double>(ctx, &rc);
    if (!rc) *op = make_op<double>(ctx, Kp);
    return rc;
}

int krylov_op32(astro_ctx *ctx, Op<float> *op) {
    if (!ctx->haveK32) return set_err(ctx, ASTRO_ERR_STATE, "FP32 stiffness not assembled");
    int rc = ASTRO_OK;
    const float *Kp = ell_of<float>(ctx, &rc);
    if (!rc) *op = make_op<float>(ctx, Kp);
    return rc;
}

int krylov_dinv(astro_ctx *ctx, int kind, double *d_dinv) {
    const unsigned grid = (ctx->P.N + 255) / 256;
    cudaStream_t s = ctx->stream;
    const int *pp = ctx->penRows ? dptr<int>(ctx->d_penPtr) : nullptr;
    if (kind == 64) {
        if (!ctx->haveK64) return set_err(ctx, ASTRO_ERR_STATE, "FP64 stiffness not assembled");
        k_dinv<double, double><<<grid, 256, 0, s>>>(dptr<double>(ctx->d_K64), dptr<int>(ctx->d_bRowPtr),
                                                    dptr<int>(ctx->d_bCol), ctx->P.N, ctx->P.dpn, pp,
                                                    dptr<int>(ctx->d_penRow), dptr<int>(ctx->d_penCol),
                                                    dptr<double>(ctx->d_penVal), d_dinv, d_dinv);
    } else {
        if (!ctx->haveK32) return set_err(ctx, ASTRO_ERR_STATE, "FP32 stiffness not assembled");
        k_dinv<float, double><<<grid, 256, 0, s>>>(dptr<float>(ctx->d_K32), dptr<int>(ctx->d_bRowPtr),
                                                   dptr<int>(ctx->d_bCol), ctx->P.N, ctx->P.dpn, pp,
                                                   dptr<int>(ctx->d_penRow), dptr<int>(ctx->d_penCol),
                                                   dptr<double>(ctx->d_penVal), d_dinv, d_dinv);
    }
    return cuda_check(ctx, cudaGetLastError(), "dinv");
}

int krylov_power_lambda(astro_ctx *ctx, int kind, double *lam) {
    if (kind != 64 && kind != 32) return set_err(ctx, ASTRO_ERR_ARG, "kind must be 64 or 32");
    DevBuf dv;
    int rc = dev_alloc(ctx, dv, sizeof(double) * ctx->P.n);
    if (!rc) rc = krylov_dinv(ctx, kind, dptr<double>(dv));
    if (!rc) {
        // the iteration runs in FP64 vectors over either matrix
        if (kind == 64) {
            Op<double> op;
            if (!(rc = krylov_op64(ctx, &op)))
                rc = ctx->P.dpn == 3 ? power_lambda<Op<double>, double, 3>(ctx, op, dptr<double>(dv), lam)
                                     : power_lambda<Op<double>, double, 6>(ctx, op, dptr<double>(dv), lam);
        } else {
            Op<float> op;
            if (!(rc = krylov_op32(ctx, &op)))
                rc = ctx->P.dpn == 3 ? power_lambda<Op<float>, double, 3>(ctx, op, dptr<double>(dv), lam)
                                     : power_lambda<Op<float>, double, 6>(ctx, op, dptr<double>(dv), lam);
        }
    }
    dev_free(dv);
    return rc;
}

// y = (K + C^T C) x for device vectors (internal layout).
int krylov_apply(astro_ctx *ctx, int kind, const double *d_x, double *d_y) {
    GmresWork W;
    W.n = ctx->P.n;
    W.nRowCtas = (ctx->P.N + kThreads - 1) / kThreads;
    int rc = dev_alloc(ctx, W.part, sizeof(double) * 2 * W.nRowCtas);
    if (rc) return rc;
    DevBuf zb;
    if ((rc = dev_alloc(ctx, zb, sizeof(double) * ctx->P.n))) return rc;
    CK(cudaMemsetAsync(zb.p, 0, sizeof(double) * ctx->P.n, ctx->stream));
    double rel;
    if (ctx->P.dpn == 3) rc = true_residual<3>(ctx, W, kind, d_x, dptr<double>(zb), &rel, d_y);
    else rc = true_residual<6>(ctx, W, kind, d_x, dptr<double>(zb), &rel, d_y);
    dev_free(zb);
    dev_free(W.part);
    return rc;
}

// r = b - A x with A the FP64 operator (K64 and the scaled constraints), device vectors in the
// solver ordering; r may alias b.
int krylov_residual64(astro_ctx *ctx, const double *d_x, const double *d_b, double *d_r) {
    GmresWork W;
    W.n = ctx->P.n;
    W.nRowCtas = (ctx->P.N + kThreads - 1) / kThreads;
    int rc = dev_alloc(ctx, W.part, sizeof(double) * 2 * W.nRowCtas);
    if (rc) return rc;
    double rel;
    if (ctx->P.dpn == 3) rc = true_residual<3>(ctx, W, 64, d_x, d_b, &rel, d_r);
    else rc = true_residual<6>(ctx, W, 64, d_x, d_b, &rel, d_r);
    dev_free(W.part);
    return rc;
}

// ---- implicit Newmark time stepping (solve, dynamic branch) --------------------------------------

namespace {

__global__ void k_axpy(int n, double a, const double *__restrict__ x, double *__restrict__ y) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] += a * x[i];
}

// acc = c1 (c2 (u - u_p - dt v_p) - (1 - 2 beta) a_p), vel = v_p + dt ((1 - gamma) a_p + gamma acc),
// then the previous state takes the new one (Working/AStrO_commandFunctions.f90:798-809)
__global__ void k_newmark_update(int n, double c1, double c2, double dt, double beta, double gamma,
                                 const double *__restrict__ u, double *__restrict__ up, double *__restrict__ vp,
                                 double *__restrict__ ap) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double acc = c1 * (c2 * (u[i] - up[i] - dt * vp[i]) - (1.0 - 2.0 * beta) * ap[i]);
    const double vel = vp[i] + dt * ((1.0 - gamma) * ap[i] + gamma * acc);
    up[i] = u[i];
    vp[i] = vel;
    ap[i] = acc;
}

}  // namespace

// Time loop on the device.  K_eff = K + c1 c2 M is assembled and the constraints scaled before the
// call; every step forms the residual with the Newmark inertia at the current state, adds the
// applied load amp[step] * pattern and the constraint load, condenses the internal DOF, solves
// K_eff du = r by FP64 Jacobi-GMRES warm-started from the previous increment (as the reference's
// gMRes), recovers the internal DOF, updates u and the Newmark state.  All vectors are device
// buffers in internal layout; the displacement, velocity, acceleration and internal DOF of every
// step can be written to the histories (reference numbering).
template <int DPN>
static int krylov_newmark_dpn(astro_ctx *ctx, const astro_newmark_opts *o, const double *d_pattern,
                              const double *h_amp, double *d_u, double *d_up, double *d_vp, double *d_ap, double *d_iu,
                              double *d_iup, const NewmarkHist &H, astro_solve_stats *st) {
    const AstroPrep &P = ctx->P;
    const int n = P.n, ni = P.intVecSize;
    const int m = o->restart > 0 ? std::min(o->restart, kMaxM) : 50;
    const int maxCycles = o->max_iters > 0 ? (o->max_iters + m - 1) / m : 200;
    const double rtol = o->rtol > 0 ? o->rtol : 1e-10;
    const double beta = o->nm_beta, gamma = o->nm_gamma, dt = o->del_t;
    const double c1 = 0.5 / beta, c2 = 2.0 / (dt * dt);
    GmresWork W;
    DevBuf load, iload, du;
    int rc = work_alloc(ctx, W, m, sizeof(double));
    if (!rc) rc = dev_alloc(ctx, load, sizeof(double) * n);
    if (!rc) rc = dev_alloc(ctx, du, sizeof(double) * n);
    if (!rc && ni) rc = dev_alloc(ctx, iload, sizeof(double) * ni);
    const double *K = rc ? nullptr : ell_of<double>(ctx, &rc);
    cudaStream_t s = ctx->stream;
    int iters = 0, cycles = 0, refs = 0, worst = ASTRO_OK;
    double worstRel = 0.0;
    if (o->method != ASTRO_SOLVER_GMRES_JACOBI_FP64 && o->method != ASTRO_SOLVER_FGMRES_MIXED &&
        o->method != ASTRO_SOLVER_FGMRES_LEARNED)
        return set_err(ctx, ASTRO_ERR_ARG, "unknown solver method");
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, s);
    if (!rc) {
        k_dinv<double, double><<<(P.N + 255) / 256, 256, 0, s>>>(
            dptr<double>(ctx->d_K64), dptr<int>(ctx->d_bRowPtr), dptr<int>(ctx->d_bCol), P.N, P.dpn,
            ctx->penRows ? dptr<int>(ctx->d_penPtr) : nullptr, dptr<int>(ctx->d_penRow), dptr<int>(ctx->d_penCol),
            dptr<double>(ctx->d_penVal), dptr<double>(W.dinv), dptr<double>(W.dinvT));
        rc = cuda_check(ctx, cudaMemsetAsync(du.p, 0, sizeof(double) * n, s), "newmark init");
    }
    ElemDevState ds;
    ds.disp = d_u;
    ds.pdisp = d_up;
    ds.pvel = d_vp;
    ds.pacc = d_ap;
    ds.idisp = d_iu;
    ds.pidisp = d_iup;
    ds.dynamic = 1;
    ds.beta = beta;
    ds.gamma = gamma;
    ds.delT = dt;
    const int grid = (n + 255) / 256;
    for (int step = 0; step < o->num_steps && !rc; ++step) {
        CK(cudaMemsetAsync(load.p, 0, sizeof(double) * n, s));
        if (ni) CK(cudaMemsetAsync(iload.p, 0, sizeof(double) * ni, s));
        // getElasticSolnLoad(0): load -= Ru (with the Newmark inertia at the current state)
        if ((rc = elem_soln_load_dev(ctx, ds, dptr<double>(load), ni ? dptr<double>(iload) : nullptr, 0, false)))
            break;
        if (d_pattern && h_amp) k_axpy<<<grid, 256, 0, s>>>(n, h_amp[step], d_pattern, dptr<double>(load));
        if ((rc = constraint_load_dev(ctx, d_u, dptr<double>(load)))) break;
        if (ni && (rc = elem_update_external_rhs(ctx, dptr<double>(iload), dptr<double>(load)))) break;
        if (o->method != ASTRO_SOLVER_GMRES_JACOBI_FP64) {
            // the mixed or learned static solver on K_eff (its workspace, FP16 operator and
            // eigenvalue estimate are reused across the steps), warm-started from the last increment
            astro_solve_opts so{};
            so.method = o->method;
            so.restart = m;
            so.max_iters = o->max_iters > 0 ? o->max_iters : 200000;
            so.rtol = rtol;
            so.inner_rtol = 1e-4;
            so.precond = o->precond;
            astro_solve_stats s2{};
            const int grc = krylov_solve_static(ctx, dptr<double>(load), dptr<double>(du), &so, &s2);
            iters += s2.iterations;
            cycles += s2.restarts;
            refs += s2.refinements;
            if (grc == ASTRO_ERR_NAN) {
                rc = set_err(ctx, ASTRO_ERR_NAN, "non-finite value in the Newmark step solve");
                break;
            }
            if (grc != ASTRO_OK && grc != ASTRO_ERR_MAXIT) {
                rc = grc;
                break;
            }
            if (grc != ASTRO_OK) worst = grc;
            worstRel = std::max(worstRel, s2.rel_residual);
        } else {
            double rel = 0.0, rn = 0.0, bn = 0.0;
            if ((rc = true_residual<DPN>(ctx, W, 64, nullptr, dptr<double>(load), &rel, dptr<double>(W.rres), &rn, &bn)))
                break;
            double est = 0.0;
            int grc = gmres_solve<double, double, DPN>(ctx, W, K, dptr<double>(du), dptr<double>(load), rtol * bn, maxCycles,
                                                     m, &iters, &cycles, &est);
            if (grc == ASTRO_ERR_NAN) {
                rc = set_err(ctx, ASTRO_ERR_NAN, "non-finite value in the Newmark step solve");
                break;
            }
            if (grc != ASTRO_OK) worst = grc;
            if (bn > 0.0) worstRel = std::max(worstRel, est / bn);
        }
        if (ni && (rc = elem_update_internal_soln(ctx, dptr<double>(du), d_iu, dptr<double>(iload)))) break;
        k_axpy<<<grid, 256, 0, s>>>(n, 1.0, dptr<double>(du), d_u);
        k_newmark_update<<<grid, 256, 0, s>>>(n, c1, c2, dt, beta, gamma, d_u, d_up, d_vp, d_ap);
        if (ni) CK(cudaMemcpyAsync(d_iup, d_iu, sizeof(double) * ni, cudaMemcpyDeviceToDevice, s));
        if (H.disp && (rc = int_to_ref_vec(ctx, d_u, H.disp + (size_t)step * n, n))) break;
        if (H.vel && (rc = int_to_ref_vec(ctx, d_vp, H.vel + (size_t)step * n, n))) break;
        if (H.acc && (rc = int_to_ref_vec(ctx, d_ap, H.acc + (size_t)step * n, n))) break;
        if (H.intDisp && ni)
            CK(cudaMemcpyAsync(H.intDisp + (size_t)step * ni, d_iu, sizeof(double) * ni, cudaMemcpyDeviceToDevice, s));
        if ((rc = cuda_check(ctx, cudaGetLastError(), "newmark step"))) break;
    }
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    work_free(W);
    dev_free(load);
    dev_free(iload);
    dev_free(du);
    if (st) {
        st->iterations = iters;
        st->restarts = cycles;
        st->refinements = refs;
        st->status = rc ? rc : worst;
        st->rel_residual = worstRel;
        st->seconds = ms * 1e-3;
        st->conditional_graph = W.condOk ? 1 : 0;
        st->residual_kind = 64;
    }
    return rc;
}

int krylov_newmark(astro_ctx *ctx, const astro_newmark_opts *o, const double *d_pattern, const double *h_amp,
                   double *d_u, double *d_up, double *d_vp, double *d_ap, double *d_iu, double *d_iup,
                   const NewmarkHist &hist, astro_solve_stats *st) {
    if (ctx->P.dpn == 3)
        return krylov_newmark_dpn<3>(ctx, o, d_pattern, h_amp, d_u, d_up, d_vp, d_ap, d_iu, d_iup, hist, st);
    return krylov_newmark_dpn<6>(ctx, o, d_pattern, h_amp, d_u, d_up, d_vp, d_ap, d_iu, d_iup, hist, st);
}
