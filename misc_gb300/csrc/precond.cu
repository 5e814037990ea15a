// Polynomial graph-convolution preconditioner of the learned solver: initialisation, eigenvalue
// estimate and training on the device.
//
// The network maps a residual v to P v = (1/lambda) sum_k W_k y_k with the hop features
// y_k = T_k(xi(D^-1 A)) D^-1 v (Chebyshev recurrence, one SpMV per hop) and one dpn x dpn weight
// W_k per hop shared by all nodes.  Training minimises the mean over sample vectors of
// ||v - A P v||^2, which is quadratic in the weights: the features of every sample are computed
// once, and each training step costs one residual pass (A z), one gradient pass (A e and the
// per-node outer products of A e with the features) and one line-search pass (A z(D)).  All of
// it runs in FP64 over the FP64 block-ELL operator; the per-CTA partial sums are reduced on the
// host in a fixed order, so the loss, the gradient and the trained weights are reproducible.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "astro_internal.h"
#include "krylov_ops.cuh"

using namespace astro_kry;

namespace {

constexpr int kT = 256;
constexpr int kTW = kT / 32;

// Y (sample s, hop k) = Y + (s * deg1 + k) * n.  y_0 = D^-1 v.
__global__ void k_tr_y0(const double *__restrict__ v, const double *__restrict__ dinv, double *__restrict__ Y, int n,
                        int deg1) {
    const int s = blockIdx.y;
    const int i = blockIdx.x * kT + threadIdx.x;
    if (i < n) Y[(size_t)s * deg1 * n + i] = dinv[i] * v[(size_t)s * n + i];
}

// y_{k+1} = c (D^-1 A y_k - theta y_k) - [k > 0] y_{k-1}, one thread per block row
template <int DPN>
__global__ void k_tr_hop(Op<double> op, const double *__restrict__ dinv, double *__restrict__ Y, int n, int deg1, int k,
                         double theta, double c) {
    const int s = blockIdx.y;
    const int r = blockIdx.x * kT + threadIdx.x;
    if (r >= op.N) return;
    double *Ys = Y + (size_t)s * deg1 * n;
    const double *yk = Ys + (size_t)k * n;
    double t[DPN];
    ell_row<double, double, double, DPN>(op, r, yk, t);
#pragma unroll
    for (int q = 0; q < DPN; ++q) {
        const size_t i = (size_t)r * DPN + q;
        double y = c * (dinv[i] * t[q] - theta * yk[i]);
        if (k > 0) y -= Ys[(size_t)(k - 1) * n + i];
        Ys[(size_t)(k + 1) * n + i] = y;
    }
}

// z_s = sum_k Wl_k y_k per node (Wl = W / lambda in device memory)
template <int DPN>
__global__ void k_tr_apply(const double *__restrict__ Y, const double *__restrict__ Wl, double *__restrict__ Z, int n,
                           int N, int deg1) {
    const int s = blockIdx.y;
    const int r = blockIdx.x * kT + threadIdx.x;
    if (r >= N) return;
    const double *Ys = Y + (size_t)s * deg1 * n;
    double z[DPN];
#pragma unroll
    for (int q = 0; q < DPN; ++q) z[q] = 0.0;
    for (int k = 0; k < deg1; ++k) {
        double y[DPN];
#pragma unroll
        for (int jj = 0; jj < DPN; ++jj) y[jj] = Ys[(size_t)k * n + (size_t)r * DPN + jj];
        const double *w = Wl + (size_t)k * DPN * DPN;
#pragma unroll
        for (int q = 0; q < DPN; ++q)
#pragma unroll
            for (int jj = 0; jj < DPN; ++jj) z[q] += w[q * DPN + jj] * y[jj];
    }
#pragma unroll
    for (int q = 0; q < DPN; ++q) Z[(size_t)s * n + (size_t)r * DPN + q] = z[q];
}

// sum over the CTA of v (every thread), written by thread 0 to *out
__device__ __forceinline__ void cta_sum(double v, double *out) {
    __shared__ double sp[kTW];
    v = warp_sum(v);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) sp[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0;
        for (int q = 0; q < kTW; ++q) a += sp[q];
        *out = a;
    }
}

// e_s = v_s - A z_s; part[s * gridDim.x + cta] = this CTA's share of ||e_s||^2
template <int DPN>
__global__ void k_tr_resid(Op<double> op, const double *__restrict__ v, const double *__restrict__ Z,
                           double *__restrict__ E, double *__restrict__ part, int n) {
    const int s = blockIdx.y;
    const int r = blockIdx.x * kT + threadIdx.x;
    double ee = 0.0;
    if (r < op.N) {
        double t[DPN];
        ell_row<double, double, double, DPN>(op, r, Z + (size_t)s * n, t);
#pragma unroll
        for (int q = 0; q < DPN; ++q) {
            const size_t i = (size_t)s * n + (size_t)r * DPN + q;
            const double e = v[i] - t[q];
            E[i] = e;
            ee += e * e;
        }
    }
    cta_sum(ee, part + (size_t)s * gridDim.x + blockIdx.x);
}

// Gradient partials: with t = (A e_s)_r, this CTA's share of sum_r t_i (y_k)_{r,j} for every
// (k, i, j), at part[((s * gridDim.x + cta) * deg1 + k) * DPN * DPN + i * DPN + j].  Each warp
// reduces its lanes' products; the CTA then adds its warps' sums.
template <int DPN>
__global__ void __launch_bounds__(kT) k_tr_grad(Op<double> op, const double *__restrict__ E, const double *__restrict__ Y,
                                                double *__restrict__ part, int n, int deg1) {
    constexpr int DD = DPN * DPN;
    extern __shared__ double sw[];  // [kTW][deg1 * DD]
    const int s = blockIdx.y;
    const int r = blockIdx.x * kT + threadIdx.x;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const bool valid = r < op.N;
    double t[DPN];
    if (valid) {
        ell_row<double, double, double, DPN>(op, r, E + (size_t)s * n, t);
    } else {
#pragma unroll
        for (int q = 0; q < DPN; ++q) t[q] = 0.0;
    }
    const double *Ys = Y + (size_t)s * deg1 * n;
    for (int k = 0; k < deg1; ++k) {
        double y[DPN];
#pragma unroll
        for (int jj = 0; jj < DPN; ++jj) y[jj] = valid ? Ys[(size_t)k * n + (size_t)r * DPN + jj] : 0.0;
#pragma unroll
        for (int q = 0; q < DPN; ++q)
#pragma unroll
            for (int jj = 0; jj < DPN; ++jj) {
                const double g = warp_sum(t[q] * y[jj]);
                if (lane == 0) sw[(size_t)wid * deg1 * DD + k * DD + q * DPN + jj] = g;
            }
    }
    __syncthreads();
    double *out = part + ((size_t)s * gridDim.x + blockIdx.x) * deg1 * DD;
    for (int q = threadIdx.x; q < deg1 * DD; q += kT) {
        double a = 0.0;
        for (int w = 0; w < kTW; ++w) a += sw[(size_t)w * deg1 * DD + q];
        out[q] = a;
    }
}

// Line search: q_s = A zd_s; part[(s * gridDim.x + cta) * 2 + {0, 1}] = shares of e.q and q.q
template <int DPN>
__global__ void k_tr_lsdots(Op<double> op, const double *__restrict__ ZD, const double *__restrict__ E,
                            double *__restrict__ part, int n) {
    const int s = blockIdx.y;
    const int r = blockIdx.x * kT + threadIdx.x;
    double eq = 0.0, qq = 0.0;
    if (r < op.N) {
        double t[DPN];
        ell_row<double, double, double, DPN>(op, r, ZD + (size_t)s * n, t);
#pragma unroll
        for (int q = 0; q < DPN; ++q) {
            const double e = E[(size_t)s * n + (size_t)r * DPN + q];
            eq += e * t[q];
            qq += t[q] * t[q];
        }
    }
    double *out = part + ((size_t)s * gridDim.x + blockIdx.x) * 2;
    cta_sum(eq, out);
    cta_sum(qq, out + 1);
}

// ---- node features and the per-node modulation network ----------------------------------

constexpr int kF = ASTRO_NODE_FEATURES;

// l_r = ln(mean diagonal entry of the node's diagonal block), the node's penalty diagonal mean
// p_r, and the CTA's share of sum_r l_r
template <class TM, int DPN>
__global__ void k_nf_diag(int N, const int *__restrict__ bRowPtr, const int *__restrict__ bCol,
                          const TM *__restrict__ K, const int *__restrict__ penPtr, const int *__restrict__ penRow,
                          const int *__restrict__ penCol, const double *__restrict__ penVal, double *__restrict__ L,
                          double *__restrict__ pd, double *__restrict__ part) {
    const int r = blockIdx.x * kT + threadIdx.x;
    double l = 0.0;
    if (r < N) {
        double d = 0.0;
        for (int b = bRowPtr[r]; b < bRowPtr[r + 1]; ++b)
            if (bCol[b] == r) {
#pragma unroll
                for (int i = 0; i < DPN; ++i) d += (double)K[(size_t)b * DPN * DPN + i * DPN + i];
            }
        double p = 0.0;
        if (penPtr)
            for (int t = penPtr[r]; t < penPtr[r + 1]; ++t)
                if (penCol[t] == r * DPN + penRow[t]) p += penVal[t];
        d /= DPN;
        l = log(fmax(fabs(d), 1e-300));
        L[r] = l;
        pd[r] = p / DPN;
    }
    cta_sum(l, part + blockIdx.x);
}

// features of every node (row-major N x kF, internal block-row order); part holds nParts CTA
// shares of sum_r l_r
template <class TM, int DPN>
__global__ void k_nf_feat(int N, int maxBlocks, const int *__restrict__ bRowPtr, const int *__restrict__ bCol,
                          const TM *__restrict__ K, const double *__restrict__ L, const double *__restrict__ pd,
                          const double *__restrict__ part, int nParts, double *__restrict__ F) {
    __shared__ double sMean;
    if (threadIdx.x == 0) {
        double a = 0.0;
        for (int q = 0; q < nParts; ++q) a += part[q];
        sMean = a / N;
    }
    __syncthreads();
    const int r = blockIdx.x * kT + threadIdx.x;
    if (r >= N) return;
    const double lr = L[r];
    double sum = 0.0, mx = 0.0, off = 0.0, dia = 0.0;
    int nb = 0;
    for (int b = bRowPtr[r]; b < bRowPtr[r + 1]; ++b) {
        const int c = bCol[b];
        double fro = 0.0;
#pragma unroll
        for (int q = 0; q < DPN * DPN; ++q) {
            const double v = (double)K[(size_t)b * DPN * DPN + q];
            fro += v * v;
        }
        fro = sqrt(fro);
        if (c == r) {
            dia = fro;
        } else {
            const double dl = L[c] - lr;
            sum += dl;
            mx = fmax(mx, fabs(dl));
            off += fro;
            ++nb;
        }
    }
    const double d = exp(lr);
    double *f = F + (size_t)r * kF;
    f[0] = lr - sMean;
    f[1] = nb ? sum / nb : 0.0;
    f[2] = mx;
    f[3] = (double)(nb + 1) / maxBlocks;
    f[4] = log1p(pd[r] / d);
    f[5] = (dia > 0.0 && off > 0.0) ? log(off / dia) : 0.0;
}

// MLP parameters packed on the device: w1 (H x kF), b1 (H), w2 (K x H), b2 (K)
struct MlpDims {
    int H, K;
};

// a_k(r) = 1 + b2[k] + sum_h w2[k][h] tanh(b1[h] + w1[h] . f(r)); a at A[k * N + r], the hidden
// activations (when hid) at hid[r * H + h]
template <class TA>
__global__ void k_mlp_fwd(int N, MlpDims D, const double *__restrict__ F, const double *__restrict__ prm,
                          TA *__restrict__ A, double *__restrict__ hid) {
    const int r = blockIdx.x * kT + threadIdx.x;
    if (r >= N) return;
    const double *w1 = prm, *b1 = w1 + D.H * kF, *w2 = b1 + D.H, *b2 = w2 + D.K * D.H;
    double f[kF], h[ASTRO_MLP_MAX_HIDDEN];
#pragma unroll
    for (int q = 0; q < kF; ++q) f[q] = F[(size_t)r * kF + q];
    for (int j = 0; j < D.H; ++j) {
        double a = b1[j];
#pragma unroll
        for (int q = 0; q < kF; ++q) a += w1[j * kF + q] * f[q];
        h[j] = tanh(a);
        if (hid) hid[(size_t)r * D.H + j] = h[j];
    }
    for (int k = 0; k < D.K; ++k) {
        double o = 1.0 + b2[k];
        for (int j = 0; j < D.H; ++j) o += w2[k * D.H + j] * h[j];
        A[(size_t)k * N + r] = (TA)o;
    }
}

// z_s = sum_k a_k(r) (Wl_k y_k) per node
template <int DPN>
__global__ void k_tr_apply_mod(const double *__restrict__ Y, const double *__restrict__ Wl,
                               const double *__restrict__ amod, double *__restrict__ Z, int n, int N, int deg1) {
    const int s = blockIdx.y;
    const int r = blockIdx.x * kT + threadIdx.x;
    if (r >= N) return;
    const double *Ys = Y + (size_t)s * deg1 * n;
    double z[DPN];
#pragma unroll
    for (int q = 0; q < DPN; ++q) z[q] = 0.0;
    for (int k = 0; k < deg1; ++k) {
        const double a = amod[(size_t)k * N + r];
        const double *w = Wl + (size_t)k * DPN * DPN;
#pragma unroll
        for (int q = 0; q < DPN; ++q) {
            double t = 0.0;
#pragma unroll
            for (int jj = 0; jj < DPN; ++jj) t += w[q * DPN + jj] * Ys[(size_t)k * n + (size_t)r * DPN + jj];
            z[q] += a * t;
        }
    }
#pragma unroll
    for (int q = 0; q < DPN; ++q) Z[(size_t)s * n + (size_t)r * DPN + q] = z[q];
}

// Gradient partials of the modulated network, all samples in one pass per CTA (deterministic):
// with t = (A e_s)_r,
//   part[cta * deg1 * DD + k * DD + i * DPN + j] = sum_s sum_{r in cta} a_k(r) t_i (y_k)_{r,j}
//   ga[k * N + r] = sum_s sum_i t_i (Wl_k y_k)_{r,i}
template <int DPN>
__global__ void __launch_bounds__(kT) k_tr_grad_mod(Op<double> op, const double *__restrict__ E,
                                                    const double *__restrict__ Y, const double *__restrict__ Wl,
                                                    const double *__restrict__ amod, double *__restrict__ part,
                                                    double *__restrict__ ga, int n, int deg1, int S) {
    constexpr int DD = DPN * DPN;
    extern __shared__ double sw[];  // [kTW][deg1 * DD]
    const int r = blockIdx.x * kT + threadIdx.x;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const bool valid = r < op.N;
    const int N = op.N;
    for (int q = threadIdx.x; q < kTW * deg1 * DD; q += kT) sw[q] = 0.0;
    __syncthreads();
    for (int s = 0; s < S; ++s) {
        double t[DPN];
        if (valid) {
            ell_row<double, double, double, DPN>(op, r, E + (size_t)s * n, t);
        } else {
#pragma unroll
            for (int q = 0; q < DPN; ++q) t[q] = 0.0;
        }
        const double *Ys = Y + (size_t)s * deg1 * n;
        for (int k = 0; k < deg1; ++k) {
            double y[DPN];
#pragma unroll
            for (int jj = 0; jj < DPN; ++jj) y[jj] = valid ? Ys[(size_t)k * n + (size_t)r * DPN + jj] : 0.0;
            const double a = valid ? amod[(size_t)k * N + r] : 0.0;
            const double *w = Wl + (size_t)k * DD;
            double g = 0.0;
#pragma unroll
            for (int q = 0; q < DPN; ++q) {
                double wy = 0.0;
#pragma unroll
                for (int jj = 0; jj < DPN; ++jj) wy += w[q * DPN + jj] * y[jj];
                g += t[q] * wy;
            }
            if (valid) ga[(size_t)k * N + r] = (s == 0 ? 0.0 : ga[(size_t)k * N + r]) + g;
#pragma unroll
            for (int q = 0; q < DPN; ++q)
#pragma unroll
                for (int jj = 0; jj < DPN; ++jj) {
                    const double v = warp_sum(a * t[q] * y[jj]);
                    if (lane == 0) sw[(size_t)wid * deg1 * DD + k * DD + q * DPN + jj] += v;
                }
        }
    }
    __syncthreads();
    double *out = part + (size_t)blockIdx.x * deg1 * DD;
    for (int q = threadIdx.x; q < deg1 * DD; q += kT) {
        double acc = 0.0;
        for (int w = 0; w < kTW; ++w) acc += sw[(size_t)w * deg1 * DD + q];
        out[q] = acc;
    }
}

// Backward pass of the perceptron: with go_k(r) = scale * ga[k * N + r] = dL/da_k(r), this CTA's
// shares of the gradients in the packed parameter layout (part[cta * P + p], P = H kF + H + K H + K)
__global__ void __launch_bounds__(kT) k_mlp_bwd(int N, MlpDims D, const double *__restrict__ F,
                                                const double *__restrict__ hid, const double *__restrict__ ga,
                                                double scale, const double *__restrict__ prm,
                                                double *__restrict__ part) {
    __shared__ double sp[kTW];
    const int r = blockIdx.x * kT + threadIdx.x;
    const bool valid = r < N;
    const int H = D.H, K = D.K;
    const double *w2 = prm + H * kF + H;
    double f[kF], h[ASTRO_MLP_MAX_HIDDEN], gp[ASTRO_MLP_MAX_HIDDEN];
#pragma unroll
    for (int q = 0; q < kF; ++q) f[q] = valid ? F[(size_t)r * kF + q] : 0.0;
    for (int j = 0; j < H; ++j) {
        h[j] = valid ? hid[(size_t)r * H + j] : 0.0;
        double gh = 0.0;
        for (int k = 0; k < K; ++k) gh += w2[k * H + j] * (valid ? scale * ga[(size_t)k * N + r] : 0.0);
        gp[j] = gh * (1.0 - h[j] * h[j]);
    }
    const int P = H * kF + H + K * H + K;
    double *out = part + (size_t)blockIdx.x * P;
    for (int p = 0; p < P; ++p) {
        double v;
        if (p < H * kF) {
            v = gp[p / kF] * f[p % kF];
        } else if (p < H * kF + H) {
            v = gp[p - H * kF];
        } else if (p < H * kF + H + K * H) {
            const int q = p - H * kF - H, k = q / H, j = q % H;
            v = (valid ? scale * ga[(size_t)k * N + r] : 0.0) * h[j];
        } else {
            const int k = p - H * kF - H - K * H;
            v = valid ? scale * ga[(size_t)k * N + r] : 0.0;
        }
        v = warp_sum(v);
        __syncthreads();
        if ((threadIdx.x & 31) == 0) sp[threadIdx.x >> 5] = v;
        __syncthreads();
        if (threadIdx.x == 0) {
            double a = 0.0;
            for (int q = 0; q < kTW; ++q) a += sp[q];
            out[p] = a;
        }
    }
}

void mlp_pack(const astro_precond_mlp *m, int K, std::vector<double> &out) {
    const int H = m->hidden;
    out.clear();
    out.insert(out.end(), m->w1, m->w1 + H * kF);
    out.insert(out.end(), m->b1, m->b1 + H);
    out.insert(out.end(), m->w2, m->w2 + K * H);
    out.insert(out.end(), m->b2, m->b2 + K);
}

void mlp_unpack(const double *g, int H, int K, astro_precond_mlp *m) {
    std::memset(m, 0, sizeof(*m));
    m->hidden = H;
    m->outputs = K;
    std::memcpy(m->w1, g, sizeof(double) * H * kF);
    std::memcpy(m->b1, g + H * kF, sizeof(double) * H);
    std::memcpy(m->w2, g + H * kF + H, sizeof(double) * K * H);
    std::memcpy(m->b2, g + H * kF + H + K * H, sizeof(double) * K);
}

}  // namespace

// Node features (internal block-row order, N x kF) of the FP64 (kind 64) or FP32 (kind 32)
// assembly with the scaled constraints; L, pd, part: scratch (allocated on first use).
int precond_node_features(astro_ctx *ctx, int kind, double *dF, DevBuf &L, DevBuf &pd, DevBuf &part, cudaStream_t s) {
    const AstroPrep &P = ctx->P;
    const int N = P.N, nCta = (N + kT - 1) / kT;
    if (kind == 64 ? !ctx->haveK64 : !(ctx->haveK32 || ctx->haveK64))
        return set_err(ctx, ASTRO_ERR_STATE, "node features: stiffness not assembled");
    int rc;
    if (!L.p && ((rc = dev_alloc(ctx, L, sizeof(double) * N)) || (rc = dev_alloc(ctx, pd, sizeof(double) * N)) ||
                 (rc = dev_alloc(ctx, part, sizeof(double) * nCta))))
        return rc;
    int maxB = 1;
    for (int r = 0; r < N; ++r) maxB = std::max(maxB, P.bRowPtr[r + 1] - P.bRowPtr[r]);
    const bool f64 = kind == 64 || !ctx->haveK32;
    const int *pp = ctx->penRows ? dptr<int>(ctx->d_penPtr) : nullptr;
    const int *br = dptr<int>(ctx->d_bRowPtr), *bc = dptr<int>(ctx->d_bCol);
    const int *prow = dptr<int>(ctx->d_penRow), *pcol = dptr<int>(ctx->d_penCol);
    const double *pval = dptr<double>(ctx->d_penVal);
    double *dl = dptr<double>(L), *dp = dptr<double>(pd), *dq = dptr<double>(part);
    if (f64) {
        const double *K = dptr<double>(ctx->d_K64);
        if (P.dpn == 3) {
            k_nf_diag<double, 3><<<nCta, kT, 0, s>>>(N, br, bc, K, pp, prow, pcol, pval, dl, dp, dq);
            k_nf_feat<double, 3><<<nCta, kT, 0, s>>>(N, maxB, br, bc, K, dl, dp, dq, nCta, dF);
        } else {
            k_nf_diag<double, 6><<<nCta, kT, 0, s>>>(N, br, bc, K, pp, prow, pcol, pval, dl, dp, dq);
            k_nf_feat<double, 6><<<nCta, kT, 0, s>>>(N, maxB, br, bc, K, dl, dp, dq, nCta, dF);
        }
    } else {
        const float *K = dptr<float>(ctx->d_K32);
        if (P.dpn == 3) {
            k_nf_diag<float, 3><<<nCta, kT, 0, s>>>(N, br, bc, K, pp, prow, pcol, pval, dl, dp, dq);
            k_nf_feat<float, 3><<<nCta, kT, 0, s>>>(N, maxB, br, bc, K, dl, dp, dq, nCta, dF);
        } else {
            k_nf_diag<float, 6><<<nCta, kT, 0, s>>>(N, br, bc, K, pp, prow, pcol, pval, dl, dp, dq);
            k_nf_feat<float, 6><<<nCta, kT, 0, s>>>(N, maxB, br, bc, K, dl, dp, dq, nCta, dF);
        }
    }
    return cuda_check(ctx, cudaGetLastError(), "node features");
}

int precond_mlp_check(astro_ctx *ctx, const astro_precond_mlp *m, int degree) {
    if (m->hidden < 0 || m->hidden > ASTRO_MLP_MAX_HIDDEN)
        return set_err(ctx, ASTRO_ERR_ARG, "perceptron hidden width out of range");
    if (m->outputs != degree + 1) return set_err(ctx, ASTRO_ERR_ARG, "perceptron outputs differ from degree + 1");
    return ASTRO_OK;
}

// the per-node scales a (float, K x N) of the perceptron on the features dF (N x kF, internal
// order); prm: packed parameters (allocated for the largest network on first use)
int precond_mlp_scales_f32(astro_ctx *ctx, const astro_precond_mlp *m, const double *dF, DevBuf &prm, float *a,
                           cudaStream_t s) {
    const int H = m->hidden, K = m->outputs;
    int rc;
    const size_t maxP = (size_t)ASTRO_MLP_MAX_HIDDEN * (kF + 1) +
                        (size_t)(ASTRO_PRECOND_MAX_DEGREE + 1) * (ASTRO_MLP_MAX_HIDDEN + 1);
    if (!prm.p && (rc = dev_alloc(ctx, prm, sizeof(double) * maxP))) return rc;
    std::vector<double> pk;
    mlp_pack(m, K, pk);
    if ((rc = cuda_check(ctx, cudaMemcpyAsync(prm.p, pk.data(), sizeof(double) * pk.size(), cudaMemcpyHostToDevice, s),
                         "mlp upload")))
        return rc;
    const int N = ctx->P.N;
    k_mlp_fwd<float><<<(N + kT - 1) / kT, kT, 0, s>>>(N, MlpDims{H, K}, dF, dptr<double>(prm), a, nullptr);
    if ((rc = cuda_check(ctx, cudaGetLastError(), "perceptron forward"))) return rc;
    return cuda_check(ctx, cudaStreamSynchronize(s), "perceptron forward");  // pk goes out of scope
}

namespace {

// Device state of a training run: samples, features and work vectors for S samples.
struct TrainSet {
    astro_ctx *ctx = nullptr;
    Op<double> op;
    int S = 0, deg = 0, deg1 = 0, dpn = 0, n = 0, N = 0, nCta = 0;
    double lam = 0.0, theta = 0.0, delta = 0.0;
    DevBuf v, dinv, Y, Z, E, part, Wl;
    // the modulation network: node features, hidden activations, scales a, dL/da, parameters
    DevBuf F, hid, amod, ga, prm, nfL, nfPd, nfPart, mpart;
    std::vector<double> hp;

    ~TrainSet() {
        DevBuf *b[] = {&v, &dinv, &Y, &Z, &E, &part, &Wl, &F, &hid, &amod, &ga, &prm, &nfL, &nfPd, &nfPart, &mpart};
        for (auto *x : b) dev_free(*x);
    }

    int sync(const char *what) { return cuda_check(ctx, cudaStreamSynchronize(ctx->stream), what); }

    // uploads the normalised samples, estimates lambda and computes the features
    int setup(astro_ctx *c, const astro_precond *p, const double *samples, int numSamples) {
        ctx = c;
        S = numSamples;
        deg = p->degree;
        deg1 = deg + 1;
        dpn = ctx->P.dpn;
        n = ctx->P.n;
        N = ctx->P.N;
        nCta = (N + kT - 1) / kT;
        int rc;
        if ((rc = krylov_op64(ctx, &op))) return rc;
        if ((rc = krylov_power_lambda(ctx, 64, &lam))) return rc;
        lam *= p->lambda_scale;
        theta = 0.5 * lam * (1.0 + 1.0 / p->ratio);
        delta = 0.5 * lam * (1.0 - 1.0 / p->ratio);
        const size_t sn = (size_t)S * n;
        const size_t gparts = (size_t)S * nCta * deg1 * dpn * dpn;
        if ((rc = dev_alloc(ctx, v, sizeof(double) * sn)) || (rc = dev_alloc(ctx, dinv, sizeof(double) * n)) ||
            (rc = dev_alloc(ctx, Y, sizeof(double) * sn * deg1)) || (rc = dev_alloc(ctx, Z, sizeof(double) * sn)) ||
            (rc = dev_alloc(ctx, E, sizeof(double) * sn)) ||
            (rc = dev_alloc(ctx, part, sizeof(double) * std::max(gparts, (size_t)2 * S * nCta))) ||
            (rc = dev_alloc(ctx, Wl, sizeof(double) * deg1 * dpn * dpn)))
            return rc;
        // normalise on the host, convert each sample to the internal layout on the device
        std::vector<double> hv((size_t)n);
        DevBuf tmp;
        if ((rc = dev_alloc(ctx, tmp, sizeof(double) * n))) return rc;
        for (int s = 0; s < S && !rc; ++s) {
            const double *src = samples + (size_t)s * n;
            double nn = 0.0;
            for (int i = 0; i < n; ++i) nn += src[i] * src[i];
            if (!(nn > 0.0) || !std::isfinite(nn)) {
                rc = set_err(ctx, ASTRO_ERR_ARG, "training sample is zero or not finite");
                break;
            }
            const double sc = 1.0 / std::sqrt(nn);
            for (int i = 0; i < n; ++i) hv[i] = src[i] * sc;
            cudaError_t e = cudaMemcpyAsync(tmp.p, hv.data(), sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream);
            if ((rc = cuda_check(ctx, e, "sample upload"))) break;
            if ((rc = ref_to_int_vec(ctx, dptr<double>(tmp), dptr<double>(v) + (size_t)s * n, n))) break;
            rc = sync("sample upload");  // hv is reused for the next sample
        }
        dev_free(tmp);
        if (rc) return rc;
        if ((rc = krylov_dinv(ctx, 64, dptr<double>(dinv)))) return rc;
        const dim3 gv((n + kT - 1) / kT, S), gr(nCta, S);
        k_tr_y0<<<gv, kT, 0, ctx->stream>>>(dptr<double>(v), dptr<double>(dinv), dptr<double>(Y), n, deg1);
        for (int k = 0; k < deg; ++k) {
            const double cc = (k == 0 ? 1.0 : 2.0) / delta;
            if (dpn == 3)
                k_tr_hop<3><<<gr, kT, 0, ctx->stream>>>(op, dptr<double>(dinv), dptr<double>(Y), n, deg1, k, theta, cc);
            else
                k_tr_hop<6><<<gr, kT, 0, ctx->stream>>>(op, dptr<double>(dinv), dptr<double>(Y), n, deg1, k, theta, cc);
        }
        return cuda_check(ctx, cudaGetLastError(), "training features");
    }

    // Z = sum_k (W_k / lambda) y_k for the weights w (host, deg1 * dpn * dpn)
    int apply(const double *w) {
        const int nw = deg1 * dpn * dpn;
        std::vector<double> wl(w, w + nw);
        for (auto &x : wl) x /= lam;
        cudaError_t e = cudaMemcpyAsync(Wl.p, wl.data(), sizeof(double) * nw, cudaMemcpyHostToDevice, ctx->stream);
        int rc;
        if ((rc = cuda_check(ctx, e, "weights upload"))) return rc;
        const dim3 gr(nCta, S);
        if (dpn == 3)
            k_tr_apply<3><<<gr, kT, 0, ctx->stream>>>(dptr<double>(Y), dptr<double>(Wl), dptr<double>(Z), n, N, deg1);
        else
            k_tr_apply<6><<<gr, kT, 0, ctx->stream>>>(dptr<double>(Y), dptr<double>(Wl), dptr<double>(Z), n, N, deg1);
        return sync("apply");  // wl goes out of scope
    }

    int fetch(size_t count, const DevBuf *src = nullptr) {
        hp.resize(count);
        cudaError_t e = cudaMemcpyAsync(hp.data(), (src ? *src : part).p, sizeof(double) * count,
                                        cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        return cuda_check(ctx, e, "partials");
    }

    // loss and gradient at w
    int loss_grad(const double *w, double *loss, double *grad) {
        int rc;
        if ((rc = apply(w))) return rc;
        const dim3 gr(nCta, S);
        const int dd = dpn * dpn;
        if (dpn == 3)
            k_tr_resid<3><<<gr, kT, 0, ctx->stream>>>(op, dptr<double>(v), dptr<double>(Z), dptr<double>(E), dptr<double>(part), n);
        else
            k_tr_resid<6><<<gr, kT, 0, ctx->stream>>>(op, dptr<double>(v), dptr<double>(Z), dptr<double>(E), dptr<double>(part), n);
        if ((rc = fetch((size_t)S * nCta))) return rc;
        double L = 0.0;
        for (int s = 0; s < S; ++s) {
            double a = 0.0;
            for (int q = 0; q < nCta; ++q) a += hp[(size_t)s * nCta + q];
            L += a;
        }
        *loss = L / S;
        if (!grad) return ASTRO_OK;
        const size_t smem = sizeof(double) * kTW * deg1 * dd;
        if (smem > 48 * 1024) {  // above the default dynamic shared memory limit (dpn 6, high degree)
            cudaError_t e = dpn == 3 ? cudaFuncSetAttribute(k_tr_grad<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)
                                     : cudaFuncSetAttribute(k_tr_grad<6>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if ((rc = cuda_check(ctx, e, "gradient shared memory"))) return rc;
        }
        if (dpn == 3)
            k_tr_grad<3><<<gr, kT, smem, ctx->stream>>>(op, dptr<double>(E), dptr<double>(Y), dptr<double>(part), n, deg1);
        else
            k_tr_grad<6><<<gr, kT, smem, ctx->stream>>>(op, dptr<double>(E), dptr<double>(Y), dptr<double>(part), n, deg1);
        if ((rc = cuda_check(ctx, cudaGetLastError(), "gradient"))) return rc;
        const size_t per = (size_t)deg1 * dd;
        if ((rc = fetch((size_t)S * nCta * per))) return rc;
        // dL/dW_k[i][j] = -(2 / (S lambda)) sum_s sum_r (A e_s)_{r,i} (y_k)_{r,j}
        for (size_t q = 0; q < per; ++q) {
            double a = 0.0;
            for (int s = 0; s < S; ++s)
                for (int c = 0; c < nCta; ++c) a += hp[((size_t)s * nCta + c) * per + q];
            grad[q] = -2.0 * a / (S * lam);
        }
        return ASTRO_OK;
    }

    // loss and gradients of the modulated network at (w, mlp): gw (deg1 dpn^2) and gm (packed
    // perceptron parameters), either may be null
    int loss_grad_mod(const double *w, const astro_precond_mlp *mlp, double *loss, double *gw, double *gm) {
        const int H = mlp->hidden, K = deg1, dd = dpn * dpn;
        const int P = H * kF + H + K * H + K;
        int rc;
        if (!F.p) {
            if ((rc = dev_alloc(ctx, F, sizeof(double) * (size_t)N * kF)) ||
                (rc = dev_alloc(ctx, hid, sizeof(double) * (size_t)N * std::max(H, 1))) ||
                (rc = dev_alloc(ctx, amod, sizeof(double) * (size_t)N * K)) ||
                (rc = dev_alloc(ctx, ga, sizeof(double) * (size_t)N * K)) ||
                (rc = dev_alloc(ctx, prm, sizeof(double) * (size_t)std::max(P, 1))) ||
                (rc = dev_alloc(ctx, mpart, sizeof(double) * (size_t)nCta * std::max(P, K * dd))))
                return rc;
            if ((rc = precond_node_features(ctx, 64, dptr<double>(F), nfL, nfPd, nfPart, ctx->stream))) return rc;
        }
        std::vector<double> pk;
        mlp_pack(mlp, K, pk);
        if ((rc = cuda_check(ctx, cudaMemcpyAsync(prm.p, pk.data(), sizeof(double) * P, cudaMemcpyHostToDevice,
                                                  ctx->stream), "mlp upload")))
            return rc;
        const unsigned gN = (unsigned)nCta;
        k_mlp_fwd<double><<<gN, kT, 0, ctx->stream>>>(N, MlpDims{H, K}, dptr<double>(F), dptr<double>(prm),
                                                     dptr<double>(amod), H ? dptr<double>(hid) : nullptr);
        std::vector<double> wl(w, w + (size_t)K * dd);
        for (auto &x : wl) x /= lam;
        if ((rc = cuda_check(ctx, cudaMemcpyAsync(Wl.p, wl.data(), sizeof(double) * K * dd, cudaMemcpyHostToDevice,
                                                  ctx->stream), "weights upload")))
            return rc;
        const dim3 gr(nCta, S);
        if (dpn == 3) {
            k_tr_apply_mod<3><<<gr, kT, 0, ctx->stream>>>(dptr<double>(Y), dptr<double>(Wl), dptr<double>(amod),
                                                         dptr<double>(Z), n, N, deg1);
            k_tr_resid<3><<<gr, kT, 0, ctx->stream>>>(op, dptr<double>(v), dptr<double>(Z), dptr<double>(E),
                                                     dptr<double>(part), n);
        } else {
            k_tr_apply_mod<6><<<gr, kT, 0, ctx->stream>>>(dptr<double>(Y), dptr<double>(Wl), dptr<double>(amod),
                                                         dptr<double>(Z), n, N, deg1);
            k_tr_resid<6><<<gr, kT, 0, ctx->stream>>>(op, dptr<double>(v), dptr<double>(Z), dptr<double>(E),
                                                     dptr<double>(part), n);
        }
        if ((rc = fetch((size_t)S * nCta))) return rc;  // synchronises: pk and wl may go
        double L = 0.0;
        for (int s = 0; s < S; ++s) {
            double a = 0.0;
            for (int q = 0; q < nCta; ++q) a += hp[(size_t)s * nCta + q];
            L += a;
        }
        *loss = L / S;
        if (!gw && !gm) return ASTRO_OK;
        const size_t smem = sizeof(double) * kTW * K * dd;
        if (smem > 48 * 1024) {
            cudaError_t e = dpn == 3 ? cudaFuncSetAttribute(k_tr_grad_mod<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)
                                     : cudaFuncSetAttribute(k_tr_grad_mod<6>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if ((rc = cuda_check(ctx, e, "gradient shared memory"))) return rc;
        }
        if (dpn == 3)
            k_tr_grad_mod<3><<<gN, kT, smem, ctx->stream>>>(op, dptr<double>(E), dptr<double>(Y), dptr<double>(Wl),
                                                           dptr<double>(amod), dptr<double>(mpart), dptr<double>(ga), n,
                                                           deg1, S);
        else
            k_tr_grad_mod<6><<<gN, kT, smem, ctx->stream>>>(op, dptr<double>(E), dptr<double>(Y), dptr<double>(Wl),
                                                           dptr<double>(amod), dptr<double>(mpart), dptr<double>(ga), n,
                                                           deg1, S);
        if ((rc = cuda_check(ctx, cudaGetLastError(), "modulated gradient"))) return rc;
        // dL/dz_s = -(2 / S) A e_s: the weights' gradient carries 1/lambda, dL/da does not
        // (Wl inside ga already holds it)
        if (gw) {
            if ((rc = fetch((size_t)nCta * K * dd, &mpart))) return rc;
            for (int q = 0; q < K * dd; ++q) {
                double a = 0.0;
                for (int c = 0; c < nCta; ++c) a += hp[(size_t)c * K * dd + q];
                gw[q] = -2.0 * a / (S * lam);
            }
        }
        if (gm) {
            if (H > 0) {
                k_mlp_bwd<<<gN, kT, 0, ctx->stream>>>(N, MlpDims{H, K}, dptr<double>(F), dptr<double>(hid),
                                                     dptr<double>(ga), -2.0 / S, dptr<double>(prm), dptr<double>(mpart));
                if ((rc = cuda_check(ctx, cudaGetLastError(), "perceptron backward"))) return rc;
                if ((rc = fetch((size_t)nCta * P, &mpart))) return rc;
                for (int q = 0; q < P; ++q) {
                    double a = 0.0;
                    for (int c = 0; c < nCta; ++c) a += hp[(size_t)c * P + q];
                    gm[q] = a;
                }
            } else {
                for (int q = 0; q < P; ++q) gm[q] = 0.0;
            }
        }
        return ASTRO_OK;
    }

    // exact line search along d from the residuals E of the last loss_grad: the minimiser of
    // (1/S) sum_s ||e_s + alpha A z_s(d)||^2 over alpha (W <- W - alpha d decreases the loss)
    int line_search(const double *d, double *alpha, double *qq_out) {
        int rc;
        if ((rc = apply(d))) return rc;
        const dim3 gr(nCta, S);
        if (dpn == 3)
            k_tr_lsdots<3><<<gr, kT, 0, ctx->stream>>>(op, dptr<double>(Z), dptr<double>(E), dptr<double>(part), n);
        else
            k_tr_lsdots<6><<<gr, kT, 0, ctx->stream>>>(op, dptr<double>(Z), dptr<double>(E), dptr<double>(part), n);
        if ((rc = fetch((size_t)S * nCta * 2))) return rc;
        double eq = 0.0, qq = 0.0;
        for (int s = 0; s < S; ++s)
            for (int c = 0; c < nCta; ++c) {
                eq += hp[((size_t)s * nCta + c) * 2];
                qq += hp[((size_t)s * nCta + c) * 2 + 1];
            }
        *qq_out = qq;
        *alpha = qq > 0.0 ? -eq / qq : 0.0;
        return ASTRO_OK;
    }
};

int train_check(astro_ctx *ctx, const astro_precond *p, const double *samples, int S) {
    if (!samples || S < 1) return set_err(ctx, ASTRO_ERR_ARG, "need at least one training sample");
    if (!ctx->haveK64) return set_err(ctx, ASTRO_ERR_STATE, "training needs the FP64 stiffness (astro_el_soln_load)");
    if (!ctx->mpcScaled && ctx->P.mpcDim > 0) return set_err(ctx, ASTRO_ERR_STATE, "astro_scale_mpc must run first");
    if (p->degree < 1 || p->degree > ASTRO_PRECOND_MAX_DEGREE) return set_err(ctx, ASTRO_ERR_ARG, "precond degree out of range");
    if (p->dpn != ctx->P.dpn) return set_err(ctx, ASTRO_ERR_ARG, "precond DOF per node differs from the model's");
    if (!(p->ratio > 1.0) || !(p->lambda_scale > 0.0)) return set_err(ctx, ASTRO_ERR_ARG, "precond ratio must be > 1");
    return ASTRO_OK;
}

}  // namespace

// Least-squares Chebyshev fit of 1/nu on [1/ratio, 1]: minimise sum_i (nu_i sum_k c_k T_k(x_i) - 1)^2
// over 400 Chebyshev nodes x_i of [-1, 1] (nu_i their image), by modified Gram-Schmidt QR.
extern "C" int astro_precond_init(int32_t degree, double ratio, int32_t dpn, astro_precond *p) {
    if (!p || degree < 1 || degree > ASTRO_PRECOND_MAX_DEGREE || !(ratio > 1.0) || (dpn != 3 && dpn != 6))
        return ASTRO_ERR_ARG;
    constexpr int M = 400;
    const int K = degree + 1;
    std::vector<double> A((size_t)M * K), rhs(M, 1.0);
    const double pi = 3.14159265358979323846;
    for (int i = 0; i < M; ++i) {
        const double x = std::cos(pi * (i + 0.5) / M);
        const double nu = 0.5 * (x + 1.0) * (1.0 - 1.0 / ratio) + 1.0 / ratio;
        double t0 = 1.0, t1 = x;
        for (int k = 0; k < K; ++k) {
            const double tk = (k == 0) ? 1.0 : (k == 1 ? x : 2.0 * x * t1 - t0);
            if (k >= 2) {
                t0 = t1;
                t1 = tk;
            }
            A[(size_t)k * M + i] = nu * tk;  // column-major
        }
    }
    std::vector<double> R((size_t)K * K, 0.0);
    for (int k = 0; k < K; ++k) {
        double *ak = &A[(size_t)k * M];
        for (int l = 0; l < k; ++l) {
            const double *al = &A[(size_t)l * M];
            double d = 0.0;
            for (int i = 0; i < M; ++i) d += al[i] * ak[i];
            R[(size_t)l * K + k] = d;
            for (int i = 0; i < M; ++i) ak[i] -= d * al[i];
        }
        double nn = 0.0;
        for (int i = 0; i < M; ++i) nn += ak[i] * ak[i];
        nn = std::sqrt(nn);
        if (!(nn > 0.0)) return ASTRO_ERR_ARG;
        R[(size_t)k * K + k] = nn;
        for (int i = 0; i < M; ++i) ak[i] /= nn;
    }
    std::vector<double> qb(K), c(K);
    for (int k = 0; k < K; ++k) {
        double d = 0.0;
        for (int i = 0; i < M; ++i) d += A[(size_t)k * M + i] * rhs[i];
        qb[k] = d;
    }
    for (int k = K - 1; k >= 0; --k) {
        double s = qb[k];
        for (int l = k + 1; l < K; ++l) s -= R[(size_t)k * K + l] * c[l];
        c[k] = s / R[(size_t)k * K + k];
    }
    std::memset(p, 0, sizeof(*p));
    p->degree = degree;
    p->dpn = dpn;
    p->ratio = ratio;
    p->lambda_scale = 1.05;
    for (int k = 0; k < K; ++k)
        for (int i = 0; i < dpn; ++i) p->weights[((size_t)k * dpn + i) * dpn + i] = c[k];
    return ASTRO_OK;
}

extern "C" int astro_precond_lambda(astro_ctx *ctx, int32_t kind, double *lambda) {
    if (!ctx || !lambda) return ASTRO_ERR_ARG;
    if (!ctx->mpcScaled && ctx->P.mpcDim > 0) return set_err(ctx, ASTRO_ERR_STATE, "astro_scale_mpc must run first");
    return krylov_power_lambda(ctx, kind, lambda);
}

extern "C" int astro_precond_loss_grad(astro_ctx *ctx, const astro_precond *p, const double *samples,
                                       int32_t num_samples, double *loss, double *grad) {
    if (!ctx || !p || !loss) return ASTRO_ERR_ARG;
    int rc;
    if ((rc = train_check(ctx, p, samples, num_samples))) return rc;
    TrainSet T;
    if ((rc = T.setup(ctx, p, samples, num_samples))) return rc;
    return T.loss_grad(p->weights, loss, grad);
}

extern "C" int astro_precond_train(astro_ctx *ctx, astro_precond *p, const double *samples, int32_t num_samples,
                                   int32_t iters, double *loss_history) {
    if (!ctx || !p || iters < 0) return ASTRO_ERR_ARG;
    int rc;
    if ((rc = train_check(ctx, p, samples, num_samples))) return rc;
    TrainSet T;
    if ((rc = T.setup(ctx, p, samples, num_samples))) return rc;
    const int nw = (p->degree + 1) * p->dpn * p->dpn;
    std::vector<double> w(p->weights, p->weights + nw), g(nw), gPrev(nw), d(nw), dPrev(nw);
    double L = 0.0;
    for (int it = 0; it <= iters; ++it) {
        if ((rc = T.loss_grad(w.data(), &L, it < iters ? g.data() : nullptr))) return rc;
        if (!std::isfinite(L)) return set_err(ctx, ASTRO_ERR_NAN, "non-finite training loss");
        if (loss_history) loss_history[it] = L;
        if (it == iters) break;
        // Polak-Ribiere+ direction
        double beta = 0.0;
        if (it > 0) {
            double num = 0.0, den = 0.0;
            for (int q = 0; q < nw; ++q) {
                num += g[q] * (g[q] - gPrev[q]);
                den += gPrev[q] * gPrev[q];
            }
            beta = den > 0.0 ? std::max(0.0, num / den) : 0.0;
        }
        for (int q = 0; q < nw; ++q) d[q] = g[q] + beta * (it > 0 ? dPrev[q] : 0.0);
        double alpha = 0.0, qq = 0.0;
        if ((rc = T.line_search(d.data(), &alpha, &qq))) return rc;
        if (!(qq > 0.0)) {  // the direction does not change the output: converged
            if (loss_history)
                for (int r = it + 1; r <= iters; ++r) loss_history[r] = L;
            break;
        }
        for (int q = 0; q < nw; ++q) w[q] -= alpha * d[q];
        gPrev = g;
        dPrev = d;
    }
    std::memcpy(p->weights, w.data(), sizeof(double) * nw);
    return ASTRO_OK;
}

// node id order <-> internal block rows
static void rows_to_nodes(astro_ctx *ctx, const std::vector<double> &in, int w, double *out) {
    const AstroPrep &P = ctx->P;
    for (int nd = 1; nd <= P.N; ++nd) {
        const int r = P.currentRank[nd] - 1;
        std::memcpy(out + (size_t)(nd - 1) * w, in.data() + (size_t)r * w, sizeof(double) * w);
    }
}

extern "C" int astro_node_features(astro_ctx *ctx, int32_t kind, double *features) {
    if (!ctx || !features || (kind != 64 && kind != 32)) return ASTRO_ERR_ARG;
    if (!ctx->mpcScaled && ctx->P.mpcDim > 0) return set_err(ctx, ASTRO_ERR_STATE, "astro_scale_mpc must run first");
    const int N = ctx->P.N;
    DevBuf F, L, pd, part;
    int rc = dev_alloc(ctx, F, sizeof(double) * (size_t)N * kF);
    if (!rc) rc = precond_node_features(ctx, kind, dptr<double>(F), L, pd, part, ctx->stream);
    std::vector<double> h((size_t)N * kF);
    if (!rc) {
        cudaError_t e = cudaMemcpyAsync(h.data(), F.p, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        rc = cuda_check(ctx, e, "features download");
    }
    if (!rc) rows_to_nodes(ctx, h, kF, features);
    DevBuf *b[] = {&F, &L, &pd, &part};
    for (auto *x : b) dev_free(*x);
    return rc;
}

extern "C" int astro_precond_mlp_scales(astro_ctx *ctx, int32_t kind, const astro_precond_mlp *mlp, double *scales) {
    if (!ctx || !mlp || !scales || (kind != 64 && kind != 32)) return ASTRO_ERR_ARG;
    if (mlp->hidden < 0 || mlp->hidden > ASTRO_MLP_MAX_HIDDEN || mlp->outputs < 1 ||
        mlp->outputs > ASTRO_PRECOND_MAX_DEGREE + 1)
        return set_err(ctx, ASTRO_ERR_ARG, "perceptron shape out of range");
    if (!ctx->mpcScaled && ctx->P.mpcDim > 0) return set_err(ctx, ASTRO_ERR_STATE, "astro_scale_mpc must run first");
    const int N = ctx->P.N, K = mlp->outputs, H = mlp->hidden;
    DevBuf F, L, pd, part, prm, a;
    int rc = dev_alloc(ctx, F, sizeof(double) * (size_t)N * kF);
    if (!rc) rc = dev_alloc(ctx, a, sizeof(double) * (size_t)N * K);
    if (!rc) rc = precond_node_features(ctx, kind, dptr<double>(F), L, pd, part, ctx->stream);
    std::vector<double> pk;
    mlp_pack(mlp, K, pk);
    if (!rc) rc = upload(ctx, prm, pk.data(), sizeof(double) * pk.size());
    if (!rc) {
        k_mlp_fwd<double><<<(N + kT - 1) / kT, kT, 0, ctx->stream>>>(N, MlpDims{H, K}, dptr<double>(F),
                                                                    dptr<double>(prm), dptr<double>(a), nullptr);
        rc = cuda_check(ctx, cudaGetLastError(), "perceptron forward");
    }
    std::vector<double> h((size_t)N * K), t((size_t)N * K);
    if (!rc) {
        cudaError_t e = cudaMemcpyAsync(h.data(), a.p, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        rc = cuda_check(ctx, e, "scales download");
    }
    if (!rc) {
        for (int k = 0; k < K; ++k)
            for (int r = 0; r < N; ++r) t[(size_t)r * K + k] = h[(size_t)k * N + r];
        rows_to_nodes(ctx, t, K, scales);
    }
    DevBuf *b[] = {&F, &L, &pd, &part, &prm, &a};
    for (auto *x : b) dev_free(*x);
    return rc;
}

extern "C" int astro_precond_mlp_loss_grad(astro_ctx *ctx, const astro_precond *p, const astro_precond_mlp *mlp,
                                           const double *samples, int32_t num_samples, double *loss,
                                           double *grad_weights, astro_precond_mlp *grad_mlp) {
    if (!ctx || !p || !mlp || !loss) return ASTRO_ERR_ARG;
    int rc;
    if ((rc = train_check(ctx, p, samples, num_samples))) return rc;
    if ((rc = precond_mlp_check(ctx, mlp, p->degree))) return rc;
    TrainSet T;
    if ((rc = T.setup(ctx, p, samples, num_samples))) return rc;
    const int H = mlp->hidden, K = p->degree + 1;
    std::vector<double> gm((size_t)H * kF + H + (size_t)K * H + K);
    if ((rc = T.loss_grad_mod(p->weights, mlp, loss, grad_weights, grad_mlp ? gm.data() : nullptr))) return rc;
    if (grad_mlp) mlp_unpack(gm.data(), H, K, grad_mlp);
    return ASTRO_OK;
}
