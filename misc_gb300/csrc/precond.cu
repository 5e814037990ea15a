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

// Device state of a training run: samples, features and work vectors for S samples.
struct TrainSet {
    astro_ctx *ctx = nullptr;
    Op<double> op;
    int S = 0, deg = 0, deg1 = 0, dpn = 0, n = 0, N = 0, nCta = 0;
    double lam = 0.0, theta = 0.0, delta = 0.0;
    DevBuf v, dinv, Y, Z, E, part, Wl;
    std::vector<double> hp;

    ~TrainSet() {
        DevBuf *b[] = {&v, &dinv, &Y, &Z, &E, &part, &Wl};
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

    int fetch(size_t count) {
        hp.resize(count);
        cudaError_t e = cudaMemcpyAsync(hp.data(), part.p, sizeof(double) * count, cudaMemcpyDeviceToHost, ctx->stream);
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
