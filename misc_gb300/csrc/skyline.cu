// The reference's own linear solve on the GPU, for the faithful drop-in path:
//   convertToLTri      (Working/AStrO_bookKeeping.f90:754-792)  K and C^T C inside the profile
//   getSparseLDLFact   (Working/AStrO_solvers.f90:10-78)        row-skyline LDL^T, no pivoting
//   solveSparseLDLFact (:83-126)                                forward by rows, backward by columns
//   gMRes              (:128-297) with rFactorMat/solveRFactor (:299-404)
// The skyline recurrences are sequential along the profile, so the factor and the solves run in
// one CTA that sweeps the rows with block-wide reductions; gMRes runs as one persistent CTA
// (sparse products, preconditioner solves, modified Gram-Schmidt, Givens QR of the Hessenberg
// matrix) so that nothing returns to the host inside the iteration.  Every loop is bounded by the
// reference's own limits (maxIt/numVecs + 1 restarts), so the kernels always terminate.  These
// are the parity path for the reference's algorithm on the small and mid-size models it is used
// for; the large systems use the Jacobi/mixed-precision solvers of krylov.cu.
#include <algorithm>
#include <cmath>

#include "astro_internal.h"

namespace {

constexpr int kT = 512;

__device__ double block_sum(double v, double *red) {
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[w] = v;
    __syncthreads();
    double s = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) s += red[q];
    return s;
}

// (K + C^T C) restricted to the skyline profile; lTri zeroed by the caller.
__global__ void k_ltri_main(const double *__restrict__ K, const int *__restrict__ bRow, const int *__restrict__ bCol,
                            long long nb, int dpn, int N, const int *__restrict__ LTR, double *lTri) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= nb * dpn * dpn) return;
    const long long k = t / (dpn * dpn);
    const int ij = (int)(t - k * dpn * dpn), i = ij / dpn, j = ij % dpn;
    const int R = bRow[k] + 1 + i * N, Cc = bCol[k] + 1 + j * N;  // 1-based reference DOF
    const int minCol = R - LTR[R] + LTR[R - 1] + 1;
    if (Cc >= minCol && Cc <= R) lTri[LTR[R] - R + Cc - 1] += K[t];
}

__global__ void k_ltri_pen(int nt, const int *__restrict__ pr, const int *__restrict__ pc, const double *__restrict__ pv,
                           const int *__restrict__ LTR, double *lTri) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt) return;
    const int R = pr[t], Cc = pc[t];
    const int minCol = R - LTR[R] + LTR[R - 1] + 1;
    if (Cc >= minCol && Cc <= R) lTri[LTR[R] - R + Cc - 1] += pv[t];
}

// getSparseLDLFact in place; rowStCol(i) = i - rowLen(i) + 1.  status[0] = 1-based row of the
// first zero or non-finite pivot.
__device__ void ldl_fact(double *A, const int *R, int n, int maxBW, double *diag, double *dLprod, int *status) {
    __shared__ double red[32];
    for (int i1 = 1; i1 <= n; ++i1) {
        const int i3 = R[i1], i2 = R[i1 - 1] + 1, len = i3 - i2;  // off-diagonal entries of row i1
        double part = 0.0;
        for (int k = threadIdx.x; k < len; k += blockDim.x) {
            const double a = A[i2 + k - 1], d = diag[i1 - len + k];
            dLprod[maxBW - len + 1 + k] = d * a;
            part += d * a * a;
        }
        const double s = block_sum(part, red);
        const double dg = A[i3 - 1] - s;
        if (threadIdx.x == 0) {
            diag[i1] = dg;
            A[i3 - 1] = dg;
            if ((dg == 0.0 || !isfinite(dg)) && status[0] == 0) status[0] = i1;
        }
        __syncthreads();
        const double fact = 1.0 / dg;
        const int imax = min(n, i1 + maxBW);
        const int stc1 = i1 - (R[i1] - R[i1 - 1]) + 1;
        for (int j = i1 + 1 + threadIdx.x; j <= imax; j += blockDim.x) {
            const int stc2 = j - (R[j] - R[j - 1]) + 1;
            const int stCol = max(stc1, stc2);
            const int rowLen = i1 - stCol;
            if (rowLen >= 0) {
                const int a = maxBW - rowLen + 1, b = R[j] - (j - stCol), t = b + rowLen;
                double d = A[t - 1];
                for (int q = 0; q < rowLen; ++q) d -= dLprod[a + q] * A[b + q - 1];
                A[t - 1] = d * fact;
            }
        }
        __syncthreads();
    }
}

// solveSparseLDLFact: forward over rows, backward over columns.
// maxBW = largest off-diagonal row length of the profile.
__device__ void ldl_solve(double *soln, const double *rhs, const double *L, const int *R, int n, int maxBW, double *z) {
    __shared__ double red[32];
    for (int i1 = 1; i1 <= n; ++i1) {
        const int i2 = R[i1 - 1] + 1, rowLen = R[i1] - i2, stCol = i1 - rowLen;
        double part = 0.0;
        for (int k = threadIdx.x; k < rowLen; k += blockDim.x) part += L[i2 + k - 1] * z[stCol + k - 1];
        const double s = block_sum(part, red);
        if (threadIdx.x == 0) z[i1 - 1] = rhs[i1 - 1] - s;
        __syncthreads();
    }
    for (int i1 = n; i1 >= 1; --i1) {
        const double dg = L[R[i1] - 1];
        const int imax = min(n, i1 + maxBW);
        double part = 0.0;
        for (int j = i1 + 1 + threadIdx.x; j <= imax; j += blockDim.x) {
            const int rowLen = R[j] - R[j - 1], stCol = j - rowLen + 1;
            if (stCol <= i1) part += L[R[j] + i1 - j - 1] * soln[j - 1];
        }
        const double s = block_sum(part, red);
        if (threadIdx.x == 0) soln[i1 - 1] = (z[i1 - 1] - s * dg) / dg;
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kT) k_ldl_fact(double *A, const int *R, int n, int maxBW, double *diag, double *dLprod,
                                                 int *status) {
    ldl_fact(A, R, n, maxBW, diag, dLprod, status);
}

__global__ void __launch_bounds__(kT) k_ldl_solve(double *soln, const double *rhs, const double *L, const int *R, int n,
                                                  int maxBW, double *z) {
    ldl_solve(soln, rhs, L, R, n, maxBW, z);
}

struct RefGmresArgs {
    double *x;
    const double *A, *Cm, *P, *b;
    const int *Ac, *AR, *Cc, *CR, *PR;
    int n, cdim, numVecs, maxIt, pBW;
    double *H, *G, *r, *t1, *t2, *z, *cv;  // H: n x (m+1) column-major; G: (m+1) x m
    int *out;                              // out[0] = restart cycles run, out[1] = status
};

// y = A x + C^T (C x) in the reference's order (C^T C part first, then the rows of A)
__device__ void ref_matvec(const RefGmresArgs &g, const double *x, double *y) {
    for (int i = threadIdx.x; i < g.cdim; i += blockDim.x) {
        double s = 0.0;
        for (int k = g.CR[i]; k < g.CR[i + 1]; ++k)
            if (g.Cc[k]) s += g.Cm[k] * x[g.Cc[k] - 1];
        g.cv[i] = s;
    }
    for (int i = threadIdx.x; i < g.n; i += blockDim.x) y[i] = 0.0;
    __syncthreads();
    if (threadIdx.x == 0)  // scatter C^T (C x) sequentially (C is small)
        for (int i = 0; i < g.cdim; ++i)
            for (int k = g.CR[i]; k < g.CR[i + 1]; ++k)
                if (g.Cc[k]) y[g.Cc[k] - 1] += g.Cm[k] * g.cv[i];
    __syncthreads();
    for (int i = threadIdx.x; i < g.n; i += blockDim.x) {
        double s = y[i];
        for (int k = g.AR[i]; k < g.AR[i + 1]; ++k)
            if (g.Ac[k]) s += g.A[k] * x[g.Ac[k] - 1];
        y[i] = s;
    }
    __syncthreads();
}

__device__ double dot_block(const double *a, const double *b, int n) {
    __shared__ double red[32];
    double p = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) p += a[i] * b[i];
    return block_sum(p, red);
}

__global__ void __launch_bounds__(kT) k_ref_gmres(RefGmresArgs g) {
    const int n = g.n, m = g.numVecs, ldg = m + 1;
    auto Hc = [&](int col) { return g.H + (size_t)col * n; };  // column col (0-based) of hMat
    // r = P^-1 (b - (A + C^T C) x)
    ref_matvec(g, g.x, g.t2);
    for (int i = threadIdx.x; i < n; i += blockDim.x) g.t1[i] = g.b[i] - g.t2[i];
    __syncthreads();
    ldl_solve(g.r, g.t1, g.P, g.PR, n, g.pBW, g.z);
    double resMag = sqrt(dot_block(g.r, g.r, n));
    const int maxOut = g.maxIt / m + 1;
    int it = 0;
    const double tol = (double)(float)1e-12;
    while (resMag > tol && it < maxOut) {
        for (int i = threadIdx.x; i < n; i += blockDim.x) Hc(0)[i] = (1.0 / resMag) * g.r[i];
        for (int i = threadIdx.x; i < ldg * m; i += blockDim.x) g.G[i] = 0.0;
        __syncthreads();
        for (int i5 = 1; i5 <= m; ++i5) {  // builds column i5 (0-based) of hMat
            ref_matvec(g, Hc(i5 - 1), g.t2);
            ldl_solve(Hc(i5), g.t2, g.P, g.PR, n, g.pBW, g.z);
            for (int i1 = 0; i1 < i5; ++i1) {
                const double dp = dot_block(Hc(i1), Hc(i5), n);
                for (int i = threadIdx.x; i < n; i += blockDim.x) Hc(i5)[i] -= dp * Hc(i1)[i];
                if (threadIdx.x == 0) g.G[(size_t)(i5 - 1) * ldg + i1] = dp;
                __syncthreads();
            }
            const double nr = sqrt(dot_block(Hc(i5), Hc(i5), n));
            for (int i = threadIdx.x; i < n; i += blockDim.x) Hc(i5)[i] = (1.0 / nr) * Hc(i5)[i];
            if (threadIdx.x == 0) g.G[(size_t)(i5 - 1) * ldg + i5] = nr;
            __syncthreads();
        }
        // Givens QR (rFactorMat, triDiag = 2) and the projected right-hand side t1 = H^T r
        if (threadIdx.x == 0) {
            const double thr = (double)(float)1e-10;
            for (int i1 = 0; i1 < m; ++i1) {
                const int i2 = i1 + 1;
                double *c1 = g.G + (size_t)i1 * ldg;
                if (fabs(c1[i2]) > thr) {
                    const double th = (c1[i1] == 0.0) ? (double)(float)1.570796326794897 : atan(c1[i2] / c1[i1]);
                    const double st = sin(th), ct = cos(th);
                    for (int i3 = i1; i3 < m; ++i3) {
                        double *c3 = g.G + (size_t)i3 * ldg;
                        const double a1 = ct * c3[i1] + st * c3[i2], a2 = -st * c3[i1] + ct * c3[i2];
                        c3[i1] = a1;
                        c3[i2] = a2;
                    }
                    c1[i2] = th;
                }
            }
        }
        __syncthreads();
        for (int k = 0; k <= m; ++k) {
            const double s = dot_block(Hc(k), g.r, n);
            if (threadIdx.x == 0) g.t1[k] = s;
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            const double thr = (double)(float)1e-10;
            for (int i1 = 0; i1 < m; ++i1) {
                const int i2 = i1 + 1;
                const double th = g.G[(size_t)i1 * ldg + i2];
                if (fabs(th) > thr) {
                    const double st = sin(th), ct = cos(th);
                    const double r1 = ct * g.t1[i1] + st * g.t1[i2], r2 = -st * g.t1[i1] + ct * g.t1[i2];
                    g.t1[i1] = r1;
                    g.t1[i2] = r2;
                }
            }
            for (int i1 = m - 1; i1 >= 0; --i1) {
                double s = g.t1[i1];
                for (int i2 = i1 + 1; i2 < m; ++i2) s -= g.G[(size_t)i2 * ldg + i1] * g.t2[i2];
                g.t2[i1] = s / g.G[(size_t)i1 * ldg + i1];
            }
        }
        __syncthreads();
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            double s = g.x[i];
            for (int k = 0; k < m; ++k) s += Hc(k)[i] * g.t2[k];
            g.x[i] = s;
        }
        __syncthreads();
        ref_matvec(g, g.x, g.t2);
        for (int i = threadIdx.x; i < n; i += blockDim.x) g.t1[i] = g.b[i] - g.t2[i];
        __syncthreads();
        ldl_solve(g.r, g.t1, g.P, g.PR, n, g.pBW, g.z);
        resMag = sqrt(dot_block(g.r, g.r, n));
        ++it;
    }
    if (threadIdx.x == 0) {
        g.out[0] = it;
        g.out[1] = isfinite(resMag) ? 0 : ASTRO_ERR_NAN;
    }
}

}  // namespace

static int skyline_maxbw(const int *R, int n) {
    int mb = 0;
    for (int i = 1; i <= n; ++i) mb = std::max(mb, R[i] - R[i - 1]);
    return mb;
}

// convertToLTri from the device matrix and the scaled constraints (internal penalty list
// converted back to reference DOF numbers).
extern "C" int astro_convert_to_ltri(astro_ctx *ctx, double *l_tri) {
    if (!ctx) return ASTRO_ERR_ARG;
    if (!ctx->haveK64) return set_err(ctx, ASTRO_ERR_STATE, "convert_to_ltri needs the FP64 stiffness (astro_el_soln_load)");
    if (ctx->P.mpcDim > 0 && !ctx->mpcScaled) return set_err(ctx, ASTRO_ERR_STATE, "astro_scale_mpc must run first");
    const AstroPrep &P = ctx->P;
    int rc;
    if ((rc = upload(ctx, ctx->d_ltRange, P.elMatLTRange.data(), sizeof(int) * (P.n + 1)))) return rc;
    if ((rc = dev_alloc(ctx, ctx->d_lt, sizeof(double) * (size_t)std::max(P.ltSize, 1)))) return rc;
    CK(cudaMemsetAsync(ctx->d_lt.p, 0, sizeof(double) * (size_t)P.ltSize, ctx->stream));
    const long long tot = (long long)P.nb * P.dpn * P.dpn;
    k_ltri_main<<<(unsigned)((tot + 255) / 256), 256, 0, ctx->stream>>>(dptr<double>(ctx->d_K64), dptr<int>(ctx->d_bRow),
                                                                         dptr<int>(ctx->d_bCol), P.nb, P.dpn, P.N,
                                                                         dptr<int>(ctx->d_ltRange), dptr<double>(ctx->d_lt));
    CK(cudaGetLastError());
    // C^T C pairs in reference numbering, in the reference's row-by-row order
    std::vector<int> pr, pc;
    std::vector<double> pv;
    for (int r = 0; r < P.mpcDim; ++r)
        for (int a = P.mpcRange[r]; a < P.mpcRange[r + 1]; ++a) {
            if (!P.mpcCols[a]) continue;
            for (int b = P.mpcRange[r]; b < P.mpcRange[r + 1]; ++b) {
                if (!P.mpcCols[b]) continue;
                pr.push_back(P.mpcCols[a]);
                pc.push_back(P.mpcCols[b]);
                pv.push_back(ctx->mpcScaledHost[a] * ctx->mpcScaledHost[b]);
            }
        }
    if (!pr.empty()) {
        // pairs sharing an (R, C) entry are accumulated in order by one thread per distinct
        // entry is not needed: with one term per constraint row each entry occurs once; general
        // constraints are accumulated sequentially.
        bool unique = true;
        {
            std::vector<long long> keys(pr.size());
            for (size_t q = 0; q < pr.size(); ++q) keys[q] = (long long)pr[q] * (P.n + 1) + pc[q];
            std::sort(keys.begin(), keys.end());
            for (size_t q = 1; q < keys.size(); ++q)
                if (keys[q] == keys[q - 1]) unique = false;
        }
        DevBuf dpr, dpc, dpv;
        if ((rc = upload(ctx, dpr, pr.data(), sizeof(int) * pr.size()))) return rc;
        if ((rc = upload(ctx, dpc, pc.data(), sizeof(int) * pc.size()))) return rc;
        if ((rc = upload(ctx, dpv, pv.data(), sizeof(double) * pv.size()))) return rc;
        const int nt = (int)pr.size();
        if (unique) {
            k_ltri_pen<<<(nt + 255) / 256, 256, 0, ctx->stream>>>(nt, dptr<int>(dpr), dptr<int>(dpc), dptr<double>(dpv),
                                                                  dptr<int>(ctx->d_ltRange), dptr<double>(ctx->d_lt));
        } else {
            for (int t = 0; t < nt; ++t)
                k_ltri_pen<<<1, 1, 0, ctx->stream>>>(1, dptr<int>(dpr) + t, dptr<int>(dpc) + t, dptr<double>(dpv) + t,
                                                     dptr<int>(ctx->d_ltRange), dptr<double>(ctx->d_lt));
        }
        CK(cudaGetLastError());
        CK(cudaStreamSynchronize(ctx->stream));
        dev_free(dpr);
        dev_free(dpc);
        dev_free(dpv);
    }
    ctx->haveLT = 1;
    ctx->ltFactored = 0;
    if (l_tri) {
        CK(cudaMemcpyAsync(l_tri, ctx->d_lt.p, sizeof(double) * (size_t)P.ltSize, cudaMemcpyDeviceToHost, ctx->stream));
    }
    CK(cudaStreamSynchronize(ctx->stream));
    return ASTRO_OK;
}

// b at least bytes long (grown, never shrunk: the buffers outlive the call)
static int sky_scratch(astro_ctx *ctx, DevBuf &b, size_t bytes) {
    return b.bytes >= bytes ? ASTRO_OK : dev_alloc(ctx, b, bytes);
}

// Threads of the row-sweeping factor and solve: the later rows a row updates (the profile's
// longest row, maxBW) are split over the threads, so a CTA wider than that only adds barrier
// cost: one warp up to 32, then multiples of 32 up to 512.
static int sky_threads(int maxBW) { return std::min(kT, std::max(32, (maxBW + 31) / 32 * 32)); }

static int ldl_fact_dev(astro_ctx *ctx, double *d_A, const int *d_R, const int *h_R, int n) {
    const int maxBW = skyline_maxbw(h_R, n);
    DevBuf &diag = ctx->d_sky[3], &dl = ctx->d_sky[4];
    int rc;
    if ((rc = sky_scratch(ctx, diag, sizeof(double) * (size_t)(n + 1))) ||
        (rc = sky_scratch(ctx, dl, sizeof(double) * (size_t)(maxBW + 2))))
        return rc;
    int *st = dptr<int>(ctx->d_status);
    CK(cudaMemsetAsync(st, 0, sizeof(int), ctx->stream));
    k_ldl_fact<<<1, sky_threads(maxBW), 0, ctx->stream>>>(d_A, d_R, n, maxBW, dptr<double>(diag), dptr<double>(dl),
                                                         st);
    CK(cudaGetLastError());
    int hs = 0;
    CK(cudaMemcpyAsync(&hs, st, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (hs) return set_err(ctx, ASTRO_ERR_PIVOT, "zero or non-finite pivot in row " + std::to_string(hs));
    return ASTRO_OK;
}

extern "C" int astro_ldl_fact(astro_ctx *ctx, double *a_l_tri, int32_t a_size, const int32_t *a_range, int32_t n) {
    if (!ctx || !a_l_tri || !a_range || n <= 0 || a_size < a_range[n]) return ASTRO_ERR_ARG;
    DevBuf &dA = ctx->d_sky[0], &dR = ctx->d_sky[1];
    int rc;
    if ((rc = sky_scratch(ctx, dA, sizeof(double) * (size_t)a_size)) ||
        (rc = sky_scratch(ctx, dR, sizeof(int) * (size_t)(n + 1))))
        return rc;
    CK(cudaMemcpyAsync(dA.p, a_l_tri, sizeof(double) * (size_t)a_size, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(dR.p, a_range, sizeof(int) * (size_t)(n + 1), cudaMemcpyHostToDevice, ctx->stream));
    rc = ldl_fact_dev(ctx, dptr<double>(dA), dptr<int>(dR), a_range, n);
    if (rc == ASTRO_OK || rc == ASTRO_ERR_PIVOT) {
        cudaError_t e = cudaMemcpyAsync(a_l_tri, dA.p, sizeof(double) * (size_t)a_size, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) rc = cuda_check(ctx, e, "ldl_fact download");
    }
    return rc;
}

extern "C" int astro_ldl_fact_resident(astro_ctx *ctx) {
    if (!ctx) return ASTRO_ERR_ARG;
    if (!ctx->haveLT) return set_err(ctx, ASTRO_ERR_STATE, "astro_convert_to_ltri must run first");
    int rc = ldl_fact_dev(ctx, dptr<double>(ctx->d_lt), dptr<int>(ctx->d_ltRange), ctx->P.elMatLTRange.data(), ctx->P.n);
    if (!rc) ctx->ltFactored = 1;
    return rc;
}

extern "C" int astro_ldl_solve(astro_ctx *ctx, double *soln, const double *rhs, const double *l_mat, int32_t l_size,
                               const int32_t *l_range, int32_t l_dim, double *z_vec) {
    if (!ctx || !soln || !rhs || !l_mat || !l_range || l_dim <= 0 || l_size < l_range[l_dim]) return ASTRO_ERR_ARG;
    const int maxBW = skyline_maxbw(l_range, l_dim) - 1;
    DevBuf &dL = ctx->d_sky[0], &dR = ctx->d_sky[1], &db = ctx->d_sky[2], &dx = ctx->d_sky[3], &dz = ctx->d_sky[4];
    int rc;
    if ((rc = sky_scratch(ctx, dL, sizeof(double) * (size_t)l_size)) ||
        (rc = sky_scratch(ctx, dR, sizeof(int) * (size_t)(l_dim + 1))) ||
        (rc = sky_scratch(ctx, db, sizeof(double) * (size_t)l_dim)) ||
        (rc = sky_scratch(ctx, dx, sizeof(double) * (size_t)l_dim)) ||
        (rc = sky_scratch(ctx, dz, sizeof(double) * (size_t)l_dim)))
        return rc;
    CK(cudaMemcpyAsync(dL.p, l_mat, sizeof(double) * (size_t)l_size, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(dR.p, l_range, sizeof(int) * (size_t)(l_dim + 1), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(db.p, rhs, sizeof(double) * (size_t)l_dim, cudaMemcpyHostToDevice, ctx->stream));
    k_ldl_solve<<<1, sky_threads(maxBW), 0, ctx->stream>>>(dptr<double>(dx), dptr<double>(db), dptr<double>(dL),
                                                          dptr<int>(dR), l_dim, maxBW, dptr<double>(dz));
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(soln, dx.p, sizeof(double) * (size_t)l_dim, cudaMemcpyDeviceToHost, ctx->stream));
    if (z_vec) CK(cudaMemcpyAsync(z_vec, dz.p, sizeof(double) * (size_t)l_dim, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return ASTRO_OK;
}

extern "C" int astro_gmres(astro_ctx *ctx, double *x_vec, const double *a_mat, const int32_t *a_cols,
                           const int32_t *a_range, int32_t a_size, int32_t a_dim, const double *c_mat,
                           const int32_t *c_cols, const int32_t *c_range, int32_t c_size, int32_t c_dim,
                           const double *p_mat, const int32_t *p_range, int32_t p_size, const double *b_vec,
                           int32_t num_vecs, int32_t max_it) {
    if (!ctx || !x_vec || !a_mat || !a_cols || !a_range || !p_mat || !p_range || !b_vec || a_dim <= 0 || num_vecs <= 0 ||
        num_vecs >= a_dim || max_it < 0 || (c_dim > 0 && (!c_mat || !c_cols || !c_range)) || a_size < a_range[a_dim] ||
        p_size < p_range[a_dim] || (c_dim > 0 && c_size < c_range[c_dim]))
        return ASTRO_ERR_ARG;
    const int n = a_dim, m = num_vecs;
    DevBuf dx, dA, dAc, dAR, dC, dCc, dCR, dP, dPR, db, dH, dG, dr, dt1, dt2, dz, dcv, dout;
    int rc = ASTRO_OK;
    // an empty constraint set gets placeholder buffers that the kernel never reads (cdim = 0)
    auto up = [&](DevBuf &b, const void *h, size_t bytes) {
        if (rc) return;
        rc = (h && bytes) ? upload(ctx, b, h, bytes) : dev_alloc(ctx, b, 16);
    };
    const bool hasC = c_dim > 0;
    up(dx, x_vec, sizeof(double) * n);
    up(dA, a_mat, sizeof(double) * a_size);
    up(dAc, a_cols, sizeof(int) * a_size);
    up(dAR, a_range, sizeof(int) * (n + 1));
    up(dC, hasC ? c_mat : nullptr, hasC ? sizeof(double) * c_size : 0);
    up(dCc, hasC ? c_cols : nullptr, hasC ? sizeof(int) * c_size : 0);
    up(dCR, hasC ? c_range : nullptr, hasC ? sizeof(int) * (c_dim + 1) : 0);
    up(dP, p_mat, sizeof(double) * p_size);
    up(dPR, p_range, sizeof(int) * (n + 1));
    up(db, b_vec, sizeof(double) * n);
    if (!rc) rc = dev_alloc(ctx, dH, sizeof(double) * (size_t)n * (m + 1));
    if (!rc) rc = dev_alloc(ctx, dG, sizeof(double) * (size_t)(m + 1) * m);
    if (!rc) rc = dev_alloc(ctx, dr, sizeof(double) * n);
    if (!rc) rc = dev_alloc(ctx, dt1, sizeof(double) * std::max(n, m + 1));
    if (!rc) rc = dev_alloc(ctx, dt2, sizeof(double) * std::max(n, m + 1));
    if (!rc) rc = dev_alloc(ctx, dz, sizeof(double) * n);
    if (!rc) rc = dev_alloc(ctx, dcv, sizeof(double) * std::max(c_dim, 1));
    if (!rc) rc = dev_alloc(ctx, dout, sizeof(int) * 4);
    int hout[2] = {0, 0};
    if (!rc) {
        RefGmresArgs g;
        g.x = dptr<double>(dx);
        g.A = dptr<double>(dA);
        g.Cm = dptr<double>(dC);
        g.P = dptr<double>(dP);
        g.b = dptr<double>(db);
        g.Ac = dptr<int>(dAc);
        g.AR = dptr<int>(dAR);
        g.Cc = dptr<int>(dCc);
        g.CR = dptr<int>(dCR);
        g.PR = dptr<int>(dPR);
        g.n = n;
        g.cdim = std::max(c_dim, 0);
        g.numVecs = m;
        g.maxIt = max_it;
        g.pBW = skyline_maxbw(p_range, n) - 1;
        g.H = dptr<double>(dH);
        g.G = dptr<double>(dG);
        g.r = dptr<double>(dr);
        g.t1 = dptr<double>(dt1);
        g.t2 = dptr<double>(dt2);
        g.z = dptr<double>(dz);
        g.cv = dptr<double>(dcv);
        g.out = dptr<int>(dout);
        k_ref_gmres<<<1, kT, 0, ctx->stream>>>(g);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpyAsync(hout, dout.p, sizeof(int) * 2, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(x_vec, dx.p, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        rc = cuda_check(ctx, e, "reference gmres");
    }
    DevBuf *bs[] = {&dx, &dA, &dAc, &dAR, &dC, &dCc, &dCR, &dP, &dPR, &db, &dH, &dG, &dr, &dt1, &dt2, &dz, &dcv, &dout};
    for (auto *p : bs) dev_free(*p);
    if (!rc && hout[1]) rc = set_err(ctx, hout[1], "non-finite residual in gmres");
    return rc;
}

// ---- allocation-free triangular solve ----------------------------------------------------------
// Some callers cannot let a solve allocate device memory: a Newmark or Newton loop that has
// already laid out nearly all of HBM for the matrix, the factor and the Krylov basis (an
// allocation there can fail half-way through a run), and callers with work in flight on other
// streams (cudaFree waits for the whole device, so a malloc/free pair around every
// preconditioner apply serialises them).  astro_ldl_solve_device_noalloc serves them: all of its
// operands are the caller's device buffers, and the forward-sweep vector z lives in the fixed
// array below, which is part of the loaded module rather than a runtime allocation.
static __device__ __align__(256) double g_ldl_noalloc_z[ASTRO_LDL_NOALLOC_MAX_DIM];  // 2 MiB

namespace {

// Same sweep as k_ldl_solve; the profile bandwidth is found on the device because the caller's
// row ranges are device memory here.
__global__ void __launch_bounds__(kT) k_ldl_solve_noalloc(double *soln, const double *rhs, const double *L,
                                                          const int *R, int n, double *z) {
    __shared__ int red[32];
    int mb = 0;
    for (int i = threadIdx.x + 1; i <= n; i += blockDim.x) mb = max(mb, R[i] - R[i - 1] - 1);
    for (int o = 16; o; o >>= 1) mb = max(mb, __shfl_xor_sync(0xffffffffu, mb, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mb;
    __syncthreads();
    mb = 0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) mb = max(mb, red[q]);
    ldl_solve(soln, rhs, L, R, n, mb, z);
}

}  // namespace

// The address of the scratch array is looked up on every call, with the context's device current:
// after the first lookup on a device (which may load the module, so make the first call before any
// stream capture begins) it is a table read, and a module loaded again after a device reset is
// never reached through a stale pointer.  Nothing in the scratch needs to start at zero: the
// forward sweep writes z(i) before any row reads it.  The scratch is shared by every context on a
// device, so calls that overlap in time on one device (from several host threads) race on it and
// must be serialised by the caller.
extern "C" int astro_ldl_solve_device_noalloc(astro_ctx *ctx, double *d_soln, const double *d_rhs,
                                              const double *d_l_mat, const int32_t *d_l_range, int32_t l_dim) {
    if (!ctx) return ASTRO_ERR_ARG;
    if (l_dim > ASTRO_LDL_NOALLOC_MAX_DIM)
        return set_err(ctx, ASTRO_ERR_ARG,
                       "l_dim " + std::to_string(l_dim) + " exceeds the allocation-free solve's limit of " +
                           std::to_string(ASTRO_LDL_NOALLOC_MAX_DIM) + " rows; use astro_ldl_solve");
    if (l_dim <= 0 || !d_soln || !d_rhs || !d_l_mat || !d_l_range)
        return set_err(ctx, ASTRO_ERR_ARG, "astro_ldl_solve_device_noalloc: null buffer or l_dim <= 0");
    int prev = -1;
    CK(cudaGetDevice(&prev));
    if (prev != ctx->device) CK(cudaSetDevice(ctx->device));
    void *z = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&z, g_ldl_noalloc_z);
    if (e == cudaSuccess) {
        k_ldl_solve_noalloc<<<1, kT, 0, ctx->stream>>>(d_soln, d_rhs, d_l_mat, d_l_range, l_dim,
                                                      static_cast<double *>(z));
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (prev != ctx->device) cudaSetDevice(prev);
    return cuda_check(ctx, e, "astro_ldl_solve_device_noalloc");
}
