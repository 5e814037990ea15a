// Block-CSR utilities: zeroing, export to the reference's scalar CSR (elasticMat/elMatCols in
// find-or-insert order, Working/AStrO_commandFunctions.f90:323-347), max |K| for the constraint
// scaling (scaleElasticMPC, :537-566), vector layout changes between the reference's
// component-major DOF numbering and the rank-major device layout, and the consistent surface
// load (intended semantics of r_getElSurfaceTraction, Working/AStrO_r_elementEqns.f90:1923-2018).
#include <algorithm>
#include <vector>

#include "astro_internal.h"

namespace {

__global__ void export_csr_kernel(const double *__restrict__ K, const int *__restrict__ bRow,
                                  const int *__restrict__ bCol, const int *__restrict__ csrPos,
                                  const int *__restrict__ elMatRange, int nb, int dpn, int N,
                                  double *__restrict__ mat, int *__restrict__ cols) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long total = (long long)nb * dpn * dpn;
    if (t >= total) return;
    const int k = (int)(t / (dpn * dpn));
    const int ij = (int)(t % (dpn * dpn));
    const int i = ij / dpn, j = ij % dpn;
    const int ra = bRow[k], rb = bCol[k];
    const int dofRow = ra + 1 + i * N;  // 1-based reference DOF
    const long long idx = (long long)elMatRange[dofRow - 1] + csrPos[(long long)k * dpn + j];
    if (mat) mat[idx] = K[t];
    if (cols) cols[idx] = rb + 1 + j * N;
}

template <class T>
__global__ void absmax_kernel(const T *__restrict__ v, long long n, unsigned long long *out) {
    double m = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        m = fmax(m, fabs((double)v[i]));
    for (int o = 16; o; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    __shared__ double s[32];
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        m = (threadIdx.x < (blockDim.x >> 5)) ? s[threadIdx.x] : 0.0;
        for (int o = 16; o; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
        // non-negative doubles order like their bit patterns
        if (threadIdx.x == 0) atomicMax(out, (unsigned long long)__double_as_longlong(m));
    }
}

// ref (component-major, 0-based index d = (c)*N + r) <-> internal (r*dpn + c)
__global__ void ref_to_int_kernel(const double *__restrict__ ref, double *__restrict__ out, int N, int dpn) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= N * dpn) return;
    const int r = t / dpn, c = t % dpn;
    out[t] = ref[(size_t)c * N + r];
}
__global__ void int_to_ref_kernel(const double *__restrict__ in, double *__restrict__ ref, int N, int dpn) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= N * dpn) return;
    const int r = t % N, c = t / N;
    ref[t] = in[(size_t)r * dpn + c];
}

// getElasticConstraintLoad (Working/AStrO_commandFunctions.f90:506-535): load += C^T (rhs - C u)
// with the scaled constraints in internal numbering (col < 0: empty slot).  First the row
// residuals t = rhs - C u (thread per row), then the scatter as a gather per target DOF: gPtr/gTerm
// list, for each constrained DOF gRow[g], its terms in the reference's row-and-term order.
__global__ void constraint_rows_kernel(int mdim, const int *__restrict__ range, const int *__restrict__ col,
                                       const double *__restrict__ val, const double *__restrict__ rhs,
                                       const double *__restrict__ u, double *__restrict__ t) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= mdim) return;
    double s = rhs[r];
    if (u)
        for (int k = range[r]; k < range[r + 1]; ++k)
            if (col[k] >= 0) s -= val[k] * u[col[k]];
    t[r] = s;
}
__global__ void constraint_gather_kernel(int ng, const int *__restrict__ gPtr, const int *__restrict__ gTerm,
                                         const int *__restrict__ gRow, const int *__restrict__ termRow,
                                         const double *__restrict__ val, const double *__restrict__ t,
                                         double *__restrict__ load) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ng) return;
    double s = load[gRow[g]];
    for (int q = gPtr[g]; q < gPtr[g + 1]; ++q) {
        const int k = gTerm[q];
        s += val[k] * t[termRow[k]];
    }
    load[gRow[g]] = s;
}

// Consistent face load.  One thread per face forms the face's nodal forces (summed over its
// Gauss points) and their target rows; faces of one call may share nodes, so a second kernel adds
// them into the load in face order (deterministic).
__global__ void surface_load_kernel(const double *__restrict__ nodes, const int *__restrict__ elist,
                                    const int *__restrict__ etype, const int *__restrict__ rank, int nf,
                                    const int *__restrict__ faceEl, const int *__restrict__ faceNum, double t0,
                                    double t1, double t2, double pressure, int dpn, double *__restrict__ fval,
                                    int *__restrict__ frow) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    const int hexF[6][4] = {{4, 3, 2, 1}, {5, 6, 7, 8}, {1, 2, 6, 5}, {2, 3, 7, 6}, {3, 4, 8, 7}, {4, 1, 5, 8}};
    const int shF[2][4] = {{1, 2, 3, 4}, {1, 4, 3, 2}};
    const int el = faceEl[f] - 1, fn = faceNum[f] - 1;
    const int *fl = (etype[el] == 8 || etype[el] == 81) ? hexF[fn] : shF[fn];
    double X[4][3];
    int nd[4];
    for (int k = 0; k < 4; ++k) {
        nd[k] = elist[8 * el + fl[k] - 1];
        for (int d = 0; d < 3; ++d) X[k][d] = nodes[3 * (nd[k] - 1) + d];
    }
    double v1[3], v2[3], nv[3];
    for (int d = 0; d < 3; ++d) {
        v1[d] = X[2][d] - X[0][d];
        v2[d] = X[3][d] - X[1][d];
    }
    nv[0] = v1[1] * v2[2] - v1[2] * v2[1];
    nv[1] = v1[2] * v2[0] - v1[0] * v2[2];
    nv[2] = v1[0] * v2[1] - v1[1] * v2[0];
    const double inv = 1.0 / sqrt(nv[0] * nv[0] + nv[1] * nv[1] + nv[2] * nv[2]);
    const double tr[3] = {t0 - pressure * nv[0] * inv, t1 - pressure * nv[1] * inv, t2 - pressure * nv[2] * inv};
    const double g = 0.57735026918962576451;
    double acc[4][3] = {};
    for (int gp = 0; gp < 4; ++gp) {
        const double s = (gp & 1) ? g : -g, r = (gp & 2) ? g : -g;
        const double N_[4] = {0.25 * (1 - s) * (1 - r), 0.25 * (1 + s) * (1 - r), 0.25 * (1 + s) * (1 + r),
                              0.25 * (1 - s) * (1 + r)};
        const double Ns[4] = {-0.25 * (1 - r), 0.25 * (1 - r), 0.25 * (1 + r), -0.25 * (1 + r)};
        const double Nr[4] = {-0.25 * (1 - s), -0.25 * (1 + s), 0.25 * (1 + s), 0.25 * (1 - s)};
        double a[3] = {0, 0, 0}, b[3] = {0, 0, 0};
        for (int k = 0; k < 4; ++k)
            for (int d = 0; d < 3; ++d) {
                a[d] += Ns[k] * X[k][d];
                b[d] += Nr[k] * X[k][d];
            }
        const double cx = a[1] * b[2] - a[2] * b[1], cy = a[2] * b[0] - a[0] * b[2], cz = a[0] * b[1] - a[1] * b[0];
        const double dA = sqrt(cx * cx + cy * cy + cz * cz);
        for (int k = 0; k < 4; ++k)
            for (int d = 0; d < 3; ++d) acc[k][d] += tr[d] * N_[k] * dA;
    }
    for (int k = 0; k < 4; ++k) {
        frow[4 * f + k] = (rank[nd[k] - 1] - 1) * dpn;
        for (int d = 0; d < 3; ++d) fval[12 * f + 3 * k + d] = acc[k][d];
    }
}

// adds the face forces into the load, one thread per target node, in face order (gPtr/gSlot list
// for node row gRow[g] its (face, corner) slots f*4 + k in increasing face order)
__global__ void face_gather_kernel(int ng, const int *__restrict__ gPtr, const int *__restrict__ gSlot,
                                   const int *__restrict__ gRow, const double *__restrict__ fval,
                                   double *__restrict__ loadInt) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ng) return;
    const int row = gRow[g];
    double s0 = loadInt[row], s1 = loadInt[row + 1], s2 = loadInt[row + 2];
    for (int q = gPtr[g]; q < gPtr[g + 1]; ++q) {
        const int sl = gSlot[q];
        s0 += fval[3 * sl];
        s1 += fval[3 * sl + 1];
        s2 += fval[3 * sl + 2];
    }
    loadInt[row] = s0;
    loadInt[row + 1] = s1;
    loadInt[row + 2] = s2;
}


}  // namespace

int bsr_zero(astro_ctx *ctx, int which) {
    const size_t nv = (size_t)ctx->P.nb * ctx->P.dpn * ctx->P.dpn;
    if ((which & 1) && ctx->d_K32.p) CK(cudaMemsetAsync(ctx->d_K32.p, 0, nv * sizeof(float), ctx->stream));
    if ((which & 2) && ctx->d_K64.p) CK(cudaMemsetAsync(ctx->d_K64.p, 0, nv * sizeof(double), ctx->stream));
    return ASTRO_OK;
}

// The reference CSR (values in d_mat and/or column numbers in d_cols, device buffers of
// elMatSize) from the block-CSR matrix, on stream s.  The column numbers depend on the mesh only.
int export_csr_dev(astro_ctx *ctx, cudaStream_t s, double *d_mat, int *d_cols) {
    const AstroPrep &P = ctx->P;
    const long long total = (long long)P.nb * P.dpn * P.dpn;
    export_csr_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(
        dptr<double>(ctx->d_K64), dptr<int>(ctx->d_bRow), dptr<int>(ctx->d_bCol), dptr<int>(ctx->d_csrPos),
        dptr<int>(ctx->d_elMatRangeRank), P.nb, P.dpn, P.N, d_mat, d_cols);
    return cuda_check(ctx, cudaGetLastError(), "export_csr");
}

// max |K| of the FP64 (kind 64) or FP32 (kind 32) block-CSR values
double bsr_absmax(astro_ctx *ctx, int *status, int kind) {
    const long long nv = (long long)ctx->P.nb * ctx->P.dpn * ctx->P.dpn;
    unsigned long long *d = dptr<unsigned long long>(ctx->d_status) + 1;
    unsigned long long h = 0;
    cudaMemsetAsync(d, 0, sizeof(unsigned long long), ctx->stream);
    if (kind == 64)
        absmax_kernel<double><<<4 * 152, 256, 0, ctx->stream>>>(dptr<double>(ctx->d_K64), nv, d);
    else
        absmax_kernel<float><<<4 * 152, 256, 0, ctx->stream>>>(dptr<float>(ctx->d_K32), nv, d);
    cudaError_t e = cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    *status = (e == cudaSuccess) ? ASTRO_OK : cuda_check(ctx, e, "absmax");
    double v;
    long long bits = (long long)h;
    memcpy(&v, &bits, sizeof(v));
    return v;
}

int constraint_load_dev(astro_ctx *ctx, const double *d_u, double *d_loadInt) {
    const int md = ctx->P.mpcDim;
    if (md == 0) return ASTRO_OK;
    if (!ctx->d_mpcVal.p) return set_err(ctx, ASTRO_ERR_STATE, "astro_scale_mpc must run first");
    constraint_rows_kernel<<<(md + 255) / 256, 256, 0, ctx->stream>>>(
        md, dptr<int>(ctx->d_mpcRange), dptr<int>(ctx->d_mpcCol), dptr<double>(ctx->d_mpcVal), dptr<double>(ctx->d_mpcRhs),
        d_u, dptr<double>(ctx->d_mpcT));
    const int ng = ctx->mpcTargets;
    constraint_gather_kernel<<<(ng + 255) / 256, 256, 0, ctx->stream>>>(
        ng, dptr<int>(ctx->d_mpcGPtr), dptr<int>(ctx->d_mpcGTerm), dptr<int>(ctx->d_mpcGRow), dptr<int>(ctx->d_mpcTermRow),
        dptr<double>(ctx->d_mpcVal), dptr<double>(ctx->d_mpcT), d_loadInt);
    return cuda_check(ctx, cudaGetLastError(), "constraint load");
}

int ref_to_int_vec(astro_ctx *ctx, const double *d_ref, double *d_int, int n) {
    ref_to_int_kernel<<<(n + 255) / 256, 256, 0, ctx->stream>>>(d_ref, d_int, ctx->P.N, ctx->P.dpn);
    return cuda_check(ctx, cudaGetLastError(), "ref_to_int");
}

int int_to_ref_vec(astro_ctx *ctx, const double *d_int, double *d_ref, int n) {
    int_to_ref_kernel<<<(n + 255) / 256, 256, 0, ctx->stream>>>(d_int, d_ref, ctx->P.N, ctx->P.dpn);
    return cuda_check(ctx, cudaGetLastError(), "int_to_ref");
}

int surface_load_dev(astro_ctx *ctx, int nf, const int *d_faceEl, const int *d_faceNum, const double *tr,
                     double pressure, double *d_loadInt) {
    if (nf <= 0) return ASTRO_OK;
    DevBuf fv, fr;
    int rc;
    if ((rc = dev_alloc(ctx, fv, sizeof(double) * 12 * (size_t)nf))) return rc;
    if ((rc = dev_alloc(ctx, fr, sizeof(int) * 4 * (size_t)nf))) {
        dev_free(fv);
        return rc;
    }
    surface_load_kernel<<<(nf + 127) / 128, 128, 0, ctx->stream>>>(
        dptr<double>(ctx->d_nodes), dptr<int>(ctx->d_elist), dptr<int>(ctx->d_etype), dptr<int>(ctx->d_rank), nf,
        d_faceEl, d_faceNum, tr[0], tr[1], tr[2], pressure, ctx->P.dpn, dptr<double>(fv), dptr<int>(fr));
    // gather lists: the (face, corner) slots of every target row, in face order
    std::vector<int> hrow(4 * (size_t)nf);
    cudaError_t e = cudaMemcpyAsync(hrow.data(), fr.p, sizeof(int) * hrow.size(), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    DevBuf gp, gs, gr;
    if (e == cudaSuccess) {
        std::vector<int> order(hrow.size());
        for (size_t q = 0; q < order.size(); ++q) order[q] = (int)q;
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return hrow[a] < hrow[b]; });
        std::vector<int> ptr(1, 0), row;
        for (size_t q = 0; q < order.size(); ++q) {
            if (q == 0 || hrow[order[q]] != hrow[order[q - 1]]) {
                if (q) ptr.push_back((int)q);
                row.push_back(hrow[order[q]]);
            }
        }
        ptr.push_back((int)order.size());
        const int ng = (int)row.size();
        if (!(rc = upload(ctx, gp, ptr.data(), sizeof(int) * ptr.size())) &&
            !(rc = upload(ctx, gs, order.data(), sizeof(int) * order.size())) &&
            !(rc = upload(ctx, gr, row.data(), sizeof(int) * row.size()))) {
            face_gather_kernel<<<(ng + 127) / 128, 128, 0, ctx->stream>>>(ng, dptr<int>(gp), dptr<int>(gs), dptr<int>(gr),
                                                                         dptr<double>(fv), d_loadInt);
            e = cudaGetLastError();
            if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        }
    }
    DevBuf *bufs[] = {&fv, &fr, &gp, &gs, &gr};
    for (auto *b : bufs) dev_free(*b);
    if (rc) return rc;
    return cuda_check(ctx, e, "surface_load");
}
