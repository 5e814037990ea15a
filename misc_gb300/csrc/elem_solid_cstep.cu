// Complex step of the solid residual for any design-variable category (brick8 and brickIM):
// the element part of getdRelasticdD (Working/AStrO_commandFunctions.f90:1172-1250) with
// c_getElRu (Working/AStrO_c_elementEqns.f90, the complex twin of r_getElRu's solid branch).
//
// Every element that depends on the design variable d (through elToD, or through ndToD for node
// coordinates) is evaluated in complex FP64 with d + i h, one thread per element:
//   * node coordinates r_getNodeCoord (designProp :945-968): the real offsets of all nodeCoord
//     variables are already in the context's node list; d's own nodes get + i h coef;
//   * orientation r_getOrientation (:187-221): the section orientation rotated (r_rotateAlpha) by
//     the global rotation vector alOrig^T locRot of the element's orientation variables;
//   * C = S^-1 of the engineering constants (r_getMaterialStiffness, :8-80; the real parts of the
//     modulus variables are already in the element's constants) and the density
//     (r_getMaterialDensity, :82-103);
//   * the residual of r_getElRuk's solid branch (Green-Lagrange strain over all shape functions,
//     bubbles included for brickIM) and, for a Newmark state, r_getElRum's solid inertia.
// d_acc -= Im(Ru) at the nodal DOF (internal layout) and d_intAcc -= Im(Ru) at the brickIM
// internal DOF, colour by colour (a colour's elements share no node: no atomics).  The complex
// path's Gauss points are the single-precision 1/sqrt(3) of the reference's c_ constants.
#include "astro_internal.h"
#include "shell_math.cuh"

namespace {

struct SolidCsArgs {
    const int *els;  // listed elements (0-based) of this colour
    int count;
    const int *etype, *elist, *rank, *esec;
    const double *nodes;      // (N,3), real design values applied
    const double *secOrig;    // (S,9) column-major section orientation as given
    const double *elMat;      // (E,9) engineering constants, real design values applied
    const double *rho;        // (E) density, real design values applied
    const int *e2dR, *e2d;    // element design maps
    const double *e2c;
    const int *n2dR, *n2d;    // node design maps (null: none)
    const double *n2c;
    const int *dcat, *dcomp;
    const double *dval;
    int dvar;
    const int *dvars;  // per listed element its design variable (batched form), or null: dvar
    int dvarBase;      // batched form: variable d accumulates at (d - dvarBase) * stride
    long long accStride, intAccStride;
    double h, gpc;
    const int *intVecOff;
    ElemDevState st;
    double *acc, *intAcc;
};

template <class T> __device__ void material_c_cs(const T ep[9], T C[6][6]) {
    T S[6][6];
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) S[i][j] = T(0.0);
    S[0][0] = T(1.0) / ep[0];
    S[0][1] = -ep[3] / ep[0];
    S[0][2] = -ep[4] / ep[0];
    S[1][1] = T(1.0) / ep[1];
    S[1][2] = -ep[5] / ep[1];
    S[2][2] = T(1.0) / ep[2];
    S[3][3] = T(1.0) / ep[6];
    S[4][4] = T(1.0) / ep[7];
    S[5][5] = T(1.0) / ep[8];
    for (int i = 1; i < 6; ++i)
        for (int j = 0; j < i; ++j) S[i][j] = S[j][i];
    // C = S^-1 by the reference's unpivoted LU (r_GetInvLU), column by column
    a_lu<T, 6>(&S[0][0], 6);
    for (int col = 0; col < 6; ++col) {
        T b[6], x[6];
        for (int i = 0; i < 6; ++i) b[i] = (i == col) ? T(1.0) : T(0.0);
        // a_lu_solve handles n <= 9
        a_lu_solve<T, 6>(&S[0][0], b, x, 6);
        for (int i = 0; i < 6; ++i) C[i][col] = x[i];
    }
}

__global__ void k_solid_cstep(SolidCsArgs A) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= A.count) return;
    const int e = A.els[q];
    const int dvar = A.dvars ? A.dvars[q] : A.dvar;
    double *acc = A.dvars ? A.acc + (size_t)(dvar - A.dvarBase) * A.accStride : A.acc;
    double *intAcc = A.intAcc && A.dvars ? A.intAcc + (size_t)(dvar - A.dvarBase) * A.intAccStride : A.intAcc;
    const int et = A.etype[e];
    const int nsf = (et == 81) ? 11 : 8;  // shape functions: nodes (+ bubbles)
    const cplx ih(0.0, A.h);
    // element design-variable terms: modulus, density, orientation
    double epR[9];
    for (int k = 0; k < 9; ++k) epR[k] = A.elMat[9 * (size_t)e + k];
    cplx ep[9];
    for (int k = 0; k < 9; ++k) ep[k] = cplx(epR[k]);
    cplx rho(A.rho[e]);
    double locR[3] = {0.0, 0.0, 0.0};
    cplx locRot[3];
    for (int t = A.e2dR[e]; t < A.e2dR[e + 1]; ++t) {
        const int d = A.e2d[t], cat = A.dcat[d - 1];
        const bool mine = d == dvar;
        if (cat == ASTRO_DCAT_ELASTIC_MODULUS && mine) ep[A.dcomp[d - 1] - 1] += A.e2c[t] * ih;
        if (cat == ASTRO_DCAT_DENSITY && mine) rho += A.e2c[t] * ih;
        if (cat == ASTRO_DCAT_ORIENTATION) {
            const int k = A.dcomp[d - 1] - 1;
            locR[k] += A.e2c[t] * A.dval[d - 1];
            if (mine) locRot[k] += A.e2c[t] * ih;
        }
    }
    for (int k = 0; k < 3; ++k) locRot[k] = locRot[k] + locR[k];
    // orientation: alOrig rotated by globRot = alOrig^T locRot (r_getOrientation)
    cplx orient[3][3];
    {
        const int sec = A.esec[e];
        cplx al[3][3], gr[3];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) al[i][j] = cplx(A.secOrig[9 * (size_t)(sec - 1) + 3 * j + i]);
        for (int i = 0; i < 3; ++i) gr[i] = al[0][i] * locRot[0] + al[1][i] * locRot[1] + al[2][i] * locRot[2];
        a_rotate<cplx>(orient, al, gr, 0, 0);
    }
    cplx C[6][6];
    material_c_cs<cplx>(ep, C);
    // node coordinates (+ i h on d's nodeCoord nodes), local frame; displacement and acceleration
    cplx X[8][3];
    double U[11][3], Ac[11][3];
    const bool dyn = A.st.dynamic != 0;
    const double c1 = dyn ? 0.5 / A.st.beta : 0.0, c2 = dyn ? 2.0 / (A.st.delT * A.st.delT) : 0.0;
    for (int a = 0; a < 8; ++a) {
        const int nd = A.elist[8 * (size_t)e + a];
        cplx g[3];
        for (int k = 0; k < 3; ++k) g[k] = cplx(A.nodes[3 * (size_t)(nd - 1) + k]);
        if (A.n2dR)
            for (int t = A.n2dR[nd - 1]; t < A.n2dR[nd]; ++t) {
                const int d = A.n2d[t];
                if (d == dvar && A.dcat[d - 1] == ASTRO_DCAT_NODE_COORD) g[A.dcomp[d - 1] - 1] += A.n2c[t] * ih;
            }
        for (int i = 0; i < 3; ++i) X[a][i] = orient[i][0] * g[0] + orient[i][1] * g[1] + orient[i][2] * g[2];
        const int r = A.rank[nd - 1] - 1;
        for (int v = 0; v < 3; ++v) {
            const size_t ix = 3 * (size_t)r + v;
            U[a][v] = A.st.disp ? A.st.disp[ix] : 0.0;
            Ac[a][v] = 0.0;
            if (dyn) {
                const double pd = A.st.pdisp ? A.st.pdisp[ix] : 0.0, pv = A.st.pvel ? A.st.pvel[ix] : 0.0,
                             pa = A.st.pacc ? A.st.pacc[ix] : 0.0;
                Ac[a][v] = c1 * (c2 * (U[a][v] - pd - A.st.delT * pv) - (1.0 - 2.0 * A.st.beta) * pa);
            }
        }
    }
    const int ioff = (et == 81) ? A.intVecOff[e] : 0;
    for (int j = 0; j < 3; ++j)
        for (int v = 0; v < 3; ++v) {
            U[8 + j][v] = (et == 81 && A.st.idisp) ? A.st.idisp[ioff + 3 * v + j] : 0.0;
            Ac[8 + j][v] = (et == 81 && dyn)
                               ? c1 * (c2 * (U[8 + j][v] - (A.st.pidisp ? A.st.pidisp[ioff + 3 * v + j] : 0.0)))
                               : 0.0;
        }
    cplx ru[11][3];
    for (int a = 0; a < 11; ++a)
        for (int v = 0; v < 3; ++v) ru[a][v] = cplx(0.0);
    for (int gp = 0; gp < 8; ++gp) {
        const double s1 = (gp & 1) ? A.gpc : -A.gpc, s2 = (gp & 2) ? A.gpc : -A.gpc, s3 = (gp & 4) ? A.gpc : -A.gpc;
        double N[11], Ns[11][3];
        for (int a = 0; a < 8; ++a) {
            const double sa = (a == 1 || a == 2 || a == 5 || a == 6) ? 1.0 : -1.0;
            const double ta = (a == 2 || a == 3 || a == 6 || a == 7) ? 1.0 : -1.0;
            const double ua = (a >= 4) ? 1.0 : -1.0;
            N[a] = 0.125 * (1.0 + sa * s1) * (1.0 + ta * s2) * (1.0 + ua * s3);
            Ns[a][0] = 0.125 * sa * (1.0 + ta * s2) * (1.0 + ua * s3);
            Ns[a][1] = 0.125 * ta * (1.0 + sa * s1) * (1.0 + ua * s3);
            Ns[a][2] = 0.125 * ua * (1.0 + sa * s1) * (1.0 + ta * s2);
        }
        N[8] = 1.0 - s1 * s1;
        N[9] = 1.0 - s2 * s2;
        N[10] = 1.0 - s3 * s3;
        for (int a = 8; a < 11; ++a)
            for (int k = 0; k < 3; ++k) Ns[a][k] = 0.0;
        Ns[8][0] = -s1 - s1;
        Ns[9][1] = -s2 - s2;
        Ns[10][2] = -s3 - s3;
        cplx J[3][3];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                cplx v(0.0);
                for (int a = 0; a < 8; ++a) v += X[a][i] * Ns[a][j];
                J[i][j] = v;
            }
        const cplx a11 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
        const cplx a12 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
        const cplx a13 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
        const cplx det = J[0][0] * a11 + J[0][1] * a12 + J[0][2] * a13;
        const cplx di = cplx(1.0) / det;
        cplx I[3][3];
        I[0][0] = di * a11;
        I[1][0] = di * a12;
        I[2][0] = di * a13;
        I[0][1] = di * (J[0][2] * J[2][1] - J[0][1] * J[2][2]);
        I[1][1] = di * (J[0][0] * J[2][2] - J[0][2] * J[2][0]);
        I[2][1] = di * (J[0][1] * J[2][0] - J[0][0] * J[2][1]);
        I[0][2] = di * (J[0][1] * J[1][2] - J[0][2] * J[1][1]);
        I[1][2] = di * (J[0][2] * J[1][0] - J[0][0] * J[1][2]);
        I[2][2] = di * (J[0][0] * J[1][1] - J[0][1] * J[1][0]);
        cplx g[11][3], ux[3][3];
        double ag[3] = {0.0, 0.0, 0.0};
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) ux[i][j] = cplx(0.0);
        for (int a = 0; a < nsf; ++a) {
            for (int j = 0; j < 3; ++j) g[a][j] = Ns[a][0] * I[0][j] + Ns[a][1] * I[1][j] + Ns[a][2] * I[2][j];
            for (int i = 0; i < 3; ++i) {
                for (int j = 0; j < 3; ++j) ux[i][j] += U[a][i] * g[a][j];
                ag[i] += Ac[a][i] * N[a];
            }
        }
        cplx uxL[3][3];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) uxL[i][j] = orient[i][0] * ux[0][j] + orient[i][1] * ux[1][j] + orient[i][2] * ux[2][j];
        cplx st[6];
        for (int j = 0; j < 3; ++j)
            st[j] = uxL[j][j] + 0.5 * (ux[0][j] * ux[0][j] + ux[1][j] * ux[1][j] + ux[2][j] * ux[2][j]);
        st[3] = uxL[0][1] + uxL[1][0] + ux[0][0] * ux[0][1] + ux[1][0] * ux[1][1] + ux[2][0] * ux[2][1];
        st[4] = uxL[0][2] + uxL[2][0] + ux[0][0] * ux[0][2] + ux[1][0] * ux[1][2] + ux[2][0] * ux[2][2];
        st[5] = uxL[1][2] + uxL[2][1] + ux[0][2] * ux[0][1] + ux[1][2] * ux[1][1] + ux[2][2] * ux[2][1];
        cplx sw[6];
        for (int i = 0; i < 6; ++i) {
            cplx s(0.0);
            for (int k = 0; k < 6; ++k) s += C[i][k] * st[k];
            sw[i] = det * s;  // unit Gauss weights
        }
        cplx Gm[3][3];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) Gm[i][j] = orient[i][j] + ux[j][i];
        for (int a = 0; a < nsf; ++a) {
            const cplx g0 = g[a][0], g1 = g[a][1], g2 = g[a][2];
            // P = Bloc(g) G, residual P^T (w detJ stress)
            for (int v = 0; v < 3; ++v) {
                const cplx P0 = g0 * Gm[0][v], P1 = g1 * Gm[1][v], P2 = g2 * Gm[2][v];
                const cplx P3 = g1 * Gm[0][v] + g0 * Gm[1][v], P4 = g2 * Gm[0][v] + g0 * Gm[2][v],
                           P5 = g2 * Gm[1][v] + g1 * Gm[2][v];
                ru[a][v] += P0 * sw[0] + P1 * sw[1] + P2 * sw[2] + P3 * sw[3] + P4 * sw[4] + P5 * sw[5];
                if (dyn && a < 8) ru[a][v] += (rho * det) * (ag[v] * N[a]);
            }
        }
    }
    for (int a = 0; a < 8; ++a) {
        const int r = A.rank[A.elist[8 * (size_t)e + a] - 1] - 1;
        for (int v = 0; v < 3; ++v) acc[3 * (size_t)r + v] -= ru[a][v].im;
    }
    if (et == 81 && intAcc)
        for (int j = 0; j < 3; ++j)
            for (int v = 0; v < 3; ++v) intAcc[ioff + 3 * v + j] -= ru[8 + j][v].im;
}

}  // namespace

// The solid elements that depend on dvar (through elToD, or through the nodeCoord terms of their
// nodes), grouped by colour.
static void solid_dvar_elements(const astro_ctx *ctx, int dvar, std::vector<int> &list, std::vector<int> &ptr) {
    const AstroPrep &P = ctx->P;
    std::vector<char> nodeDep;
    if (!ctx->n2dRange.empty() && ctx->dCat[dvar - 1] == ASTRO_DCAT_NODE_COORD) {
        nodeDep.assign((size_t)P.N + 1, 0);
        for (int nd = 1; nd <= P.N; ++nd)
            for (int q = ctx->n2dRange[nd - 1]; q < ctx->n2dRange[nd]; ++q)
                if (ctx->n2d[q] == dvar) nodeDep[nd] = 1;
    }
    list.clear();
    ptr.assign(1, 0);
    for (int col = 0; col < P.ncolors; ++col) {
        for (int k = P.colorPtr[col]; k < P.colorPtr[col + 1]; ++k) {
            const int e = P.colorEls[k];
            bool dep = false;
            for (int q = ctx->e2dRange[e]; q < ctx->e2dRange[e + 1]; ++q) dep = dep || ctx->e2d[q] == dvar;
            if (!nodeDep.empty())
                for (int a = 0; a < 8; ++a) dep = dep || nodeDep[ctx->elist[8 * (size_t)e + a]];
            if (dep) list.push_back(e);
        }
        ptr.push_back((int)list.size());
    }
}

static SolidCsArgs solid_cs_args(astro_ctx *ctx, int dvar, double h, const ElemDevState &s, double *d_acc,
                                 double *d_intAcc) {
    SolidCsArgs A;
    A.etype = dptr<int>(ctx->d_etype);
    A.elist = dptr<int>(ctx->d_elist);
    A.rank = dptr<int>(ctx->d_rank);
    A.esec = dptr<int>(ctx->d_esec);
    A.nodes = dptr<double>(ctx->d_nodes);
    A.secOrig = dptr<double>(ctx->d_secOrig);
    A.elMat = dptr<double>(ctx->d_elMat);
    A.rho = dptr<double>(ctx->d_elRho);
    A.e2dR = dptr<int>(ctx->d_e2dR);
    A.e2d = dptr<int>(ctx->d_e2d);
    A.e2c = dptr<double>(ctx->d_e2c);
    A.n2dR = ctx->n2dRange.empty() ? nullptr : dptr<int>(ctx->d_n2dR);
    A.n2d = ctx->n2dRange.empty() ? nullptr : dptr<int>(ctx->d_n2d);
    A.n2c = ctx->n2dRange.empty() ? nullptr : dptr<double>(ctx->d_n2c);
    A.dcat = dptr<int>(ctx->d_dCat);
    A.dcomp = dptr<int>(ctx->d_dComp);
    A.dval = dptr<double>(ctx->d_dVal);
    A.dvar = dvar;
    A.h = h;
    A.gpc = LIT(0.577350269189626);  // c_1rt3, a single-precision literal
    A.intVecOff = dptr<int>(ctx->d_intVecOff);
    A.st = s;
    A.acc = d_acc;
    A.intAcc = d_intAcc;
    A.dvars = nullptr;
    A.dvarBase = 1;
    A.accStride = A.intAccStride = 0;
    return A;
}

int solid_drdd(astro_ctx *ctx, int dvar, double h, const ElemDevState &s, double *d_acc, double *d_intAcc) {
    std::vector<int> list, ptr;
    solid_dvar_elements(ctx, dvar, list, ptr);
    if (list.empty()) return ASTRO_OK;
    DevBuf dl;
    int rc;
    if ((rc = upload(ctx, dl, list.data(), sizeof(int) * list.size()))) return rc;
    SolidCsArgs A = solid_cs_args(ctx, dvar, h, s, d_acc, d_intAcc);
    for (size_t col = 0; col + 1 < ptr.size(); ++col) {
        const int cnt = ptr[col + 1] - ptr[col];
        if (!cnt) continue;
        A.els = dptr<int>(dl) + ptr[col];
        A.count = cnt;
        k_solid_cstep<<<(cnt + 63) / 64, 64, 0, ctx->stream>>>(A);
    }
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    dev_free(dl);
    return cuda_check(ctx, e, "solid complex-step kernel");
}

// Design variables d0 .. d0+nd-1 at once: one launch per colour over the (element, variable) pairs
// of that colour, variable d accumulating at d_acc + (d-d0) n (and d_intAcc + (d-d0) ni).  Each
// variable's accumulator receives its elements' terms in the same colour order as solid_drdd,
// so the results are the same; the launches are nd times wider.
int solid_drdd_batch(astro_ctx *ctx, int d0, int nd, double h, const ElemDevState &s, double *d_acc,
                     double *d_intAcc) {
    const int ncol = ctx->P.ncolors;
    std::vector<std::vector<int>> els(ncol), dvs(ncol);
    for (int d = d0; d < d0 + nd; ++d) {
        std::vector<int> list, ptr;
        solid_dvar_elements(ctx, d, list, ptr);
        for (int col = 0; col + 1 < (int)ptr.size(); ++col)
            for (int k = ptr[col]; k < ptr[col + 1]; ++k) {
                els[col].push_back(list[k]);
                dvs[col].push_back(d);
            }
    }
    std::vector<int> all, allD, start(1, 0);
    for (int col = 0; col < ncol; ++col) {
        all.insert(all.end(), els[col].begin(), els[col].end());
        allD.insert(allD.end(), dvs[col].begin(), dvs[col].end());
        start.push_back((int)all.size());
    }
    if (all.empty()) return ASTRO_OK;
    DevBuf dl, dd;
    int rc;
    if ((rc = upload(ctx, dl, all.data(), sizeof(int) * all.size())) ||
        (rc = upload(ctx, dd, allD.data(), sizeof(int) * allD.size())))
        return rc;
    SolidCsArgs A = solid_cs_args(ctx, 0, h, s, d_acc, d_intAcc);
    A.dvarBase = d0;
    A.accStride = ctx->P.n;
    A.intAccStride = ctx->P.intVecSize;
    for (int col = 0; col < ncol; ++col) {
        const int cnt = start[col + 1] - start[col];
        if (!cnt) continue;
        A.els = dptr<int>(dl) + start[col];
        A.dvars = dptr<int>(dd) + start[col];
        A.count = cnt;
        k_solid_cstep<<<(cnt + 63) / 64, 64, 0, ctx->stream>>>(A);
    }
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    dev_free(dl);
    dev_free(dd);
    return cuda_check(ctx, e, "solid complex-step kernel (batched)");
}

namespace {

// r_getOrientation (Working/AStrO_r_designPropertyFunctions.f90:187-221) with the real values of
// the element's orientation design variables: the section frame rotated by alOrig^T locRot.
__global__ void k_solid_orient(int E, const int *__restrict__ esec, const double *__restrict__ secOrig,
                               const int *__restrict__ e2dR, const int *__restrict__ e2d, const double *__restrict__ e2c,
                               const int *__restrict__ dcat, const int *__restrict__ dcomp,
                               const double *__restrict__ dval, double *__restrict__ orientEl) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    double locRot[3] = {0.0, 0.0, 0.0};
    for (int t = e2dR[e]; t < e2dR[e + 1]; ++t) {
        const int d = e2d[t];
        if (dcat[d - 1] == ASTRO_DCAT_ORIENTATION) locRot[dcomp[d - 1] - 1] += e2c[t] * dval[d - 1];
    }
    const int sec = esec[e];
    double al[3][3], gr[3], out[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) al[i][j] = secOrig[9 * (size_t)(sec - 1) + 3 * j + i];
    for (int i = 0; i < 3; ++i) gr[i] = al[0][i] * locRot[0] + al[1][i] * locRot[1] + al[2][i] * locRot[2];
    a_rotate<double>(out, al, gr, 0, 0);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) orientEl[9 * (size_t)e + 3 * j + i] = out[i][j];
}

}  // namespace

int solid_orient_prepare(astro_ctx *ctx) {
    const int E = ctx->P.E;
    k_solid_orient<<<(E + 127) / 128, 128, 0, ctx->stream>>>(
        E, dptr<int>(ctx->d_esec), dptr<double>(ctx->d_secOrig), dptr<int>(ctx->d_e2dR), dptr<int>(ctx->d_e2d),
        dptr<double>(ctx->d_e2c), dptr<int>(ctx->d_dCat), dptr<int>(ctx->d_dComp), dptr<double>(ctx->d_dVal),
        dptr<double>(ctx->d_secOrient));
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    return cuda_check(ctx, e, "solid orientation design variables");
}
