// Thermal path: heat conduction (and capacitance in transient steps) of the brick8 and shell4
// elements, assembly into the reference's thermal CSR, thermal constraints, heat generation and a
// device solve.
//
// Reference: getThermalSolnLoad (Working/AStrO_commandFunctions.f90:16-72), r_getElRt /
// r_getElRtk / r_getElRtm (Working/AStrO_r_elementEqns.f90:2062-2204), the conductivity and
// specific heat staging (Working/AStrO_r_designPropertyFunctions.f90:129-186, 527-644),
// getThermalAppliedLoad's bodyHeatGen branch (commandFunctions :78-139, through r_getElBodyForce),
// getThermalConstraintLoad / scaleThermalMPC (:197-258), buildThermalMPC
// (Working/AStrO_bookKeeping.f90:614-752) and allocateThermalMat (:413-472).
//
// GB300 mapping: one DOF per node, so the thermal matrix lives as the values of the model's
// node-block pattern with 1 x 1 blocks, in rank order (the reference numbers thermal DOF by
// currentRank too).  Element kernels run one thread per element, colour by colour (no atomics,
// fixed summation order); the property stage (per element conductivity in the element frame,
// heat capacity, shell thickness) runs once per thermal setup.  The solve is a Jacobi-
// preconditioned conjugate gradient in FP64 on K_T + C^T C with its scalars kept on the device.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <vector>

#include "astro_internal.h"
#include "shell_props.cuh"

namespace {

constexpr int kProps = 11;  // per element: conductivity 3x3 row-major, heat capacity, thickness

struct ThermPlan {
    int nMat = 0;
    DevBuf d_props, d_val, d_pos, d_rowStart, d_elMatId, d_matCond, d_matSH, d_layCond, d_laySH;
    int matSize = 0, haveMat = 0;
    // constraints: rows of (internal column, coefficient), unscaled and scaled
    int mpcDim = 0;
    std::vector<int> mRange, mCol;
    std::vector<double> mVal, mRhs, sVal, sRhs;
    int scaled = 0;
    DevBuf d_mRange, d_mCol, d_sVal, d_sRhs, d_penPtr, d_penCol, d_penVal;
    int penCount = 0;
    std::vector<int> rowStart;  // thermMatRange(0:N)
};

ThermPlan *plan_of(astro_ctx *ctx) { return static_cast<ThermPlan *>(ctx->thermal); }

// Inputs of the per-element thermal properties: the material (solids) or layer (shells) values
// as given, and the element design-variable maps.
struct ThPropArgs {
    int shell;
    const int *esec, *elMatId;
    const double *elDen;  // solid density, the real density design terms applied
    const double *matCond, *matSH;
    const int *layRange;
    const LayerDev *lay;
    const double *layCond, *laySH;
    const int *e2dR, *e2d;  // null: no design variables
    const double *e2c;
    const int *dcat, *dlay, *dcomp;
    const double *dval;
};

// One element's thermal properties with its design-variable terms, + i h on variable `pert`
// (0 = none): the conductivity tc in the element frame, the heat capacity sh (density x specific
// heat; per area for shells, the layers summed) and the shell section thickness secT.  Solids:
// r_getMaterialThermCond / r_getMaterialSpecHeat (Working/AStrO_r_designPropertyFunctions.f90:129-186)
// and r_getMaterialDensity (:82-103); shells: r_getShellThermCond / r_getShellSpecHeat
// (:527-644), every layer's conductivity, specific heat, density, thickness and angle with its
// 'layup' terms.  Each value takes its terms one at a time in the element's term order.
template <class T>
__device__ void th_props_t(const ThPropArgs &A, int e, int pert, double h, T tc[3][3], T &sh, T &secT) {
    auto add_terms = [&](T &v, int cat, int layerNum, int comp) {
        if (!A.e2dR) return;
        for (int q = A.e2dR[e]; q < A.e2dR[e + 1]; ++q) {
            const int d = A.e2d[q] - 1;
            if (A.dcat[d] != cat || (layerNum && A.dlay[d] != layerNum) || (comp && A.dcomp[d] != comp)) continue;
            T dv = T(A.dval[d]);
            if (d + 1 == pert) dv = dv + pert_i<T>(h);
            v = v + A.e2c[q] * dv;
        }
    };
    auto fill = [](T t[3][3], const T *v) {
        t[0][0] = v[0];
        t[1][1] = v[1];
        t[2][2] = v[2];
        t[0][1] = t[1][0] = v[3];
        t[0][2] = t[2][0] = v[4];
        t[1][2] = t[2][1] = v[5];
    };
    if (!A.shell) {
        const int mat = A.elMatId[e];
        T cv[6];
        for (int k = 0; k < 6; ++k) {
            cv[k] = T(A.matCond[6 * (mat - 1) + k]);
            add_terms(cv[k], ASTRO_DCAT_THERMAL_COND, 0, k + 1);
        }
        fill(tc, cv);
        T rho = T(A.elDen[e]);
        if (pert && A.e2dR)
            for (int q = A.e2dR[e]; q < A.e2dR[e + 1]; ++q)
                if (A.e2d[q] == pert && A.dcat[pert - 1] == ASTRO_DCAT_DENSITY) rho = rho + A.e2c[q] * pert_i<T>(h);
        T spec = T(A.matSH[mat - 1]);
        add_terms(spec, ASTRO_DCAT_SPEC_HEAT, 0, 0);
        sh = rho * spec;
        secT = T(0.0);
        return;
    }
    const int sec = A.esec[e];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) tc[i][j] = T(0.0);
    sh = T(0.0);
    secT = T(0.0);
    for (int li = A.layRange[sec - 1], ln = 1; li < A.layRange[sec]; ++li, ++ln) {
        const LayerDev L = A.lay[li];
        T t = T(L.t), ang = T(L.angle), rho = T(L.rho), spec = T(A.laySH[li]), cv[6];
        add_terms(t, ASTRO_DCAT_LAYUP_THICKNESS, ln, 0);
        add_terms(ang, ASTRO_DCAT_LAYUP_ANGLE, ln, 0);
        add_terms(rho, ASTRO_DCAT_LAYUP_DENSITY, ln, 0);
        add_terms(spec, ASTRO_DCAT_LAYUP_SPEC_HEAT, ln, 0);
        for (int k = 0; k < 6; ++k) {
            cv[k] = T(A.layCond[6 * li + k]);
            add_terms(cv[k], ASTRO_DCAT_LAYUP_THERMAL_COND, ln, k + 1);
        }
        T tl[3][3], al[3][3], pr[3][3];
        fill(tl, cv);
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) al[i][j] = T(0.0);
        al[2][2] = T(1.0);
        al[0][0] = a_cos(ang);
        al[1][0] = a_sin(ang);
        al[0][1] = -al[1][0];
        al[1][1] = al[0][0];
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                T v = T(0.0);
                for (int k = 0; k < 3; ++k) v = v + tl[a][k] * al[b][k];
                pr[a][b] = v;
            }
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                T v = T(0.0);
                for (int k = 0; k < 3; ++k) v = v + al[a][k] * pr[k][b];
                tc[a][b] = tc[a][b] + t * v;
            }
        sh = sh + t * rho * spec;
        secT = secT + t;
    }
}

// per element: conductivity in the element frame, heat capacity and shell thickness (real values
// of the design variables applied)
__global__ void k_th_props(ThPropArgs A, int E, double *__restrict__ out) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    double tc[3][3], sh, secT;
    th_props_t<double>(A, e, 0, 0.0, tc, sh, secT);
    double *o = out + (size_t)kProps * e;
    for (int i = 0; i < 9; ++i) o[i] = tc[i / 3][i % 3];
    o[9] = sh;
    o[10] = secT;
}

// Gauss point g of the element: shape functions, their global gradient in the element frame and
// w detJ (r_getIntPtData; shells with dxds(3,3) = 1).  r3 is the Gauss abscissa (the real path's
// 1/sqrt(3) or the complex path's single-precision literal); the shape functions are real, the
// geometry T.
template <class T>
__device__ __forceinline__ void th_point_t(int shell, const T Xl[8][3], double r3, int g, double N[8], T Nx[8][3],
                                           T &wdet) {
    const int npe = shell ? 4 : 8;
    double dN[8][3];
    if (shell) {
        const double s1 = (g & 1) ? r3 : -r3, s2 = (g & 2) ? r3 : -r3;
        const double sx[4] = {-1.0, 1.0, 1.0, -1.0}, sy[4] = {-1.0, -1.0, 1.0, 1.0};
        for (int n = 0; n < 4; ++n) {
            N[n] = 0.25 * (1.0 + sx[n] * s1) * (1.0 + sy[n] * s2);
            dN[n][0] = 0.25 * sx[n] * (1.0 + sy[n] * s2);
            dN[n][1] = 0.25 * sy[n] * (1.0 + sx[n] * s1);
            dN[n][2] = 0.0;
        }
    } else {
        const double s1 = (g & 1) ? r3 : -r3, s2 = (g & 2) ? r3 : -r3, s3 = (g & 4) ? r3 : -r3;
        const double sx[8] = {-1, 1, 1, -1, -1, 1, 1, -1}, sy[8] = {-1, -1, 1, 1, -1, -1, 1, 1},
                     sz[8] = {-1, -1, -1, -1, 1, 1, 1, 1};
        for (int n = 0; n < 8; ++n) {
            const double a1 = 1.0 + sx[n] * s1, a2 = 1.0 + sy[n] * s2, a3 = 1.0 + sz[n] * s3;
            N[n] = 0.125 * a1 * a2 * a3;
            dN[n][0] = 0.125 * sx[n] * a2 * a3;
            dN[n][1] = 0.125 * sy[n] * a1 * a3;
            dN[n][2] = 0.125 * sz[n] * a1 * a2;
        }
    }
    T J[3][3];
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            T s = T(0.0);
            for (int n = 0; n < npe; ++n) s = s + Xl[n][a] * dN[n][b];
            J[a][b] = s;
        }
    if (shell) J[2][2] = T(1.0);
    const T c11 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
    const T c12 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
    const T c13 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
    const T det = J[0][0] * c11 + J[0][1] * c12 + J[0][2] * c13;
    const T di = T(1.0) / det;
    T I[3][3];
    I[0][0] = di * c11;
    I[1][0] = di * c12;
    I[2][0] = di * c13;
    I[0][1] = di * (J[0][2] * J[2][1] - J[0][1] * J[2][2]);
    I[1][1] = di * (J[0][0] * J[2][2] - J[0][2] * J[2][0]);
    I[2][1] = di * (J[0][1] * J[2][0] - J[0][0] * J[2][1]);
    I[0][2] = di * (J[0][1] * J[1][2] - J[0][2] * J[1][1]);
    I[1][2] = di * (J[0][2] * J[1][0] - J[0][0] * J[1][2]);
    I[2][2] = di * (J[0][0] * J[1][1] - J[0][1] * J[1][0]);
    for (int n = 0; n < npe; ++n)
        for (int b = 0; b < 3; ++b) Nx[n][b] = dN[n][0] * I[0][b] + dN[n][1] * I[1][b] + dN[n][2] * I[2][b];
    wdet = det;  // unit weights
}

__device__ __forceinline__ void th_point(int shell, const double Xl[8][3], int g, double N[8], double Nx[8][3],
                                         double &wdet) {
    th_point_t<double>(shell, Xl, AK<double>::rt3, g, N, Nx, wdet);
}

struct ThArgs {
    const double *nodes, *orient;  // bricks: per element column-major; shells: ShellProps
    const ShellProps *sprops;
    const int *elist, *rank, *els, *elBlk;
    const double *props;
    const double *temp, *ptemp, *ptdot;
    int count, shell, dynamic, buildMat;
    double gamma, delT;
    double *load, *val;
};

__device__ void th_frame(const ThArgs &A, int e, double Xl[8][3], int rk[8]) {
    const int npe = A.shell ? 4 : 8;
    double Or[3][3];
    if (A.shell) {
        for (int i = 0; i < 9; ++i) Or[i / 3][i % 3] = A.sprops[e].orient[i];
    } else {
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) Or[i][j] = A.orient[9 * (size_t)e + 3 * j + i];
    }
    for (int a = 0; a < npe; ++a) {
        const int nd = A.elist[8 * (size_t)e + a] - 1;
        rk[a] = A.rank[nd] - 1;
        const double X0 = A.nodes[3 * (size_t)nd], X1 = A.nodes[3 * (size_t)nd + 1], X2 = A.nodes[3 * (size_t)nd + 2];
        for (int i = 0; i < 3; ++i) Xl[a][i] = Or[i][0] * X0 + Or[i][1] * X1 + Or[i][2] * X2;
    }
}

// r_getElRt of one element per thread: thermalLoad(rank) -= Rt, K_T += dRt/dT (colour order)
__global__ void k_th_elem(ThArgs A) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= A.count) return;
    const int e = A.els[q];
    const int npe = A.shell ? 4 : 8, ngp = A.shell ? 4 : 8;
    double Xl[8][3];
    int rk[8];
    th_frame(A, e, Xl, rk);
    const double *pp = A.props + (size_t)kProps * e;
    double tc[3][3];
    for (int i = 0; i < 9; ++i) tc[i / 3][i % 3] = pp[i];
    double T[8], Td[8];
    for (int a = 0; a < npe; ++a) {
        T[a] = A.temp ? A.temp[rk[a]] : 0.0;
        if (A.dynamic) {
            const double pT = A.ptemp ? A.ptemp[rk[a]] : 0.0, pTd = A.ptdot ? A.ptdot[rk[a]] : 0.0;
            Td[a] = (1.0 / A.gamma) * ((1.0 / A.delT) * (T[a] - pT) - 1.0 * (1.0 - A.gamma) * pTd);
        }
    }
    double Rt[8], K[8][8], Rm[8], M[8][8];
    for (int a = 0; a < 8; ++a) {
        Rt[a] = 0.0;
        Rm[a] = 0.0;
        for (int b = 0; b < 8; ++b) K[a][b] = M[a][b] = 0.0;
    }
    for (int g = 0; g < ngp; ++g) {
        double N[8], Nx[8][3], wd;
        th_point(A.shell, Xl, g, N, Nx, wd);
        double Tx[3] = {0.0, 0.0, 0.0}, qv[3];
        for (int a = 0; a < npe; ++a)
            for (int k = 0; k < 3; ++k) Tx[k] = Tx[k] + Nx[a][k] * T[a];
        for (int i = 0; i < 3; ++i) qv[i] = wd * (tc[i][0] * Tx[0] + tc[i][1] * Tx[1] + tc[i][2] * Tx[2]);
        for (int a = 0; a < npe; ++a) Rt[a] = Rt[a] + Nx[a][0] * qv[0] + Nx[a][1] * qv[1] + Nx[a][2] * qv[2];
        if (A.buildMat) {
            double kN[8][3];
            for (int a = 0; a < npe; ++a)
                for (int k = 0; k < 3; ++k)
                    kN[a][k] = wd * (Nx[a][0] * tc[0][k] + Nx[a][1] * tc[1][k] + Nx[a][2] * tc[2][k]);
            for (int a = 0; a < npe; ++a)
                for (int b = 0; b < npe; ++b)
                    K[a][b] = K[a][b] + Nx[a][0] * kN[b][0] + Nx[a][1] * kN[b][1] + Nx[a][2] * kN[b][2];
        }
        if (A.dynamic) {
            const double c = wd * pp[9];
            double pt = 0.0;
            for (int a = 0; a < npe; ++a) pt = pt + Td[a] * N[a];
            pt = c * pt;
            for (int a = 0; a < npe; ++a) Rm[a] = Rm[a] + pt * N[a];
            if (A.buildMat)
                for (int a = 0; a < npe; ++a)
                    for (int b = 0; b < npe; ++b) M[a][b] = M[a][b] + N[a] * (c * N[b]);
        }
    }
    if (A.dynamic) {
        const double f = 1.0 / (A.gamma * A.delT);
        for (int a = 0; a < npe; ++a) {
            Rt[a] = Rt[a] + Rm[a];
            if (A.buildMat)
                for (int b = 0; b < npe; ++b) K[a][b] = K[a][b] + f * M[a][b];
        }
    }
    if (A.load)
        for (int a = 0; a < npe; ++a) A.load[rk[a]] -= Rt[a];
    if (A.buildMat)
        for (int a = 0; a < npe; ++a)
            for (int b = 0; b < npe; ++b) A.val[A.elBlk[(size_t)npe * npe * e + npe * a + b]] += K[a][b];
}

// bodyHeatGen: q * integral of N (times the section thickness for shells), listed elements of a
// colour (an element listed twice adds twice)
__global__ void k_th_heatgen(ThArgs A, double qv, const double *__restrict__ mult) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= A.count) return;
    const int e = A.els[q];
    const int npe = A.shell ? 4 : 8, ngp = A.shell ? 4 : 8;
    double Xl[8][3];
    int rk[8];
    th_frame(A, e, Xl, rk);
    double w[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int g = 0; g < ngp; ++g) {
        double N[8], Nx[8][3], wd;
        th_point(A.shell, Xl, g, N, Nx, wd);
        for (int a = 0; a < npe; ++a) w[a] = w[a] + qv * N[a] * wd;
    }
    const double t = A.shell ? A.props[(size_t)kProps * e + 10] : 1.0;
    for (int a = 0; a < npe; ++a) A.load[rk[a]] += mult[q] * (t * w[a]);
}

// thermal CSR export in the reference's column order
__global__ void k_th_export(int nb, const int *__restrict__ bRow, const int *__restrict__ bCol,
                            const int *__restrict__ rowStart, const int *__restrict__ pos,
                            const double *__restrict__ val, double *__restrict__ mat, int *__restrict__ cols) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nb) return;
    const int at = rowStart[bRow[k]] + pos[k];
    mat[at] = val[k];
    cols[at] = bCol[k] + 1;
}

__global__ void k_th_absmax(const double *__restrict__ v, int n, unsigned long long *out) {
    double m = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) m = fmax(m, fabs(v[i]));
    for (int o = 16; o; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(m));
}

// getThermalConstraintLoad, rows in order (single thread: a handful of rows, fixed order)
__global__ void k_th_mpc_load(int rows, const int *__restrict__ range, const int *__restrict__ col,
                              const double *__restrict__ val, const double *__restrict__ rhs,
                              const double *__restrict__ temp, double *__restrict__ load) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    for (int r = 0; r < rows; ++r) {
        double v = rhs[r];
        for (int k = range[r]; k < range[r + 1]; ++k)
            if (col[k] >= 0) v = v - val[k] * (temp ? temp[col[k]] : 0.0);
        for (int k = range[r]; k < range[r + 1]; ++k)
            if (col[k] >= 0) load[col[k]] = load[col[k]] + val[k] * v;
    }
}

// ---- conjugate gradients on K_T + C^T C -------------------------------------------------------
constexpr int kCgBlocks = 304, kCgThreads = 256;

__global__ void k_cg_spmv(int N, const int *__restrict__ rp, const int *__restrict__ ci, const double *__restrict__ v,
                          const int *__restrict__ pp, const int *__restrict__ pc, const double *__restrict__ pv,
                          const double *__restrict__ x, double *__restrict__ y, double *__restrict__ dinv) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= N) return;
    double s = 0.0, d = 0.0;
    for (int k = rp[r]; k < rp[r + 1]; ++k) {
        s = s + v[k] * x[ci[k]];
        if (ci[k] == r) d = d + v[k];
    }
    if (pp)
        for (int k = pp[r]; k < pp[r + 1]; ++k) {
            s = s + pv[k] * x[pc[k]];
            if (pc[k] == r) d = d + pv[k];
        }
    y[r] = s;
    if (dinv) dinv[r] = 1.0 / d;
}

// partial dot products (deterministic: fixed grid, fixed reduction order)
__global__ void k_cg_dot(int n, const double *__restrict__ a, const double *__restrict__ b, double *__restrict__ part) {
    __shared__ double sm[kCgThreads / 32];
    double s = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) s = s + a[i] * b[i];
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < kCgThreads / 32; ++w) t = t + sm[w];
        part[blockIdx.x] = t;
    }
}

__global__ void k_cg_sum(const double *__restrict__ part, double *__restrict__ out) {
    if (threadIdx.x != 0) return;
    double t = 0.0;
    for (int i = 0; i < kCgBlocks; ++i) t = t + part[i];
    *out = t;
}

// s: [0] rz, [1] pAp, [2] rz_new, [3] rr
__global__ void k_cg_step(int n, const double *__restrict__ s, double *__restrict__ x, double *__restrict__ r,
                          const double *__restrict__ p, const double *__restrict__ Ap, const double *__restrict__ dinv,
                          double *__restrict__ z) {
    const double alpha = s[0] / s[1];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        x[i] = x[i] + alpha * p[i];
        r[i] = r[i] - alpha * Ap[i];
        z[i] = dinv[i] * r[i];
    }
}

__global__ void k_cg_init(int n, const double *__restrict__ b, const double *__restrict__ Ax,
                          const double *__restrict__ dinv, double *__restrict__ r, double *__restrict__ z,
                          double *__restrict__ p) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        r[i] = b[i] - Ax[i];
        z[i] = dinv[i] * r[i];
        p[i] = z[i];
    }
}

__global__ void k_cg_dir(int n, double *__restrict__ s, const double *__restrict__ z, double *__restrict__ p) {
    const double beta = s[2] / s[0];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = z[i] + beta * p[i];
}

__global__ void k_cg_shift(double *s) {
    if (threadIdx.x == 0) s[0] = s[2];
}

}  // namespace

void thermal_release(astro_ctx *ctx) {
    ThermPlan *T = plan_of(ctx);
    if (!T) return;
    DevBuf *b[] = {&T->d_props,   &T->d_val,    &T->d_pos,    &T->d_rowStart, &T->d_elMatId, &T->d_matCond,
                   &T->d_matSH,   &T->d_layCond, &T->d_laySH, &T->d_mRange,   &T->d_mCol,    &T->d_sVal,
                   &T->d_sRhs,    &T->d_penPtr, &T->d_penCol, &T->d_penVal};
    for (DevBuf *x : b) dev_free(*x);
    delete T;
    ctx->thermal = nullptr;
}

static ThPropArgs th_prop_args(astro_ctx *ctx, ThermPlan *T) {
    ThPropArgs A = {};
    const bool dv = ctx->numDvars > 0 && ctx->d_e2dR.p;
    A.shell = ctx->hasShell;
    A.esec = dptr<int>(ctx->d_esec);
    A.elMatId = ctx->hasSolid ? dptr<int>(T->d_elMatId) : nullptr;
    A.elDen = ctx->hasSolid ? dptr<double>(ctx->d_elRho) : nullptr;
    A.matCond = dptr<double>(T->d_matCond);
    A.matSH = dptr<double>(T->d_matSH);
    A.layRange = ctx->hasShell ? dptr<int>(ctx->d_shLayRange) : nullptr;
    A.lay = ctx->hasShell ? dptr<LayerDev>(ctx->d_shLay) : nullptr;
    A.layCond = dptr<double>(T->d_layCond);
    A.laySH = dptr<double>(T->d_laySH);
    A.e2dR = dv ? dptr<int>(ctx->d_e2dR) : nullptr;
    A.e2d = dv ? dptr<int>(ctx->d_e2d) : nullptr;
    A.e2c = dv ? dptr<double>(ctx->d_e2c) : nullptr;
    A.dcat = dv ? dptr<int>(ctx->d_dCat) : nullptr;
    A.dlay = dv ? dptr<int>(ctx->d_dLayer) : nullptr;
    A.dcomp = dv ? dptr<int>(ctx->d_dComp) : nullptr;
    A.dval = dv ? dptr<double>(ctx->d_dVal) : nullptr;
    return A;
}

extern "C" int astro_thermal_setup(astro_ctx *ctx, const astro_thermal_props *p, int32_t *therm_mat_size,
                                   int32_t *therm_mpc_dim) {
    if (!ctx || !p || p->num_materials < 1 || !p->material_therm_cond || !p->material_spec_heat) return ASTRO_ERR_ARG;
    if (ctx->hasShell && ctx->hasSolid) return set_err(ctx, ASTRO_ERR_UNSUPPORTED, "thermal path on a mixed mesh");
    const AstroPrep &P = ctx->P;
    const int N = P.N, E = P.E;
    if (ctx->hasSolid)
        for (int e = 0; e < E; ++e)
            if (ctx->elMatId[e] > p->num_materials) return set_err(ctx, ASTRO_ERR_ARG, "thermal: material out of range");
    for (int m : ctx->layMat)
        if (m < 1 || m > p->num_materials) return set_err(ctx, ASTRO_ERR_ARG, "thermal: layer material out of range");
    // constraint rows (buildThermalMPC on expanded equations: duplicate columns in a row skipped)
    std::vector<int> mRange(1, 0), mCol;
    std::vector<double> mVal, mRhs;
    for (int r = 0; r < p->num_mpc; ++r) {
        const int t0 = p->mpc_range[r], t1 = p->mpc_range[r + 1];
        const int base = (int)mCol.size();
        for (int t = t0; t < t1; ++t) {
            const int nd = p->mpc_node[t];
            if (nd < 1 || nd > N) return set_err(ctx, ASTRO_ERR_ARG, "thermal: constraint node out of range");
            mCol.push_back(-1);
            mVal.push_back(0.0);
        }
        for (int t = t0; t < t1; ++t) {
            const int col = P.currentRank[p->mpc_node[t]] - 1;
            for (int s = base; s < base + (t1 - t0); ++s) {
                if (mCol[s] < 0) {
                    mCol[s] = col;
                    mVal[s] = p->mpc_coef[t];
                    break;
                }
                if (mCol[s] == col) break;
            }
        }
        mRange.push_back((int)mCol.size());
        mRhs.push_back(p->mpc_rhs[r]);
    }
    thermal_release(ctx);
    ThermPlan *T = new ThermPlan();
    ctx->thermal = T;
    T->nMat = p->num_materials;
    T->mpcDim = p->num_mpc;
    T->mRange = mRange;
    T->mCol = mCol;
    T->mVal = mVal;
    T->mRhs = mRhs;
    // thermMatRange and the reference's column order: first insertion in the element loop
    std::vector<int> pos(P.nb, -1), fillRow(N, 0);
    T->rowStart.assign(N + 1, 0);
    for (int r = 0; r < N; ++r) T->rowStart[r + 1] = T->rowStart[r] + (P.bRowPtr[r + 1] - P.bRowPtr[r]);
    std::vector<int> rowOf(P.nb);
    for (int r = 0; r < N; ++r)
        for (int k = P.bRowPtr[r]; k < P.bRowPtr[r + 1]; ++k) rowOf[k] = r;
    const int npe = P.npe;
    for (int e = 0; e < E; ++e)
        for (int a = 0; a < npe; ++a)
            for (int b = 0; b < npe; ++b) {
                const int k = P.elBlk[(size_t)npe * npe * e + npe * a + b];
                if (pos[k] < 0) pos[k] = fillRow[rowOf[k]]++;
            }
    T->matSize = T->rowStart[N];
    int rc;
    std::vector<double> layCond(6 * std::max<size_t>(ctx->layMat.size(), 1)), laySH(std::max<size_t>(ctx->layMat.size(), 1));
    for (size_t l = 0; l < ctx->layMat.size(); ++l) {
        for (int k = 0; k < 6; ++k) layCond[6 * l + k] = p->material_therm_cond[6 * (ctx->layMat[l] - 1) + k];
        laySH[l] = p->material_spec_heat[ctx->layMat[l] - 1];
    }
    std::vector<int> rowStartI(T->rowStart.begin(), T->rowStart.end());
    if ((rc = upload(ctx, T->d_pos, pos.data(), sizeof(int) * P.nb)) ||
        (rc = upload(ctx, T->d_rowStart, rowStartI.data(), sizeof(int) * (N + 1))) ||
        (rc = upload(ctx, T->d_matCond, p->material_therm_cond, sizeof(double) * 6 * p->num_materials)) ||
        (rc = upload(ctx, T->d_matSH, p->material_spec_heat, sizeof(double) * p->num_materials)) ||
        (rc = upload(ctx, T->d_layCond, layCond.data(), sizeof(double) * layCond.size())) ||
        (rc = upload(ctx, T->d_laySH, laySH.data(), sizeof(double) * laySH.size())) ||
        (rc = dev_alloc(ctx, T->d_props, sizeof(double) * kProps * (size_t)E)) ||
        (rc = dev_alloc(ctx, T->d_val, sizeof(double) * (size_t)P.nb)))
        return rc;
    if (ctx->hasSolid && (rc = upload(ctx, T->d_elMatId, ctx->elMatId.data(), sizeof(int) * E))) return rc;
    k_th_props<<<(E + 127) / 128, 128, 0, ctx->stream>>>(th_prop_args(ctx, T), E, dptr<double>(T->d_props));
    rc = cuda_check(ctx, cudaGetLastError(), "thermal properties");
    if (!rc) rc = cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "thermal properties");
    if (rc) return rc;
    if (therm_mat_size) *therm_mat_size = T->matSize;
    if (therm_mpc_dim) *therm_mpc_dim = T->mpcDim;
    return ASTRO_OK;
}

static ThArgs th_args(astro_ctx *ctx, ThermPlan *T) {
    ThArgs A = {};
    A.nodes = dptr<double>(ctx->d_nodes);
    A.orient = ctx->hasSolid ? dptr<double>(ctx->d_secOrient) : nullptr;
    A.sprops = ctx->hasShell ? dptr<ShellProps>(ctx->d_secABD) : nullptr;
    A.elist = dptr<int>(ctx->d_elist);
    A.rank = dptr<int>(ctx->d_rank);
    A.elBlk = dptr<int>(ctx->d_elBlk);
    A.props = dptr<double>(T->d_props);
    A.shell = ctx->hasShell;
    return A;
}

// host vector (rank order) -> device, or null
static int up_opt(astro_ctx *ctx, DevBuf &b, const double *h, int n) {
    if (!h) return ASTRO_OK;
    return upload(ctx, b, h, sizeof(double) * n);
}

extern "C" int astro_thermal_soln_load(astro_ctx *ctx, int32_t build_mat, const astro_thermal_state *st,
                                       double *thermal_load, double *therm_mat, int32_t *therm_cols) {
    if (!ctx || !thermal_load) return ASTRO_ERR_ARG;
    ThermPlan *T = plan_of(ctx);
    if (!T) return set_err(ctx, ASTRO_ERR_STATE, "thermal: astro_thermal_setup not called");
    if (st && st->dynamic && !(st->nm_gamma != 0.0 && st->del_t != 0.0))
        return set_err(ctx, ASTRO_ERR_ARG, "thermal: dynamic step needs gamma and a time step");
    const AstroPrep &P = ctx->P;
    const int N = P.N;
    cudaStream_t s = ctx->stream;
    DevBuf dT, dpT, dpTd, dL;
    int rc;
    if ((rc = up_opt(ctx, dT, st ? st->node_temp : nullptr, N)) ||
        (rc = up_opt(ctx, dpT, st ? st->prev_temp : nullptr, N)) ||
        (rc = up_opt(ctx, dpTd, st ? st->prev_tdot : nullptr, N)) ||
        (rc = upload(ctx, dL, thermal_load, sizeof(double) * N))) {
        DevBuf *v[] = {&dT, &dpT, &dpTd, &dL};
        for (DevBuf *x : v) dev_free(*x);
        return rc;
    }
    ThArgs A = th_args(ctx, T);
    A.temp = dT.p ? dptr<double>(dT) : nullptr;
    A.ptemp = dpT.p ? dptr<double>(dpT) : nullptr;
    A.ptdot = dpTd.p ? dptr<double>(dpTd) : nullptr;
    A.dynamic = st ? st->dynamic : 0;
    A.gamma = st ? st->nm_gamma : 0.5;
    A.delT = st ? st->del_t : 0.0;
    A.buildMat = build_mat == 1;
    A.load = dptr<double>(dL);
    A.val = dptr<double>(T->d_val);
    if (A.buildMat) cudaMemsetAsync(T->d_val.p, 0, sizeof(double) * P.nb, s);
    for (int col = 0; col < P.ncolors; ++col) {
        A.els = dptr<int>(ctx->d_colorEls) + P.colorPtr[col];
        A.count = P.colorPtr[col + 1] - P.colorPtr[col];
        if (A.count) k_th_elem<<<(A.count + 127) / 128, 128, 0, s>>>(A);
    }
    rc = cuda_check(ctx, cudaGetLastError(), "thermal elements");
    if (!rc && A.buildMat) {
        T->haveMat = 1;
        T->scaled = 0;
        if (therm_mat && therm_cols) {
            DevBuf dm, dc;
            if (!(rc = dev_alloc(ctx, dm, sizeof(double) * T->matSize)) &&
                !(rc = dev_alloc(ctx, dc, sizeof(int) * T->matSize))) {
                k_th_export<<<(P.nb + 255) / 256, 256, 0, s>>>(P.nb, dptr<int>(ctx->d_bRow), dptr<int>(ctx->d_bCol),
                                                               dptr<int>(T->d_rowStart), dptr<int>(T->d_pos),
                                                               dptr<double>(T->d_val), dptr<double>(dm), dptr<int>(dc));
                cudaError_t e = cudaMemcpyAsync(therm_mat, dm.p, sizeof(double) * T->matSize, cudaMemcpyDeviceToHost, s);
                if (e == cudaSuccess)
                    e = cudaMemcpyAsync(therm_cols, dc.p, sizeof(int) * T->matSize, cudaMemcpyDeviceToHost, s);
                if (e == cudaSuccess) e = cudaStreamSynchronize(s);
                rc = cuda_check(ctx, e, "thermal export");
            }
            dev_free(dm);
            dev_free(dc);
        }
    }
    if (!rc) {
        cudaError_t e = cudaMemcpyAsync(thermal_load, dL.p, sizeof(double) * N, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        rc = cuda_check(ctx, e, "thermal load");
    }
    DevBuf *v[] = {&dT, &dpT, &dpTd, &dL};
    for (DevBuf *x : v) dev_free(*x);
    return rc;
}

extern "C" int astro_thermal_scale_mpc(astro_ctx *ctx, double *mpc_mat, double *mpc_rhs) {
    if (!ctx) return ASTRO_ERR_ARG;
    ThermPlan *T = plan_of(ctx);
    if (!T || !T->haveMat) return set_err(ctx, ASTRO_ERR_STATE, "thermal: conductivity matrix not assembled");
    const AstroPrep &P = ctx->P;
    cudaStream_t s = ctx->stream;
    DevBuf d;
    int rc = dev_alloc(ctx, d, sizeof(unsigned long long));
    if (rc) return rc;
    unsigned long long h = 0;
    cudaMemsetAsync(d.p, 0, sizeof(unsigned long long), s);
    k_th_absmax<<<4 * 152, 256, 0, s>>>(dptr<double>(T->d_val), P.nb, dptr<unsigned long long>(d));
    cudaError_t e = cudaMemcpyAsync(&h, d.p, sizeof(h), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    dev_free(d);
    if ((rc = cuda_check(ctx, e, "thermal scale"))) return rc;
    double maxMat;
    long long bits = (long long)h;
    std::memcpy(&maxMat, &bits, sizeof(maxMat));
    // scaleThermalMPC: each row to unit length, then times 100 max|thermMat|
    T->sVal = T->mVal;
    T->sRhs = T->mRhs;
    for (int r = 0; r < T->mpcDim; ++r) {
        double mag = 0.0;
        for (int k = T->mRange[r]; k < T->mRange[r + 1]; ++k) mag = mag + T->sVal[k] * T->sVal[k];
        mag = std::sqrt(mag);
        for (int k = T->mRange[r]; k < T->mRange[r + 1]; ++k) T->sVal[k] = (1.0 / mag) * T->sVal[k];
        T->sRhs[r] = (1.0 / mag) * T->sRhs[r];
    }
    for (double &v : T->sVal) v = 100.0 * maxMat * v;
    for (double &v : T->sRhs) v = 100.0 * maxMat * v;
    // penalty C^T C by row
    std::map<std::pair<int, int>, double> pen;
    for (int r = 0; r < T->mpcDim; ++r)
        for (int a = T->mRange[r]; a < T->mRange[r + 1]; ++a)
            for (int b = T->mRange[r]; b < T->mRange[r + 1]; ++b)
                if (T->mCol[a] >= 0 && T->mCol[b] >= 0) pen[{T->mCol[a], T->mCol[b]}] += T->sVal[a] * T->sVal[b];
    std::vector<int> pp(P.N + 1, 0), pc;
    std::vector<double> pv;
    for (auto &kv : pen) pp[kv.first.first + 1]++;
    for (int r = 0; r < P.N; ++r) pp[r + 1] += pp[r];
    for (auto &kv : pen) {
        pc.push_back(kv.first.second);
        pv.push_back(kv.second);
    }
    T->penCount = (int)pc.size();
    std::vector<int> mr(T->mRange), mc(T->mCol);
    if (mc.empty()) mc.push_back(-1);
    std::vector<double> sv(T->sVal), sr(T->sRhs);
    if (sv.empty()) sv.push_back(0.0);
    if (sr.empty()) sr.push_back(0.0);
    if (pc.empty()) {
        pc.push_back(0);
        pv.push_back(0.0);
    }
    if ((rc = upload(ctx, T->d_mRange, mr.data(), sizeof(int) * mr.size())) ||
        (rc = upload(ctx, T->d_mCol, mc.data(), sizeof(int) * mc.size())) ||
        (rc = upload(ctx, T->d_sVal, sv.data(), sizeof(double) * sv.size())) ||
        (rc = upload(ctx, T->d_sRhs, sr.data(), sizeof(double) * sr.size())) ||
        (rc = upload(ctx, T->d_penPtr, pp.data(), sizeof(int) * pp.size())) ||
        (rc = upload(ctx, T->d_penCol, pc.data(), sizeof(int) * pc.size())) ||
        (rc = upload(ctx, T->d_penVal, pv.data(), sizeof(double) * pv.size())))
        return rc;
    T->scaled = 1;
    if (mpc_mat) std::copy(T->sVal.begin(), T->sVal.end(), mpc_mat);
    if (mpc_rhs) std::copy(T->sRhs.begin(), T->sRhs.end(), mpc_rhs);
    return ASTRO_OK;
}

extern "C" int astro_thermal_constraint_load(astro_ctx *ctx, const double *node_temp, double *thermal_load) {
    if (!ctx || !thermal_load) return ASTRO_ERR_ARG;
    ThermPlan *T = plan_of(ctx);
    if (!T) return set_err(ctx, ASTRO_ERR_STATE, "thermal: astro_thermal_setup not called");
    if (T->mpcDim == 0) return ASTRO_OK;
    if (!T->scaled) return set_err(ctx, ASTRO_ERR_STATE, "thermal: constraints not scaled (astro_thermal_scale_mpc)");
    const int N = ctx->P.N;
    DevBuf dT, dL;
    int rc = up_opt(ctx, dT, node_temp, N);
    if (!rc) rc = upload(ctx, dL, thermal_load, sizeof(double) * N);
    if (!rc) {
        k_th_mpc_load<<<1, 32, 0, ctx->stream>>>(T->mpcDim, dptr<int>(T->d_mRange), dptr<int>(T->d_mCol),
                                                 dptr<double>(T->d_sVal), dptr<double>(T->d_sRhs),
                                                 dT.p ? dptr<double>(dT) : nullptr, dptr<double>(dL));
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(thermal_load, dL.p, sizeof(double) * N, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        rc = cuda_check(ctx, e, "thermal constraint load");
    }
    dev_free(dT);
    dev_free(dL);
    return rc;
}

extern "C" int astro_thermal_heat_gen(astro_ctx *ctx, double q, const int32_t *elements, int32_t count,
                                      double *thermal_load) {
    if (!ctx || !thermal_load || count < 0) return ASTRO_ERR_ARG;
    ThermPlan *T = plan_of(ctx);
    if (!T) return set_err(ctx, ASTRO_ERR_STATE, "thermal: astro_thermal_setup not called");
    const AstroPrep &P = ctx->P;
    if (elements)
        for (int k = 0; k < count; ++k)
            if (elements[k] < 1 || elements[k] > P.E) return set_err(ctx, ASTRO_ERR_ARG, "element number out of range");
    std::vector<int> on((size_t)P.E, elements ? 0 : 1);
    if (elements)
        for (int k = 0; k < count; ++k) ++on[elements[k] - 1];
    std::vector<int> list, ptr(1, 0);
    std::vector<double> mult;
    for (int col = 0; col < P.ncolors; ++col) {
        for (int k = P.colorPtr[col]; k < P.colorPtr[col + 1]; ++k)
            if (on[P.colorEls[k]]) {
                list.push_back(P.colorEls[k]);
                mult.push_back((double)on[P.colorEls[k]]);
            }
        ptr.push_back((int)list.size());
    }
    if (list.empty()) return ASTRO_OK;
    DevBuf dl, dm, dL;
    int rc = upload(ctx, dl, list.data(), sizeof(int) * list.size());
    if (!rc) rc = upload(ctx, dm, mult.data(), sizeof(double) * mult.size());
    if (!rc) rc = upload(ctx, dL, thermal_load, sizeof(double) * P.N);
    if (!rc) {
        ThArgs A = th_args(ctx, T);
        A.load = dptr<double>(dL);
        for (int col = 0; col < P.ncolors; ++col) {
            A.count = ptr[col + 1] - ptr[col];
            if (!A.count) continue;
            A.els = dptr<int>(dl) + ptr[col];
            k_th_heatgen<<<(A.count + 127) / 128, 128, 0, ctx->stream>>>(A, q, dptr<double>(dm) + ptr[col]);
        }
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(thermal_load, dL.p, sizeof(double) * P.N, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        rc = cuda_check(ctx, e, "heat generation");
    }
    dev_free(dl);
    dev_free(dm);
    dev_free(dL);
    return rc;
}

// thermal -= component 1 of the traction load (the surfaceFlux branch takes the flux as the first
// traction component and subtracts the element's component-1 nodal forces)
__global__ void k_th_flux_extract(int N, int dpn, const double *__restrict__ el, double *__restrict__ load) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < N) load[r] = load[r] - el[(size_t)r * dpn];
}

extern "C" int astro_thermal_surface_flux(astro_ctx *ctx, int32_t nfaces, const int32_t *face_el,
                                          const int32_t *face_num, double flux, double *thermal_load) {
    if (!ctx || !thermal_load || nfaces < 0 || (nfaces && (!face_el || !face_num))) return ASTRO_ERR_ARG;
    if (!plan_of(ctx)) return set_err(ctx, ASTRO_ERR_STATE, "thermal: astro_thermal_setup not called");
    const AstroPrep &P = ctx->P;
    for (int f = 0; f < nfaces; ++f) {
        const int e = face_el[f], fn = face_num[f];
        if (e < 1 || e > P.E) return set_err(ctx, ASTRO_ERR_ARG, "face element out of range");
        if (fn < 1 || fn > ((ctx->etype[e - 1] == 8 || ctx->etype[e - 1] == 81) ? 6 : 2)) return set_err(ctx, ASTRO_ERR_ARG, "face number out of range");
    }
    if (!nfaces) return ASTRO_OK;
    DevBuf dfe, dfn, del, dL;
    int rc = upload(ctx, dfe, face_el, sizeof(int) * nfaces);
    if (!rc) rc = upload(ctx, dfn, face_num, sizeof(int) * nfaces);
    if (!rc) rc = dev_alloc(ctx, del, sizeof(double) * P.n);
    if (!rc) rc = upload(ctx, dL, thermal_load, sizeof(double) * P.N);
    if (!rc) {
        cudaMemsetAsync(del.p, 0, sizeof(double) * P.n, ctx->stream);
        const double tr[3] = {flux, 0.0, 0.0};
        rc = surface_load_dev(ctx, nfaces, dptr<int>(dfe), dptr<int>(dfn), tr, 0.0, dptr<double>(del));
    }
    if (!rc) {
        k_th_flux_extract<<<(P.N + 255) / 256, 256, 0, ctx->stream>>>(P.N, P.dpn, dptr<double>(del), dptr<double>(dL));
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(thermal_load, dL.p, sizeof(double) * P.N, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        rc = cuda_check(ctx, e, "surface flux");
    }
    DevBuf *v[] = {&dfe, &dfn, &del, &dL};
    for (DevBuf *x : v) dev_free(*x);
    return rc;
}

extern "C" int astro_thermal_solve(astro_ctx *ctx, const double *rhs, double *dtemp, double rtol, int32_t max_iters,
                                   astro_solve_stats *stats) {
    if (!ctx || !rhs || !dtemp || !(rtol > 0.0) || max_iters < 1) return ASTRO_ERR_ARG;
    ThermPlan *T = plan_of(ctx);
    if (!T || !T->haveMat) return set_err(ctx, ASTRO_ERR_STATE, "thermal: conductivity matrix not assembled");
    if (T->mpcDim > 0 && !T->scaled)
        return set_err(ctx, ASTRO_ERR_STATE, "thermal: constraints not scaled (astro_thermal_scale_mpc)");
    const AstroPrep &P = ctx->P;
    const int N = P.N;
    cudaStream_t s = ctx->stream;
    DevBuf b, x, r, z, p, Ap, dinv, part, sc;
    int rc;
    if ((rc = upload(ctx, b, rhs, sizeof(double) * N)) || (rc = upload(ctx, x, dtemp, sizeof(double) * N)) ||
        (rc = dev_alloc(ctx, r, sizeof(double) * N)) || (rc = dev_alloc(ctx, z, sizeof(double) * N)) ||
        (rc = dev_alloc(ctx, p, sizeof(double) * N)) || (rc = dev_alloc(ctx, Ap, sizeof(double) * N)) ||
        (rc = dev_alloc(ctx, dinv, sizeof(double) * N)) || (rc = dev_alloc(ctx, part, sizeof(double) * kCgBlocks)) ||
        (rc = dev_alloc(ctx, sc, sizeof(double) * 8))) {
        DevBuf *v[] = {&b, &x, &r, &z, &p, &Ap, &dinv, &part, &sc};
        for (DevBuf *q : v) dev_free(*q);
        return rc;
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const unsigned rg = (N + 255) / 256;
    const int *pp = T->mpcDim ? dptr<int>(T->d_penPtr) : nullptr;
    double *S = dptr<double>(sc);
    auto spmv = [&](const double *in, double *out, double *dv) {
        k_cg_spmv<<<rg, 256, 0, s>>>(N, dptr<int>(ctx->d_bRowPtr), dptr<int>(ctx->d_bCol), dptr<double>(T->d_val), pp,
                                     pp ? dptr<int>(T->d_penCol) : nullptr, pp ? dptr<double>(T->d_penVal) : nullptr,
                                     in, out, dv);
    };
    auto dot = [&](const double *a, const double *bb, int slot) {
        k_cg_dot<<<kCgBlocks, kCgThreads, 0, s>>>(N, a, bb, dptr<double>(part));
        k_cg_sum<<<1, 32, 0, s>>>(dptr<double>(part), S + slot);
    };
    cudaEventRecord(e0, s);
    // r = b - A x, z = D^-1 r, p = z
    spmv(dptr<double>(x), dptr<double>(Ap), dptr<double>(dinv));
    k_cg_init<<<kCgBlocks, kCgThreads, 0, s>>>(N, dptr<double>(b), dptr<double>(Ap), dptr<double>(dinv),
                                               dptr<double>(r), dptr<double>(z), dptr<double>(p));
    dot(dptr<double>(b), dptr<double>(b), 4);
    dot(dptr<double>(r), dptr<double>(z), 0);
    double bb = 0.0, rr = 0.0;
    int it = 0, status = ASTRO_ERR_MAXIT;
    cudaMemcpyAsync(&bb, S + 4, sizeof(double), cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    const double bn = std::sqrt(bb);
    if (bn == 0.0) status = ASTRO_OK;
    while (!rc && status == ASTRO_ERR_MAXIT && it < max_iters) {
        const int chunk = std::min(16, max_iters - it);
        for (int k = 0; k < chunk; ++k) {
            spmv(dptr<double>(p), dptr<double>(Ap), nullptr);
            dot(dptr<double>(p), dptr<double>(Ap), 1);
            k_cg_step<<<kCgBlocks, kCgThreads, 0, s>>>(N, S, dptr<double>(x), dptr<double>(r), dptr<double>(p),
                                                       dptr<double>(Ap), dptr<double>(dinv), dptr<double>(z));
            dot(dptr<double>(r), dptr<double>(z), 2);
            k_cg_dir<<<kCgBlocks, kCgThreads, 0, s>>>(N, S, dptr<double>(z), dptr<double>(p));
            k_cg_shift<<<1, 32, 0, s>>>(S);
        }
        it += chunk;
        dot(dptr<double>(r), dptr<double>(r), 3);
        cudaError_t e = cudaMemcpyAsync(&rr, S + 3, sizeof(double), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if ((rc = cuda_check(ctx, e, "thermal solve"))) break;
        if (!std::isfinite(rr)) {
            status = ASTRO_ERR_NAN;
            break;
        }
        if (std::sqrt(rr) <= rtol * bn) status = ASTRO_OK;
    }
    cudaEventRecord(e1, s);
    if (!rc) {
        cudaError_t e = cudaMemcpyAsync(dtemp, x.p, sizeof(double) * N, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        rc = cuda_check(ctx, e, "thermal solve");
    }
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        stats->iterations = it;
        stats->status = rc ? rc : status;
        stats->rel_residual = bn > 0.0 ? std::sqrt(rr) / bn : 0.0;
        stats->residual_kind = 64;
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        stats->seconds = ms * 1e-3;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    DevBuf *v[] = {&b, &x, &r, &z, &p, &Ap, &dinv, &part, &sc};
    for (DevBuf *q : v) dev_free(*q);
    if (rc) return rc;
    if (status == ASTRO_ERR_MAXIT) return set_err(ctx, ASTRO_ERR_MAXIT, "thermal solve: iteration limit");
    if (status == ASTRO_ERR_NAN) return set_err(ctx, ASTRO_ERR_NAN, "thermal solve: non-finite residual");
    return ASTRO_OK;
}

// ---- design sensitivities (getdRthermaldD, Working/AStrO_commandFunctions.f90:1016-1170) ---------
// Complex step: the elements that depend on the design variable are evaluated in complex FP64
// with d + i h, one thread per element, colour by colour (a colour's elements share no node), and
// Im / h is accumulated at their nodes.  The complex path's Gauss points are the single-precision
// 1/sqrt(3) of the reference's c_ constants.
namespace {

struct ThCsArgs {
    int dvar;
    double h;
    const double *secOrig;  // (S,9) column-major section orientation as given
    const int *n2dR, *n2d;  // node design maps (null: none)
    const double *n2c;
    const double *mult;     // per listed element: how often the load lists it (heat generation)
    double q;               // heat generation per unit volume
    double *out;            // rank-order derivative
};

// The element frame and its nodes in it, in T: nodes with + i h coef on d's nodeCoord terms
// (r_getNodeCoord, designProp :945-968; the real offsets of every nodeCoord variable are already
// in the node list), the section orientation rotated by its orientation variables
// (r_getOrientation, :187-221) and, for shells, correctAlpha.
template <class T>
__device__ void th_frame_t(const ThArgs &A, const ThPropArgs &P, const ThCsArgs &C, int e, T Xl[8][3], int rk[8]) {
    const int npe = A.shell ? 4 : 8;
    const T ih = pert_i<T>(C.h);
    T Xg[8][3];
    for (int a = 0; a < npe; ++a) {
        const int nd = A.elist[8 * (size_t)e + a];
        rk[a] = A.rank[nd - 1] - 1;
        for (int k = 0; k < 3; ++k) Xg[a][k] = T(A.nodes[3 * (size_t)(nd - 1) + k]);
        if (C.n2dR)
            for (int t = C.n2dR[nd - 1]; t < C.n2dR[nd]; ++t) {
                const int d = C.n2d[t];
                if (d == C.dvar && P.dcat[d - 1] == ASTRO_DCAT_NODE_COORD) Xg[a][P.dcomp[d - 1] - 1] += C.n2c[t] * ih;
            }
    }
    T loc[3] = {T(0.0), T(0.0), T(0.0)};
    if (P.e2dR)
        for (int q = P.e2dR[e]; q < P.e2dR[e + 1]; ++q) {
            const int d = P.e2d[q];
            if (P.dcat[d - 1] != ASTRO_DCAT_ORIENTATION) continue;
            T v = T(P.dval[d - 1]);
            if (d == C.dvar) v = v + ih;
            loc[P.dcomp[d - 1] - 1] = loc[P.dcomp[d - 1] - 1] + P.e2c[q] * v;
        }
    const int sec = P.esec[e];
    T al[3][3], gr[3], orient[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) al[i][j] = T(C.secOrig[9 * (size_t)(sec - 1) + 3 * j + i]);
    for (int i = 0; i < 3; ++i) gr[i] = al[0][i] * loc[0] + al[1][i] * loc[1] + al[2][i] * loc[2];
    a_rotate<T>(orient, al, gr, 0, 0);
    if (A.shell) {
        T X4[4][3];
        for (int a = 0; a < 4; ++a)
            for (int k = 0; k < 3; ++k) X4[a][k] = Xg[a][k];
        shell_correct_alpha<T>(orient, X4);
    }
    for (int a = 0; a < npe; ++a)
        for (int i = 0; i < 3; ++i) Xl[a][i] = orient[i][0] * Xg[a][0] + orient[i][1] * Xg[a][1] + orient[i][2] * Xg[a][2];
}

// The complex Gauss point, called out of line.  Inlined into k_th_elem_cs, this CUDA 13.0 build
// for sm_103a returned wrong shape-function gradients for every node but the first, although
// the parametric derivatives and the inverse Jacobian inside the routine were right.  The same source
// built for the host, built with -G, or called out of line gives the right gradients.
__device__ __noinline__ void th_point_cs(int shell, const cplx Xl[8][3], int g, double N[8], cplx Nx[8][3],
                                         cplx &wdet) {
    th_point_t<cplx>(shell, Xl, AK<cplx>::rt3, g, N, Nx, wdet);
}

// element part: out[rank] += Im(Rt) / h (r_getElRtk + r_getElRtm in complex)
__global__ void k_th_elem_cs(ThArgs A, ThPropArgs P, ThCsArgs C) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= A.count) return;
    const int e = A.els[q];
    const int npe = A.shell ? 4 : 8, ngp = A.shell ? 4 : 8;
    cplx Xl[8][3];
    int rk[8];
    th_frame_t<cplx>(A, P, C, e, Xl, rk);
    cplx tc[3][3], sh, secT;
    th_props_t<cplx>(P, e, C.dvar, C.h, tc, sh, secT);
    double T[8], Td[8];
    for (int a = 0; a < npe; ++a) {
        T[a] = A.temp ? A.temp[rk[a]] : 0.0;
        Td[a] = 0.0;
        if (A.dynamic) {
            const double pT = A.ptemp ? A.ptemp[rk[a]] : 0.0, pTd = A.ptdot ? A.ptdot[rk[a]] : 0.0;
            Td[a] = (1.0 / A.gamma) * ((1.0 / A.delT) * (T[a] - pT) - 1.0 * (1.0 - A.gamma) * pTd);
        }
    }
    cplx Rt[8];
    for (int g = 0; g < ngp; ++g) {
        double N[8];
        cplx Nx[8][3], wd;
        th_point_cs(A.shell, Xl, g, N, Nx, wd);
        cplx Tx[3];
        for (int a = 0; a < npe; ++a)
            for (int k = 0; k < 3; ++k) Tx[k] = Tx[k] + Nx[a][k] * T[a];
        cplx qv[3];
        for (int i = 0; i < 3; ++i) qv[i] = wd * (tc[i][0] * Tx[0] + tc[i][1] * Tx[1] + tc[i][2] * Tx[2]);
        for (int a = 0; a < npe; ++a) Rt[a] = Rt[a] + Nx[a][0] * qv[0] + Nx[a][1] * qv[1] + Nx[a][2] * qv[2];
        if (A.dynamic) {
            double pt = 0.0;
            for (int a = 0; a < npe; ++a) pt = pt + Td[a] * N[a];
            const cplx c = (wd * sh) * pt;
            for (int a = 0; a < npe; ++a) Rt[a] = Rt[a] + c * N[a];
        }
    }
    const double hInv = 1.0 / C.h;
    for (int a = 0; a < npe; ++a) C.out[rk[a]] += hInv * Rt[a].im;
}

// bodyHeatGen branch: out[rank] -= mult Im(q integral of N (times the section thickness for
// shells)) / h
__global__ void k_th_heatgen_cs(ThArgs A, ThPropArgs P, ThCsArgs C) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= A.count) return;
    const int e = A.els[q];
    const int npe = A.shell ? 4 : 8, ngp = A.shell ? 4 : 8;
    cplx Xl[8][3];
    int rk[8];
    th_frame_t<cplx>(A, P, C, e, Xl, rk);
    cplx w[8];
    for (int g = 0; g < ngp; ++g) {
        double N[8];
        cplx Nx[8][3], wd;
        th_point_cs(A.shell, Xl, g, N, Nx, wd);
        for (int a = 0; a < npe; ++a) w[a] = w[a] + (C.q * N[a]) * wd;
    }
    cplx t = cplx(1.0);
    if (A.shell) {
        cplx tc[3][3], sh;
        th_props_t<cplx>(P, e, C.dvar, C.h, tc, sh, t);
    }
    const double hInv = 1.0 / C.h;
    for (int a = 0; a < npe; ++a) C.out[rk[a]] -= C.mult[q] * (hInv * (t * w[a]).im);
}

// surfaceFlux branch, one thread per face: the face's four nodal values Im(flux integral of
// N dA) / h, dA the true area element (as the load itself), into fv[4 f + k]
__global__ void k_th_flux_cs(int nf, const int *__restrict__ faceEl, const int *__restrict__ faceNum,
                             const int *__restrict__ etype, const int *__restrict__ elist,
                             const double *__restrict__ nodes, const int *__restrict__ n2dR,
                             const int *__restrict__ n2d, const double *__restrict__ n2c, const int *__restrict__ dcat,
                             const int *__restrict__ dcomp, int dvar, double h, double flux, double *__restrict__ fv) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    const int hexF[6][4] = {{4, 3, 2, 1}, {5, 6, 7, 8}, {1, 2, 6, 5}, {2, 3, 7, 6}, {3, 4, 8, 7}, {4, 1, 5, 8}};
    const int shF[2][4] = {{1, 2, 3, 4}, {1, 4, 3, 2}};
    const int el = faceEl[f] - 1, fn = faceNum[f] - 1;
    const int *fl = (etype[el] == 8 || etype[el] == 81) ? hexF[fn] : shF[fn];
    cplx X[4][3];
    for (int k = 0; k < 4; ++k) {
        const int nd = elist[8 * (size_t)el + fl[k] - 1];
        for (int d = 0; d < 3; ++d) X[k][d] = cplx(nodes[3 * (size_t)(nd - 1) + d]);
        if (n2dR)
            for (int t = n2dR[nd - 1]; t < n2dR[nd]; ++t)
                if (n2d[t] == dvar && dcat[dvar - 1] == ASTRO_DCAT_NODE_COORD)
                    X[k][dcomp[dvar - 1] - 1] += cplx(0.0, n2c[t] * h);
    }
    const double g = AK<cplx>::rt3;
    cplx acc[4];
    for (int gp = 0; gp < 4; ++gp) {
        const double s = (gp & 1) ? g : -g, r = (gp & 2) ? g : -g;
        const double N_[4] = {0.25 * (1 - s) * (1 - r), 0.25 * (1 + s) * (1 - r), 0.25 * (1 + s) * (1 + r),
                              0.25 * (1 - s) * (1 + r)};
        const double Ns[4] = {-0.25 * (1 - r), 0.25 * (1 - r), 0.25 * (1 + r), -0.25 * (1 + r)};
        const double Nr[4] = {-0.25 * (1 - s), -0.25 * (1 + s), 0.25 * (1 + s), 0.25 * (1 - s)};
        cplx a[3], b[3];
        for (int k = 0; k < 4; ++k)
            for (int d = 0; d < 3; ++d) {
                a[d] = a[d] + Ns[k] * X[k][d];
                b[d] = b[d] + Nr[k] * X[k][d];
            }
        const cplx cx = a[1] * b[2] - a[2] * b[1], cy = a[2] * b[0] - a[0] * b[2], cz = a[0] * b[1] - a[1] * b[0];
        const cplx s2 = cx * cx + cy * cy + cz * cz;
        // principal square root to first order in the imaginary part (exact for the complex step)
        const double re = sqrt(s2.re);
        const cplx dA(re, s2.im / (2.0 * re));
        for (int k = 0; k < 4; ++k) acc[k] = acc[k] + (flux * N_[k]) * dA;
    }
    for (int k = 0; k < 4; ++k) fv[4 * (size_t)f + k] = acc[k].im / h;
}

// out[row[g]] += the face values of its slots, in face order (gPtr / gSlot as face_gather_kernel)
__global__ void k_th_face_gather(int ng, const int *__restrict__ gPtr, const int *__restrict__ gSlot,
                                 const int *__restrict__ gRow, const double *__restrict__ fv, double *__restrict__ out) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ng) return;
    double s = out[gRow[g]];
    for (int q = gPtr[g]; q < gPtr[g + 1]; ++q) s = s + fv[gSlot[q]];
    out[gRow[g]] = s;
}

// 'nodeLoad' / 'thermal' variables (d_component 7) active at t (dActTime(1) < t < dActTime(2)):
// mode 0 load[rank] += coef d of every variable, mode 1 load[rank] -= coef for dvar only
__global__ void k_th_node_dload(int N, const int *__restrict__ rank, const int *__restrict__ n2dR,
                                const int *__restrict__ n2d, const double *__restrict__ n2c,
                                const int *__restrict__ dcat, const int *__restrict__ dcomp,
                                const double *__restrict__ dval, const double *__restrict__ act, double t, int mode,
                                int dvar, double *__restrict__ load) {
    const int nd = blockIdx.x * blockDim.x + threadIdx.x;
    if (nd >= N) return;
    double v = load[rank[nd] - 1];
    for (int q = n2dR[nd]; q < n2dR[nd + 1]; ++q) {
        const int d = n2d[q];
        if (dcat[d - 1] != ASTRO_DCAT_NODE_LOAD || dcomp[d - 1] != 7 || (mode == 1 && d != dvar)) continue;
        if (act && !(t > act[2 * (d - 1)] && act[2 * (d - 1) + 1] > t)) continue;
        v = v + (mode == 0 ? n2c[q] * dval[d - 1] : -n2c[q]);
    }
    load[rank[nd] - 1] = v;
}

}  // namespace

// Per element (0-based): 1 when it depends on dvar (getdToElComp, Working/AStrO_bookKeeping.f90:7-129:
// the element's own design variables, and the nodeCoord variables of its nodes).
static std::vector<char> th_dependents(const astro_ctx *ctx, int dvar) {
    const AstroPrep &P = ctx->P;
    std::vector<char> dep((size_t)P.E, 0);
    for (int e = 0; e < P.E; ++e)
        for (int q = ctx->e2dRange[e]; q < ctx->e2dRange[e + 1]; ++q)
            if (ctx->e2d[q] == dvar) dep[e] = 1;
    if (!ctx->n2dRange.empty() && ctx->dCat[dvar - 1] == ASTRO_DCAT_NODE_COORD) {
        std::vector<char> nd((size_t)P.N + 1, 0);
        for (int n = 1; n <= P.N; ++n)
            for (int q = ctx->n2dRange[n - 1]; q < ctx->n2dRange[n]; ++q)
                if (ctx->n2d[q] == dvar) nd[n] = 1;
        for (int e = 0; e < P.E; ++e)
            for (int a = 0; a < P.npe; ++a)
                if (nd[ctx->elist[8 * (size_t)e + a]]) dep[e] = 1;
    }
    return dep;
}

static int th_check_dvar(astro_ctx *ctx, int dvar, double h) {
    if (!plan_of(ctx)) return set_err(ctx, ASTRO_ERR_STATE, "thermal: astro_thermal_setup not called");
    if (dvar < 1 || dvar > ctx->numDvars)
        return set_err(ctx, ASTRO_ERR_ARG, "design variable " + std::to_string(dvar) + " out of range");
    if (!(h > 0.0)) return set_err(ctx, ASTRO_ERR_ARG, "complex step h must be positive");
    return ASTRO_OK;
}

static ThCsArgs th_cs_args(astro_ctx *ctx, int dvar, double h, double *out) {
    ThCsArgs C = {};
    C.dvar = dvar;
    C.h = h;
    C.secOrig = dptr<double>(ctx->d_secOrig);
    const bool nd = !ctx->n2dRange.empty();
    C.n2dR = nd ? dptr<int>(ctx->d_n2dR) : nullptr;
    C.n2d = nd ? dptr<int>(ctx->d_n2d) : nullptr;
    C.n2c = nd ? dptr<double>(ctx->d_n2c) : nullptr;
    C.out = out;
    return C;
}

// The listed elements (with multiplicity, or all when elements is null) that depend on dvar, by
// colour.
static void th_listed_dependents(const astro_ctx *ctx, const std::vector<char> &dep, const int32_t *elements,
                                 int count, std::vector<int> &list, std::vector<double> &mult, std::vector<int> &ptr) {
    const AstroPrep &P = ctx->P;
    std::vector<int> times((size_t)P.E, elements ? 0 : 1);
    if (elements)
        for (int k = 0; k < count; ++k) ++times[elements[k] - 1];
    list.clear();
    mult.clear();
    ptr.assign(1, 0);
    for (int col = 0; col < P.ncolors; ++col) {
        for (int k = P.colorPtr[col]; k < P.colorPtr[col + 1]; ++k) {
            const int e = P.colorEls[k];
            if (dep[e] && times[e]) {
                list.push_back(e);
                mult.push_back((double)times[e]);
            }
        }
        ptr.push_back((int)list.size());
    }
}

// Runs `launch(els, count, mult)` over the colours of the listed elements with the derivative
// vector on the device, then copies it back.
template <class F>
static int th_cs_run(astro_ctx *ctx, const std::vector<int> &list, const std::vector<double> &mult,
                     const std::vector<int> &ptr, double *drtdd, bool zero, F launch) {
    const int N = ctx->P.N;
    DevBuf dl, dm, dout;
    int rc = ASTRO_OK;
    struct Free {
        DevBuf *b[3];
        ~Free() {
            for (auto *x : b) dev_free(*x);
        }
    } fr{{&dl, &dm, &dout}};
    if (zero) {
        if ((rc = dev_alloc(ctx, dout, sizeof(double) * N))) return rc;
        CK(cudaMemsetAsync(dout.p, 0, sizeof(double) * N, ctx->stream));
    } else if ((rc = upload(ctx, dout, drtdd, sizeof(double) * N))) {
        return rc;
    }
    if (!list.empty()) {
        if ((rc = upload(ctx, dl, list.data(), sizeof(int) * list.size())) ||
            (rc = upload(ctx, dm, mult.data(), sizeof(double) * mult.size())))
            return rc;
        for (size_t col = 0; col + 1 < ptr.size(); ++col) {
            const int cnt = ptr[col + 1] - ptr[col];
            if (cnt) launch(dptr<int>(dl) + ptr[col], cnt, dptr<double>(dm) + ptr[col], dptr<double>(dout));
        }
        if ((rc = cuda_check(ctx, cudaGetLastError(), "thermal complex step"))) return rc;
    }
    CK(cudaMemcpyAsync(drtdd, dout.p, sizeof(double) * N, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return ASTRO_OK;
}

extern "C" int astro_thermal_drdd(astro_ctx *ctx, int32_t dvar, double h, const astro_thermal_state *st,
                                  double *drtdd) {
    if (!ctx || !drtdd) return ASTRO_ERR_ARG;
    int rc;
    if ((rc = th_check_dvar(ctx, dvar, h))) return rc;
    if (st && st->dynamic && !(st->nm_gamma != 0.0 && st->del_t != 0.0))
        return set_err(ctx, ASTRO_ERR_ARG, "thermal: dynamic step needs gamma and a time step");
    ThermPlan *T = plan_of(ctx);
    const int N = ctx->P.N;
    std::vector<int> list, ptr;
    std::vector<double> mult;
    th_listed_dependents(ctx, th_dependents(ctx, dvar), nullptr, 0, list, mult, ptr);
    DevBuf dT, dpT, dpTd;
    struct Free {
        DevBuf *b[3];
        ~Free() {
            for (auto *x : b) dev_free(*x);
        }
    } fr{{&dT, &dpT, &dpTd}};
    if ((rc = up_opt(ctx, dT, st ? st->node_temp : nullptr, N)) ||
        (rc = up_opt(ctx, dpT, st ? st->prev_temp : nullptr, N)) ||
        (rc = up_opt(ctx, dpTd, st ? st->prev_tdot : nullptr, N)))
        return rc;
    ThArgs A = th_args(ctx, T);
    A.temp = dT.p ? dptr<double>(dT) : nullptr;
    A.ptemp = dpT.p ? dptr<double>(dpT) : nullptr;
    A.ptdot = dpTd.p ? dptr<double>(dpTd) : nullptr;
    A.dynamic = st ? st->dynamic : 0;
    A.gamma = st ? st->nm_gamma : 0.5;
    A.delT = st ? st->del_t : 0.0;
    const ThPropArgs Pa = th_prop_args(ctx, T);
    return th_cs_run(ctx, list, mult, ptr, drtdd, true, [&](const int *els, int cnt, const double *, double *out) {
        ThArgs a = A;
        a.els = els;
        a.count = cnt;
        k_th_elem_cs<<<(cnt + 63) / 64, 64, 0, ctx->stream>>>(a, Pa, th_cs_args(ctx, dvar, h, out));
    });
}

extern "C" int astro_thermal_heat_gen_drdd(astro_ctx *ctx, int32_t dvar, double h, double q, const int32_t *elements,
                                           int32_t count, double *drtdd) {
    if (!ctx || !drtdd || count < 0) return ASTRO_ERR_ARG;
    int rc;
    if ((rc = th_check_dvar(ctx, dvar, h))) return rc;
    const AstroPrep &P = ctx->P;
    if (elements)
        for (int k = 0; k < count; ++k)
            if (elements[k] < 1 || elements[k] > P.E) return set_err(ctx, ASTRO_ERR_ARG, "element number out of range");
    ThermPlan *T = plan_of(ctx);
    std::vector<int> list, ptr;
    std::vector<double> mult;
    th_listed_dependents(ctx, th_dependents(ctx, dvar), elements, count, list, mult, ptr);
    if (list.empty()) return ASTRO_OK;
    const ThArgs A = th_args(ctx, T);
    const ThPropArgs Pa = th_prop_args(ctx, T);
    return th_cs_run(ctx, list, mult, ptr, drtdd, false, [&](const int *els, int cnt, const double *m, double *out) {
        ThArgs a = A;
        a.els = els;
        a.count = cnt;
        ThCsArgs C = th_cs_args(ctx, dvar, h, out);
        C.mult = m;
        C.q = q;
        k_th_heatgen_cs<<<(cnt + 63) / 64, 64, 0, ctx->stream>>>(a, Pa, C);
    });
}

extern "C" int astro_thermal_surface_flux_drdd(astro_ctx *ctx, int32_t dvar, double h, int32_t nfaces,
                                               const int32_t *face_el, const int32_t *face_num, double flux,
                                               double *drtdd) {
    if (!ctx || !drtdd || nfaces < 0 || (nfaces && (!face_el || !face_num))) return ASTRO_ERR_ARG;
    int rc;
    if ((rc = th_check_dvar(ctx, dvar, h))) return rc;
    const AstroPrep &P = ctx->P;
    for (int f = 0; f < nfaces; ++f) {
        const int e = face_el[f], fn = face_num[f];
        if (e < 1 || e > P.E) return set_err(ctx, ASTRO_ERR_ARG, "face element out of range");
        if (fn < 1 || fn > ((ctx->etype[e - 1] == 8 || ctx->etype[e - 1] == 81) ? 6 : 2))
            return set_err(ctx, ASTRO_ERR_ARG, "face number out of range");
    }
    // the faces whose element depends on dvar, and the gather lists of their corner values
    static const int hexF[6][4] = {{4, 3, 2, 1}, {5, 6, 7, 8}, {1, 2, 6, 5}, {2, 3, 7, 6}, {3, 4, 8, 7}, {4, 1, 5, 8}};
    static const int shF[2][4] = {{1, 2, 3, 4}, {1, 4, 3, 2}};
    const std::vector<char> dep = th_dependents(ctx, dvar);
    std::vector<int> fe, fnum, slotRow;
    for (int f = 0; f < nfaces; ++f) {
        const int e = face_el[f] - 1;
        if (!dep[e]) continue;
        fe.push_back(face_el[f]);
        fnum.push_back(face_num[f]);
        const int *fl = (ctx->etype[e] == 8 || ctx->etype[e] == 81) ? hexF[face_num[f] - 1] : shF[face_num[f] - 1];
        for (int k = 0; k < 4; ++k) slotRow.push_back(P.currentRank[ctx->elist[8 * (size_t)e + fl[k] - 1]] - 1);
    }
    if (fe.empty()) return ASTRO_OK;
    std::vector<int> order(slotRow.size());
    for (size_t k = 0; k < order.size(); ++k) order[k] = (int)k;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return slotRow[a] < slotRow[b]; });
    std::vector<int> gPtr(1, 0), gRow;
    for (size_t k = 0; k < order.size(); ++k) {
        if (k == 0 || slotRow[order[k]] != slotRow[order[k - 1]]) {
            if (k) gPtr.push_back((int)k);
            gRow.push_back(slotRow[order[k]]);
        }
    }
    gPtr.push_back((int)order.size());
    const int nf = (int)fe.size(), ng = (int)gRow.size(), N = P.N;
    DevBuf dfe, dfn, dfv, dgp, dgs, dgr, dout;
    struct Free {
        DevBuf *b[7];
        ~Free() {
            for (auto *x : b) dev_free(*x);
        }
    } fr{{&dfe, &dfn, &dfv, &dgp, &dgs, &dgr, &dout}};
    if ((rc = upload(ctx, dfe, fe.data(), sizeof(int) * nf)) || (rc = upload(ctx, dfn, fnum.data(), sizeof(int) * nf)) ||
        (rc = dev_alloc(ctx, dfv, sizeof(double) * 4 * (size_t)nf)) ||
        (rc = upload(ctx, dgp, gPtr.data(), sizeof(int) * gPtr.size())) ||
        (rc = upload(ctx, dgs, order.data(), sizeof(int) * order.size())) ||
        (rc = upload(ctx, dgr, gRow.data(), sizeof(int) * ng)) || (rc = upload(ctx, dout, drtdd, sizeof(double) * N)))
        return rc;
    const bool nd = !ctx->n2dRange.empty();
    k_th_flux_cs<<<(nf + 127) / 128, 128, 0, ctx->stream>>>(
        nf, dptr<int>(dfe), dptr<int>(dfn), dptr<int>(ctx->d_etype), dptr<int>(ctx->d_elist), dptr<double>(ctx->d_nodes),
        nd ? dptr<int>(ctx->d_n2dR) : nullptr, nd ? dptr<int>(ctx->d_n2d) : nullptr,
        nd ? dptr<double>(ctx->d_n2c) : nullptr, dptr<int>(ctx->d_dCat), dptr<int>(ctx->d_dComp), dvar, h, flux,
        dptr<double>(dfv));
    k_th_face_gather<<<(ng + 127) / 128, 128, 0, ctx->stream>>>(ng, dptr<int>(dgp), dptr<int>(dgs), dptr<int>(dgr),
                                                                 dptr<double>(dfv), dptr<double>(dout));
    if ((rc = cuda_check(ctx, cudaGetLastError(), "surface flux derivative"))) return rc;
    CK(cudaMemcpyAsync(drtdd, dout.p, sizeof(double) * N, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return ASTRO_OK;
}

static int th_node_dload(astro_ctx *ctx, double t, int mode, int dvar, double *vec) {
    const AstroPrep &P = ctx->P;
    if (ctx->n2dRange.empty()) return ASTRO_OK;
    DevBuf dv, act;
    int rc;
    struct Free {
        DevBuf *b[2];
        ~Free() {
            for (auto *x : b) dev_free(*x);
        }
    } fr{{&dv, &act}};
    if ((rc = upload(ctx, dv, vec, sizeof(double) * P.N))) return rc;
    if (!ctx->dActTime.empty() && (rc = upload(ctx, act, ctx->dActTime.data(), sizeof(double) * ctx->dActTime.size())))
        return rc;
    k_th_node_dload<<<(P.N + 127) / 128, 128, 0, ctx->stream>>>(
        P.N, dptr<int>(ctx->d_rank), dptr<int>(ctx->d_n2dR), dptr<int>(ctx->d_n2d), dptr<double>(ctx->d_n2c),
        dptr<int>(ctx->d_dCat), dptr<int>(ctx->d_dComp), dptr<double>(ctx->d_dVal), act.p ? dptr<double>(act) : nullptr,
        t, mode, dvar, dptr<double>(dv));
    if ((rc = cuda_check(ctx, cudaGetLastError(), "thermal nodal design load"))) return rc;
    CK(cudaMemcpyAsync(vec, dv.p, sizeof(double) * P.N, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return ASTRO_OK;
}

extern "C" int astro_thermal_design_node_load(astro_ctx *ctx, double time, double *thermal_load) {
    if (!ctx || !thermal_load) return ASTRO_ERR_ARG;
    return th_node_dload(ctx, time, 0, 0, thermal_load);
}

extern "C" int astro_thermal_node_load_drdd(astro_ctx *ctx, int32_t dvar, double time, double *drtdd) {
    if (!ctx || !drtdd) return ASTRO_ERR_ARG;
    if (dvar < 1 || dvar > ctx->numDvars)
        return set_err(ctx, ASTRO_ERR_ARG, "design variable " + std::to_string(dvar) + " out of range");
    return th_node_dload(ctx, time, 1, dvar, drtdd);
}
