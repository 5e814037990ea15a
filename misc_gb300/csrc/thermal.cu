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

// per element: conductivity in the element frame and heat capacity per volume (per area for
// shells, the section's layers summed), and the shell section thickness
__global__ void k_th_props(int E, int shell, const int *__restrict__ esec, const int *__restrict__ elMatId,
                           const double *__restrict__ elDen, const double *__restrict__ matCond,
                           const double *__restrict__ matSH, const int *__restrict__ layRange,
                           const LayerDev *__restrict__ lay, const double *__restrict__ layCond,
                           const double *__restrict__ laySH, const int *__restrict__ e2dR, const int *__restrict__ e2d,
                           const double *__restrict__ e2c, const int *__restrict__ dcat, const int *__restrict__ dlay,
                           const double *__restrict__ dval, double *__restrict__ out) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    double *o = out + (size_t)kProps * e;
    auto fill = [](double t[3][3], const double *v) {
        t[0][0] = v[0];
        t[1][1] = v[1];
        t[2][2] = v[2];
        t[0][1] = t[1][0] = v[3];
        t[0][2] = t[2][0] = v[4];
        t[1][2] = t[2][1] = v[5];
    };
    double tc[3][3];
    if (!shell) {
        const int mat = elMatId[e];
        fill(tc, matCond + 6 * (mat - 1));
        for (int i = 0; i < 9; ++i) o[i] = tc[i / 3][i % 3];
        o[9] = elDen[e] * matSH[mat - 1];
        o[10] = 0.0;
        return;
    }
    const int sec = esec[e];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) tc[i][j] = 0.0;
    double sh = 0.0, secT = 0.0;
    for (int li = layRange[sec - 1], ln = 1; li < layRange[sec]; ++li, ++ln) {
        double t = lay[li].t;
        if (e2dR)
            for (int q = e2dR[e]; q < e2dR[e + 1]; ++q) {
                const int d = e2d[q] - 1;
                if (dcat[d] == ASTRO_DCAT_LAYUP_THICKNESS && dlay[d] == ln) t = t + e2c[q] * dval[d];
            }
        double tl[3][3], al[3][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}, {0.0, 0.0, 1.0}}, pr[3][3];
        fill(tl, layCond + 6 * li);
        al[0][0] = a_cos(lay[li].angle);
        al[1][0] = a_sin(lay[li].angle);
        al[0][1] = -al[1][0];
        al[1][1] = al[0][0];
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                double s = 0.0;
                for (int k = 0; k < 3; ++k) s = s + tl[a][k] * al[b][k];
                pr[a][b] = s;
            }
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                double s = 0.0;
                for (int k = 0; k < 3; ++k) s = s + al[a][k] * pr[k][b];
                tc[a][b] = tc[a][b] + t * s;
            }
        sh = sh + t * lay[li].rho * laySH[li];
        secT = secT + t;
    }
    for (int i = 0; i < 9; ++i) o[i] = tc[i / 3][i % 3];
    o[9] = sh;
    o[10] = secT;
}

// Gauss point g of the element: shape functions, their global gradient in the element frame and
// w detJ (r_getIntPtData; shells with dxds(3,3) = 1)
__device__ __forceinline__ void th_point(int shell, const double Xl[8][3], int g, double N[8], double Nx[8][3],
                                         double &wdet) {
    const double r3 = 0.57735026918962576451;  // r_1rt3
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
    double J[3][3];
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            double s = 0.0;
            for (int n = 0; n < npe; ++n) s = s + Xl[n][a] * dN[n][b];
            J[a][b] = s;
        }
    if (shell) J[2][2] = 1.0;
    const double c11 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
    const double c12 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
    const double c13 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
    const double det = J[0][0] * c11 + J[0][1] * c12 + J[0][2] * c13;
    const double di = 1.0 / det;
    double I[3][3];
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
    DevBuf den;
    if (ctx->hasSolid) {
        if ((rc = upload(ctx, T->d_elMatId, ctx->elMatId.data(), sizeof(int) * E)) ||
            (rc = upload(ctx, den, ctx->elDensity.data(), sizeof(double) * E)))
            return rc;
    }
    const bool dv = ctx->numDvars > 0 && ctx->d_e2dR.p;
    k_th_props<<<(E + 127) / 128, 128, 0, ctx->stream>>>(
        E, ctx->hasShell, dptr<int>(ctx->d_esec), ctx->hasSolid ? dptr<int>(T->d_elMatId) : nullptr,
        ctx->hasSolid ? dptr<double>(den) : nullptr, dptr<double>(T->d_matCond), dptr<double>(T->d_matSH),
        ctx->hasShell ? dptr<int>(ctx->d_shLayRange) : nullptr, ctx->hasShell ? dptr<LayerDev>(ctx->d_shLay) : nullptr,
        dptr<double>(T->d_layCond), dptr<double>(T->d_laySH), dv ? dptr<int>(ctx->d_e2dR) : nullptr,
        dv ? dptr<int>(ctx->d_e2d) : nullptr, dv ? dptr<double>(ctx->d_e2c) : nullptr,
        dv ? dptr<int>(ctx->d_dCat) : nullptr, dv ? dptr<int>(ctx->d_dLayer) : nullptr,
        dv ? dptr<double>(ctx->d_dVal) : nullptr, dptr<double>(T->d_props));
    rc = cuda_check(ctx, cudaGetLastError(), "thermal properties");
    if (!rc) rc = cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "thermal properties");
    dev_free(den);
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
