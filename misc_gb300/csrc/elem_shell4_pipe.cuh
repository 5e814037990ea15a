// shell4 element evaluation as a pipeline of one-thread-per-item kernels over per-element global
// scratch (device code; the algorithm is described in elem_shell4.cu).  For one colour's
// elements at a time:
//   frame    thread per element:            state gather; then thread per (element, rotation):
//                                            the instantaneous frame and its first and second
//                                            rotation derivatives (ten rotations); then thread
//                                            per element: axial vectors, the (0,0) instantaneous
//                                            DOF, Newmark acceleration
//   gauss    thread per (element, point):    shape functions, Jacobian, section forces ABD def
//   dedu     thread per (element, point, i): first derivative of the deformation vector
//   kcol     thread per (element, column j): column j of K (material + stress part) and Ru_j,
//                                            plus the Newmark mass column
//   cond     thread per element:             8x8 internal LU; then thread per (element,
//                                            column): condensation, outputs and the colour-ordered
//                                            block-CSR update (with a matrix only)
//   scatter  thread per (element, DOF):      residual into the load vectors
#pragma once
#include "bounds.cuh"
#include "shell_props.cuh"

namespace {

constexpr double kShellRt3 = 0.57735026918962576451;  // r_1rt3
constexpr double kShellRt3c = LIT(0.577350269189626);  // c_1rt3 (single-precision literal)

struct ShellFrame {
    double io[16][9];   // instantaneous frame, block 4a+b (a,b = rotation components, 0 = none)
    double dr[16][3];   // axial vectors of the frame derivatives
    double U0[6][11];   // instantaneous DOF at the current state
    double u[6][11];    // gathered state (nodal + incompatible modes)
    double X[4][3];     // global coordinates
    double Xl[4][3];    // local coordinates (orient X)
    double rot[3];      // element mean rotation
    double acc[6][4];   // Newmark acceleration of the nodal DOF (dynamic)
    double inam[6][4];  // section mass times the instantaneous nodal acceleration (dynamic)
};

struct ShellGP {
    double Nv[11];
    double Nx[11][3];
    double wdet;
    double F[9];        // section forces ABD def
};

struct ShellPipe {
    const double *nodes;
    const int *elist, *rank, *els, *elBlk;
    int count;
    const ShellProps *props;
    const double *disp, *pdisp, *pvel, *pacc, *idisp;
    int dynamic;
    double beta, gamma, delT;
    int buildMat, quirk;
    int massOnly;    // residual = the Newmark mass term alone (the gravitational load)
    double gpc;      // Gauss point coordinate: r_1rt3, or the complex path's single-precision c_1rt3
    ShellFrame *fr;
    ShellGP *gp;     // count*4
    double *dedU;    // count*4*32*9
    double *Kf;      // count*32*33: column j = 33 values (K(0..31, j), Ru_j)
    double *K, *load, *intLoad, *intMat, *keOut, *ruOut;
    // sizes the index guards of the checked build test against (bounds.cuh): nodes, elements,
    // block-CSR blocks, elements the scratch above holds; status receives the failing guard's site
    int nNodes, nEls, nBlocks, scratchEls;
    int *status;
};

// The frame stage in three parts: the gather (per element), the ten frame rotations (per
// element and rotation: the instantaneous frame and its first and second derivatives, the costly
// part), then the axial vectors, the (0,0) instantaneous DOF and the Newmark acceleration.
__device__ void pipe_frame_gather(const ShellPipe &A, int q) {
    ASTRO_GUARD(A.status, 101, ASTRO_IN(q, A.scratchEls));
    const int e = A.els[q];
    ASTRO_GUARD(A.status, 102, ASTRO_IN(e, A.nEls));
    const int *el = A.elist + 8 * (size_t)e;
    for (int a = 0; a < 4; ++a) ASTRO_GUARD(A.status, 103, ASTRO_IN(el[a] - 1, A.nNodes));
    const ShellProps &P = A.props[e];
    ShellFrame &F = A.fr[q];
    double orient[3][3];
    for (int i = 0; i < 9; ++i) orient[i / 3][i % 3] = P.orient[i];
    for (int a = 0; a < 4; ++a)
        for (int k = 0; k < 3; ++k) F.X[a][k] = A.nodes[3 * (size_t)(el[a] - 1) + k];
    for (int r = 0; r < 6; ++r)
        for (int c = 0; c < 11; ++c) {
            F.u[r][c] = 0.0;
            F.U0[r][c] = 0.0;
        }
    int rk[4];
    for (int a = 0; a < 4; ++a) rk[a] = A.rank[el[a] - 1] - 1;
    for (int a = 0; a < 4; ++a) ASTRO_GUARD(A.status, 104, ASTRO_IN(rk[a], A.nNodes));
    if (A.disp)
        for (int a = 0; a < 4; ++a)
            for (int v = 0; v < 6; ++v) F.u[v][a] = A.disp[6 * (size_t)rk[a] + v];
    if (A.idisp)
        for (int k = 24; k < 32; ++k) {
            int var, nd;
            dof_of(k, var, nd);
            ASTRO_GUARD(A.status, 105, ASTRO_IN(var - 1, 6) && ASTRO_IN(nd - 1, 11));
            F.u[var - 1][nd - 1] = A.idisp[8 * (size_t)e + k - 24];
        }
    for (int a = 0; a < 4; ++a)
        for (int i = 0; i < 3; ++i) F.Xl[a][i] = orient[i][0] * F.X[a][0] + orient[i][1] * F.X[a][1] + orient[i][2] * F.X[a][2];
    for (int k = 0; k < 3; ++k) F.rot[k] = 0.25 * (F.u[3 + k][0] + F.u[3 + k][1] + F.u[3 + k][2] + F.u[3 + k][3]);
}

__device__ void pipe_frame_rot(const ShellPipe &A, int q, int v) {
    ASTRO_GUARD(A.status, 111, ASTRO_IN(q, A.scratchEls) && ASTRO_IN(v, 10));
    const int e = A.els[q];
    ASTRO_GUARD(A.status, 112, ASTRO_IN(e, A.nEls));
    const ShellProps &P = A.props[e];
    ShellFrame &F = A.fr[q];
    double orient[3][3];
    for (int i = 0; i < 9; ++i) orient[i / 3][i % 3] = P.orient[i];
    // frame and derivatives (r_getInstOrient): (0,0), (i,0) and (i,j) i <= j
    {
        const int bi = (v == 0) ? 0 : (v < 4 ? v : (v < 7 ? 1 : (v < 9 ? 2 : 3)));
        const int bj = (v < 4) ? 0 : (v < 7 ? v - 3 : (v < 9 ? v - 5 : 3));
        ASTRO_GUARD(A.status, 113, ASTRO_IN(bi, 4) && ASTRO_IN(bj, 4));
        double out[3][3];
        a_rotate<double>(out, orient, F.rot, bi, bj);
        int b1, b2;
        if (v == 0) b1 = b2 = 0;
        else if (bj == 0) {
            b1 = bi;
            b2 = 4 * bi;
        } else {
            b1 = 4 * bi + bj;
            b2 = 4 * bj + bi;
        }
        for (int t = 0; t < 9; ++t) {
            F.io[b1][t] = out[t / 3][t % 3];
            F.io[b2][t] = out[t / 3][t % 3];
        }
    }
}

__device__ void pipe_frame_rest(const ShellPipe &A, int q) {
    ASTRO_GUARD(A.status, 121, ASTRO_IN(q, A.scratchEls));
    const int e = A.els[q];
    ASTRO_GUARD(A.status, 122, ASTRO_IN(e, A.nEls));
    const int *el = A.elist + 8 * (size_t)e;
    const ShellProps &P = A.props[e];
    ShellFrame &F = A.fr[q];
    double orient[3][3];
    for (int i = 0; i < 9; ++i) orient[i / 3][i % 3] = P.orient[i];
    int rk[4];
    for (int a = 0; a < 4; ++a) rk[a] = A.rank[el[a] - 1] - 1;
    for (int a = 0; a < 4; ++a) ASTRO_GUARD(A.status, 123, ASTRO_IN(rk[a], A.nNodes));
    for (int v = 1; v < 10; ++v) {
        const int bi = (v < 4) ? v : (v < 7 ? 1 : (v < 9 ? 2 : 3));
        const int bj = (v < 4) ? 0 : (v < 7 ? v - 3 : (v < 9 ? v - 5 : 3));
        const int blk = (bj == 0) ? bi : 4 * bi + bj;
        ASTRO_GUARD(A.status, 124, ASTRO_IN(blk, 16) && ASTRO_IN(4 * bi + bj, 16) && ASTRO_IN(4 * bj + bi, 16));
        double pr[3][3];
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b)
                pr[a][b] = F.io[blk][3 * a] * F.io[0][3 * b] + F.io[blk][3 * a + 1] * F.io[0][3 * b + 1] +
                           F.io[blk][3 * a + 2] * F.io[0][3 * b + 2];
        const double ax[3] = {pr[1][2], pr[2][0], pr[0][1]};
        for (int a = 0; a < 3; ++a) {
            if (bj == 0) {
                F.dr[bi][a] = ax[a];
                F.dr[4 * bi][a] = ax[a];
            } else {
                F.dr[4 * bi + bj][a] = ax[a];
                F.dr[4 * bj + bi][a] = ax[a];
            }
        }
    }
    // (0,0) instantaneous DOF (r_getInstDof dv = dv2 = 0)
    for (int a = 0; a < 4; ++a) {
        for (int i = 0; i < 3; ++i) {
            double s = 0.0;
            for (int k = 0; k < 3; ++k) s += F.io[0][3 * i + k] * (F.u[k][a] + F.X[a][k]) - orient[i][k] * F.X[a][k];
            F.U0[i][a] = s;
        }
        double del[3];
        for (int k = 0; k < 3; ++k) del[k] = F.u[3 + k][a] - F.rot[k];
        for (int i = 0; i < 3; ++i) {
            double s = 0.0;
            for (int k = 0; k < 3; ++k) {
                s += F.dr[k + 1][i] * del[k];
                for (int m = 0; m < 3; ++m) s += 0.5 * F.dr[4 * (k + 1) + m + 1][i] * del[k] * del[m];
            }
            F.U0[3 + i][a] = s;
        }
    }
    for (int k = 24; k < 32; ++k) {
        int var, nd;
        dof_of(k, var, nd);
        ASTRO_GUARD(A.status, 125, ASTRO_IN(var - 1, 6) && ASTRO_IN(nd - 1, 11));
        F.U0[var - 1][nd - 1] = F.u[var - 1][nd - 1];
    }
    if (A.dynamic) {
        const double c1 = 0.5 / A.beta, c2 = 2.0 / (A.delT * A.delT);
        for (int a = 0; a < 4; ++a)
            for (int v = 0; v < 6; ++v) {
                const size_t ix = 6 * (size_t)rk[a] + v;
                const double pd = A.pdisp ? A.pdisp[ix] : 0.0, pv = A.pvel ? A.pvel[ix] : 0.0,
                             pa = A.pacc ? A.pacc[ix] : 0.0;
                F.acc[v][a] = c1 * (c2 * (F.u[v][a] - pd - A.delT * pv) - (1.0 - 2.0 * A.beta) * pa);
            }
    }
}

__device__ void pipe_gauss(const ShellPipe &A, int q, int g) {
    ASTRO_GUARD(A.status, 131, ASTRO_IN(q, A.scratchEls) && ASTRO_IN(g, 4) && ASTRO_IN(A.els[q], A.nEls));
    const ShellFrame &F = A.fr[q];
    ShellGP &G = A.gp[4 * (size_t)q + g];
    const ShellProps &P = A.props[A.els[q]];
    const double r3 = A.gpc;
    const double s1 = (g & 1) ? r3 : -r3, s2 = (g & 2) ? r3 : -r3;
    double N[11], d0[11], d1[11];
    N[0] = 0.25 * (1 - s1) * (1 - s2); d0[0] = -0.25 * (1 - s2); d1[0] = -0.25 * (1 - s1);
    N[1] = 0.25 * (1 + s1) * (1 - s2); d0[1] = 0.25 * (1 - s2);  d1[1] = -0.25 * (1 + s1);
    N[2] = 0.25 * (1 + s1) * (1 + s2); d0[2] = 0.25 * (1 + s2);  d1[2] = 0.25 * (1 + s1);
    N[3] = 0.25 * (1 - s1) * (1 + s2); d0[3] = -0.25 * (1 + s2); d1[3] = 0.25 * (1 - s1);
    N[4] = 1 - s1 * s1;                d0[4] = -s1 - s1;         d1[4] = 0.0;
    N[5] = 1 - s2 * s2;                d0[5] = 0.0;              d1[5] = -s2 - s2;
    N[6] = (1 - s1 * s1) * (1 - s2);   d0[6] = (-s1 - s1) * (1 - s2); d1[6] = -(1 - s1 * s1);
    N[7] = (1 - s2 * s2) * (1 + s1);   d0[7] = (1 - s2 * s2);    d1[7] = (-s2 - s2) * (1 + s1);
    N[8] = (1 - s1 * s1) * (1 + s2);   d0[8] = (-s1 - s1) * (1 + s2); d1[8] = (1 - s1 * s1);
    N[9] = (1 - s2 * s2) * (1 - s1);   d0[9] = -(1 - s2 * s2);   d1[9] = (-s2 - s2) * (1 - s1);
    N[10] = 0.0;                       d0[10] = 0.0;             d1[10] = 0.0;
    double J[3][3];
    for (int a = 0; a < 3; ++a) {
        double x0 = 0.0, x1 = 0.0;
        for (int n = 0; n < 4; ++n) {
            x0 += F.Xl[n][a] * d0[n];
            x1 += F.Xl[n][a] * d1[n];
        }
        J[a][0] = x0;
        J[a][1] = x1;
        J[a][2] = 0.0;
    }
    J[2][2] = 1.0;  // shells: dxds(3,3) = 1 (r_getIntPtData)
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
    for (int n = 0; n < 11; ++n) {
        G.Nv[n] = N[n];
        for (int b = 0; b < 3; ++b) G.Nx[n][b] = d0[n] * I[0][b] + d1[n] * I[1][b];
    }
    G.wdet = det;  // unit Gauss weights
    double ux[3][3], rx[3][3], pr[3];
    for (int a = 0; a < 3; ++a) {
        pr[a] = 0.0;
        for (int n = 0; n < 4; ++n) pr[a] += F.U0[3 + a][n] * N[n];
        for (int b = 0; b < 3; ++b) {
            double su = 0.0, sr = 0.0;
            for (int n = 0; n < 10; ++n) {
                su += F.U0[a][n] * G.Nx[n][b];
                sr += F.U0[3 + a][n] * G.Nx[n][b];
            }
            ux[a][b] = su;
            rx[a][b] = sr;
        }
    }
    const double dv[9] = {ux[0][0], ux[1][1], ux[0][1] + ux[1][0], rx[1][0], -rx[0][1], rx[1][1] - rx[0][0],
                          ux[2][0] + pr[1], ux[2][1] - pr[0], 2.0 * pr[2] - ux[1][0] + ux[0][1]};
    for (int a = 0; a < 9; ++a) {
        double s = 0.0;
        for (int b = 0; b < 9; ++b) s += P.ABD[9 * a + b] * dv[b];
        G.F[a] = s;
    }
}

__device__ __forceinline__ void shell_def(const double ux[3][3], const double rx[3][3], const double pr[3], double d[9]) {
    d[0] = ux[0][0];
    d[1] = ux[1][1];
    d[2] = ux[0][1] + ux[1][0];
    d[3] = rx[1][0];
    d[4] = -rx[0][1];
    d[5] = rx[1][1] - rx[0][0];
    d[6] = ux[2][0] + pr[1];
    d[7] = ux[2][1] - pr[0];
    d[8] = 2.0 * pr[2] - ux[1][0] + ux[0][1];
}

// first derivative of the deformation vector with respect to element DOF i (0-based)
__device__ void def_first(const ShellFrame &F, const ShellGP &G, int i, int quirk, double d[9]) {
    int var, nd;
    dof_of(i, var, nd);
    double ux[3][3] = {}, rx[3][3] = {}, pr[3] = {0.0, 0.0, 0.0};
    if (var <= 3) {
        if (nd <= 4) {
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) ux[a][b] = F.io[0][3 * a + var - 1] * G.Nx[nd - 1][b];
        } else {
            for (int b = 0; b < 3; ++b) ux[var - 1][b] = G.Nx[nd - 1][b];
        }
    } else {
        const int v = var - 3;
        for (int a = 0; a < 3; ++a) {
            double tr[4];
            for (int n = 0; n < 4; ++n) {
                double s = 0.0;
                for (int k = 0; k < 3; ++k) s += F.io[v][3 * a + k] * (F.u[k][n] + F.X[n][k]);
                tr[n] = 0.25 * s;
            }
            for (int b = 0; b < 3; ++b) ux[a][b] = tr[0] * G.Nx[0][b] + tr[1] * G.Nx[1][b] + tr[2] * G.Nx[2][b] + tr[3] * G.Nx[3][b];
        }
        double del[3];
        for (int k = 0; k < 3; ++k) del[k] = F.u[3 + k][nd - 1] - F.rot[k];
        for (int a = 0; a < 3; ++a) {
            double s = F.dr[v][a];
            for (int m = 1; m <= 3; ++m) s += 0.5 * F.dr[4 * v + m][a] * del[m - 1] + 0.5 * F.dr[4 * m + v][a] * del[m - 1];
            pr[a] = s * G.Nv[nd - 1];
            if (quirk) pr[a] -= 0.25 * F.dr[v][a];
            for (int b = 0; b < 3; ++b) rx[a][b] = s * G.Nx[nd - 1][b];
        }
    }
    shell_def(ux, rx, pr, d);
}

// second derivative of the deformation vector with respect to DOF i and j (0-based)
__device__ void def_second(const ShellFrame &F, const ShellGP &G, int i, int j, double d[9]) {
    int vi, ni, vj, nj;
    dof_of(i, vi, ni);
    dof_of(j, vj, nj);
    int var1, nd1, var2, nd2;
    if (vi < vj) {
        var1 = vi; nd1 = ni; var2 = vj; nd2 = nj;
    } else {
        var1 = vj; nd1 = nj; var2 = vi; nd2 = ni;
    }
    double ux[3][3] = {}, rx[3][3] = {}, pr[3] = {0.0, 0.0, 0.0};
    if (var1 < 4 && var2 >= 4) {
        const int v2 = var2 - 3;
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) ux[a][b] = 0.25 * F.io[v2][3 * a + var1 - 1] * G.Nx[nd1 - 1][b];
    } else if (var1 >= 4 && var2 >= 4) {
        const int blk = 4 * (var1 - 3) + (var2 - 3);
        for (int a = 0; a < 3; ++a) {
            double tr[4];
            for (int n = 0; n < 4; ++n) {
                double s = 0.0;
                for (int k = 0; k < 3; ++k) s += F.io[blk][3 * a + k] * (F.u[k][n] + F.X[n][k]);
                tr[n] = 0.0625 * s;
            }
            for (int b = 0; b < 3; ++b) ux[a][b] = tr[0] * G.Nx[0][b] + tr[1] * G.Nx[1][b] + tr[2] * G.Nx[2][b] + tr[3] * G.Nx[3][b];
        }
        if (nd1 == nd2)
            for (int a = 0; a < 3; ++a) {
                pr[a] = F.dr[blk][a] * G.Nv[nd1 - 1];
                for (int b = 0; b < 3; ++b) rx[a][b] = F.dr[blk][a] * G.Nx[nd1 - 1][b];
            }
    }
    shell_def(ux, rx, pr, d);
}

__device__ void pipe_dedu(const ShellPipe &A, int q, int g, int i) {
    ASTRO_GUARD(A.status, 141, ASTRO_IN(q, A.scratchEls) && ASTRO_IN(g, 4) && ASTRO_IN(i, 32));
    {
        int var, nd;
        dof_of(i, var, nd);
        ASTRO_GUARD(A.status, 142, var >= 1 && var <= 6 && nd >= 1 && nd <= 10);
    }
    double d[9];
    def_first(A.fr[q], A.gp[4 * (size_t)q + g], i, A.quirk, d);
    double *o = A.dedU + (((size_t)q * 4 + g) * 32 + i) * 9;
    for (int a = 0; a < 9; ++a) o[a] = d[a];
}

// Newmark mass column j (< 24) of r_getElRum: the static frame keeps only its first columns, so
// the derivative of the instantaneous DOF is sparse: translation var at node nd maps to io0(:,var),
// rotation v at node nd to drIdrG(:,v).  With the consistent rotation derivative (quirk) a rotation
// DOF also moves the element mean rotation, so every node's instantaneous rotation changes by
// -drIdrG(:,v)/4: at a point the derivative is then drIdrG(:,v) (N(nd) - sum_k N(k) / 4).
__device__ __forceinline__ void mass_dof(const ShellFrame &F, int i, int &nd, double bv[6]) {
    int var;
    dof_of(i, var, nd);
    for (int r = 0; r < 6; ++r) bv[r] = 0.0;
    if (var <= 3)
        for (int r = 0; r < 3; ++r) bv[r] = F.io[0][3 * r + var - 1];
    else
        for (int r = 0; r < 3; ++r) bv[3 + r] = F.dr[var - 3][r];
}

// instNodalAcc = sum_i acc(var_i, nd_i) * d instU / d u_i (nodal part) and iNAM = M instNodalAcc
// for node n of the element (r_getElRum), the DOF of the node in their order
// the shape-function weight of DOF (var, nd) in the derivative of the instantaneous DOF at a
// point (see mass_dof)
__device__ __forceinline__ double mass_weight(const ShellGP &G, int var, int nd, int quirk) {
    double w = G.Nv[nd - 1];
    if (quirk && var >= 4) w -= 0.25 * (G.Nv[0] + G.Nv[1] + G.Nv[2] + G.Nv[3]);
    return w;
}

__device__ void pipe_inam(const ShellPipe &A, int q, int n) {
    ASTRO_GUARD(A.status, 151, ASTRO_IN(q, A.scratchEls) && ASTRO_IN(n, 4) && ASTRO_IN(A.els[q], A.nEls));
    const ShellProps &P = A.props[A.els[q]];
    ShellFrame &F = A.fr[q];
    double ina[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int var = 1; var <= 6; ++var) {
        int nd;
        double bv[6];
        mass_dof(F, (var - 1) * 4 + n, nd, bv);
        const double a = F.acc[var - 1][nd - 1];
        for (int r = 0; r < 6; ++r) ina[r] += a * bv[r];
    }
    // consistent rotation derivative: the rotation DOF of every node also reach node n through the
    // mean rotation, -1/4 each
    if (A.quirk)
        for (int v = 1; v <= 3; ++v)
            for (int j = 0; j < 4; ++j) {
                const double a = 0.25 * F.acc[2 + v][j];
                for (int r = 0; r < 3; ++r) ina[3 + r] -= a * F.dr[v][r];
            }
    for (int r = 0; r < 6; ++r) {
        double s = 0.0;
        for (int k = 0; k < 6; ++k) s += P.M[6 * r + k] * ina[k];
        F.inam[r][n] = s;
    }
}

__device__ void pipe_kcol(const ShellPipe &A, int q, int j) {
    ASTRO_GUARD(A.status, 161, ASTRO_IN(q, A.scratchEls) && ASTRO_IN(j, 32) && ASTRO_IN(A.els[q], A.nEls));
    const ShellProps &P = A.props[A.els[q]];
    const ShellFrame &F = A.fr[q];
    double *out = A.Kf + ((size_t)q * 32 + j) * 33;
    double Kc[32];
    for (int i = 0; i < 32; ++i) Kc[i] = 0.0;
    double ru = 0.0;
    for (int g = 0; g < 4; ++g) {
        const ShellGP &G = A.gp[4 * (size_t)q + g];
        const double *dj = A.dedU + (((size_t)q * 4 + g) * 32 + j) * 9;
        const double wd = G.wdet;
        bool stressed = false;
        for (int a = 0; a < 9; ++a) {
            if (!A.massOnly) ru += G.F[a] * (wd * dj[a]);
            if (G.F[a] != 0.0) stressed = true;
        }
        if (!A.buildMat) continue;
        double c[9];
        for (int a = 0; a < 9; ++a) {
            double s = 0.0;
            for (int b = 0; b < 9; ++b) s += P.ABD[9 * a + b] * dj[b];
            c[a] = wd * s;
        }
        for (int i = 0; i < 32; ++i) {
            const double *di = A.dedU + (((size_t)q * 4 + g) * 32 + i) * 9;
            double s = 0.0;
            for (int a = 0; a < 9; ++a) s += di[a] * c[a];
            Kc[i] += s;
        }
        if (stressed) {
            for (int i = 0; i < 32; ++i) {
                double d2[9];
                def_second(F, G, i < j ? i : j, i < j ? j : i, d2);
                double s = 0.0;
                for (int a = 0; a < 9; ++a) s += G.F[a] * (wd * d2[a]);
                Kc[i] += s;
            }
        }
    }
    if (A.dynamic && j < 24) {
        const double c1 = 0.5 / A.beta, c2 = 2.0 / (A.delT * A.delT);
        const double(*inam)[4] = F.inam;
        int ndj, varj;
        double bj[6];
        mass_dof(F, j, ndj, bj);
        {
            int t;
            dof_of(j, varj, t);
        }
        double rum = 0.0, mcol[24];
        for (int i = 0; i < 24; ++i) mcol[i] = 0.0;
        for (int g = 0; g < 4; ++g) {
            const ShellGP &G = A.gp[4 * (size_t)q + g];
            const double wd = G.wdet;
            double du[6], fi[6];
            const double wj = mass_weight(G, varj, ndj, A.quirk);
            for (int r = 0; r < 6; ++r) {
                du[r] = bj[r] * wj;
                fi[r] = inam[r][0] * G.Nv[0] + inam[r][1] * G.Nv[1] + inam[r][2] * G.Nv[2] + inam[r][3] * G.Nv[3];
            }
            for (int r = 0; r < 6; ++r) rum += fi[r] * (wd * du[r]);
            if (A.buildMat) {
                double Mdu[6];
                for (int r = 0; r < 6; ++r) {
                    double s = 0.0;
                    for (int k = 0; k < 6; ++k) s += P.M[6 * r + k] * du[k];
                    Mdu[r] = wd * s;
                }
                for (int i = 0; i < 24; ++i) {
                    int ndi, vari, t;
                    double bi[6];
                    mass_dof(F, i, ndi, bi);
                    dof_of(i, vari, t);
                    const double wi = mass_weight(G, vari, ndi, A.quirk);
                    double s = 0.0;
                    for (int r = 0; r < 6; ++r) s += (bi[r] * wi) * Mdu[r];
                    mcol[i] += s;
                }
            }
        }
        ru += rum;
        if (A.buildMat)
            for (int i = 0; i < 24; ++i) Kc[i] += (c1 * c2) * mcol[i];
    }
    for (int i = 0; i < 32; ++i) out[i] = Kc[i];
    out[32] = ru;
}

// static condensation (r_condenseMat on rows/cols 25..32) with a matrix, split: the 8x8 internal
// LU per element, then one thread per (element, column j < 24) for the column's solve, its
// update, and its outputs (block-CSR, element matrix, internal rows); the residual is scattered
// by k_shell_scatter
__device__ void pipe_cond_lu(const ShellPipe &A, int q) {
    ASTRO_GUARD(A.status, 171, ASTRO_IN(q, A.scratchEls));
    const int e = A.els[q];
    ASTRO_GUARD(A.status, 172, ASTRO_IN(e, A.nEls));
    double *Kq = A.Kf + (size_t)q * 32 * 33;
    double L[8][8];
    for (int r = 0; r < 8; ++r)
        for (int c = 0; c < 8; ++c) L[r][c] = Kq[33 * (24 + c) + 24 + r];
    a_lu<double, 8>(&L[0][0], 8);
    for (int r = 0; r < 8; ++r)
        for (int c = 0; c < 8; ++c) Kq[33 * (24 + c) + 24 + r] = L[r][c];
    if (A.intMat) {
        double *dst = A.intMat + 256 * (size_t)e;
        for (int c = 24; c < 32; ++c)
            for (int k = 0; k < 8; ++k) dst[8 * c + k] = Kq[33 * c + 24 + k];
    }
}

__device__ void pipe_cond_col(const ShellPipe &A, int q, int j) {
    ASTRO_GUARD(A.status, 181, ASTRO_IN(q, A.scratchEls) && ASTRO_IN(j, 24));
    const int e = A.els[q];
    ASTRO_GUARD(A.status, 182, ASTRO_IN(e, A.nEls));
    double *Kq = A.Kf + (size_t)q * 32 * 33;
    double L[8][8];
    for (int r = 0; r < 8; ++r)
        for (int c = 0; c < 8; ++c) L[r][c] = Kq[33 * (24 + c) + 24 + r];
    double b[8], x[8];
    for (int k = 0; k < 8; ++k) b[k] = Kq[33 * j + 24 + k];
    a_lu_solve<double, 8>(&L[0][0], b, x, 8);
    for (int i = 0; i < 24; ++i) {
        double s = Kq[33 * j + i];
        for (int k = 0; k < 8; ++k) s -= Kq[33 * (24 + k) + i] * x[k];
        Kq[33 * j + i] = s;
    }
    if (A.intMat) {
        double *dst = A.intMat + 256 * (size_t)e;
        for (int k = 0; k < 8; ++k) dst[8 * j + k] = Kq[33 * j + 24 + k];
    }
    const int cvar = j / 4, bn = j % 4;
    for (int i = 0; i < 24; ++i) {
        const double v = Kq[33 * j + i];
        if (A.K) {
            const int rvar = i / 4, a = i % 4;
            const int blk = A.elBlk[16 * (size_t)e + 4 * a + bn];
            ASTRO_GUARD(A.status, 183, ASTRO_IN(blk, A.nBlocks));
            A.K[36 * (size_t)blk + 6 * rvar + cvar] += v;
        }
        if (A.keOut) A.keOut[576 * (size_t)e + 24 * (size_t)j + i] = v;
    }
}

__global__ void k_shell_cond_lu(ShellPipe A) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < A.count) pipe_cond_lu(A, q);
}
__global__ void k_shell_cond_col(ShellPipe A) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < 24 * A.count) pipe_cond_col(A, t / 24, t % 24);
}

__global__ void k_shell_frame(ShellPipe A) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < A.count) pipe_frame_gather(A, q);
}
__global__ void k_shell_frame_rot(ShellPipe A) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < 10 * A.count) pipe_frame_rot(A, t / 10, t % 10);
}
__global__ void k_shell_frame_rest(ShellPipe A) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < A.count) pipe_frame_rest(A, q);
}
__global__ void k_shell_inam(ShellPipe A) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < 4 * A.count) pipe_inam(A, t / 4, t % 4);
}
// residual scatter without a matrix: one thread per (element, DOF) (a colour's elements share no
// node, an element's DOF are distinct entries)
__global__ void k_shell_scatter(ShellPipe A) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 32 * A.count) return;
    const int q = t / 32, i = t % 32;
    ASTRO_GUARD(A.status, 191, ASTRO_IN(q, A.scratchEls));
    const int e = A.els[q];
    ASTRO_GUARD(A.status, 192, ASTRO_IN(e, A.nEls));
    const double ru = A.Kf[(size_t)q * 32 * 33 + 33 * i + 32];
    if (i < 24) {
        const int var = i / 4, a = i % 4;
        ASTRO_GUARD(A.status, 193, ASTRO_IN(A.elist[8 * (size_t)e + a] - 1, A.nNodes));
        const int r = A.rank[A.elist[8 * (size_t)e + a] - 1] - 1;
        ASTRO_GUARD(A.status, 194, ASTRO_IN(r, A.nNodes));
        if (A.load) A.load[6 * (size_t)r + var] -= ru;
        if (A.ruOut) A.ruOut[24 * (size_t)e + i] = ru;
    } else if (A.intLoad) {
        A.intLoad[8 * (size_t)e + i - 24] -= ru;
    }
}
__global__ void k_shell_gauss(ShellPipe A) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < 4 * A.count) pipe_gauss(A, t / 4, t % 4);
}
__global__ void k_shell_dedu(ShellPipe A) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < 128 * A.count) pipe_dedu(A, t / 128, (t / 32) % 4, t % 32);
}
__global__ void k_shell_kcol(ShellPipe A) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < 32 * A.count) pipe_kcol(A, t / 32, t % 32);
}

}  // namespace
