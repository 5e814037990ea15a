// brickIM (element type 81): brick8 plus three incompatible bubbles N9 = 1 - s1^2, N10 = 1 - s2^2,
// N11 = 1 - s3^2 (r_EvalN / r_EvalNs, Working/AStrO_r_elementEqns.f90:38-42, :138-142) whose nine
// DOF (three components each, dofTable 25..33 component-major over the bubbles, :377-398) are
// condensed per element (r_condenseMat, :2722-2743).  The Jacobian is the brick8 one (the
// bubbles carry no geometry, r_getIntPtData :580-620 sums over numNds = 8), and the stiffness,
// residual and stress stiffness follow the solid branch of r_getElRuk (:2424-2530) over all
// eleven shape functions; the consistent mass of r_getElRum's solid branch (:2628-2653) couples
// the nodal DOF only, while the Gauss-point acceleration includes the bubbles' (the element's
// gathered state has their displacements and previous displacements, no velocities).
//
// One warp per element, FP64 (brickIM is not on a benchmarked workload; the FP64 pipe bounds it):
//   phase 1, lane gp < 8: Jacobian, its inverse, the eleven gradients, the displacement gradient
//            over the eleven shape functions, Green-Lagrange strain, stress, G = Or + ux^T and the
//            acceleration at the point;
//   phase 2, the 88 (point, shape function) items over the lanes: P = Bloc(g) G,
//            Q = w detJ C P, t = w detJ S g and the residual contribution P^T (w detJ stress);
//   phase 3, the 66 shape-function pairs a <= b over the lanes: the 3x3 blocks of the 33x33
//            element matrix (material + stress + Newmark mass) in shared memory;
//   phase 4, condensation: the unpivoted LU of the internal 9x9 block (one lane), then the 24
//            nodal columns in parallel (each column's update reads only the unchanged internal
//            rows and columns, so the order of the reference's column loop does not matter);
//   outputs: the condensed 24x24 into the block-CSR matrix (colour-ordered, the first element to
//            touch a block writes it), the internal rows (9 x 33, intElasticMat) and the residual
//            (nodal load -= Ru, internal load -= Ru of the bubbles, as getElasticSolnLoad).
#include "astro_internal.h"
#include "bounds.cuh"
#include "shell_math.cuh"

namespace {

constexpr int kRmw81 = 22;  // ceil(64 blocks / 3 blocks per step)

struct Hex81Args {
    const int *els;            // element ids (0-based) of this colour, all of type 81
    int count;
    const int *elBlk;          // (E,64) block of node pair (a,b)
    const unsigned long long *elFirst;
    const int *elist, *rank;
    const int *intVecOff;      // intVecRange (E+1): first internal DOF of each element
    const int *intMatOff;      // intMatRange (E+1)
    const double *nodes;       // (N,3)
    const double *orient;      // (E,9) column-major section orientation, or null (identity)
    const double *elC;         // (E,9) C11 C12 C13 C22 C23 C33 C44 C55 C66
    const double *CItem;       // (count,9) C per listed element (complex step), or null
    const double *rho;         // (E) density
    ElemDevState st;
    double gpc;                // Gauss point coordinate
    int build;                 // element matrix (1) or residual only (0)
    double *K, *loadInt, *intLoad, *intMat, *keOut, *ruOut;
    int nNodes, nEls, nBlocks;
    int *status;
};

struct Hex81Smem {
    double X[8][3];            // node coordinates in the section frame, relative to node 1
    double U[11][3], A[11][3]; // displacement (global components) and acceleration per shape function
    double g[8][11][3];        // gradients per point
    double N[8][11];
    double Gm[8][3][3], sw[8][6], ag[8][3], wd[8];
    union {
        struct {
            double P[88][18], Q[88][18];
            double t[88][3], r[88][3];
            double mN[88];     // c1 c2 rho w detJ N (nodal shape functions only)
        } u;
        double K[33 * 33];     // element matrix, column-major
    };
    int blk[64];
};

__device__ __forceinline__ int dof81(int a, int v) { return a < 8 ? 8 * v + a : 24 + 3 * v + (a - 8); }

__global__ void __launch_bounds__(32) hex81_kernel(Hex81Args A) {
    __shared__ Hex81Smem S;
    const int lane = threadIdx.x;
    const int item = blockIdx.x;
    if (item >= A.count) return;
    const int e = A.els[item];
    ASTRO_GUARD_WARP(A.status, 301, ASTRO_IN(e, A.nEls));
    // every index the warp dereferences below, tested once by the whole warp
    ASTRO_GUARD_WARP(A.status, 302,
                     lane >= 8 || (ASTRO_IN(A.elist[8 * (size_t)e + lane] - 1, A.nNodes) &&
                                   ASTRO_IN(A.rank[A.elist[8 * (size_t)e + lane] - 1] - 1, A.nNodes)));
    ASTRO_GUARD_WARP(A.status, 303, !A.build || (ASTRO_IN(A.elBlk[64 * (size_t)e + lane], A.nBlocks) &&
                                                 ASTRO_IN(A.elBlk[64 * (size_t)e + 32 + lane], A.nBlocks)));
    const double *cp = A.CItem ? A.CItem + 9 * (size_t)item : A.elC + 9 * (size_t)e;
    const double c[9] = {cp[0], cp[1], cp[2], cp[3], cp[4], cp[5], cp[6], cp[7], cp[8]};
    double Or[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) Or[i][j] = A.orient ? A.orient[9 * (size_t)e + 3 * j + i] : (i == j ? 1.0 : 0.0);
    const bool dyn = A.st.dynamic != 0;
    const double c1 = dyn ? 0.5 / A.st.beta : 0.0, c2 = dyn ? 2.0 / (A.st.delT * A.st.delT) : 0.0;
    const int ioff = A.intVecOff[e];
    // gather: lanes 0..7 the nodes, lanes 8..10 the bubbles
    if (lane < 11) {
        double u[3] = {0.0, 0.0, 0.0}, ac[3] = {0.0, 0.0, 0.0};
        if (lane < 8) {
            const int nd = A.elist[8 * (size_t)e + lane];
            const int nd0 = A.elist[8 * (size_t)e];
            for (int i = 0; i < 3; ++i) {
                const double x = A.nodes[3 * (size_t)(nd - 1)] - A.nodes[3 * (size_t)(nd0 - 1)],
                             y = A.nodes[3 * (size_t)(nd - 1) + 1] - A.nodes[3 * (size_t)(nd0 - 1) + 1],
                             z = A.nodes[3 * (size_t)(nd - 1) + 2] - A.nodes[3 * (size_t)(nd0 - 1) + 2];
                S.X[lane][i] = Or[i][0] * x + Or[i][1] * y + Or[i][2] * z;
            }
            const int r = A.rank[nd - 1] - 1;
            for (int v = 0; v < 3; ++v) {
                const size_t ix = 3 * (size_t)r + v;
                u[v] = A.st.disp ? A.st.disp[ix] : 0.0;
                if (dyn) {
                    const double pd = A.st.pdisp ? A.st.pdisp[ix] : 0.0, pv = A.st.pvel ? A.st.pvel[ix] : 0.0,
                                 pa = A.st.pacc ? A.st.pacc[ix] : 0.0;
                    ac[v] = c1 * (c2 * (u[v] - pd - A.st.delT * pv) - (1.0 - 2.0 * A.st.beta) * pa);
                }
            }
        } else {
            const int j = lane - 8;
            for (int v = 0; v < 3; ++v) {
                const int k = ioff + 3 * v + j;
                u[v] = A.st.idisp ? A.st.idisp[k] : 0.0;
                if (dyn) ac[v] = c1 * (c2 * (u[v] - (A.st.pidisp ? A.st.pidisp[k] : 0.0)));
            }
        }
        for (int v = 0; v < 3; ++v) {
            S.U[lane][v] = u[v];
            S.A[lane][v] = ac[v];
        }
    }
    if (A.build) {
        S.blk[lane] = A.elBlk[64 * (size_t)e + lane];
        S.blk[lane + 32] = A.elBlk[64 * (size_t)e + lane + 32];
    }
    __syncwarp();
    // ---- phase 1: lane gp < 8 ---------------------------------------------------------------------
    if (lane < 8) {
        const int gp = lane;
        const double s1 = (gp & 1) ? A.gpc : -A.gpc, s2 = (gp & 2) ? A.gpc : -A.gpc, s3 = (gp & 4) ? A.gpc : -A.gpc;
        double Ns[11][3], N[11];
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
        double J[3][3];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                double v = 0.0;
                for (int a = 0; a < 8; ++a) v += S.X[a][i] * Ns[a][j];
                J[i][j] = v;
            }
        const double a11 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
        const double a12 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
        const double a13 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
        const double det = J[0][0] * a11 + J[0][1] * a12 + J[0][2] * a13;
        const double di = 1.0 / det;
        double I[3][3];
        I[0][0] = di * a11;
        I[1][0] = di * a12;
        I[2][0] = di * a13;
        I[0][1] = di * (J[0][2] * J[2][1] - J[0][1] * J[2][2]);
        I[1][1] = di * (J[0][0] * J[2][2] - J[0][2] * J[2][0]);
        I[2][1] = di * (J[0][1] * J[2][0] - J[0][0] * J[2][1]);
        I[0][2] = di * (J[0][1] * J[1][2] - J[0][2] * J[1][1]);
        I[1][2] = di * (J[0][2] * J[1][0] - J[0][0] * J[1][2]);
        I[2][2] = di * (J[0][0] * J[1][1] - J[0][1] * J[1][0]);
        double ux[3][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}}, ag[3] = {0.0, 0.0, 0.0};
        for (int a = 0; a < 11; ++a) {
            double gg[3];
            for (int j = 0; j < 3; ++j) gg[j] = Ns[a][0] * I[0][j] + Ns[a][1] * I[1][j] + Ns[a][2] * I[2][j];
            for (int j = 0; j < 3; ++j) S.g[gp][a][j] = gg[j];
            S.N[gp][a] = N[a];
            for (int i = 0; i < 3; ++i) {
                for (int j = 0; j < 3; ++j) ux[i][j] += S.U[a][i] * gg[j];
                ag[i] += S.A[a][i] * N[a];
            }
        }
        double uxL[3][3];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) uxL[i][j] = Or[i][0] * ux[0][j] + Or[i][1] * ux[1][j] + Or[i][2] * ux[2][j];
        double st[6];
        for (int j = 0; j < 3; ++j) st[j] = uxL[j][j] + 0.5 * (ux[0][j] * ux[0][j] + ux[1][j] * ux[1][j] + ux[2][j] * ux[2][j]);
        st[3] = uxL[0][1] + uxL[1][0] + ux[0][0] * ux[0][1] + ux[1][0] * ux[1][1] + ux[2][0] * ux[2][1];
        st[4] = uxL[0][2] + uxL[2][0] + ux[0][0] * ux[0][2] + ux[1][0] * ux[1][2] + ux[2][0] * ux[2][2];
        st[5] = uxL[1][2] + uxL[2][1] + ux[0][2] * ux[0][1] + ux[1][2] * ux[1][1] + ux[2][2] * ux[2][1];
        const double wd = det;  // unit Gauss weights
        S.wd[gp] = wd;
        S.sw[gp][0] = wd * (c[0] * st[0] + c[1] * st[1] + c[2] * st[2]);
        S.sw[gp][1] = wd * (c[1] * st[0] + c[3] * st[1] + c[4] * st[2]);
        S.sw[gp][2] = wd * (c[2] * st[0] + c[4] * st[1] + c[5] * st[2]);
        S.sw[gp][3] = wd * (c[6] * st[3]);
        S.sw[gp][4] = wd * (c[7] * st[4]);
        S.sw[gp][5] = wd * (c[8] * st[5]);
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) S.Gm[gp][i][j] = Or[i][j] + ux[j][i];
        for (int i = 0; i < 3; ++i) S.ag[gp][i] = ag[i];
    }
    __syncwarp();
    // ---- phase 2: items (gp, a), a < 11 -------------------------------------------------------------
    const double rhoE = A.rho ? A.rho[e] : 0.0;
    for (int it = lane; it < 88; it += 32) {
        const int gp = it / 11, a = it % 11;
        const double g0 = S.g[gp][a][0], g1 = S.g[gp][a][1], g2 = S.g[gp][a][2], wd = S.wd[gp];
        double P[6][3];
        for (int v = 0; v < 3; ++v) {
            const double G0 = S.Gm[gp][0][v], G1 = S.Gm[gp][1][v], G2 = S.Gm[gp][2][v];
            P[0][v] = g0 * G0;
            P[1][v] = g1 * G1;
            P[2][v] = g2 * G2;
            P[3][v] = g1 * G0 + g0 * G1;
            P[4][v] = g2 * G0 + g0 * G2;
            P[5][v] = g2 * G1 + g1 * G2;
        }
        const double *sw = S.sw[gp];
        for (int v = 0; v < 3; ++v) {
            double r = 0.0;
            for (int q = 0; q < 6; ++q) r += P[q][v] * sw[q];
            // Newmark inertia of the nodal DOF: rho w detJ N_a (acceleration at the point)
            if (dyn && a < 8) r += rhoE * wd * S.ag[gp][v] * S.N[gp][a];
            S.u.r[it][v] = r;
        }
        if (A.build) {
            for (int q = 0; q < 6; ++q)
                for (int v = 0; v < 3; ++v) S.u.P[it][3 * q + v] = P[q][v];
            for (int v = 0; v < 3; ++v) {
                S.u.Q[it][v] = wd * (c[0] * P[0][v] + c[1] * P[1][v] + c[2] * P[2][v]);
                S.u.Q[it][3 + v] = wd * (c[1] * P[0][v] + c[3] * P[1][v] + c[4] * P[2][v]);
                S.u.Q[it][6 + v] = wd * (c[2] * P[0][v] + c[4] * P[1][v] + c[5] * P[2][v]);
                S.u.Q[it][9 + v] = wd * c[6] * P[3][v];
                S.u.Q[it][12 + v] = wd * c[7] * P[4][v];
                S.u.Q[it][15 + v] = wd * c[8] * P[5][v];
            }
            S.u.t[it][0] = sw[0] * g0 + sw[3] * g1 + sw[4] * g2;
            S.u.t[it][1] = sw[3] * g0 + sw[1] * g1 + sw[5] * g2;
            S.u.t[it][2] = sw[4] * g0 + sw[5] * g1 + sw[2] * g2;
            S.u.mN[it] = (dyn && a < 8) ? c1 * c2 * rhoE * wd * S.N[gp][a] : 0.0;
        }
    }
    __syncwarp();
    // residual per shape function (lanes 0..10), summed over the points in order
    double ru[3] = {0.0, 0.0, 0.0};
    if (lane < 11)
        for (int gp = 0; gp < 8; ++gp)
            for (int v = 0; v < 3; ++v) ru[v] += S.u.r[11 * gp + lane][v];
    if (lane < 11) {
        if (lane < 8) {
            if (A.loadInt) {
                const int r = A.rank[A.elist[8 * (size_t)e + lane] - 1] - 1;
                for (int v = 0; v < 3; ++v) A.loadInt[3 * (size_t)r + v] -= ru[v];
            }
            if (A.ruOut)
                for (int v = 0; v < 3; ++v) A.ruOut[24 * (size_t)e + 8 * v + lane] = ru[v];
        } else if (A.intLoad) {
            for (int v = 0; v < 3; ++v) A.intLoad[ioff + 3 * v + lane - 8] -= ru[v];
        }
    }
    if (!A.build) return;
    // ---- phase 3: pairs a <= b of the 11 shape functions (66) -----------------------------------------
    double kt[3][10];  // up to three pairs per lane: 9 entries + the diagonal term
    int pa[3], pb[3];
    for (int k = 0; k < 3; ++k) {
        for (int q = 0; q < 10; ++q) kt[k][q] = 0.0;
        int t = lane + 32 * k, a = 0;
        pa[k] = pb[k] = -1;
        if (t >= 66) continue;
        while (t >= 11 - a) {  // row-major upper triangle of the 11 x 11 pairs (t < 66: a stays < 11)
            t -= 11 - a;
            ++a;
        }
        pa[k] = a;
        pb[k] = a + t;
        for (int gp = 0; gp < 8; ++gp) {
            const int ia = 11 * gp + pa[k], ib = 11 * gp + pb[k];
            for (int q = 0; q < 6; ++q)
                for (int v = 0; v < 3; ++v)
                    for (int x = 0; x < 3; ++x) kt[k][3 * v + x] += S.u.P[ia][3 * q + v] * S.u.Q[ib][3 * q + x];
            double dg = S.g[gp][pa[k]][0] * S.u.t[ib][0] + S.g[gp][pa[k]][1] * S.u.t[ib][1] +
                        S.g[gp][pa[k]][2] * S.u.t[ib][2];
            if (pa[k] < 8 && pb[k] < 8) dg += S.N[gp][pa[k]] * S.u.mN[ib];
            kt[k][9] += dg;
        }
    }
    __syncwarp();
    for (int k = 0; k < 3; ++k) {
        if (pa[k] < 0) continue;
        const int a = pa[k], b = pb[k];
        for (int v = 0; v < 3; ++v)
            for (int x = 0; x < 3; ++x) {
                const double val = kt[k][3 * v + x] + (v == x ? kt[k][9] : 0.0);
                S.K[33 * dof81(b, x) + dof81(a, v)] = val;
                S.K[33 * dof81(a, v) + dof81(b, x)] = val;  // K_ba = K_ab^T
            }
    }
    __syncwarp();
    // ---- phase 4: condensation of the nine internal DOF -------------------------------------------
    if (lane == 0) {
        double L[9][9];
        for (int r = 0; r < 9; ++r)
            for (int cc = 0; cc < 9; ++cc) L[r][cc] = S.K[33 * (24 + cc) + 24 + r];
        a_lu<double, 9>(&L[0][0], 9);
        for (int r = 0; r < 9; ++r)
            for (int cc = 0; cc < 9; ++cc) S.K[33 * (24 + cc) + 24 + r] = L[r][cc];
    }
    __syncwarp();
    if (lane < 24) {
        double L[9][9], bb[9], x[9];
        for (int r = 0; r < 9; ++r)
            for (int cc = 0; cc < 9; ++cc) L[r][cc] = S.K[33 * (24 + cc) + 24 + r];
        for (int k = 0; k < 9; ++k) bb[k] = S.K[33 * lane + 24 + k];
        a_lu_solve<double, 9>(&L[0][0], bb, x, 9);
        for (int i = 0; i < 24; ++i) {
            double s = S.K[33 * lane + i];
            for (int k = 0; k < 9; ++k) s -= S.K[33 * (24 + k) + i] * x[k];
            S.K[33 * lane + i] = s;
        }
    }
    __syncwarp();
    // ---- outputs ---------------------------------------------------------------------------------------
    if (A.intMat) {
        double *dst = A.intMat + A.intMatOff[e];
        for (int q = lane; q < 297; q += 32) {
            const int col = q / 9, k = q % 9;
            dst[q] = S.K[33 * col + 24 + k];
        }
    }
    if (A.keOut) {
        double *ke = A.keOut + 576 * (size_t)e;
        for (int q = lane; q < 576; q += 32) ke[q] = S.K[33 * (q / 24) + q % 24];
    }
    if (A.K) {
        const unsigned long long first = A.elFirst[e];
        const int grp = lane / 9, qq = lane - 9 * grp, bi = qq / 3, bj = qq % 3;
        for (int stp = 0; stp < kRmw81; ++stp) {
            const int j = 3 * stp + grp;  // block (a, b) = (j / 8, j % 8), entry (bi, bj)
            if (grp < 3 && j < 64) {
                const int a = j >> 3, b = j & 7;
                double *dst = A.K + 9 * (size_t)S.blk[j] + qq;
                const double v = S.K[33 * (8 * bj + b) + 8 * bi + a];
                *dst = ((first >> j) & 1ull) ? v : *dst + v;
            }
        }
    }
}

// updateExternalRHS (Working/AStrO_commandFunctions.f90:568-607, intended loop bounds) for the
// brickIM elements: ext -= K_ni K_ii^-1 int per element, from the stored internal rows.
__global__ void k_hex81_ext_rhs(int count, const int *__restrict__ els, const int *__restrict__ elist,
                                const int *__restrict__ rank, const int *__restrict__ intVecOff,
                                const int *__restrict__ intMatOff, const double *__restrict__ intMat,
                                const double *__restrict__ intVec, double *__restrict__ ext) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= count) return;
    const int e = els[q];
    const double *R = intMat + intMatOff[e];  // R[9 * col + k] = K(24 + k, col)
    double L[9][9], b[9], x[9];
    for (int r = 0; r < 9; ++r)
        for (int c = 0; c < 9; ++c) L[r][c] = R[9 * (24 + c) + r];
    for (int k = 0; k < 9; ++k) b[k] = intVec[intVecOff[e] + k];
    a_lu_solve<double, 9>(&L[0][0], b, x, 9);
    for (int i = 0; i < 24; ++i) {
        const int v = i / 8, a = i % 8;
        const int r = rank[elist[8 * (size_t)e + a] - 1] - 1;
        double s = 0.0;
        for (int k = 0; k < 9; ++k) s += R[9 * i + k] * x[k];
        ext[3 * (size_t)r + v] -= s;
    }
}

// updateInternalSoln (:609-651, intended loop bounds): int_soln += K_ii^-1 (int_rhs - K_in u).
__global__ void k_hex81_int_soln(int count, const int *__restrict__ els, const int *__restrict__ elist,
                                 const int *__restrict__ rank, const int *__restrict__ intVecOff,
                                 const int *__restrict__ intMatOff, const double *__restrict__ intMat,
                                 const double *__restrict__ u, double *__restrict__ intSoln,
                                 const double *__restrict__ intRhs) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= count) return;
    const int e = els[q];
    const double *R = intMat + intMatOff[e];
    double L[9][9], b[9], x[9];
    for (int r = 0; r < 9; ++r)
        for (int c = 0; c < 9; ++c) L[r][c] = R[9 * (24 + c) + r];
    const int o = intVecOff[e];
    for (int k = 0; k < 9; ++k) b[k] = intRhs ? intRhs[o + k] : 0.0;
    for (int i = 0; i < 24; ++i) {
        const int v = i / 8, a = i % 8;
        const int r = rank[elist[8 * (size_t)e + a] - 1] - 1;
        const double ui = u[3 * (size_t)r + v];
        for (int k = 0; k < 9; ++k) b[k] -= R[9 * i + k] * ui;
    }
    a_lu_solve<double, 9>(&L[0][0], b, x, 9);
    for (int k = 0; k < 9; ++k) intSoln[o + k] += x[k];
}

}  // namespace

// The brickIM elements of every colour (element lists of the context's type-81 colour split):
// build 1 assembles into K (block-CSR, no zeroing needed), 0 evaluates the residual only.
int hex81_run(astro_ctx *ctx, const int *d_list, const std::vector<int> &ptr, int build, double *K,
              const ElemDevState &st, const double *CItem, double gpc, double *d_loadInt, double *d_intLoad,
              double *d_intMat, double *d_ke, double *d_ru) {
    Hex81Args A;
    A.elBlk = dptr<int>(ctx->d_elBlk);
    A.elFirst = dptr<unsigned long long>(ctx->d_elFirst);
    A.elist = dptr<int>(ctx->d_elist);
    A.rank = dptr<int>(ctx->d_rank);
    A.intVecOff = dptr<int>(ctx->d_intVecOff);
    A.intMatOff = dptr<int>(ctx->d_intMatOff);
    A.nodes = dptr<double>(ctx->d_nodes);
    A.orient = ctx->orientIdentity ? nullptr : dptr<double>(ctx->d_secOrient);
    A.elC = dptr<double>(ctx->d_elC);
    A.rho = dptr<double>(ctx->d_elRho);
    A.st = st;
    A.gpc = gpc;
    A.build = build;
    A.K = K;
    A.loadInt = d_loadInt;
    A.intLoad = d_intLoad;
    A.intMat = d_intMat;
    A.keOut = d_ke;
    A.ruOut = d_ru;
    A.nNodes = ctx->P.N;
    A.nEls = ctx->P.E;
    A.nBlocks = ctx->P.nb;
    A.status = ASTRO_CHECKED ? dptr<int>(ctx->d_guard) : nullptr;
    for (size_t col = 0; col + 1 < ptr.size(); ++col) {
        const int cnt = ptr[col + 1] - ptr[col];
        if (!cnt) continue;
        A.els = d_list + ptr[col];
        A.count = cnt;
        A.CItem = CItem ? CItem + 9 * (size_t)ptr[col] : nullptr;
        hex81_kernel<<<cnt, 32, 0, ctx->stream>>>(A);
    }
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && ASTRO_CHECKED) e = cudaStreamSynchronize(ctx->stream);
    if (e == cudaSuccess && ASTRO_CHECKED) return guard_status(ctx, "brickIM kernel");
    return cuda_check(ctx, e, "brickIM kernel launch");
}

int hex81_update_external_rhs(astro_ctx *ctx, const double *d_intVec, double *d_extInt) {
    const int cnt = (int)ctx->c81Els.size();
    if (!cnt) return ASTRO_OK;
    const int *els = dptr<int>(ctx->d_c81Els);
    // colour by colour: a colour's elements share no node, so the scatter needs no atomics
    for (size_t col = 0; col + 1 < ctx->c81Ptr.size(); ++col) {
        const int c = ctx->c81Ptr[col + 1] - ctx->c81Ptr[col];
        if (!c) continue;
        k_hex81_ext_rhs<<<(c + 127) / 128, 128, 0, ctx->stream>>>(
            c, els + ctx->c81Ptr[col], dptr<int>(ctx->d_elist), dptr<int>(ctx->d_rank), dptr<int>(ctx->d_intVecOff),
            dptr<int>(ctx->d_intMatOff), dptr<double>(ctx->d_intMat), d_intVec, d_extInt);
    }
    return cuda_check(ctx, cudaGetLastError(), "brickIM updateExternalRHS");
}

int hex81_update_internal_soln(astro_ctx *ctx, const double *d_extInt, double *d_intSoln, const double *d_intRhs) {
    const int cnt = (int)ctx->c81Els.size();
    if (!cnt) return ASTRO_OK;
    k_hex81_int_soln<<<(cnt + 127) / 128, 128, 0, ctx->stream>>>(
        cnt, dptr<int>(ctx->d_c81Els), dptr<int>(ctx->d_elist), dptr<int>(ctx->d_rank), dptr<int>(ctx->d_intVecOff),
        dptr<int>(ctx->d_intMatOff), dptr<double>(ctx->d_intMat), d_extInt, d_intSoln, d_intRhs);
    return cuda_check(ctx, cudaGetLastError(), "brickIM updateInternalSoln");
}
