// Device code of the shell4 element (see elem_shell4.cu for the algorithm description).
#pragma once
#include "shell_math.cuh"


namespace {

constexpr int kSW = 2;  // warps (elements) per CTA

struct ShellProps {       // per element, FP64
    double orient[9];     // row-major, after correctAlpha
    double ABD[81];       // row-major 9x9
    double M[36];         // row-major 6x6 section mass
};

struct LayerDev {
    double E1, E2, nu12, G12, t, angle, rho;
};

// dofTable of shell4 (component-major nodal DOF, then the incompatible modes)
__device__ __forceinline__ void dof_of(int i, int &var, int &nd) {  // i = 0..31, var/nd 1-based
    if (i < 24) {
        var = i / 4 + 1;
        nd = i % 4 + 1;
    } else {
        const int tv[8] = {1, 1, 2, 2, 3, 3, 3, 3}, tn[8] = {5, 6, 5, 6, 7, 8, 9, 10};
        var = tv[i - 24];
        nd = tn[i - 24];
    }
}

// Section properties of one element: orientation with correctAlpha (:240-286), ABD by layer
// integration (r_getShellStiffness, designProp :259-363) and section mass (r_getShellMass,
// :469-525).  Layer thicknesses include the design-variable terms (+ i h on `pertDvar`).
template <class T>
__device__ void shell_props(const double *nodes, const int *el, const double *secOrient, int sec, const int *layRange,
                            const LayerDev *lay, const double *zoff, const int *e2dR, const int *e2d, const double *e2c,
                            const int *dcat, const int *dlay, const double *dval, int e, int pertDvar, double h,
                            T orient[3][3], T ABD[9][9], T Ms[6][6]) {
    T X[4][3];
    for (int a = 0; a < 4; ++a)
        for (int k = 0; k < 3; ++k) X[a][k] = T(nodes[3 * (el[a] - 1) + k]);
    T al[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) al[i][j] = T(secOrient[9 * (sec - 1) + 3 * j + i]);  // column-major input
    // r_getOrientation with no orientation design variables: rotation by zero
    {
        const T z[3] = {T(0.0), T(0.0), T(0.0)};
        a_rotate<T>(orient, al, z, 0, 0);
    }
    // correctAlpha
    {
        T v1[3], v2[3], v3[3];
        for (int k = 0; k < 3; ++k) {
            v1[k] = X[2][k] - X[0][k];
            v2[k] = X[3][k] - X[1][k];
        }
        v3[0] = v1[1] * v2[2] - v1[2] * v2[1];
        v3[1] = v1[2] * v2[0] - v1[0] * v2[2];
        v3[2] = v1[0] * v2[1] - v1[1] * v2[0];
        for (int k = 0; k < 3; ++k) v1[k] = orient[2][k];
        T dp = v1[0] * v3[0] + v1[1] * v3[1] + v1[2] * v3[2];
        if (a_greater(T(0.0), dp))
            for (int k = 0; k < 3; ++k) v3[k] = -v3[k];
        dp = v3[0] * v3[0] + v3[1] * v3[1] + v3[2] * v3[2];
        T mag = a_sqrt(dp);
        for (int k = 0; k < 3; ++k) v2[k] = (T(1.0) / mag) * v3[k];
        v3[0] = v1[1] * v2[2] - v1[2] * v2[1];
        v3[1] = v1[2] * v2[0] - v1[0] * v2[2];
        v3[2] = v1[0] * v2[1] - v1[1] * v2[0];
        dp = v3[0] * v3[0] + v3[1] * v3[1] + v3[2] * v3[2];
        mag = a_sqrt(dp);
        if (absT(mag) > LIT(1e-5)) {
            const T th = a_asin(mag);
            for (int k = 0; k < 3; ++k) v3[k] = (th / mag) * v3[k];
            T a0[3][3];
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) a0[i][j] = orient[i][j];
            a_rotate<T>(orient, a0, v3, 0, 0);
        }
    }
    // layer thicknesses with design variables
    const int l0 = layRange[sec - 1], l1 = layRange[sec];
    auto thick = [&](int li, int layerNum) {
        T t = T(lay[li].t);
        if (e2dR)
            for (int q = e2dR[e]; q < e2dR[e + 1]; ++q) {
                const int d = e2d[q] - 1;
                if (dcat[d] == ASTRO_DCAT_LAYUP_THICKNESS && dlay[d] == layerNum) {
                    T dv = T(dval[d]);
                    if (d + 1 == pertDvar) dv = dv + pert_i<T>(h);
                    t = t + e2c[q] * dv;
                }
            }
        return t;
    };
    T secT = T(0.0);
    for (int li = l0, ln = 1; li < l1; ++li, ++ln) secT = secT + thick(li, ln);
    const T zo = T(zoff[sec - 1]);
    for (int i = 0; i < 9; ++i)
        for (int j = 0; j < 9; ++j) ABD[i][j] = T(0.0);
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) Ms[i][j] = T(0.0);
    T z = -0.5 * secT * (zo + T(1.0));
    T zm = z;
    for (int li = l0, ln = 1; li < l1; ++li, ++ln) {
        const LayerDev L = lay[li];
        const T tl = thick(li, ln);
        const T zn = z + tl;
        T S[3][3] = {{T(1.0) / T(L.E1), -T(L.nu12) / T(L.E1), T(0.0)},
                     {-T(L.nu12) / T(L.E1), T(1.0) / T(L.E2), T(0.0)},
                     {T(0.0), T(0.0), T(1.0) / T(L.G12)}};
        T Q[3][3];
        a_lu<T, 3>(&S[0][0], 3);
        for (int c = 0; c < 3; ++c) {
            T b[3] = {T(0.0), T(0.0), T(0.0)}, x[3];
            b[c] = T(1.0);
            a_lu_solve<T, 3>(&S[0][0], b, x, 3);
            for (int r = 0; r < 3; ++r) Q[r][c] = x[r];
        }
        const T a11 = a_cos(T(L.angle)), a21 = a_sin(T(L.angle));
        const T a12 = -a21, a22 = a11;
        T Ts[3][3] = {{a11 * a11, a12 * a12, 2.0 * a11 * a12},
                      {a21 * a21, a22 * a22, 2.0 * a22 * a21},
                      {a11 * a21, a12 * a22, a11 * a22 + a12 * a21}};
        T Te[3][3];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) Te[i][j] = Ts[i][j];
        for (int k = 0; k < 3; ++k) Te[k][2] = 0.5 * Te[k][2];
        for (int k = 0; k < 3; ++k) Te[2][k] = 2.0 * Te[2][k];
        T TeI[3][3];
        a_lu<T, 3>(&Te[0][0], 3);
        for (int c = 0; c < 3; ++c) {
            T b[3] = {T(0.0), T(0.0), T(0.0)}, x[3];
            b[c] = T(1.0);
            a_lu_solve<T, 3>(&Te[0][0], b, x, 3);
            for (int r = 0; r < 3; ++r) TeI[r][c] = x[r];
        }
        T W[3][3], Qb[3][3];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) W[i][j] = Q[i][0] * TeI[0][j] + Q[i][1] * TeI[1][j] + Q[i][2] * TeI[2][j];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) Qb[i][j] = Ts[i][0] * W[0][j] + Ts[i][1] * W[1][j] + Ts[i][2] * W[2][j];
        const T f0 = zn - z, f1 = 0.5 * (zn * zn - z * z), f2 = AK<T>::o3 * (zn * zn * zn - z * z * z);
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                ABD[i][j] = ABD[i][j] + f0 * Qb[i][j];
                ABD[i][j + 3] = ABD[i][j + 3] + f1 * Qb[i][j];
                ABD[i + 3][j + 3] = ABD[i + 3][j + 3] + f2 * Qb[i][j];
            }
        z = zn;
        // mass (r_getShellMass)
        const T zn2 = zm + tl;
        const T m0 = T(L.rho) * (zn2 - zm), m1 = 0.5 * L.rho * (zn2 * zn2 - zm * zm),
                m2 = AK<T>::o3 * L.rho * (zn2 * zn2 * zn2 - zm * zm * zm);
        for (int k = 0; k < 3; ++k) {
            Ms[k][k] = Ms[k][k] + m0;
            Ms[k + 3][k + 3] = Ms[k + 3][k + 3] + m2;
        }
        Ms[0][4] = Ms[0][4] + m1;
        Ms[1][3] = Ms[1][3] - m1;
        zm = zn2;
    }
    for (int i = 1; i < 6; ++i)
        for (int j = 0; j < i; ++j) {
            ABD[i][j] = ABD[j][i];
            Ms[i][j] = Ms[j][i];
        }
    ABD[6][6] = ABD[2][2];
    ABD[7][7] = ABD[2][2];
    ABD[8][8] = ABD[2][2];
}

struct ShellArgs {
    const double *nodes;
    const int *elist;
    const int *rank;
    const int *colorEls;
    int count;
    const int *elBlk;  // (E,16) block of node pair (a,b)
    const ShellProps *props;
    const double *disp, *pdisp, *pvel, *pacc;  // internal layout (rank*6 + c) or null
    const double *idisp, *pidisp;              // internal DOF (E*8) or null
    int dynamic;
    double beta, gamma, delT;
    int buildMat;
    int quirkMeanRot;
    double *K;         // BSR FP64 (nb*36) or null
    double *load;      // internal layout, -= Ru (nodal)
    double *intLoad;   // (E*8), -= Ru (internal)
    double *intMat;    // (E*256) condensed internal rows
    double *keOut;     // (E,24,24) column-major element DOF order
    double *ruOut;     // (E,24)
    int *status;       // bounds-check status (checked builds)
    long long nE, nN, nn, nnb;
};

struct ShellShared {
    double io[16][3][3];  // instantaneous frame and its derivatives, block 4a+b
    double dr[16][3];     // axial vectors
    double U0[6][11];     // (0,0) instantaneous DOF (local translations/rotations)
    double Nv[11], Nx[11][3];
    double dedU[32][9];
    double Kc[32][33];    // element matrix (column-major by lane), padded
    double lu[8][8];
    double X[4][3], Xl[4][3], u[6][11];
    double orient[3][3], ABD[9][9], M[6][6];
    double rot[3];
    double misc[8];
};

// first derivative of the deformation vector with respect to element DOF i (0-based)
__device__ void def_first(const ShellShared &S, int i, double gi, const double Nv[11], const double Nx[11][3],
                          int quirk, double d[9]) {
    int var, nd;
    dof_of(i, var, nd);
    double ux[3][3] = {}, rx[3][3] = {}, pr[3] = {0, 0, 0};
    if (var <= 3) {
        if (nd <= 4) {
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) ux[a][b] = S.io[0][a][var - 1] * Nx[nd - 1][b];
        } else {
            for (int b = 0; b < 3; ++b) ux[var - 1][b] = Nx[nd - 1][b];
        }
    } else {
        const int v = var - 3;
        // translations: frame derivative acting on (u + X) of all nodes, / numNds
        double tr[3][4];
        for (int a = 0; a < 3; ++a)
            for (int n = 0; n < 4; ++n) {
                double s = 0.0;
                for (int k = 0; k < 3; ++k) s += S.io[v][a][k] * (S.u[k][n] + S.X[n][k]);
                tr[a][n] = 0.25 * s;
            }
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                double s = 0.0;
                for (int n = 0; n < 4; ++n) s += tr[a][n] * Nx[n][b];
                ux[a][b] = s;
            }
        // rotation of node nd: drIdrG e_v + second-order term with delRot = theta_nd - mean
        double del[3];
        for (int k = 0; k < 3; ++k) del[k] = S.u[3 + k][nd - 1] - S.rot[k];
        double w[3];
        for (int a = 0; a < 3; ++a) {
            double s = S.dr[v][a];
            for (int k = 0; k < 3; ++k) {

            }
            // 0.5 * sum_{k,m} dr(4k+m) (e_v(k) del(m) + del(k) e_v(m)) = 0.5 sum_m dr(4v+m) del(m) + 0.5 sum_k dr(4k+v) del(k)
            for (int m = 1; m <= 3; ++m) s += 0.5 * S.dr[4 * v + m][a] * del[m - 1] + 0.5 * S.dr[4 * m + v][a] * del[m - 1];
            w[a] = s;
        }
        if (quirk) {
            // consistent variant: every node's relative rotation also moves with the mean
            for (int a = 0; a < 3; ++a) {
                pr[a] = w[a] * Nv[nd - 1] - 0.25 * S.dr[v][a];
                for (int b = 0; b < 3; ++b) rx[a][b] = w[a] * Nx[nd - 1][b];
            }
        } else {
            for (int a = 0; a < 3; ++a) {
                pr[a] = w[a] * Nv[nd - 1];
                for (int b = 0; b < 3; ++b) rx[a][b] = w[a] * Nx[nd - 1][b];
            }
        }
    }
    d[0] = ux[0][0];
    d[1] = ux[1][1];
    d[2] = ux[0][1] + ux[1][0];
    d[3] = rx[1][0];
    d[4] = -rx[0][1];
    d[5] = rx[1][1] - rx[0][0];
    d[6] = ux[2][0] + pr[1];
    d[7] = ux[2][1] - pr[0];
    d[8] = 2.0 * pr[2] - ux[1][0] + ux[0][1];
    (void)gi;
}

// second derivative of the deformation vector with respect to DOF i and j (0-based)
__device__ void def_second(const ShellShared &S, int i, int j, const double Nv[11], const double Nx[11][3], double d[9]) {
    int vi, ni, vj, nj;
    dof_of(i, vi, ni);
    dof_of(j, vj, nj);
    int var1, nd1, var2, nd2;
    if (vi < vj) {
        var1 = vi; nd1 = ni; var2 = vj; nd2 = nj;
    } else {
        var1 = vj; nd1 = nj; var2 = vi; nd2 = ni;
    }
    double ux[3][3] = {}, rx[3][3] = {}, pr[3] = {0, 0, 0};
    if (var1 < 4 && var2 >= 4) {
        const int v2 = var2 - 3;
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) ux[a][b] = 0.25 * S.io[v2][a][var1 - 1] * Nx[nd1 - 1][b];
    } else if (var1 >= 4 && var2 >= 4) {
        const int v1 = var1 - 3, v2 = var2 - 3, blk = 4 * v1 + v2;
        double tr[3][4];
        for (int a = 0; a < 3; ++a)
            for (int n = 0; n < 4; ++n) {
                double s = 0.0;
                for (int k = 0; k < 3; ++k) s += S.io[blk][a][k] * (S.u[k][n] + S.X[n][k]);
                tr[a][n] = 0.0625 * s;
            }
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                double s = 0.0;
                for (int n = 0; n < 4; ++n) s += tr[a][n] * Nx[n][b];
                ux[a][b] = s;
            }
        if (nd1 == nd2) {
            for (int a = 0; a < 3; ++a) {
                pr[a] = S.dr[blk][a] * Nv[nd1 - 1];
                for (int b = 0; b < 3; ++b) rx[a][b] = S.dr[blk][a] * Nx[nd1 - 1][b];
            }
        }
    }
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

// Bounds-checked builds (-DASTRO_BOUNDS_CHECK): an out-of-range index records the site in a
// status word (first one wins) and the access is skipped, so the kernel never faults.
#ifdef ASTRO_BOUNDS_CHECK
#define BCHK(idx, bound, site) bchk(A.status, (long long)(idx), (long long)(bound), (site))
__device__ __forceinline__ bool bchk(int *status, long long idx, long long bound, int site) {
    if (idx >= 0 && idx < bound) return true;
    if (status) atomicCAS(status, 0, site);
    return false;
}
#else
#define BCHK(idx, bound, site) true
#endif

__global__ void __launch_bounds__(32 * kSW) shell_kernel(ShellArgs A) {
    __shared__ ShellShared SS[kSW];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int item = blockIdx.x * kSW + w;
    if (item >= A.count) return;
    ShellShared &S = SS[w];
    int e = A.colorEls[item];
    if (!BCHK(e, A.nE, 1)) e = 0;
    const int *el = A.elist + 8 * (size_t)e;
    const ShellProps &P = A.props[e];
    // ---- gather -------------------------------------------------------------------------------
    if (lane < 9) S.orient[lane / 3][lane % 3] = P.orient[lane];
    for (int k = lane; k < 81; k += 32) S.ABD[k / 9][k % 9] = P.ABD[k];
    for (int k = lane; k < 36; k += 32) S.M[k / 6][k % 6] = P.M[k];
    if (lane < 12) {
        const int a = lane / 3, k = lane % 3;
        const long long ix = 3 * (long long)(el[a] - 1) + k;
        S.X[a][k] = BCHK(ix, 3 * A.nN, 2) ? A.nodes[ix] : 0.0;
    }
    for (int k = lane; k < 66; k += 32) {
        S.u[k / 11][k % 11] = 0.0;
        S.U0[k / 11][k % 11] = 0.0;
    }
    __syncwarp();
    if (lane < 24) {  // nodal state (component-major element DOF)
        const int var = lane / 4, a = lane % 4;
        const int r = BCHK(el[a] - 1, A.nN, 3) ? A.rank[el[a] - 1] - 1 : 0;
        S.u[var][a] = (A.disp && BCHK(6 * (long long)r + var, A.nn, 4)) ? A.disp[6 * (size_t)r + var] : 0.0;
    } else if (A.idisp) {
        int var, nd;
        dof_of(lane, var, nd);
        if (BCHK(var - 1, 6, 5) && BCHK(nd - 1, 11, 6) && BCHK(8 * (long long)e + lane - 24, 8 * A.nE, 7))
            S.u[var - 1][nd - 1] = A.idisp[8 * (size_t)e + lane - 24];
    }
    __syncwarp();
    if (lane < 12) {
        const int a = lane / 3, i = lane % 3;
        S.Xl[a][i] = S.orient[i][0] * S.X[a][0] + S.orient[i][1] * S.X[a][1] + S.orient[i][2] * S.X[a][2];
    }
    if (lane < 3) S.rot[lane] = 0.25 * (S.u[3 + lane][0] + S.u[3 + lane][1] + S.u[3 + lane][2] + S.u[3 + lane][3]);
    __syncwarp();
    // ---- instantaneous frame and derivatives (r_getInstOrient): ten rotations on ten lanes ----
    {
        // lane 0: (0,0); lanes 1..3: (i,0); lanes 4..9: (i,j), i <= j
        const int pi[10] = {0, 1, 2, 3, 1, 1, 1, 2, 2, 3}, pj[10] = {0, 0, 0, 0, 1, 2, 3, 2, 3, 3};
        if (lane < 10) {
            double al[3][3], out[3][3];
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) al[a][b] = S.orient[a][b];
            a_rotate<double>(out, al, S.rot, pi[lane], pj[lane]);
            const int bi = pi[lane], bj = pj[lane];
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) {
                    if (lane == 0) S.io[0][a][b] = out[a][b];
                    else if (bj == 0) {
                        S.io[bi][a][b] = out[a][b];      // block (0,i) at 3i
                        S.io[4 * bi][a][b] = out[a][b];  // block (i,0) at 12i
                    } else {
                        S.io[4 * bi + bj][a][b] = out[a][b];
                        S.io[4 * bj + bi][a][b] = out[a][b];
                    }
                }
        }
        __syncwarp();
        if (lane >= 1 && lane < 10) {
            const int bi = pi[lane], bj = pj[lane];
            const int blk = (bj == 0) ? bi : 4 * bi + bj;
            double pr[3][3];
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b)
                    pr[a][b] = S.io[blk][a][0] * S.io[0][b][0] + S.io[blk][a][1] * S.io[0][b][1] +
                               S.io[blk][a][2] * S.io[0][b][2];
            const double ax[3] = {pr[1][2], pr[2][0], pr[0][1]};
            for (int a = 0; a < 3; ++a) {
                if (bj == 0) {
                    S.dr[bi][a] = ax[a];
                    S.dr[4 * bi][a] = ax[a];
                } else {
                    S.dr[4 * bi + bj][a] = ax[a];
                    S.dr[4 * bj + bi][a] = ax[a];
                }
            }
        }
        __syncwarp();
    }
    // ---- (0,0) instantaneous DOF (r_getInstDof dv = dv2 = 0) -----------------------------------
    if (lane < 12) {
        const int i = lane / 4, a = lane % 4;
        double s = 0.0;
        for (int k = 0; k < 3; ++k) s += S.io[0][i][k] * (S.u[k][a] + S.X[a][k]) - S.orient[i][k] * S.X[a][k];
        S.U0[i][a] = s;
    } else if (lane < 24) {
        const int i = (lane - 12) / 4, a = (lane - 12) % 4;
        double del[3];
        for (int k = 0; k < 3; ++k) del[k] = S.u[3 + k][a] - S.rot[k];
        double s = 0.0;
        for (int k = 0; k < 3; ++k) {
            s += S.dr[k + 1][i] * del[k];
            for (int m = 0; m < 3; ++m) s += 0.5 * S.dr[4 * (k + 1) + m + 1][i] * del[k] * del[m];
        }
        S.U0[3 + i][a] = s;
    } else {
        // internal DOF copied from the global vector; remaining slots zero
        int var, nd;
        dof_of(lane, var, nd);
        S.U0[var - 1][nd - 1] = S.u[var - 1][nd - 1];
    }
    if (lane < 6) S.U0[lane][10] = 0.0;
    if (lane >= 3 && lane < 6) {
        for (int nd = 5; nd <= 10; ++nd) S.U0[lane][nd - 1] = 0.0;
    }
    __syncwarp();
    // ---- Gauss loop ------------------------------------------------------------------------------
    double Kcol[32];
    for (int k = 0; k < 32; ++k) Kcol[k] = 0.0;
    double ru = 0.0;
    const double g = 0.57735026918962576451;
    for (int gp = 0; gp < 4; ++gp) {
        const double s1 = (gp & 1) ? g : -g, s2 = (gp & 2) ? g : -g;
        if (lane < 11) {
            double N = 0.0, d0 = 0.0, d1 = 0.0;
            switch (lane) {
                case 0: N = 0.25 * (1 - s1) * (1 - s2); d0 = -0.25 * (1 - s2); d1 = -0.25 * (1 - s1); break;
                case 1: N = 0.25 * (1 + s1) * (1 - s2); d0 = 0.25 * (1 - s2); d1 = -0.25 * (1 + s1); break;
                case 2: N = 0.25 * (1 + s1) * (1 + s2); d0 = 0.25 * (1 + s2); d1 = 0.25 * (1 + s1); break;
                case 3: N = 0.25 * (1 - s1) * (1 + s2); d0 = -0.25 * (1 + s2); d1 = 0.25 * (1 - s1); break;
                case 4: N = 1 - s1 * s1; d0 = -s1 - s1; break;
                case 5: N = 1 - s2 * s2; d1 = -s2 - s2; break;
                case 6: N = (1 - s1 * s1) * (1 - s2); d0 = (-s1 - s1) * (1 - s2); d1 = -(1 - s1 * s1); break;
                case 7: N = (1 - s2 * s2) * (1 + s1); d0 = (1 - s2 * s2); d1 = (-s2 - s2) * (1 + s1); break;
                case 8: N = (1 - s1 * s1) * (1 + s2); d0 = (-s1 - s1) * (1 + s2); d1 = (1 - s1 * s1); break;
                case 9: N = (1 - s2 * s2) * (1 - s1); d0 = -(1 - s2 * s2); d1 = (-s2 - s2) * (1 - s1); break;
                default: break;
            }
            S.Nv[lane] = N;
            S.Nx[lane][0] = d0;  // natural derivatives for now
            S.Nx[lane][1] = d1;
            S.Nx[lane][2] = 0.0;
        }
        __syncwarp();
        // Jacobian from the local node coordinates, dxds(3,3) = 1 for shells
        double J[3][3];
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                double s = 0.0;
                if (b < 2)
                    for (int n = 0; n < 4; ++n) s += S.Xl[n][a] * S.Nx[n][b];
                J[a][b] = s;
            }
        J[2][2] = 1.0;
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
        double nsv[3] = {0, 0, 0};
        if (lane < 11) {
            nsv[0] = S.Nx[lane][0];
            nsv[1] = S.Nx[lane][1];
        }
        __syncwarp();
        if (lane < 11)
            for (int b = 0; b < 3; ++b) S.Nx[lane][b] = nsv[0] * I[0][b] + nsv[1] * I[1][b] + nsv[2] * I[2][b];
        __syncwarp();
        double Nv[11], Nx[11][3];
        for (int k = 0; k < 11; ++k) {
            Nv[k] = S.Nv[k];
            for (int b = 0; b < 3; ++b) Nx[k][b] = S.Nx[k][b];
        }
        const double wdet = det;  // unit weights
        // (0,0) deformation and section forces (every lane, identical)
        double ux[3][3], rx[3][3], pr[3];
        for (int a = 0; a < 3; ++a) {
            pr[a] = 0.0;
            for (int n = 0; n < 4; ++n) pr[a] += S.U0[3 + a][n] * Nv[n];
            for (int b = 0; b < 3; ++b) {
                double su = 0.0, sr = 0.0;
                for (int n = 0; n < 10; ++n) {
                    su += S.U0[a][n] * Nx[n][b];
                    sr += S.U0[3 + a][n] * Nx[n][b];
                }
                ux[a][b] = su;
                rx[a][b] = sr;
            }
        }
        double d0[9] = {ux[0][0], ux[1][1], ux[0][1] + ux[1][0], rx[1][0], -rx[0][1], rx[1][1] - rx[0][0],
                        ux[2][0] + pr[1], ux[2][1] - pr[0], 2.0 * pr[2] - ux[1][0] + ux[0][1]};
        double F[9];
        bool stressed = false;
        for (int a = 0; a < 9; ++a) {
            double s = 0.0;
            for (int b = 0; b < 9; ++b) s += S.ABD[a][b] * d0[b];
            F[a] = s;
            if (s != 0.0) stressed = true;
        }
        // first derivatives (lane = DOF)
        double de[9];
        def_first(S, lane, 0.0, Nv, Nx, A.quirkMeanRot, de);
        {
            double s = 0.0;
            for (int a = 0; a < 9; ++a) s += F[a] * (wdet * de[a]);
            ru += s;
        }
        for (int a = 0; a < 9; ++a) S.dedU[lane][a] = de[a];
        __syncwarp();
        if (A.buildMat) {
            // material part: column `lane` += dedU^T ABD dedU(:,lane) wdet
            double c[9];
            for (int a = 0; a < 9; ++a) {
                double s = 0.0;
                for (int b = 0; b < 9; ++b) s += S.ABD[a][b] * de[b];
                c[a] = wdet * s;
            }
            for (int i = 0; i < 32; ++i) {
                double s = 0.0;
                for (int a = 0; a < 9; ++a) s += S.dedU[i][a] * c[a];
                Kcol[i] += s;
            }
            // stress (geometric) part
            if (stressed) {
                for (int i = 0; i < 32; ++i) {
                    double d2[9];
                    const int lo = i < lane ? i : lane, hi = i < lane ? lane : i;
                    def_second(S, lo, hi, Nv, Nx, d2);
                    double s = 0.0;
                    for (int a = 0; a < 9; ++a) s += F[a] * (wdet * d2[a]);
                    Kcol[i] += s;
                }
            }
        }
        __syncwarp();
    }
    // ---- Newmark inertia (r_getElRum / r_getElRu dynamic branch) -------------------------------
    if (A.dynamic && lane < 32) {
        // (not exercised by the static paths; kept minimal: handled in a later revision)
    }
    // ---- static condensation (r_condenseMat) ---------------------------------------------------
    for (int i = 0; i < 32; ++i) S.Kc[lane][i] = Kcol[i];  // Kc[col][row]
    __syncwarp();
    if (A.buildMat) {
        if (lane == 0) {
            for (int r = 0; r < 8; ++r)
                for (int c2 = 0; c2 < 8; ++c2) S.lu[r][c2] = S.Kc[24 + c2][24 + r];
            a_lu<double, 8>(&S.lu[0][0], 8);
            for (int r = 0; r < 8; ++r)
                for (int c2 = 0; c2 < 8; ++c2) S.Kc[24 + c2][24 + r] = S.lu[r][c2];
        }
        __syncwarp();
        double upd[24];
        if (lane < 24) {
            double b[8], x[8];
            for (int k = 0; k < 8; ++k) b[k] = S.Kc[lane][24 + k];
            a_lu_solve<double, 8>(&S.lu[0][0], b, x, 8);
            for (int i = 0; i < 24; ++i) {
                double s = S.Kc[lane][i];
                for (int k = 0; k < 8; ++k) s -= S.Kc[24 + k][i] * x[k];
                upd[i] = s;
            }
        }
        __syncwarp();
        if (lane < 24)
            for (int i = 0; i < 24; ++i) S.Kc[lane][i] = upd[i];
        __syncwarp();
        if (A.intMat) {
            // intElasticMat: for column c = 1..32, rows 25..32
            double *dst = A.intMat + 256 * (size_t)e;
            for (int k = 0; k < 8; ++k) dst[8 * lane + k] = S.Kc[lane][24 + k];
        }
    }
    // ---- outputs -------------------------------------------------------------------------------
    if (lane < 24) {
        const int var = lane / 4, a = lane % 4;
        const int r = BCHK(el[a] - 1, A.nN, 8) ? A.rank[el[a] - 1] - 1 : 0;
        if (A.load && BCHK(6 * (long long)r + var, A.nn, 9)) A.load[6 * (size_t)r + var] -= ru;
        if (A.ruOut) A.ruOut[24 * (size_t)e + lane] = ru;
    } else if (A.intLoad) {
        A.intLoad[8 * (size_t)e + lane - 24] -= ru;
    }
    if (A.buildMat && lane < 24) {
        const int cvar = lane / 4, b = lane % 4;  // column DOF (component, node)
        if (A.K) {
            for (int i = 0; i < 24; ++i) {
                const int rvar = i / 4, a = i % 4;
                const int blk = A.elBlk[16 * (size_t)e + 4 * a + b];
                if (BCHK(blk, A.nnb, 10)) A.K[36 * (size_t)blk + 6 * rvar + cvar] += S.Kc[lane][i];
            }
        }
        if (A.keOut) {
            double *ke = A.keOut + 576 * (size_t)e;
            for (int i = 0; i < 24; ++i) ke[24 * (size_t)lane + i] = S.Kc[lane][i];
        }
    }
}

__global__ void shell_props_kernel(int E, const double *nodes, const int *elist, const int *esec, const double *secOrient,
                                   const int *layRange, const LayerDev *lay, const double *zoff, const int *e2dR,
                                   const int *e2d, const double *e2c, const int *dcat, const int *dlay,
                                   const double *dval, ShellProps *out) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    double o[3][3], ABD[9][9], M[6][6];
    shell_props<double>(nodes, elist + 8 * (size_t)e, secOrient, esec[e], layRange, lay, zoff, e2dR, e2d, e2c, dcat, dlay,
                        dval, e, 0, 0.0, o, ABD, M);
    ShellProps &P = out[e];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) P.orient[3 * i + j] = o[i][j];
    for (int i = 0; i < 9; ++i)
        for (int j = 0; j < 9; ++j) P.ABD[9 * i + j] = ABD[i][j];
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) P.M[6 * i + j] = M[i][j];
}

}  // namespace
