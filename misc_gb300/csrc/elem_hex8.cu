// brick8 element stiffness/residual and colour-ordered assembly into the block-CSR matrix.
//
// Formulation (same quantities as r_getElRuk's solid branch, Working/AStrO_r_elementEqns.f90:
// 2424-2530, written in block form): at each of the 2x2x2 Gauss points (+-1/sqrt(3), unit
// weights, :363-376) with shape derivatives Nx taken in the local frame (locNds = orient *
// globNds, :471-478; Jacobian inverse by cofactors, :212-238),
//   ux      = sum_a disp(:,a) Nx(a,:)            (displacement gradient)
//   strain  = Green-Lagrange strain of r_getNLStrain (:634-648), stress = C strain
//   G       = orient + ux^T                        (the first strain derivative is Bloc(Nx_a) G)
//   K_ab   += w detJ [ G^T Bloc(Nx_a)^T C Bloc(Nx_b) G + (Nx_a^T S Nx_b) I3 ]
//   Ru_a   += w detJ G^T Bloc(Nx_a)^T stress
// with S the stress tensor (second strain derivative, :663-676).  C = S^-1 of the engineering
// constants (r_getMaterialStiffness, Working/AStrO_r_designPropertyFunctions.f90:8-80) is formed
// per element by an unpivoted LU exactly as the reference.
//
// Mapping: one warp per element; lane l owns the node-pair blocks (a,b) = (l/8, l%8) and
// (l/8+4, l%8), i.e. 18 accumulators; lanes 0..7 evaluate node a's shape data and reduce the
// Jacobian and displacement gradient by shuffles.  Elements are processed colour by colour so a
// colour's blocks land in disjoint block rows: plain read-add-write, no atomics, bit-reproducible.
#include "astro_internal.h"
#include "dfloat.cuh"
#include "shell_math.cuh"

namespace {

constexpr int kWarpsPerBlock = 4;
constexpr double kRt3 = 0.57735026918962576451;  // r_1rt3 = 1/sqrt(3) in double
constexpr double kRt3c = LIT(0.577350269189626);  // c_1rt3: a single-precision literal

template <class T> struct Hex8Args {
    const double *nodes;     // (N,3) by node id
    const int *elist;        // (E,8)
    const int *rank;         // currentRank (N) 1-based, indexed by node id - 1
    const int *colorEls;     // element ids of this colour
    int count;               // elements in this colour
    const int *elBlk;        // (E,64)
    const double *elMat;     // (E,9) engineering constants
    const double *orient;    // (E,9) column-major orientation, or nullptr for identity
    const double *disp;      // internal-layout displacement (rank-major, 3 per node) or nullptr
    T *Kbsr;                 // BSR values (nb*9) or nullptr
    double *Kbsr64;          // FP64 BSR to add into as well (FP32 kernel writing both) or nullptr
    double *loadInt;         // internal-layout load, -= Ru (or nullptr)
    double *keOut;           // element matrices (E, 24,24) column-major, element DOF order, or nullptr
    double *ruOut;           // (E,24) or nullptr
    double gpc;              // Gauss point coordinate (1/sqrt(3) of the real or the complex path)
    const double *Cover;     // per listed element a 6x6 row-major C used instead of elMat, or nullptr
};

// C = S^-1 by the reference's unpivoted LU (r_GetInvLU / r_LUFactor / r_SolveLUxb).
template <class T, class P> __device__ void material_c(const P *ep, T C[6][6]) {
    T S[6][6];
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) S[i][j] = T(0);
    T E1 = T(ep[0]), E2 = T(ep[1]), E3 = T(ep[2]);
    S[0][0] = T(1) / E1;
    S[0][1] = -T(ep[3]) / E1;
    S[0][2] = -T(ep[4]) / E1;
    S[1][1] = T(1) / E2;
    S[1][2] = -T(ep[5]) / E2;
    S[2][2] = T(1) / E3;
    S[3][3] = T(1) / T(ep[6]);
    S[4][4] = T(1) / T(ep[7]);
    S[5][5] = T(1) / T(ep[8]);
    for (int i = 1; i < 6; ++i)
        for (int j = 0; j < i; ++j) S[i][j] = S[j][i];
    // LU in place (Doolittle, no pivoting), row i1 then column i1
    for (int i1 = 0; i1 < 6; ++i1) {
        for (int i2 = i1; i2 < 6; ++i2)
            for (int i3 = 0; i3 < i1; ++i3) S[i1][i2] -= S[i1][i3] * S[i3][i2];
        T f = T(1) / S[i1][i1];
        for (int i2 = i1 + 1; i2 < 6; ++i2) {
            for (int i3 = 0; i3 < i1; ++i3) S[i2][i1] -= S[i2][i3] * S[i3][i1];
            S[i2][i1] = f * S[i2][i1];
        }
    }
    for (int col = 0; col < 6; ++col) {
        T z[6], x[6];
        for (int i = 0; i < 6; ++i) {
            z[i] = (i == col) ? T(1) : T(0);
            for (int k = 0; k < i; ++k) z[i] -= S[i][k] * z[k];
        }
        x[5] = z[5] / S[5][5];
        for (int i = 4; i >= 0; --i) {
            T f = T(1) / S[i][i], dp = T(0);
            for (int k = i + 1; k < 6; ++k) dp += S[i][k] * x[k];
            x[i] = f * (z[i] - dp);
        }
        for (int i = 0; i < 6; ++i) C[i][col] = x[i];
    }
}

// M = Bloc(g)^T C Bloc(h), Bloc the 6x3 small-strain operator in Voigt order
// [e11, e22, e33, g12, g13, g23].
template <class T> __device__ __forceinline__ void btcb(const T C[6][6], const T g[3], const T h[3], T M[3][3]) {
    T CB[6][3];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        CB[i][0] = C[i][0] * h[0] + C[i][3] * h[1] + C[i][4] * h[2];
        CB[i][1] = C[i][1] * h[1] + C[i][3] * h[0] + C[i][5] * h[2];
        CB[i][2] = C[i][2] * h[2] + C[i][4] * h[0] + C[i][5] * h[1];
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        M[0][k] = g[0] * CB[0][k] + g[1] * CB[3][k] + g[2] * CB[4][k];
        M[1][k] = g[1] * CB[1][k] + g[0] * CB[3][k] + g[2] * CB[5][k];
        M[2][k] = g[2] * CB[2][k] + g[0] * CB[4][k] + g[1] * CB[5][k];
    }
}

template <class T> __device__ __forceinline__ T wsum8(T v) {
    // sum over lanes 0..7 (the other lanes hold zeros) delivered to all lanes
    v += __shfl_xor_sync(0xffffffffu, v, 1);
    v += __shfl_xor_sync(0xffffffffu, v, 2);
    v += __shfl_xor_sync(0xffffffffu, v, 4);
    return __shfl_sync(0xffffffffu, v, 0);
}

template <class T, bool GENERAL>
__global__ void __launch_bounds__(32 * kWarpsPerBlock) hex8_kernel(Hex8Args<T> A) {
    __shared__ T sNx[kWarpsPerBlock][8][3];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int item = blockIdx.x * kWarpsPerBlock + w;
    if (item >= A.count) return;
    const int e = A.colorEls[item];
    const int a = lane & 7;   // node handled in the per-node phase (lanes 0..7 meaningful)
    const int bA0 = lane >> 3, bA1 = (lane >> 3) + 4, bB = lane & 7;
    // material
    T C[6][6];
    if (A.Cover) {
        for (int i = 0; i < 6; ++i)
            for (int j = 0; j < 6; ++j) C[i][j] = T(A.Cover[36 * (size_t)item + 6 * i + j]);
    } else {
        material_c<T>(A.elMat + 9 * (size_t)e, C);
    }
    T Or[3][3];
    if (GENERAL && A.orient) {
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) Or[i][j] = T(A.orient[9 * (size_t)e + 3 * j + i]);
    } else {
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) Or[i][j] = (i == j) ? T(1) : T(0);
    }
    // node data (lanes 0..7)
    const int nd = A.elist[8 * (size_t)e + a];
    T X[3], U[3] = {T(0), T(0), T(0)};
    {
        T g0 = T(A.nodes[3 * (size_t)(nd - 1)]), g1 = T(A.nodes[3 * (size_t)(nd - 1) + 1]),
          g2 = T(A.nodes[3 * (size_t)(nd - 1) + 2]);
        for (int i = 0; i < 3; ++i) X[i] = Or[i][0] * g0 + Or[i][1] * g1 + Or[i][2] * g2;
        if (GENERAL && A.disp) {
            const int r = A.rank[nd - 1] - 1;
            for (int i = 0; i < 3; ++i) U[i] = T(A.disp[3 * (size_t)r + i]);
        }
    }
    const T sa = (a == 1 || a == 2 || a == 5 || a == 6) ? T(1) : T(-1);
    const T ta = (a == 2 || a == 3 || a == 6 || a == 7) ? T(1) : T(-1);
    const T ua = (a >= 4) ? T(1) : T(-1);
    const T g = T(A.gpc);  // 1/sqrt(3): r_1rt3, or the complex path's single-precision c_1rt3
    T acc0[3][3], acc1[3][3], ru[3] = {T(0), T(0), T(0)};
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) acc0[i][j] = acc1[i][j] = T(0);
    for (int gp = 0; gp < 8; ++gp) {
        const T s1 = (gp & 1) ? g : -g, s2 = (gp & 2) ? g : -g, s3 = (gp & 4) ? g : -g;
        // shape derivatives of node a (r_EvalNs brick8 branch)
        T Ns[3];
        Ns[0] = T(0.125) * sa * (T(1) + ta * s2) * (T(1) + ua * s3);
        Ns[1] = T(0.125) * ta * (T(1) + sa * s1) * (T(1) + ua * s3);
        Ns[2] = T(0.125) * ua * (T(1) + sa * s1) * (T(1) + ta * s2);
        const bool act = lane < 8;
        T J[3][3];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) J[i][j] = wsum8<T>(act ? X[i] * Ns[j] : T(0));
        // cofactor inverse (r_getDetInv)
        T a11 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
        T a12 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
        T a13 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
        T det = J[0][0] * a11 + J[0][1] * a12 + J[0][2] * a13;
        T di = T(1) / det;
        T I[3][3];
        I[0][0] = di * a11;
        I[1][0] = di * a12;
        I[2][0] = di * a13;
        I[0][1] = di * (J[0][2] * J[2][1] - J[0][1] * J[2][2]);
        I[1][1] = di * (J[0][0] * J[2][2] - J[0][2] * J[2][0]);
        I[2][1] = di * (J[0][1] * J[2][0] - J[0][0] * J[2][1]);
        I[0][2] = di * (J[0][1] * J[1][2] - J[0][2] * J[1][1]);
        I[1][2] = di * (J[0][2] * J[1][0] - J[0][0] * J[1][2]);
        I[2][2] = di * (J[0][0] * J[1][1] - J[0][1] * J[1][0]);
        T nx[3];
#pragma unroll
        for (int j = 0; j < 3; ++j) nx[j] = Ns[0] * I[0][j] + Ns[1] * I[1][j] + Ns[2] * I[2][j];
        if (act) {
            sNx[w][a][0] = nx[0];
            sNx[w][a][1] = nx[1];
            sNx[w][a][2] = nx[2];
        }
        __syncwarp();
        const T wdet = det;  // unit Gauss weights
        T Gm[3][3], S3[3][3], stress[6];
        bool nonlin = false;
        if (GENERAL) {
            T ux[3][3];
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j) ux[i][j] = wsum8<T>(act ? U[i] * nx[j] : T(0));
            // Green-Lagrange strain (r_getNLStrain dv = dv2 = 0)
            T uxL[3][3];
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) uxL[i][j] = Or[i][0] * ux[0][j] + Or[i][1] * ux[1][j] + Or[i][2] * ux[2][j];
            T st[6];
            st[0] = uxL[0][0] + T(0.5) * (ux[0][0] * ux[0][0] + ux[1][0] * ux[1][0] + ux[2][0] * ux[2][0]);
            st[1] = uxL[1][1] + T(0.5) * (ux[0][1] * ux[0][1] + ux[1][1] * ux[1][1] + ux[2][1] * ux[2][1]);
            st[2] = uxL[2][2] + T(0.5) * (ux[0][2] * ux[0][2] + ux[1][2] * ux[1][2] + ux[2][2] * ux[2][2]);
            st[3] = uxL[0][1] + uxL[1][0] + ux[0][0] * ux[0][1] + ux[1][0] * ux[1][1] + ux[2][0] * ux[2][1];
            st[4] = uxL[0][2] + uxL[2][0] + ux[0][0] * ux[0][2] + ux[1][0] * ux[1][2] + ux[2][0] * ux[2][2];
            st[5] = uxL[1][2] + uxL[2][1] + ux[0][2] * ux[0][1] + ux[1][2] * ux[1][1] + ux[2][2] * ux[2][1];
            for (int i = 0; i < 6; ++i) {
                stress[i] = T(0);
                for (int k = 0; k < 6; ++k) stress[i] += C[i][k] * st[k];
            }
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) {
                    Gm[i][j] = Or[i][j] + ux[j][i];
                    if (Gm[i][j] != ((i == j) ? T(1) : T(0))) nonlin = true;
                }
            S3[0][0] = stress[0];
            S3[1][1] = stress[1];
            S3[2][2] = stress[2];
            S3[0][1] = S3[1][0] = stress[3];
            S3[0][2] = S3[2][0] = stress[4];
            S3[1][2] = S3[2][1] = stress[5];
            // residual of node a (lanes 0..7)
            if (act) {
                T bs[3];  // Bloc(nx)^T stress
                bs[0] = nx[0] * stress[0] + nx[1] * stress[3] + nx[2] * stress[4];
                bs[1] = nx[1] * stress[1] + nx[0] * stress[3] + nx[2] * stress[5];
                bs[2] = nx[2] * stress[2] + nx[0] * stress[4] + nx[1] * stress[5];
                for (int v = 0; v < 3; ++v) ru[v] += wdet * (Gm[0][v] * bs[0] + Gm[1][v] * bs[1] + Gm[2][v] * bs[2]);
            }
        }
        // blocks (bA0,bB) and (bA1,bB)
        T h[3] = {sNx[w][bB][0], sNx[w][bB][1], sNx[w][bB][2]};
#pragma unroll
        for (int half = 0; half < 2; ++half) {
            const int ia = half ? bA1 : bA0;
            T gg[3] = {sNx[w][ia][0], sNx[w][ia][1], sNx[w][ia][2]};
            T M[3][3];
            btcb<T>(C, gg, h, M);
            T (&acc)[3][3] = half ? acc1 : acc0;
            if (GENERAL && nonlin) {
                T MG[3][3];
                for (int i = 0; i < 3; ++i)
                    for (int k = 0; k < 3; ++k) MG[i][k] = M[i][0] * Gm[0][k] + M[i][1] * Gm[1][k] + M[i][2] * Gm[2][k];
                T geo = T(0);
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j) geo += gg[i] * S3[i][j] * h[j];
                for (int i = 0; i < 3; ++i)
                    for (int k = 0; k < 3; ++k)
                        acc[i][k] += wdet * (Gm[0][i] * MG[0][k] + Gm[1][i] * MG[1][k] + Gm[2][i] * MG[2][k] +
                                             ((i == k) ? geo : T(0)));
            } else {
#pragma unroll
                for (int i = 0; i < 3; ++i)
#pragma unroll
                    for (int k = 0; k < 3; ++k) acc[i][k] += wdet * M[i][k];
            }
        }
        __syncwarp();
    }
    // outputs
    const int *blk = A.elBlk + 64 * (size_t)e;
#pragma unroll
    for (int half = 0; half < 2; ++half) {
        const int ia = half ? bA1 : bA0;
        T (&acc)[3][3] = half ? acc1 : acc0;
        const int k = blk[ia * 8 + bB];
        if (A.Kbsr) {
            T *dst = A.Kbsr + 9 * (size_t)k;
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j) dst[3 * i + j] += acc[i][j];
        }
        if (A.Kbsr64) {
            double *dst = A.Kbsr64 + 9 * (size_t)k;
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j) dst[3 * i + j] += (double)acc[i][j];
        }
        if (A.keOut) {
            double *ke = A.keOut + 576 * (size_t)e;
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) ke[(size_t)(8 * j + bB) * 24 + (8 * i + ia)] = (double)acc[i][j];
        }
    }
    if (GENERAL && lane < 8) {
        if (A.loadInt) {
            const int r = A.rank[nd - 1] - 1;
            for (int v = 0; v < 3; ++v) A.loadInt[3 * (size_t)r + v] -= (double)ru[v];
        }
        if (A.ruOut)
            for (int v = 0; v < 3; ++v) A.ruOut[24 * (size_t)e + 8 * v + a] = (double)ru[v];
    }
}

// ---------------------------------------------------------------------------------------------
// Zero-state brick8 stiffness and assembly: FP32 for the mixed-precision solver's matrix, FP64
// for getElasticSolnLoad from the undeformed state (where the residual is exactly zero and the
// tangent is the small-strain stiffness).  Per element (one warp):
//   * the orthotropic C of the element, computed once per context by the reference's LU
//     (r_getMaterialStiffness);
//   * the node coordinates in the section frame (orient X, as r_getElementData stages them);
//   * the eight Gauss-point Jacobians in one round: lane (g, s) with g = lane/4, s = lane%4 forms
//     the contribution of nodes 2s and 2s+1 to J at point g, the four lanes of a point reduce it
//     with two xor-shuffles, invert it, and write the gradients g_a and w detJ g_a of their two
//     nodes to shared memory;
//   * lane l owns the node pairs (l/8, l%8) and (l/8+4, l%8).  For a pair (a, b) the 3x3
//     moment M = sum_gp w detJ g_a g_b^T is accumulated (9 products per point), and the block
//     follows from the orthotropic C in one contraction (21 products):
//       K00 = C11 M00 + C44 M11 + C55 M22,  K01 = C12 M01 + C44 M10,  K02 = C13 M02 + C55 M20, ...
//     which is the sparse B^T C B of the element summed over the points, reassociated; a rotated
//     section frame maps the block back with orient^T K orient.  GB300 issues FP64 at 1/64 of
//     its FP32 rate, so in the FP64 kernel the moments, which are most of the arithmetic, are
//     accumulated in double-float (pairs of floats with error-free products and sums, about 48
//     significant bits) and only the Jacobians and the final contraction run in FP64;
//   * the 64 blocks go through shared memory and are added into the block-CSR matrix three whole
//     blocks (27 lanes, 9 contiguous values each) per warp instruction, instead of one lane per
//     block touching a different cache line for every value; the first element (in colour order)
//     to touch a block writes it, so an assembly pass needs no zeroing.  In FP32 the old values
//     are fetched before the arithmetic so their latency overlaps it (in FP64 the registers are
//     better spent on occupancy).
constexpr int kRmwSteps = 22;  // ceil(64 blocks / 3 blocks per step)

template <class T> struct FastCfg;
template <> struct FastCfg<float> {
    static constexpr int FW = 2, MINB = 14;  // warps per CTA, CTAs per SM (small CTAs: shorter colour tails)
    static constexpr bool PREFETCH = true;
};
template <class T> struct Hex8FastArgs {
    const int *colorEls;
    int count;
    const int *elBlk;
    const unsigned long long *elFirst;
    const float2 *Xdf;     // (E,8,3) node coordinates in the section frame, double-float (high parts used)
    const float2 *Cdf;     // (E,9) orthotropic C, double-float (high parts used)
    const double *orient;  // (E,9) column-major section orientation (used when ROT)
    T *K;                  // BSR values or null
    double *keOut;         // element matrices (E,24,24) column-major, element DOF order, or null
};

template <class T> struct OrthoC {
    T C11, C12, C13, C22, C23, C33, C44, C55, C66;
};

template <class T> __device__ __forceinline__ void ortho_block(const OrthoC<T> &c, const T M[9], T K[9]) {
    K[0] = c.C11 * M[0] + c.C44 * M[4] + c.C55 * M[8];
    K[1] = c.C12 * M[1] + c.C44 * M[3];
    K[2] = c.C13 * M[2] + c.C55 * M[6];
    K[3] = c.C12 * M[3] + c.C44 * M[1];
    K[4] = c.C22 * M[4] + c.C44 * M[0] + c.C66 * M[8];
    K[5] = c.C23 * M[5] + c.C66 * M[7];
    K[6] = c.C13 * M[6] + c.C55 * M[2];
    K[7] = c.C23 * M[7] + c.C66 * M[5];
    K[8] = c.C33 * M[8] + c.C55 * M[0] + c.C66 * M[4];
}

// K <- Or^T K Or (row-major 3x3)
template <class T> __device__ __forceinline__ void rotate_block(const T Or[3][3], T K[9]) {
    T W[3][3];
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int j = 0; j < 3; ++j) W[k][j] = K[3 * k] * Or[0][j] + K[3 * k + 1] * Or[1][j] + K[3 * k + 2] * Or[2][j];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) K[3 * i + j] = Or[0][i] * W[0][j] + Or[1][i] * W[1][j] + Or[2][i] * W[2][j];
}

// per-warp shared staging of the Gauss-point gradients: g_a and h_a = w detJ g_a
template <class T> struct GradSmem;
template <> struct GradSmem<float> {
    float4 g[8][8], h[8][8];  // [gauss point][node]
    __device__ void put(int gp, int a, float gx, float gy, float gz, float d) {
        g[gp][a] = make_float4(gx, gy, gz, 0.f);
        h[gp][a] = make_float4(d * gx, d * gy, d * gz, 0.f);
    }
};
// 3x3 moments of the pairs (a0, b) and (a1, b): M = sum_gp g_a h_b^T
__device__ __forceinline__ void pair_moments(const GradSmem<float> &S, int a0, int a1, int b, float M0[9],
                                             float M1[9]) {
#pragma unroll
    for (int q = 0; q < 9; ++q) M0[q] = M1[q] = 0.f;
#pragma unroll
    for (int gp = 0; gp < 8; ++gp) {
        const float4 hb = S.h[gp][b], ga = S.g[gp][a0], gc = S.g[gp][a1];
        M0[0] += ga.x * hb.x; M0[1] += ga.x * hb.y; M0[2] += ga.x * hb.z;
        M0[3] += ga.y * hb.x; M0[4] += ga.y * hb.y; M0[5] += ga.y * hb.z;
        M0[6] += ga.z * hb.x; M0[7] += ga.z * hb.y; M0[8] += ga.z * hb.z;
        M1[0] += gc.x * hb.x; M1[1] += gc.x * hb.y; M1[2] += gc.x * hb.z;
        M1[3] += gc.y * hb.x; M1[4] += gc.y * hb.y; M1[5] += gc.y * hb.z;
        M1[6] += gc.z * hb.x; M1[7] += gc.z * hb.y; M1[8] += gc.z * hb.z;
    }
}
template <class T, bool ROT>
__global__ void __launch_bounds__(32 * FastCfg<T>::FW, FastCfg<T>::MINB) hex8_fast_kernel(Hex8FastArgs<T> A) {
    constexpr int FW = FastCfg<T>::FW;
    constexpr bool PREFETCH = FastCfg<T>::PREFETCH;
    __shared__ GradSmem<T> sG[FW];
    __shared__ T sK[FW][64 * 9];  // element blocks, block j = 8a + b at 9j (row-major 3x3)
    __shared__ int sBlk[FW][64];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int item = blockIdx.x * FW + w;
    if (item >= A.count) return;
    const int e = A.colorEls[item];
    // block targets; in the cooperative phase lane = 9 grp + qq handles entry qq of block 3 st + grp
    sBlk[w][lane] = A.elBlk[64 * (size_t)e + lane];
    sBlk[w][lane + 32] = A.elBlk[64 * (size_t)e + lane + 32];
    const unsigned long long first = A.elFirst[e];
    const int grp = lane / 9, qq = lane - 9 * grp;
    __syncwarp();
    T ov[PREFETCH ? kRmwSteps : 1];
    if (PREFETCH) {
#pragma unroll
        for (int st = 0; st < kRmwSteps; ++st) {
            const int j = 3 * st + grp;
            ov[st] = T(0);
            if (A.K && grp < 3 && j < 64 && !((first >> j) & 1ull)) ov[st] = A.K[9 * (size_t)sBlk[w][j] + qq];
        }
    }
    // Jacobian at Gauss point gp = lane/4 from nodes 2s, 2s+1 (s = lane%4), from the node
    // coordinates in the section frame (single-precision parts of the double-float copy)
    {
        const int gp = lane >> 2, s = lane & 3;
        const T gq = (T)kRt3, eighth = T(0.125);
        const T s1 = (gp & 1) ? gq : -gq, s2 = (gp & 2) ? gq : -gq, s3 = (gp & 4) ? gq : -gq;
        T J[9], n[2][3];
#pragma unroll
        for (int q = 0; q < 9; ++q) J[q] = T(0);
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const int a = 2 * s + k;
            const float2 *xp = A.Xdf + 24 * (size_t)e + 3 * a;
            const T X0 = xp[0].x, X1 = xp[1].x, X2 = xp[2].x;
        const T sa = (a == 1 || a == 2 || a == 5 || a == 6) ? T(1) : T(-1);
            const T ta = (a == 2 || a == 3 || a == 6 || a == 7) ? T(1) : T(-1);
            const T ua = (a >= 4) ? T(1) : T(-1);
            n[k][0] = eighth * sa * (T(1) + ta * s2) * (T(1) + ua * s3);
            n[k][1] = eighth * ta * (T(1) + sa * s1) * (T(1) + ua * s3);
            n[k][2] = eighth * ua * (T(1) + sa * s1) * (T(1) + ta * s2);
            J[0] += X0 * n[k][0]; J[1] += X0 * n[k][1]; J[2] += X0 * n[k][2];
            J[3] += X1 * n[k][0]; J[4] += X1 * n[k][1]; J[5] += X1 * n[k][2];
            J[6] += X2 * n[k][0]; J[7] += X2 * n[k][1]; J[8] += X2 * n[k][2];
        }
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            J[q] += __shfl_xor_sync(0xffffffffu, J[q], 1);
            J[q] += __shfl_xor_sync(0xffffffffu, J[q], 2);
        }
        const T a11 = J[4] * J[8] - J[5] * J[7], a12 = J[5] * J[6] - J[3] * J[8], a13 = J[3] * J[7] - J[4] * J[6];
        const T dt = J[0] * a11 + J[1] * a12 + J[2] * a13, di = T(1) / dt;
        const T I00 = di * a11, I10 = di * a12, I20 = di * a13;
        const T I01 = di * (J[2] * J[7] - J[1] * J[8]), I11 = di * (J[0] * J[8] - J[2] * J[6]),
                I21 = di * (J[1] * J[6] - J[0] * J[7]);
        const T I02 = di * (J[1] * J[5] - J[2] * J[4]), I12 = di * (J[2] * J[3] - J[0] * J[5]),
                I22 = di * (J[0] * J[4] - J[1] * J[3]);
#pragma unroll
        for (int k = 0; k < 2; ++k)
            sG[w].put(gp, 2 * s + k, n[k][0] * I00 + n[k][1] * I10 + n[k][2] * I20,
                      n[k][0] * I01 + n[k][1] * I11 + n[k][2] * I21, n[k][0] * I02 + n[k][1] * I12 + n[k][2] * I22,
                      dt);
    }
    __syncwarp();
    const int a0 = lane >> 3, a1 = a0 + 4, b = lane & 7;
    T M0[9], M1[9];
    pair_moments(sG[w], a0, a1, b, M0, M1);
    OrthoC<T> c;
    {
        const float2 *cp = A.Cdf + 9 * (size_t)e;
        c.C11 = cp[0].x;
        c.C12 = cp[1].x;
        c.C13 = cp[2].x;
        c.C22 = cp[3].x;
        c.C23 = cp[4].x;
        c.C33 = cp[5].x;
        c.C44 = cp[6].x;
        c.C55 = cp[7].x;
        c.C66 = cp[8].x;
    }
    T K0[9], K1[9];
    ortho_block<T>(c, M0, K0);
    ortho_block<T>(c, M1, K1);
    if (ROT) {
        T Or[3][3];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) Or[i][j] = (T)A.orient[9 * (size_t)e + 3 * j + i];
        rotate_block<T>(Or, K0);
        rotate_block<T>(Or, K1);
    }
    if (A.K) {
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            sK[w][9 * lane + q] = K0[q];
            sK[w][9 * (lane + 32) + q] = K1[q];
        }
        __syncwarp();
#pragma unroll
        for (int st = 0; st < kRmwSteps; ++st) {
            const int j = 3 * st + grp;
            if (grp < 3 && j < 64) {
                T *dst = A.K + 9 * (size_t)sBlk[w][j] + qq;
                T old;
                if (PREFETCH)
                    old = ov[PREFETCH ? st : 0];
                else
                    old = ((first >> j) & 1ull) ? T(0) : *dst;
                *dst = old + sK[w][9 * j + qq];
            }
        }
    }
    if (A.keOut) {
        double *ke = A.keOut + 576 * (size_t)e;
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                ke[(size_t)(8 * j + b) * 24 + (8 * i + a0)] = (double)K0[3 * i + j];
                ke[(size_t)(8 * j + b) * 24 + (8 * i + a1)] = (double)K1[3 * i + j];
            }
    }
}

// FP64 zero-state kernel in double-float.  Same mapping as hex8_fast_kernel; the Jacobians,
// their inverses, the gradients, the moments and the contraction with C run on the FP32 pipe in
// double-float, from node coordinates (section frame) and C split once per context; FP64 is
// used for the delivered blocks (and the rotation back from a rotated section frame).
struct Hex8DfArgs {
    const int *colorEls;
    int count;
    const int *elBlk;
    const unsigned long long *elFirst;
    const float2 *Xdf;     // (E,8,3) node coordinates in the section frame, double-float
    const float2 *Cdf;     // (E,9) orthotropic C, double-float
    const double *orient;  // (E,9) column-major section orientation (used when ROT)
    double *K;             // BSR values or null
    double *keOut;         // element matrices (E,24,24) column-major, element DOF order, or null
};

constexpr int kDfW = 4;  // warps per CTA
constexpr float kRt3Hi = (float)kRt3;
constexpr float kRt3Lo = (float)(kRt3 - (double)kRt3Hi);

struct DfGrad {
    float4 gh[8][8], gl[8][8], hh[8][8], hl[8][8];  // [gauss point][node]: g_a and w detJ g_a
};

__device__ __forceinline__ void df_ortho(const DF c[9], const DF M[9], DF K[9]) {
    // c = C11 C12 C13 C22 C23 C33 C44 C55 C66
    K[0] = df_add(df_add(df_mul(c[0], M[0]), df_mul(c[6], M[4])), df_mul(c[7], M[8]));
    K[1] = df_add(df_mul(c[1], M[1]), df_mul(c[6], M[3]));
    K[2] = df_add(df_mul(c[2], M[2]), df_mul(c[7], M[6]));
    K[3] = df_add(df_mul(c[1], M[3]), df_mul(c[6], M[1]));
    K[4] = df_add(df_add(df_mul(c[3], M[4]), df_mul(c[6], M[0])), df_mul(c[8], M[8]));
    K[5] = df_add(df_mul(c[4], M[5]), df_mul(c[8], M[7]));
    K[6] = df_add(df_mul(c[2], M[6]), df_mul(c[7], M[2]));
    K[7] = df_add(df_mul(c[4], M[7]), df_mul(c[8], M[5]));
    K[8] = df_add(df_add(df_mul(c[5], M[8]), df_mul(c[7], M[0])), df_mul(c[8], M[4]));
}

// 4 CTAs per SM: 128 registers, no spills (3 CTAs let ptxas take 167 and ran 11 % slower)
template <bool ROT> __global__ void __launch_bounds__(32 * kDfW, 4) hex8_df_kernel(Hex8DfArgs A) {
    __shared__ DfGrad sG[kDfW];
    __shared__ double sK[kDfW][64 * 9];
    __shared__ int sBlk[kDfW][64];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int item = blockIdx.x * kDfW + w;
    if (item >= A.count) return;
    const int e = A.colorEls[item];
    sBlk[w][lane] = A.elBlk[64 * (size_t)e + lane];
    sBlk[w][lane + 32] = A.elBlk[64 * (size_t)e + lane + 32];
    const unsigned long long first = A.elFirst[e];
    const int grp = lane / 9, qq = lane - 9 * grp;
    // Jacobian at Gauss point gp = lane/4 from nodes 2s, 2s+1 (s = lane%4)
    {
        const int gp = lane >> 2, s = lane & 3;
        const DF G{kRt3Hi, kRt3Lo}, one{1.f, 0.f};
        const DF s1 = (gp & 1) ? G : df_neg(G), s2 = (gp & 2) ? G : df_neg(G), s3 = (gp & 4) ? G : df_neg(G);
        DF J[9], n[2][3];
#pragma unroll
        for (int q = 0; q < 9; ++q) J[q] = DF{0.f, 0.f};
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const int a = 2 * s + k;
            const float2 *xp = A.Xdf + 24 * (size_t)e + 3 * a;
            const float2 x0 = xp[0], x1 = xp[1], x2 = xp[2];
            const DF X[3] = {DF{x0.x, x0.y}, DF{x1.x, x1.y}, DF{x2.x, x2.y}};
            const bool sp = (a == 1 || a == 2 || a == 5 || a == 6), tp = (a == 2 || a == 3 || a == 6 || a == 7),
                       up = (a >= 4);
            const DF p1 = df_add(one, sp ? s1 : df_neg(s1));  // 1 + sa s1
            const DF p2 = df_add(one, tp ? s2 : df_neg(s2));
            const DF p3 = df_add(one, up ? s3 : df_neg(s3));
            n[k][0] = df_scale2(df_mul(p2, p3), sp ? 0.125f : -0.125f);
            n[k][1] = df_scale2(df_mul(p1, p3), tp ? 0.125f : -0.125f);
            n[k][2] = df_scale2(df_mul(p1, p2), up ? 0.125f : -0.125f);
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j) J[3 * i + j] = df_add(J[3 * i + j], df_mul(X[i], n[k][j]));
        }
#pragma unroll
        for (int q = 0; q < 9; ++q) {
#pragma unroll
            for (int m = 1; m <= 2; m <<= 1) {
                const DF o{__shfl_xor_sync(0xffffffffu, J[q].hi, m), __shfl_xor_sync(0xffffffffu, J[q].lo, m)};
                J[q] = df_add(J[q], o);
            }
        }
        const DF a11 = df_sub(df_mul(J[4], J[8]), df_mul(J[5], J[7]));
        const DF a12 = df_sub(df_mul(J[5], J[6]), df_mul(J[3], J[8]));
        const DF a13 = df_sub(df_mul(J[3], J[7]), df_mul(J[4], J[6]));
        const DF dt = df_add(df_add(df_mul(J[0], a11), df_mul(J[1], a12)), df_mul(J[2], a13));
        const DF di = df_rcp(dt);
        DF I[3][3];
        I[0][0] = df_mul(di, a11);
        I[1][0] = df_mul(di, a12);
        I[2][0] = df_mul(di, a13);
        I[0][1] = df_mul(di, df_sub(df_mul(J[2], J[7]), df_mul(J[1], J[8])));
        I[1][1] = df_mul(di, df_sub(df_mul(J[0], J[8]), df_mul(J[2], J[6])));
        I[2][1] = df_mul(di, df_sub(df_mul(J[1], J[6]), df_mul(J[0], J[7])));
        I[0][2] = df_mul(di, df_sub(df_mul(J[1], J[5]), df_mul(J[2], J[4])));
        I[1][2] = df_mul(di, df_sub(df_mul(J[2], J[3]), df_mul(J[0], J[5])));
        I[2][2] = df_mul(di, df_sub(df_mul(J[0], J[4]), df_mul(J[1], J[3])));
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            DF g[3], h[3];
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                g[j] = df_add(df_add(df_mul(n[k][0], I[0][j]), df_mul(n[k][1], I[1][j])), df_mul(n[k][2], I[2][j]));
                h[j] = df_mul(dt, g[j]);  // unit Gauss weights
            }
            const int a = 2 * s + k;
            sG[w].gh[gp][a] = make_float4(g[0].hi, g[1].hi, g[2].hi, 0.f);
            sG[w].gl[gp][a] = make_float4(g[0].lo, g[1].lo, g[2].lo, 0.f);
            sG[w].hh[gp][a] = make_float4(h[0].hi, h[1].hi, h[2].hi, 0.f);
            sG[w].hl[gp][a] = make_float4(h[0].lo, h[1].lo, h[2].lo, 0.f);
        }
    }
    __syncwarp();
    const int a0 = lane >> 3, a1 = a0 + 4, b = lane & 7;
    DF M0[9], M1[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) M0[q] = M1[q] = DF{0.f, 0.f};
#pragma unroll
    for (int gp = 0; gp < 8; ++gp) {
        const float4 hh = sG[w].hh[gp][b], hl = sG[w].hl[gp][b];
        const float4 ah = sG[w].gh[gp][a0], al = sG[w].gl[gp][a0], ch = sG[w].gh[gp][a1], cl = sG[w].gl[gp][a1];
        const float gah[3] = {ah.x, ah.y, ah.z}, gal[3] = {al.x, al.y, al.z};
        const float gch[3] = {ch.x, ch.y, ch.z}, gcl[3] = {cl.x, cl.y, cl.z};
        const float hbh[3] = {hh.x, hh.y, hh.z}, hbl[3] = {hl.x, hl.y, hl.z};
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                df_acc(M0[3 * i + j], gah[i], gal[i], hbh[j], hbl[j]);
                df_acc(M1[3 * i + j], gch[i], gcl[i], hbh[j], hbl[j]);
            }
    }
    DF c[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) {
        const float2 v = A.Cdf[9 * (size_t)e + q];
        c[q] = DF{v.x, v.y};
        M0[q] = df_norm(M0[q]);
        M1[q] = df_norm(M1[q]);
    }
    double K0[9], K1[9];
    {
        DF k0[9], k1[9];
        df_ortho(c, M0, k0);
        df_ortho(c, M1, k1);
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            K0[q] = df_to_double(k0[q]);
            K1[q] = df_to_double(k1[q]);
        }
    }
    if (ROT) {
        double Or[3][3];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) Or[i][j] = A.orient[9 * (size_t)e + 3 * j + i];
        rotate_block<double>(Or, K0);
        rotate_block<double>(Or, K1);
    }
    if (A.K) {
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            sK[w][9 * lane + q] = K0[q];
            sK[w][9 * (lane + 32) + q] = K1[q];
        }
        __syncwarp();
#pragma unroll
        for (int st = 0; st < kRmwSteps; ++st) {
            const int j = 3 * st + grp;
            if (grp < 3 && j < 64) {
                double *dst = A.K + 9 * (size_t)sBlk[w][j] + qq;
                const double v = sK[w][9 * j + qq];
                *dst = ((first >> j) & 1ull) ? v : *dst + v;
            }
        }
    }
    if (A.keOut) {
        double *ke = A.keOut + 576 * (size_t)e;
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                ke[(size_t)(8 * j + b) * 24 + (8 * i + a0)] = K0[3 * i + j];
                ke[(size_t)(8 * j + b) * 24 + (8 * i + a1)] = K1[3 * i + j];
            }
    }
}

// Node coordinates of every brick element in its section frame (orient X, FP64) and its C, both
// split into double-float for hex8_df_kernel.
__global__ void k_elem_df(int E, const double *__restrict__ nodes, const int *__restrict__ elist,
                          const double *__restrict__ orient, const double *__restrict__ elC, float2 *__restrict__ Xdf,
                          float2 *__restrict__ Cdf) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    double Or[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) Or[i][j] = orient ? orient[9 * (size_t)e + 3 * j + i] : (i == j ? 1.0 : 0.0);
    for (int a = 0; a < 8; ++a) {
        const int nd = elist[8 * (size_t)e + a];
        const double *x = nodes + 3 * (size_t)(nd - 1);
        for (int i = 0; i < 3; ++i) {
            const double y = Or[i][0] * x[0] + Or[i][1] * x[1] + Or[i][2] * x[2];
            const DF d = df_from_double(y);
            Xdf[24 * (size_t)e + 3 * a + i] = make_float2(d.hi, d.lo);
        }
    }
    for (int q = 0; q < 9; ++q) {
        const DF d = df_from_double(elC[9 * (size_t)e + q]);
        Cdf[9 * (size_t)e + q] = make_float2(d.hi, d.lo);
    }
}

// Orthotropic C of every brick element by the reference's LU (r_getMaterialStiffness): the
// normal 3x3 block and the shear diagonal of C = S^-1.
__global__ void k_elem_c(int E, const double *__restrict__ elMat, double *__restrict__ elC) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    double C[6][6];
    material_c<double>(elMat + 9 * (size_t)e, C);
    double *o = elC + 9 * (size_t)e;
    o[0] = C[0][0];
    o[1] = C[0][1];
    o[2] = C[0][2];
    o[3] = C[1][1];
    o[4] = C[1][2];
    o[5] = C[2][2];
    o[6] = C[3][3];
    o[7] = C[4][4];
    o[8] = C[5][5];
}

// Imaginary part of the complex-step material stiffness of each listed element:
// eProps(c) + coef (d + i h) for the elastic-modulus design variable dvar (the real parts of all
// design-variable terms are already in elMat), then C = S^-1 in complex arithmetic.
__global__ void k_hex_cim(int count, const int *__restrict__ els, const double *__restrict__ elMat,
                          const int *__restrict__ e2dR, const int *__restrict__ e2d, const double *__restrict__ e2c,
                          const int *__restrict__ dcat, const int *__restrict__ dcomp, int dvar, double h,
                          double *__restrict__ Cim) {
    const int item = blockIdx.x * blockDim.x + threadIdx.x;
    if (item >= count) return;
    const int e = els[item];
    cplx ep[9];
    for (int k = 0; k < 9; ++k) ep[k] = cplx(elMat[9 * (size_t)e + k]);
    for (int q = e2dR[e]; q < e2dR[e + 1]; ++q) {
        const int d = e2d[q];
        if (d == dvar && dcat[d - 1] == ASTRO_DCAT_ELASTIC_MODULUS) ep[dcomp[d - 1] - 1] += cplx(0.0, e2c[q] * h);
    }
    cplx C[6][6];
    material_c<cplx>(ep, C);
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) Cim[36 * (size_t)item + 6 * i + j] = C[i][j].im;
}

}  // namespace

template <class T, bool ROT> static void hex8_fast_launch(astro_ctx *ctx, const Hex8FastArgs<T> &A0) {
    const AstroPrep &P = ctx->P;
    constexpr int FW = FastCfg<T>::FW;
    Hex8FastArgs<T> A = A0;
    for (int col = 0; col < P.ncolors; ++col) {
        const int cnt = P.colorPtr[col + 1] - P.colorPtr[col];
        if (!cnt) continue;
        A.colorEls = dptr<int>(ctx->d_colorEls) + P.colorPtr[col];
        A.count = cnt;
        hex8_fast_kernel<T, ROT><<<(cnt + FW - 1) / FW, 32 * FW, 0, ctx->stream>>>(A);
    }
}

// Zero-state stiffness of every element, colour by colour, into K (block-CSR, written without a
// prior zeroing) and/or the element matrices d_ke.
template <class T> static int hex8_fast_run(astro_ctx *ctx, T *K, double *d_ke) {
    Hex8FastArgs<T> A;
    A.colorEls = nullptr;
    A.count = 0;
    A.elBlk = dptr<int>(ctx->d_elBlk);
    A.elFirst = dptr<unsigned long long>(ctx->d_elFirst);
    A.Xdf = dptr<float2>(ctx->d_elXdf);
    A.Cdf = dptr<float2>(ctx->d_elCdf);
    A.orient = dptr<double>(ctx->d_secOrient);
    A.K = K;
    A.keOut = d_ke;
    if (ctx->orientIdentity)
        hex8_fast_launch<T, false>(ctx, A);
    else
        hex8_fast_launch<T, true>(ctx, A);
    return cuda_check(ctx, cudaGetLastError(), "brick8 zero-state kernel launch");
}

// precision 64: general FP64 kernel (state, orientation); 32: FP32 kernel at zero state.
// store bit 1: FP32 BSR, bit 2: FP64 BSR (the FP32 kernel adds its values into both when asked).
static int hex8_run(astro_ctx *ctx, int precision, int store, const double *d_disp, double *d_loadInt, double *d_ke,
                    double *d_ru) {
    const AstroPrep &P = ctx->P;
    for (int col = 0; col < P.ncolors; ++col) {
        const int cnt = P.colorPtr[col + 1] - P.colorPtr[col];
        if (!cnt) continue;
        dim3 grid((cnt + kWarpsPerBlock - 1) / kWarpsPerBlock), block(32 * kWarpsPerBlock);
        if (precision == 64) {
            Hex8Args<double> A;
            A.nodes = dptr<double>(ctx->d_nodes);
            A.elist = dptr<int>(ctx->d_elist);
            A.rank = dptr<int>(ctx->d_rank);
            A.colorEls = dptr<int>(ctx->d_colorEls) + P.colorPtr[col];
            A.count = cnt;
            A.elBlk = dptr<int>(ctx->d_elBlk);
            A.elMat = dptr<double>(ctx->d_elMat);
            A.orient = ctx->orientIdentity ? nullptr : dptr<double>(ctx->d_secOrient);
            A.disp = d_disp;
            A.Kbsr = (store & 2) ? dptr<double>(ctx->d_K64) : nullptr;
            A.Kbsr64 = nullptr;
            A.loadInt = d_loadInt;
            A.keOut = d_ke;
            A.ruOut = d_ru;
            A.gpc = kRt3;
            A.Cover = nullptr;
            hex8_kernel<double, true><<<grid, block, 0, ctx->stream>>>(A);
        } else {
            Hex8Args<float> A;
            A.nodes = dptr<double>(ctx->d_nodes);
            A.elist = dptr<int>(ctx->d_elist);
            A.rank = dptr<int>(ctx->d_rank);
            A.colorEls = dptr<int>(ctx->d_colorEls) + P.colorPtr[col];
            A.count = cnt;
            A.elBlk = dptr<int>(ctx->d_elBlk);
            A.elMat = dptr<double>(ctx->d_elMat);
            A.orient = nullptr;
            A.disp = nullptr;
            A.Kbsr = (store & 1) ? dptr<float>(ctx->d_K32) : nullptr;
            A.Kbsr64 = (store & 2) ? dptr<double>(ctx->d_K64) : nullptr;
            A.loadInt = nullptr;
            A.keOut = d_ke;
            A.ruOut = nullptr;
            A.gpc = kRt3;
            A.Cover = nullptr;
            hex8_kernel<float, false><<<grid, block, 0, ctx->stream>>>(A);
        }
    }
    return cuda_check(ctx, cudaGetLastError(), "hex8 kernel launch");
}

// FP64 zero-state stiffness (double-float kernel), colour by colour.
static int hex8_df_run(astro_ctx *ctx, double *K, double *d_ke) {
    const AstroPrep &P = ctx->P;
    Hex8DfArgs A;
    A.elBlk = dptr<int>(ctx->d_elBlk);
    A.elFirst = dptr<unsigned long long>(ctx->d_elFirst);
    A.Xdf = dptr<float2>(ctx->d_elXdf);
    A.Cdf = dptr<float2>(ctx->d_elCdf);
    A.orient = dptr<double>(ctx->d_secOrient);
    A.K = K;
    A.keOut = d_ke;
    for (int col = 0; col < P.ncolors; ++col) {
        const int cnt = P.colorPtr[col + 1] - P.colorPtr[col];
        if (!cnt) continue;
        A.colorEls = dptr<int>(ctx->d_colorEls) + P.colorPtr[col];
        A.count = cnt;
        const unsigned grid = (cnt + kDfW - 1) / kDfW;
        if (ctx->orientIdentity)
            hex8_df_kernel<false><<<grid, 32 * kDfW, 0, ctx->stream>>>(A);
        else
            hex8_df_kernel<true><<<grid, 32 * kDfW, 0, ctx->stream>>>(A);
    }
    return cuda_check(ctx, cudaGetLastError(), "brick8 FP64 zero-state kernel launch");
}

int hex8_prepare(astro_ctx *ctx) {
    const int E = ctx->P.E;
    int rc;
    if ((rc = dev_alloc(ctx, ctx->d_elC, sizeof(double) * 9 * (size_t)E))) return rc;
    k_elem_c<<<(E + 127) / 128, 128, 0, ctx->stream>>>(E, dptr<double>(ctx->d_elMat), dptr<double>(ctx->d_elC));
    if ((rc = dev_alloc(ctx, ctx->d_elXdf, sizeof(float2) * 24 * (size_t)E))) return rc;
    if ((rc = dev_alloc(ctx, ctx->d_elCdf, sizeof(float2) * 9 * (size_t)E))) return rc;
    k_elem_df<<<(E + 127) / 128, 128, 0, ctx->stream>>>(
        E, dptr<double>(ctx->d_nodes), dptr<int>(ctx->d_elist), ctx->orientIdentity ? nullptr : dptr<double>(ctx->d_secOrient),
        dptr<double>(ctx->d_elC), dptr<float2>(ctx->d_elXdf), dptr<float2>(ctx->d_elCdf));
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    return cuda_check(ctx, e, "brick8 material stiffness");
}

int launch_hex8_assemble(astro_ctx *ctx, int precision, int store) {
    if (precision == 32) return hex8_fast_run<float>(ctx, (store & 1) ? dptr<float>(ctx->d_K32) : nullptr, nullptr);
    return hex8_df_run(ctx, (store & 2) ? dptr<double>(ctx->d_K64) : nullptr, nullptr);
}

// getElasticSolnLoad for bricks.  From the undeformed state (no displacement) the residual is
// zero and the tangent is the small-strain stiffness, which the zero-state kernel writes into the
// block-CSR matrix without a prior zeroing; any other state takes the general kernel (Green-
// Lagrange strain, stress stiffness, residual), which adds into a zeroed matrix.
int hex8_soln_load(astro_ctx *ctx, int buildMat, const double *d_disp, double *d_loadInt) {
    if (!d_disp) return buildMat ? hex8_df_run(ctx, dptr<double>(ctx->d_K64), nullptr) : ASTRO_OK;
    return hex8_run(ctx, 64, buildMat ? 2 : 0, d_disp, d_loadInt, nullptr, nullptr);
}

int launch_hex8_element_mats(astro_ctx *ctx, int precision, double *d_ke) {
    if (precision == 32) return hex8_fast_run<float>(ctx, nullptr, d_ke);
    return hex8_df_run(ctx, nullptr, d_ke);
}

int hex8_element_mats_state(astro_ctx *ctx, const double *d_disp, double *d_ke, double *d_ru) {
    if (!d_disp && !d_ru) return hex8_df_run(ctx, nullptr, d_ke);
    return hex8_run(ctx, 64, 0, d_disp, nullptr, d_ke, d_ru);
}

int hex8_drdd(astro_ctx *ctx, int dvar, double h, const double *d_disp, double *d_acc) {
    std::vector<int> list, ptr;
    dvar_elements_by_colour(ctx, dvar, list, ptr);
    const int cnt = (int)list.size();
    if (!cnt) return ASTRO_OK;
    DevBuf dl, dC, dR, dE, dEC, dCat, dComp;
    struct Free {
        DevBuf *b[7];
        ~Free() {
            for (auto *x : b) dev_free(*x);
        }
    } fr{{&dl, &dC, &dR, &dE, &dEC, &dCat, &dComp}};
    int rc;
    if ((rc = upload(ctx, dl, list.data(), sizeof(int) * cnt))) return rc;
    if ((rc = dev_alloc(ctx, dC, sizeof(double) * 36 * (size_t)cnt))) return rc;
    if ((rc = upload(ctx, dR, ctx->e2dRange.data(), sizeof(int) * ctx->e2dRange.size()))) return rc;
    if ((rc = upload(ctx, dE, ctx->e2d.data(), sizeof(int) * ctx->e2d.size()))) return rc;
    if ((rc = upload(ctx, dEC, ctx->e2c.data(), sizeof(double) * ctx->e2c.size()))) return rc;
    if ((rc = upload(ctx, dCat, ctx->dCat.data(), sizeof(int) * ctx->dCat.size()))) return rc;
    if ((rc = upload(ctx, dComp, ctx->dComp.data(), sizeof(int) * ctx->dComp.size()))) return rc;
    k_hex_cim<<<(cnt + 127) / 128, 128, 0, ctx->stream>>>(cnt, dptr<int>(dl), dptr<double>(ctx->d_elMat), dptr<int>(dR),
                                                          dptr<int>(dE), dptr<double>(dEC), dptr<int>(dCat),
                                                          dptr<int>(dComp), dvar, h, dptr<double>(dC));
    const AstroPrep &P = ctx->P;
    for (int col = 0; col < P.ncolors; ++col) {
        const int c = ptr[col + 1] - ptr[col];
        if (!c) continue;
        Hex8Args<double> A;
        A.nodes = dptr<double>(ctx->d_nodes);
        A.elist = dptr<int>(ctx->d_elist);
        A.rank = dptr<int>(ctx->d_rank);
        A.colorEls = dptr<int>(dl) + ptr[col];
        A.count = c;
        A.elBlk = dptr<int>(ctx->d_elBlk);
        A.elMat = dptr<double>(ctx->d_elMat);
        A.orient = ctx->orientIdentity ? nullptr : dptr<double>(ctx->d_secOrient);
        A.disp = d_disp;
        A.Kbsr = nullptr;
        A.Kbsr64 = nullptr;
        A.loadInt = d_acc;
        A.keOut = nullptr;
        A.ruOut = nullptr;
        A.gpc = kRt3c;
        A.Cover = dptr<double>(dC) + 36 * (size_t)ptr[col];
        hex8_kernel<double, true><<<(c + kWarpsPerBlock - 1) / kWarpsPerBlock, 32 * kWarpsPerBlock, 0, ctx->stream>>>(A);
    }
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    return cuda_check(ctx, e, "brick8 complex-step kernels");
}
