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
// Kernels, one warp per element: hex8_fast_kernel (FP32, zero state), hex8_df_kernel (FP64 zero
// state in double-float), hex8_gen_kernel (any state and orientation, double-float; also the
// complex step with the imaginary part of C).  Elements are processed colour by colour so a
// colour's blocks land in disjoint block rows: plain read-add-write, no atomics, bit-reproducible.
#include "astro_internal.h"
#include "dfloat.cuh"
#include "shell_math.cuh"

namespace {

constexpr double kRt3 = 0.57735026918962576451;  // r_1rt3 = 1/sqrt(3) in double
constexpr double kRt3c = LIT(0.577350269189626);  // c_1rt3: a single-precision literal

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
    static constexpr bool PREFETCH = true;
};
// The zero-state kernel's warps per CTA (FW) is a template parameter: 1, 2 (the default: small
// CTAs give shorter colour tails) or 4, picked per context by astro_autotune; the launch bounds ask
// the register allocator for 28 warps per SM in every case.
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
template <class T, bool ROT, int FW>
__global__ void __launch_bounds__(32 * FW, 32 / FW) hex8_fast_kernel(Hex8FastArgs<T> A) {
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
    // colour launches chain by programmatic dependent launch: the next colour's CTAs may be
    // scheduled now and compute their element blocks while this colour finishes; the blocks a
    // colour reads and adds into are the previous colour's output, so it waits for that grid
    // before its first read of K (a no-op without a programmatic edge)
    asm volatile("griddepcontrol.launch_dependents;");
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
    asm volatile("griddepcontrol.wait;" ::: "memory");
    T ov[PREFETCH ? kRmwSteps : 1];
    if (PREFETCH) {
#pragma unroll
        for (int st = 0; st < kRmwSteps; ++st) {
            const int j = 3 * st + grp;
            ov[st] = T(0);
            if (A.K && grp < 3 && j < 64 && !((first >> j) & 1ull)) ov[st] = A.K[9 * (size_t)sBlk[w][j] + qq];
        }
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
template <bool ROT> __global__ void __launch_bounds__(32 * kDfW, 6) hex8_df_kernel(Hex8DfArgs A) {
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
    asm volatile("griddepcontrol.launch_dependents;");  // chained colours, as in hex8_fast_kernel
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
    asm volatile("griddepcontrol.wait;" ::: "memory");  // the previous colour's blocks are complete
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

// ---------------------------------------------------------------------------------------------
// General-state brick8 element (Green-Lagrange strain, stress stiffness, residual, any section
// orientation) in double-float: the quantities of hex8_kernel<double, true> reorganised for the
// FP32 pipe.  With G = Or + ux^T at a Gauss point (Or the section orientation, ux the gradient of
// the global displacement along the local axes) and Bloc(g) the 6x3 small-strain operator of the
// shape gradient g, the nonlinear strain-displacement block of node a is P_a = Bloc(g_a) G (6x3),
// and with Q_b = w detJ C P_b, S the stress tensor and t_b = w detJ S g_b:
//   K_ab = sum_gp ( P_a^T Q_b + (g_a . t_b) I3 ),   Ru_a = sum_gp w detJ P_a^T stress,
// plus, for a Newmark state, the consistent mass c1 c2 rho w detJ N_a N_b I3 in K and the
// inertia rho w detJ N_a (sum_b N_b acc_b) in Ru (the fourth components of g and t carry N_a and
// c1 c2 rho w detJ N_b, so the pair loop adds the mass with the stress term).
// Phase 1, lane (gp, s) = (lane / 4, lane % 4) handles nodes 2s and 2s+1 at point gp: the
// Jacobian and displacement gradient are reduced over the four lanes of the point, then the lane
// writes P, Q, g and t of its two nodes to shared memory (double-float) and keeps their residual.
// Phase 2 (with a matrix), the 36 node-pair tiles a <= b times the 8 Gauss points are 288 units,
// nine consecutive ones per lane in tile-major order, so every lane finishes one tile it shares
// with a neighbour and starts the next: each tile is the sum of at most two partials (fixed order,
// deterministic), and K_ba = K_ab^T fills the lower half.  Phase 3 writes the 64 blocks through
// shared memory into the block-CSR matrix, three whole blocks per warp instruction; the first
// element (in colour order) to touch a block writes it instead of adding.
struct Hex8GenArgs {
    const int *colorEls;
    int count;
    const int *elBlk;
    const unsigned long long *elFirst;
    const int *elist, *rank;
    const float2 *Xdf;     // (E,8,3) node coordinates in the section frame, double-float
    const float2 *Cdf;     // (E,9) orthotropic C, double-float (indexed by element)
    const float2 *CdfItem; // (count,9) C per listed element (indexed by list position) or null
    const double *orient;  // (E,9) column-major section orientation (ROT)
    const double *disp;    // internal-layout displacement (3 per node, rank-major) or null
    // Newmark inertia (r_getElRum solid branch, Working/AStrO_r_elementEqns.f90:2628-2653): the
    // previous displacement, velocity and acceleration, density per element; dyn = 0 without it
    const double *pdisp, *pvel, *pacc, *rho;
    int dyn;
    double beta, delT;
    double *K;             // BSR values or null
    double *loadInt;       // internal-layout load, -= Ru (or null)
    double *keOut;         // element matrices (E,24,24) column-major, element DOF order, or null
    double *ruOut;         // (E,24) or null
    float gpcHi, gpcLo;    // Gauss point coordinate (1/sqrt(3) of the real or the complex path)
};

constexpr int kGenW = 2;  // warps per CTA

struct GenSmem {
    union {
        struct {
            float Ph[64][18], Pl[64][18], Qh[64][18], Ql[64][18];  // item gp*8 + a: 6x3 row-major
            float4 gh[64], gl[64], th[64], tl[64];
        } u;
        struct {
            float part[36][2][20];  // tile partials: 9 entries + geometric term, (hi, lo) pairs
            double K[64 * 9];       // element blocks, block j = 8a + b at 9j (row-major 3x3)
        } o;
    };
    int blk[64];
};

__constant__ unsigned char c_tileA[36], c_tileB[36];

__device__ __forceinline__ DF df_shfl_xor(DF v, int m) {
    return DF{__shfl_xor_sync(0xffffffffu, v.hi, m), __shfl_xor_sync(0xffffffffu, v.lo, m)};
}
__device__ __forceinline__ DF df_fma(DF a, DF b, DF c) { return df_add(df_mul(a, b), c); }

template <bool ROT, bool BUILD>
__global__ void __launch_bounds__(32 * kGenW) hex8_gen_kernel(Hex8GenArgs A) {
    __shared__ GenSmem sm[kGenW];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int item = blockIdx.x * kGenW + w;
    if (item >= A.count) return;
    GenSmem &S = sm[w];
    const int e = A.colorEls[item];
    asm volatile("griddepcontrol.launch_dependents;");  // chained colours, as in hex8_fast_kernel
    if (BUILD) {
        S.blk[lane] = A.elBlk[64 * (size_t)e + lane];
        S.blk[lane + 32] = A.elBlk[64 * (size_t)e + lane + 32];
    }
    const DF one{1.f, 0.f}, zero{0.f, 0.f};
    DF c[9];  // C11 C12 C13 C22 C23 C33 C44 C55 C66
    {
        const float2 *cp = A.CdfItem ? A.CdfItem + 9 * (size_t)item : A.Cdf + 9 * (size_t)e;
#pragma unroll
        for (int q = 0; q < 9; ++q) c[q] = DF{cp[q].x, cp[q].y};
    }
    DF Or[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
            Or[i][j] = ROT ? df_from_double(A.orient[9 * (size_t)e + 3 * j + i]) : ((i == j) ? one : zero);
    // ---- phase 1: lane (gp, s), nodes 2s and 2s+1 ---------------------------------------------
    const int gp = lane >> 2, s = lane & 3;
    DF ru[2][3];
    {
        const DF G{A.gpcHi, A.gpcLo};
        const DF s1 = (gp & 1) ? G : df_neg(G), s2 = (gp & 2) ? G : df_neg(G), s3 = (gp & 4) ? G : df_neg(G);
        DF J[9], n[2][3], U[2][3], Nv[2], Ac[2][3];
#pragma unroll
        for (int q = 0; q < 9; ++q) J[q] = zero;
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const int a = 2 * s + k;
            const float2 *xp = A.Xdf + 24 * (size_t)e + 3 * a;
            const float2 x0 = xp[0], x1 = xp[1], x2 = xp[2];
            const DF X[3] = {DF{x0.x, x0.y}, DF{x1.x, x1.y}, DF{x2.x, x2.y}};
            const bool sp = (a == 1 || a == 2 || a == 5 || a == 6), tp = (a == 2 || a == 3 || a == 6 || a == 7),
                       up = (a >= 4);
            const DF p1 = df_add(one, sp ? s1 : df_neg(s1));
            const DF p2 = df_add(one, tp ? s2 : df_neg(s2));
            const DF p3 = df_add(one, up ? s3 : df_neg(s3));
            n[k][0] = df_scale2(df_mul(p2, p3), sp ? 0.125f : -0.125f);
            n[k][1] = df_scale2(df_mul(p1, p3), tp ? 0.125f : -0.125f);
            n[k][2] = df_scale2(df_mul(p1, p2), up ? 0.125f : -0.125f);
            Nv[k] = df_scale2(df_mul(df_mul(p1, p2), p3), 0.125f);
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j) J[3 * i + j] = df_fma(X[i], n[k][j], J[3 * i + j]);
            const int nd = A.elist[8 * (size_t)e + a];
            const int r = A.rank[nd - 1] - 1;
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                const size_t ix = 3 * (size_t)r + i;
                const double u = A.disp ? A.disp[ix] : 0.0;
                U[k][i] = df_from_double(u);
                double ac = 0.0;
                if (A.dyn) {
                    // accNext of r_getElRu (:2684-2696) in FP64
                    const double c1 = 0.5 / A.beta, c2 = 2.0 / (A.delT * A.delT);
                    const double pd = A.pdisp ? A.pdisp[ix] : 0.0, pv = A.pvel ? A.pvel[ix] : 0.0,
                                 pa = A.pacc ? A.pacc[ix] : 0.0;
                    ac = c1 * (c2 * (u - pd - A.delT * pv) - (1.0 - 2.0 * A.beta) * pa);
                }
                Ac[k][i] = df_from_double(ac);
            }
        }
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            J[q] = df_add(J[q], df_shfl_xor(J[q], 1));
            J[q] = df_add(J[q], df_shfl_xor(J[q], 2));
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
        DF g[2][3];
#pragma unroll
        for (int k = 0; k < 2; ++k)
#pragma unroll
            for (int j = 0; j < 3; ++j)
                g[k][j] = df_add(df_add(df_mul(n[k][0], I[0][j]), df_mul(n[k][1], I[1][j])), df_mul(n[k][2], I[2][j]));
        // displacement gradient ux[i][j] = sum_a U_a[i] g_a[j] (global components, local axes)
        DF ux[3][3];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                DF v = df_add(df_mul(U[0][i], g[0][j]), df_mul(U[1][i], g[1][j]));
                v = df_add(v, df_shfl_xor(v, 1));
                ux[i][j] = df_add(v, df_shfl_xor(v, 2));
            }
        // Green-Lagrange strain in the section frame, stress, and G = Or + ux^T
        DF uxL[3][3];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j)
                uxL[i][j] = ROT ? df_add(df_add(df_mul(Or[i][0], ux[0][j]), df_mul(Or[i][1], ux[1][j])),
                                         df_mul(Or[i][2], ux[2][j]))
                                : ux[i][j];
        DF st[6];
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            DF q2 = df_add(df_add(df_mul(ux[0][j], ux[0][j]), df_mul(ux[1][j], ux[1][j])), df_mul(ux[2][j], ux[2][j]));
            st[j] = df_add(uxL[j][j], df_scale2(q2, 0.5f));
        }
        {
            const int pi[3] = {0, 0, 2}, pj[3] = {1, 2, 1};  // shear pairs (e12, e13, e23)
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                const int i = pi[q], j = pj[q];
                DF v = df_add(uxL[i][j], uxL[j][i]);
                v = df_add(v, df_add(df_add(df_mul(ux[0][i], ux[0][j]), df_mul(ux[1][i], ux[1][j])),
                                     df_mul(ux[2][i], ux[2][j])));
                st[3 + q] = v;
            }
        }
        // w detJ (unit Gauss weights) folded into C and the stress
        DF cw[9], sw[6];
#pragma unroll
        for (int q = 0; q < 9; ++q) cw[q] = df_mul(dt, c[q]);
        sw[0] = df_add(df_add(df_mul(cw[0], st[0]), df_mul(cw[1], st[1])), df_mul(cw[2], st[2]));
        sw[1] = df_add(df_add(df_mul(cw[1], st[0]), df_mul(cw[3], st[1])), df_mul(cw[4], st[2]));
        sw[2] = df_add(df_add(df_mul(cw[2], st[0]), df_mul(cw[4], st[1])), df_mul(cw[5], st[2]));
        sw[3] = df_mul(cw[6], st[3]);
        sw[4] = df_mul(cw[7], st[4]);
        sw[5] = df_mul(cw[8], st[5]);
        DF Gm[3][3];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) Gm[i][j] = df_add(Or[i][j], ux[j][i]);
        // Newmark inertia: acceleration at the point, rho w detJ, and c1 c2 rho w detJ
        DF ag[3] = {zero, zero, zero}, rw = zero, mw = zero;
        if (A.dyn) {
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                DF v = df_add(df_mul(Nv[0], Ac[0][i]), df_mul(Nv[1], Ac[1][i]));
                v = df_add(v, df_shfl_xor(v, 1));
                ag[i] = df_add(v, df_shfl_xor(v, 2));
            }
            const double c1 = 0.5 / A.beta, c2 = 2.0 / (A.delT * A.delT);
            rw = df_mul(df_from_double(A.rho[e]), dt);
            mw = df_mul(df_from_double(c1 * c2), rw);
        }
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const int a = 2 * s + k;
            const DF g0 = g[k][0], g1 = g[k][1], g2 = g[k][2];
            DF P[6][3];
#pragma unroll
            for (int v = 0; v < 3; ++v) {
                P[0][v] = df_mul(g0, Gm[0][v]);
                P[1][v] = df_mul(g1, Gm[1][v]);
                P[2][v] = df_mul(g2, Gm[2][v]);
                P[3][v] = df_add(df_mul(g1, Gm[0][v]), df_mul(g0, Gm[1][v]));
                P[4][v] = df_add(df_mul(g2, Gm[0][v]), df_mul(g0, Gm[2][v]));
                P[5][v] = df_add(df_mul(g2, Gm[1][v]), df_mul(g1, Gm[2][v]));
            }
            // residual of node a at this point: P^T (w detJ stress), plus the inertia
#pragma unroll
            for (int v = 0; v < 3; ++v) {
                DF r = df_mul(P[0][v], sw[0]);
#pragma unroll
                for (int q = 1; q < 6; ++q) r = df_fma(P[q][v], sw[q], r);
                if (A.dyn) r = df_fma(df_mul(rw, Nv[k]), ag[v], r);
                ru[k][v] = r;
            }
            if (BUILD) {
                const int it = gp * 8 + a;
#pragma unroll
                for (int q = 0; q < 6; ++q)
#pragma unroll
                    for (int v = 0; v < 3; ++v) {
                        S.u.Ph[it][3 * q + v] = P[q][v].hi;
                        S.u.Pl[it][3 * q + v] = P[q][v].lo;
                    }
#pragma unroll
                for (int v = 0; v < 3; ++v) {
                    DF Q[6];
                    Q[0] = df_add(df_add(df_mul(cw[0], P[0][v]), df_mul(cw[1], P[1][v])), df_mul(cw[2], P[2][v]));
                    Q[1] = df_add(df_add(df_mul(cw[1], P[0][v]), df_mul(cw[3], P[1][v])), df_mul(cw[4], P[2][v]));
                    Q[2] = df_add(df_add(df_mul(cw[2], P[0][v]), df_mul(cw[4], P[1][v])), df_mul(cw[5], P[2][v]));
                    Q[3] = df_mul(cw[6], P[3][v]);
                    Q[4] = df_mul(cw[7], P[4][v]);
                    Q[5] = df_mul(cw[8], P[5][v]);
#pragma unroll
                    for (int q = 0; q < 6; ++q) {
                        S.u.Qh[it][3 * q + v] = Q[q].hi;
                        S.u.Ql[it][3 * q + v] = Q[q].lo;
                    }
                }
                // t = (w detJ S) g with S the symmetric stress tensor of the Voigt vector
                const DF t0 = df_add(df_add(df_mul(sw[0], g0), df_mul(sw[3], g1)), df_mul(sw[4], g2));
                const DF t1 = df_add(df_add(df_mul(sw[3], g0), df_mul(sw[1], g1)), df_mul(sw[5], g2));
                const DF t2 = df_add(df_add(df_mul(sw[4], g0), df_mul(sw[5], g1)), df_mul(sw[2], g2));
                const DF na = A.dyn ? Nv[k] : zero, mn = A.dyn ? df_mul(mw, Nv[k]) : zero;
                S.u.gh[it] = make_float4(g0.hi, g1.hi, g2.hi, na.hi);
                S.u.gl[it] = make_float4(g0.lo, g1.lo, g2.lo, na.lo);
                S.u.th[it] = make_float4(t0.hi, t1.hi, t2.hi, mn.hi);
                S.u.tl[it] = make_float4(t0.lo, t1.lo, t2.lo, mn.lo);
            }
        }
    }
    // residual: sum over the eight points (lanes with the same s), delivered by lanes 0..3
#pragma unroll
    for (int k = 0; k < 2; ++k)
#pragma unroll
        for (int v = 0; v < 3; ++v)
#pragma unroll
            for (int m = 4; m <= 16; m <<= 1) ru[k][v] = df_add(ru[k][v], df_shfl_xor(ru[k][v], m));
    // the previous colour's load entries and blocks are complete before the first update
    asm volatile("griddepcontrol.wait;" ::: "memory");
    if (lane < 4) {
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const int a = 2 * lane + k;
            if (A.loadInt) {
                const int r = A.rank[A.elist[8 * (size_t)e + a] - 1] - 1;
#pragma unroll
                for (int v = 0; v < 3; ++v) A.loadInt[3 * (size_t)r + v] -= df_to_double(ru[k][v]);
            }
            if (A.ruOut)
#pragma unroll
                for (int v = 0; v < 3; ++v) A.ruOut[24 * (size_t)e + 8 * v + a] = df_to_double(ru[k][v]);
        }
    }
    if (!BUILD) return;
    __syncwarp();
    // ---- phase 2: units 9 lane .. 9 lane + 8 of the 288 (tile, point) units ------------------------
    const int u0 = 9 * lane;
    const int tA = u0 >> 3;                 // first tile (shared with the previous lane unless u0 % 8 == 0)
    const int usw = 8 * (tA + 1) - u0;      // unit at which the second tile starts (1..8)
    DF acc[9], geo = zero, acc0[9], geo0 = zero;
#pragma unroll
    for (int q = 0; q < 9; ++q) acc[q] = acc0[q] = zero;
    // one unit per trip: unrolled, the nine units' double-float bodies overflow the instruction
    // cache (the kernel's leading stall was instruction fetch)
#pragma unroll 1
    for (int u = 0; u < 9; ++u) {
        if (u == usw) {
#pragma unroll
            for (int q = 0; q < 9; ++q) {
                acc0[q] = acc[q];
                acc[q] = zero;
            }
            geo0 = geo;
            geo = zero;
        }
        const int unit = u0 + u, t = unit >> 3, p = unit & 7;
        const int ia = 8 * p + c_tileA[t], ib = 8 * p + c_tileB[t];
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            float ph[3], pl[3], qh[3], ql[3];
#pragma unroll
            for (int v = 0; v < 3; ++v) {
                ph[v] = S.u.Ph[ia][3 * q + v];
                pl[v] = S.u.Pl[ia][3 * q + v];
                qh[v] = S.u.Qh[ib][3 * q + v];
                ql[v] = S.u.Ql[ib][3 * q + v];
            }
#pragma unroll
            for (int v = 0; v < 3; ++v)
#pragma unroll
                for (int x = 0; x < 3; ++x) df_acc(acc[3 * v + x], ph[v], pl[v], qh[x], ql[x]);
        }
        const float4 gh = S.u.gh[ia], gl = S.u.gl[ia], th = S.u.th[ib], tl = S.u.tl[ib];
        df_acc(geo, gh.x, gl.x, th.x, tl.x);
        df_acc(geo, gh.y, gl.y, th.y, tl.y);
        df_acc(geo, gh.z, gl.z, th.z, tl.z);
        df_acc(geo, gh.w, gl.w, th.w, tl.w);  // consistent mass (zero without inertia)
    }
    __syncwarp();
    // partials: the first tile to slot 0 when it starts on this lane (u0 % 8 == 0), else slot 1;
    // the second tile starts here, slot 0
    {
        float *d0 = S.o.part[tA][(u0 & 7) ? 1 : 0];
        float *d1 = S.o.part[tA + 1][0];
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            const DF x0 = df_norm(acc0[q]), x1 = df_norm(acc[q]);
            d0[2 * q] = x0.hi;
            d0[2 * q + 1] = x0.lo;
            d1[2 * q] = x1.hi;
            d1[2 * q + 1] = x1.lo;
        }
        const DF y0 = df_norm(geo0), y1 = df_norm(geo);
        d0[18] = y0.hi;
        d0[19] = y0.lo;
        d1[18] = y1.hi;
        d1[19] = y1.lo;
    }
    __syncwarp();
    // ---- phase 3: blocks (a0, b) and (a1, b), a0 = lane / 8, a1 = a0 + 4, b = lane % 8 -----------
    const int b = lane & 7;
#pragma unroll
    for (int half = 0; half < 2; ++half) {
        const int a = (lane >> 3) + 4 * half;
        const int lo = min(a, b), hi = max(a, b);
        const int t = lo * 8 - (lo * (lo - 1)) / 2 + (hi - lo);  // row-major upper-triangle index
        const bool two = (8 * t) / 9 != (8 * t + 7) / 9;        // the tile spans two lanes
        const float *p0 = S.o.part[t][0], *p1 = S.o.part[t][1];
        double Kb[9];
        const DF gs = two ? df_add(DF{p0[18], p0[19]}, DF{p1[18], p1[19]}) : DF{p0[18], p0[19]};
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            DF v = two ? df_add(DF{p0[2 * q], p0[2 * q + 1]}, DF{p1[2 * q], p1[2 * q + 1]}) : DF{p0[2 * q], p0[2 * q + 1]};
            if (q == 0 || q == 4 || q == 8) v = df_add(v, gs);
            Kb[q] = df_to_double(v);
        }
        double *dst = S.o.K + 9 * (8 * a + b);
        // tile (lo, hi) holds K_lo,hi; block (a, b) with a > b is its transpose
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) dst[3 * i + j] = (a <= b) ? Kb[3 * i + j] : Kb[3 * j + i];
    }
    __syncwarp();
    if (A.K) {
        const unsigned long long first = A.elFirst[e];
        const int grp = lane / 9, qq = lane - 9 * grp;
#pragma unroll
        for (int stp = 0; stp < kRmwSteps; ++stp) {
            const int j = 3 * stp + grp;
            if (grp < 3 && j < 64) {
                double *dst = A.K + 9 * (size_t)S.blk[j] + qq;
                const double v = S.o.K[9 * j + qq];
                *dst = ((first >> j) & 1ull) ? v : *dst + v;
            }
        }
    }
    if (A.keOut) {
        double *ke = A.keOut + 576 * (size_t)e;
#pragma unroll
        for (int half = 0; half < 2; ++half) {
            const int a = (lane >> 3) + 4 * half;
            const double *src = S.o.K + 9 * (8 * a + b);
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) ke[(size_t)(8 * j + b) * 24 + (8 * i + a)] = src[3 * i + j];
        }
    }
}

// Node coordinates of every brick element in its section frame (orient X, relative to the
// element's first node, FP64) and its C, both split into double-float for the element kernels.
__global__ void k_elem_df(int E, const double *__restrict__ nodes, const int *__restrict__ elist,
                          const double *__restrict__ orient, const double *__restrict__ elC, float2 *__restrict__ Xdf,
                          float2 *__restrict__ Cdf) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    double Or[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) Or[i][j] = orient ? orient[9 * (size_t)e + 3 * j + i] : (i == j ? 1.0 : 0.0);
    // relative to the element's first node: the Jacobian only sees coordinate differences, and
    // taking them here in FP64 keeps the FP32 kernel from losing bits to cancellation (absolute
    // coordinates are up to about 60 element sizes larger than the differences in a block)
    const double *x0 = nodes + 3 * (size_t)(elist[8 * (size_t)e] - 1);
    for (int a = 0; a < 8; ++a) {
        const int nd = elist[8 * (size_t)e + a];
        const double *xa = nodes + 3 * (size_t)(nd - 1);
        const double x[3] = {xa[0] - x0[0], xa[1] - x0[1], xa[2] - x0[2]};
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

}  // namespace

// One colour launch; a colour after the first chains on its predecessor by programmatic dependent
// launch (the kernels wait for it before their first read-modify-write).
template <class Kern, class Args>
static void colour_launch(Kern kernel, unsigned grid, unsigned block, cudaStream_t s, bool chained, const Args &A) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = chained ? 1 : 0;
    cudaLaunchKernelEx(&cfg, kernel, A);
}

template <class T, bool ROT, int FW> static void hex8_fast_launch(astro_ctx *ctx, const Hex8FastArgs<T> &A0) {
    Hex8FastArgs<T> A = A0;
    const std::vector<int> &ptr = ctx->c8Ptr;
    bool chained = false;  // a colour after the first: programmatic dependent launch on its predecessor
    for (size_t col = 0; col + 1 < ptr.size(); ++col) {
        const int cnt = ptr[col + 1] - ptr[col];
        if (!cnt) continue;
        A.colorEls = dptr<int>(ctx->d_c8Els) + ptr[col];
        A.count = cnt;
        colour_launch(hex8_fast_kernel<T, ROT, FW>, (cnt + FW - 1) / FW, 32 * FW, ctx->stream, chained, A);
        chained = true;
    }
}

// Zero-state stiffness of every brick8 element, colour by colour, into K (block-CSR, written
// without a prior zeroing) and/or the element matrices d_ke.
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
    // warps per CTA: the autotuned choice of this context (astro_autotune), else 2
    switch (ctx->tuneHex8Warps) {
        case 1:
            ctx->orientIdentity ? hex8_fast_launch<T, false, 1>(ctx, A) : hex8_fast_launch<T, true, 1>(ctx, A);
            break;
        case 4:
            ctx->orientIdentity ? hex8_fast_launch<T, false, 4>(ctx, A) : hex8_fast_launch<T, true, 4>(ctx, A);
            break;
        default:
            ctx->orientIdentity ? hex8_fast_launch<T, false, 2>(ctx, A) : hex8_fast_launch<T, true, 2>(ctx, A);
    }
    return cuda_check(ctx, cudaGetLastError(), "brick8 zero-state kernel launch");
}

// General-state element kernel (double-float), colour by colour over the brick8 elements of list
// (colour c covering list[ptr[c] .. ptr[c+1])): the block-CSR matrix (with build), the residual
// into d_loadInt (load -= Ru), element matrices and residuals, at state s (with the Newmark
// inertia when s.dynamic).  CdfItem: per listed element its C (double-float, the complex step's
// imaginary part) instead of the element's own; gpc the Gauss point coordinate.
static int hex8_gen_run(astro_ctx *ctx, const int *d_list, const std::vector<int> &ptr, bool build, double *K,
                        const ElemDevState &s, double *d_loadInt, double *d_ke, double *d_ru, const float2 *CdfItem,
                        double gpc) {
    Hex8GenArgs A;
    A.elBlk = dptr<int>(ctx->d_elBlk);
    A.elFirst = dptr<unsigned long long>(ctx->d_elFirst);
    A.elist = dptr<int>(ctx->d_elist);
    A.rank = dptr<int>(ctx->d_rank);
    A.Xdf = dptr<float2>(ctx->d_elXdf);
    A.Cdf = dptr<float2>(ctx->d_elCdf);
    A.orient = dptr<double>(ctx->d_secOrient);
    A.disp = s.disp;
    A.pdisp = s.pdisp;
    A.pvel = s.pvel;
    A.pacc = s.pacc;
    A.rho = dptr<double>(ctx->d_elRho);
    A.dyn = s.dynamic ? 1 : 0;
    A.beta = s.beta;
    A.delT = s.delT;
    A.K = K;
    A.loadInt = d_loadInt;
    A.keOut = d_ke;
    A.ruOut = d_ru;
    const DF g = df_from_double(gpc);
    A.gpcHi = g.hi;
    A.gpcLo = g.lo;
    const bool rot = !ctx->orientIdentity;
    bool chained = false;
    for (size_t col = 0; col + 1 < ptr.size(); ++col) {
        const int cnt = ptr[col + 1] - ptr[col];
        if (!cnt) continue;
        A.colorEls = d_list + ptr[col];
        A.count = cnt;
        A.CdfItem = CdfItem ? CdfItem + 9 * (size_t)ptr[col] : nullptr;
        const unsigned grid = (cnt + kGenW - 1) / kGenW;
        if (build) {
            if (rot)
                colour_launch(hex8_gen_kernel<true, true>, grid, 32 * kGenW, ctx->stream, chained, A);
            else
                colour_launch(hex8_gen_kernel<false, true>, grid, 32 * kGenW, ctx->stream, chained, A);
        } else {
            if (rot)
                colour_launch(hex8_gen_kernel<true, false>, grid, 32 * kGenW, ctx->stream, chained, A);
            else
                colour_launch(hex8_gen_kernel<false, false>, grid, 32 * kGenW, ctx->stream, chained, A);
        }
        chained = true;
    }
    return cuda_check(ctx, cudaGetLastError(), "brick8 general-state kernel launch");
}

// FP64 zero-state stiffness of brick8 elements (double-float kernel), colour by colour over list
// (colour c covering list[ptr[c] .. ptr[c+1])).
static int hex8_df_run(astro_ctx *ctx, double *K, double *d_ke, const int *d_list, const std::vector<int> &ptr) {
    Hex8DfArgs A;
    A.elBlk = dptr<int>(ctx->d_elBlk);
    A.elFirst = dptr<unsigned long long>(ctx->d_elFirst);
    A.Xdf = dptr<float2>(ctx->d_elXdf);
    A.Cdf = dptr<float2>(ctx->d_elCdf);
    A.orient = dptr<double>(ctx->d_secOrient);
    A.K = K;
    A.keOut = d_ke;
    bool chained = false;
    for (size_t col = 0; col + 1 < ptr.size(); ++col) {
        const int cnt = ptr[col + 1] - ptr[col];
        if (!cnt) continue;
        A.colorEls = d_list + ptr[col];
        A.count = cnt;
        const unsigned grid = (cnt + kDfW - 1) / kDfW;
        if (ctx->orientIdentity)
            colour_launch(hex8_df_kernel<false>, grid, 32 * kDfW, ctx->stream, chained, A);
        else
            colour_launch(hex8_df_kernel<true>, grid, 32 * kDfW, ctx->stream, chained, A);
        chained = true;
    }
    return cuda_check(ctx, cudaGetLastError(), "brick8 FP64 zero-state kernel launch");
}

int hex8_prepare(astro_ctx *ctx) {
    const int E = ctx->P.E;
    int rc;
    // node-pair tiles (a, b), a <= b, in row-major upper-triangle order, for hex8_gen_kernel
    unsigned char ta[36], tb[36];
    for (int a = 0, t = 0; a < 8; ++a)
        for (int b = a; b < 8; ++b, ++t) {
            ta[t] = (unsigned char)a;
            tb[t] = (unsigned char)b;
        }
    CK(cudaMemcpyToSymbol(c_tileA, ta, sizeof(ta)));
    CK(cudaMemcpyToSymbol(c_tileB, tb, sizeof(tb)));
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
    return hex8_df_run(ctx, (store & 2) ? dptr<double>(ctx->d_K64) : nullptr, nullptr, dptr<int>(ctx->d_c8Els),
                       ctx->c8Ptr);
}

// getElasticSolnLoad for solid meshes.  brick8: from the undeformed state without inertia the
// residual is zero and the tangent is the small-strain stiffness (the zero-state double-float
// kernel); any other state takes the general kernel.  brickIM: the FP64 brickIM kernel, which also
// writes the condensed internal rows and the internal load.  Both write each block of the
// block-CSR matrix first (colour order), so no zeroing pass is needed.
int solid_soln_load(astro_ctx *ctx, int build, const ElemDevState &s, double *d_loadInt, double *d_intLoad,
                    double *d_ke, double *d_ru) {
    const bool toK = build && !d_ke, mat = build || d_ke;
    double *K = toK ? dptr<double>(ctx->d_K64) : nullptr;
    const bool zero8 = !s.disp && !s.dynamic && !d_ru;  // brick8 residual is zero: zero-state kernel
    // one pass over the colours with the given brick8 and brickIM colour lists
    auto pass = [&](const std::vector<int> &p8, const std::vector<int> &p81) -> int {
        int rc;
        if (p8.back() > p8.front()) {
            if (zero8) {
                if (mat && (rc = hex8_df_run(ctx, K, d_ke, dptr<int>(ctx->d_c8Els), p8))) return rc;
            } else if ((rc = hex8_gen_run(ctx, dptr<int>(ctx->d_c8Els), p8, mat, K, s, d_loadInt, d_ke, d_ru, nullptr,
                                          kRt3))) {
                return rc;
            }
        }
        if (p81.back() > p81.front() &&
            (rc = hex81_run(ctx, dptr<int>(ctx->d_c81Els), p81, mat ? 1 : 0, K, s, nullptr, kRt3, d_loadInt, d_intLoad,
                            toK ? dptr<double>(ctx->d_intMat) : nullptr, d_ke, d_ru)))
            return rc;
        return ASTRO_OK;
    };
    if (!ctx->has81 || ctx->c8Els.empty()) return pass(ctx->c8Ptr, ctx->c81Ptr);
    // both types: colour by colour, so that the first element (in colour order) to touch a
    // block of the matrix is the one that writes it
    for (size_t col = 0; col + 1 < ctx->c8Ptr.size(); ++col) {
        const std::vector<int> p8 = {ctx->c8Ptr[col], ctx->c8Ptr[col + 1]}, p81 = {ctx->c81Ptr[col], ctx->c81Ptr[col + 1]};
        const int rc = pass(p8, p81);
        if (rc) return rc;
    }
    return ASTRO_OK;
}

int launch_hex8_element_mats(astro_ctx *ctx, int precision, double *d_ke) {
    if (precision == 32) return hex8_fast_run<float>(ctx, nullptr, d_ke);
    ElemDevState s;
    return solid_soln_load(ctx, 1, s, nullptr, nullptr, d_ke, nullptr);
}
