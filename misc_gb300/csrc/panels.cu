// Batched panels: LDL^T factorisation and multi-right-hand-side solves of a model made of many
// independent panels (the connected components of its mesh), K + C^T C of the device-resident FP64
// stiffness, in one persistent launch per phase.
//
// The reference solves such a batch one model at a time with the row-skyline LDL^T of
// getSparseLDLFact / solveSparseLDLFact (Working/AStrO_solvers.f90:10-126): the same factorisation
// without pivoting, in exact arithmetic the same factor on the envelope.  Here:
//   ordering  each panel's nodes sorted by their coordinate along the panel's longest extent, then
//             the next (a structured panel becomes column by column along its short side: the
//             lower bandwidth is about dpn * (short side + 2) DOF);
//   storage   per panel the lower band in 32 x 32 FP64 tiles, column-major within a tile: tile
//             (J, d) holds block row J + d of block column J, d = 0 .. bt (bt = ceil(bw / 32));
//   factor    right-looking blocked LDL^T, one thread-block cluster per panel: every CTA of the
//             cluster factors the diagonal tile in shared memory, the CTAs split the panel rows
//             below it (L = A L_JJ^-T D^-1) and then the band's trailing tile updates
//             (A_IK -= L_IJ D_J L_KJ^T), with a cluster barrier after each of the two phases.
//             Panels are assigned to clusters by longest-processing-time first on the host, so a
//             cluster never waits on another (no spin-waits, no inter-cluster dependencies);
//   solve     one CTA per (panel, group of up to 8 right-hand sides): forward sweep with unit L,
//             D^-1, backward sweep with L^T; the eight warps split the band's tiles of a block row
//             and warp 0 reduces and solves the diagonal tile with shuffles.
// The trailing tile updates carry almost all of the factor's arithmetic.  They run in FP64 by
// default; ASTRO_OPT_BAND_FP64_UPDATE = 0 runs them on the tensor cores as an FP64-exact
// emulation instead (measured slower on GB300 than the FP64 update for these 32 x 32 tiles: 28
// level products of legacy mma.sync per tile against 32 FP64 multiply-adds per output, plus the
// slicing) (the error-free splitting of Ozaki, Ogita, Oishi and Rump, "Error-free transformations
// of matrix multiplication by using fast routines of matrix multiplication and its applications",
// Numer. Algorithms 59, 2012, with BF16 slices):
//   * after the tiles L_IJ of block column J are formed, every row of D_J-scaled L_IJ and of L_IJ
//     is scaled by a power of two 2^e (|row| / 2^e < 1) and cut into kSlices slices of 8 bits,
//     t_p = trunc(2^(8p) x - ...), integers in [-255, 255] that BF16 holds exactly:
//     x = sum_p t_p 2^(-8p) + O(2^(-8 kSlices));
//   * for a tile pair the slice products with the same level l = p + q are summed by BF16 tensor
//     core MMAs into one FP32 accumulator: every product is an integer below 2^16, 32 of them sum
//     below 2^21 and at most 7 pairs share a level, so the FP32 sums are exact;
//   * each output gets sum_l 2^(-8 l) S_l in FP64, scaled by 2^(e_row + e_col): 7 FP64 operations
//     per output instead of 32 multiply-adds.  With 7 slices the update carries about 56 bits,
//     beyond FP64's 53.
// The FP64 update stays available (ASTRO_OPT_BAND_FP64_UPDATE) for comparison.
#include <cooperative_groups.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <numeric>
#include <vector>

#include "astro_internal.h"
#include "dfloat.cuh"

namespace cg = cooperative_groups;

namespace {

constexpr int TB = 32;  // tile edge
constexpr int TT = TB * TB;
constexpr int kThreads = 256;
constexpr int kGroups = kThreads / TB;  // warps per CTA
constexpr int kSolveCols = 8;           // right-hand sides per solve CTA
constexpr int kSlices = 7;              // 8-bit slices per FP64 value in the emulated tile update
constexpr int kLevels = kSlices;        // levels l = p + q = 2 .. kSlices + 1 of the slice products

struct PanelMeta {
    long long band;   // first double of the panel's tiles
    long long xUnit;  // rows of the padded right-hand-side layout before this panel (times nrhs)
    int n;            // DOF
    int nbc;          // block columns, ceil(n / 32)
    int bt;           // tiles below the diagonal tile in a block column
    int nfac;         // block columns the factorisation eliminates (nbc; fewer for a partial factor)
};

struct SolveItem {
    int panel, col0, ncol, pad;
};

struct PanelPlan {
    int np = 0;
    int cs = 0, workers = 0;
    int factored = 0, kVersion = -1, penVersion = -1;
    int maxBw = 0;
    long long bandDoubles = 0, xRows = 0;
    std::vector<PanelMeta> meta;
    std::vector<int> panelOf, pos;  // per rank (0-based)
    std::vector<double> work;
    std::vector<int> sched, schedPtr;
    DevBuf d_meta, d_sched, d_schedPtr, d_panelOf, d_pos, d_band, d_status, d_penI, d_penJ, d_penV;
    DevBuf d_slices, d_sexp;  // per worker: BF16 slices and row scales of one block column's tiles
    long long sliceStride = 0;
    int expStride = 0, maxBt = 0;
    int penCount = 0;
    double factorSeconds = 0.0;
    // double-float copies for the many-column solve (k_band_solve_cases), built from factor
    // generation dfGen; the items and the right-hand-side block for casesCols columns
    int factorGen = 0, dfGen = -1, casesCols = 0, ring = 0;
    DevBuf d_Lf, d_Lb, d_Wf, d_Wb, d_Dinv, d_items, d_X;
    // astro_panels_solve's work buffers (grow-only): right-hand sides in both orderings, the
    // refinement's residuals, the panel-layout block and the items
    DevBuf d_sRef, d_sVec, d_sRes, d_sBi, d_sX, d_sItems;
    // twisted many-column solve of a single panel (twist_prepare): panels top (block rows
    // 0 .. K+m-1), bottom (block rows K .. nbc-1, reversed) and window (the m block rows K ..)
    int twist = 0, twK = 0, twM = 0, twGen = -1, twCols = 0;
    long long twBandDoubles = 0, twRows = 0;
    double twFactorSeconds = 0.0;
    std::vector<PanelMeta> twMeta;
    DevBuf d_twMeta, d_twBand, d_twAw, d_twSched, d_twSchedPtr, d_twStatus, d_twLf, d_twLb, d_twWf, d_twWb, d_twDinv,
        d_twItems, d_twX;
};

__device__ __forceinline__ size_t tile_off(const PanelMeta &M, int J, int d) {
    return (size_t)M.band + ((size_t)J * (M.bt + 1) + d) * TT;
}

// lower-band entries of the BSR stiffness (dpn x dpn row-major blocks) into the tiles
__global__ void k_band_fill(int nb, int dpn, const int *__restrict__ bRow, const int *__restrict__ bCol,
                            const double *__restrict__ K, const int *__restrict__ panelOf, const int *__restrict__ pos,
                            const PanelMeta *__restrict__ meta, double *__restrict__ band) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const int bs = dpn * dpn;
    if (t >= (long long)nb * bs) return;
    const int b = (int)(t / bs), q = (int)(t % bs), a = q / dpn, c = q % dpn;
    const int r = bRow[b], col = bCol[b];
    const int i = pos[r] * dpn + a, j = pos[col] * dpn + c;
    if (j > i) return;
    const PanelMeta &M = meta[panelOf[r]];
    const int I = i / TB, J = j / TB;
    band[tile_off(M, J, I - J) + (j % TB) * TB + (i % TB)] = K[(size_t)b * bs + q];
}

// + C^T C (penalty entries, internal numbering; each (row, column) once)
__global__ void k_band_pen(int cnt, int dpn, const int *__restrict__ pi, const int *__restrict__ pj,
                           const double *__restrict__ pv, const int *__restrict__ panelOf, const int *__restrict__ pos,
                           const PanelMeta *__restrict__ meta, double *__restrict__ band) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= cnt) return;
    const int ri = pi[t] / dpn, rj = pj[t] / dpn;
    const int i = pos[ri] * dpn + pi[t] % dpn, j = pos[rj] * dpn + pj[t] % dpn;
    if (j > i) return;
    const PanelMeta &M = meta[panelOf[ri]];
    const int I = i / TB, J = j / TB;
    band[tile_off(M, J, I - J) + (j % TB) * TB + (i % TB)] += pv[t];
}

// unit diagonal on the padding rows of each panel's last block
__global__ void k_band_pad(const PanelMeta *__restrict__ meta, double *__restrict__ band) {
    const PanelMeta M = meta[blockIdx.x];
    const int i = M.n + threadIdx.x;
    if (i >= M.nbc * TB) return;
    band[tile_off(M, i / TB, 0) + (i % TB) * TB + (i % TB)] = 1.0;
}

// D = A B + D for one m16n8k16 BF16 tile with FP32 accumulation (tensor cores)
__device__ __forceinline__ void mma_bf16(float d[4], const unsigned a[4], const unsigned b[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ unsigned ld_pair(const uint16_t *p) { return __ldcg(reinterpret_cast<const unsigned *>(p)); }

// ---- tcgen05 (5th-generation tensor cores) for the emulated trailing update -----------------------
// One work item is a group of 4 block rows d0 .. d0+3 of block column J against block row e: the
// 128 x 32 product of the 7 slices of L D_J (rows) and of L (columns), every level
// l = p + q in its own 32-column FP32 accumulator in tensor memory (7 x 32 = 224 of the CTA's 256
// columns).  Operands sit in shared memory in the no-swizzle K-major core-matrix layout: element
// (r, k) of a slice at ((r / 8) * 4 + k / 8) * 64 + (r % 8) * 8 + k % 8, i.e. 8-row x 16-byte core
// matrices, 128 B apart along K and 512 B apart along the rows.
constexpr int kTcRows = 4 * TB;                          // rows of the A operand (4 block rows)
constexpr int kTcSliceA = kTcRows * TB;                  // bf16 elements per A slice
constexpr int kTcSliceB = TB * TB;                       // bf16 elements per B slice
constexpr int kTcSmem = kSlices * (kTcSliceA + kTcSliceB) * 2;  // bytes of dynamic shared memory
constexpr int kTcCols = 256;                             // tensor-memory columns per CTA
constexpr int kTcWaitLimit = 1 << 24;                    // polls of the MMA-completion barrier

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ int tc_cm(int r, int k) { return ((r >> 3) * (TB / 8) + (k >> 3)) * 64 + (r & 7) * 8 + (k & 7); }

// shared-memory matrix descriptor: start, leading (K) and stride (row-group) byte offsets, no
// swizzle, descriptor version 1
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr) {
    return (uint64_t)((saddr >> 4) & 0x3FFF) | ((uint64_t)(128 >> 4) << 16) | ((uint64_t)(512 >> 4) << 32) |
           ((uint64_t)1 << 46);
}

// kind::f16 instruction descriptor: FP32 accumulator, BF16 A and B, both K-major, N = 32, M = 128
constexpr uint32_t kTcIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(TB >> 3) << 17) | ((uint32_t)(kTcRows >> 4) << 24);

__device__ __forceinline__ void tc_mma(uint32_t tmem, uint64_t da, uint64_t db, uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(tmem),
        "l"(da), "l"(db), "r"(kTcIdesc), "r"(accumulate));
}

// 16 consecutive FP32 columns of this warp's 32 tensor-memory lanes
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float v[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

// one block row's 7 slices (rows row0 .. row0+31 of the operand) from the global scratch (row-major
// [p][r][k]) into the core-matrix layout; zeros when src is null.  16 bytes per thread and step.
__device__ __forceinline__ void tc_stage(const uint16_t *src, uint16_t *dst, int sliceElems, int row0, int t) {
    for (int x = t; x < kSlices * TB * (TB / 8); x += kThreads) {
        const int p = x / (TB * (TB / 8)), r = (x / (TB / 8)) % TB, k8 = x % (TB / 8);
        uint4 v = make_uint4(0u, 0u, 0u, 0u);
        if (src) v = __ldcg(reinterpret_cast<const uint4 *>(src + (size_t)p * TT + r * TB + k8 * 8));
        *reinterpret_cast<uint4 *>(dst + (size_t)p * sliceElems + tc_cm(row0 + r, k8 * 8)) = v;
    }
}

// Slices of one tile of block column J (tile d, version v: 0 = L D_J, 1 = L) by one warp: lane r
// takes row r, its power-of-two scale e_r (|row| / 2^e_r < 1) and kSlices 8-bit slices as BF16
// integers, row-major [r][k] per slice.
__device__ void split_tile(const double *T, const double (*sL)[TB + 1], int v, uint16_t *S, int *E, int lane) {
    double x[TB];
    double mx = 0.0;
#pragma unroll
    for (int k = 0; k < TB; ++k) {
        x[k] = __ldcg(T + k * TB + lane);
        if (v == 0) x[k] *= sL[k][k];
        mx = fmax(mx, fabs(x[k]));
    }
    int e = 0;
    if (mx > 0.0) frexp(mx, &e);
    E[lane] = e;
#pragma unroll
    for (int k = 0; k < TB; ++k) x[k] = ldexp(x[k], -e);
    for (int p = 0; p < kSlices; ++p) {
        uint16_t *Sp = S + (size_t)p * TT + lane * TB;
#pragma unroll
        for (int k = 0; k < TB; k += 2) {
            const double y0 = x[k] * 256.0, y1 = x[k + 1] * 256.0;
            const double t0 = trunc(y0), t1 = trunc(y1);
            x[k] = y0 - t0;
            x[k + 1] = y1 - t1;
            const unsigned lo = __bfloat16_as_ushort(__float2bfloat16_rn((float)t0)),
                           hi = __bfloat16_as_ushort(__float2bfloat16_rn((float)t1));
            *reinterpret_cast<unsigned *>(Sp + k) = lo | (hi << 16);
        }
    }
}

// Blocked band LDL^T, one cluster per panel (the cluster's panels listed in sched).  MODE 0: the
// trailing updates in FP64; MODE 1 and 2: the tensor-core emulation described at the top of the
// file, MODE 1 on mma.sync (16 x 8 blocks per warp), MODE 2 on tcgen05 (128 x 32 per MMA, the
// accumulators in tensor memory), with the slices of each worker (cluster) in
// slices + worker * sliceStride and their scales in sexp + worker * expStride.  Both emulations
// sum every level exactly and combine the levels in the same order: identical results.
template <int MODE>
__global__ void __launch_bounds__(kThreads, MODE == 2 ? 1 : 2) k_band_ldl(const PanelMeta *__restrict__ meta, const int *__restrict__ sched,
                                                       const int *__restrict__ schedPtr, double *band, int *status,
                                                       uint16_t *slices, int *sexp, long long sliceStride,
                                                       int expStride) {
    constexpr bool TC = MODE == 1 || MODE == 2;
    cg::cluster_group cl = cg::this_cluster();
    const int crank = (int)cl.block_rank(), cs = (int)cl.num_blocks();
    const int worker = blockIdx.x / cs;
    uint16_t *wsl = TC ? slices + (size_t)worker * sliceStride : nullptr;
    int *wex = TC ? sexp + (size_t)worker * expStride : nullptr;
    __shared__ double sL[TB][TB + 1];  // diagonal tile: L below the diagonal, D on it
    __shared__ double sDi[TB];         // D^-1
    __shared__ double sA[TB][TB + 1], sB[TB][TB + 1];
    const int t = threadIdx.x;
    // MODE 2: tensor memory, the completion barrier of the MMAs and the operand staging
    extern __shared__ __align__(1024) uint16_t tcSmem[];
    __shared__ __align__(8) unsigned long long tcBar;
    __shared__ uint32_t tcBase;
    uint32_t tcPhase = 0;
    bool tcFailed = false;
    if constexpr (MODE == 2) {
        if (t < 32) {
            asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&tcBase)),
                         "r"(kTcCols));
            asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
        }
        if (t == 0) asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(&tcBar)), "r"(1));
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    }
    for (int q = schedPtr[worker]; q < schedPtr[worker + 1]; ++q) {
        const int p = sched[q];
        const PanelMeta M = meta[p];
        for (int J = 0; J < M.nfac; ++J) {
            // A. the diagonal tile, factored by every CTA of the cluster into its shared memory
            double *Td = band + tile_off(M, J, 0);
            for (int e = t; e < TT; e += kThreads) sL[e % TB][e / TB] = __ldcg(Td + e);
            __syncthreads();
            for (int k = 0; k < TB; ++k) {
                const double inv = 1.0 / sL[k][k];
                const int j = t % TB;
                if (j > k)
                    for (int i = t / TB; i < TB; i += kGroups)
                        if (i >= j) sL[i][j] -= sL[i][k] * sL[j][k] * inv;
                __syncthreads();
                if (t > k && t < TB) sL[t][k] *= inv;
                __syncthreads();
            }
            if (crank == 0 && t < TB && J * TB + t < M.n) {
                const double dk = sL[t][t];
                if (!(dk != 0.0 && isfinite(dk))) atomicCAS(status, 0, p + 1);
            }
            if (t < TB) sDi[t] = 1.0 / sL[t][t];
            __syncthreads();
            // B. the tiles below: L_IJ = A_IJ L_JJ^-T D^-1, one row per thread across the cluster
            for (int rho = crank * kThreads + t; rho < M.bt * TB; rho += cs * kThreads) {
                const int d = 1 + rho / TB, r = rho % TB;
                if (J + d >= M.nbc) continue;
                double *T = band + tile_off(M, J, d);
                double w[TB];
#pragma unroll
                for (int c = 0; c < TB; ++c) w[c] = __ldcg(T + c * TB + r);
#pragma unroll
                for (int k = 1; k < TB; ++k) {
                    double s = w[k];
#pragma unroll
                    for (int m = 0; m < k; ++m) s -= w[m] * sL[k][m];
                    w[k] = s;
                }
#pragma unroll
                for (int c = 0; c < TB; ++c) __stcg(T + c * TB + r, w[c] * sDi[c]);
            }
            __threadfence();
            cl.sync();
            // every CTA has read the unfactored diagonal tile: store the factored one
            if (crank == 0)
                for (int e = t; e < TT; e += kThreads) __stcg(Td + e, sL[e % TB][e / TB]);
            const int nt = M.bt * (M.bt + 1) / 2;
            if constexpr (TC) {
                // B2. slices of the tiles below the diagonal (versions L D_J and L), one warp each
                const int lane = t & 31, wg = crank * kGroups + (t >> 5);
                for (int uu = wg; uu < 2 * M.bt; uu += cs * kGroups) {
                    const int d = 1 + uu / 2, v = uu % 2;
                    if (J + d >= M.nbc) continue;
                    split_tile(band + tile_off(M, J, d), sL, v, wsl + (size_t)uu * kSlices * TT, wex + uu * TB, lane);
                }
                __threadfence();
                cl.sync();
                if constexpr (MODE == 2) {
                    // C. trailing update on tcgen05: items (group gi of block rows d0 .. d0+3, block
                    // column e <= d0 + 3), round-robin over the cluster; a CTA keeps its A operand
                    // while consecutive items share the group
                    uint16_t *sAop = tcSmem, *sBop = tcSmem + kSlices * kTcSliceA;
                    const int ng = (M.bt + 3) / 4;
                    int nItems = 0;
                    for (int gi = 0; gi < ng; ++gi) nItems += min(4 * gi + 4, M.bt);
                    int curG = -1, gi = 0, gBase = 0;  // item index of group gi's first item
                    const int w = t >> 5;
                    for (int u = crank; u < nItems; u += cs) {
                        while (u >= gBase + min(4 * gi + 4, M.bt)) {
                            gBase += min(4 * gi + 4, M.bt);
                            ++gi;
                        }
                        const int d0 = 1 + 4 * gi, e = 1 + (u - gBase);
                        if (J + e >= M.nbc || tcFailed) continue;
                        if (gi != curG) {
                            for (int b = 0; b < 4; ++b) {
                                const int d = d0 + b;
                                const bool ok = d <= M.bt && J + d < M.nbc;
                                tc_stage(ok ? wsl + (size_t)(2 * (d - 1)) * kSlices * TT : nullptr, sAop, kTcSliceA,
                                         b * TB, t);
                            }
                            curG = gi;
                        }
                        tc_stage(wsl + (size_t)(2 * (e - 1) + 1) * kSlices * TT, sBop, kTcSliceB, 0, t);
                        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
                        __syncthreads();
                        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                        if (t == 0) {
                            const uint32_t aBase = smem_addr(sAop), bBase = smem_addr(sBop);
#pragma unroll 1
                            for (int li = 0; li < kLevels; ++li) {  // level l = li + 2 = p + q
                                uint32_t acc = 0;
#pragma unroll 1
                                for (int p = 1; p <= kSlices; ++p) {
                                    const int q = li + 2 - p;
                                    if (q < 1 || q > kSlices) continue;
#pragma unroll
                                    for (int kk = 0; kk < 2; ++kk) {
                                        tc_mma(tcBase + li * TB, tc_desc(aBase + (p - 1) * kTcSliceA * 2 + kk * 256),
                                               tc_desc(bBase + (q - 1) * kTcSliceB * 2 + kk * 256), acc);
                                        acc = 1;
                                    }
                                }
                            }
                            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                             smem_addr(&tcBar))
                                         : "memory");
                        }
                        uint32_t done = 0;
                        for (int it = 0; it < kTcWaitLimit && !done; ++it)
                            asm volatile(
                                "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                                " selp.u32 %0, 1, 0, p;\n}"
                                : "=r"(done)
                                : "r"(smem_addr(&tcBar)), "r"(tcPhase)
                                : "memory");
                        tcPhase ^= 1u;
                        if (!done) {
                            tcFailed = true;
                            atomicCAS(status, 0, -1);
                        }
                        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                        // epilogue: warp w reads lanes 32 (w % 4) .. of block row d0 + w % 4 and
                        // columns 16 (w / 4) ..; the levels combined in FP64 as in MODE 1
                        const int d = d0 + (w & 3), c0 = 16 * (w >> 2);
                        if (done && d <= M.bt && J + d < M.nbc && d >= e) {
                            double sum[16];
#pragma unroll
                            for (int j = 0; j < 16; ++j) sum[j] = 0.0;
                            double sc = 1.0 / 65536.0;  // 2^(-8 l), l = 2 ..
#pragma unroll 1
                            for (int li = 0; li < kLevels; ++li) {
                                float v[16];
                                tc_ld16(tcBase + ((uint32_t)(32 * (w & 3)) << 16) + li * TB + c0, v);
#pragma unroll
                                for (int j = 0; j < 16; ++j) sum[j] += (double)v[j] * sc;
                                sc *= 1.0 / 256.0;
                            }
                            double *Tt = band + tile_off(M, J + e, d - e);
                            const int rr = lane;
                            const int ea = __ldcg(wex + 2 * (d - 1) * TB + rr);
                            const int *EB = wex + (2 * (e - 1) + 1) * TB;
#pragma unroll
                            for (int j = 0; j < 16; ++j) {
                                double *pt = Tt + (c0 + j) * TB + rr;
                                __stcg(pt, __ldcg(pt) - ldexp(sum[j], ea + __ldcg(EB + c0 + j)));
                            }
                        }
                        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
                        __syncthreads();
                    }
                    __threadfence();
                    cl.sync();
                    continue;
                }
                // C. trailing update, tensor cores: warp w computes the 16 x 8 block (mi, ni) of the
                // 32 x 32 tile, every level l of the slice products in its own FP32 accumulator
                const int w = t >> 5, g = lane >> 2, tg = lane & 3, mi = w >> 2, ni = w & 3;
                for (int u = crank; u < nt; u += cs) {
                    int d = 1, rem = u;
                    while (rem >= d) {
                        rem -= d;
                        ++d;
                    }
                    const int e = 1 + rem;
                    if (J + d >= M.nbc) continue;
                    const uint16_t *SA = wsl + (size_t)(2 * (d - 1)) * kSlices * TT;
                    const uint16_t *SB = wsl + (size_t)(2 * (e - 1) + 1) * kSlices * TT;
                    unsigned a[kSlices][2][4], b[kSlices][2][2];
                    const int ra = (16 * mi + g) * TB, rb = (8 * ni + g) * TB;
#pragma unroll
                    for (int p = 0; p < kSlices; ++p)
#pragma unroll
                        for (int ks = 0; ks < 2; ++ks) {
                            const uint16_t *pa = SA + (size_t)p * TT + 16 * ks + 2 * tg;
                            const uint16_t *pb = SB + (size_t)p * TT + 16 * ks + 2 * tg;
                            a[p][ks][0] = ld_pair(pa + ra);
                            a[p][ks][1] = ld_pair(pa + ra + 8 * TB);
                            a[p][ks][2] = ld_pair(pa + ra + 8);
                            a[p][ks][3] = ld_pair(pa + ra + 8 * TB + 8);
                            b[p][ks][0] = ld_pair(pb + rb);
                            b[p][ks][1] = ld_pair(pb + rb + 8);
                        }
                    float acc[kLevels][4];
#pragma unroll
                    for (int li = 0; li < kLevels; ++li)
#pragma unroll
                        for (int i = 0; i < 4; ++i) acc[li][i] = 0.f;
#pragma unroll
                    for (int li = 0; li < kLevels; ++li) {  // level l = li + 2 = p + q
#pragma unroll
                        for (int p = 1; p <= kSlices; ++p) {
                            const int q = li + 2 - p;
                            if (q < 1 || q > kSlices) continue;
#pragma unroll
                            for (int ks = 0; ks < 2; ++ks) mma_bf16(acc[li], a[p - 1][ks], b[q - 1][ks]);
                        }
                    }
                    double *Tt = band + tile_off(M, J + e, d - e);
                    const int *EA = wex + 2 * (d - 1) * TB, *EB = wex + (2 * (e - 1) + 1) * TB;
#pragma unroll
                    for (int i = 0; i < 4; ++i) {
                        const int rr = 16 * mi + g + (i >> 1) * 8, cc = 8 * ni + 2 * tg + (i & 1);
                        double sum = 0.0, sc = 1.0 / 65536.0;  // 2^(-8 l), l = 2 ..
#pragma unroll
                        for (int li = 0; li < kLevels; ++li) {
                            sum += (double)acc[li][i] * sc;
                            sc *= 1.0 / 256.0;
                        }
                        double *pt = Tt + cc * TB + rr;
                        __stcg(pt, __ldcg(pt) - ldexp(sum, __ldcg(EA + rr) + __ldcg(EB + cc)));
                    }
                }
                __threadfence();
                cl.sync();
                continue;
            }
            // C. trailing update of the band: tile (J+e, d-e) -= L_{J+d,J} D_J L_{J+e,J}^T, 1 <= e <= d
            for (int u = crank; u < nt; u += cs) {
                int d = 1, rem = u;
                while (rem >= d) {
                    rem -= d;
                    ++d;
                }
                const int e = 1 + rem;
                if (J + d >= M.nbc) continue;
                const double *Ld = band + tile_off(M, J, d), *Le = band + tile_off(M, J, e);
                __syncthreads();
                for (int x = t; x < TT; x += kThreads) {
                    const int r = x % TB, c = x / TB;
                    sA[r][c] = __ldcg(Ld + x) * sL[c][c];
                    sB[r][c] = __ldcg(Le + x);
                }
                __syncthreads();
                const int r = t % TB, c0 = (t / TB) * 4;
                double acc[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll 8
                for (int k = 0; k < TB; ++k) {
                    const double a = sA[r][k];
#pragma unroll
                    for (int cc = 0; cc < 4; ++cc) acc[cc] += a * sB[c0 + cc][k];
                }
                double *Tt = band + tile_off(M, J + e, d - e);
#pragma unroll
                for (int cc = 0; cc < 4; ++cc) {
                    double *pt = Tt + (c0 + cc) * TB + r;
                    __stcg(pt, __ldcg(pt) - acc[cc]);
                }
            }
            __threadfence();
            cl.sync();
        }
    }
    if constexpr (MODE == 2) {
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        if (t < 32)
            asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tcBase), "r"(kTcCols));
    }
}

// ---- the band LDL^T carried in double-float (ASTRO_OPT_BAND_FP64_UPDATE = 3) ---------------
//
// The band converted in place to (hi, lo) float pairs (same 8 bytes per value), factored with
// every step in double-float arithmetic on the FP32 pipe, then converted back to FP64: the steps
// of k_band_ldl (the diagonal tile in shared memory in every CTA of the cluster, the rows below
// split over the cluster, the trailing updates split over the cluster) with no FP64 instruction
// inside.  About 48 significant bits per operation: a factor for solves that refine against the
// FP64 operator.

__global__ void k_band_df_convert(long long n, double *band, int toDf) {
    float2 *bf = reinterpret_cast<float2 *>(band);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        if (toDf) {
            const DF v = df_from_double(band[i]);
            bf[i] = make_float2(v.hi, v.lo);
        } else {
            const float2 v = bf[i];
            band[i] = (double)v.x + (double)v.y;
        }
    }
}

__device__ __forceinline__ DF df_of(float2 v) { return DF{v.x, v.y}; }
__device__ __forceinline__ float2 f2_of(DF v) { return make_float2(v.hi, v.lo); }

// scratch + worker * scratchStride: the block column's tiles below the diagonal times D_J, tile d
// at (d - 1) TT
__global__ void __launch_bounds__(kThreads, 2) k_band_ldl_df(const PanelMeta *__restrict__ meta,
                                                             const int *__restrict__ sched,
                                                             const int *__restrict__ schedPtr, float2 *band,
                                                             int *status, float2 *scratch, long long scratchStride) {
    cg::cluster_group cl = cg::this_cluster();
    const int crank = (int)cl.block_rank(), cs = (int)cl.num_blocks();
    const int worker = blockIdx.x / cs;
    float2 *wdf = scratch + (size_t)worker * scratchStride;
    __shared__ float2 sL[TB][TB + 1];  // diagonal tile: L below the diagonal, D on it
    __shared__ float2 sDi[TB];         // D^-1
    __shared__ float2 fA[TB][TB + 1], fB[TB][TB + 1];
    const int t = threadIdx.x;
    for (int q = schedPtr[worker]; q < schedPtr[worker + 1]; ++q) {
        const int p = sched[q];
        const PanelMeta M = meta[p];
        for (int J = 0; J < M.nfac; ++J) {
            // A. the diagonal tile
            float2 *Td = band + tile_off(M, J, 0);
            for (int e = t; e < TT; e += kThreads) sL[e % TB][e / TB] = __ldcg(Td + e);
            __syncthreads();
            for (int k = 0; k < TB; ++k) {
                const DF inv = df_rcp(df_of(sL[k][k]));
                const int j = t % TB;
                if (j > k) {
                    const DF f = df_mul(df_of(sL[j][k]), inv);
                    for (int i = t / TB; i < TB; i += kGroups)
                        if (i >= j) sL[i][j] = f2_of(df_sub(df_of(sL[i][j]), df_mul(df_of(sL[i][k]), f)));
                }
                __syncthreads();
                if (t > k && t < TB) sL[t][k] = f2_of(df_mul(df_of(sL[t][k]), inv));
                __syncthreads();
            }
            if (crank == 0 && t < TB && J * TB + t < M.n) {
                const float dk = sL[t][t].x;
                if (!(dk != 0.f && isfinite(dk))) atomicCAS(status, 0, p + 1);
            }
            if (t < TB) sDi[t] = f2_of(df_rcp(df_of(sL[t][t])));
            __syncthreads();
            // B. the tiles below: L_IJ = A_IJ L_JJ^-T D^-1, one row per thread across the cluster
            for (int rho = crank * kThreads + t; rho < M.bt * TB; rho += cs * kThreads) {
                const int d = 1 + rho / TB, r = rho % TB;
                if (J + d >= M.nbc) continue;
                float2 *T = band + tile_off(M, J, d);
                DF w[TB];
#pragma unroll
                for (int c = 0; c < TB; ++c) w[c] = df_of(__ldcg(T + c * TB + r));
#pragma unroll
                for (int k = 1; k < TB; ++k) {
                    DF acc = {0.f, 0.f};
#pragma unroll
                    for (int m = 0; m < k; ++m) {
                        const float2 l = sL[k][m];
                        df_acc(acc, w[m].hi, w[m].lo, l.x, l.y);
                    }
                    w[k] = df_sub(w[k], df_norm(acc));
                }
#pragma unroll
                for (int c = 0; c < TB; ++c) __stcg(T + c * TB + r, f2_of(df_mul(w[c], df_of(sDi[c]))));
            }
            __threadfence();
            cl.sync();
            // every CTA has read the unfactored diagonal tile: store the factored one
            if (crank == 0)
                for (int e = t; e < TT; e += kThreads) __stcg(Td + e, sL[e % TB][e / TB]);
            // B2. L D_J of the tiles below into the worker's scratch
            for (int x = crank * kThreads + t; x < M.bt * TT; x += cs * kThreads) {
                const int d = 1 + x / TT, el = x % TT;
                if (J + d >= M.nbc) continue;
                __stcg(wdf + x, f2_of(df_mul(df_of(__ldcg(band + tile_off(M, J, d) + el)), df_of(sL[el / TB][el / TB]))));
            }
            __threadfence();
            cl.sync();
            // C. trailing update: tile (J+e, d-e) -= (L D_J)_{J+d} L_{J+e}^T, 1 <= e <= d; the next
            // item's operands and outputs are loaded into registers while the current one computes
            const int nt = M.bt * (M.bt + 1) / 2;
            const int r = t % TB, c0 = (t / TB) * 4;
            auto item = [&](int u, int &d, int &e) {
                d = 1;
                int rem = u;
                while (rem >= d) {
                    rem -= d;
                    ++d;
                }
                e = 1 + rem;
            };
            auto next = [&](int u) {  // the first item >= u of this CTA inside the band
                for (; u < nt; u += cs) {
                    int d, e;
                    item(u, d, e);
                    if (J + d < M.nbc) break;
                }
                return u;
            };
            float2 ra[TT / kThreads], rb[TT / kThreads], ro[4];
            auto fetch = [&](int u) {
                int d, e;
                item(u, d, e);
                const float2 *Ad = wdf + (size_t)(d - 1) * TT, *Be = band + tile_off(M, J, e);
#pragma unroll
                for (int j = 0; j < TT / kThreads; ++j) {
                    ra[j] = __ldcg(Ad + t + j * kThreads);
                    rb[j] = __ldcg(Be + t + j * kThreads);
                }
                const float2 *Tt = band + tile_off(M, J + e, d - e);
#pragma unroll
                for (int cc = 0; cc < 4; ++cc) ro[cc] = __ldcg(Tt + (c0 + cc) * TB + r);
            };
            int u = next(crank);
            if (u < nt) fetch(u);
            while (u < nt) {
                const int un = next(u + cs);
                __syncthreads();
#pragma unroll
                for (int j = 0; j < TT / kThreads; ++j) {
                    const int x = t + j * kThreads;
                    fA[x % TB][x / TB] = ra[j];
                    fB[x % TB][x / TB] = rb[j];
                }
                __syncthreads();
                float2 o[4];
#pragma unroll
                for (int cc = 0; cc < 4; ++cc) o[cc] = ro[cc];
                int d, e;
                item(u, d, e);
                if (un < nt) fetch(un);
                DF acc[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
#pragma unroll 8
                for (int k = 0; k < TB; ++k) {
                    const float2 a = fA[r][k];
#pragma unroll
                    for (int cc = 0; cc < 4; ++cc) {
                        const float2 b = fB[c0 + cc][k];
                        df_acc(acc[cc], a.x, a.y, b.x, b.y);
                    }
                }
                float2 *Tt = band + tile_off(M, J + e, d - e);
#pragma unroll
                for (int cc = 0; cc < 4; ++cc)
                    __stcg(Tt + (c0 + cc) * TB + r, f2_of(df_sub(df_of(o[cc]), df_norm(acc[cc]))));
                u = un;
            }
            __threadfence();
            cl.sync();
        }
    }
}

// Forward and backward sweeps for the right-hand sides col0 .. col0+ncol-1 of one panel, in
// place in X (panel block: nrhs columns of npad rows).
__global__ void __launch_bounds__(kThreads) k_band_solve(const PanelMeta *__restrict__ meta,
                                                         const SolveItem *__restrict__ items,
                                                         const double *__restrict__ band, double *X, int nrhs) {
    extern __shared__ double sm[];
    double(*sT)[TB][TB + 1] = reinterpret_cast<double(*)[TB][TB + 1]>(sm);
    double(*sP)[TB][kSolveCols + 1] = reinterpret_cast<double(*)[TB][kSolveCols + 1]>(sm + kGroups * TB * (TB + 1));
    const SolveItem it = items[blockIdx.x];
    const PanelMeta M = meta[it.panel];
    const int npad = M.nbc * TB, ncol = it.ncol;
    double *Xp = X + (size_t)M.xUnit * nrhs + (size_t)it.col0 * npad;
    const int t = threadIdx.x, r = t % TB, g = t / TB;
    // forward: L y = b
    for (int I = 0; I < M.nbc; ++I) {
        double acc[kSolveCols];
#pragma unroll
        for (int c = 0; c < kSolveCols; ++c) acc[c] = 0.0;
        const int dmax = min(M.bt, I);
        for (int d = 1 + g; d <= dmax; d += kGroups) {
            const double *L = band + tile_off(M, I - d, d);
            const double *y = Xp + (size_t)(I - d) * TB;
            for (int k = 0; k < TB; ++k) {
                const double l = L[k * TB + r];
#pragma unroll
                for (int c = 0; c < kSolveCols; ++c)
                    if (c < ncol) acc[c] += l * y[(size_t)c * npad + k];
            }
        }
#pragma unroll
        for (int c = 0; c < kSolveCols; ++c) sP[g][r][c] = acc[c];
        __syncthreads();
        if (g == 0) {
            const double *Ld = band + tile_off(M, I, 0);
            double v[kSolveCols];
#pragma unroll
            for (int c = 0; c < kSolveCols; ++c) {
                double s = 0.0;
                for (int q = 0; q < kGroups; ++q) s += sP[q][r][c];
                v[c] = (c < ncol) ? Xp[(size_t)c * npad + I * TB + r] - s : 0.0;
            }
            for (int k = 0; k < TB; ++k) {
                const double lk = Ld[k * TB + r];
#pragma unroll
                for (int c = 0; c < kSolveCols; ++c) {
                    const double yk = __shfl_sync(0xffffffffu, v[c], k);
                    if (r > k) v[c] -= lk * yk;
                }
            }
#pragma unroll
            for (int c = 0; c < kSolveCols; ++c)
                if (c < ncol) Xp[(size_t)c * npad + I * TB + r] = v[c];
        }
        __syncthreads();
    }
    // backward: L^T x = D^-1 y
    for (int J = M.nbc - 1; J >= 0; --J) {
        double acc[kSolveCols];
#pragma unroll
        for (int c = 0; c < kSolveCols; ++c) acc[c] = 0.0;
        const int dmax = min(M.bt, M.nbc - 1 - J);
        for (int d = 1 + g; d <= dmax; d += kGroups) {
            const double *L = band + tile_off(M, J, d);
            for (int col = 0; col < TB; ++col) sT[g][r][col] = L[col * TB + r];
            __syncwarp();
            const double *x = Xp + (size_t)(J + d) * TB;
            for (int k = 0; k < TB; ++k) {
                const double l = sT[g][k][r];
#pragma unroll
                for (int c = 0; c < kSolveCols; ++c)
                    if (c < ncol) acc[c] += l * x[(size_t)c * npad + k];
            }
            __syncwarp();
        }
#pragma unroll
        for (int c = 0; c < kSolveCols; ++c) sP[g][r][c] = acc[c];
        __syncthreads();
        if (g == 0) {
            const double *Ld = band + tile_off(M, J, 0);
            for (int col = 0; col < TB; ++col) sT[0][r][col] = Ld[col * TB + r];
            __syncwarp();
            const double dinv = 1.0 / sT[0][r][r];
            double v[kSolveCols];
#pragma unroll
            for (int c = 0; c < kSolveCols; ++c) {
                double s = 0.0;
                for (int q = 0; q < kGroups; ++q) s += sP[q][r][c];
                v[c] = (c < ncol) ? Xp[(size_t)c * npad + J * TB + r] * dinv - s : 0.0;
            }
            for (int k = TB - 1; k >= 0; --k) {
                const double lkr = sT[0][k][r];
#pragma unroll
                for (int c = 0; c < kSolveCols; ++c) {
                    const double xk = __shfl_sync(0xffffffffu, v[c], k);
                    if (r < k) v[c] -= lkr * xk;
                }
            }
#pragma unroll
            for (int c = 0; c < kSolveCols; ++c)
                if (c < ncol) Xp[(size_t)c * npad + J * TB + r] = v[c];
            __syncwarp();
        }
        __syncthreads();
    }
}

// The sweeps of k_band_solve in double-float on the FP32 pipe, from the copies k_band_dfprep makes
// of the factor (off-diagonal tiles as stored, Lf, and transposed, Lb; W = L_JJ^-1 column-major,
// Wf, and row-major, Wb; D^-1).  The warps split a block row's off-diagonal tiles as in
// k_band_solve; the diagonal step is the product with W (one warp per right-hand side) instead of
// a 32-step substitution.  The solved block rows stay in a shared-memory ring of `ring` >= bt + 1
// rows; the forward sweep leaves y in X as (hi, lo) float pairs, which the backward sweep
// overwrites with the FP64 value of the solution.  Items have 1 .. kSolveCols columns (a
// template instantiation each).
template <int NC>
__device__ __forceinline__ void band_solve_df_item(const PanelMeta &M, const float2 *__restrict__ Lf,
                                                   const float2 *__restrict__ Lb, const float2 *__restrict__ Wfp,
                                                   const float2 *__restrict__ Wbp, const float2 *__restrict__ Dinv,
                                                   double *Xp, int ring, float2 *sRing, float2 *sP, float2 *sV) {
    const int npad = M.nbc * TB;
    float2 *Yp = reinterpret_cast<float2 *>(Xp);
    const int t = threadIdx.x, r = t % TB, g = t / TB;
    for (int sweep = 0; sweep < 2; ++sweep) {
        const bool fwd = sweep == 0;
        const float2 *Lt = fwd ? Lf : Lb;
        for (int s = 0; s < M.nbc; ++s) {
            const int I = fwd ? s : M.nbc - 1 - s;
            // partial products: forward sum_d L_{I,I-d} y_{I-d}; backward sum_d L_{I+d,I}^T x_{I+d}
            DF acc[NC];
#pragma unroll
            for (int c = 0; c < NC; ++c) acc[c] = DF{0.f, 0.f};
            const int dmax = min(M.bt, fwd ? I : M.nbc - 1 - I);
            for (int d = 1 + g; d <= dmax; d += kGroups) {
                const int J = fwd ? I - d : I + d;
                const float2 *T = Lt + tile_off(M, fwd ? J : I, d);
                const float2 *y = sRing + (size_t)(J % ring) * kSolveCols * TB;
#pragma unroll 4
                for (int k = 0; k < TB; ++k) {
                    const float2 l = __ldg(T + k * TB + r);
#pragma unroll
                    for (int c = 0; c < NC; ++c) {
                        const float2 v = y[c * TB + k];
                        df_acc(acc[c], l.x, l.y, v.x, v.y);
                    }
                }
            }
#pragma unroll
            for (int c = 0; c < NC; ++c) {
                const DF a = df_norm(acc[c]);
                sP[(g * kSolveCols + c) * TB + r] = make_float2(a.hi, a.lo);
            }
            __syncthreads();
            if (g < NC) {
                const int c = g;
                const size_t xi = (size_t)c * npad + (size_t)I * TB + r;
                DF v;
                if (fwd) {
                    v = df_from_double(Xp[xi]);
                } else {
                    const float2 yv = Yp[xi], di = __ldg(Dinv + M.xUnit + (size_t)I * TB + r);
                    v = df_mul(DF{yv.x, yv.y}, DF{di.x, di.y});
                }
                for (int q = 0; q < kGroups; ++q) {
                    const float2 p = sP[(q * kSolveCols + c) * TB + r];
                    v = df_sub(v, DF{p.x, p.y});
                }
                sV[c * TB + r] = make_float2(v.hi, v.lo);
                __syncwarp();
                // forward y = W v (W[r][k] at Wf[k TB + r]); backward x = W^T v (W[k][r] at Wb[k TB + r])
                const float2 *W = (fwd ? Wfp : Wbp) + (size_t)I * TT;
                DF o = {0.f, 0.f}, o2 = {0.f, 0.f};
#pragma unroll 4
                for (int k = 0; k < TB; k += 2) {
                    const float2 w0 = __ldg(W + k * TB + r), w1 = __ldg(W + (k + 1) * TB + r);
                    const float2 v0 = sV[c * TB + k], v1 = sV[c * TB + k + 1];
                    df_acc(o, w0.x, w0.y, v0.x, v0.y);
                    df_acc(o2, w1.x, w1.y, v1.x, v1.y);
                }
                o = df_add(df_norm(o), df_norm(o2));
                sRing[((size_t)(I % ring) * kSolveCols + c) * TB + r] = make_float2(o.hi, o.lo);
                if (fwd)
                    Yp[xi] = make_float2(o.hi, o.lo);
                else
                    Xp[xi] = df_to_double(o);
            }
            __syncthreads();
        }
    }
}

__global__ void __launch_bounds__(kThreads) k_band_solve_df(const PanelMeta *__restrict__ meta,
                                                            const SolveItem *__restrict__ items,
                                                            const float2 *__restrict__ Lf,
                                                            const float2 *__restrict__ Lb,
                                                            const float2 *__restrict__ Wf,
                                                            const float2 *__restrict__ Wb,
                                                            const float2 *__restrict__ Dinv, double *X, int nrhs,
                                                            int ring) {
    extern __shared__ float2 sdf[];
    float2 *sRing = sdf;                                // [ring][kSolveCols][TB]
    float2 *sP = sRing + (size_t)ring * kSolveCols * TB;  // [kGroups][kSolveCols][TB]
    float2 *sV = sP + kGroups * kSolveCols * TB;        // [kSolveCols][TB]
    const SolveItem it = items[blockIdx.x];
    const PanelMeta M = meta[it.panel];
    double *Xp = X + (size_t)M.xUnit * nrhs + (size_t)it.col0 * (M.nbc * TB);
    const float2 *Wfp = Wf + (size_t)M.xUnit * TB, *Wbp = Wb + (size_t)M.xUnit * TB;
    // the work of a group is in proportion to its columns: the item's column count picks the
    // instantiation
    switch (it.ncol) {
    case 1: band_solve_df_item<1>(M, Lf, Lb, Wfp, Wbp, Dinv, Xp, ring, sRing, sP, sV); break;
    case 2: band_solve_df_item<2>(M, Lf, Lb, Wfp, Wbp, Dinv, Xp, ring, sRing, sP, sV); break;
    case 3: band_solve_df_item<3>(M, Lf, Lb, Wfp, Wbp, Dinv, Xp, ring, sRing, sP, sV); break;
    case 4: band_solve_df_item<4>(M, Lf, Lb, Wfp, Wbp, Dinv, Xp, ring, sRing, sP, sV); break;
    case 5: band_solve_df_item<5>(M, Lf, Lb, Wfp, Wbp, Dinv, Xp, ring, sRing, sP, sV); break;
    case 6: band_solve_df_item<6>(M, Lf, Lb, Wfp, Wbp, Dinv, Xp, ring, sRing, sP, sV); break;
    case 7: band_solve_df_item<7>(M, Lf, Lb, Wfp, Wbp, Dinv, Xp, ring, sRing, sP, sV); break;
    default: band_solve_df_item<kSolveCols>(M, Lf, Lb, Wfp, Wbp, Dinv, Xp, ring, sRing, sP, sV); break;
    }
}

// ---- many right-hand sides of one large band: the time-stepping solve ----------------------
//
// k_band_solve gives a (panel, group of columns) to one CTA, which suits many small panels.  A
// single large band (a model's K_eff, factored once and solved at every time step) is instead a
// chain of nbc dependent block rows per sweep, and FP64 runs at about 1/64 of the FP32 rate: one
// CTA per column would spend tens of microseconds per block row.  So each (panel, column) gets a
// cluster of CS CTAs (2, 4 or 8, autotuned) and the arithmetic runs in double-float on the FP32 pipe:
//   * producer CTAs (ranks 1 .. CS-1), one warp per tile: for block row I they form
//     sum_{d >= 2} L_{I,I-d} y_{I-d} from the solved rows in their shared-memory ring, reduce it
//     across the CTA and store it into the leader's shared memory (distributed shared memory);
//   * the leader (rank 0) forms L_{I,I-1} y_{I-1} from the row it solved last, waits at the
//     cluster barrier, subtracts the partials from b_I and applies W_I = L_II^-1 (inverted once
//     after the factorisation): y_I = W_I (b_I - ...), pushed into every CTA's ring;
//   * one cluster barrier per block row (release / acquire orders the stores into distributed
//     shared memory); the producers run one row ahead of the leader (their tiles need rows
//     up to I - 2 only);
//   * backward sweep the same with L^T (transposed copies of the tiles and of W) on D^-1 y.
// The band is copied once into double-float tiles in the forward (column-major) and backward
// (row-major) layouts, so every tile load of a warp is 32 consecutive float2 per k.
constexpr int kCW = 8;   // warps per CTA (the CTAs per cluster, CS, is a template parameter: 2, 4 or 8)
constexpr int kPrepW = 4;  // warps per CTA of the band copy

struct CaseItem {
    int panel, col;
    int t0, t1;  // steps t0 .. t1-1 of the sweep (0 .. nbc-1 forward, nbc .. 2 nbc-1 backward)
};

// DF copies of the band: off-diagonal tiles as they are (Lf) and transposed (Lb); per block
// column W = L_JJ^-1 (unit lower) in both layouts and D^-1, one warp per block column
__global__ void k_band_dfprep(const PanelMeta *__restrict__ meta, int np, const double *__restrict__ band,
                              float2 *__restrict__ Lf, float2 *__restrict__ Lb, float2 *__restrict__ Wf,
                              float2 *__restrict__ Wb, float2 *__restrict__ Dinv) {
    __shared__ double sT[kPrepW][TB][TB + 1];
    const int w = threadIdx.x / 32, lane = threadIdx.x % 32;
    // global block-column index over all panels
    long long gJ = (long long)blockIdx.x * kPrepW + w;
    int p = 0;
    for (; p < np; ++p) {
        if (gJ < meta[p].nbc) break;
        gJ -= meta[p].nbc;
    }
    if (p >= np) return;
    const PanelMeta M = meta[p];
    const int J = (int)gJ;
    if (J >= M.nfac) {
        // a block column the (partial) factorisation left: no elimination, W = I, D^-1 = 1
        for (int d = 1; d <= M.bt && J + d < M.nbc; ++d) {
            const size_t o = tile_off(M, J, d);
            for (int e = lane; e < TT; e += 32) Lf[o + e] = Lb[o + e] = make_float2(0.f, 0.f);
        }
        const size_t ow = (size_t)M.xUnit * TB + (size_t)J * TT;
        for (int i = 0; i < TB; ++i) {
            const float2 v = make_float2(i == lane ? 1.f : 0.f, 0.f);
            Wf[ow + (size_t)lane * TB + i] = v;
            Wb[ow + (size_t)i * TB + lane] = v;
        }
        Dinv[(size_t)M.xUnit + (size_t)J * TB + lane] = make_float2(1.f, 0.f);
        return;
    }
    // each value converted once (the conversions run on the FP64 pipe), the transpose from shared
    // memory in double-float
    float2(*sF)[TB + 1] = reinterpret_cast<float2(*)[TB + 1]>(&sT[w][0][0]);
    for (int d = 1; d <= M.bt; ++d) {
        if (J + d >= M.nbc) break;
        const size_t o = tile_off(M, J, d);
        for (int e = lane; e < TT; e += 32) {
            const DF v = df_from_double(band[o + e]);
            Lf[o + e] = make_float2(v.hi, v.lo);
            sF[e % TB][e / TB] = make_float2(v.hi, v.lo);  // [row][col]
        }
        __syncwarp();
        // Lb[k * TB + r] = L[k][r]
        for (int e = lane; e < TT; e += 32) Lb[o + e] = sF[e / TB][e % TB];
        __syncwarp();
    }
    const size_t od = tile_off(M, J, 0);
    for (int e = lane; e < TT; e += 32) sT[w][e % TB][e / TB] = band[od + e];
    __syncwarp();
    // column `lane` of W: L w = e_lane by forward substitution (unit diagonal)
    double x[TB];
#pragma unroll
    for (int i = 0; i < TB; ++i) {
        double v = (i == lane) ? 1.0 : 0.0;
#pragma unroll
        for (int k = 0; k < i; ++k) v -= sT[w][i][k] * x[k];
        x[i] = v;
    }
    const size_t ow = (size_t)M.xUnit * TB + (size_t)J * TT;
    const double dl = sT[w][lane][lane];
    __syncwarp();
#pragma unroll
    for (int i = 0; i < TB; ++i) {
        const DF v = df_from_double(x[i]);  // W[i][lane]
        Wb[ow + (size_t)i * TB + lane] = make_float2(v.hi, v.lo);  // row-major: W[i][k] at i*TB + k
        sF[i][lane] = make_float2(v.hi, v.lo);
    }
    __syncwarp();
    // column-major (W[i][k] at k*TB + i) through shared memory, so the stores are coalesced
#pragma unroll 4
    for (int k = 0; k < TB; ++k) Wf[ow + (size_t)k * TB + lane] = sF[lane][k];
    const DF dv = df_from_double(1.0 / dl);
    Dinv[(size_t)M.xUnit + (size_t)J * TB + lane] = make_float2(dv.hi, dv.lo);
}

__device__ __forceinline__ void cluster_barrier() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n" ::: "memory");
    asm volatile("barrier.cluster.wait.acquire.aligned;\n" ::: "memory");
}


// sum of v[0 .. K-1] pairwise (log2 K dependent additions instead of K - 1)
template <int K> __device__ __forceinline__ DF df_tree_sum(DF (&v)[K]) {
#pragma unroll
    for (int st = 1; st < K; st *= 2)
#pragma unroll
        for (int i = 0; i + st < K; i += 2 * st) v[i] = df_add(v[i], v[i + st]);
    return v[0];
}

// acc[r] += sum_{k in [k0, k1)} T[k * TB + r] v[k] (T a DF tile in global memory, v in shared)
__device__ __forceinline__ void df_tile_rows(DF &acc, const float2 *__restrict__ T, const float2 *v, int r, int k0,
                                             int k1) {
    DF a2 = {0.f, 0.f};
    int k = k0;
    for (; k + 1 < k1; k += 2) {
        const float2 l0 = __ldg(T + k * TB + r), l1 = __ldg(T + (k + 1) * TB + r);
        const float2 y0 = v[k], y1 = v[k + 1];
        df_acc(acc, l0.x, l0.y, y0.x, y0.y);
        df_acc(a2, l1.x, l1.y, y1.x, y1.y);
    }
    if (k < k1) {
        const float2 l0 = __ldg(T + k * TB + r);
        const float2 y0 = v[k];
        df_acc(acc, l0.x, l0.y, y0.x, y0.y);
    }
    acc = df_add(df_norm(acc), df_norm(a2));
}

template <int CS>
__global__ void __launch_bounds__(kCW * 32, 1) k_band_solve_cases(const PanelMeta *__restrict__ meta,
                                                               const CaseItem *__restrict__ items,
                                                               const float2 *__restrict__ Lf,
                                                               const float2 *__restrict__ Lb,
                                                               const float2 *__restrict__ Wf,
                                                               const float2 *__restrict__ Wb,
                                                               const float2 *__restrict__ Dinv, double *X, int nrhs,
                                                               int ring) {
    constexpr int kProdWarps = (CS - 1) * kCW;
    cg::cluster_group cl = cg::this_cluster();
    const int rank = (int)cl.block_rank();
    extern __shared__ float2 smf[];
    float2 *sRing = smf;                           // [ring][TB]: solved rows
    float2 *sRed = sRing + (size_t)ring * TB;      // [kCW][TB]: per-warp partials
    float2 *sPart = sRed + kCW * TB;               // [2][CS][TB]: CTA partials (leader)
    float2 *sV = sPart + 2 * CS * TB;             // [TB]
    const CaseItem it = items[blockIdx.x / CS];
    const PanelMeta M = meta[it.panel];
    const int w = threadIdx.x / 32, r = threadIdx.x % 32;
    const int nbc = M.nbc, bt = M.bt;
    double *Xp = X + (size_t)M.xUnit * nrhs + (size_t)it.col * nbc * TB;
    const size_t wOff = (size_t)M.xUnit * TB;
    float2 *leaderPart = cl.map_shared_rank(sPart, 0);
    // step t = 0 .. 2 nbc - 1: forward rows I = t, then backward rows I = 2 nbc - 1 - t
    auto rowOf = [&](int t) { return t < nbc ? t : 2 * nbc - 1 - t; };
    // tiles below (forward) or right of (backward) the row that exist: min(bt, I) / min(bt, nbc - 1 - I)
    auto dmaxOf = [&](int t) { return t < nbc ? min(bt, t) : min(bt, t - nbc); };
    // tile d of step t: forward L_{I,I-d} = tile (I-d, d) of Lf; backward L_{I+d,I}^T = tile (I, d) of Lb
    auto tileOf = [&](int t, int d) {
        const int I = rowOf(t);
        return t < nbc ? Lf + tile_off(M, I - d, d) : Lb + tile_off(M, I, d);
    };
    auto srcOf = [&](int t, int d) { return t < nbc ? rowOf(t) - d : rowOf(t) + d; };
    // Each warp's next tile is loaded into registers one step ahead, so the loads are in flight
    // during the cluster barrier and the leader's part of the step: producers the first tile of
    // the warp (pf, the lane's row of it), the leader its four columns of L_{I,I+-1} (pl) and of
    // W (pw), and warp 0 the right-hand side (pb) and D^-1 (pd).
    const int d0 = 2 + (rank - 1) * kCW + w;
    float2 pf[TB], pl[4], pw[4], pd = make_float2(0.f, 0.f);
    double pb = 0.0;
    const int t0 = it.t0, t1 = it.t1;
    auto prefetch = [&](int t) {
        if (t >= t1) return;
        const int dm = dmaxOf(t), I = rowOf(t);
        if (rank > 0) {
            if (d0 <= dm) {
                const float2 *T = tileOf(t, d0);
#pragma unroll
                for (int k = 0; k < TB; ++k) pf[k] = __ldg(T + k * TB + r);
            }
        } else {
            if (dm >= 1) {
                const float2 *T = tileOf(t, 1);
#pragma unroll
                for (int k = 0; k < 4; ++k) pl[k] = __ldg(T + (4 * w + k) * TB + r);
            }
            const float2 *Wt = (t < nbc ? Wf : Wb) + wOff + (size_t)I * TT;
#pragma unroll
            for (int k = 0; k < 4; ++k) pw[k] = __ldg(Wt + (4 * w + k) * TB + r);
            if (w == 0) {
                pb = Xp[(size_t)I * TB + r];
                if (t >= nbc) pd = __ldg(Dinv + M.xUnit + (size_t)I * TB + r);
            }
        }
    };
    // a backward sweep that starts below the last row (the rows after it solved already, in X):
    // those rows into every CTA's ring
    if (t0 > nbc) {
        const int I0 = 2 * nbc - 1 - t0;
        for (int R = I0 + 1 + w; R <= min(nbc - 1, I0 + bt); R += kCW) {
            const DF v = df_from_double(Xp[(size_t)R * TB + r]);
            sRing[(size_t)(R % ring) * TB + r] = make_float2(v.hi, v.lo);
        }
    }
    prefetch(t0);
    for (int t = t0; t < t1; ++t) {
        const int I = rowOf(t), dmax = dmaxOf(t), q = t < nbc ? t : t - nbc;
        __syncthreads();  // the leader's last row is in its ring
        if (rank > 0) {
            DF acc = {0.f, 0.f}, a2 = {0.f, 0.f};
            if (d0 <= dmax) {
                const float2 *v = sRing + (size_t)(srcOf(t, d0) % ring) * TB;
#pragma unroll
                for (int k = 0; k < TB; k += 2) {
                    const float2 y0 = v[k], y1 = v[k + 1];
                    df_acc(acc, pf[k].x, pf[k].y, y0.x, y0.y);
                    df_acc(a2, pf[k + 1].x, pf[k + 1].y, y1.x, y1.y);
                }
                acc = df_add(df_norm(acc), df_norm(a2));
            }
            for (int d = d0 + kProdWarps; d <= dmax; d += kProdWarps)
                df_tile_rows(acc, tileOf(t, d), sRing + (size_t)(srcOf(t, d) % ring) * TB, r, 0, TB);
            prefetch(t + 1);
            sRed[w * TB + r] = make_float2(acc.hi, acc.lo);
            __syncthreads();
            if (w == 0) {
                DF pv[kCW];
#pragma unroll
                for (int k = 0; k < kCW; ++k) pv[k] = DF{sRed[k * TB + r].x, sRed[k * TB + r].y};
                const DF s = df_tree_sum(pv);
                leaderPart[((q & 1) * CS + rank) * TB + r] = make_float2(s.hi, s.lo);
            }
            cluster_barrier();
        } else {
            // L_{I,I+-1} times the row solved last, split over the warps by k
            DF acc = {0.f, 0.f};
            if (dmax >= 1) {
                const float2 *v = sRing + (size_t)(srcOf(t, 1) % ring) * TB + 4 * w;
#pragma unroll
                for (int k = 0; k < 4; ++k) df_acc(acc, pl[k].x, pl[k].y, v[k].x, v[k].y);
                acc = df_norm(acc);
            }
            sRed[w * TB + r] = make_float2(acc.hi, acc.lo);
            cluster_barrier();
            if (w == 0) {
                DF v = df_from_double(pb);
                if (t >= nbc) v = df_mul(v, DF{pd.x, pd.y});
                DF pv[kCW + CS];  // the leader's warps' partials, then the producers' (slot CS: zero)
#pragma unroll
                for (int k = 0; k < kCW; ++k) pv[k] = DF{sRed[k * TB + r].x, sRed[k * TB + r].y};
                pv[kCW] = DF{0.f, 0.f};
#pragma unroll
                for (int c = 1; c < CS; ++c) {
                    const float2 pc = sPart[((q & 1) * CS + c) * TB + r];
                    pv[kCW + c] = DF{pc.x, pc.y};
                }
                v = df_sub(v, df_tree_sum(pv));
                sV[r] = make_float2(v.hi, v.lo);
            }
            __syncthreads();
            // y_I = W v (forward) or x_I = W^T v (backward), split over the warps by k
            DF a = {0.f, 0.f};
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const float2 vk = sV[4 * w + k];
                df_acc(a, pw[k].x, pw[k].y, vk.x, vk.y);
            }
            a = df_norm(a);
            sRed[w * TB + r] = make_float2(a.hi, a.lo);
            __syncthreads();
            if (w == 0) {
                DF pv[kCW];
#pragma unroll
                for (int k = 0; k < kCW; ++k) pv[k] = DF{sRed[k * TB + r].x, sRed[k * TB + r].y};
                const DF y = df_tree_sum(pv);
                const float2 yv = make_float2(y.hi, y.lo);
                const size_t slot = (size_t)(I % ring) * TB + r;
                for (int c = 0; c < CS; ++c) cl.map_shared_rank(sRing, c)[slot] = yv;
                Xp[(size_t)I * TB + r] = df_to_double(y);
            }
            prefetch(t + 1);  // after the row's store: the first backward row reads it back
        }
        // the forward sweep's last rows are pushed before the backward sweep, and every row
        // before any CTA exits
        if (t == nbc - 1 || t == t1 - 1) cluster_barrier();
    }
}

// internal-layout columns (nrhs x n) <-> the padded panel layout
__global__ void k_vec_add(long long n, const double *__restrict__ x, double *__restrict__ y) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] += x[i];
}

__global__ void k_panel_move(int n, int dpn, int nrhs, double *__restrict__ vec, const int *__restrict__ panelOf,
                             const int *__restrict__ pos, const PanelMeta *__restrict__ meta, double *__restrict__ X,
                             int toPanel) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)n * nrhs) return;
    const int c = (int)(t / n), i = (int)(t % n), r = i / dpn, a = i % dpn;
    const PanelMeta &M = meta[panelOf[r]];
    const size_t xi = (size_t)M.xUnit * nrhs + (size_t)c * M.nbc * TB + (size_t)pos[r] * dpn + a;
    if (toPanel)
        X[xi] = vec[t];
    else
        vec[t] = X[xi];
}

// ---- twisted many-column solve of one panel ----------------------------------------------------
// The panel's band A (n DOF, nbc block rows, bt tiles below the diagonal) is split at block row K
// into a top panel T = A[0 : K+m, 0 : K+m] and a bottom panel B = A[K : nbc, K : nbc] taken in
// reversed order (band position ig -> rev - ig, padded with unit rows at its start), overlapping in the
// window of m = bt block rows K .. K+m-1.  T and B are factored (LDL^T) up to the window only, so
// their window tiles hold the Schur complements S_T and S_B of their outer parts; the window
// matrix S = S_T + S_B - A_window (B's part reversed) is factored as a third panel.  A solve is
// then: forward sweeps of T and B (the window's tiles zero and its W the identity, so the window
// rows come out as c_T = b_w - L_wT y_T and c_B), c = c_T + c_B - b_w, S x_w = c, and backward
// sweeps of T and B from the window outwards: two chains of about nbc / 2 block rows each way
// instead of one of nbc (the twisted factorisation of a band, assembled from Schur complements).
struct TwistGeom {
    int n, dpn, K32, nT, nbB32;  // DOF, DOF per node, window start, top rows, bottom padded rows
    int rev;                     // B's row of band position ig >= K32: rev - ig (rev = nbB32 + K32 - 1)
};

__device__ __forceinline__ double *tw_at(double *band, const PanelMeta &M, int row, int col) {  // row >= col
    const int J = col / TB;
    return band + tile_off(M, J, row / TB - J) + (col % TB) * TB + (row % TB);
}

// BSR entries of K (and, with penalty, the C^T C entries) into T and B
__global__ void k_tw_fill(int nb, TwistGeom G, const int *__restrict__ bRow, const int *__restrict__ bCol,
                          const double *__restrict__ K, const int *__restrict__ pos, const PanelMeta *__restrict__ meta,
                          double *__restrict__ band) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const int bs = G.dpn * G.dpn;
    if (t >= (long long)nb * bs) return;
    const int b = (int)(t / bs), q = (int)(t % bs), a = q / G.dpn, c = q % G.dpn;
    const int i = pos[bRow[b]] * G.dpn + a, j = pos[bCol[b]] * G.dpn + c;
    if (j > i) return;
    const double v = K[(size_t)b * bs + q];
    if (i < G.nT) *tw_at(band, meta[0], i, j) = v;
    if (j >= G.K32) *tw_at(band, meta[1], G.rev - j, G.rev - i) = v;
}

__global__ void k_tw_pen(int cnt, TwistGeom G, const int *__restrict__ pi, const int *__restrict__ pj,
                         const double *__restrict__ pv, const int *__restrict__ pos, const PanelMeta *__restrict__ meta,
                         double *__restrict__ band) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= cnt) return;
    const int i = pos[pi[t] / G.dpn] * G.dpn + pi[t] % G.dpn, j = pos[pj[t] / G.dpn] * G.dpn + pj[t] % G.dpn;
    if (j > i) return;
    if (i < G.nT) *tw_at(band, meta[0], i, j) += pv[t];
    if (j >= G.K32) *tw_at(band, meta[1], G.rev - j, G.rev - i) += pv[t];
}

// unit diagonal on B's leading padding rows
__global__ void k_tw_pad(TwistGeom G, const PanelMeta *__restrict__ meta, double *__restrict__ band) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < G.nbB32 - (G.n - G.K32)) *tw_at(band, meta[1], i, i) = 1.0;
}

// the window of T before its factorisation (A_window) into Aw (window panel layout), or, with
// assemble, S = S_T + S_B - A_window into the window panel: one thread per lower entry
__global__ void k_tw_window(TwistGeom G, int w, const PanelMeta *__restrict__ meta, double *__restrict__ band,
                            double *__restrict__ Aw, int assemble) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)w * w) return;
    const int s1 = (int)(t / w), s2 = (int)(t % w);
    if (s2 > s1) return;
    PanelMeta Ma = meta[2];  // the window panel's tile layout, from the start of Aw
    Ma.band = 0;
    double *pa = tw_at(Aw, Ma, s1, s2);
    const double vt = *tw_at(band, meta[0], G.K32 + s1, G.K32 + s2);
    if (!assemble) {
        *pa = vt;
        return;
    }
    const double vb = *tw_at(band, meta[1], G.nbB32 - 1 - s2, G.nbB32 - 1 - s1);
    *tw_at(band, meta[2], s1, s2) = vt + vb - *pa;
}

// internal-layout columns -> T, B and the window's b_w (mode 0); c_w = c_T + c_B - b_w (mode 1);
// x_w -> T and B (mode 2); T, window, B -> internal layout (mode 3)
__global__ void k_tw_move(int nc, TwistGeom G, int w, double *__restrict__ vec, const int *__restrict__ pos,
                          const PanelMeta *__restrict__ meta, double *__restrict__ X, int mode) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const PanelMeta &T = meta[0], &B = meta[1], &S = meta[2];
    const int len = (mode == 1 || mode == 2) ? w : G.n;
    if (t >= (long long)len * nc) return;
    const int c = (int)(t / len), i = (int)(t % len);
    double *XT = X + (size_t)T.xUnit * nc + (size_t)c * T.nbc * TB;
    double *XB = X + (size_t)B.xUnit * nc + (size_t)c * B.nbc * TB;
    double *XS = X + (size_t)S.xUnit * nc + (size_t)c * S.nbc * TB;
    if (mode == 1) {
        XS[i] = XT[G.K32 + i] + XB[G.nbB32 - 1 - i] - XS[i];
        return;
    }
    if (mode == 2) {
        XT[G.K32 + i] = XS[i];
        XB[G.nbB32 - 1 - i] = XS[i];
        return;
    }
    const int ig = pos[i / G.dpn] * G.dpn + i % G.dpn;
    double *v = vec + (size_t)c * G.n + i;
    if (mode == 0) {
        if (ig < G.nT) XT[ig] = *v;
        if (ig >= G.K32) XB[G.rev - ig] = *v;
        if (ig >= G.K32 && ig < G.nT) XS[ig - G.K32] = *v;
    } else {
        *v = ig < G.K32 ? XT[ig] : (ig < G.nT ? XS[ig - G.K32] : XB[G.rev - ig]);
    }
}

constexpr size_t kSolveSmem = sizeof(double) * (kGroups * TB * (TB + 1) + kGroups * TB * (kSolveCols + 1));

// connected components, orderings, bandwidths, storage and the cluster schedule
int plan_build(astro_ctx *ctx, PanelPlan &L, int cs) {
    const AstroPrep &P = ctx->P;
    const int N = P.N, dpn = P.dpn;
    // union-find over nodes (1-based ids) through the elements
    std::vector<int> par(N + 1);
    std::iota(par.begin(), par.end(), 0);
    auto find = [&](int x) {
        while (par[x] != x) x = par[x] = par[par[x]];
        return x;
    };
    for (int e = 0; e < P.E; ++e) {
        int first = 0;
        for (int k = 0; k < 8; ++k) {
            const int nd = ctx->elist[8 * (size_t)e + k];
            if (nd < 1) continue;
            if (!first) {
                first = nd;
                continue;
            }
            const int a = find(first), b = find(nd);
            if (a != b) par[std::max(a, b)] = std::min(a, b);
        }
    }
    std::vector<int> compId(N + 1, -1), roots;
    for (int nd = 1; nd <= N; ++nd) {
        const int r = find(nd);
        if (compId[r] < 0) {
            compId[r] = (int)roots.size();
            roots.push_back(r);
        }
        compId[nd] = compId[r];
    }
    const int np = (int)roots.size();
    std::vector<std::vector<int>> members(np);
    for (int nd = 1; nd <= N; ++nd) members[compId[nd]].push_back(nd);
    L.np = np;
    L.panelOf.assign(N, 0);
    L.pos.assign(N, 0);
    for (int p = 0; p < np; ++p) {
        auto &mb = members[p];
        double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
        for (int nd : mb)
            for (int d = 0; d < 3; ++d) {
                lo[d] = std::min(lo[d], ctx->nodes[3 * (size_t)(nd - 1) + d]);
                hi[d] = std::max(hi[d], ctx->nodes[3 * (size_t)(nd - 1) + d]);
            }
        int ax[3] = {0, 1, 2};
        std::stable_sort(ax, ax + 3, [&](int a, int b) { return hi[a] - lo[a] > hi[b] - lo[b]; });
        std::stable_sort(mb.begin(), mb.end(), [&](int a, int b) {
            for (int k = 0; k < 3; ++k) {
                const double xa = ctx->nodes[3 * (size_t)(a - 1) + ax[k]], xb = ctx->nodes[3 * (size_t)(b - 1) + ax[k]];
                if (xa != xb) return xa < xb;
            }
            return a < b;
        });
        for (int k = 0; k < (int)mb.size(); ++k) {
            const int r = P.currentRank[mb[k]] - 1;
            L.panelOf[r] = p;
            L.pos[r] = k;
        }
    }
    // node bandwidth of each panel from the block pattern and the penalty couplings
    std::vector<int> bwn(np, 0);
    for (int r = 0; r < N; ++r)
        for (int q = P.bRowPtr[r]; q < P.bRowPtr[r + 1]; ++q) {
            const int c = P.bCol[q];
            if (L.panelOf[c] != L.panelOf[r]) return set_err(ctx, ASTRO_ERR_ARG, "panels: coupled components");
            bwn[L.panelOf[r]] = std::max(bwn[L.panelOf[r]], std::abs(L.pos[r] - L.pos[c]));
        }
    for (size_t k = 0; k < ctx->penI.size(); ++k) {
        const int ri = ctx->penI[k] / dpn, rj = ctx->penJ[k] / dpn;
        if (L.panelOf[ri] != L.panelOf[rj])
            return set_err(ctx, ASTRO_ERR_UNSUPPORTED, "panels: a constraint couples two panels");
        bwn[L.panelOf[ri]] = std::max(bwn[L.panelOf[ri]], std::abs(L.pos[ri] - L.pos[rj]));
    }
    L.meta.assign(np, PanelMeta{});
    L.work.assign(np, 0.0);
    long long band = 0, xr = 0;
    L.maxBw = 0;
    for (int p = 0; p < np; ++p) {
        PanelMeta &M = L.meta[p];
        M.n = (int)members[p].size() * dpn;
        M.nbc = (M.n + TB - 1) / TB;
        const int bw = bwn[p] * dpn + dpn - 1;
        L.maxBw = std::max(L.maxBw, bw);
        M.bt = (bw + TB - 1) / TB;
        M.band = band;
        M.xUnit = xr;
        M.nfac = M.nbc;
        band += (long long)M.nbc * (M.bt + 1) * TT;
        xr += (long long)M.nbc * TB;
        L.work[p] = (double)M.nbc * (0.5 * M.bt * (M.bt + 1) + 2.0);
    }
    L.bandDoubles = band;
    L.xRows = xr;
    // clusters: as many as fit at once, panels by longest processing time first
    L.cs = cs;
    int maxClusters = 0;
    {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(cs * 64);
        cfg.blockDim = dim3(kThreads);
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = cs;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        // workers as resident clusters of the variants without dynamic shared memory (FP64 and
        // mma.sync updates); the tcgen05 variant's shared memory fits two CTAs per SM, so its
        // surplus clusters wait for the resident ones (and at most two CTAs per SM hold tensor
        // memory: the allocation never waits)
        cudaFuncSetAttribute(k_band_ldl<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem);
        if (cudaOccupancyMaxActiveClusters(&maxClusters, k_band_ldl<1>, &cfg) != cudaSuccess) {
            cudaGetLastError();
            maxClusters = 0;
        }
    }
    if (maxClusters < 1) {
        int sms = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
        maxClusters = std::max(1, sms / cs);
    }
    L.workers = std::max(1, std::min(np, maxClusters));
    std::vector<int> order(np);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return L.work[a] > L.work[b]; });
    std::vector<double> load(L.workers, 0.0);
    std::vector<std::vector<int>> lists(L.workers);
    for (int p : order) {
        const int w = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        lists[w].push_back(p);
        load[w] += L.work[p];
    }
    L.sched.clear();
    L.schedPtr.assign(1, 0);
    for (auto &l : lists) {
        L.sched.insert(L.sched.end(), l.begin(), l.end());
        L.schedPtr.push_back((int)L.sched.size());
    }
    // slice scratch of the tensor-core trailing update, one block column's tiles per worker
    L.maxBt = 0;
    for (const PanelMeta &M : L.meta) L.maxBt = std::max(L.maxBt, M.bt);
    L.sliceStride = 2LL * std::max(L.maxBt, 1) * kSlices * TT;
    L.expStride = 2 * std::max(L.maxBt, 1) * TB;
    int rc;
    if ((rc = dev_alloc(ctx, L.d_slices, sizeof(uint16_t) * (size_t)L.sliceStride * L.workers)) ||
        (rc = dev_alloc(ctx, L.d_sexp, sizeof(int) * (size_t)L.expStride * L.workers)))
        return rc;
    if ((rc = upload(ctx, L.d_meta, L.meta.data(), sizeof(PanelMeta) * np)) ||
        (rc = upload(ctx, L.d_sched, L.sched.data(), sizeof(int) * L.sched.size())) ||
        (rc = upload(ctx, L.d_schedPtr, L.schedPtr.data(), sizeof(int) * L.schedPtr.size())) ||
        (rc = upload(ctx, L.d_panelOf, L.panelOf.data(), sizeof(int) * N)) ||
        (rc = upload(ctx, L.d_pos, L.pos.data(), sizeof(int) * N)) ||
        (rc = dev_alloc(ctx, L.d_status, sizeof(int))))
        return rc;
    return ASTRO_OK;
}

void plan_free(PanelPlan *L) {
    DevBuf *b[] = {&L->d_meta,  &L->d_sched, &L->d_schedPtr, &L->d_panelOf, &L->d_pos,  &L->d_band,
                   &L->d_status, &L->d_penI, &L->d_penJ,     &L->d_penV,    &L->d_slices, &L->d_sexp,
                   &L->d_Lf,    &L->d_Lb,    &L->d_Wf,       &L->d_Wb,      &L->d_Dinv,  &L->d_items,
                   &L->d_X,     &L->d_twMeta, &L->d_twBand, &L->d_twAw,  &L->d_twSched, &L->d_twSchedPtr,
                   &L->d_twStatus, &L->d_twLf, &L->d_twLb, &L->d_twWf, &L->d_twWb, &L->d_twDinv,
                   &L->d_twItems, &L->d_twX, &L->d_sRef, &L->d_sVec, &L->d_sRes, &L->d_sBi, &L->d_sX,
                   &L->d_sItems};
    for (DevBuf *x : b) dev_free(*x);
}

void fill_info(const PanelPlan &L, astro_panels_info *info) {
    if (!info) return;
    info->num_panels = L.np;
    info->max_bandwidth = L.maxBw;
    info->band_bytes = L.bandDoubles * (long long)sizeof(double);
    info->cluster_size = L.cs;
    info->workers = L.workers;
    info->factor_seconds = L.factorSeconds;
}

}  // namespace

void panels_release(astro_ctx *ctx) {
    if (!ctx->panels) return;
    PanelPlan *L = static_cast<PanelPlan *>(ctx->panels);
    plan_free(L);
    delete L;
    ctx->panels = nullptr;
}

// The plan (orderings, storage, schedule) and, with factor, the band LDL^T of every panel; without
// it only the plan and the constraint terms, for a caller that factors in its own layout
// (the twisted many-column solve).
int panels_factor_impl(astro_ctx *ctx, int32_t cluster_size, astro_panels_info *info, int factor) {
    if (!ctx) return ASTRO_ERR_ARG;
    if (cluster_size == 0) cluster_size = ctx->tunePanelCluster ? ctx->tunePanelCluster : 8;  // autotuned or 8
    if (cluster_size != 1 && cluster_size != 2 && cluster_size != 4 && cluster_size != 8)
        return set_err(ctx, ASTRO_ERR_ARG, "panels: cluster_size must be 1, 2, 4 or 8");
    if (!ctx->haveK64) return set_err(ctx, ASTRO_ERR_STATE, "panels: FP64 stiffness not assembled");
    if (ctx->P.mpcDim > 0 && !ctx->mpcScaled)
        return set_err(ctx, ASTRO_ERR_STATE, "panels: constraints not scaled (astro_scale_mpc)");
    PanelPlan *L = static_cast<PanelPlan *>(ctx->panels);
    if (L && L->cs != cluster_size) {
        panels_release(ctx);
        L = nullptr;
    }
    int rc;
    if (!L) {
        L = new PanelPlan();
        ctx->panels = L;
        if ((rc = plan_build(ctx, *L, cluster_size))) {
            panels_release(ctx);
            return rc;
        }
    }
    const auto t0 = std::chrono::steady_clock::now();
    cudaStream_t s = ctx->stream;
    const AstroPrep &P = ctx->P;
    if (L->penVersion != ctx->penVersion) {
        L->penCount = (int)ctx->penI.size();
        if (L->penCount &&
            ((rc = upload(ctx, L->d_penI, ctx->penI.data(), sizeof(int) * L->penCount)) ||
             (rc = upload(ctx, L->d_penJ, ctx->penJ.data(), sizeof(int) * L->penCount)) ||
             (rc = upload(ctx, L->d_penV, ctx->penV.data(), sizeof(double) * L->penCount))))
            return rc;
    }
    if (!factor) {
        L->kVersion = ctx->k64Version;
        L->penVersion = ctx->penVersion;
        L->factored = 0;
        L->factorGen++;
        fill_info(*L, info);
        return ASTRO_OK;
    }
    if (!L->d_band.p && (rc = dev_alloc(ctx, L->d_band, sizeof(double) * (size_t)L->bandDoubles))) return rc;
    CK(cudaMemsetAsync(L->d_band.p, 0, sizeof(double) * (size_t)L->bandDoubles, s));
    CK(cudaMemsetAsync(L->d_status.p, 0, sizeof(int), s));
    const long long fillN = (long long)P.nb * P.dpn * P.dpn;
    k_band_fill<<<(unsigned)((fillN + 255) / 256), 256, 0, s>>>(
        P.nb, P.dpn, dptr<int>(ctx->d_bRow), dptr<int>(ctx->d_bCol), dptr<double>(ctx->d_K64),
        dptr<int>(L->d_panelOf), dptr<int>(L->d_pos), dptr<PanelMeta>(L->d_meta), dptr<double>(L->d_band));
    if (L->penCount)
        k_band_pen<<<(L->penCount + 255) / 256, 256, 0, s>>>(
            L->penCount, P.dpn, dptr<int>(L->d_penI), dptr<int>(L->d_penJ), dptr<double>(L->d_penV),
            dptr<int>(L->d_panelOf), dptr<int>(L->d_pos), dptr<PanelMeta>(L->d_meta), dptr<double>(L->d_band));
    k_band_pad<<<L->np, TB, 0, s>>>(dptr<PanelMeta>(L->d_meta), dptr<double>(L->d_band));
    if ((rc = cuda_check(ctx, cudaGetLastError(), "panel band fill"))) return rc;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(L->workers * L->cs);
    cfg.blockDim = dim3(kThreads);
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = L->cs;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    if (ctx->bandFp64Update == 1) {
        CK(cudaLaunchKernelEx(&cfg, k_band_ldl<0>, (const PanelMeta *)dptr<PanelMeta>(L->d_meta),
                              (const int *)dptr<int>(L->d_sched), (const int *)dptr<int>(L->d_schedPtr),
                              dptr<double>(L->d_band), dptr<int>(L->d_status), (uint16_t *)nullptr, (int *)nullptr,
                              0LL, 0));
    } else if (ctx->bandFp64Update == 3) {
        // the band in double-float for the factorisation, FP64 again after it
        const long long nb = L->bandDoubles;
        const unsigned cgr = (unsigned)std::min<long long>((nb + 255) / 256, 152LL * 16);
        k_band_df_convert<<<cgr, 256, 0, s>>>(nb, dptr<double>(L->d_band), 1);
        CK(cudaLaunchKernelEx(&cfg, k_band_ldl_df, (const PanelMeta *)dptr<PanelMeta>(L->d_meta),
                              (const int *)dptr<int>(L->d_sched), (const int *)dptr<int>(L->d_schedPtr),
                              dptr<float2>(L->d_band), dptr<int>(L->d_status), dptr<float2>(L->d_slices),
                              L->sliceStride / 4));
        k_band_df_convert<<<cgr, 256, 0, s>>>(nb, dptr<double>(L->d_band), 0);
    } else if (ctx->bandFp64Update == 2) {
        CK(cudaLaunchKernelEx(&cfg, k_band_ldl<1>, (const PanelMeta *)dptr<PanelMeta>(L->d_meta),
                              (const int *)dptr<int>(L->d_sched), (const int *)dptr<int>(L->d_schedPtr),
                              dptr<double>(L->d_band), dptr<int>(L->d_status), dptr<uint16_t>(L->d_slices),
                              dptr<int>(L->d_sexp), L->sliceStride, L->expStride));
    } else {
        cfg.dynamicSmemBytes = kTcSmem;
        CK(cudaLaunchKernelEx(&cfg, k_band_ldl<2>, (const PanelMeta *)dptr<PanelMeta>(L->d_meta),
                              (const int *)dptr<int>(L->d_sched), (const int *)dptr<int>(L->d_schedPtr),
                              dptr<double>(L->d_band), dptr<int>(L->d_status), dptr<uint16_t>(L->d_slices),
                              dptr<int>(L->d_sexp), L->sliceStride, L->expStride));
    }
    int status = 0;
    CK(cudaMemcpyAsync(&status, L->d_status.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    L->factorSeconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    L->kVersion = ctx->k64Version;
    L->penVersion = ctx->penVersion;
    L->factored = status == 0;
    L->factorGen++;
    fill_info(*L, info);
    if (status < 0)
        return set_err(ctx, ASTRO_ERR_STATE, "panels: the tensor-core MMAs of the trailing update did not complete");
    if (status) return set_err(ctx, ASTRO_ERR_PIVOT, "panels: zero or non-finite pivot in panel " + std::to_string(status - 1));
    return ASTRO_OK;
}

extern "C" int astro_panels_factor(astro_ctx *ctx, int32_t cluster_size, astro_panels_info *info) {
    return panels_factor_impl(ctx, cluster_size, info, 1);
}

// A device buffer of at least `bytes`, reallocated only to grow.
static int grow(astro_ctx *ctx, DevBuf &b, size_t bytes) {
    return b.p && b.bytes >= bytes ? ASTRO_OK : dev_alloc(ctx, b, bytes);
}

// The double-float copies of the current factorisation (k_band_dfprep), made once per factor.
static int panels_df_copies(astro_ctx *ctx, PanelPlan *L) {
    if (L->dfGen == L->factorGen) return ASTRO_OK;
    int rc;
    const size_t nb = (size_t)L->bandDoubles, nd = (size_t)L->xRows;
    if ((rc = grow(ctx, L->d_Lf, sizeof(float2) * nb)) || (rc = grow(ctx, L->d_Lb, sizeof(float2) * nb)) ||
        (rc = grow(ctx, L->d_Wf, sizeof(float2) * nd * TB)) || (rc = grow(ctx, L->d_Wb, sizeof(float2) * nd * TB)) ||
        (rc = grow(ctx, L->d_Dinv, sizeof(float2) * nd)))
        return rc;
    long long cols = 0;
    for (const PanelMeta &M : L->meta) cols += M.nbc;
    k_band_dfprep<<<(unsigned)((cols + kPrepW - 1) / kPrepW), kPrepW * 32, 0, ctx->stream>>>(
        dptr<PanelMeta>(L->d_meta), L->np, dptr<double>(L->d_band), dptr<float2>(L->d_Lf), dptr<float2>(L->d_Lb),
        dptr<float2>(L->d_Wf), dptr<float2>(L->d_Wb), dptr<float2>(L->d_Dinv));
    if ((rc = cuda_check(ctx, cudaGetLastError(), "band double-float copy"))) return rc;
    L->dfGen = L->factorGen;
    return ASTRO_OK;
}

static int panels_solve_dev(astro_ctx *ctx, PanelPlan *L, int nrhs, double *d_vec) {
    const AstroPrep &P = ctx->P;
    cudaStream_t s = ctx->stream;
    int rc;
    const size_t xs = (size_t)L->xRows * nrhs;
    DevBuf &X = L->d_sX;
    if ((rc = grow(ctx, X, sizeof(double) * xs))) return rc;
    CK(cudaMemsetAsync(X.p, 0, sizeof(double) * xs, s));
    const long long mv = (long long)P.n * nrhs;
    const unsigned mg = (unsigned)((mv + 255) / 256);
    k_panel_move<<<mg, 256, 0, s>>>(P.n, P.dpn, nrhs, d_vec, dptr<int>(L->d_panelOf), dptr<int>(L->d_pos),
                                    dptr<PanelMeta>(L->d_meta), dptr<double>(X), 1);
    // one item per (panel, group of right-hand sides), the largest panels first
    const int groups = (nrhs + kSolveCols - 1) / kSolveCols;
    std::vector<int> order(L->np);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        return (double)L->meta[a].n * (L->meta[a].bt + 1) > (double)L->meta[b].n * (L->meta[b].bt + 1);
    });
    std::vector<SolveItem> items;
    for (int p : order) {
        int c0 = 0;
        for (int gidx = 0; gidx < groups; ++gidx) {
            const int nc = nrhs / groups + (gidx < nrhs % groups ? 1 : 0);
            items.push_back({p, c0, nc, 0});
            c0 += nc;
        }
    }
    DevBuf &dItems = L->d_sItems;
    if ((rc = grow(ctx, dItems, sizeof(SolveItem) * items.size()))) return rc;
    CK(cudaMemcpyAsync(dItems.p, items.data(), sizeof(SolveItem) * items.size(), cudaMemcpyHostToDevice, s));
    if (ctx->panelsSolve == 1) {
        CK(cudaFuncSetAttribute(k_band_solve, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSolveSmem));
        k_band_solve<<<(unsigned)items.size(), kThreads, kSolveSmem, s>>>(
            dptr<PanelMeta>(L->d_meta), dptr<SolveItem>(dItems), dptr<double>(L->d_band), dptr<double>(X), nrhs);
    } else {
        if ((rc = panels_df_copies(ctx, L))) return rc;
        const int ring = L->maxBt + 1;
        const size_t smem = sizeof(float2) * kSolveCols * TB * ((size_t)ring + kGroups + 1);
        CK(cudaFuncSetAttribute(k_band_solve_df, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_band_solve_df<<<(unsigned)items.size(), kThreads, smem, s>>>(
            dptr<PanelMeta>(L->d_meta), dptr<SolveItem>(dItems), dptr<float2>(L->d_Lf), dptr<float2>(L->d_Lb),
            dptr<float2>(L->d_Wf), dptr<float2>(L->d_Wb), dptr<float2>(L->d_Dinv), dptr<double>(X), nrhs, ring);
    }
    k_panel_move<<<mg, 256, 0, s>>>(P.n, P.dpn, nrhs, d_vec, dptr<int>(L->d_panelOf), dptr<int>(L->d_pos),
                                    dptr<PanelMeta>(L->d_meta), dptr<double>(X), 0);
    rc = cuda_check(ctx, cudaGetLastError(), "panel solve");
    if (!rc) rc = cuda_check(ctx, cudaStreamSynchronize(s), "panel solve");
    return rc;
}

extern "C" int astro_panels_solve(astro_ctx *ctx, int32_t num_rhs, const double *rhs, double *x,
                                  astro_panels_info *info) {
    if (!ctx || num_rhs < 1 || !rhs || !x) return ASTRO_ERR_ARG;
    PanelPlan *L = static_cast<PanelPlan *>(ctx->panels);
    if (!L || !L->factored || L->kVersion != ctx->k64Version || L->penVersion != ctx->penVersion)
        return set_err(ctx, ASTRO_ERR_STATE, "panels: no current factorisation (astro_panels_factor)");
    const int n = ctx->P.n;
    const auto t0 = std::chrono::steady_clock::now();
    const size_t nt = (size_t)n * num_rhs;
    DevBuf &ref = L->d_sRef, &vec = L->d_sVec;
    int rc = grow(ctx, ref, sizeof(double) * nt);
    if (!rc) rc = grow(ctx, vec, sizeof(double) * nt);
    if (!rc) rc = copy_to_device(ctx, ref.p, rhs, sizeof(double) * nt, "panels: upload");
    for (int c = 0; c < num_rhs && !rc; ++c)
        rc = ref_to_int_vec(ctx, dptr<double>(ref) + (size_t)c * n, dptr<double>(vec) + (size_t)c * n, n);
    if (!rc) rc = panels_solve_dev(ctx, L, num_rhs, dptr<double>(vec));
    if (!rc && ctx->panelsSolve == 0) {
        // one refinement pass: r = b - A x with the FP64 operator, x += the double-float solve of r
        DevBuf &bi = L->d_sBi, &res = L->d_sRes;
        rc = grow(ctx, bi, sizeof(double) * (size_t)n);
        if (!rc) rc = grow(ctx, res, sizeof(double) * nt);
        for (int c = 0; c < num_rhs && !rc; ++c) {
            rc = ref_to_int_vec(ctx, dptr<double>(ref) + (size_t)c * n, dptr<double>(bi), n);
            if (!rc)
                rc = krylov_residual64(ctx, dptr<double>(vec) + (size_t)c * n, dptr<double>(bi),
                                       dptr<double>(res) + (size_t)c * n);
        }
        if (!rc) rc = panels_solve_dev(ctx, L, num_rhs, dptr<double>(res));
        if (!rc) {
            k_vec_add<<<(unsigned)((nt + 255) / 256), 256, 0, ctx->stream>>>((long long)nt, dptr<double>(res),
                                                                            dptr<double>(vec));
            rc = cuda_check(ctx, cudaGetLastError(), "panels: refinement");
        }
    }
    for (int c = 0; c < num_rhs && !rc; ++c)
        rc = int_to_ref_vec(ctx, dptr<double>(vec) + (size_t)c * n, dptr<double>(ref) + (size_t)c * n, n);
    if (!rc) rc = copy_to_host(ctx, x, ref.p, sizeof(double) * nt, "panels: download");
    if (info) {
        fill_info(*L, info);
        info->solve_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    return rc;
}

extern "C" int astro_panels_solve_batched(astro_ctx *ctx, int32_t num_rhs, const double *rhs, double *x,
                                          astro_panels_info *info) {
    if (!ctx) return ASTRO_ERR_ARG;
    PanelPlan *L = static_cast<PanelPlan *>(ctx->panels);
    int rc;
    if (!L || !L->factored || L->kVersion != ctx->k64Version || L->penVersion != ctx->penVersion)
        if ((rc = astro_panels_factor(ctx, L ? L->cs : 0, info))) return rc;
    return astro_panels_solve(ctx, num_rhs, rhs, x, info);
}

// ---- the many-column solve of one factorisation (time stepping) ---------------------------

// Prepares k_band_solve_cases for ncols right-hand-side columns of the current factorisation:
// the double-float band copies (once per factorisation), the (panel, column) items and the
// panel-layout block.  Allocates; call before any stream capture.
static int twist_prepare(astro_ctx *ctx, PanelPlan *L, int ncols);

// Whether the many-column solve of the current plan runs twisted (ASTRO_OPT_CASES_TWIST: 0 off, 1
// when the single panel has at least 8 windows of block rows, 2 whenever the split leaves rows
// outside the window).
static bool twist_wanted(const astro_ctx *ctx, const PanelPlan *L) {
    if (!L || L->np != 1) return false;
    const PanelMeta &M0 = L->meta[0];
    const int m = std::max(1, M0.bt), K = (M0.nbc - m) / 2;
    if (K < 1) return false;
    return ctx->casesTwist == 2 || (ctx->casesTwist == 1 && M0.nbc >= 8 * (m + 1));
}

int panels_cases_would_twist(astro_ctx *ctx) { return twist_wanted(ctx, static_cast<PanelPlan *>(ctx->panels)); }

int panels_cases_prepare(astro_ctx *ctx, int ncols, size_t *bytes) {
    PanelPlan *L = static_cast<PanelPlan *>(ctx->panels);
    if (ncols < 1) return set_err(ctx, ASTRO_ERR_ARG, "panels: no right-hand sides");
    if (!L || L->kVersion != ctx->k64Version || L->penVersion != ctx->penVersion)
        return set_err(ctx, ASTRO_ERR_STATE, "panels: no current plan (astro_panels_factor)");
    cudaStream_t s = ctx->stream;
    int rc;
    L->twist = twist_wanted(ctx, L);
    L->ring = L->maxBt + 2;
    const size_t smem = sizeof(float2) * ((size_t)L->ring * TB + kCW * TB + 2 * 8 * TB + TB);
    if (L->twist) {
        if ((L->twGen != L->factorGen || L->twCols != ncols) && (rc = twist_prepare(ctx, L, ncols))) return rc;
        L->factorSeconds = L->twFactorSeconds;
        CK(cudaFuncSetAttribute(k_band_solve_cases<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        CK(cudaFuncSetAttribute(k_band_solve_cases<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        CK(cudaFuncSetAttribute(k_band_solve_cases<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        if (bytes) *bytes = 2 * sizeof(float2) * (size_t)L->twBandDoubles;
        return cuda_check(ctx, cudaStreamSynchronize(s), "panels cases prepare");
    }
    if (!L->factored) return set_err(ctx, ASTRO_ERR_STATE, "panels: no current factorisation (astro_panels_factor)");
    if ((rc = panels_df_copies(ctx, L))) return rc;
    if (L->casesCols != ncols) {
        std::vector<CaseItem> items;
        for (int p = 0; p < L->np; ++p)
            for (int c = 0; c < ncols; ++c) items.push_back({p, c, 0, 2 * L->meta[p].nbc});
        dev_free(L->d_items);
        dev_free(L->d_X);
        if ((rc = upload(ctx, L->d_items, items.data(), sizeof(CaseItem) * items.size())) ||
            (rc = dev_alloc(ctx, L->d_X, sizeof(double) * (size_t)L->xRows * ncols)))
            return rc;
        CK(cudaMemsetAsync(L->d_X.p, 0, sizeof(double) * (size_t)L->xRows * ncols, s));
        L->casesCols = ncols;
    }
    CK(cudaFuncSetAttribute(k_band_solve_cases<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    CK(cudaFuncSetAttribute(k_band_solve_cases<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    CK(cudaFuncSetAttribute(k_band_solve_cases<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    if (bytes) *bytes = 2 * sizeof(float2) * (size_t)L->bandDoubles;
    return cuda_check(ctx, cudaStreamSynchronize(s), "panels cases prepare");
}

// The twisted solve's structures for one panel (see k_tw_fill): the three panels, their fill
// and partial factorisations (FP64 trailing updates), the window matrix and its factor, the
// double-float copies, the items of the three cluster launches and the right-hand-side blocks.
static int twist_prepare(astro_ctx *ctx, PanelPlan *L, int ncols) {
    const AstroPrep &P = ctx->P;
    cudaStream_t s = ctx->stream;
    const PanelMeta M0 = L->meta[0];
    const int nbc = M0.nbc, bt = M0.bt, m = std::max(1, bt), K = (nbc - m) / 2;
    const int nbcT = K + m, nbcB = nbc - K;
    L->twK = K;
    L->twM = m;
    std::vector<PanelMeta> mt(3);
    long long band = 0, rows = 0;
    auto put = [&](PanelMeta &M, int n, int nb, int b, int nfac) {
        M.n = n;
        M.nbc = nb;
        M.bt = b;
        M.nfac = nfac;
        M.band = band;
        M.xUnit = rows;
        band += (long long)nb * (b + 1) * TT;
        rows += (long long)nb * TB;
    };
    put(mt[0], nbcT * TB, nbcT, bt, K);
    put(mt[1], nbcB * TB, nbcB, bt, nbcB - m);
    put(mt[2], m * TB, m, m - 1, m);
    L->twMeta = mt;
    L->twBandDoubles = band;
    L->twRows = rows;
    TwistGeom G;
    G.n = M0.n;
    G.dpn = P.dpn;
    G.K32 = K * TB;
    G.nT = nbcT * TB;
    G.nbB32 = nbcB * TB;
    G.rev = G.nbB32 + G.K32 - 1;
    const int w = m * TB;
    int rc;
    const int sched[3] = {0, 1, 2}, schedPtr[3] = {0, 1, 2}, schedPtrS[2] = {0, 1};
    if ((rc = upload(ctx, L->d_twMeta, mt.data(), sizeof(PanelMeta) * 3)) ||
        (rc = upload(ctx, L->d_twSched, sched, sizeof(sched))) ||
        (rc = upload(ctx, L->d_twSchedPtr, schedPtr, sizeof(schedPtr))) ||
        (rc = dev_alloc(ctx, L->d_twBand, sizeof(double) * (size_t)band)) ||
        (rc = dev_alloc(ctx, L->d_twAw, sizeof(double) * (size_t)m * m * TT)) ||
        (rc = dev_alloc(ctx, L->d_twStatus, sizeof(int))))
        return rc;
    DevBuf dSchedPtrS;
    if ((rc = upload(ctx, dSchedPtrS, schedPtrS, sizeof(schedPtrS)))) return rc;
    const auto t0 = std::chrono::steady_clock::now();
    const PanelMeta *dm = dptr<PanelMeta>(L->d_twMeta);
    double *db = dptr<double>(L->d_twBand);
    CK(cudaMemsetAsync(L->d_twBand.p, 0, sizeof(double) * (size_t)band, s));
    CK(cudaMemsetAsync(L->d_twAw.p, 0, sizeof(double) * (size_t)m * m * TT, s));
    CK(cudaMemsetAsync(L->d_twStatus.p, 0, sizeof(int), s));
    const long long fillN = (long long)P.nb * P.dpn * P.dpn;
    k_tw_fill<<<(unsigned)((fillN + 255) / 256), 256, 0, s>>>(P.nb, G, dptr<int>(ctx->d_bRow), dptr<int>(ctx->d_bCol),
                                                            dptr<double>(ctx->d_K64), dptr<int>(L->d_pos), dm, db);
    if (L->penCount)
        k_tw_pen<<<(L->penCount + 255) / 256, 256, 0, s>>>(L->penCount, G, dptr<int>(L->d_penI), dptr<int>(L->d_penJ),
                                                           dptr<double>(L->d_penV), dptr<int>(L->d_pos), dm, db);
    k_tw_pad<<<(G.nbB32 + 255) / 256, 256, 0, s>>>(G, dm, db);
    const unsigned wg = (unsigned)(((long long)w * w + 255) / 256);
    k_tw_window<<<wg, 256, 0, s>>>(G, w, dm, db, dptr<double>(L->d_twAw), 0);
    if ((rc = cuda_check(ctx, cudaGetLastError(), "twisted band fill"))) return rc;
    // the partial factorisations of T and B (one cluster each), the window matrix, its factor
    auto factor = [&](int workers, const int *schedBase, const int *schedP) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(workers * L->cs);
        cfg.blockDim = dim3(kThreads);
        cfg.stream = s;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = L->cs;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        return cudaLaunchKernelEx(&cfg, k_band_ldl<0>, dm, schedBase, schedP, db,
                                  dptr<int>(L->d_twStatus), (uint16_t *)nullptr, (int *)nullptr, 0LL, 0);
    };
    CK(factor(2, dptr<int>(L->d_twSched), dptr<int>(L->d_twSchedPtr)));
    k_tw_window<<<wg, 256, 0, s>>>(G, w, dm, db, dptr<double>(L->d_twAw), 1);
    // the window panel alone: its schedule is sched + 2 (panel 2) with schedPtr {0, 1}
    CK(factor(1, dptr<int>(L->d_twSched) + 2, dptr<int>(dSchedPtrS)));
    int status = 0;
    CK(cudaMemcpyAsync(&status, L->d_twStatus.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    dev_free(dSchedPtrS);
    if (status) return set_err(ctx, ASTRO_ERR_PIVOT, "panels: zero or non-finite pivot in the twisted factorisation");
    L->twFactorSeconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    const size_t nd = (size_t)rows;
    if ((rc = dev_alloc(ctx, L->d_twLf, sizeof(float2) * (size_t)band)) ||
        (rc = dev_alloc(ctx, L->d_twLb, sizeof(float2) * (size_t)band)) ||
        (rc = dev_alloc(ctx, L->d_twWf, sizeof(float2) * nd * TB)) ||
        (rc = dev_alloc(ctx, L->d_twWb, sizeof(float2) * nd * TB)) ||
        (rc = dev_alloc(ctx, L->d_twDinv, sizeof(float2) * nd)))
        return rc;
    const long long cols = (long long)nbcT + nbcB + m;
    k_band_dfprep<<<(unsigned)((cols + kPrepW - 1) / kPrepW), kPrepW * 32, 0, s>>>(
        dm, 3, db, dptr<float2>(L->d_twLf), dptr<float2>(L->d_twLb), dptr<float2>(L->d_twWf), dptr<float2>(L->d_twWb),
        dptr<float2>(L->d_twDinv));
    if ((rc = cuda_check(ctx, cudaGetLastError(), "twisted double-float copy"))) return rc;
    // items: forward T and B, the window, backward T and B (from the row before the window)
    std::vector<CaseItem> items;
    for (int c = 0; c < ncols; ++c) {
        items.push_back({0, c, 0, nbcT});
        items.push_back({1, c, 0, nbcB});
    }
    for (int c = 0; c < ncols; ++c) items.push_back({2, c, 0, 2 * m});
    for (int c = 0; c < ncols; ++c) {
        items.push_back({0, c, nbcT + m, 2 * nbcT});
        items.push_back({1, c, nbcB + m, 2 * nbcB});
    }
    dev_free(L->d_twX);
    if ((rc = upload(ctx, L->d_twItems, items.data(), sizeof(CaseItem) * items.size())) ||
        (rc = dev_alloc(ctx, L->d_twX, sizeof(double) * nd * ncols)))
        return rc;
    CK(cudaMemsetAsync(L->d_twX.p, 0, sizeof(double) * nd * ncols, s));
    L->twCols = ncols;
    L->twGen = L->factorGen;
    return cuda_check(ctx, cudaStreamSynchronize(s), "twisted prepare");
}

// x = (K + C^T C)^-1 b for the prepared number of columns, in place in d_vec (ncols x n, internal
// numbering): moves, one cluster launch, moves.  No allocation, no synchronisation (capturable).
int panels_cases_solve(astro_ctx *ctx, double *d_vec, cudaStream_t s) {
    PanelPlan *L = static_cast<PanelPlan *>(ctx->panels);
    if (!L || (L->twist ? (L->twGen != L->factorGen || !L->twCols) : (L->dfGen != L->factorGen || !L->casesCols)))
        return set_err(ctx, ASTRO_ERR_STATE, "panels: cases not prepared");
    const AstroPrep &P = ctx->P;
    const int nc = L->twist ? L->twCols : L->casesCols;
    const long long mv = (long long)P.n * nc;
    const unsigned mg = (unsigned)((mv + 255) / 256);
    // CTAs per case: the autotuned choice of this context (astro_autotune), else 4
    const int cs = (ctx->tuneCasesCluster == 2 || ctx->tuneCasesCluster == 8) ? ctx->tuneCasesCluster : 4;
    if (L->twist) {
        // move in, forward sweeps of T and B, window right-hand side, window solve, window
        // solution to T and B, backward sweeps, move out
        const PanelMeta *dm = dptr<PanelMeta>(L->d_twMeta);
        TwistGeom G;
        G.n = P.n;
        G.dpn = P.dpn;
        G.K32 = L->twK * TB;
        G.nT = L->twMeta[0].nbc * TB;
        G.nbB32 = L->twMeta[1].nbc * TB;
        G.rev = G.nbB32 + G.K32 - 1;
        const int w = L->twM * TB;
        double *X = dptr<double>(L->d_twX);
        const unsigned wgm = (unsigned)(((long long)w * nc + 255) / 256);
        auto sweep = [&](int first, int count) {
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3((unsigned)(count * cs));
            cfg.blockDim = dim3(kCW * 32);
            cfg.dynamicSmemBytes = sizeof(float2) * ((size_t)L->ring * TB + kCW * TB + 2 * cs * TB + TB);
            cfg.stream = s;
            cudaLaunchAttribute at[1];
            at[0].id = cudaLaunchAttributeClusterDimension;
            at[0].val.clusterDim.x = cs;
            at[0].val.clusterDim.y = 1;
            at[0].val.clusterDim.z = 1;
            cfg.attrs = at;
            cfg.numAttrs = 1;
            auto kern = cs == 2 ? k_band_solve_cases<2> : (cs == 8 ? k_band_solve_cases<8> : k_band_solve_cases<4>);
            return cudaLaunchKernelEx(&cfg, kern, dm, (const CaseItem *)dptr<CaseItem>(L->d_twItems) + first,
                                      (const float2 *)dptr<float2>(L->d_twLf), (const float2 *)dptr<float2>(L->d_twLb),
                                      (const float2 *)dptr<float2>(L->d_twWf), (const float2 *)dptr<float2>(L->d_twWb),
                                      (const float2 *)dptr<float2>(L->d_twDinv), X, nc, L->ring);
        };
        k_tw_move<<<mg, 256, 0, s>>>(nc, G, w, d_vec, dptr<int>(L->d_pos), dm, X, 0);
        CK(sweep(0, 2 * nc));
        k_tw_move<<<wgm, 256, 0, s>>>(nc, G, w, d_vec, dptr<int>(L->d_pos), dm, X, 1);
        CK(sweep(2 * nc, nc));
        k_tw_move<<<wgm, 256, 0, s>>>(nc, G, w, d_vec, dptr<int>(L->d_pos), dm, X, 2);
        CK(sweep(3 * nc, 2 * nc));
        k_tw_move<<<mg, 256, 0, s>>>(nc, G, w, d_vec, dptr<int>(L->d_pos), dm, X, 3);
        return cuda_check(ctx, cudaGetLastError(), "panels twisted cases solve");
    }
    k_panel_move<<<mg, 256, 0, s>>>(P.n, P.dpn, nc, d_vec, dptr<int>(L->d_panelOf), dptr<int>(L->d_pos),
                                    dptr<PanelMeta>(L->d_meta), dptr<double>(L->d_X), 1);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(L->np * nc * cs));
    cfg.blockDim = dim3(kCW * 32);
    cfg.dynamicSmemBytes = sizeof(float2) * ((size_t)L->ring * TB + kCW * TB + 2 * cs * TB + TB);
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = cs;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    auto kern = cs == 2 ? k_band_solve_cases<2> : (cs == 8 ? k_band_solve_cases<8> : k_band_solve_cases<4>);
    CK(cudaLaunchKernelEx(&cfg, kern, (const PanelMeta *)dptr<PanelMeta>(L->d_meta),
                          (const CaseItem *)dptr<CaseItem>(L->d_items), (const float2 *)dptr<float2>(L->d_Lf),
                          (const float2 *)dptr<float2>(L->d_Lb), (const float2 *)dptr<float2>(L->d_Wf),
                          (const float2 *)dptr<float2>(L->d_Wb), (const float2 *)dptr<float2>(L->d_Dinv),
                          dptr<double>(L->d_X), nc, L->ring));
    k_panel_move<<<mg, 256, 0, s>>>(P.n, P.dpn, nc, d_vec, dptr<int>(L->d_panelOf), dptr<int>(L->d_pos),
                                    dptr<PanelMeta>(L->d_meta), dptr<double>(L->d_X), 0);
    return cuda_check(ctx, cudaGetLastError(), "panels cases solve");
}

// Kernel launches of one panels_cases_solve (3, or 7 for the twisted solve).
int panels_cases_launches(astro_ctx *ctx) {
    PanelPlan *L = static_cast<PanelPlan *>(ctx->panels);
    return (L && L->twist) ? 7 : 3;
}

// Columns of the prepared many-column solve of the current factorisation (0: none prepared).
int panels_cases_columns(astro_ctx *ctx) {
    PanelPlan *L = static_cast<PanelPlan *>(ctx->panels);
    if (L && L->twist) return L->twGen == L->factorGen ? L->twCols : 0;
    return (L && L->factored && L->dfGen == L->factorGen) ? L->casesCols : 0;
}

// Shape of the current plan: panels, largest bandwidth (DOF), band bytes, factor seconds.
void panels_shape(astro_ctx *ctx, int *np, int *bw, long long *bandBytes, double *factorSeconds) {
    PanelPlan *L = static_cast<PanelPlan *>(ctx->panels);
    if (!L) return;
    if (np) *np = L->np;
    if (bw) *bw = L->maxBw;
    if (bandBytes) *bandBytes = (L->twist ? L->twBandDoubles : L->bandDoubles) * (long long)sizeof(double);
    if (factorSeconds) *factorSeconds = L->factorSeconds;
}
