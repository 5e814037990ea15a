// Building blocks shared by the Krylov solvers and the polynomial preconditioner: launch
// constants, the solver's device control block, the block-ELL operator descriptor and its row
// products, warp sums, and the last-CTA-to-arrive test used for deterministic reductions.
#pragma once
#include <cuda_fp16.h>
#include <cuda_runtime.h>

namespace astro_kry {

constexpr int kMaxM = 64;
constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kGsThreads = 1024;  // threads per CTA of the Gram-Schmidt passes
constexpr int kGsWarps = kGsThreads / 32;
constexpr int kChunk = 1024;      // vector rows per CTA in the Gram-Schmidt passes (one per thread)
constexpr int kRowThreads = 4;    // threads per block row in the SpMV

struct GmresCtl {
    double H[(kMaxM + 1) * kMaxM];  // column-major (m+1) x m, Givens-rotated in place
    double cs[kMaxM], sn[kMaxM], g[kMaxM + 1];
    double h1[kMaxM + 1];
    double y[kMaxM];
    double inv;      // 1 / ||w|| of the last step (scales w into the next basis vector)
    double target;   // absolute residual target
    double resest;   // |g[j]| after the last step
    int j;           // completed Arnoldi steps in this cycle
    int done;        // converged / broke down / cycle full: later steps are no-ops
    int breakdown;
    int nonfinite;
    unsigned arrive[3];  // CTAs finished in the current dots / update / update-and-norm launch
    int reorth;          // this step's first pass lost more than half of ||w||^2: run the second
    int reorths;         // second passes run in this cycle
};

template <class TM> struct Op {
    const TM *K;        // block-ELL values: entry q of slot s of block row r at (s*DPN*DPN + q)*ld + r
    const int *col;     // block column of slot s of row r at col[s*ld + r]
    int S, ld;          // slots per row, row stride
    const int *penPtr;  // (N+1) penalty entries per block row, or null
    const int *penRow;
    const int *penCol;
    const double *penVal;
    int N, dpn;
};

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ float warp_sum(float v) {
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// y = (A x)_r for block row r, one thread: the products accumulate in TA (the matrix precision
// for the Krylov steps, FP64 for true residuals).  Slots are taken three at a time so that their
// column, x and value loads are in flight together.
template <class TA, class TM, class TX, int DPN>
__device__ __forceinline__ void ell_row(const Op<TM> &op, int r, const TX *__restrict__ x, TA y[DPN]) {
    constexpr int G = 3;
#pragma unroll
    for (int i = 0; i < DPN; ++i) y[i] = TA(0);
    const size_t ld = (size_t)op.ld;
    for (int s0 = 0; s0 < op.S; s0 += G) {
        int c[G];
#pragma unroll
        for (int g = 0; g < G; ++g) c[g] = (s0 + g < op.S) ? __ldg(op.col + (size_t)(s0 + g) * ld + r) : -1;
        TA xv[G][DPN];
#pragma unroll
        for (int g = 0; g < G; ++g)
#pragma unroll
            for (int jj = 0; jj < DPN; ++jj) xv[g][jj] = (c[g] >= 0) ? (TA)x[(size_t)c[g] * DPN + jj] : TA(0);
#pragma unroll
        for (int g = 0; g < G; ++g) {
            if (s0 + g >= op.S) break;
            const TM *kp = op.K + (size_t)(s0 + g) * DPN * DPN * ld + r;
#pragma unroll
            for (int i = 0; i < DPN; ++i)
#pragma unroll
                for (int jj = 0; jj < DPN; ++jj) y[i] += (TA)__ldg(kp + (size_t)(i * DPN + jj) * ld) * xv[g][jj];
        }
    }
    if (op.penPtr) {
        for (int t = op.penPtr[r]; t < op.penPtr[r + 1]; ++t) {
            const TA p = (TA)(op.penVal[t] * (double)x[op.penCol[t]]);
            const int i = op.penRow[t];
#pragma unroll
            for (int q = 0; q < DPN; ++q) y[q] += (q == i) ? p : TA(0);
        }
    }
}

// Partial (A x)_r over the slots s = sub, sub + kRowThreads, ... of block row r; the products
// accumulate in TA.  The kRowThreads threads of a row are adjacent lanes and combine their
// partials with xor-shuffles (result in all of them); thread sub == 0 adds the penalty.
template <class TA, class TM, class TX, int DPN>
__device__ __forceinline__ void ell_row_part(const Op<TM> &op, int r, int sub, const TX *__restrict__ x, TA y[DPN]) {
#pragma unroll
    for (int i = 0; i < DPN; ++i) y[i] = TA(0);
    const size_t ld = (size_t)op.ld;
    for (int s = sub; s < op.S; s += kRowThreads) {
        const int c = __ldg(op.col + (size_t)s * ld + r);
        TA xv[DPN];
#pragma unroll
        for (int jj = 0; jj < DPN; ++jj) xv[jj] = (TA)x[(size_t)c * DPN + jj];
        const TM *kp = op.K + (size_t)s * DPN * DPN * ld + r;
#pragma unroll
        for (int i = 0; i < DPN; ++i)
#pragma unroll
            for (int jj = 0; jj < DPN; ++jj) y[i] += (TA)__ldg(kp + (size_t)(i * DPN + jj) * ld) * xv[jj];
    }
    if (sub == 0 && op.penPtr) {
        for (int t = op.penPtr[r]; t < op.penPtr[r + 1]; ++t) {
            const TA p = (TA)(op.penVal[t] * (double)x[op.penCol[t]]);
            const int i = op.penRow[t];
#pragma unroll
            for (int q = 0; q < DPN; ++q) y[q] += (q == i) ? p : TA(0);
        }
    }
#pragma unroll
    for (int m = 1; m < kRowThreads; m <<= 1)
#pragma unroll
        for (int i = 0; i < DPN; ++i) y[i] += __shfl_xor_sync(0xffffffffu, y[i], m);
}

// Warp-per-slot-group SpMV mapping: a CTA of kThreads covers kCtaRows = 32 * kThreads / (32 *
// kRowThreads) block rows; warp w takes the 32 consecutive rows (w / kRowThreads) * 32 + lane
// and the slots s = w % kRowThreads, + kRowThreads, ...  Every value, column and penalty load of
// a warp instruction then covers 32 consecutive rows of one (slot, entry) plane: one contiguous
// segment.  The kRowThreads partials of a row meet in shared memory (ell_cta_reduce).
constexpr int kCtaRows = kThreads / kRowThreads;

struct CtaRow {
    int r;     // block row
    int sub;   // slot group (warp-uniform)
    int rloc;  // row within the CTA
    bool valid;
};
__device__ __forceinline__ CtaRow cta_row(int N) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    CtaRow c;
    c.sub = w % kRowThreads;
    c.rloc = (w / kRowThreads) * 32 + lane;
    c.r = blockIdx.x * kCtaRows + c.rloc;
    c.valid = c.r < N;
    return c;
}

// Partial (A x)_r over the slots s = sub, sub + kRowThreads, ...; slot group 0 adds the penalty.
template <class TA, class TM, class TX, int DPN>
__device__ __forceinline__ void ell_row_group(const Op<TM> &op, int r, int sub, const TX *__restrict__ x, TA y[DPN]) {
#pragma unroll
    for (int i = 0; i < DPN; ++i) y[i] = TA(0);
    const size_t ld = (size_t)op.ld;
    int s = sub;
    // two slots per trip so that their column, x and value loads are in flight together
    for (; s + kRowThreads < op.S; s += 2 * kRowThreads) {
        const int c0 = __ldg(op.col + (size_t)s * ld + r);
        const int c1 = __ldg(op.col + (size_t)(s + kRowThreads) * ld + r);
        TA x0[DPN], x1[DPN];
#pragma unroll
        for (int jj = 0; jj < DPN; ++jj) {
            x0[jj] = (TA)x[(size_t)c0 * DPN + jj];
            x1[jj] = (TA)x[(size_t)c1 * DPN + jj];
        }
        const TM *k0 = op.K + (size_t)s * DPN * DPN * ld + r;
        const TM *k1 = op.K + (size_t)(s + kRowThreads) * DPN * DPN * ld + r;
#pragma unroll
        for (int i = 0; i < DPN; ++i)
#pragma unroll
            for (int jj = 0; jj < DPN; ++jj)
                y[i] += (TA)__ldg(k0 + (size_t)(i * DPN + jj) * ld) * x0[jj] +
                        (TA)__ldg(k1 + (size_t)(i * DPN + jj) * ld) * x1[jj];
    }
    if (s < op.S) {
        const int c = __ldg(op.col + (size_t)s * ld + r);
        TA xv[DPN];
#pragma unroll
        for (int jj = 0; jj < DPN; ++jj) xv[jj] = (TA)x[(size_t)c * DPN + jj];
        const TM *kp = op.K + (size_t)s * DPN * DPN * ld + r;
#pragma unroll
        for (int i = 0; i < DPN; ++i)
#pragma unroll
            for (int jj = 0; jj < DPN; ++jj) y[i] += (TA)__ldg(kp + (size_t)(i * DPN + jj) * ld) * xv[jj];
    }
    if (sub == 0 && op.penPtr) {
        for (int t = op.penPtr[r]; t < op.penPtr[r + 1]; ++t) {
            const TA p = (TA)(op.penVal[t] * (double)x[op.penCol[t]]);
            const int i = op.penRow[t];
#pragma unroll
            for (int q = 0; q < DPN; ++q) y[q] += (q == i) ? p : TA(0);
        }
    }
}

// FP16 block-vector operator of the polynomial preconditioner: the dpn x dpn block of slot s of
// block row r is stored as NV = dpn^2 / 8 uint4 planes (eight FP16 entries each, row-major) at
// Kv[(s * NV + p) * ld + r] and a remainder plane of REM = dpn^2 mod 8 entries at
// Kr[s * ld + r] (one __half for dpn 3, a uint2 of four for dpn 6).  A warp instruction then
// moves 16 bytes per lane over 32 consecutive rows, so one slot costs NV + 1 value loads instead
// of dpn^2.
template <int DPN> struct BvShape {
    static constexpr int DD = DPN * DPN, NV = DD / 8, REM = DD % 8;
};
template <int REM> struct BvRem;
template <> struct BvRem<1> {
    using T = unsigned short;
};
template <> struct BvRem<4> {
    using T = uint2;
};

struct OpH {
    const uint4 *Kv;
    const void *Kr;
    const int *col;
    int S, ld;
    const int *penPtr;  // penalty lists as in Op (values scaled like the matrix)
    const int *penRow;
    const int *penCol;
    const double *penVal;
    int N, dpn;
};

__device__ __forceinline__ float h2f_bits(unsigned short b) { return __half2float(__ushort_as_half(b)); }

// the block's entries as floats, row-major
template <int DPN>
__device__ __forceinline__ void bv_load(const OpH &op, int s, int r, float v[DPN * DPN]) {
    using Sh = BvShape<DPN>;
    const size_t ld = (size_t)op.ld;
    const size_t sr = (size_t)s * ld + r;
#pragma unroll
    for (int p = 0; p < Sh::NV; ++p) {
        const uint4 u = __ldg(op.Kv + ((size_t)s * Sh::NV + p) * ld + r);
        const unsigned w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            v[8 * p + 2 * k] = h2f_bits((unsigned short)(w[k] & 0xffffu));
            v[8 * p + 2 * k + 1] = h2f_bits((unsigned short)(w[k] >> 16));
        }
    }
    const typename BvRem<Sh::REM>::T *kr = static_cast<const typename BvRem<Sh::REM>::T *>(op.Kr);
    if constexpr (Sh::REM == 1) {
        v[8 * Sh::NV] = h2f_bits(__ldg(kr + sr));
    } else {
        const uint2 u = __ldg(kr + sr);
        v[8 * Sh::NV] = h2f_bits((unsigned short)(u.x & 0xffffu));
        v[8 * Sh::NV + 1] = h2f_bits((unsigned short)(u.x >> 16));
        v[8 * Sh::NV + 2] = h2f_bits((unsigned short)(u.y & 0xffffu));
        v[8 * Sh::NV + 3] = h2f_bits((unsigned short)(u.y >> 16));
    }
}

// Partial (A^ x)_r over the slot group, FP32 products, block-vector loads (two slots per trip).
template <class TA, class TX, int DPN>
__device__ __forceinline__ void ell_row_group(const OpH &op, int r, int sub, const TX *__restrict__ x, TA y[DPN]) {
    constexpr int DD = DPN * DPN;
#pragma unroll
    for (int i = 0; i < DPN; ++i) y[i] = TA(0);
    const size_t ld = (size_t)op.ld;
    int s = sub;
    for (; s + kRowThreads < op.S; s += 2 * kRowThreads) {
        const int c0 = __ldg(op.col + (size_t)s * ld + r);
        const int c1 = __ldg(op.col + (size_t)(s + kRowThreads) * ld + r);
        float k0[DD], k1[DD];
        bv_load<DPN>(op, s, r, k0);
        bv_load<DPN>(op, s + kRowThreads, r, k1);
        TA x0[DPN], x1[DPN];
#pragma unroll
        for (int jj = 0; jj < DPN; ++jj) {
            x0[jj] = (TA)x[(size_t)c0 * DPN + jj];
            x1[jj] = (TA)x[(size_t)c1 * DPN + jj];
        }
#pragma unroll
        for (int i = 0; i < DPN; ++i)
#pragma unroll
            for (int jj = 0; jj < DPN; ++jj) y[i] += (TA)k0[i * DPN + jj] * x0[jj] + (TA)k1[i * DPN + jj] * x1[jj];
    }
    if (s < op.S) {
        const int c = __ldg(op.col + (size_t)s * ld + r);
        float kv[DD];
        bv_load<DPN>(op, s, r, kv);
        TA xv[DPN];
#pragma unroll
        for (int jj = 0; jj < DPN; ++jj) xv[jj] = (TA)x[(size_t)c * DPN + jj];
#pragma unroll
        for (int i = 0; i < DPN; ++i)
#pragma unroll
            for (int jj = 0; jj < DPN; ++jj) y[i] += (TA)kv[i * DPN + jj] * xv[jj];
    }
    if (sub == 0 && op.penPtr) {
        for (int t = op.penPtr[r]; t < op.penPtr[r + 1]; ++t) {
            const TA p = (TA)(op.penVal[t] * (double)x[op.penCol[t]]);
            const int i = op.penRow[t];
#pragma unroll
            for (int q = 0; q < DPN; ++q) y[q] += (q == i) ? p : TA(0);
        }
    }
}

// One entry point for the row products of both operator kinds.
template <class TA, int DPN, class TM>
__device__ __forceinline__ void row_group(const Op<TM> &op, int r, int sub, const TA *__restrict__ x, TA y[DPN]) {
    ell_row_group<TA, TM, TA, DPN>(op, r, sub, x, y);
}
template <class TA, int DPN>
__device__ __forceinline__ void row_group(const OpH &op, int r, int sub, const TA *__restrict__ x, TA y[DPN]) {
    ell_row_group<TA, TA, DPN>(op, r, sub, x, y);
}

// Adds the partials of slot groups 1.. to those of group 0 (in group order); true for the
// group-0 thread, which then holds (A x)_r.  Every thread of the CTA must call it.
template <class TA, int DPN>
__device__ __forceinline__ bool ell_cta_reduce(TA y[DPN], const CtaRow &c) {
    __shared__ TA sp[kRowThreads - 1][kCtaRows][DPN];
    if (c.sub > 0) {
#pragma unroll
        for (int q = 0; q < DPN; ++q) sp[c.sub - 1][c.rloc][q] = y[q];
    }
    __syncthreads();
    if (c.sub != 0) return false;
#pragma unroll
    for (int g = 0; g < kRowThreads - 1; ++g)
#pragma unroll
        for (int q = 0; q < DPN; ++q) y[q] += sp[g][c.rloc][q];
    return true;
}

// True in the last CTA of the launch to arrive; the threads that wrote partials have fenced them
// before the barrier.  That CTA resets the counter for the next launch.  No CTA waits for another.
__device__ __forceinline__ bool last_to_arrive(unsigned *counter) {
    __shared__ bool amLast;
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned prev = atomicAdd(counter, 1u);
        amLast = (prev == gridDim.x - 1);
        if (amLast) *counter = 0u;
    }
    __syncthreads();
    if (amLast) __threadfence();
    return amLast;
}

}  // namespace astro_kry

struct astro_ctx;
// Block-ELL operator of A = K + C^T C over the FP64 (kind 64) or FP32 (kind 32) device-resident
// K (the solver copy is rebuilt when the assembly changed); the pointer type follows the kind.
int krylov_op64(astro_ctx *ctx, astro_kry::Op<double> *op);
int krylov_op32(astro_ctx *ctx, astro_kry::Op<float> *op);
// 1 / diag(A) in FP64 (n values, internal layout) from the kind's K.
int krylov_dinv(astro_ctx *ctx, int kind, double *d_dinv);
// Largest eigenvalue of D^-1 A: 50 power iterations from a fixed start vector (deterministic).
int krylov_power_lambda(astro_ctx *ctx, int kind, double *lam);
