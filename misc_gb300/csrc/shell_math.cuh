// Device scalar math of AStrO's element library, generic over T in {double, cplx} so that the
// complex-step twin (Working/AStrO_c_*.f90) runs the same code path as the real one
// (Working/AStrO_r_*.f90).
//
// The reference evaluates sqrt, sin, cos and asin with its own routines
// (Working/AStrO_r_overloadFunctions.f90:24-171): Newton iteration for sqrt from 1 with the
// stopping test |delta| <= 1e-13 or 50 steps, seven-term Taylor series (about 0 for |x| < pi/4,
// about pi/2 otherwise) for sin, and Newton iteration for asin.  Their numeric literals are Fortran
// default-real constants, i.e. float32 values promoted to double; LIT() reproduces that rounding.
// The wrap of the angle into [0, 2pi) follows the routine's evident intent (the variable it
// leaves unset for 0 <= theta <= 2pi takes theta itself).
#pragma once
#include <cuda_runtime.h>

#define LIT(x) ((double)(float)(x))

struct cplx {
    double re, im;
    __host__ __device__ cplx() : re(0), im(0) {}
    __host__ __device__ cplx(double r) : re(r), im(0) {}
    __host__ __device__ cplx(double r, double i) : re(r), im(i) {}
};
__device__ __forceinline__ cplx operator+(cplx a, cplx b) { return cplx(a.re + b.re, a.im + b.im); }
__device__ __forceinline__ cplx operator-(cplx a, cplx b) { return cplx(a.re - b.re, a.im - b.im); }
__device__ __forceinline__ cplx operator-(cplx a) { return cplx(-a.re, -a.im); }
__device__ __forceinline__ cplx operator*(cplx a, cplx b) {
    return cplx(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
__device__ __forceinline__ cplx operator*(double s, cplx a) { return cplx(s * a.re, s * a.im); }
__device__ __forceinline__ cplx operator*(cplx a, double s) { return cplx(s * a.re, s * a.im); }
__device__ __forceinline__ cplx operator/(cplx a, cplx b) {
    // Smith's algorithm
    if (fabs(b.re) >= fabs(b.im)) {
        const double r = b.im / b.re, d = b.re + b.im * r;
        return cplx((a.re + a.im * r) / d, (a.im - a.re * r) / d);
    }
    const double r = b.re / b.im, d = b.re * r + b.im;
    return cplx((a.re * r + a.im) / d, (a.im * r - a.re) / d);
}
__device__ __forceinline__ cplx operator+(cplx a, double s) { return cplx(a.re + s, a.im); }
__device__ __forceinline__ cplx operator-(cplx a, double s) { return cplx(a.re - s, a.im); }
__device__ __forceinline__ cplx operator-(double s, cplx a) { return cplx(s - a.re, -a.im); }
__device__ __forceinline__ cplx &operator+=(cplx &a, cplx b) { a = a + b; return a; }
__device__ __forceinline__ cplx &operator-=(cplx &a, cplx b) { a = a - b; return a; }

__device__ __forceinline__ double absT(double x) { return fabs(x); }
__device__ __forceinline__ double absT(cplx x) { return hypot(x.re, x.im); }
__device__ __forceinline__ double reT(double x) { return x; }
__device__ __forceinline__ double reT(cplx x) { return x.re; }
__device__ __forceinline__ double imT(double) { return 0.0; }
__device__ __forceinline__ double imT(cplx x) { return x.im; }
template <class T> __device__ __forceinline__ T pert_i(double h);  // i*h for complex, 0 for real
template <> __device__ __forceinline__ double pert_i<double>(double) { return 0.0; }
template <> __device__ __forceinline__ cplx pert_i<cplx>(double h) { return cplx(0.0, h); }
__device__ __forceinline__ bool isZeroT(double x) { return x == 0.0; }
__device__ __forceinline__ bool isZeroT(cplx x) { return x.re == 0.0 && x.im == 0.0; }

template <class T> struct AK;  // per-T constants of Working/AStrO_constantVals.f90
template <> struct AK<double> {
    static constexpr double pi = LIT(3.141592653589793);
    static constexpr double o6 = 1.0 / 6.0;
    static constexpr double o3 = 1.0 / 3.0;
    static constexpr double rt3 = 0.57735026918962576451;  // 1/sqrt(3) in double
};
template <> struct AK<cplx> {
    static constexpr double pi = LIT(3.14159265358979323846);
    static constexpr double o6 = 0.166666666666666;
    static constexpr double o3 = 0.333333333333333;
    static constexpr double rt3 = LIT(0.577350269189626);
};

// a > b in the reference's sense (r_greater: shift b towards a by 10 % of the distance)
template <class T> __device__ __forceinline__ bool a_greater(T a, T b) {
    const T shifted = b + T(LIT(1e-1) * absT(a - b));
    return absT(a - shifted) < absT(a - b);
}

template <class T> __device__ T a_sqrt(T x) {
    T s = T(1.0), d = T(1.0);
    for (int it = 0; it < 50 && absT(d) > LIT(1e-13); ++it) {
        d = -(s * s - x) / (T(2.0) * s);
        s = s + d;
    }
    return s;
}

template <class T> __device__ T a_sin_quarter(T th) {
    if (absT(th) < LIT(0.7853981633974483)) {
        const double c[7] = {1.0, -LIT(1.666666666666666e-1), LIT(8.333333333333333e-3), -LIT(1.984126984126984e-4),
                             LIT(2.755731922398589e-6), -LIT(2.505210838544171e-8), LIT(1.6059043836821614e-10)};
        const T t2 = th * th;
        T s = T(c[6]);
        for (int k = 5; k >= 0; --k) s = s * t2 + T(c[k]);
        return s * th;
    }
    const double c[7] = {1.0, -0.5, LIT(4.1666666666666666e-2), -LIT(1.388888888888889e-3), LIT(2.4801587301587301e-5),
                         -LIT(2.755731922398589e-7), LIT(2.0876756987868098e-9)};
    const T d = th - 0.5 * AK<T>::pi;
    const T t2 = d * d;
    T s = T(c[6]);
    for (int k = 5; k >= 0; --k) s = s * t2 + T(c[k]);
    return s;
}

template <class T> __device__ T a_sin(T th) {
    const double pi = AK<T>::pi;
    T m = th;
    if (a_greater(th, T(2.0 * pi))) m = th - (double)(int)absT(0.5 * th * T(1.0 / pi)) * 2.0 * pi;
    if (a_greater(T(0.0), th)) m = th + (double)((int)absT(0.5 * th * T(1.0 / pi)) + 1) * 2.0 * pi;
    if (a_greater(m, T(1.5 * pi))) return -a_sin_quarter(T(2.0 * pi) - m);
    if (a_greater(m, T(pi))) return -a_sin_quarter(m - pi);
    if (a_greater(m, T(0.5 * pi))) return a_sin_quarter(T(pi) - m);
    return a_sin_quarter(m);
}

template <class T> __device__ __forceinline__ T a_cos(T th) { return a_sin(th + 0.5 * AK<T>::pi); }

template <class T> __device__ T a_asin(T s) {
    T x = T(0.0), d = T(1.0);
    for (int it = 0; it < 20 && absT(d) > LIT(1e-13); ++it) {
        d = -(a_sin(x) - s) / a_cos(x);
        x = x + d;
    }
    return x;
}

// Unpivoted LU of rows/cols 0..n-1 of a row-major n x n array and the solve of the reference
// (r_LUFactor / r_SolveLUxb, Working/AStrO_r_designPropertyFunctions.f90:1015-1073).
template <class T, int LD> __device__ void a_lu(T *A, int n) {
    for (int i = 0; i < n; ++i) {
        for (int j = i; j < n; ++j)
            for (int k = 0; k < i; ++k) A[i * LD + j] = A[i * LD + j] - A[i * LD + k] * A[k * LD + j];
        const T f = T(1.0) / A[i * LD + i];
        for (int j = i + 1; j < n; ++j) {
            for (int k = 0; k < i; ++k) A[j * LD + i] = A[j * LD + i] - A[j * LD + k] * A[k * LD + i];
            A[j * LD + i] = f * A[j * LD + i];
        }
    }
}
template <class T, int LD> __device__ void a_lu_solve(const T *A, const T *b, T *x, int n) {
    T z[9];
    for (int i = 0; i < n; ++i) {
        z[i] = b[i];
        for (int k = 0; k < i; ++k) z[i] = z[i] - A[i * LD + k] * z[k];
    }
    x[n - 1] = z[n - 1] / A[(n - 1) * LD + n - 1];
    for (int i = n - 2; i >= 0; --i) {
        const T f = T(1.0) / A[i * LD + i];
        T dp = T(0.0);
        for (int k = i + 1; k < n; ++k) dp = dp + A[i * LD + k] * x[k];
        x[i] = f * (z[i] - dp);
    }
}

// Rotation of the frame aGL (rows = local axes) by the rotation vector rot, or its derivative
// with respect to rot(dv1) [and rot(dv2)] (r_rotateAlpha, :1075-1463).  For |rot| < 1e-5 the
// reference uses a third-order expansion, otherwise the exact rotation built from an orthonormal
// frame whose first row is the rotation axis.
template <class T>
__device__ void a_rotate(T out[3][3], const T aGL[3][3], const T rot[3], int dv1, int dv2) {
    const double o6 = AK<T>::o6, o3 = AK<T>::o3;
    const T Rmag = a_sqrt(rot[0] * rot[0] + rot[1] * rot[1] + rot[2] * rot[2]);
    T M[3][3];  // rotation (or its derivative) expressed before aGL
    if (absT(Rmag) < LIT(1e-5)) {
        T r[3], d1[3] = {T(0.0), T(0.0), T(0.0)}, d2[3] = {T(0.0), T(0.0), T(0.0)};
        for (int i = 0; i < 3; ++i) {
            r[i] = aGL[i][0] * rot[0] + aGL[i][1] * rot[1] + aGL[i][2] * rot[2];
            if (dv1) d1[i] = aGL[i][dv1 - 1];
            if (dv2) d2[i] = aGL[i][dv2 - 1];
        }
        const T tv = o6 * (r[2] * r[2] + r[0] * r[0] + r[1] * r[1]);
        if (dv1 + dv2 == 0) {
            M[0][0] = T(1.0) - 0.5 * (r[1] * r[1] + r[2] * r[2]);
            M[1][0] = 0.5 * r[0] * r[1] - r[2] + tv * r[2];
            M[2][0] = 0.5 * r[0] * r[2] + r[1] - tv * r[1];
            M[0][1] = 0.5 * r[0] * r[1] + r[2] - tv * r[2];
            M[1][1] = T(1.0) - 0.5 * (r[0] * r[0] + r[2] * r[2]);
            M[2][1] = 0.5 * r[1] * r[2] - r[0] + tv * r[0];
            M[0][2] = 0.5 * r[0] * r[2] - r[1] + tv * r[1];
            M[1][2] = 0.5 * r[1] * r[2] + r[0] - tv * r[0];
            M[2][2] = T(1.0) - 0.5 * (r[0] * r[0] + r[1] * r[1]);
        } else if (dv1 * dv2 == 0) {
            const T dt = o3 * (d1[2] * r[2] + d1[0] * r[0] + d1[1] * r[1]);
            M[0][0] = -(r[1] * d1[1] + r[2] * d1[2]);
            M[1][0] = 0.5 * (d1[0] * r[1] + r[0] * d1[1]) - d1[2] + dt * r[2] + tv * d1[2];
            M[2][0] = 0.5 * (d1[0] * r[2] + r[0] * d1[2]) + d1[1] - dt * r[1] - tv * d1[1];
            M[0][1] = 0.5 * (d1[0] * r[1] + r[0] * d1[1]) + d1[2] - dt * r[2] - tv * d1[2];
            M[1][1] = -(r[0] * d1[0] + r[2] * d1[2]);
            M[2][1] = 0.5 * (d1[1] * r[2] + r[1] * d1[2]) - d1[0] + dt * r[0] + tv * d1[0];
            M[0][2] = 0.5 * (d1[0] * r[2] + r[0] * d1[2]) - d1[1] + dt * r[1] + tv * d1[1];
            M[1][2] = 0.5 * (d1[1] * r[2] + r[1] * d1[2]) + d1[0] - dt * r[0] - tv * d1[0];
            M[2][2] = -(d1[0] * r[0] + d1[1] * r[1]);
        } else {
            const T dt1 = o3 * (d1[2] * r[2] + d1[0] * r[0] + d1[1] * r[1]);
            const T dt2 = o3 * (d2[2] * r[2] + d2[0] * r[0] + d2[1] * r[1]);
            const T ddt = o3 * (d1[2] * d2[2] + d1[0] * d2[0] + d1[1] * d2[1]);
            M[0][0] = -(d2[1] * d1[1] + d2[2] * d1[2]);
            M[1][0] = 0.5 * (d1[0] * d2[1] + d2[0] * d1[1]) + ddt * r[2] + dt1 * d2[2] + dt2 * d1[2];
            M[2][0] = 0.5 * (d1[0] * d2[2] + d2[0] * d1[2]) - ddt * r[1] - dt1 * d2[1] - dt2 * d1[1];
            M[0][1] = 0.5 * (d1[0] * d2[1] + d2[0] * d1[1]) - ddt * r[2] - dt1 * d2[2] - dt2 * d1[2];
            M[1][1] = -(d2[0] * d1[0] + d2[2] * d1[2]);
            M[2][1] = 0.5 * (d1[1] * d2[2] + d2[1] * d1[2]) + ddt * r[0] + dt1 * d2[0] + dt2 * d1[0];
            M[0][2] = 0.5 * (d1[0] * d2[2] + d2[0] * d1[2]) + ddt * r[1] + dt1 * d2[1] + dt2 * d1[1];
            M[1][2] = 0.5 * (d1[1] * d2[2] + d2[1] * d1[2]) - ddt * r[0] + dt1 * d2[0] + dt2 * d1[0];
            M[2][2] = -(d1[0] * d2[0] + d1[1] * d2[1]);
        }
        // expansion is applied on the left of aGL
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) out[i][j] = M[i][0] * aGL[0][j] + M[i][1] * aGL[1][j] + M[i][2] * aGL[2][j];
        return;
    }
    // exact rotation: a1 = orthonormal frame with first row along rot, a2 = a1 rotated about it
    const T sR = a_sin(Rmag), cR = a_cos(Rmag);
    T dRm1 = T(0.0), dRm2 = T(0.0), d2Rm = T(0.0);
    T e1[3] = {T(0.0), T(0.0), T(0.0)}, e2[3] = {T(0.0), T(0.0), T(0.0)};
    if (dv1) e1[dv1 - 1] = T(1.0);
    if (dv2) e2[dv2 - 1] = T(1.0);
    if (dv1 && !dv2) {
        dRm1 = (T(1.0) / a_sqrt(rot[0] * rot[0] + rot[1] * rot[1] + rot[2] * rot[2])) * (rot[dv1 - 1] * e1[dv1 - 1]);
    } else if (dv1 && dv2) {
        const T inv = T(1.0) / Rmag;
        d2Rm = (dv1 == dv2) ? inv * e1[dv1 - 1] * e2[dv1 - 1] : T(0.0);
        d2Rm = d2Rm - (inv * inv * inv) * rot[dv1 - 1] * e1[dv1 - 1] * rot[dv2 - 1] * e2[dv2 - 1];
        dRm1 = inv * (rot[dv1 - 1] * e1[dv1 - 1]);
        dRm2 = inv * (rot[dv2 - 1] * e2[dv2 - 1]);
    }
    const T dsR1 = cR * dRm1, dsR2 = cR * dRm2, dcR1 = -sR * dRm1, dcR2 = -sR * dRm2;
    const T d2sR = -sR * dRm2 * dRm1 + cR * d2Rm, d2cR = -cR * dRm2 * dRm1 - sR * d2Rm;
    T a1[3][3], b1[3][3], b2[3][3], c1[3][3];  // a1 and its derivatives wrt dv1 (b1), dv2 (b2), both (c1)
    for (int k = 0; k < 3; ++k) {
        a1[0][k] = (T(1.0) / Rmag) * rot[k];
        b1[0][k] = (T(-1.0) / (Rmag * Rmag)) * dRm1 * rot[k] + (T(1.0) / Rmag) * e1[k];
        b2[0][k] = (T(-1.0) / (Rmag * Rmag)) * dRm2 * rot[k] + (T(1.0) / Rmag) * e2[k];
        T t = (2.0 * dRm1 * dRm2 / Rmag) * rot[k] - d2Rm * rot[k] - dRm1 * e2[k] - dRm2 * e1[k];
        c1[0][k] = (T(1.0) / (Rmag * Rmag)) * t;
    }
    int p = 0;
    if (absT(a1[0][1]) < absT(a1[0][0])) p = 1;
    if (absT(a1[0][2]) < absT(a1[0][p])) p = 2;
    a1[2][p] = b1[2][p] = b2[2][p] = c1[2][p] = T(0.0);
    a1[1][p] = a_sqrt(T(1.0) - a1[0][p] * a1[0][p]);
    const T q = a1[1][p];
    if (dv1 && !dv2) {
        b1[1][p] = -a1[0][p] * b1[0][p] / q;
    } else if (dv1 && dv2) {
        b1[1][p] = -a1[0][p] * b1[0][p] * (T(1.0) / q);
        b2[1][p] = -a1[0][p] * b2[0][p] * (T(1.0) / q);
        c1[1][p] = -(b2[0][p] * b1[0][p] + a1[0][p] * c1[0][p]) * (T(1.0) / q);
        c1[1][p] = c1[1][p] - a1[0][p] * b1[0][p] * a1[0][p] * b2[0][p] * (T(1.0) / (q * q * q));
    }
    for (int k = 0; k < 3; ++k) {
        if (k == p) continue;
        a1[1][k] = -a1[0][p] * a1[0][k] / q;
        if (dv1 && !dv2) {
            b1[1][k] = -b1[0][p] * a1[0][k] / q - a1[0][p] * b1[0][k] / q;
            b1[1][k] = b1[1][k] + a1[0][p] * a1[0][k] * b1[1][p] / (q * q);
        } else if (dv1 && dv2) {
            b1[1][k] = -b1[0][p] * a1[0][k] / q - a1[0][p] * b1[0][k] / q;
            b1[1][k] = b1[1][k] + a1[0][p] * a1[0][k] * b1[1][p] / (q * q);
            b2[1][k] = -b2[0][p] * a1[0][k] / q - a1[0][p] * b2[0][k] / q;
            b2[1][k] = b2[1][k] + a1[0][p] * a1[0][k] * b2[1][p] / (q * q);
            T t = -(c1[0][p] * a1[0][k] + b1[0][p] * b2[0][k]) / q;
            t = t - (b2[0][p] * b1[0][k] + a1[0][p] * c1[0][k]) / q;
            t = t + b1[0][p] * a1[0][k] * b2[1][p] / (q * q);
            t = t + a1[0][p] * b1[0][k] * b2[1][p] / (q * q);
            t = t + b2[0][p] * a1[0][k] * b1[1][p] / (q * q);
            t = t + a1[0][p] * b2[0][k] * b1[1][p] / (q * q);
            t = t + a1[0][p] * a1[0][k] * c1[1][p] / (q * q);
            t = t - 2.0 * a1[0][p] * a1[0][k] * b1[1][p] * b2[1][p] / (q * q * q);
            c1[1][k] = t;
        }
    }
    const int cp[3][2] = {{1, 2}, {2, 0}, {0, 1}};
    for (int k = 0; k < 3; ++k) {
        const int u = cp[k][0], v = cp[k][1];
        a1[2][k] = a1[0][u] * a1[1][v] - a1[0][v] * a1[1][u];
        b1[2][k] = b1[0][u] * a1[1][v] + a1[0][u] * b1[1][v] - b1[0][v] * a1[1][u] - a1[0][v] * b1[1][u];
        b2[2][k] = b2[0][u] * a1[1][v] + a1[0][u] * b2[1][v] - b2[0][v] * a1[1][u] - a1[0][v] * b2[1][u];
        T t = c1[0][u] * a1[1][v] + b1[0][u] * b2[1][v] + b2[0][u] * b1[1][v] + a1[0][u] * c1[1][v];
        c1[2][k] = t - c1[0][v] * a1[1][u] - b1[0][v] * b2[1][u] - b2[0][v] * b1[1][u] - a1[0][v] * c1[1][u];
    }
    // a2 = rotation of rows 2,3 of a1 by the angle |rot|, with derivatives
    T a2[3][3], g1[3][3], g2[3][3], h1[3][3];
    for (int k = 0; k < 3; ++k) {
        a2[0][k] = a1[0][k];
        g1[0][k] = b1[0][k];
        g2[0][k] = b2[0][k];
        h1[0][k] = c1[0][k];
        a2[1][k] = cR * a1[1][k] - sR * a1[2][k];
        g1[1][k] = dcR1 * a1[1][k] + cR * b1[1][k] - dsR1 * a1[2][k] - sR * b1[2][k];
        g2[1][k] = dcR2 * a1[1][k] + cR * b2[1][k] - dsR2 * a1[2][k] - sR * b2[2][k];
        h1[1][k] = d2cR * a1[1][k] + dcR1 * b2[1][k] + dcR2 * b1[1][k] + cR * c1[1][k];
        h1[1][k] = h1[1][k] - d2sR * a1[2][k] - dsR1 * b2[2][k] - dsR2 * b1[2][k] - sR * c1[2][k];
        a2[2][k] = sR * a1[1][k] + cR * a1[2][k];
        g1[2][k] = dsR1 * a1[1][k] + sR * b1[1][k] + dcR1 * a1[2][k] + cR * b1[2][k];
        g2[2][k] = dsR2 * a1[1][k] + sR * b2[1][k] + dcR2 * a1[2][k] + cR * b2[2][k];
        h1[2][k] = d2sR * a1[1][k] + dsR1 * b2[1][k] + dsR2 * b1[1][k] + sR * c1[1][k];
        h1[2][k] = h1[2][k] + d2cR * a1[2][k] + dcR1 * b2[2][k] + dcR2 * b1[2][k] + cR * c1[2][k];
    }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            T s = T(0.0);
            for (int k = 0; k < 3; ++k) {
                if (dv1 + dv2 == 0) s = s + a2[k][i] * a1[k][j];
                else if (dv1 * dv2 == 0) s = s + g1[k][i] * a1[k][j] + a2[k][i] * b1[k][j];
                else {
                    s = s + h1[k][i] * a1[k][j] + g1[k][i] * b2[k][j];
                    s = s + g2[k][i] * b1[k][j] + a2[k][i] * c1[k][j];
                }
            }
            M[i][j] = s;
        }
    // the exact branch applies the rotation on the right of aGL
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) out[i][j] = aGL[i][0] * M[0][j] + aGL[i][1] * M[1][j] + aGL[i][2] * M[2][j];
}
