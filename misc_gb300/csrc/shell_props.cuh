// shell4 section properties and element DOF table (device code).
#pragma once
#include "shell_math.cuh"


namespace {


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

// correctAlpha (Working/AStrO_r_elementEqns.f90:240-286, shell4 branch): the frame's third axis
// turned onto the normal of the element's diagonals (orient rows are the local axes).
template <class T> __device__ void shell_correct_alpha(T orient[3][3], const T X[4][3]) {
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

// Section properties of one element: orientation (r_getOrientation, designProp :187-221) with
// correctAlpha (:240-286), ABD by layer integration (r_getShellStiffness, :259-363) and section
// mass (r_getShellMass, :469-525).  The design-variable terms of the element (+ i h on
// `pertDvar`) enter as the reference applies them: orientation variables rotate the section frame,
// layer thickness, layer angle and layer density variables the layer's values, zOffset variables
// the section offset.
template <class T>
__device__ void shell_props(const double *nodes, const int *el, const double *secOrient, int sec, const int *layRange,
                            const LayerDev *lay, const double *zoff, const int *e2dR, const int *e2d, const double *e2c,
                            const int *dcat, const int *dlay, const int *dcomp, const double *dval, int e,
                            int pertDvar, double h, T orient[3][3], T ABD[9][9], T Ms[6][6]) {
    T X[4][3];
    for (int a = 0; a < 4; ++a)
        for (int k = 0; k < 3; ++k) X[a][k] = T(nodes[3 * (el[a] - 1) + k]);
    T al[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) al[i][j] = T(secOrient[9 * (sec - 1) + 3 * j + i]);  // column-major input
    // sum of the element's design-variable terms of one category (layer 0 = any)
    auto dsum = [&](int cat, int layerNum, int comp) {
        T s = T(0.0);
        if (e2dR)
            for (int q = e2dR[e]; q < e2dR[e + 1]; ++q) {
                const int d = e2d[q] - 1;
                if (dcat[d] != cat || (layerNum && dlay[d] != layerNum) || (comp && dcomp[d] != comp)) continue;
                T dv = T(dval[d]);
                if (d + 1 == pertDvar) dv = dv + pert_i<T>(h);
                s = s + e2c[q] * dv;
            }
        return s;
    };
    // r_getOrientation: the section frame rotated by globRot = alOrig^T locRot
    {
        T loc[3], gr[3];
        for (int k = 0; k < 3; ++k) loc[k] = dsum(ASTRO_DCAT_ORIENTATION, 0, k + 1);
        for (int i = 0; i < 3; ++i) gr[i] = al[0][i] * loc[0] + al[1][i] * loc[1] + al[2][i] * loc[2];
        a_rotate<T>(orient, al, gr, 0, 0);
    }
    shell_correct_alpha<T>(orient, X);
    // layer thicknesses with design variables
    const int l0 = layRange[sec - 1], l1 = layRange[sec];
    auto thick = [&](int li, int layerNum) { return T(lay[li].t) + dsum(ASTRO_DCAT_LAYUP_THICKNESS, layerNum, 0); };
    T secT = T(0.0);
    for (int li = l0, ln = 1; li < l1; ++li, ++ln) secT = secT + thick(li, ln);
    const T zo = T(zoff[sec - 1]) + dsum(ASTRO_DCAT_LAYUP_ZOFFSET, 0, 0);  // r_getElThickOffset
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
        // the layer's (E1, E2, nu12, G12) with its 'layup' modulus / poissonRatio / shearModulus terms
        const T E1 = T(L.E1) + dsum(ASTRO_DCAT_LAYUP_MODULUS, ln, 1), E2 = T(L.E2) + dsum(ASTRO_DCAT_LAYUP_MODULUS, ln, 2);
        const T nu12 = T(L.nu12) + dsum(ASTRO_DCAT_LAYUP_MODULUS, ln, 3), G12 = T(L.G12) + dsum(ASTRO_DCAT_LAYUP_MODULUS, ln, 4);
        T S[3][3] = {{T(1.0) / E1, -nu12 / E1, T(0.0)}, {-nu12 / E1, T(1.0) / E2, T(0.0)}, {T(0.0), T(0.0), T(1.0) / G12}};
        T Q[3][3];
        a_lu<T, 3>(&S[0][0], 3);
        for (int c = 0; c < 3; ++c) {
            T b[3] = {T(0.0), T(0.0), T(0.0)}, x[3];
            b[c] = T(1.0);
            a_lu_solve<T, 3>(&S[0][0], b, x, 3);
            for (int r = 0; r < 3; ++r) Q[r][c] = x[r];
        }
        const T ang = T(L.angle) + dsum(ASTRO_DCAT_LAYUP_ANGLE, ln, 0);
        const T a11 = a_cos(ang), a21 = a_sin(ang);
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
        const T rho = T(L.rho) + dsum(ASTRO_DCAT_LAYUP_DENSITY, ln, 0);
        const T m0 = rho * (zn2 - zm), m1 = 0.5 * rho * (zn2 * zn2 - zm * zm),
                m2 = AK<T>::o3 * rho * (zn2 * zn2 * zn2 - zm * zm * zm);
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

__global__ void shell_props_kernel(int E, const double *nodes, const int *elist, const int *esec, const double *secOrient,
                                   const int *layRange, const LayerDev *lay, const double *zoff, const int *e2dR,
                                   const int *e2d, const double *e2c, const int *dcat, const int *dlay,
                                   const int *dcomp, const double *dval, ShellProps *out) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    double o[3][3], ABD[9][9], M[6][6];
    shell_props<double>(nodes, elist + 8 * (size_t)e, secOrient, esec[e], layRange, lay, zoff, e2dR, e2d, e2c, dcat, dlay,
                        dcomp, dval, e, 0, 0.0, o, ABD, M);
    ShellProps &P = out[e];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) P.orient[3 * i + j] = o[i][j];
    for (int i = 0; i < 9; ++i)
        for (int j = 0; j < 9; ++j) P.ABD[9 * i + j] = ABD[i][j];
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) P.M[6 * i + j] = M[i][j];
}

}  // namespace
