// ORACLE (test infrastructure only): element stiffness/residual drivers and section properties,
// restated from Working/AStrO_r_elementEqns.f90 and Working/AStrO_r_designPropertyFunctions.f90
// (complex twins via T = std::complex<double>).  Thermal and beam terms are not restated: the
// configurations served here carry no temperature field, no thermal expansion and no beams, so
// those terms are identically zero in the reference as well.
#pragma once
#include "oracle_elements.hpp"
#include "../include/astro_gpu.h"

namespace orc {

// Per-element data gathered by r_getElementData (:552-578).
template <class T> struct ElemData {
    int eType, numNds, dofPerNd, numIntDof, numIntPts;
    int dofTable[33][2];
    T intPts[8][3];
    double ipWt[8];
    A2<T, 3, 10> locNds, globNds;
    A2<T, 3, 3> orient;
    A2<T, 6, 6> cMat, sMass;
    A2<T, 9, 9> ABD;
    T den;
    A2<T, 6, 11> disp, acc, pDisp, pVel, pAcc;
};

// Design-variable perturbation: which design variable (1-based, 0 = none) gets +i*h.
template <class T> struct DPert {
    int dvar = 0;
    double h = 0.0;
};

template <class T> static T dval(const astro_model *m, int d, const DPert<T> &p) {
    T v = T(m->d_value[d - 1]);
    if (d == p.dvar) v = v + pert_imag<T>(p.h);
    return v;
}

// sum over the element's design-variable terms of one category (and layer / component when
// given, 0 = any): elToCoef(i) * dVec(elToD(i)), the loops of r_getMaterialDensity (:96-101),
// r_getOrientation (:201-207), r_getElThickOffset (:249-255) and the layer loops of
// r_getShellStiffness / r_getShellMass (:289-303, :502-510)
template <class T>
static T el_dsum(const astro_model *m, int el, int cat, int layer, int comp, const DPert<T> &p) {
    T s = T(0.0);
    if (m->num_dvars <= 0 || !m->el_to_d_range) return s;
    for (int q = m->el_to_d_range[el - 1]; q < m->el_to_d_range[el]; ++q) {
        const int d = m->el_to_d[q];
        if (m->d_category[d - 1] != cat) continue;
        if (layer && (!m->d_layer || m->d_layer[d - 1] != layer)) continue;
        if (comp && (!m->d_component || m->d_component[d - 1] != comp)) continue;
        s = s + m->el_to_coef[q] * dval(m, d, p);
    }
    return s;
}

// the same over a node's terms (ndToD, r_getNodeCoord :958-964)
template <class T> static T nd_dsum(const astro_model *m, int node, int cat, int comp, const DPert<T> &p) {
    T s = T(0.0);
    if (m->num_dvars <= 0 || !m->nd_to_d_range) return s;
    for (int q = m->nd_to_d_range[node - 1]; q < m->nd_to_d_range[node]; ++q) {
        const int d = m->nd_to_d[q];
        if (m->d_category[d - 1] != cat) continue;
        if (comp && (!m->d_component || m->d_component[d - 1] != comp)) continue;
        s = s + m->nd_to_coef[q] * dval(m, d, p);
    }
    return s;
}

// r_getElementProfile, Working/AStrO_r_elementEqns.f90:334-449 (types 8, 81 and 41)
template <class T> static int t_getElementProfile(ElemData<T> &e, int eType) {
    std::memset(e.dofTable, 0, sizeof(e.dofTable));
    const double rt3 = KC<T>::rt3();
    e.eType = eType;
    if (eType == 8 || eType == 81) {
        e.numNds = 8;
        e.dofPerNd = 3;
        e.numIntDof = (eType == 81) ? 9 : 0;
        e.numIntPts = 8;
        const int sg[8][3] = {{-1, -1, -1}, {1, -1, -1}, {-1, 1, -1}, {1, 1, -1},
                              {-1, -1, 1},  {1, -1, 1},  {-1, 1, 1},  {1, 1, 1}};
        for (int g = 0; g < 8; ++g) {
            for (int k = 0; k < 3; ++k) e.intPts[g][k] = T(rt3 * (double)sg[g][k]);
            e.ipWt[g] = 1.0;
        }
        if (eType == 81) {  // internal DOF 25..33: component-major over the bubbles 9..11 (:390-397)
            int i3 = 24;
            for (int i1 = 1; i1 <= 3; ++i1)
                for (int i2 = 9; i2 <= 11; ++i2) {
                    e.dofTable[i3][0] = i1;
                    e.dofTable[i3][1] = i2;
                    ++i3;
                }
        }
    } else if (eType == 41) {
        e.numNds = 4;
        e.dofPerNd = 6;
        e.numIntDof = 8;
        e.numIntPts = 4;
        const int sg[4][2] = {{-1, -1}, {1, -1}, {-1, 1}, {1, 1}};
        for (int g = 0; g < 4; ++g) {
            e.intPts[g][0] = T(rt3 * (double)sg[g][0]);
            e.intPts[g][1] = T(rt3 * (double)sg[g][1]);
            e.intPts[g][2] = T(0.0);
            e.ipWt[g] = 1.0;
        }
        const int it[8][2] = {{1, 5}, {1, 6}, {2, 5}, {2, 6}, {3, 7}, {3, 8}, {3, 9}, {3, 10}};
        for (int k = 0; k < 8; ++k) {
            e.dofTable[24 + k][0] = it[k][0];
            e.dofTable[24 + k][1] = it[k][1];
        }
    } else {
        return -1;
    }
    int i3 = 0;
    for (int i1 = 1; i1 <= e.dofPerNd; ++i1)
        for (int i2 = 1; i2 <= e.numNds; ++i2) {
            e.dofTable[i3][0] = i1;
            e.dofTable[i3][1] = i2;
            ++i3;
        }
    return 0;
}

// correctAlpha, Working/AStrO_r_elementEqns.f90:240-286 (shell4 branch)
template <class T> static void t_correctAlpha(A2<T, 3, 3> &alpha, const A2<T, 3, 10> &nodes) {
    A1<T, 3> v1, v2, v3;
    for (int k = 1; k <= 3; ++k) {
        v1(k) = nodes(k, 3) - nodes(k, 1);
        v2(k) = nodes(k, 4) - nodes(k, 2);
    }
    v3(1) = v1(2) * v2(3) - v1(3) * v2(2);
    v3(2) = v1(3) * v2(1) - v1(1) * v2(3);
    v3(3) = v1(1) * v2(2) - v1(2) * v2(1);
    for (int k = 1; k <= 3; ++k) v1(k) = alpha(3, k);
    T dp = v1(1) * v3(1) + v1(2) * v3(2) + v1(3) * v3(3);
    if (t_greater(T(0.0), dp))
        for (int k = 1; k <= 3; ++k) v3(k) = -v3(k);
    dp = v3(1) * v3(1) + v3(2) * v3(2) + v3(3) * v3(3);
    T mag = t_sqrt(dp);
    for (int k = 1; k <= 3; ++k) v2(k) = (T(1.0) / mag) * v3(k);
    v3(1) = v1(2) * v2(3) - v1(3) * v2(2);
    v3(2) = v1(3) * v2(1) - v1(1) * v2(3);
    v3(3) = v1(1) * v2(2) - v1(2) * v2(1);
    dp = v3(1) * v3(1) + v3(2) * v3(2) + v3(3) * v3(3);
    mag = t_sqrt(dp);
    if (absT(mag) > F(1e-5)) {
        T theta = t_asin(mag);
        for (int k = 1; k <= 3; ++k) v3(k) = (theta / mag) * v3(k);
        A2<T, 3, 3> alpha0 = alpha;
        t_rotateAlpha(alpha, alpha0, v3, 0, 0);
    }
}

// r_getMaterialStiffness, Working/AStrO_r_designPropertyFunctions.f90:8-80 (engineering-constant
// branch; C = S^-1 by the reference's unpivoted LU).
template <class T>
static void t_getMaterialStiffness(A2<T, 6, 6> &CMat, const astro_model *m, int el, const DPert<T> &p) {
    int sec = m->element_section[el - 1];
    int mat = m->section_mat_id[sec - 1];
    T eProps[9];
    for (int k = 0; k < 9; ++k) eProps[k] = T(m->material_elastic[9 * (mat - 1) + k]);
    if (m->num_dvars > 0 && m->el_to_d_range) {
        for (int i1 = m->el_to_d_range[el - 1] + 1; i1 <= m->el_to_d_range[el]; ++i1) {
            int d = m->el_to_d[i1 - 1];
            if (m->d_category[d - 1] == ASTRO_DCAT_ELASTIC_MODULUS) {
                int i3 = m->d_component[d - 1];
                eProps[i3 - 1] = eProps[i3 - 1] + m->el_to_coef[i1 - 1] * dval(m, d, p);
            }
        }
    }
    A2<T, 6, 6> S;
    S.fill(T(0.0));
    S(1, 1) = T(1.0) / eProps[0];
    S(1, 2) = -eProps[3] / eProps[0];
    S(1, 3) = -eProps[4] / eProps[0];
    S(2, 2) = T(1.0) / eProps[1];
    S(2, 3) = -eProps[5] / eProps[1];
    S(3, 3) = T(1.0) / eProps[2];
    S(4, 4) = T(1.0) / eProps[6];
    S(5, 5) = T(1.0) / eProps[7];
    S(6, 6) = T(1.0) / eProps[8];
    for (int i1 = 2; i1 <= 6; ++i1)
        for (int i2 = 1; i2 <= i1 - 1; ++i2) S(i1, i2) = S(i2, i1);
    CMat.fill(T(0.0));
    t_GetInvLU(&CMat(1, 1), &S(1, 1), 6, 1, 6);
}

// r_getElThickOffset (:223-257), r_getShellStiffness (:259-363), r_getShellMass (:469-525)
template <class T>
static T layer_thickness(const astro_model *m, int el, int layerNum, int layerIdx, const DPert<T> &p) {
    T t = T(m->layup_thickness[layerIdx - 1]);
    if (m->num_dvars > 0 && m->el_to_d_range) {
        for (int i2 = m->el_to_d_range[el - 1] + 1; i2 <= m->el_to_d_range[el]; ++i2) {
            int d = m->el_to_d[i2 - 1];
            if (m->d_category[d - 1] == ASTRO_DCAT_LAYUP_THICKNESS && m->d_layer[d - 1] == layerNum)
                t = t + m->el_to_coef[i2 - 1] * dval(m, d, p);
        }
    }
    return t;
}

template <class T>
static void t_getShellStiffness(A2<T, 9, 9> &ABD, const astro_model *m, int el, const DPert<T> &p) {
    int sec = m->element_section[el - 1];
    int l0 = m->sec_layup_range[sec - 1], l1 = m->sec_layup_range[sec];
    T secThick = T(0.0);
    for (int i1 = l0 + 1, ln = 1; i1 <= l1; ++i1, ++ln) secThick = secThick + layer_thickness(m, el, ln, i1, p);
    T zOff = T(m->section_z_offset[sec - 1]) + el_dsum(m, el, ASTRO_DCAT_LAYUP_ZOFFSET, 0, 0, p);
    ABD.fill(T(0.0));
    T zCrd = -0.5 * secThick * (zOff + T(1.0));
    int layerNum = 0;
    for (int i1 = l0 + 1; i1 <= l1; ++i1) {
        layerNum++;
        int mat = m->layup_mat_id[i1 - 1];
        T lp[6];
        // layerProps(1:4) = (E1, E2, nu12, G12) with the layer's 'layup' modulus (dComponent),
        // poissonRatio (3) and shearModulus (4) terms (:289-303)
        lp[0] = T(m->material_elastic[9 * (mat - 1) + 0]) + el_dsum(m, el, ASTRO_DCAT_LAYUP_MODULUS, layerNum, 1, p);
        lp[1] = T(m->material_elastic[9 * (mat - 1) + 1]) + el_dsum(m, el, ASTRO_DCAT_LAYUP_MODULUS, layerNum, 2, p);
        lp[2] = T(m->material_elastic[9 * (mat - 1) + 3]) + el_dsum(m, el, ASTRO_DCAT_LAYUP_MODULUS, layerNum, 3, p);
        lp[3] = T(m->material_elastic[9 * (mat - 1) + 6]) + el_dsum(m, el, ASTRO_DCAT_LAYUP_MODULUS, layerNum, 4, p);
        lp[4] = layer_thickness(m, el, layerNum, i1, p);
        lp[5] = T(m->layup_angle[i1 - 1]) + el_dsum(m, el, ASTRO_DCAT_LAYUP_ANGLE, layerNum, 0, p);
        T zNext = zCrd + lp[4];
        A2<T, 3, 3> S, Q, Ts, Te, TeInv;
        S.fill(T(0.0));
        S(1, 1) = T(1.0) / lp[0];
        S(1, 2) = -lp[2] / lp[0];
        S(2, 2) = T(1.0) / lp[1];
        S(3, 3) = T(1.0) / lp[3];
        S(2, 1) = S(1, 2);
        Q.fill(T(0.0));
        t_GetInvLU(&Q(1, 1), &S(1, 1), 3, 1, 3);
        T a11 = t_cos(lp[5]);
        T a21 = t_sin(lp[5]);
        T a12 = -a21, a22 = a11;
        Ts(1, 1) = a11 * a11;
        Ts(1, 2) = a12 * a12;
        Ts(1, 3) = 2.0 * a11 * a12;
        Ts(2, 1) = a21 * a21;
        Ts(2, 2) = a22 * a22;
        Ts(2, 3) = 2.0 * a22 * a21;
        Ts(3, 1) = a11 * a21;
        Ts(3, 2) = a12 * a22;
        Ts(3, 3) = a11 * a22 + a12 * a21;
        Te = Ts;
        for (int k = 1; k <= 3; ++k) Te(k, 3) = 0.5 * Te(k, 3);
        for (int k = 1; k <= 3; ++k) Te(3, k) = 2.0 * Te(3, k);
        TeInv.fill(T(0.0));
        t_GetInvLU(&TeInv(1, 1), &Te(1, 1), 3, 1, 3);
        Te.fill(T(0.0));
        for (int i2 = 1; i2 <= 3; ++i2)
            for (int i3 = 1; i3 <= 3; ++i3)
                for (int i4 = 1; i4 <= 3; ++i4) Te(i2, i3) = Te(i2, i3) + Q(i2, i4) * TeInv(i4, i3);
        Q.fill(T(0.0));
        for (int i2 = 1; i2 <= 3; ++i2)
            for (int i3 = 1; i3 <= 3; ++i3)
                for (int i4 = 1; i4 <= 3; ++i4) Q(i2, i3) = Q(i2, i3) + Ts(i2, i4) * Te(i4, i3);
        T f0 = zNext - zCrd, f1 = 0.5 * (zNext * zNext - zCrd * zCrd);
        T f2 = KC<T>::o3() * (zNext * zNext * zNext - zCrd * zCrd * zCrd);
        for (int i = 1; i <= 3; ++i)
            for (int j = 1; j <= 3; ++j) {
                ABD(i, j) = ABD(i, j) + f0 * Q(i, j);
                ABD(i, j + 3) = ABD(i, j + 3) + f1 * Q(i, j);
                ABD(i + 3, j + 3) = ABD(i + 3, j + 3) + f2 * Q(i, j);
            }
        zCrd = zNext;
    }
    for (int i1 = 2; i1 <= 6; ++i1)
        for (int i2 = 1; i2 <= i1 - 1; ++i2) ABD(i1, i2) = ABD(i2, i1);
    ABD(7, 7) = ABD(3, 3);
    ABD(8, 8) = ABD(3, 3);
    ABD(9, 9) = ABD(3, 3);
}

template <class T>
static void t_getShellMass(A2<T, 6, 6> &M, const astro_model *m, int el, const DPert<T> &p) {
    int sec = m->element_section[el - 1];
    int l0 = m->sec_layup_range[sec - 1], l1 = m->sec_layup_range[sec];
    T secThick = T(0.0);
    for (int i1 = l0 + 1, ln = 1; i1 <= l1; ++i1, ++ln) secThick = secThick + layer_thickness(m, el, ln, i1, p);
    T zOff = T(m->section_z_offset[sec - 1]) + el_dsum(m, el, ASTRO_DCAT_LAYUP_ZOFFSET, 0, 0, p);
    M.fill(T(0.0));
    T zCrd = -0.5 * secThick * (zOff + T(1.0));
    int layerNum = 0;
    for (int i1 = l0 + 1; i1 <= l1; ++i1) {
        layerNum++;
        int mat = m->layup_mat_id[i1 - 1];
        T den = T(m->material_density[mat - 1]) + el_dsum(m, el, ASTRO_DCAT_LAYUP_DENSITY, layerNum, 0, p);
        T th = layer_thickness(m, el, layerNum, i1, p);
        T zNext = zCrd + th;
        T f0 = den * (zNext - zCrd), f1 = 0.5 * den * (zNext * zNext - zCrd * zCrd);
        T f2 = KC<T>::o3() * den * (zNext * zNext * zNext - zCrd * zCrd * zCrd);
        for (int k = 1; k <= 3; ++k) {
            M(k, k) = M(k, k) + f0;
            M(k + 3, k + 3) = M(k + 3, k + 3) + f2;
        }
        // unitB(1,2) = 1, unitB(2,1) = -1 in the (1:3,4:6) block
        M(1, 5) = M(1, 5) + f1;
        M(2, 4) = M(2, 4) - f1;
        zCrd = zNext;
    }
    for (int i1 = 2; i1 <= 6; ++i1)
        for (int i2 = 1; i2 <= i1 - 1; ++i2) M(i1, i2) = M(i2, i1);
}

// Nodal state of the model in global DOF numbering (NULL = zeros).
struct GState {
    const double *disp = nullptr, *vel = nullptr, *acc = nullptr;
    const double *pdisp = nullptr, *pvel = nullptr, *pacc = nullptr;
    const double *intDisp = nullptr, *pIntDisp = nullptr;
    int dynamic = 0;
    double beta = 0.25, gamma = 0.5, delT = 0.0;
};

// r_getElementData (:552-578) = profile + properties (:451-498) + solution gather (:500-550, Q5
// resolved: global node for nDofIndex, vel/acc not swapped).
template <class T>
static int t_getElementData(ElemData<T> &e, const astro_model *m, const int *nDofIndex, const int *intVecRange,
                            int el, const GState &s, const DPert<T> &p) {
    int eType = m->element_type[el - 1];
    if (t_getElementProfile(e, eType) != 0) return -1;
    // r_getNodeCoord (designProp :945-968): unused columns stay 1.0; nodeCoord design variables
    // move coordinate dComponent of their nodes
    e.globNds.fill(T(1.0));
    for (int i1 = 1; i1 <= 8; ++i1) {
        int nd = m->element_list[8 * (el - 1) + i1 - 1];
        if (nd > 0)
            for (int k = 1; k <= 3; ++k)
                e.globNds(k, i1) = T(m->node_list[3 * (nd - 1) + k - 1]) + nd_dsum(m, nd, ASTRO_DCAT_NODE_COORD, k, p);
    }
    // r_getOrientation (:187-221): the section orientation rotated by the orientation design
    // variables' local rotation vector, expressed in global axes (globRot = alOrig^T locRot)
    int sec = m->element_section[el - 1];
    A2<T, 3, 3> alOrig;
    for (int j = 1; j <= 3; ++j)
        for (int i = 1; i <= 3; ++i) alOrig(i, j) = T(m->section_orient[9 * (sec - 1) + 3 * (j - 1) + (i - 1)]);
    A1<T, 3> locRot, globRot;
    for (int k = 1; k <= 3; ++k) locRot(k) = el_dsum(m, el, ASTRO_DCAT_ORIENTATION, 0, k, p);
    for (int i1 = 1; i1 <= 3; ++i1) {
        globRot(i1) = T(0.0);
        for (int i2 = 1; i2 <= 3; ++i2) globRot(i1) = globRot(i1) + alOrig(i2, i1) * locRot(i2);
    }
    t_rotateAlpha(e.orient, alOrig, globRot, 0, 0);
    if (eType == 41) t_correctAlpha(e.orient, e.globNds);
    e.locNds.fill(T(0.0));
    for (int i1 = 1; i1 <= 3; ++i1)
        for (int i2 = 1; i2 <= 10; ++i2)
            for (int i3 = 1; i3 <= 3; ++i3) e.locNds(i1, i2) = e.locNds(i1, i2) + e.orient(i1, i3) * e.globNds(i3, i2);
    if (eType == 8 || eType == 81) {
        t_getMaterialStiffness(e.cMat, m, el, p);
        int mat = m->section_mat_id[sec - 1];
        e.den = T(m->material_density ? m->material_density[mat - 1] : 0.0) +
                el_dsum(m, el, ASTRO_DCAT_DENSITY, 0, 0, p);  // r_getMaterialDensity (:82-103)
        e.ABD.fill(T(0.0));
        e.sMass.fill(T(0.0));
    } else {
        e.cMat.fill(T(0.0));
        t_getShellStiffness(e.ABD, m, el, p);
        t_getShellMass(e.sMass, m, el, p);
        e.den = T(0.0);
    }
    // state gather
    e.disp.fill(T(0.0));
    e.acc.fill(T(0.0));
    e.pDisp.fill(T(0.0));
    e.pVel.fill(T(0.0));
    e.pAcc.fill(T(0.0));
    for (int i1 = 1; i1 <= e.numNds; ++i1) {
        int nd = m->element_list[8 * (el - 1) + i1 - 1];
        for (int i2 = 1; i2 <= e.dofPerNd; ++i2) {
            int i4 = nDofIndex[6 * (nd - 1) + i2 - 1];
            if (i4 <= 0) continue;
            if (s.pdisp) e.pDisp(i2, i1) = T(s.pdisp[i4 - 1]);
            if (s.pacc) e.pAcc(i2, i1) = T(s.pacc[i4 - 1]);
            if (s.pvel) e.pVel(i2, i1) = T(s.pvel[i4 - 1]);
            if (s.disp) e.disp(i2, i1) = T(s.disp[i4 - 1]);
            if (s.acc) e.acc(i2, i1) = T(s.acc[i4 - 1]);
        }
    }
    if (e.numIntDof != 0) {
        int i1 = intVecRange[el - 1];
        int i2 = e.numNds * e.dofPerNd;
        for (int i3 = 1; i3 <= e.numIntDof; ++i3) {
            int i4 = i2 + i3;
            int i5 = e.dofTable[i4 - 1][0], i6 = e.dofTable[i4 - 1][1];
            if (s.intDisp) e.disp(i5, i6) = T(s.intDisp[i1 + i3 - 1]);
            if (s.pIntDisp) e.pDisp(i5, i6) = T(s.pIntDisp[i1 + i3 - 1]);
        }
    }
    return 0;
}

// r_getElRuk, Working/AStrO_r_elementEqns.f90:2206-2533 (shell4 and brick8 branches; Q3 resolved
// to i3 = 0; thermal terms zero).
template <class T>
static void t_getElRuk(A1<T, 33> &Ruk, A2<T, 33, 33> &dRdU, int buildMat, const ElemData<T> &e,
                       const A2<T, 6, 11> &disp) {
    const int eType = e.eType, numNds = e.numNds;
    A2<T, 9, 33> dedU, cdedU;
    A2<T, 3, 48> instOri;
    A2<T, 3, 16> drIdrG;
    A1<T, 3> elRot, ptRot;
    A2<T, 6, 11> instDofMat;
    A1<T, 11> Nvec;
    A2<T, 11, 3> Nx;
    T detJ;
    A2<T, 3, 3> ux, rx;
    A1<T, 9> shDef, shFrcMom;
    if (eType == 41) {
        elRot.fill(T(0.0));
        for (int i1 = 1; i1 <= numNds; ++i1)
            for (int k = 1; k <= 3; ++k) elRot(k) = elRot(k) + disp(3 + k, i1);
        for (int k = 1; k <= 3; ++k) elRot(k) = (T(1.0) / (double)numNds) * elRot(k);
        t_getInstOrient(instOri, drIdrG, e.orient, elRot);
    }
    Ruk.fill(T(0.0));
    dRdU.fill(T(0.0));
    dedU.fill(T(0.0));
    const int ndof = e.numNds * e.dofPerNd + e.numIntDof;
    for (int i1 = 1; i1 <= e.numIntPts; ++i1) {
        t_getIntPtData(Nvec, Nx, detJ, e.locNds, e.intPts[i1 - 1], eType, numNds);
        const T wdet = detJ * e.ipWt[i1 - 1];
        if (eType == 41) {
            t_getInstDof(instDofMat, disp, e.globNds, instOri, e.orient, elRot, drIdrG, numNds, e.dofTable, 0, 0);
            ptRot.fill(T(0.0));
            for (int i2 = 1; i2 <= numNds; ++i2)
                for (int i3 = 1; i3 <= 3; ++i3) ptRot(i3) = ptRot(i3) + instDofMat(3 + i3, i2) * Nvec(i2);
            ux.fill(T(0.0));
            rx.fill(T(0.0));
            for (int i2 = 1; i2 <= 3; ++i2)
                for (int i3 = 1; i3 <= 3; ++i3)
                    for (int i4 = 1; i4 <= 10; ++i4) {
                        ux(i2, i3) = ux(i2, i3) + instDofMat(i2, i4) * Nx(i4, i3);
                        rx(i2, i3) = rx(i2, i3) + instDofMat(i2 + 3, i4) * Nx(i4, i3);
                    }
            t_getShellDef(shDef, ux, ptRot, rx);
            shFrcMom.fill(T(0.0));
            for (int i2 = 1; i2 <= 9; ++i2)
                for (int i3 = 1; i3 <= 9; ++i3) shFrcMom(i2) = shFrcMom(i2) + e.ABD(i2, i3) * shDef(i3);
            for (int i4 = 1; i4 <= ndof; ++i4) {
                t_getInstDof(instDofMat, disp, e.globNds, instOri, e.orient, elRot, drIdrG, numNds, e.dofTable, i4, 0);
                ptRot.fill(T(0.0));
                for (int i5 = 1; i5 <= numNds; ++i5)
                    for (int k = 1; k <= 3; ++k) ptRot(k) = ptRot(k) + instDofMat(3 + k, i5) * Nvec(i5);
                ux.fill(T(0.0));
                rx.fill(T(0.0));
                if (e.dofTable[i4 - 1][0] < 4) {
                    int i7 = e.dofTable[i4 - 1][1];
                    for (int i5 = 1; i5 <= 3; ++i5)
                        for (int i6 = 1; i6 <= 3; ++i6) ux(i5, i6) = ux(i5, i6) + instDofMat(i5, i7) * Nx(i7, i6);
                } else {
                    for (int i6 = 1; i6 <= 3; ++i6)
                        for (int i7 = 1; i7 <= 3; ++i7)
                            for (int i8 = 1; i8 <= numNds; ++i8) ux(i6, i7) = ux(i6, i7) + instDofMat(i6, i8) * Nx(i8, i7);
                    int i5 = e.dofTable[i4 - 1][1];
                    if (g_quirk_mean_rot_derivative) {  // diagnostic switch only, see oracle_elements.hpp
                        for (int j = 1; j <= numNds; ++j)
                            for (int i6 = 1; i6 <= 3; ++i6)
                                for (int i7 = 1; i7 <= 3; ++i7) rx(i6, i7) = rx(i6, i7) + instDofMat(i6 + 3, j) * Nx(j, i7);
                    } else {
                        for (int i6 = 1; i6 <= 3; ++i6)
                            for (int i7 = 1; i7 <= 3; ++i7) rx(i6, i7) = rx(i6, i7) + instDofMat(i6 + 3, i5) * Nx(i5, i7);
                    }
                }
                t_getShellDef(shDef, ux, ptRot, rx);
                if (buildMat == 1)
                    for (int k = 1; k <= 9; ++k) dedU(k, i4) = shDef(k);
                for (int k = 1; k <= 9; ++k) shDef(k) = wdet * shDef(k);
                for (int i5 = 1; i5 <= 9; ++i5) Ruk(i4) = Ruk(i4) + shFrcMom(i5) * shDef(i5);
                if (buildMat == 1) {
                    for (int i10 = i4; i10 <= ndof; ++i10) {
                        t_getInstDof(instDofMat, disp, e.globNds, instOri, e.orient, elRot, drIdrG, numNds, e.dofTable, i4,
                                     i10);
                        ptRot.fill(T(0.0));
                        for (int i5 = 1; i5 <= numNds; ++i5)
                            for (int k = 1; k <= 3; ++k) ptRot(k) = ptRot(k) + instDofMat(3 + k, i5) * Nvec(i5);
                        int var1, nd1, var2, nd2;
                        if (e.dofTable[i4 - 1][0] < e.dofTable[i10 - 1][0]) {
                            var1 = e.dofTable[i4 - 1][0];
                            nd1 = e.dofTable[i4 - 1][1];
                            var2 = e.dofTable[i10 - 1][0];
                            nd2 = e.dofTable[i10 - 1][1];
                        } else {
                            var1 = e.dofTable[i10 - 1][0];
                            nd1 = e.dofTable[i10 - 1][1];
                            var2 = e.dofTable[i4 - 1][0];
                            nd2 = e.dofTable[i4 - 1][1];
                        }
                        ux.fill(T(0.0));
                        rx.fill(T(0.0));
                        if (var1 < 4 && var2 >= 4) {
                            for (int i5 = 1; i5 <= 3; ++i5)
                                for (int i6 = 1; i6 <= 3; ++i6) {
                                    ux(i5, i6) = ux(i5, i6) + instDofMat(i5, nd1) * Nx(nd1, i6);
                                    rx(i5, i6) = rx(i5, i6) + instDofMat(i5 + 3, nd2) * Nx(nd2, i6);
                                }
                        } else if (var1 >= 4 && var2 >= 4) {
                            for (int i6 = 1; i6 <= 3; ++i6)
                                for (int i7 = 1; i7 <= 3; ++i7)
                                    for (int i8 = 1; i8 <= numNds; ++i8)
                                        ux(i6, i7) = ux(i6, i7) + instDofMat(i6, i8) * Nx(i8, i7);
                            if (nd1 == nd2)
                                for (int i6 = 1; i6 <= 3; ++i6)
                                    for (int i7 = 1; i7 <= 3; ++i7)
                                        rx(i6, i7) = rx(i6, i7) + instDofMat(i6 + 3, nd1) * Nx(nd1, i7);
                        }
                        t_getShellDef(shDef, ux, ptRot, rx);
                        for (int k = 1; k <= 9; ++k) shDef(k) = wdet * shDef(k);
                        for (int i5 = 1; i5 <= 9; ++i5) dRdU(i4, i10) = dRdU(i4, i10) + shFrcMom(i5) * shDef(i5);
                        dRdU(i10, i4) = dRdU(i4, i10);
                    }
                }
            }
        } else {
            A1<T, 6> strain, stress;
            ux.fill(T(0.0));
            for (int i2 = 1; i2 <= 3; ++i2)
                for (int i3 = 1; i3 <= 3; ++i3)
                    for (int i4 = 1; i4 <= 11; ++i4) ux(i2, i3) = ux(i2, i3) + disp(i2, i4) * Nx(i4, i3);
            t_getNLStrain(strain, ux, Nx, e.orient, 0, 0, e.dofTable);
            stress.fill(T(0.0));
            for (int i2 = 1; i2 <= 6; ++i2)
                for (int i3 = 1; i3 <= 6; ++i3) stress(i2) = stress(i2) + e.cMat(i2, i3) * strain(i3);
            for (int i3 = 1; i3 <= ndof; ++i3) {
                t_getNLStrain(strain, ux, Nx, e.orient, i3, 0, e.dofTable);
                if (buildMat == 1)
                    for (int k = 1; k <= 6; ++k) dedU(k, i3) = strain(k);
                for (int k = 1; k <= 6; ++k) strain(k) = wdet * strain(k);
                for (int i4 = 1; i4 <= 6; ++i4) Ruk(i3) = Ruk(i3) + stress(i4) * strain(i4);
                for (int i5 = i3; i5 <= ndof; ++i5) {
                    t_getNLStrain(strain, ux, Nx, e.orient, i3, i5, e.dofTable);
                    for (int k = 1; k <= 6; ++k) strain(k) = wdet * strain(k);
                    for (int i4 = 1; i4 <= 6; ++i4) dRdU(i3, i5) = dRdU(i3, i5) + stress(i4) * strain(i4);
                    dRdU(i5, i3) = dRdU(i3, i5);
                }
            }
        }
        if (buildMat == 1) {
            const int nr = (eType == 41) ? 9 : 6;
            cdedU.fill(T(0.0));
            for (int i2 = 1; i2 <= nr; ++i2)
                for (int i3 = 1; i3 <= ndof; ++i3)
                    for (int i4 = 1; i4 <= nr; ++i4) {
                        T c = (eType == 41) ? e.ABD(i2, i4) : e.cMat(i2, i4);
                        cdedU(i2, i3) = cdedU(i2, i3) + c * dedU(i4, i3);
                    }
            for (int i2 = 1; i2 <= nr; ++i2)
                for (int i3 = 1; i3 <= ndof; ++i3) cdedU(i2, i3) = wdet * cdedU(i2, i3);
            for (int i2 = 1; i2 <= ndof; ++i2)
                for (int i3 = 1; i3 <= ndof; ++i3)
                    for (int i4 = 1; i4 <= nr; ++i4) dRdU(i2, i3) = dRdU(i2, i3) + dedU(i4, i2) * cdedU(i4, i3);
        }
    }
}

// r_getElRum, Working/AStrO_r_elementEqns.f90:2535-2657
template <class T>
static void t_getElRum(A1<T, 33> &Rum, A2<T, 33, 33> &dRdA, int buildMat, const ElemData<T> &e,
                       const A2<T, 3, 48> &statInOri, const A2<T, 3, 16> &statdrIdrG, const A1<T, 3> &statRot,
                       const A2<T, 6, 11> &disp, const A2<T, 6, 11> &acc) {
    const int eType = e.eType, numNds = e.numNds;
    static thread_local A2<T, 6, 11> blk[25];  // blk[0]: (0,0), blk[i]: derivative wrt DOF i
    A2<T, 6, 4> instNodalAcc, iNAM;
    A1<T, 11> Nvec;
    A2<T, 11, 3> Nx;
    T detJ;
    A2<T, 6, 33> dudU, MdudU;
    const int nn = numNds * e.dofPerNd;
    if (eType == 41) {
        t_getInstDof(blk[0], disp, e.globNds, statInOri, e.orient, statRot, statdrIdrG, numNds, e.dofTable, 0, 0);
        instNodalAcc.fill(T(0.0));
        for (int i2 = 1; i2 <= nn; ++i2) {
            t_getInstDof(blk[i2], disp, e.globNds, statInOri, e.orient, statRot, statdrIdrG, numNds, e.dofTable, i2, 0);
            int i4 = e.dofTable[i2 - 1][0], i5 = e.dofTable[i2 - 1][1];
            for (int c = 1; c <= 4; ++c)
                for (int r = 1; r <= 6; ++r) instNodalAcc(r, c) = instNodalAcc(r, c) + acc(i4, i5) * blk[i2](r, c);
        }
        iNAM.fill(T(0.0));
        for (int i1 = 1; i1 <= 6; ++i1)
            for (int i2 = 1; i2 <= numNds; ++i2)
                for (int i3 = 1; i3 <= 6; ++i3) iNAM(i1, i2) = iNAM(i1, i2) + e.sMass(i1, i3) * instNodalAcc(i3, i2);
    }
    Rum.fill(T(0.0));
    dRdA.fill(T(0.0));
    for (int i1 = 1; i1 <= e.numIntPts; ++i1) {
        t_getIntPtData(Nvec, Nx, detJ, e.locNds, e.intPts[i1 - 1], eType, numNds);
        const T wdet = detJ * e.ipWt[i1 - 1];
        if (eType == 41) {
            A1<T, 6> inerFrc, delU;
            inerFrc.fill(T(0.0));
            for (int i2 = 1; i2 <= 6; ++i2)
                for (int i3 = 1; i3 <= numNds; ++i3) inerFrc(i2) = inerFrc(i2) + iNAM(i2, i3) * Nvec(i3);
            for (int i4 = 1; i4 <= nn; ++i4) {
                delU.fill(T(0.0));
                for (int i5 = 1; i5 <= 6; ++i5)
                    for (int i6 = 1; i6 <= numNds; ++i6) delU(i5) = delU(i5) + blk[i4](i5, i6) * Nvec(i6);
                if (buildMat == 1)
                    for (int k = 1; k <= 6; ++k) dudU(k, i4) = delU(k);
                for (int k = 1; k <= 6; ++k) delU(k) = wdet * delU(k);
                for (int i5 = 1; i5 <= 6; ++i5) Rum(i4) = Rum(i4) + inerFrc(i5) * delU(i5);
            }
            if (buildMat == 1) {
                MdudU.fill(T(0.0));
                for (int i4 = 1; i4 <= 6; ++i4)
                    for (int i5 = 1; i5 <= nn; ++i5)
                        for (int i6 = 1; i6 <= 6; ++i6) MdudU(i4, i5) = MdudU(i4, i5) + e.sMass(i4, i6) * dudU(i6, i5);
                for (int i4 = 1; i4 <= 6; ++i4)
                    for (int i5 = 1; i5 <= nn; ++i5) MdudU(i4, i5) = wdet * MdudU(i4, i5);
                for (int i4 = 1; i4 <= nn; ++i4)
                    for (int i5 = 1; i5 <= nn; ++i5)
                        for (int i6 = 1; i6 <= 6; ++i6) dRdA(i4, i5) = dRdA(i4, i5) + dudU(i6, i4) * MdudU(i6, i5);
            }
        } else {
            dudU.fill(T(0.0));
            for (int i3 = 1; i3 <= nn; ++i3) {
                int i4 = e.dofTable[i3 - 1][0], i5 = e.dofTable[i3 - 1][1];
                T accI = T(0.0);
                for (int i6 = 1; i6 <= 11; ++i6) accI = accI + acc(i4, i6) * Nvec(i6);
                accI = wdet * accI;
                Rum(i3) = Rum(i3) + e.den * accI * Nvec(i5);
                if (buildMat == 1) dudU(i4, i3) = Nvec(i5);
            }
            if (buildMat == 1) {
                for (int r = 1; r <= 6; ++r)
                    for (int c = 1; c <= 33; ++c) MdudU(r, c) = (e.den * detJ * e.ipWt[i1 - 1]) * dudU(r, c);
                for (int i4 = 1; i4 <= nn; ++i4)
                    for (int i5 = 1; i5 <= nn; ++i5)
                        for (int i6 = 1; i6 <= 3; ++i6) dRdA(i4, i5) = dRdA(i4, i5) + dudU(i6, i4) * MdudU(i6, i5);
            }
        }
    }
}

// getElasticSolnLoad element body (Working/AStrO_commandFunctions.f90:280-322) for one element:
// static orientation, r_getElRu (Working/AStrO_r_elementEqns.f90:2659-2720; Rayleigh terms are
// zero by the driver's defaults) and, for buildMat, r_condenseMat (:2722-2743).
template <class T>
static int t_element(A1<T, 33> &Ru, A2<T, 33, 33> &dRdU, const astro_model *m, const int *nDofIndex,
                     const int *intVecRange, int el, int buildMat, const GState &s, const DPert<T> &p,
                     ElemData<T> *eOut = nullptr) {
    ElemData<T> e;
    if (t_getElementData(e, m, nDofIndex, intVecRange, el, s, p) != 0) return -1;
    A1<T, 3> statRot;
    statRot.fill(T(0.0));
    for (int i2 = 1; i2 <= e.numNds; ++i2)
        for (int k = 1; k <= 3; ++k) statRot(k) = statRot(k) + e.disp(3 + k, i2);
    for (int k = 1; k <= 3; ++k) statRot(k) = (T(1.0) / (double)e.numNds) * statRot(k);
    A2<T, 3, 48> statInOri;
    A2<T, 3, 16> statdrIdrG;
    t_getInstOrient(statInOri, statdrIdrG, e.orient, statRot);
    for (int c = 4; c <= 48; ++c)
        for (int r = 1; r <= 3; ++r) statInOri(r, c) = T(0.0);
    for (int c = 4; c <= 16; ++c)
        for (int r = 1; r <= 3; ++r) statdrIdrG(r, c) = T(0.0);
    t_getElRuk(Ru, dRdU, buildMat, e, e.disp);
    if (s.dynamic == 1) {
        const double c1 = 0.5 / s.beta, c2 = 2.0 / (s.delT * s.delT);
        A2<T, 6, 11> accNext;
        for (int c = 1; c <= 11; ++c)
            for (int r = 1; r <= 6; ++r)
                accNext(r, c) = c1 * (c2 * (e.disp(r, c) - e.pDisp(r, c) - s.delT * e.pVel(r, c)) -
                                      (1.0 - 2.0 * s.beta) * e.pAcc(r, c));
        A1<T, 33> Rum;
        A2<T, 33, 33> dRdA;
        t_getElRum(Rum, dRdA, buildMat, e, statInOri, statdrIdrG, statRot, e.disp, accNext);
        for (int k = 1; k <= 33; ++k) Ru(k) = Ru(k) + Rum(k);
        if (buildMat == 1)
            for (int c = 1; c <= 33; ++c)
                for (int r = 1; r <= 33; ++r) dRdU(r, c) = dRdU(r, c) + (c1 * c2) * dRdA(r, c);
    }
    if (eOut) *eOut = e;
    return 0;
}

// r_condenseMat, Working/AStrO_r_elementEqns.f90:2722-2743
template <class T> static void t_condenseMat(A2<T, 33, 33> &mat, int stRow, int endRow) {
    T resVec[33], bVec[33], zVec[33];
    t_LUFactor(&mat(1, 1), 33, stRow, endRow);
    for (int i1 = 1; i1 <= stRow - 1; ++i1) {
        for (int k = 1; k <= 33; ++k) {
            bVec[k - 1] = mat(k, i1);
            resVec[k - 1] = T(0.0);
        }
        t_SolveLUxb(resVec, &mat(1, 1), bVec, zVec, 33, stRow, endRow);
        for (int i2 = 1; i2 <= stRow - 1; ++i2)
            for (int i3 = stRow; i3 <= endRow; ++i3) mat(i2, i1) = mat(i2, i1) - mat(i2, i3) * resVec[i3 - 1];
    }
}

}  // namespace orc
