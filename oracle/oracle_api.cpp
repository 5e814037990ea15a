// ORACLE (test infrastructure only): model-level restatement of AStrO's hot path -- analysis
// preparation (node reordering, DOF map, CSR/skyline structure, constraints), getElasticSolnLoad
// assembly, constraint scaling/loads, convertToLTri, the skyline LDL^T factor/solve and the
// reference GMRES -- exported as plain C functions for ctypes.  Only tests/, smoke() and the
// CPU-baseline leg of bench.py load this library.  See oracle_elements.hpp for the parity status.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <vector>

#include "oracle_element_driver.hpp"

using namespace orc;

int orc::g_quirk_mean_rot_derivative = 0;

struct OracleCtx {
    const astro_model *m;
    int numNodes, numEls;
    int solverMaxBW;
    std::vector<int> currentRank, originalRank, nDofIndex;  // nDofIndex(6,N)
    std::vector<int> nCRange, nodalConn;
    int elMatDim, elMatSize, elMatLTSize;
    std::vector<int> elMatRange, elMatLTRange;
    std::vector<int> intVecRange, intMatRange;
    int intVecSize, intMatSize;
    int mpcDim, mpcSize;
    std::vector<int> mpcRange, mpcCols;
    std::vector<double> mpcMat, mpcRhs;
};

// solverMaxBW as set by the *solve command (Working/AStrO_runJob.f90:106-114): smallest b with
// b^3 >= 27*numNodes^2, evaluated in default (32-bit, wrapping) integers as the reference does.
static int solver_max_bw(int numNodes) {
    int32_t nnd2 = (int32_t)((uint32_t)27u * (uint32_t)numNodes * (uint32_t)numNodes);
    int32_t b = 1, bw3 = 1;
    while (bw3 < nnd2) {
        b = b + 1;
        bw3 = (int32_t)((uint32_t)b * (uint32_t)b * (uint32_t)b);
    }
    return b;
}

// levelSortNodes, Working/AStrO_bookKeeping.f90:233-331 (breadth-first reordering from the node
// of fewest element-node incidences; nearest-node restart when a component is exhausted).
static void levelSortNodes(OracleCtx &c, int &nextAvail, int stopLength, int ndof, std::vector<int> &ndInserted,
                           std::vector<int> &ndBlockNum, int &currentBlock, int solverBlockDim) {
    const astro_model *m = c.m;
    const int numNodes = c.numNodes;
    auto nRange = [&](int i) { return c.nCRange[i]; };
    auto ndofOf = [&](int nd) { return c.nDofIndex[6 * (nd - 1)]; };
    auto nearest = [&](int from) {
        double minDist = 1e100;
        int stNd = 0;
        for (int i4 = 1; i4 <= numNodes; ++i4) {
            if (ndInserted[i4 - 1] == 0 && ndofOf(i4) == ndof) {
                double v0 = m->node_list[3 * (i4 - 1)] - m->node_list[3 * (from - 1)];
                double v1 = m->node_list[3 * (i4 - 1) + 1] - m->node_list[3 * (from - 1) + 1];
                double v2 = m->node_list[3 * (i4 - 1) + 2] - m->node_list[3 * (from - 1) + 2];
                double dist = std::sqrt(v0 * v0 + v1 * v1 + v2 * v2);
                if (dist < minDist) {
                    minDist = dist;
                    stNd = i4;
                }
            }
        }
        return stNd;
    };
    int minCon = 1000, stNd = 0;
    for (int i1 = 1; i1 <= numNodes; ++i1) {
        if (ndofOf(i1) == ndof) {
            int i2 = nRange(i1) - nRange(i1 - 1);
            if (i2 < minCon) {
                stNd = i1;
                minCon = i2;
            }
        }
    }
    c.originalRank[nextAvail - 1] = stNd;
    int currentNd = stNd, currentInd = nextAvail, blockSt = nextAvail;
    currentBlock++;
    ndBlockNum[stNd - 1] = currentBlock;
    nextAvail++;
    ndInserted[stNd - 1] = 1;
    while (nextAvail <= stopLength) {
        int i1 = nRange(currentNd - 1) + 1;
        while (i1 <= nRange(currentNd)) {
            int i2 = c.nodalConn[i1 - 1];
            if (i2 != 0 && ndInserted[i2 - 1] == 0) {
                c.originalRank[nextAvail - 1] = i2;
                nextAvail++;
                ndInserted[i2 - 1] = 1;
                ndBlockNum[i2 - 1] = currentBlock;
                int i3 = nextAvail - blockSt;
                if (i3 == solverBlockDim && nextAvail <= numNodes) {
                    stNd = nearest(i2);
                    c.originalRank[nextAvail - 1] = stNd;
                    currentNd = stNd;
                    currentInd = nextAvail;
                    ndInserted[stNd - 1] = 1;
                    blockSt = nextAvail;
                    currentBlock++;
                    ndBlockNum[stNd - 1] = currentBlock;
                    nextAvail++;
                    i1 = nRange(currentNd - 1);
                }
            }
            i1++;
        }
        currentInd++;
        if (currentInd == nextAvail && nextAvail <= stopLength) {
            int from = c.originalRank[nextAvail - 2];
            stNd = nearest(from);
            c.originalRank[nextAvail - 1] = stNd;
            currentInd = nextAvail;
            ndInserted[stNd - 1] = 1;
            ndBlockNum[stNd - 1] = currentBlock;
            nextAvail++;
        }
        if (currentInd <= numNodes) currentNd = c.originalRank[currentInd - 1];
    }
}

static GState to_gstate(const astro_state *s) {
    GState g;
    if (!s) return g;
    g.disp = s->node_disp;
    g.vel = s->node_vel;
    g.acc = s->node_acc;
    g.pdisp = s->prev_disp;
    g.pvel = s->prev_vel;
    g.pacc = s->prev_acc;
    g.intDisp = s->internal_disp;
    g.pIntDisp = s->prev_int_disp;
    g.dynamic = s->dynamic;
    g.beta = s->nm_beta;
    g.gamma = s->nm_gamma;
    g.delT = s->del_t;
    return g;
}

// r_getNodeDLoad (Working/AStrO_r_designPropertyFunctions.f90:970-994, Q6 resolved: the loop runs
// over the node's own terms): the elastic nodal design load of a node at time t, components
// 1..6 and the thermal ndLd(7), for the variables active (dActTime(1) < t < dActTime(2), r_greater), with design variable
// pert (if any) at d + i h.
template <class T> static void t_node_dload(const astro_model *m, int node, double t, const DPert<T> &p, T ld[7]) {
    for (int k = 0; k < 7; ++k) ld[k] = T(0.0);
    if (!m->nd_to_d_range || m->num_dvars <= 0) return;
    for (int q = m->nd_to_d_range[node - 1]; q < m->nd_to_d_range[node]; ++q) {
        const int d = m->nd_to_d[q];
        if (m->d_category[d - 1] != ASTRO_DCAT_NODE_LOAD) continue;
        if (m->d_act_time && !(t > m->d_act_time[2 * (d - 1)] && m->d_act_time[2 * (d - 1) + 1] > t)) continue;
        const int comp = m->d_component ? m->d_component[d - 1] : 0;
        if (comp < 1 || comp > 7) continue;  // 7: the 'thermal' subcategory, ndLd(7)
        ld[comp - 1] = ld[comp - 1] + m->nd_to_coef[q] * dval(m, d, p);
    }
}

// One face of the surface load (the per-face body of orc_surface_load): nodes (r_getNodeCoord:
// coordinates with the nodeCoord terms, design variable p.dvar at d + i h), the face normal, the
// traction t - pressure n, and the consistent nodal values of the integral of N t dA on the true
// area with the 2x2 Gauss rule (abscissa KC<T>::rt3).
template <class T>
static void t_face_load(const astro_model *m, int el, int fn, const double *traction, double pressure,
                        const DPert<T> &p, int nodes[4], T val[4][3]) {
    static const int hexF[6][4] = {{4, 3, 2, 1}, {5, 6, 7, 8}, {1, 2, 6, 5}, {2, 3, 7, 6}, {3, 4, 8, 7}, {4, 1, 5, 8}};
    static const int shF[2][4] = {{1, 2, 3, 4}, {1, 4, 3, 2}};
    const double rt3 = KC<T>::rt3();
    const int t = m->element_type[el - 1];
    const int *fl = (t == 8 || t == 81) ? hexF[fn - 1] : shF[fn - 1];
    T X[4][3];
    for (int k = 0; k < 4; ++k) {
        nodes[k] = m->element_list[8 * (el - 1) + fl[k] - 1];
        for (int d = 0; d < 3; ++d)
            X[k][d] = T(m->node_list[3 * (nodes[k] - 1) + d]) + nd_dsum(m, nodes[k], ASTRO_DCAT_NODE_COORD, d + 1, p);
    }
    T v1[3], v2[3], nv[3];
    for (int d = 0; d < 3; ++d) {
        v1[d] = X[2][d] - X[0][d];
        v2[d] = X[3][d] - X[1][d];
    }
    nv[0] = v1[1] * v2[2] - v1[2] * v2[1];
    nv[1] = v1[2] * v2[0] - v1[0] * v2[2];
    nv[2] = v1[0] * v2[1] - v1[1] * v2[0];
    const T mag = std::sqrt(nv[0] * nv[0] + nv[1] * nv[1] + nv[2] * nv[2]);
    for (int d = 0; d < 3; ++d) nv[d] = nv[d] / mag;
    T tr[3];
    for (int d = 0; d < 3; ++d) tr[d] = traction[d] - pressure * nv[d];
    for (int k = 0; k < 4; ++k)
        for (int d = 0; d < 3; ++d) val[k][d] = T(0.0);
    const double gp[4][2] = {{-rt3, -rt3}, {rt3, -rt3}, {-rt3, rt3}, {rt3, rt3}};
    for (int g = 0; g < 4; ++g) {
        const double s = gp[g][0], r = gp[g][1];
        const double N[4] = {0.25 * (1 - s) * (1 - r), 0.25 * (1 + s) * (1 - r), 0.25 * (1 + s) * (1 + r),
                             0.25 * (1 - s) * (1 + r)};
        const double Ns[4] = {-0.25 * (1 - r), 0.25 * (1 - r), 0.25 * (1 + r), -0.25 * (1 + r)};
        const double Nr[4] = {-0.25 * (1 - s), -0.25 * (1 + s), 0.25 * (1 + s), 0.25 * (1 - s)};
        T a[3] = {T(0.0), T(0.0), T(0.0)}, b[3] = {T(0.0), T(0.0), T(0.0)};
        for (int k = 0; k < 4; ++k)
            for (int d = 0; d < 3; ++d) {
                a[d] += Ns[k] * X[k][d];
                b[d] += Nr[k] * X[k][d];
            }
        const T cx = a[1] * b[2] - a[2] * b[1], cy = a[2] * b[0] - a[0] * b[2], cz = a[0] * b[1] - a[1] * b[0];
        const T dA = std::sqrt(cx * cx + cy * cy + cz * cz);
        for (int k = 0; k < 4; ++k)
            for (int d = 0; d < 3; ++d) val[k][d] += tr[d] * N[k] * dA;
    }
}

// getdToElComp (Working/AStrO_bookKeeping.f90:7-129): the element depends on dvar through its own
// design-variable terms or a nodeCoord term of one of its nodes.
static bool el_depends(const astro_model *m, int el, int dvar) {
    bool dep = false;
    if (m->el_to_d_range)
        for (int q = m->el_to_d_range[el - 1]; q < m->el_to_d_range[el]; ++q) dep = dep || m->el_to_d[q] == dvar;
    if (m->nd_to_d_range && m->d_category[dvar - 1] == ASTRO_DCAT_NODE_COORD)
        for (int k = 0; k < 8; ++k) {
            const int nd = m->element_list[8 * (el - 1) + k];
            if (nd > 0)
                for (int q = m->nd_to_d_range[nd - 1]; q < m->nd_to_d_range[nd]; ++q) dep = dep || m->nd_to_d[q] == dvar;
        }
    return dep;
}

extern "C" {

// analysisPrep, Working/AStrO_bookKeeping.f90:794-1039, with allocateElasticMat (:333-411) and
// buildElasticMPC (:474-612) for pre-expanded equations.  Returns NULL on unsupported input.
OracleCtx *orc_create(const astro_model *m) {
    OracleCtx *c = new OracleCtx();
    c->m = m;
    const int N = m->num_nodes, E = m->num_els;
    c->numNodes = N;
    c->numEls = E;
    c->solverMaxBW = solver_max_bw(N);
    c->currentRank.assign(N, 0);
    c->originalRank.assign(N, 0);
    c->nDofIndex.assign(6 * N, 0);
    c->nCRange.assign(N + 1, 0);
    for (int i1 = 1; i1 <= E; ++i1) {
        int eT = m->element_type[i1 - 1];
        int ndof = (eT == 41 || eT == 3 || eT == 2) ? 6 : 3;
        for (int i2 = 1; i2 <= 8; ++i2) {
            int i3 = m->element_list[8 * (i1 - 1) + i2 - 1];
            if (i3 != 0) {
                for (int i4 = 1; i4 <= 8; ++i4) {
                    int i5 = m->element_list[8 * (i1 - 1) + i4 - 1];
                    if (i5 != 0 && i5 != i3) c->nCRange[i3]++;
                }
                c->nDofIndex[6 * (i3 - 1)] = ndof;
            }
        }
    }
    int numSolidNds = 0;
    for (int i1 = 1; i1 <= N; ++i1)
        if (c->nDofIndex[6 * (i1 - 1)] == 3) numSolidNds++;
    int numSectionNds = N - numSolidNds;
    for (int i1 = 2; i1 <= N; ++i1) c->nCRange[i1] += c->nCRange[i1 - 1];
    int nCSize = c->nCRange[N];
    c->nodalConn.assign(nCSize, 0);
    for (int i1 = 1; i1 <= E; ++i1)
        for (int i2 = 1; i2 <= 8; ++i2) {
            int i3 = m->element_list[8 * (i1 - 1) + i2 - 1];
            if (i3 == 0) continue;
            for (int i4 = 1; i4 <= 8; ++i4) {
                int i5 = m->element_list[8 * (i1 - 1) + i4 - 1];
                if (i5 == 0 || i5 == i3) continue;
                int i6 = c->nCRange[i3 - 1] + 1;
                int inserted = 0;
                while (i6 <= c->nCRange[i3] && inserted == 0) {
                    if (c->nodalConn[i6 - 1] == 0) {
                        c->nodalConn[i6 - 1] = i5;
                        inserted = 1;
                    } else if (c->nodalConn[i6 - 1] == i5) {
                        inserted = 1;
                    }
                    i6++;
                }
            }
        }
    std::vector<int> ndInserted(N, 0), ndBlockNum(N, 0);
    int nextAvail = 1, currentBlock = 0;
    if (numSolidNds > 0) levelSortNodes(*c, nextAvail, numSolidNds, 3, ndInserted, ndBlockNum, currentBlock, N);
    if (nextAvail <= N) levelSortNodes(*c, nextAvail, N, 6, ndInserted, ndBlockNum, currentBlock, N);
    for (int i1 = 1; i1 <= N; ++i1) c->currentRank[c->originalRank[i1 - 1] - 1] = i1;
    for (int i1 = 1; i1 <= N; ++i1) {
        int t = c->nDofIndex[6 * (i1 - 1)];
        if (t == 3) {
            for (int i2 = 1; i2 <= 3; ++i2) c->nDofIndex[6 * (i1 - 1) + i2 - 1] = c->currentRank[i1 - 1] + (i2 - 1) * numSolidNds;
        } else if (t == 6) {
            for (int i2 = 1; i2 <= 6; ++i2)
                c->nDofIndex[6 * (i1 - 1) + i2 - 1] = c->currentRank[i1 - 1] + (i2 - 1) * numSectionNds + 2 * numSolidNds;
        }
    }
    const int n = 3 * numSolidNds + 6 * numSectionNds;
    c->elMatDim = n;
    c->intVecRange.assign(E + 1, 0);
    c->intMatRange.assign(E + 1, 0);
    for (int i1 = 1; i1 <= E; ++i1) {
        int t = m->element_type[i1 - 1];
        if (t == 41) {
            c->intVecRange[i1] = 8;
            c->intMatRange[i1] = 256;
        } else if (t == 81) {  // allocateElasticMat's internal sizes (Working/AStrO_bookKeeping.f90:978-1003)
            c->intVecRange[i1] = 9;
            c->intMatRange[i1] = 297;
        } else if (t != 8) {
            delete c;
            return nullptr;
        }
    }
    for (int i1 = 2; i1 <= E; ++i1) {
        c->intVecRange[i1] += c->intVecRange[i1 - 1];
        c->intMatRange[i1] += c->intMatRange[i1 - 1];
    }
    c->intVecSize = c->intVecRange[E];
    c->intMatSize = c->intMatRange[E];
    // allocateElasticMat
    auto ndi = [&](int comp, int nd) { return c->nDofIndex[6 * (nd - 1) + comp - 1]; };
    c->elMatRange.assign(n + 1, 0);
    c->elMatLTRange.assign(n + 1, 0);
    for (int i1 = 1; i1 <= N; ++i1)
        for (int i2 = 1; i2 <= 6; ++i2) {
            int i3 = ndi(i2, i1);
            if (i3 == 0) continue;
            for (int i4 = 1; i4 <= 6; ++i4)
                if (ndi(i4, i1) != 0) c->elMatRange[i3]++;
            for (int i4 = c->nCRange[i1 - 1] + 1; i4 <= c->nCRange[i1]; ++i4) {
                int i5 = c->nodalConn[i4 - 1];
                if (i5 == 0) continue;
                for (int i6 = 1; i6 <= 6; ++i6)
                    if (ndi(i6, i5) != 0) c->elMatRange[i3]++;
            }
        }
    for (int i1 = 2; i1 <= n; ++i1) c->elMatRange[i1] += c->elMatRange[i1 - 1];
    c->elMatSize = c->elMatRange[n];
    for (int i1 = 1; i1 <= N; ++i1)
        for (int i2 = 1; i2 <= 6; ++i2) {
            int i3 = ndi(i2, i1);
            if (i3 == 0) continue;
            c->elMatLTRange[i3] = 1;
            for (int i4 = c->nCRange[i1 - 1] + 1; i4 <= c->nCRange[i1]; ++i4) {
                int i5 = c->nodalConn[i4 - 1];
                if (i5 == 0) continue;
                int i6 = c->currentRank[i1 - 1] - c->currentRank[i5 - 1];
                if (i6 >= 0 && i6 <= c->solverMaxBW) {
                    int i7 = ndi(i2, i5);
                    if (i7 != 0 && i7 <= i3) {
                        int i8 = i3 - i7 + 1;
                        if (i8 > c->elMatLTRange[i3]) c->elMatLTRange[i3] = i8;
                    }
                }
            }
        }
    for (int i1 = 2; i1 <= n; ++i1) c->elMatLTRange[i1] += c->elMatLTRange[i1 - 1];
    c->elMatLTSize = c->elMatLTRange[n];
    // buildElasticMPC for expanded equations: duplicate columns in a row are skipped (slot stays 0)
    c->mpcDim = m->num_mpc;
    c->mpcRange.assign(c->mpcDim + 1, 0);
    for (int k = 0; k <= c->mpcDim; ++k) c->mpcRange[k] = m->num_mpc ? m->mpc_range[k] : 0;
    c->mpcSize = c->mpcRange[c->mpcDim];
    c->mpcCols.assign(c->mpcSize, 0);
    c->mpcMat.assign(c->mpcSize, 0.0);
    c->mpcRhs.assign(c->mpcDim, 0.0);
    for (int r = 1; r <= c->mpcDim; ++r) {
        for (int t = c->mpcRange[r - 1]; t < c->mpcRange[r]; ++t) {
            int col = ndi(m->mpc_dof[t], m->mpc_node[t]);
            for (int s = c->mpcRange[r - 1]; s < c->mpcRange[r]; ++s) {
                if (c->mpcCols[s] == 0) {
                    c->mpcMat[s] = m->mpc_coef[t];
                    c->mpcCols[s] = col;
                    break;
                } else if (c->mpcCols[s] == col) {
                    break;
                }
            }
        }
        c->mpcRhs[r - 1] = m->mpc_rhs[r - 1];
    }
    return c;
}

void orc_destroy(OracleCtx *c) { delete c; }

// Debug probe: shell deformation vectors def(9) at the Gauss points of element el at `s`.
int orc_debug_shell_def(const OracleCtx *c, int el, const astro_state *s, double *out) {
    ElemData<double> e;
    DPert<double> p;
    GState g = to_gstate(s);
    if (t_getElementData(e, c->m, c->nDofIndex.data(), c->intVecRange.data(), el, g, p) != 0) return 1;
    A1<double, 3> elRot;
    elRot.fill(0.0);
    for (int i1 = 1; i1 <= e.numNds; ++i1)
        for (int k = 1; k <= 3; ++k) elRot(k) += e.disp(3 + k, i1) / e.numNds;
    A2<double, 3, 48> instOri;
    A2<double, 3, 16> drIdrG;
    t_getInstOrient(instOri, drIdrG, e.orient, elRot);
    for (int gp = 1; gp <= e.numIntPts; ++gp) {
        A1<double, 11> Nvec;
        A2<double, 11, 3> Nx;
        double detJ;
        t_getIntPtData(Nvec, Nx, detJ, e.locNds, e.intPts[gp - 1], 41, 4);
        A2<double, 6, 11> U;
        t_getInstDof(U, e.disp, e.globNds, instOri, e.orient, elRot, drIdrG, 4, e.dofTable, 0, 0);
        A1<double, 3> ptRot;
        ptRot.fill(0.0);
        for (int i2 = 1; i2 <= 4; ++i2)
            for (int k = 1; k <= 3; ++k) ptRot(k) += U(3 + k, i2) * Nvec(i2);
        A2<double, 3, 3> ux, rx;
        ux.fill(0.0);
        rx.fill(0.0);
        for (int i2 = 1; i2 <= 3; ++i2)
            for (int i3 = 1; i3 <= 3; ++i3)
                for (int i4 = 1; i4 <= 10; ++i4) {
                    ux(i2, i3) += U(i2, i4) * Nx(i4, i3);
                    rx(i2, i3) += U(i2 + 3, i4) * Nx(i4, i3);
                }
        A1<double, 9> d;
        t_getShellDef(d, ux, ptRot, rx);
        for (int k = 0; k < 9; ++k) out[(gp - 1) * 9 + k] = d.a[k];
    }
    return 0;
}

void orc_set_quirk(int which, int value) {
    if (which == 1) g_quirk_mean_rot_derivative = value;
}

void orc_dims(const OracleCtx *c, int32_t *out) {
    out[0] = c->elMatDim;
    out[1] = c->elMatSize;
    out[2] = c->elMatLTSize;
    out[3] = c->mpcDim;
    out[4] = c->mpcSize;
    out[5] = c->intVecSize;
    out[6] = c->intMatSize;
    out[7] = c->solverMaxBW;
}

void orc_get_prep(const OracleCtx *c, int32_t *currentRank, int32_t *nDofIndex, int32_t *elMatRange,
                  int32_t *elMatLTRange, int32_t *mpcRange, int32_t *mpcCols, double *mpcMat, double *mpcRhs) {
    if (currentRank) std::copy(c->currentRank.begin(), c->currentRank.end(), currentRank);
    if (nDofIndex) std::copy(c->nDofIndex.begin(), c->nDofIndex.end(), nDofIndex);
    if (elMatRange) std::copy(c->elMatRange.begin(), c->elMatRange.end(), elMatRange);
    if (elMatLTRange) std::copy(c->elMatLTRange.begin(), c->elMatLTRange.end(), elMatLTRange);
    if (mpcRange) std::copy(c->mpcRange.begin(), c->mpcRange.end(), mpcRange);
    if (mpcCols) std::copy(c->mpcCols.begin(), c->mpcCols.end(), mpcCols);
    if (mpcMat) std::copy(c->mpcMat.begin(), c->mpcMat.end(), mpcMat);
    if (mpcRhs) std::copy(c->mpcRhs.begin(), c->mpcRhs.end(), mpcRhs);
}


// One element (1-based) in FP64: Ru(33) and dRdU(33,33) column-major, before condensation.
int orc_element(const OracleCtx *c, int el, int buildMat, const astro_state *s, double *Ru, double *dRdU) {
    A1<double, 33> R;
    A2<double, 33, 33> K;
    DPert<double> p;
    if (t_element(R, K, c->m, c->nDofIndex.data(), c->intVecRange.data(), el, buildMat, to_gstate(s), p) != 0)
        return 1;
    for (int k = 0; k < 33; ++k) Ru[k] = R.a[k];
    if (dRdU) std::memcpy(dRdU, &K(1, 1), sizeof(double) * 33 * 33);
    return 0;
}

// One element in complex FP64 with design variable dvar perturbed by i*h: real and imaginary
// parts of Ru(33) and dRdU(33,33).
int orc_element_c(const OracleCtx *c, int el, int buildMat, const astro_state *s, int dvar, double h, double *RuRe,
                  double *RuIm, double *KRe, double *KIm) {
    A1<cd, 33> R;
    A2<cd, 33, 33> K;
    DPert<cd> p;
    p.dvar = dvar;
    p.h = h;
    if (t_element(R, K, c->m, c->nDofIndex.data(), c->intVecRange.data(), el, buildMat, to_gstate(s), p) != 0)
        return 1;
    for (int k = 0; k < 33; ++k) {
        RuRe[k] = R.a[k].real();
        RuIm[k] = R.a[k].imag();
    }
    if (KRe)
        for (int j = 1; j <= 33; ++j)
            for (int i = 1; i <= 33; ++i) {
                KRe[(j - 1) * 33 + i - 1] = K(i, j).real();
                KIm[(j - 1) * 33 + i - 1] = K(i, j).imag();
            }
    return 0;
}

// getdRelasticdD element part, Working/AStrO_commandFunctions.f90:1172-1250: the elements that
// depend on design variable dvar are re-evaluated in complex FP64 with d_value(dvar) + i h
// (c_getElRu with buildMat = 0), and Im(Ru) * (1/h) is summed into dRudD at the element's global
// DOF (Q10 resolved: the global index, not the element-local one) and into intdRudD at its
// internal DOF.  Both outputs are zeroed first, as the reference does.  Elements are visited in
// ascending order (the order getdToElComp lists them).
int orc_drdd_complex(const OracleCtx *c, int dvar, double h, const astro_state *s, double *dRudD, double *intdRudD) {
    const astro_model *m = c->m;
    std::fill(dRudD, dRudD + c->elMatDim, 0.0);
    if (intdRudD && c->intVecSize > 0) std::fill(intdRudD, intdRudD + c->intVecSize, 0.0);
    if (dvar < 1 || dvar > m->num_dvars) return 1;
    const double hInv = 1.0 / h;
    GState g = to_gstate(s);
    DPert<cd> p;
    p.dvar = dvar;
    p.h = h;
    for (int el = 1; el <= c->numEls; ++el) {
        // getdToElComp (Working/AStrO_bookKeeping.f90:7-129): the element's own design variables
        // and those of its nodes
        bool dep = false;
        if (m->el_to_d_range)
            for (int q = m->el_to_d_range[el - 1]; q < m->el_to_d_range[el]; ++q) dep = dep || m->el_to_d[q] == dvar;
        if (m->nd_to_d_range)
            for (int k = 0; k < 8; ++k) {
                const int nd = m->element_list[8 * (el - 1) + k];
                if (nd > 0)
                    for (int q = m->nd_to_d_range[nd - 1]; q < m->nd_to_d_range[nd]; ++q)
                        dep = dep || (m->nd_to_d[q] == dvar && m->d_category[dvar - 1] == ASTRO_DCAT_NODE_COORD);
            }
        if (!dep) continue;
        A1<cd, 33> Ru;
        A2<cd, 33, 33> K;
        ElemData<cd> e;
        if (t_element(Ru, K, m, c->nDofIndex.data(), c->intVecRange.data(), el, 0, g, p, &e) != 0) return 1;
        const int nd = e.numNds * e.dofPerNd;
        for (int i = 1; i <= nd; ++i) {
            const int var = e.dofTable[i - 1][0];
            const int node = m->element_list[8 * (el - 1) + e.dofTable[i - 1][1] - 1];
            const int dof = c->nDofIndex[6 * (node - 1) + var - 1];
            dRudD[dof - 1] += hInv * Ru(i).imag();
        }
        if (e.numIntDof > 0 && intdRudD) {
            int k = c->intVecRange[el - 1];
            for (int i = nd + 1; i <= nd + e.numIntDof; ++i) intdRudD[k++] += hInv * Ru(i).imag();
        }
    }
    return 0;
}

// Element matrices of elements el0..el1 (1-based, inclusive) in FP64 after static condensation,
// nodal part only (nd x nd per element, column-major, nd = numNds*dofPerNd = 24).  Used by the
// CPU baseline timing and the per-element parity tests.
int orc_element_matrices(const OracleCtx *c, int el0, int el1, const astro_state *s, double *ke_out) {
    GState g = to_gstate(s);
    DPert<double> p;
    for (int el = el0; el <= el1; ++el) {
        A1<double, 33> R;
        A2<double, 33, 33> K;
        if (t_element(R, K, c->m, c->nDofIndex.data(), c->intVecRange.data(), el, 1, g, p) != 0) return 1;
        int t = c->m->element_type[el - 1];
        if (t == 41) t_condenseMat(K, 25, 32);
        if (t == 81) t_condenseMat(K, 25, 33);
        double *o = ke_out + (size_t)(el - el0) * 576;
        for (int j = 1; j <= 24; ++j)
            for (int i = 1; i <= 24; ++i) o[(j - 1) * 24 + i - 1] = K(i, j);
    }
    return 0;
}

// getElasticSolnLoad, Working/AStrO_commandFunctions.f90:260-351 (Q7 resolved: CSR columns start
// zeroed by this call).  elasticLoad(n) and intElasticLoad are accumulated (-= Ru).
int orc_el_soln_load(const OracleCtx *c, int buildMat, const astro_state *s, double *elasticLoad,
                     double *intElasticLoad, double *elasticMat, int32_t *elMatCols, double *intElasticMat) {
    const astro_model *m = c->m;
    GState g = to_gstate(s);
    DPert<double> p;
    if (buildMat == 1) {
        std::fill(elasticMat, elasticMat + c->elMatSize, 0.0);
        std::fill(elMatCols, elMatCols + c->elMatSize, 0);
    }
    for (int i1 = 1; i1 <= c->numEls; ++i1) {
        A1<double, 33> Ru;
        A2<double, 33, 33> dRdU;
        ElemData<double> e;
        if (t_element(Ru, dRdU, m, c->nDofIndex.data(), c->intVecRange.data(), i1, buildMat, g, p, &e) != 0) return 1;
        int i3 = e.numNds * e.dofPerNd;
        for (int i2 = 1; i2 <= i3; ++i2) {
            int i4 = e.dofTable[i2 - 1][0];
            int i5 = m->element_list[8 * (i1 - 1) + e.dofTable[i2 - 1][1] - 1];
            int i6 = c->nDofIndex[6 * (i5 - 1) + i4 - 1];
            elasticLoad[i6 - 1] -= Ru(i2);
        }
        if (e.numIntDof != 0 && intElasticLoad) {
            int i4 = c->intVecRange[i1 - 1] + 1, i5 = c->intVecRange[i1];
            for (int k = i4; k <= i5; ++k) intElasticLoad[k - 1] -= Ru(i3 + k - i4 + 1);
        }
        if (buildMat == 1) {
            if (e.numIntDof > 0) {
                int i2 = e.numNds * e.dofPerNd + 1, i3b = e.numNds * e.dofPerNd + e.numIntDof;
                t_condenseMat(dRdU, i2, i3b);
                int i4 = c->intMatRange[i1 - 1] + 1;
                if (intElasticMat)
                    for (int i5 = 1; i5 <= i3b; ++i5)
                        for (int i6 = i2; i6 <= i3b; ++i6) intElasticMat[(i4++) - 1] = dRdU(i6, i5);
            }
            int i2 = e.numNds * e.dofPerNd;
            for (int i3c = 1; i3c <= i2; ++i3c) {
                int i5 = e.dofTable[i3c - 1][0];
                int i6 = m->element_list[8 * (i1 - 1) + e.dofTable[i3c - 1][1] - 1];
                int kGi = c->nDofIndex[6 * (i6 - 1) + i5 - 1];
                for (int i4 = 1; i4 <= i2; ++i4) {
                    int v = e.dofTable[i4 - 1][0];
                    int nd = m->element_list[8 * (i1 - 1) + e.dofTable[i4 - 1][1] - 1];
                    int kGj = c->nDofIndex[6 * (nd - 1) + v - 1];
                    int k = c->elMatRange[kGi - 1] + 1;
                    int inserted = 0;
                    while (inserted == 0 && k <= c->elMatRange[kGi]) {
                        int col = elMatCols[k - 1];
                        if (col == 0) {
                            elasticMat[k - 1] = dRdU(i3c, i4);
                            elMatCols[k - 1] = kGj;
                            inserted = 1;
                        } else if (col == kGj) {
                            elasticMat[k - 1] += dRdU(i3c, i4);
                            inserted = 1;
                        }
                        k++;
                    }
                }
            }
        }
    }
    return 0;
}

// scaleElasticMPC, Working/AStrO_commandFunctions.f90:537-566 (in place on the given arrays)
void orc_scale_mpc(const double *elasticMat, int elMatSize, double *mpcMat, double *mpcRhs, const int32_t *mpcRange,
                   int mpcDim) {
    double maxMat = 0.0;
    for (int i1 = 0; i1 < elMatSize; ++i1) {
        double r = std::fabs(elasticMat[i1]);
        if (r > maxMat) maxMat = r;
    }
    for (int i1 = 1; i1 <= mpcDim; ++i1) {
        int i3 = mpcRange[i1 - 1] + 1, i4 = mpcRange[i1];
        double rowMag = 0.0;
        for (int i2 = i3; i2 <= i4; ++i2) rowMag += mpcMat[i2 - 1] * mpcMat[i2 - 1];
        rowMag = std::sqrt(rowMag);
        for (int i2 = i3; i2 <= i4; ++i2) mpcMat[i2 - 1] = (1.0 / rowMag) * mpcMat[i2 - 1];
        mpcRhs[i1 - 1] = (1.0 / rowMag) * mpcRhs[i1 - 1];
    }
    int mpcSize = mpcRange[mpcDim];
    for (int k = 0; k < mpcSize; ++k) mpcMat[k] = 100.0 * maxMat * mpcMat[k];
    for (int k = 0; k < mpcDim; ++k) mpcRhs[k] = 100.0 * maxMat * mpcRhs[k];
}

// getElasticConstraintLoad, :506-535
void orc_constraint_load(const double *mpcMat, const int32_t *mpcCols, const int32_t *mpcRange, const double *mpcRhs,
                         int mpcDim, const double *nodeDisp, double *elasticLoad) {
    std::vector<double> t(mpcRhs, mpcRhs + mpcDim);
    for (int i1 = 1; i1 <= mpcDim; ++i1)
        for (int i2 = mpcRange[i1 - 1] + 1; i2 <= mpcRange[i1]; ++i2) {
            int i3 = mpcCols[i2 - 1];
            if (i3 != 0 && nodeDisp) t[i1 - 1] -= mpcMat[i2 - 1] * nodeDisp[i3 - 1];
        }
    for (int i1 = 1; i1 <= mpcDim; ++i1)
        for (int i2 = mpcRange[i1 - 1] + 1; i2 <= mpcRange[i1]; ++i2) {
            int i3 = mpcCols[i2 - 1];
            if (i3 != 0) elasticLoad[i3 - 1] += mpcMat[i2 - 1] * t[i1 - 1];
        }
}

// convertToLTri, Working/AStrO_bookKeeping.f90:754-792
void orc_convert_to_ltri(double *lTri, const int32_t *lTRange, int lTSize, const double *mainMat, const int32_t *mainCols,
                         const int32_t *mainRange, int mainSize, int mainDim, const double *cMat, const int32_t *cCols,
                         const int32_t *cRange, int cSize, int cDim) {
    (void)mainSize;
    (void)cSize;
    std::fill(lTri, lTri + lTSize, 0.0);
    for (int i1 = 1; i1 <= mainDim; ++i1) {
        int minCol = i1 - lTRange[i1] + lTRange[i1 - 1] + 1;
        for (int i2 = mainRange[i1 - 1] + 1; i2 <= mainRange[i1]; ++i2) {
            int i3 = mainCols[i2 - 1];
            if (i3 >= minCol && i3 <= i1) {
                int i4 = lTRange[i1] - i1 + i3;
                lTri[i4 - 1] += mainMat[i2 - 1];
            }
        }
    }
    for (int i1 = 1; i1 <= cDim; ++i1)
        for (int i2 = cRange[i1 - 1] + 1; i2 <= cRange[i1]; ++i2) {
            int i4 = cCols[i2 - 1];
            if (i4 == 0) continue;
            int minCol = i4 - lTRange[i4] + lTRange[i4 - 1] + 1;
            for (int i3 = cRange[i1 - 1] + 1; i3 <= cRange[i1]; ++i3) {
                int i5 = cCols[i3 - 1];
                if (i5 >= minCol && i5 <= i4) {
                    int i6 = lTRange[i4] - i4 + i5;
                    lTri[i6 - 1] += cMat[i2 - 1] * cMat[i3 - 1];
                }
            }
        }
}

// getSparseLDLFact, Working/AStrO_solvers.f90:10-78
void orc_ldl_fact(double *ALTri, int ASize, const int32_t *ARange, int n) {
    (void)ASize;
    std::vector<int> rowStCol(n + 1);
    std::vector<double> diagvec(n + 1);
    int maxBW = 0;
    for (int i1 = 1; i1 <= n; ++i1) {
        int rowLen = ARange[i1] - ARange[i1 - 1];
        rowStCol[i1] = i1 - rowLen + 1;
        if (rowLen > maxBW) maxBW = rowLen;
    }
    std::vector<double> dLprod(maxBW + 1);
    for (int i1 = 1; i1 <= n; ++i1) {
        int i3 = ARange[i1];
        int i2 = ARange[i1 - 1] + 1;
        int i5 = maxBW, i6 = i1 - 1;
        for (int i4 = i3 - 1; i4 >= i2; --i4) {
            dLprod[i5] = diagvec[i6] * ALTri[i4 - 1];
            i5--;
            i6--;
        }
        i5 = i1 - i3 + i2;
        double diag = ALTri[i3 - 1];
        for (int i4 = i2; i4 <= i3 - 1; ++i4) {
            diag -= diagvec[i5] * ALTri[i4 - 1] * ALTri[i4 - 1];
            i5++;
        }
        diagvec[i1] = diag;
        ALTri[i3 - 1] = diag;
        double fact = 1.0 / diag;
        int imax = std::min(n, i1 + maxBW);
        for (int j = i1 + 1; j <= imax; ++j) {
            int stCol = std::max(rowStCol[i1], rowStCol[j]);
            int rowLen = i1 - stCol;
            if (rowLen >= 0) {
                int a = maxBW - rowLen + 1;
                int b = ARange[j] - (j - stCol);
                int t = b + rowLen;
                double d = ALTri[t - 1];
                for (int k = 0; k <= rowLen - 1; ++k) d -= dLprod[a + k] * ALTri[b + k - 1];
                ALTri[t - 1] = d * fact;
            }
        }
    }
}

// solveSparseLDLFact, Working/AStrO_solvers.f90:83-126
void orc_ldl_solve(double *soln, const double *rhs, const double *Lmat, int LSize, const int32_t *LRange, int Ldim,
                   double *zVec) {
    (void)LSize;
    int maxBW = 0;
    for (int i1 = 1; i1 <= Ldim; ++i1) {
        int i2 = LRange[i1 - 1] + 1;
        int rowLen = LRange[i1] - i2;
        if (rowLen > maxBW) maxBW = rowLen;
        int stCol = i1 - rowLen;
        zVec[i1 - 1] = rhs[i1 - 1];
        for (int i3 = 0; i3 <= rowLen - 1; ++i3) zVec[i1 - 1] -= Lmat[i2 + i3 - 1] * zVec[stCol + i3 - 1];
    }
    for (int i1 = Ldim; i1 >= 1; --i1) {
        double dtProd = 0.0;
        double diag = Lmat[LRange[i1] - 1];
        int imax = std::min(Ldim, i1 + maxBW);
        for (int i2 = i1 + 1; i2 <= imax; ++i2) {
            int rowLen = LRange[i2] - LRange[i2 - 1];
            int stCol = i2 - rowLen + 1;
            if (stCol <= i1) {
                int i3 = LRange[i2] + i1 - i2;
                dtProd += Lmat[i3 - 1] * soln[i2 - 1];
            }
        }
        dtProd = dtProd * diag;
        soln[i1 - 1] = (zVec[i1 - 1] - dtProd) / diag;
    }
}

// rFactorMat (triDiag = 2 branch used by gMRes), Working/AStrO_solvers.f90:299-353
static void rFactorMat(std::vector<double> &A, int rowDim, int colDim) {
    auto a = [&](int i, int j) -> double & { return A[(size_t)(j - 1) * rowDim + i - 1]; };
    for (int i1 = 1; i1 <= colDim; ++i1) {
        int maxRow = std::min(i1 + 1, rowDim), maxCol = colDim;
        for (int i2 = i1 + 1; i2 <= maxRow; ++i2) {
            if (std::fabs(a(i2, i1)) > F(1e-10)) {
                double theta;
                if (a(i1, i1) == 0.0)
                    theta = F(1.570796326794897);
                else
                    theta = std::atan(a(i2, i1) / a(i1, i1));
                double st = std::sin(theta), ct = std::cos(theta);
                for (int i3 = i1; i3 <= maxCol; ++i3) {
                    double a1 = ct * a(i1, i3) + st * a(i2, i3);
                    double a2 = -st * a(i1, i3) + ct * a(i2, i3);
                    a(i1, i3) = a1;
                    a(i2, i3) = a2;
                }
                a(i2, i1) = theta;
            }
        }
    }
}

// solveRFactor (triDiag = 2), :355-404
static void solveRFactor(double *soln, const std::vector<double> &A, double *bVec, int rowDim, int colDim) {
    auto a = [&](int i, int j) { return A[(size_t)(j - 1) * rowDim + i - 1]; };
    for (int i1 = 1; i1 <= colDim; ++i1) {
        int maxRow = std::min(i1 + 1, rowDim);
        for (int i2 = i1 + 1; i2 <= maxRow; ++i2) {
            if (std::fabs(a(i2, i1)) > F(1e-10)) {
                double st = std::sin(a(i2, i1)), ct = std::cos(a(i2, i1));
                double r1 = ct * bVec[i1 - 1] + st * bVec[i2 - 1];
                double r2 = -st * bVec[i1 - 1] + ct * bVec[i2 - 1];
                bVec[i1 - 1] = r1;
                bVec[i2 - 1] = r2;
            }
        }
    }
    for (int i1 = colDim; i1 >= 1; --i1) {
        soln[i1 - 1] = bVec[i1 - 1];
        for (int i2 = i1 + 1; i2 <= colDim; ++i2) soln[i1 - 1] -= a(i1, i2) * soln[i2 - 1];
        soln[i1 - 1] = soln[i1 - 1] / a(i1, i1);
    }
}

// (A + C^T C) x with the reference's loop order: C x, C^T(.), then A x added.
static void ref_matvec(std::vector<double> &out, const double *x, const double *Amat, const int32_t *Acols,
                       const int32_t *ARange, int ADim, const double *Cmat, const int32_t *Ccols, const int32_t *CRange,
                       int CDim, std::vector<double> &t1) {
    std::fill(t1.begin(), t1.end(), 0.0);
    for (int i1 = 1; i1 <= CDim; ++i1)
        for (int i2 = CRange[i1 - 1] + 1; i2 <= CRange[i1]; ++i2) {
            int i3 = Ccols[i2 - 1];
            if (i3 != 0) t1[i1 - 1] += Cmat[i2 - 1] * x[i3 - 1];
        }
    std::fill(out.begin(), out.end(), 0.0);
    for (int i1 = 1; i1 <= CDim; ++i1)
        for (int i2 = CRange[i1 - 1] + 1; i2 <= CRange[i1]; ++i2) {
            int i3 = Ccols[i2 - 1];
            if (i3 != 0) out[i3 - 1] += Cmat[i2 - 1] * t1[i1 - 1];
        }
    for (int i1 = 1; i1 <= ADim; ++i1)
        for (int i2 = ARange[i1 - 1] + 1; i2 <= ARange[i1]; ++i2) {
            int i3 = Acols[i2 - 1];
            if (i3 != 0) out[i1 - 1] += Amat[i2 - 1] * x[i3 - 1];
        }
}

// gMRes, Working/AStrO_solvers.f90:128-297.  Returns the number of restart cycles run.
int orc_gmres(double *xVec, const double *Amat, const int32_t *Acols, const int32_t *ARange, int ASize, int ADim,
              const double *Cmat, const int32_t *Ccols, const int32_t *CRange, int CSize, int CDim, const double *Pmat,
              const int32_t *PRange, int PSize, const double *bVec, int numVecs, int maxIt) {
    (void)ASize;
    (void)CSize;
    const int n = ADim;
    std::vector<double> zVec(n), rVec(n), tempV1(std::max(n, numVecs + 1)), tempV2(std::max(n, numVecs + 1));
    std::vector<double> hMat((size_t)n * (numVecs + 1)), h2Ah((size_t)(numVecs + 1) * numVecs);
    std::vector<double> cbuf(std::max(CDim, 1)), mv(n), rhs(n);
    auto H = [&](int i, int j) -> double & { return hMat[(size_t)(j - 1) * n + i - 1]; };
    auto G = [&](int i, int j) -> double & { return h2Ah[(size_t)(j - 1) * (numVecs + 1) + i - 1]; };
    ref_matvec(mv, xVec, Amat, Acols, ARange, ADim, Cmat, Ccols, CRange, CDim, cbuf);
    for (int i = 0; i < n; ++i) rhs[i] = bVec[i] - mv[i];
    orc_ldl_solve(rVec.data(), rhs.data(), Pmat, PSize, PRange, n, zVec.data());
    double resMag = 0.0;
    for (int i = 0; i < n; ++i) resMag += rVec[i] * rVec[i];
    resMag = std::sqrt(resMag);
    int maxOutIt = maxIt / numVecs + 1;
    int i4 = 0;
    std::vector<double> col(n);
    while (resMag > F(1e-12) && i4 < maxOutIt) {
        for (int i = 1; i <= n; ++i) H(i, 1) = (1.0 / resMag) * rVec[i - 1];
        std::fill(h2Ah.begin(), h2Ah.end(), 0.0);
        for (int i5 = 2; i5 <= numVecs + 1; ++i5) {
            ref_matvec(mv, &H(1, i5 - 1), Amat, Acols, ARange, ADim, Cmat, Ccols, CRange, CDim, cbuf);
            orc_ldl_solve(&H(1, i5), mv.data(), Pmat, PSize, PRange, n, zVec.data());
            for (int i1 = 1; i1 <= i5 - 1; ++i1) {
                double dp = 0.0;
                for (int i2 = 1; i2 <= n; ++i2) dp += H(i2, i1) * H(i2, i5);
                for (int i2 = 1; i2 <= n; ++i2) H(i2, i5) = H(i2, i5) - dp * H(i2, i1);
                G(i1, i5 - 1) = dp;
            }
            double dp = 0.0;
            for (int i2 = 1; i2 <= n; ++i2) dp += H(i2, i5) * H(i2, i5);
            dp = std::sqrt(dp);
            for (int i2 = 1; i2 <= n; ++i2) H(i2, i5) = (1.0 / dp) * H(i2, i5);
            G(i5, i5 - 1) = dp;
        }
        rFactorMat(h2Ah, numVecs + 1, numVecs);
        std::fill(tempV1.begin(), tempV1.end(), 0.0);
        for (int i1 = 1; i1 <= n; ++i1)
            for (int i2 = 1; i2 <= numVecs + 1; ++i2) tempV1[i2 - 1] += H(i1, i2) * rVec[i1 - 1];
        std::fill(tempV2.begin(), tempV2.begin() + numVecs, 0.0);
        solveRFactor(tempV2.data(), h2Ah, tempV1.data(), numVecs + 1, numVecs);
        for (int i1 = 1; i1 <= n; ++i1)
            for (int i2 = 1; i2 <= numVecs; ++i2) xVec[i1 - 1] += H(i1, i2) * tempV2[i2 - 1];
        ref_matvec(mv, xVec, Amat, Acols, ARange, ADim, Cmat, Ccols, CRange, CDim, cbuf);
        for (int i = 0; i < n; ++i) rhs[i] = bVec[i] - mv[i];
        orc_ldl_solve(rVec.data(), rhs.data(), Pmat, PSize, PRange, n, zVec.data());
        resMag = 0.0;
        for (int i = 0; i < n; ++i) resMag += rVec[i] * rVec[i];
        resMag = std::sqrt(resMag);
        i4++;
    }
    return i4;
}

// getElasticAppliedLoad's design nodal loads (Working/AStrO_commandFunctions.f90:494-502):
// elasticLoad(nDofIndex(c, node)) += ndLd(c).
void orc_design_node_load(const OracleCtx *c, double t, double *elasticLoad) {
    DPert<double> p;
    for (int nd = 1; nd <= c->numNodes; ++nd) {
        double ld[7];
        t_node_dload(c->m, nd, t, p, ld);
        for (int k = 1; k <= 6; ++k) {
            const int dof = c->nDofIndex[6 * (nd - 1) + k - 1];
            if (dof > 0) elasticLoad[dof - 1] += ld[k - 1];
        }
    }
}

// getdRelasticdD's nodal-load branch (:1364-1373): dRudD(dof) -= Im(ndLd(d + i h)) / h at the nodes
// of the design variable (dToNd).
void orc_node_load_drdd(const OracleCtx *c, int dvar, double t, double h, double *dRudD) {
    const astro_model *m = c->m;
    if (!m->nd_to_d_range) return;
    DPert<cd> p;
    p.dvar = dvar;
    p.h = h;
    for (int nd = 1; nd <= c->numNodes; ++nd) {
        bool dep = false;
        for (int q = m->nd_to_d_range[nd - 1]; q < m->nd_to_d_range[nd]; ++q) dep = dep || m->nd_to_d[q] == dvar;
        if (!dep) continue;
        cd ld[7];
        t_node_dload(m, nd, t, p, ld);
        for (int k = 1; k <= 6; ++k) {
            const int dof = c->nDofIndex[6 * (nd - 1) + k - 1];
            if (dof > 0) dRudD[dof - 1] -= ld[k - 1].imag() / h;
        }
    }
}

// updateExternalRHS (Working/AStrO_commandFunctions.f90:568-607) with the Q9 loop bound resolved
// to the internal rows nodalDof+1..totalDof.
void orc_update_external_rhs(const OracleCtx *c, double *extVec, const double *intVec, const double *intElasticMat) {
    const astro_model *m = c->m;
    for (int i1 = 1; i1 <= c->numEls; ++i1) {
        const int et = m->element_type[i1 - 1];
        if (et != 41 && et != 81) continue;
        // r_getElementProfile: shell4 4 nodes x 6 DOF + 8 internal, brickIM 8 nodes x 3 DOF + 9
        const int nn = (et == 41) ? 4 : 8, nodalDof = 24, numInt = (et == 41) ? 8 : 9, totalDof = nodalDof + numInt;
        A2<double, 33, 33> K;
        K.fill(0.0);
        int i4 = c->intMatRange[i1 - 1] + 1;
        for (int i2 = 1; i2 <= totalDof; ++i2)
            for (int i3 = nodalDof + 1; i3 <= totalDof; ++i3) K(i3, i2) = intElasticMat[(i4++) - 1];
        double t1[33] = {0}, t2[33] = {0}, z[33] = {0};
        int v0 = c->intVecRange[i1 - 1];
        for (int k = 1; k <= numInt; ++k) t2[nodalDof + k - 1] = intVec[v0 + k - 1];
        t_SolveLUxb(t1, &K(1, 1), t2, z, 33, nodalDof + 1, totalDof);
        for (int i2 = 1; i2 <= nodalDof; ++i2) {
            int comp = (i2 - 1) / nn + 1, lnd = (i2 - 1) % nn + 1;
            int nd = m->element_list[8 * (i1 - 1) + lnd - 1];
            int i6 = c->nDofIndex[6 * (nd - 1) + comp - 1];
            for (int i3 = nodalDof + 1; i3 <= totalDof; ++i3) extVec[i6 - 1] -= K(i3, i2) * t1[i3 - 1];
        }
    }
}

// updateInternalSoln (:609-651), Q9 resolved likewise.
void orc_update_internal_soln(const OracleCtx *c, const double *extSoln, double *intSoln, const double *intRHS,
                              const double *intElasticMat) {
    const astro_model *m = c->m;
    for (int i1 = 1; i1 <= c->numEls; ++i1) {
        const int et = m->element_type[i1 - 1];
        if (et != 41 && et != 81) continue;
        const int nn = (et == 41) ? 4 : 8, nodalDof = 24, numInt = (et == 41) ? 8 : 9, totalDof = nodalDof + numInt;
        A2<double, 33, 33> K;
        K.fill(0.0);
        int i4 = c->intMatRange[i1 - 1] + 1;
        for (int i2 = 1; i2 <= totalDof; ++i2)
            for (int i3 = nodalDof + 1; i3 <= totalDof; ++i3) K(i3, i2) = intElasticMat[(i4++) - 1];
        double t1[33] = {0}, t2[33] = {0}, z[33] = {0};
        int v0 = c->intVecRange[i1 - 1];
        for (int k = 1; k <= numInt; ++k) t2[nodalDof + k - 1] = intRHS ? intRHS[v0 + k - 1] : 0.0;
        for (int i2 = 1; i2 <= nodalDof; ++i2) {
            int comp = (i2 - 1) / nn + 1, lnd = (i2 - 1) % nn + 1;
            int nd = m->element_list[8 * (i1 - 1) + lnd - 1];
            int i6 = c->nDofIndex[6 * (nd - 1) + comp - 1];
            for (int i3 = nodalDof + 1; i3 <= totalDof; ++i3) t2[i3 - 1] -= K(i3, i2) * extSoln[i6 - 1];
        }
        t_SolveLUxb(t1, &K(1, 1), t2, z, 33, nodalDof + 1, totalDof);
        for (int k = 1; k <= numInt; ++k) intSoln[v0 + k - 1] += t1[nodalDof + k - 1];
    }
}

// Consistent surface load with the intended semantics of the reference's surface branch
// (getElasticAppliedLoad :441-500, r_getElSurfaceTraction Working/AStrO_r_elementEqns.f90:1923-2018,
// faces from r_getElementFaces :288-332): Q8 resolved -- true face area (|dx/ds x dx/dt|), face
// shape function k applied to the face's k-th element node, contributions accumulated over faces.
// t = traction - pressure * n, with n the face normal of r_getElSurfaceNormal.
// getElasticAppliedLoad, body-force branch (Working/AStrO_commandFunctions.f90:393-441): for the
// listed elements (1-based; every element when nels = 0) r_getElBodyForce
// (Working/AStrO_r_elementEqns.f90:1801-1869) scattered into elasticLoad.  kind 0 'bodyForce'
// (vals = force per volume, 6 components), 1 'gravitational' (vals = acceleration, 6 components),
// 2 'centrifugal' (vals = center(3), axis(3), angVel; r_getElCentAcc, :1871-1921).
int orc_body_load(const OracleCtx *c, int kind, const double *vals, int nels, const int32_t *els, const astro_state *s,
                  double *elasticLoad) {
    const astro_model *m = c->m;
    GState g = to_gstate(s);
    DPert<double> p;
    const int count = nels > 0 ? nels : c->numEls;
    for (int k = 0; k < count; ++k) {
        const int el = nels > 0 ? els[k] : k + 1;
        ElemData<double> e;
        if (t_getElementData(e, m, c->nDofIndex.data(), c->intVecRange.data(), el, g, p) != 0) return 1;
        double bdy[6];
        if (kind == 2) {
            double cent[3] = {0.0, 0.0, 0.0};
            for (int i1 = 1; i1 <= e.numNds; ++i1)
                for (int i2 = 1; i2 <= 3; ++i2) cent[i2 - 1] = cent[i2 - 1] + e.globNds(i2, i1) + e.disp(i2, i1);
            double nnInv = (double)e.numNds;
            nnInv = 1.0 / nnInv;
            for (int i2 = 0; i2 < 3; ++i2) cent[i2] = nnInv * cent[i2];
            double pos[3], unit[3];
            for (int i2 = 0; i2 < 3; ++i2) pos[i2] = cent[i2] - vals[i2];
            double dp = vals[3] * vals[3] + vals[4] * vals[4] + vals[5] * vals[5];
            const double mag = std::sqrt(dp);
            for (int i2 = 0; i2 < 3; ++i2) unit[i2] = (1.0 / mag) * vals[3 + i2];
            dp = pos[0] * unit[0] + pos[1] * unit[1] + pos[2] * unit[2];
            for (int i2 = 0; i2 < 3; ++i2) pos[i2] = pos[i2] - dp * unit[i2];
            for (int i2 = 0; i2 < 3; ++i2) bdy[i2] = vals[6] * vals[6] * pos[i2];
            bdy[3] = bdy[4] = bdy[5] = 0.0;
        } else {
            for (int i2 = 0; i2 < 6; ++i2) bdy[i2] = vals[i2];
        }
        A1<double, 33> ndFrc;
        ndFrc.fill(0.0);
        if (kind >= 1) {
            // isGrav: the element's mass residual for the acceleration bdy at every node, with the
            // static orientation of the element's mean rotation
            A1<double, 3> statRot;
            statRot.fill(0.0);
            for (int i4 = 1; i4 <= e.numNds; ++i4)
                for (int q = 1; q <= 3; ++q) statRot(q) = statRot(q) + e.disp(3 + q, i4);
            double nnInv = (double)e.numNds;
            nnInv = 1.0 / nnInv;
            for (int q = 1; q <= 3; ++q) statRot(q) = nnInv * statRot(q);
            A2<double, 3, 48> statInOri;
            A2<double, 3, 16> statdrIdrG;
            t_getInstOrient(statInOri, statdrIdrG, e.orient, statRot);
            for (int cc = 4; cc <= 48; ++cc)
                for (int r = 1; r <= 3; ++r) statInOri(r, cc) = 0.0;
            for (int cc = 4; cc <= 16; ++cc)
                for (int r = 1; r <= 3; ++r) statdrIdrG(r, cc) = 0.0;
            A2<double, 6, 11> fakeAcc;
            fakeAcc.fill(0.0);
            for (int i1 = 1; i1 <= e.numNds; ++i1)
                for (int r = 1; r <= 6; ++r) fakeAcc(r, i1) = bdy[r - 1];
            A2<double, 33, 33> dRdA;
            t_getElRum(ndFrc, dRdA, 0, e, statInOri, statdrIdrG, statRot, e.disp, fakeAcc);
        } else {
            for (int i1 = 1; i1 <= e.numIntPts; ++i1) {
                A1<double, 11> Nvec;
                A2<double, 11, 3> Nx;
                double detJ;
                t_getIntPtData(Nvec, Nx, detJ, e.locNds, e.intPts[i1 - 1], e.eType, e.numNds);
                const int i3 = e.numNds * e.dofPerNd;
                detJ = detJ * e.ipWt[i1 - 1];
                for (int i2 = 1; i2 <= i3; ++i2) {
                    const int i4 = e.dofTable[i2 - 1][0], i5 = e.dofTable[i2 - 1][1];
                    ndFrc(i2) = ndFrc(i2) + bdy[i4 - 1] * Nvec(i5) * detJ;
                }
            }
            if (e.eType == 41) {
                // r_getElThickOffset: the section's total thickness
                const int sec = m->element_section[el - 1];
                double thick = 0.0;
                for (int i1 = m->sec_layup_range[sec - 1] + 1, ln = 1; i1 <= m->sec_layup_range[sec]; ++i1, ++ln)
                    thick = thick + layer_thickness(m, el, ln, i1, p);
                for (int q = 1; q <= 33; ++q) ndFrc(q) = thick * ndFrc(q);
            }
        }
        const int ndDof = e.numNds * e.dofPerNd;
        for (int i4 = 1; i4 <= ndDof; ++i4) {
            const int i5 = e.dofTable[i4 - 1][0];
            const int i6 = m->element_list[8 * (el - 1) + e.dofTable[i4 - 1][1] - 1];
            const int i7 = c->nDofIndex[6 * (i6 - 1) + i5 - 1];
            elasticLoad[i7 - 1] += ndFrc(i4);
        }
    }
    return 0;
}

void orc_surface_load(const OracleCtx *c, int nfaces, const int32_t *faceEl, const int32_t *faceNum,
                      const double *traction, double pressure, double *elasticLoad) {
    DPert<double> p;
    for (int f = 0; f < nfaces; ++f) {
        int nodes[4];
        double val[4][3];
        t_face_load(c->m, faceEl[f], faceNum[f], traction, pressure, p, nodes, val);
        for (int k = 0; k < 4; ++k)
            for (int d = 0; d < 3; ++d) {
                const int dof = c->nDofIndex[6 * (nodes[k] - 1) + d];
                elasticLoad[dof - 1] += val[k][d];
            }
    }
}

// ---- thermal path ---------------------------------------------------------------------------
// Thermal material data are not part of astro_model: materialThermCond(6, num_materials)
// (k11 k22 k33 k12 k13 k23) and materialSpecHeat(num_materials) are passed beside it.

}  // extern "C"

// v += the element's terms of one design category (layer / component 0 = any), one term at a time
// in the element's term order, as the property routines loop over elToD.
template <class T>
static void th_terms(const astro_model *m, int el, T &v, int cat, int layer, int comp, const DPert<T> &p) {
    if (m->num_dvars <= 0 || !m->el_to_d_range) return;
    for (int q = m->el_to_d_range[el - 1]; q < m->el_to_d_range[el]; ++q) {
        const int d = m->el_to_d[q];
        if (m->d_category[d - 1] != cat) continue;
        if (layer && (!m->d_layer || m->d_layer[d - 1] != layer)) continue;
        if (comp && (!m->d_component || m->d_component[d - 1] != comp)) continue;
        v = v + m->el_to_coef[q] * dval(m, d, p);
    }
}

// r_getMaterialThermCond (Working/AStrO_r_designPropertyFunctions.f90:129-161, 'thermalCond' terms)
// for solids and r_getShellThermCond (:527-600: sum over layers of the layer thickness times the
// layer conductivity rotated by the layup angle, the layer's 'layup' thermalCond / angle /
// thickness terms applied) for shells; thisSH as r_getElRtm selects it
// (Working/AStrO_r_elementEqns.f90:2136-2142): density (r_getMaterialDensity :82-103) x specHeat
// (r_getMaterialSpecHeat :164-186) for solids, r_getShellSpecHeat (:602-644: sum of thickness x
// density x specHeat, each with its layer terms) for shells.  secThick: the shell section
// thickness (r_getElThickOffset).  Design variable p.dvar at d + i h.
template <class T>
static void therm_props(const astro_model *m, const double *cond, const double *sh, int el, T tc[3][3], T &thisSH,
                        T &secThick, const DPert<T> &p) {
    const int et = m->element_type[el - 1], sec = m->element_section[el - 1];
    auto fill = [](T t[3][3], const T *v) {
        t[0][0] = v[0];
        t[1][1] = v[1];
        t[2][2] = v[2];
        t[0][1] = t[1][0] = v[3];
        t[0][2] = t[2][0] = v[4];
        t[1][2] = t[2][1] = v[5];
    };
    secThick = T(0.0);
    if (et != 41) {
        const int mat = m->section_mat_id[sec - 1];
        T cv[6];
        for (int k = 0; k < 6; ++k) {
            cv[k] = T(cond[6 * (mat - 1) + k]);
            th_terms(m, el, cv[k], ASTRO_DCAT_THERMAL_COND, 0, k + 1, p);
        }
        fill(tc, cv);
        T den = T(m->material_density ? m->material_density[mat - 1] : 0.0), spec = T(sh[mat - 1]);
        th_terms(m, el, den, ASTRO_DCAT_DENSITY, 0, 0, p);
        th_terms(m, el, spec, ASTRO_DCAT_SPEC_HEAT, 0, 0, p);
        thisSH = den * spec;
        return;
    }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) tc[i][j] = T(0.0);
    thisSH = T(0.0);
    for (int i1 = m->sec_layup_range[sec - 1] + 1, ln = 1; i1 <= m->sec_layup_range[sec]; ++i1, ++ln) {
        const int mat = m->layup_mat_id[i1 - 1];
        T cv[6], tl[3][3], al[3][3], pr[3][3], tg[3][3];
        for (int k = 0; k < 6; ++k) {
            cv[k] = T(cond[6 * (mat - 1) + k]);
            th_terms(m, el, cv[k], ASTRO_DCAT_LAYUP_THERMAL_COND, ln, k + 1, p);
        }
        fill(tl, cv);
        T ang = T(m->layup_angle[i1 - 1]), den = T(m->material_density ? m->material_density[mat - 1] : 0.0),
          spec = T(sh[mat - 1]);
        th_terms(m, el, ang, ASTRO_DCAT_LAYUP_ANGLE, ln, 0, p);
        th_terms(m, el, den, ASTRO_DCAT_LAYUP_DENSITY, ln, 0, p);
        th_terms(m, el, spec, ASTRO_DCAT_LAYUP_SPEC_HEAT, ln, 0, p);
        const T lt = layer_thickness(m, el, ln, i1, p);
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) al[a][b] = T(0.0);
        al[2][2] = T(1.0);
        al[0][0] = t_cos(ang);
        al[1][0] = t_sin(ang);
        al[0][1] = -al[1][0];
        al[1][1] = al[0][0];
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                pr[a][b] = T(0.0);
                for (int k = 0; k < 3; ++k) pr[a][b] = pr[a][b] + tl[a][k] * al[b][k];
            }
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                tg[a][b] = T(0.0);
                for (int k = 0; k < 3; ++k) tg[a][b] = tg[a][b] + al[a][k] * pr[k][b];
            }
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) tc[a][b] = tc[a][b] + lt * tg[a][b];
        thisSH = thisSH + lt * den * spec;
        secThick = secThick + lt;
    }
}

extern "C" {

// getThermalSolnLoad (Working/AStrO_commandFunctions.f90:16-72) with r_getElRt / r_getElRtk /
// r_getElRtm (Working/AStrO_r_elementEqns.f90:2062-2204): thermalLoad(rank) -= Rt, and for
// buildMat the CSR thermMat over ranks with find-or-insert columns (0 = empty slot).  Node
// vectors (temperature, previous temperature and rate) are in rank order, as nodeTemp.  The CSR
// row ranges (thermMatRange: 1 + the node's neighbours, allocateThermalMat, bookKeeping
// :413-441) are returned in range (0:numNodes) when non-null.
int orc_thermal_soln_load(const OracleCtx *c, const double *cond, const double *sh, int buildMat,
                          const double *nodeTemp, const double *prevTemp, const double *prevTdot, int dynamic,
                          double gamma, double delT, double *thermalLoad, double *thermMat, int32_t *thermCols,
                          int32_t *range) {
    const astro_model *m = c->m;
    const int N = c->numNodes;
    std::vector<int> tr(N + 1, 0);
    for (int i1 = 1; i1 <= N; ++i1) {
        const int i3 = c->currentRank[i1 - 1];
        tr[i3] = tr[i3] + 1;
        for (int i4 = c->nCRange[i1 - 1] + 1; i4 <= c->nCRange[i1]; ++i4)
            if (c->nodalConn[i4 - 1] != 0) tr[i3] = tr[i3] + 1;
    }
    for (int i1 = 2; i1 <= N; ++i1) tr[i1] += tr[i1 - 1];
    if (range)
        for (int i = 0; i <= N; ++i) range[i] = tr[i];
    if (buildMat == 1)
        for (int i = 0; i < tr[N]; ++i) {
            thermMat[i] = 0.0;
            thermCols[i] = 0;
        }
    GState g;
    DPert<double> p;
    for (int el = 1; el <= c->numEls; ++el) {
        ElemData<double> e;
        if (t_getElementData(e, m, c->nDofIndex.data(), c->intVecRange.data(), el, g, p) != 0) return 1;
        double tc[3][3], thisSH, secThick;
        therm_props(m, cond, sh, el, tc, thisSH, secThick, p);
        const int nn = e.numNds;
        double temp[10] = {0}, pT[10] = {0}, pTd[10] = {0};
        for (int i = 0; i < nn; ++i) {
            const int rk = c->currentRank[m->element_list[8 * (el - 1) + i] - 1];
            temp[i] = nodeTemp ? nodeTemp[rk - 1] : 0.0;
            pT[i] = prevTemp ? prevTemp[rk - 1] : 0.0;
            pTd[i] = prevTdot ? prevTdot[rk - 1] : 0.0;
        }
        double Rt[10] = {0}, dRdt[10][10] = {{0}};
        // r_getElRtk
        for (int i1 = 1; i1 <= e.numIntPts; ++i1) {
            A1<double, 11> Nvec;
            A2<double, 11, 3> Nx;
            double detJ;
            t_getIntPtData(Nvec, Nx, detJ, e.locNds, e.intPts[i1 - 1], e.eType, nn);
            double Tx[3] = {0, 0, 0}, q[3] = {0, 0, 0};
            for (int i2 = 1; i2 <= nn; ++i2)
                for (int i3 = 1; i3 <= 3; ++i3) Tx[i3 - 1] = Tx[i3 - 1] + Nx(i2, i3) * temp[i2 - 1];
            for (int i2 = 0; i2 < 3; ++i2)
                for (int i3 = 0; i3 < 3; ++i3) q[i2] = q[i2] + tc[i2][i3] * Tx[i3];
            const double wd = detJ * e.ipWt[i1 - 1];
            for (int k = 0; k < 3; ++k) q[k] = wd * q[k];
            for (int i2 = 1; i2 <= nn; ++i2)
                for (int i3 = 1; i3 <= 3; ++i3) Rt[i2 - 1] = Rt[i2 - 1] + Nx(i2, i3) * q[i3 - 1];
            if (buildMat == 1) {
                double kNx[11][3] = {{0}};
                for (int i2 = 1; i2 <= nn; ++i2)
                    for (int i3 = 1; i3 <= 3; ++i3)
                        for (int i4 = 1; i4 <= 3; ++i4) kNx[i2 - 1][i3 - 1] = kNx[i2 - 1][i3 - 1] + Nx(i2, i4) * tc[i4 - 1][i3 - 1];
                for (int i2 = 0; i2 < nn; ++i2)
                    for (int k = 0; k < 3; ++k) kNx[i2][k] = wd * kNx[i2][k];
                for (int i2 = 1; i2 <= nn; ++i2)
                    for (int i3 = 1; i3 <= nn; ++i3)
                        for (int i4 = 1; i4 <= 3; ++i4) dRdt[i2 - 1][i3 - 1] = dRdt[i2 - 1][i3 - 1] + Nx(i2, i4) * kNx[i3 - 1][i4 - 1];
            }
        }
        if (dynamic == 1) {
            // r_getElRtm with Tdot from the generalised trapezoid rule
            double Td[10];
            for (int i1 = 0; i1 < nn; ++i1)
                Td[i1] = (1.0 / gamma) * ((1.0 / delT) * (temp[i1] - pT[i1]) - 1.0 * (1.0 - gamma) * pTd[i1]);
            double Rtm[10] = {0}, dRdTd[10][10] = {{0}};
            for (int i1 = 1; i1 <= e.numIntPts; ++i1) {
                A1<double, 11> Nvec;
                A2<double, 11, 3> Nx;
                double detJ;
                t_getIntPtData(Nvec, Nx, detJ, e.locNds, e.intPts[i1 - 1], e.eType, nn);
                double pt = 0.0;
                for (int i2 = 1; i2 <= nn; ++i2) pt = pt + Td[i2 - 1] * Nvec(i2);
                pt = detJ * e.ipWt[i1 - 1] * thisSH * pt;
                for (int i2 = 1; i2 <= nn; ++i2) Rtm[i2 - 1] = Rtm[i2 - 1] + pt * Nvec(i2);
                if (buildMat == 1) {
                    double cpN[11];
                    for (int i2 = 1; i2 <= 11; ++i2) cpN[i2 - 1] = detJ * e.ipWt[i1 - 1] * thisSH * Nvec(i2);
                    for (int i2 = 1; i2 <= nn; ++i2)
                        for (int i3 = 1; i3 <= nn; ++i3) dRdTd[i2 - 1][i3 - 1] = dRdTd[i2 - 1][i3 - 1] + Nvec(i2) * cpN[i3 - 1];
                }
            }
            for (int k = 0; k < nn; ++k) Rt[k] = Rt[k] + Rtm[k];
            if (buildMat == 1)
                for (int a = 0; a < nn; ++a)
                    for (int b = 0; b < nn; ++b) dRdt[a][b] = dRdt[a][b] + (1.0 / (gamma * delT)) * dRdTd[a][b];
        }
        for (int i2 = 1; i2 <= nn; ++i2) {
            const int i3 = c->currentRank[m->element_list[8 * (el - 1) + i2 - 1] - 1];
            thermalLoad[i3 - 1] = thermalLoad[i3 - 1] - Rt[i2 - 1];
        }
        if (buildMat == 1)
            for (int i2 = 1; i2 <= nn; ++i2) {
                const int Kgi = c->currentRank[m->element_list[8 * (el - 1) + i2 - 1] - 1];
                for (int i3 = 1; i3 <= nn; ++i3) {
                    const int Kgj = c->currentRank[m->element_list[8 * (el - 1) + i3 - 1] - 1];
                    int i4 = tr[Kgi - 1] + 1;
                    int inserted = 0;
                    while (inserted == 0 && i4 <= tr[Kgi]) {
                        const int i6 = thermCols[i4 - 1];
                        if (i6 == 0) {
                            thermMat[i4 - 1] = dRdt[i2 - 1][i3 - 1];
                            thermCols[i4 - 1] = Kgj;
                            inserted = 1;
                        } else if (i6 == Kgj) {
                            thermMat[i4 - 1] = thermMat[i4 - 1] + dRdt[i2 - 1][i3 - 1];
                            inserted = 1;
                        }
                        i4 = i4 + 1;
                    }
                }
            }
    }
    return 0;
}


// getdRthermaldD (Working/AStrO_commandFunctions.f90:1016-1170), element part (:1040-1059):
// dRtdD (rank order) zeroed, then for every element that depends on dvar c_getElRt with buildMat
// 0 (c_getElRtk, plus c_getElRtm when dynamic, Working/AStrO_c_elementEqns.f90) at d + i h, and
// Im(Rt) / h summed at the element's nodes.  Temperatures as orc_thermal_soln_load.
int orc_thermal_drdd(const OracleCtx *c, const double *cond, const double *sh, int dvar, double h,
                     const double *nodeTemp, const double *prevTemp, const double *prevTdot, int dynamic,
                     double gamma, double delT, double *dRtdD) {
    const astro_model *m = c->m;
    std::fill(dRtdD, dRtdD + c->numNodes, 0.0);
    if (dvar < 1 || dvar > m->num_dvars) return 1;
    GState g;
    DPert<cd> p;
    p.dvar = dvar;
    p.h = h;
    for (int el = 1; el <= c->numEls; ++el) {
        if (!el_depends(m, el, dvar)) continue;
        ElemData<cd> e;
        if (t_getElementData(e, m, c->nDofIndex.data(), c->intVecRange.data(), el, g, p) != 0) return 1;
        cd tc[3][3], thisSH, secThick;
        therm_props(m, cond, sh, el, tc, thisSH, secThick, p);
        const int nn = e.numNds;
        double temp[10] = {0}, Td[10] = {0};
        int rk[10];
        for (int i = 0; i < nn; ++i) {
            rk[i] = c->currentRank[m->element_list[8 * (el - 1) + i] - 1];
            temp[i] = nodeTemp ? nodeTemp[rk[i] - 1] : 0.0;
            const double pT = prevTemp ? prevTemp[rk[i] - 1] : 0.0, pTd = prevTdot ? prevTdot[rk[i] - 1] : 0.0;
            if (dynamic == 1) Td[i] = (1.0 / gamma) * ((1.0 / delT) * (temp[i] - pT) - 1.0 * (1.0 - gamma) * pTd);
        }
        cd Rt[10];
        for (int i = 0; i < 10; ++i) Rt[i] = cd(0.0);
        for (int i1 = 1; i1 <= e.numIntPts; ++i1) {
            A1<cd, 11> Nvec;
            A2<cd, 11, 3> Nx;
            cd detJ;
            t_getIntPtData(Nvec, Nx, detJ, e.locNds, e.intPts[i1 - 1], e.eType, nn);
            cd Tx[3] = {cd(0.0), cd(0.0), cd(0.0)}, q[3] = {cd(0.0), cd(0.0), cd(0.0)};
            for (int i2 = 1; i2 <= nn; ++i2)
                for (int i3 = 1; i3 <= 3; ++i3) Tx[i3 - 1] = Tx[i3 - 1] + Nx(i2, i3) * temp[i2 - 1];
            for (int i2 = 0; i2 < 3; ++i2)
                for (int i3 = 0; i3 < 3; ++i3) q[i2] = q[i2] + tc[i2][i3] * Tx[i3];
            const cd wd = detJ * e.ipWt[i1 - 1];
            for (int k = 0; k < 3; ++k) q[k] = wd * q[k];
            for (int i2 = 1; i2 <= nn; ++i2)
                for (int i3 = 1; i3 <= 3; ++i3) Rt[i2 - 1] = Rt[i2 - 1] + Nx(i2, i3) * q[i3 - 1];
        }
        if (dynamic == 1) {
            cd Rtm[10];
            for (int i = 0; i < 10; ++i) Rtm[i] = cd(0.0);
            for (int i1 = 1; i1 <= e.numIntPts; ++i1) {
                A1<cd, 11> Nvec;
                A2<cd, 11, 3> Nx;
                cd detJ;
                t_getIntPtData(Nvec, Nx, detJ, e.locNds, e.intPts[i1 - 1], e.eType, nn);
                cd pt = cd(0.0);
                for (int i2 = 1; i2 <= nn; ++i2) pt = pt + Td[i2 - 1] * Nvec(i2);
                pt = detJ * e.ipWt[i1 - 1] * thisSH * pt;
                for (int i2 = 1; i2 <= nn; ++i2) Rtm[i2 - 1] = Rtm[i2 - 1] + pt * Nvec(i2);
            }
            for (int k = 0; k < nn; ++k) Rt[k] = Rt[k] + Rtm[k];
        }
        for (int i = 0; i < nn; ++i) dRtdD[rk[i] - 1] += (1.0 / h) * Rt[i].imag();
    }
    return 0;
}

// getdRthermaldD's bodyHeatGen branch (:1065-1108): for the listed elements (all when nels = 0;
// an element listed twice counts twice) that depend on dvar, c_getElBodyForce with the heat
// generation q as the first body-force component (times the section thickness for shells), and
// dRtdD(rank) -= Im(component-1 nodal value) / h.
int orc_thermal_heat_gen_drdd(const OracleCtx *c, int dvar, double h, double q, int nels, const int32_t *els,
                              double *dRtdD) {
    const astro_model *m = c->m;
    if (dvar < 1 || dvar > m->num_dvars) return 1;
    GState g;
    DPert<cd> p;
    p.dvar = dvar;
    p.h = h;
    const int count = nels > 0 ? nels : c->numEls;
    for (int k = 0; k < count; ++k) {
        const int el = nels > 0 ? els[k] : k + 1;
        if (!el_depends(m, el, dvar)) continue;
        ElemData<cd> e;
        if (t_getElementData(e, m, c->nDofIndex.data(), c->intVecRange.data(), el, g, p) != 0) return 1;
        cd w[10];
        for (int i = 0; i < 10; ++i) w[i] = cd(0.0);
        for (int i1 = 1; i1 <= e.numIntPts; ++i1) {
            A1<cd, 11> Nvec;
            A2<cd, 11, 3> Nx;
            cd detJ;
            t_getIntPtData(Nvec, Nx, detJ, e.locNds, e.intPts[i1 - 1], e.eType, e.numNds);
            detJ = detJ * e.ipWt[i1 - 1];
            for (int a = 1; a <= e.numNds; ++a) w[a - 1] = w[a - 1] + q * Nvec(a) * detJ;
        }
        if (e.eType == 41) {
            const int sec = m->element_section[el - 1];
            cd thick = cd(0.0);
            for (int i1 = m->sec_layup_range[sec - 1] + 1, ln = 1; i1 <= m->sec_layup_range[sec]; ++i1, ++ln)
                thick = thick + layer_thickness(m, el, ln, i1, p);
            for (int a = 0; a < e.numNds; ++a) w[a] = thick * w[a];
        }
        for (int a = 0; a < e.numNds; ++a)
            dRtdD[c->currentRank[m->element_list[8 * (el - 1) + a] - 1] - 1] -= w[a].imag() / h;
    }
    return 0;
}

// getdRthermaldD's surfaceFlux branch (:1109-1152): for the given faces whose element depends on
// dvar, the face load of the flux as the first traction component at d + i h, and
// dRtdD(rank) += Im(component-1 nodal value) / h.
int orc_thermal_surface_flux_drdd(const OracleCtx *c, int dvar, double h, int nfaces, const int32_t *faceEl,
                                  const int32_t *faceNum, double flux, double *dRtdD) {
    const astro_model *m = c->m;
    if (dvar < 1 || dvar > m->num_dvars) return 1;
    DPert<cd> p;
    p.dvar = dvar;
    p.h = h;
    const double tr[3] = {flux, 0.0, 0.0};
    for (int f = 0; f < nfaces; ++f) {
        if (!el_depends(m, faceEl[f], dvar)) continue;
        int nodes[4];
        cd val[4][3];
        t_face_load(m, faceEl[f], faceNum[f], tr, 0.0, p, nodes, val);
        for (int k = 0; k < 4; ++k) dRtdD[c->currentRank[nodes[k] - 1] - 1] += val[k][0].imag() / h;
    }
    return 0;
}

// getThermalAppliedLoad's closing loop (:182-186): thermalLoad(rank) += ndLd(7) of every node.
void orc_thermal_design_node_load(const OracleCtx *c, double t, double *thermalLoad) {
    DPert<double> p;
    for (int nd = 1; nd <= c->numNodes; ++nd) {
        double ld[7];
        t_node_dload(c->m, nd, t, p, ld);
        thermalLoad[c->currentRank[nd - 1] - 1] += ld[6];
    }
}

// getdRthermaldD's node branch (:1162-1167): dRtdD(rank) -= Im(ndLd(7)(d + i h)) / h at the nodes of
// the design variable.
void orc_thermal_node_load_drdd(const OracleCtx *c, int dvar, double t, double h, double *dRtdD) {
    const astro_model *m = c->m;
    if (!m->nd_to_d_range) return;
    DPert<cd> p;
    p.dvar = dvar;
    p.h = h;
    for (int nd = 1; nd <= c->numNodes; ++nd) {
        bool dep = false;
        for (int q = m->nd_to_d_range[nd - 1]; q < m->nd_to_d_range[nd]; ++q) dep = dep || m->nd_to_d[q] == dvar;
        if (!dep) continue;
        cd ld[7];
        t_node_dload(m, nd, t, p, ld);
        dRtdD[c->currentRank[nd - 1] - 1] -= ld[6].imag() / h;
    }
}

}  // extern "C"
