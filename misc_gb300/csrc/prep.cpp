// Host-side analysis preparation: integer set-up run once per context.
//
// Produces the reference's own numbering so that exported arrays are interchangeable with the
// Fortran's (analysisPrep, Working/AStrO_bookKeeping.f90:794-1039):
//   * node adjacency in first-seen order (nodalConn without its empty slots, :822-882);
//   * breadth-first node ranks from the node with the fewest element incidences, with the
//     nearest-unnumbered-node restart (levelSortNodes, :233-331);
//   * component-major DOF numbers (:900-912), CSR row lengths and skyline profile
//     (allocateElasticMat, :333-411) with the bandwidth cap solverMaxBW of the *solve command
//     (Working/AStrO_runJob.f90:106-114, 32-bit wrapping arithmetic as in the reference);
//   * the constraint matrix of pre-expanded equations (buildElasticMPC, :474-612).
// GPU-specific structures built here: the rank-ordered block-CSR pattern, the element-to-block
// scatter map, a greedy element colouring (no two elements of a colour share a node), and the
// position of every block entry inside the reference CSR row (the reference fills rows by
// find-or-insert in element order, Working/AStrO_commandFunctions.f90:323-347; that order depends
// only on the row's node, so one sequence per node describes all its rows).
#include <algorithm>
#include <cmath>
#include <cstring>

#include "astro_internal.h"

static int solver_max_bw(int numNodes) {
    int32_t target = (int32_t)((uint32_t)27u * (uint32_t)numNodes * (uint32_t)numNodes);
    int32_t b = 1, b3 = 1;
    while (b3 < target) {
        ++b;
        b3 = (int32_t)((uint32_t)b * (uint32_t)b * (uint32_t)b);
    }
    return b;
}

int astro_prep_build(astro_ctx *c, const astro_model *m) {
    AstroPrep &P = c->P;
    const int N = m->num_nodes, E = m->num_els;
    P.N = N;
    P.E = E;
    int nSolidEl = 0, nShellEl = 0;
    for (int e = 0; e < E; ++e) {
        int t = m->element_type[e];
        if (t == 8 || t == 81) nSolidEl++;
        else if (t == 41) nShellEl++;
        else return set_err(c, ASTRO_ERR_UNSUPPORTED, "element type " + std::to_string(t) +
                                                          " is not supported (8 = brick8, 81 = brickIM, 41 = shell4)");
    }
    if (nSolidEl && nShellEl) return set_err(c, ASTRO_ERR_UNSUPPORTED, "meshes mixing solid and shell4 elements are not supported");
    c->hasSolid = nSolidEl > 0;
    c->hasShell = nShellEl > 0;
    P.dpn = c->hasShell ? 6 : 3;
    P.npe = c->hasShell ? 4 : 8;
    const int dpn = P.dpn, npe = P.npe;
    auto EL = [&](int e, int k) { return m->element_list[8 * e + k]; };  // 0-based e, k
    for (int e = 0; e < E; ++e)
        for (int k = 0; k < 8; ++k) {
            int nd = EL(e, k);
            if (nd < 0 || nd > N) return set_err(c, ASTRO_ERR_ARG, "element_list entry out of range");
            if (k < npe && nd == 0) return set_err(c, ASTRO_ERR_ARG, "element with a missing node");
        }
    // element incidences per node (nCRange differences) and first-seen adjacency
    std::vector<int> incid(N + 1, 0), used(N + 1, 0);
    std::vector<std::vector<int>> adjL(N + 1);
    for (int e = 0; e < E; ++e)
        for (int i2 = 0; i2 < 8; ++i2) {
            int a = EL(e, i2);
            if (!a) continue;
            used[a] = 1;
            for (int i4 = 0; i4 < 8; ++i4) {
                int b = EL(e, i4);
                if (!b || b == a) continue;
                incid[a]++;
                auto &L = adjL[a];
                if (std::find(L.begin(), L.end(), b) == L.end()) L.push_back(b);
            }
        }
    for (int a = 1; a <= N; ++a)
        if (!used[a]) return set_err(c, ASTRO_ERR_UNSUPPORTED, "node " + std::to_string(a) + " belongs to no element");
    P.adjPtr.assign(N + 2, 0);
    for (int a = 1; a <= N; ++a) P.adjPtr[a + 1] = P.adjPtr[a] + (int)adjL[a].size();
    P.adj.resize(P.adjPtr[N + 1]);
    for (int a = 1; a <= N; ++a) std::copy(adjL[a].begin(), adjL[a].end(), P.adj.begin() + P.adjPtr[a]);
    // breadth-first ranks
    P.solverMaxBW = solver_max_bw(N);
    P.originalRank.assign(N + 1, 0);
    std::vector<char> ins(N + 1, 0);
    auto nearest = [&](int from) {
        double best = 1e100;
        int pick = 0;
        const double *xf = m->node_list + 3 * (from - 1);
        for (int q = 1; q <= N; ++q) {
            if (ins[q]) continue;
            const double *xq = m->node_list + 3 * (q - 1);
            double dx = xq[0] - xf[0], dy = xq[1] - xf[1], dz = xq[2] - xf[2];
            double d = std::sqrt(dx * dx + dy * dy + dz * dz);
            if (d < best) {
                best = d;
                pick = q;
            }
        }
        return pick;
    };
    {
        int start = 0, minCon = 1000;
        for (int a = 1; a <= N; ++a)
            if (incid[a] < minCon) {
                minCon = incid[a];
                start = a;
            }
        int next = 1;
        P.originalRank[next] = start;
        ins[start] = 1;
        int cur = start, curInd = next, blockSt = next;
        ++next;
        while (next <= N) {
            for (int q = P.adjPtr[cur]; q < P.adjPtr[cur + 1]; ++q) {
                int b = P.adj[q];
                if (ins[b]) continue;
                P.originalRank[next++] = b;
                ins[b] = 1;
                if (next - blockSt == N && next <= N) {  // block restart (solverBlockDim = numNodes)
                    int s = nearest(b);
                    P.originalRank[next] = s;
                    cur = s;
                    curInd = next;
                    ins[s] = 1;
                    blockSt = next;
                    ++next;
                    q = P.adjPtr[cur] - 1;
                }
            }
            ++curInd;
            if (curInd == next && next <= N) {
                int s = nearest(P.originalRank[next - 1]);
                P.originalRank[next] = s;
                curInd = next;
                ins[s] = 1;
                ++next;
            }
            if (curInd <= N) cur = P.originalRank[curInd];
        }
    }
    P.currentRank.assign(N + 1, 0);
    for (int r = 1; r <= N; ++r) P.currentRank[P.originalRank[r]] = r;
    // component-major DOF numbers
    P.n = dpn * N;
    const int n = P.n;
    P.nDofIndex.assign(6 * N, 0);
    for (int a = 1; a <= N; ++a)
        for (int k = 1; k <= dpn; ++k) P.nDofIndex[6 * (a - 1) + k - 1] = P.currentRank[a] + (k - 1) * N;
    // CSR row lengths: dpn * (1 + degree); skyline profile per row
    P.elMatRange.assign(n + 1, 0);
    P.elMatLTRange.assign(n + 1, 0);
    for (int a = 1; a <= N; ++a) {
        int deg = P.adjPtr[a + 1] - P.adjPtr[a];
        int ra = P.currentRank[a];
        int minR = ra;
        for (int q = P.adjPtr[a]; q < P.adjPtr[a + 1]; ++q) {
            int rb = P.currentRank[P.adj[q]];
            int d = ra - rb;
            if (d >= 0 && d <= P.solverMaxBW) minR = std::min(minR, rb);
        }
        for (int k = 1; k <= dpn; ++k) {
            int dof = ra + (k - 1) * N;
            P.elMatRange[dof] = dpn * (1 + deg);
            P.elMatLTRange[dof] = ra - minR + 1;
        }
    }
    for (int i = 1; i <= n; ++i) {
        P.elMatRange[i] += P.elMatRange[i - 1];
        P.elMatLTRange[i] += P.elMatLTRange[i - 1];
    }
    P.elMatSize = P.elMatRange[n];
    P.ltSize = P.elMatLTRange[n];
    // internal DOF ranges (allocateElasticMat, Working/AStrO_bookKeeping.f90:978-1003): shell4 8
    // internal DOF, 8 x 32 condensed rows; brickIM 9 internal DOF, 9 x 33 rows
    P.intVecRange.assign(E + 1, 0);
    P.intMatRange.assign(E + 1, 0);
    for (int e = 1; e <= E; ++e) {
        int t = m->element_type[e - 1];
        P.intVecRange[e] = P.intVecRange[e - 1] + (t == 41 ? 8 : (t == 81 ? 9 : 0));
        P.intMatRange[e] = P.intMatRange[e - 1] + (t == 41 ? 256 : (t == 81 ? 297 : 0));
    }
    P.intVecSize = P.intVecRange[E];
    P.intMatSize = P.intMatRange[E];
    // block-CSR pattern over ranks: row r holds r and its neighbours, sorted
    P.bRowPtr.assign(N + 1, 0);
    std::vector<int> tmp;
    for (int r = 1; r <= N; ++r) {
        int a = P.originalRank[r];
        P.bRowPtr[r] = P.bRowPtr[r - 1] + 1 + (P.adjPtr[a + 1] - P.adjPtr[a]);
    }
    P.nb = P.bRowPtr[N];
    P.bCol.resize(P.nb);
    for (int r = 1; r <= N; ++r) {
        int a = P.originalRank[r];
        tmp.clear();
        tmp.push_back(r - 1);
        for (int q = P.adjPtr[a]; q < P.adjPtr[a + 1]; ++q) tmp.push_back(P.currentRank[P.adj[q]] - 1);
        std::sort(tmp.begin(), tmp.end());
        std::copy(tmp.begin(), tmp.end(), P.bCol.begin() + P.bRowPtr[r - 1]);
    }
    auto blockIndex = [&](int ra0, int rb0) {  // 0-based ranks
        auto b0 = P.bCol.begin() + P.bRowPtr[ra0], b1 = P.bCol.begin() + P.bRowPtr[ra0 + 1];
        auto it = std::lower_bound(b0, b1, rb0);
        return (int)(it - P.bCol.begin());
    };
    // element -> block map
    P.elBlk.resize((size_t)E * npe * npe);
    for (int e = 0; e < E; ++e)
        for (int i = 0; i < npe; ++i)
            for (int j = 0; j < npe; ++j)
                P.elBlk[(size_t)e * npe * npe + i * npe + j] =
                    blockIndex(P.currentRank[EL(e, i)] - 1, P.currentRank[EL(e, j)] - 1);
    // greedy colouring
    {
        std::vector<uint64_t> mask(N + 1, 0);
        std::vector<int> col(E, 0);
        int maxc = 0;
        for (int e = 0; e < E; ++e) {
            uint64_t f = 0;
            for (int i = 0; i < npe; ++i) f |= mask[EL(e, i)];
            if (~f == 0) return set_err(c, ASTRO_ERR_UNSUPPORTED, "element colouring needs more than 64 colours");
            int k = __builtin_ctzll(~f);
            col[e] = k;
            maxc = std::max(maxc, k + 1);
            for (int i = 0; i < npe; ++i) mask[EL(e, i)] |= (1ull << k);
        }
        P.ncolors = maxc;
        P.colorPtr.assign(maxc + 1, 0);
        for (int e = 0; e < E; ++e) P.colorPtr[col[e] + 1]++;
        for (int k = 0; k < maxc; ++k) P.colorPtr[k + 1] += P.colorPtr[k];
        P.colorEls.resize(E);
        std::vector<int> fill(P.colorPtr.begin(), P.colorPtr.end() - 1);
        for (int e = 0; e < E; ++e) P.colorEls[fill[col[e]]++] = e;
        // first-touch flags in colour order (lets an assembly pass write without zeroing first)
        P.elFirst.assign(E, 0ull);
        std::vector<char> seen(P.nb, 0);
        for (int q = 0; q < E; ++q) {
            const int e = P.colorEls[q];
            for (int ab = 0; ab < npe * npe; ++ab) {
                const int k = P.elBlk[(size_t)e * npe * npe + ab];
                if (!seen[k]) {
                    seen[k] = 1;
                    P.elFirst[e] |= (1ull << ab);
                }
            }
        }
    }
    // reference CSR positions: per node, the first-insertion sequence of (component, node)
    {
        std::vector<int> elPtr(N + 2, 0), elOf;
        for (int e = 0; e < E; ++e)
            for (int i = 0; i < npe; ++i) elPtr[EL(e, i) + 1]++;
        for (int a = 1; a <= N + 1; ++a) elPtr[a] += elPtr[a - 1];
        elOf.resize(elPtr[N + 1]);
        std::vector<int> f(elPtr.begin(), elPtr.end());
        for (int e = 0; e < E; ++e)
            for (int i = 0; i < npe; ++i) elOf[f[EL(e, i)]++] = e;  // ascending e per node
        P.csrPosInRow.assign((size_t)P.nb * dpn, -1);
        std::vector<int> stamp((size_t)(N + 1) * dpn, -1);
        std::vector<int> posOf((size_t)(N + 1) * dpn, 0);
        for (int a = 1; a <= N; ++a) {
            int pos = 0;
            for (int q = elPtr[a]; q < elPtr[a + 1]; ++q) {
                int e = elOf[q];
                for (int cc = 0; cc < dpn; ++cc)
                    for (int j = 0; j < npe; ++j) {
                        int b = EL(e, j);
                        size_t key = (size_t)b * dpn + cc;
                        if (stamp[key] != a) {
                            stamp[key] = a;
                            posOf[key] = pos++;
                        }
                    }
            }
            int ra0 = P.currentRank[a] - 1;
            for (int k = P.bRowPtr[ra0]; k < P.bRowPtr[ra0 + 1]; ++k) {
                int b = P.originalRank[P.bCol[k] + 1];
                for (int cc = 0; cc < dpn; ++cc) P.csrPosInRow[(size_t)k * dpn + cc] = posOf[(size_t)b * dpn + cc];
            }
        }
    }
    // constraints
    P.mpcDim = m->num_mpc;
    P.mpcRange.assign(P.mpcDim + 1, 0);
    for (int k = 0; k <= P.mpcDim && P.mpcDim > 0; ++k) P.mpcRange[k] = m->mpc_range[k];
    P.mpcSize = P.mpcRange[P.mpcDim];
    P.mpcCols.assign(P.mpcSize, 0);
    P.mpcMat.assign(P.mpcSize, 0.0);
    P.mpcRhs.assign(P.mpcDim, 0.0);
    for (int r = 0; r < P.mpcDim; ++r) {
        for (int t = P.mpcRange[r]; t < P.mpcRange[r + 1]; ++t) {
            int nd = m->mpc_node[t], dof = m->mpc_dof[t];
            if (nd < 1 || nd > N || dof < 1 || dof > 6) return set_err(c, ASTRO_ERR_ARG, "constraint term out of range");
            int col = P.nDofIndex[6 * (nd - 1) + dof - 1];
            for (int s = P.mpcRange[r]; s < P.mpcRange[r + 1]; ++s) {
                if (P.mpcCols[s] == 0) {
                    P.mpcCols[s] = col;
                    P.mpcMat[s] = m->mpc_coef[t];
                    break;
                }
                if (P.mpcCols[s] == col) break;
            }
        }
        P.mpcRhs[r] = m->mpc_rhs[r];
    }
    return ASTRO_OK;
}
