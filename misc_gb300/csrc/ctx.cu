// C-ABI entry points (include/astro_gpu.h): context life cycle, model upload, and the
// reference-facing calls (getElasticSolnLoad, scaleElasticMPC, getElasticConstraintLoad, the
// surface load, the static solve).  Host arrays use the reference's numbering; device arrays
// use the rank-major layout described in astro_internal.h.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>

#include "astro_internal.h"

static std::mutex g_err_mu;
static std::string g_create_err;

int set_err(astro_ctx *c, int code, const std::string &msg) {
    if (c) c->err = msg;
    else {
        std::lock_guard<std::mutex> g(g_err_mu);
        g_create_err = msg;
    }
    return code;
}

// Checked build: the site of the first index guard that failed since the last call (bounds.cuh),
// as ASTRO_ERR_BOUNDS; the word is cleared for the next launch.
int guard_status(astro_ctx *c, const char *what) {
    int site = 0;
    cudaError_t e = cudaMemcpyAsync(&site, c->d_guard.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_check(c, e, what);
    if (!site) return ASTRO_OK;
    cudaMemsetAsync(c->d_guard.p, 0, sizeof(int), c->stream);
    return set_err(c, ASTRO_ERR_BOUNDS, std::string(what) + ": index guard " + std::to_string(site) + " failed");
}

int cuda_check(astro_ctx *c, cudaError_t e, const char *what) {
    if (e == cudaSuccess) return ASTRO_OK;
    return set_err(c, e == cudaErrorMemoryAllocation ? ASTRO_ERR_NOMEM : ASTRO_ERR_CUDA,
                   std::string(what) + ": " + cudaGetErrorString(e));
}

int dev_alloc(astro_ctx *c, DevBuf &b, size_t bytes) {
    dev_free(b);
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMalloc(&b.p, bytes);
    if (e != cudaSuccess) {
        b.p = nullptr;
        return cuda_check(c, e, "cudaMalloc");
    }
    b.bytes = bytes;
    return ASTRO_OK;
}

void dev_free(DevBuf &b) {
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.bytes = 0;
}

int upload(astro_ctx *c, DevBuf &b, const void *h, size_t bytes) {
    int rc = dev_alloc(c, b, bytes);
    if (rc) return rc;
    if (bytes) {
        // on the context's (non-blocking) stream, then waited for: a copy on the legacy stream is
        // not ordered before the kernels that read it
        cudaError_t e = cudaMemcpyAsync(b.p, h, bytes, cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) return cuda_check(c, e, "upload");
    }
    return ASTRO_OK;
}

static void free_all(astro_ctx *c) {
    host_stage_release(c);
    krylov_release(c);
    panels_release(c);
    thermal_release(c);
    if (c->asmExec) cudaGraphExecDestroy(c->asmExec);
    if (c->asmGraph) cudaGraphDestroy(c->asmGraph);
    c->asmExec = nullptr;
    c->asmGraph = nullptr;
    DevBuf *bufs[] = {&c->d_nodes,  &c->d_elist,   &c->d_elMat,   &c->d_esec,    &c->d_secABD,   &c->d_secOrient,
                      &c->d_colorEls, &c->d_elBlk, &c->d_rank,    &c->d_bRowPtr, &c->d_bCol,     &c->d_bRow,
                      &c->d_etype,  &c->d_elFirst, &c->d_K64p, &c->d_K32p, &c->d_ellCol, &c->d_K64,     &c->d_K32,     &c->d_csrPos,  &c->d_elMatRangeRank,
                      &c->d_intMat, &c->d_mpcRange, &c->d_mpcCol, &c->d_mpcVal,  &c->d_mpcRhs, &c->d_mpcT, &c->d_mpcGPtr, &c->d_mpcGTerm, &c->d_mpcGRow, &c->d_mpcTermRow, &c->d_penRow,
                      &c->d_penPtr, &c->d_penCol,  &c->d_penVal,  &c->d_ltRange, &c->d_lt,       &c->d_scratch,
                      &c->d_status, &c->d_shLayRange, &c->d_shLay, &c->d_shZoff, &c->d_e2dR, &c->d_e2d,
                      &c->d_e2c, &c->d_dCat, &c->d_dLayer, &c->d_dVal, &c->d_elC, &c->d_elXdf, &c->d_elCdf, &c->d_ioRef,
                      &c->d_ioInt, &c->d_exMat, &c->d_exCols, &c->d_shFr, &c->d_shGp, &c->d_shDe, &c->d_shKf,
                      &c->d_guard, &c->d_c8Els, &c->d_c81Els, &c->d_intVecOff, &c->d_intMatOff, &c->d_elRho,
                      &c->d_secOrig, &c->d_n2dR, &c->d_n2d, &c->d_n2c, &c->d_dComp};
    for (DevBuf *b : bufs) dev_free(*b);
    for (DevBuf &b : c->d_sky) dev_free(b);
}

// internal (rank-major) index of reference DOF d (1-based)
static inline int ref2int(const AstroPrep &P, int d) {
    const int c = (d - 1) / P.N, r = (d - 1) % P.N;
    return r * P.dpn + c;
}

extern "C" int astro_last_error(const astro_ctx *ctx, char *buf, int32_t len) {
    if (!buf || len <= 0) return ASTRO_ERR_ARG;
    std::string s;
    if (ctx) s = ctx->err;
    else {
        std::lock_guard<std::mutex> g(g_err_mu);
        s = g_create_err;
    }
    std::strncpy(buf, s.c_str(), (size_t)len - 1);
    buf[len - 1] = 0;
    return ASTRO_OK;
}

extern "C" int astro_ctx_create(const astro_model *m, astro_ctx **out) {
    if (!m || !out) return set_err(nullptr, ASTRO_ERR_ARG, "null argument");
    *out = nullptr;
    if (m->num_nodes <= 0 || m->num_els <= 0 || !m->node_list || !m->element_list || !m->element_type ||
        !m->element_section)
        return set_err(nullptr, ASTRO_ERR_ARG, "model has no nodes/elements");
    int ndev = 0;
    cudaError_t ce = cudaGetDeviceCount(&ndev);
    if (ce != cudaSuccess || ndev == 0)
        return set_err(nullptr, ASTRO_ERR_CUDA, std::string("no CUDA device: ") + cudaGetErrorString(ce));
    astro_ctx *ctx = new astro_ctx();
    int rc = astro_prep_build(ctx, m);
    if (rc) {
        set_err(nullptr, rc, ctx->err);
        delete ctx;
        return rc;
    }
    AstroPrep &P = ctx->P;
    cudaGetDevice(&ctx->device);
    if ((ce = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking)) != cudaSuccess) {
        set_err(nullptr, ASTRO_ERR_CUDA, std::string("stream: ") + cudaGetErrorString(ce));
        delete ctx;
        return ASTRO_ERR_CUDA;
    }
    // host model copies
    ctx->nodes.assign(m->node_list, m->node_list + 3 * (size_t)P.N);
    ctx->elist.assign(m->element_list, m->element_list + 8 * (size_t)P.E);
    ctx->etype.assign(m->element_type, m->element_type + P.E);
    ctx->esec.assign(m->element_section, m->element_section + P.E);
    const int S = m->num_sections;
    ctx->secOrient.assign(9 * (size_t)std::max(S, 1), 0.0);
    for (int s = 0; s < S; ++s)
        for (int k = 0; k < 9; ++k) ctx->secOrient[9 * s + k] = m->section_orient[9 * s + k];
    auto fail = [&](int code, const std::string &msg) {
        set_err(nullptr, code, msg);
        free_all(ctx);
        if (ctx->stream) cudaStreamDestroy(ctx->stream);
        if (ctx->stream2) cudaStreamDestroy(ctx->stream2);
        delete ctx;
        return code;
    };
    for (int e = 0; e < P.E; ++e) {
        int s = ctx->esec[e];
        if (s < 1 || s > S) return fail(ASTRO_ERR_ARG, "element_section out of range");
    }
    if (m->num_dvars > 0) {
        if (!m->el_to_d_range || !m->el_to_d || !m->el_to_coef || !m->d_category || !m->d_value)
            return fail(ASTRO_ERR_ARG, "design variables without their element maps");
        for (int d = 0; d < m->num_dvars; ++d) {
            const int cat = m->d_category[d];
            if (cat < ASTRO_DCAT_LAYUP_THICKNESS || cat > ASTRO_DCAT_LAYUP_MODULUS)
                return fail(ASTRO_ERR_UNSUPPORTED, "design-variable category not supported");
            const int comp = m->d_component ? m->d_component[d] : 0;
            const int maxComp = cat == ASTRO_DCAT_ELASTIC_MODULUS ? 9
                                : cat == ASTRO_DCAT_NODE_LOAD ? 7
                                : (cat == ASTRO_DCAT_THERMAL_COND || cat == ASTRO_DCAT_LAYUP_THERMAL_COND) ? 6
                                : cat == ASTRO_DCAT_LAYUP_MODULUS                                          ? 4
                                                                                                          : 3;
            if ((cat == ASTRO_DCAT_ELASTIC_MODULUS || cat == ASTRO_DCAT_ORIENTATION || cat == ASTRO_DCAT_NODE_COORD ||
                 cat == ASTRO_DCAT_NODE_LOAD || cat == ASTRO_DCAT_THERMAL_COND || cat == ASTRO_DCAT_LAYUP_THERMAL_COND ||
                 cat == ASTRO_DCAT_LAYUP_MODULUS) &&
                (comp < 1 || comp > maxComp))
                return fail(ASTRO_ERR_ARG, "design variable " + std::to_string(d + 1) + " needs d_component in 1.." +
                                               std::to_string(maxComp));
            if ((cat == ASTRO_DCAT_LAYUP_THICKNESS || cat == ASTRO_DCAT_LAYUP_ANGLE || cat == ASTRO_DCAT_LAYUP_DENSITY ||
                 cat == ASTRO_DCAT_LAYUP_THERMAL_COND || cat == ASTRO_DCAT_LAYUP_SPEC_HEAT ||
                 cat == ASTRO_DCAT_LAYUP_MODULUS) &&
                (!m->d_layer || m->d_layer[d] < 1))
                return fail(ASTRO_ERR_ARG, "layer design variable needs d_layer >= 1");
        }
        const int nE2D = m->el_to_d_range[P.E];
        for (int q = 0; q < nE2D; ++q)
            if (m->el_to_d[q] < 1 || m->el_to_d[q] > m->num_dvars) return fail(ASTRO_ERR_ARG, "el_to_d out of range");
        if (m->nd_to_d_range) {
            if (!m->nd_to_d || !m->nd_to_coef) return fail(ASTRO_ERR_ARG, "nd_to_d_range without nd_to_d / nd_to_coef");
            const int nN2D = m->nd_to_d_range[P.N];
            for (int q = 0; q < nN2D; ++q)
                if (m->nd_to_d[q] < 1 || m->nd_to_d[q] > m->num_dvars) return fail(ASTRO_ERR_ARG, "nd_to_d out of range");
            ctx->n2dRange.assign(m->nd_to_d_range, m->nd_to_d_range + P.N + 1);
            ctx->n2d.assign(m->nd_to_d, m->nd_to_d + nN2D);
            ctx->n2c.assign(m->nd_to_coef, m->nd_to_coef + nN2D);
            // r_getNodeCoord: the real values of the nodeCoord variables move the nodes of every
            // element (the complex step adds its own imaginary part)
            for (int nd = 1; nd <= P.N; ++nd)
                for (int q = ctx->n2dRange[nd - 1]; q < ctx->n2dRange[nd]; ++q) {
                    const int d = ctx->n2d[q];
                    if (m->d_category[d - 1] == ASTRO_DCAT_NODE_COORD)
                        ctx->nodes[3 * (size_t)(nd - 1) + m->d_component[d - 1] - 1] += ctx->n2c[q] * m->d_value[d - 1];
                }
        }
        if (m->d_act_time) ctx->dActTime.assign(m->d_act_time, m->d_act_time + 2 * (size_t)m->num_dvars);
        ctx->numDvars = m->num_dvars;
        ctx->e2dRange.assign(m->el_to_d_range, m->el_to_d_range + P.E + 1);
        ctx->e2d.assign(m->el_to_d, m->el_to_d + nE2D);
        ctx->e2c.assign(m->el_to_coef, m->el_to_coef + nE2D);
        ctx->dCat.assign(m->d_category, m->d_category + m->num_dvars);
        ctx->dVal.assign(m->d_value, m->d_value + m->num_dvars);
        ctx->dComp.assign(m->num_dvars, 0);
        ctx->dLayer.assign(m->num_dvars, 0);
        if (m->d_component) ctx->dComp.assign(m->d_component, m->d_component + m->num_dvars);
        if (m->d_layer) ctx->dLayer.assign(m->d_layer, m->d_layer + m->num_dvars);
    }
    if (ctx->hasSolid) {
        ctx->elMat.resize(9 * (size_t)P.E);
        ctx->elDensity.assign((size_t)P.E, 0.0);
        ctx->elMatId.assign((size_t)P.E, 0);
        std::vector<double> orientEl(9 * (size_t)P.E);
        for (int e = 0; e < P.E; ++e) {
            int s = ctx->esec[e];
            int mat = m->section_mat_id[s - 1];
            if (mat < 1 || mat > m->num_materials) return fail(ASTRO_ERR_ARG, "section material out of range");
            for (int k = 0; k < 9; ++k) ctx->elMat[9 * (size_t)e + k] = m->material_elastic[9 * (size_t)(mat - 1) + k];
            if (m->material_density) ctx->elDensity[e] = m->material_density[mat - 1];
            ctx->elMatId[e] = mat;
            // elastic-modulus design variables: eProps(c) += coef * d (r_getMaterialStiffness);
            // density variables: den += coef * d (r_getMaterialDensity); orientation variables
            // rotate the element's frame (applied on the device below)
            if (m->num_dvars > 0)
                for (int q = m->el_to_d_range[e]; q < m->el_to_d_range[e + 1]; ++q) {
                    const int d = m->el_to_d[q];
                    if (m->d_category[d - 1] == ASTRO_DCAT_ELASTIC_MODULUS) {
                        double &v = ctx->elMat[9 * (size_t)e + m->d_component[d - 1] - 1];
                        v = v + m->el_to_coef[q] * m->d_value[d - 1];
                    } else if (m->d_category[d - 1] == ASTRO_DCAT_DENSITY) {
                        ctx->elDensity[e] += m->el_to_coef[q] * m->d_value[d - 1];
                    } else if (m->d_category[d - 1] == ASTRO_DCAT_ORIENTATION) {
                        ctx->orientIdentity = 0;
                    }
                }
            for (int k = 0; k < 9; ++k) {
                double v = ctx->secOrient[9 * (s - 1) + k];
                orientEl[9 * (size_t)e + k] = v;
                if (v != ((k % 4 == 0) ? 1.0 : 0.0)) ctx->orientIdentity = 0;
            }
        }
        if ((rc = upload(ctx, ctx->d_elMat, ctx->elMat.data(), sizeof(double) * ctx->elMat.size())))
            return fail(rc, ctx->err);
        if ((rc = upload(ctx, ctx->d_secOrient, orientEl.data(), sizeof(double) * orientEl.size())))
            return fail(rc, ctx->err);
    }
    // device structures
    std::vector<int> rank1(P.N), bRow(P.nb), colorEls(P.colorEls);
    for (int a = 1; a <= P.N; ++a) rank1[a - 1] = P.currentRank[a];
    for (int r = 0; r < P.N; ++r)
        for (int k = P.bRowPtr[r]; k < P.bRowPtr[r + 1]; ++k) bRow[k] = r;
#define UP(buf, vec)                                                                          \
    if ((rc = upload(ctx, ctx->buf, (vec).data(), sizeof((vec)[0]) * (vec).size()))) return fail(rc, ctx->err);
    UP(d_nodes, ctx->nodes);
    UP(d_elist, ctx->elist);
    UP(d_etype, ctx->etype);
    UP(d_esec, ctx->esec);
    UP(d_rank, rank1);
    UP(d_bRowPtr, P.bRowPtr);
    UP(d_bCol, P.bCol);
    UP(d_bRow, bRow);
    UP(d_colorEls, colorEls);
    UP(d_elBlk, P.elBlk);
    UP(d_elFirst, P.elFirst);
    UP(d_csrPos, P.csrPosInRow);
    UP(d_elMatRangeRank, P.elMatRange);
#undef UP
    if ((rc = dev_alloc(ctx, ctx->d_status, 256))) return fail(rc, ctx->err);
    cudaMemset(ctx->d_status.p, 0, 256);
    if ((rc = dev_alloc(ctx, ctx->d_guard, sizeof(int)))) return fail(rc, ctx->err);
    cudaMemset(ctx->d_guard.p, 0, sizeof(int));
    // section orientations as given, and the design-variable maps (the complex step's inputs)
    if ((rc = upload(ctx, ctx->d_secOrig, ctx->secOrient.data(), sizeof(double) * ctx->secOrient.size())))
        return fail(rc, ctx->err);
    if (ctx->numDvars > 0) {
        std::vector<int> e2d(ctx->e2d), n2d(ctx->n2d), n2r(ctx->n2dRange);
        std::vector<double> e2c(ctx->e2c), n2c(ctx->n2c);
        if (e2d.empty()) e2d.push_back(0), e2c.push_back(0.0);
        if (n2d.empty()) n2d.push_back(0), n2c.push_back(0.0);
        if (n2r.empty()) n2r.assign((size_t)P.N + 1, 0);
        if ((rc = upload(ctx, ctx->d_e2dR, ctx->e2dRange.data(), sizeof(int) * ctx->e2dRange.size())) ||
            (rc = upload(ctx, ctx->d_e2d, e2d.data(), sizeof(int) * e2d.size())) ||
            (rc = upload(ctx, ctx->d_e2c, e2c.data(), sizeof(double) * e2c.size())) ||
            (rc = upload(ctx, ctx->d_n2dR, n2r.data(), sizeof(int) * n2r.size())) ||
            (rc = upload(ctx, ctx->d_n2d, n2d.data(), sizeof(int) * n2d.size())) ||
            (rc = upload(ctx, ctx->d_n2c, n2c.data(), sizeof(double) * n2c.size())) ||
            (rc = upload(ctx, ctx->d_dCat, ctx->dCat.data(), sizeof(int) * ctx->dCat.size())) ||
            (rc = upload(ctx, ctx->d_dComp, ctx->dComp.data(), sizeof(int) * ctx->dComp.size())) ||
            (rc = upload(ctx, ctx->d_dLayer, ctx->dLayer.data(), sizeof(int) * ctx->dLayer.size())) ||
            (rc = upload(ctx, ctx->d_dVal, ctx->dVal.data(), sizeof(double) * ctx->dVal.size())))
            return fail(rc, ctx->err);
    }
    if (ctx->hasShell && (rc = shell_sections_prepare(ctx, m))) return fail(rc, ctx->err);
    if (ctx->hasSolid) {
        // colour-grouped element lists by type (brick8 / brickIM), internal-DOF offsets, density
        ctx->c8Ptr.assign(1, 0);
        ctx->c81Ptr.assign(1, 0);
        for (int col = 0; col < P.ncolors; ++col) {
            for (int k = P.colorPtr[col]; k < P.colorPtr[col + 1]; ++k) {
                const int e = P.colorEls[k];
                (ctx->etype[e] == 81 ? ctx->c81Els : ctx->c8Els).push_back(e);
            }
            ctx->c8Ptr.push_back((int)ctx->c8Els.size());
            ctx->c81Ptr.push_back((int)ctx->c81Els.size());
        }
        ctx->has81 = !ctx->c81Els.empty();
        std::vector<int> c8(ctx->c8Els), c81(ctx->c81Els);
        if (c8.empty()) c8.push_back(0);
        if (c81.empty()) c81.push_back(0);
        if ((rc = upload(ctx, ctx->d_c8Els, c8.data(), sizeof(int) * c8.size())) ||
            (rc = upload(ctx, ctx->d_c81Els, c81.data(), sizeof(int) * c81.size())) ||
            (rc = upload(ctx, ctx->d_intVecOff, P.intVecRange.data(), sizeof(int) * P.intVecRange.size())) ||
            (rc = upload(ctx, ctx->d_intMatOff, P.intMatRange.data(), sizeof(int) * P.intMatRange.size())) ||
            (rc = upload(ctx, ctx->d_elRho, ctx->elDensity.data(), sizeof(double) * ctx->elDensity.size())))
            return fail(rc, ctx->err);
        if (P.intMatSize && (rc = dev_alloc(ctx, ctx->d_intMat, sizeof(double) * (size_t)P.intMatSize)))
            return fail(rc, ctx->err);
        if (!ctx->orientIdentity && ctx->numDvars > 0 && (rc = solid_orient_prepare(ctx))) return fail(rc, ctx->err);
        if ((rc = hex8_prepare(ctx))) return fail(rc, ctx->err);
    }
    // unscaled constraints in internal numbering
    ctx->mpcScaledHost = P.mpcMat;
    ctx->mpcRhsScaledHost = P.mpcRhs;
    *out = ctx;
    return ASTRO_OK;
}

extern "C" int astro_ctx_destroy(astro_ctx *ctx) {
    if (!ctx) return ASTRO_OK;
    cudaStreamSynchronize(ctx->stream);
    free_all(ctx);
    cudaStreamDestroy(ctx->stream);
    if (ctx->stream2) {
        cudaStreamSynchronize(ctx->stream2);
        cudaStreamDestroy(ctx->stream2);
    }
    delete ctx;
    return ASTRO_OK;
}

extern "C" int astro_get_dims(const astro_ctx *ctx, astro_dims *o) {
    if (!ctx || !o) return ASTRO_ERR_ARG;
    const AstroPrep &P = ctx->P;
    o->el_mat_dim = P.n;
    o->el_mat_size = P.elMatSize;
    o->el_mat_lt_size = P.ltSize;
    o->el_mpc_dim = P.mpcDim;
    o->el_mpc_size = P.mpcSize;
    o->int_vec_size = P.intVecSize;
    o->int_mat_size = P.intMatSize;
    o->solver_max_bw = P.solverMaxBW;
    o->dof_per_node = P.dpn;
    o->num_blocks = P.nb;
    o->num_colors = P.ncolors;
    return ASTRO_OK;
}

extern "C" void *astro_ctx_stream(const astro_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

extern "C" int astro_get_prep(const astro_ctx *ctx, int32_t *current_rank, int32_t *n_dof_index, int32_t *el_mat_range,
                              int32_t *el_mat_lt_range, int32_t *mpc_range, int32_t *mpc_cols, double *mpc_mat,
                              double *mpc_rhs) {
    if (!ctx) return ASTRO_ERR_ARG;
    const AstroPrep &P = ctx->P;
    if (current_rank) std::copy(P.currentRank.begin() + 1, P.currentRank.end(), current_rank);
    if (n_dof_index) std::copy(P.nDofIndex.begin(), P.nDofIndex.end(), n_dof_index);
    if (el_mat_range) std::copy(P.elMatRange.begin(), P.elMatRange.end(), el_mat_range);
    if (el_mat_lt_range) std::copy(P.elMatLTRange.begin(), P.elMatLTRange.end(), el_mat_lt_range);
    if (mpc_range) std::copy(P.mpcRange.begin(), P.mpcRange.end(), mpc_range);
    if (mpc_cols) std::copy(P.mpcCols.begin(), P.mpcCols.end(), mpc_cols);
    if (mpc_mat) std::copy(P.mpcMat.begin(), P.mpcMat.end(), mpc_mat);
    if (mpc_rhs) std::copy(P.mpcRhs.begin(), P.mpcRhs.end(), mpc_rhs);
    return ASTRO_OK;
}

int ensure_K(astro_ctx *ctx, int which) {
    const size_t nv = (size_t)ctx->P.nb * ctx->P.dpn * ctx->P.dpn;
    int rc;
    if ((which & 2) && !ctx->d_K64.p && (rc = dev_alloc(ctx, ctx->d_K64, nv * sizeof(double)))) return rc;
    if ((which & 1) && !ctx->d_K32.p && (rc = dev_alloc(ctx, ctx->d_K32, nv * sizeof(float)))) return rc;
    return ASTRO_OK;
}

// state vectors (reference numbering, host) -> internal layout on the device
struct DevState {
    DevBuf disp, vel, acc, pdisp, pvel, pacc, idisp, pidisp;
    ~DevState() {
        DevBuf *b[] = {&disp, &vel, &acc, &pdisp, &pvel, &pacc, &idisp, &pidisp};
        for (auto *x : b) dev_free(*x);
    }
};

// A state vector that is all zero stays null on the device: every kernel reads a null state
// vector as zeros, and the brick kernels take the zero-state path.
static int state_vec_up(astro_ctx *ctx, const double *h, DevBuf &dst, bool zero_is_null = true) {
    if (!h) return ASTRO_OK;
    const int n = ctx->P.n;
    if (zero_is_null) {
        bool nz = false;
        for (int i = 0; i < n && !nz; ++i) nz = h[i] != 0.0;
        if (!nz) return ASTRO_OK;
    }
    DevBuf tmp;
    int rc = upload(ctx, tmp, h, sizeof(double) * n);
    if (!rc) rc = dev_alloc(ctx, dst, sizeof(double) * n);
    if (!rc) rc = ref_to_int_vec(ctx, dptr<double>(tmp), dptr<double>(dst), n);
    if (!rc) rc = cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "state upload");
    dev_free(tmp);
    return rc;
}

// Element evaluation state on the device: nodal vectors converted to the internal layout (in S),
// internal-DOF vectors uploaded as they are (intVecRange order).
static int elem_state(astro_ctx *ctx, const astro_state *state, DevState &S, ElemDevState &ds) {
    int rc;
    if (!state) return ASTRO_OK;
    const size_t ni = (size_t)ctx->P.intVecSize;
    if (state->internal_disp && (rc = upload(ctx, S.idisp, state->internal_disp, sizeof(double) * ni))) return rc;
    if (state->prev_int_disp && (rc = upload(ctx, S.pidisp, state->prev_int_disp, sizeof(double) * ni))) return rc;
    ds.disp = S.disp.p ? dptr<double>(S.disp) : nullptr;
    ds.pdisp = S.pdisp.p ? dptr<double>(S.pdisp) : nullptr;
    ds.pvel = S.pvel.p ? dptr<double>(S.pvel) : nullptr;
    ds.pacc = S.pacc.p ? dptr<double>(S.pacc) : nullptr;
    ds.idisp = S.idisp.p ? dptr<double>(S.idisp) : nullptr;
    ds.pidisp = S.pidisp.p ? dptr<double>(S.pidisp) : nullptr;
    ds.dynamic = state->dynamic;
    ds.beta = state->nm_beta;
    ds.gamma = state->nm_gamma;
    ds.delT = state->del_t;
    if (ds.dynamic && !(ds.delT > 0.0 && ds.beta > 0.0))
        return set_err(ctx, ASTRO_ERR_ARG, "dynamic evaluation needs del_t > 0 and nm_beta > 0");
    return ASTRO_OK;
}

// Persistent device buffers of the getElasticSolnLoad boundary, allocated on first use.
int ensure_io(astro_ctx *ctx, bool exportMat) {
    const AstroPrep &P = ctx->P;
    int rc;
    if (!ctx->d_ioRef.p && (rc = dev_alloc(ctx, ctx->d_ioRef, sizeof(double) * P.n))) return rc;
    if (!ctx->d_ioInt.p && (rc = dev_alloc(ctx, ctx->d_ioInt, sizeof(double) * P.n))) return rc;
    if (exportMat) {
        if (!ctx->d_exMat.p && (rc = dev_alloc(ctx, ctx->d_exMat, sizeof(double) * (size_t)P.elMatSize))) return rc;
        if (!ctx->d_exCols.p && (rc = dev_alloc(ctx, ctx->d_exCols, sizeof(int) * (size_t)P.elMatSize))) return rc;
    }
    if (!ctx->stream2) CK(cudaStreamCreateWithFlags(&ctx->stream2, cudaStreamNonBlocking));
    return ASTRO_OK;
}

// getElasticSolnLoad (Working/AStrO_commandFunctions.f90:260-351).  The reference CSR column
// numbers depend on the mesh only, so they are formed on a second stream and copied to the host
// while the element kernels run; the values follow the last colour.
extern "C" int astro_el_soln_load(astro_ctx *ctx, int32_t build_mat, const astro_state *state, double *elastic_load,
                                  double *int_elastic_load, double *elastic_mat, int32_t *el_mat_cols,
                                  double *int_elastic_mat) {
    if (!ctx || !elastic_load) return ASTRO_ERR_ARG;
    const AstroPrep &P = ctx->P;
    const int n = P.n;
    const bool exportMat = build_mat == 1 && (elastic_mat || el_mat_cols);
    int rc;
    if ((rc = ensure_io(ctx, exportMat))) return rc;
    DevState S;
    if (state) {
        if ((rc = state_vec_up(ctx, state->node_disp, S.disp))) return rc;
        if (ctx->hasShell || state->dynamic) {
            if ((rc = state_vec_up(ctx, state->prev_disp, S.pdisp))) return rc;
            if ((rc = state_vec_up(ctx, state->prev_vel, S.pvel))) return rc;
            if ((rc = state_vec_up(ctx, state->prev_acc, S.pacc))) return rc;
        }
    }
    if (exportMat && el_mat_cols && (rc = export_csr_dev(ctx, ctx->stream2, nullptr, dptr<int>(ctx->d_exCols))))
        return rc;
    double *dRef = dptr<double>(ctx->d_ioRef), *dl = dptr<double>(ctx->d_ioInt);
    CK(cudaMemcpyAsync(dRef, elastic_load, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
    if ((rc = ref_to_int_vec(ctx, dRef, dl, n))) return rc;
    if (build_mat == 1) {
        if ((rc = ensure_K(ctx, 2))) return rc;
        // the solid kernels write every block (first touch in colour order), the shell one adds
        if (ctx->hasShell && (rc = bsr_zero(ctx, 2))) return rc;
    }
    {
        DevBuf il;
        if (int_elastic_load && P.intVecSize) {
            if ((rc = upload(ctx, il, int_elastic_load, sizeof(double) * P.intVecSize))) return rc;
        }
        ElemDevState ds;
        if ((rc = elem_state(ctx, state, S, ds))) return rc;
        if (ctx->hasSolid)
            rc = solid_soln_load(ctx, build_mat == 1, ds, dl, il.p ? dptr<double>(il) : nullptr, nullptr, nullptr);
        else
            rc = launch_shell4_assemble(ctx, ds, dl, il.p ? dptr<double>(il) : nullptr, build_mat == 1, nullptr,
                                        nullptr);
        if (!rc && il.p) {
            cudaError_t e = cudaMemcpyAsync(int_elastic_load, il.p, sizeof(double) * P.intVecSize,
                                            cudaMemcpyDeviceToHost, ctx->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
            rc = cuda_check(ctx, e, "int load download");
        }
        dev_free(il);
    }
    if (rc) {
        cudaStreamSynchronize(ctx->stream2);
        return rc;
    }
    // a copy into pageable host memory returns when it is done, so it is issued after the element
    // kernels have been launched and runs while they execute
    if (exportMat && el_mat_cols)
        CK(cudaMemcpyAsync(el_mat_cols, ctx->d_exCols.p, sizeof(int) * (size_t)P.elMatSize, cudaMemcpyDeviceToHost,
                           ctx->stream2));
    if (build_mat == 1) {
        ctx->haveK64 = 1;
        ctx->k64Version++;
        ctx->haveIntMat = P.intVecSize > 0;
    }
    // load back to reference numbering
    if ((rc = int_to_ref_vec(ctx, dl, dRef, n))) return rc;
    CK(cudaMemcpyAsync(elastic_load, dRef, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    if (exportMat && elastic_mat) {
        if ((rc = export_csr_dev(ctx, ctx->stream, dptr<double>(ctx->d_exMat), nullptr))) return rc;
        CK(cudaMemcpyAsync(elastic_mat, ctx->d_exMat.p, sizeof(double) * (size_t)P.elMatSize, cudaMemcpyDeviceToHost,
                           ctx->stream));
    }
    if (build_mat == 1 && int_elastic_mat && P.intMatSize && ctx->d_intMat.p)
        CK(cudaMemcpyAsync(int_elastic_mat, ctx->d_intMat.p, sizeof(double) * P.intMatSize, cudaMemcpyDeviceToHost,
                           ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream2));
    ctx->mpcScaled = 0;
    ctx->haveLT = 0;
    ctx->ltFactored = 0;
    return ASTRO_OK;
}

int elem_soln_load_dev(astro_ctx *ctx, const ElemDevState &s, double *d_loadInt, double *d_intLoad, int build,
                       bool sync) {
    if (ctx->hasSolid) {
        const int rc = solid_soln_load(ctx, build, s, d_loadInt, d_intLoad, nullptr, nullptr);
        if (rc || !sync) return rc;
        return cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "solid elements");
    }
    if (build) {
        const int rc = bsr_zero(ctx, 2);
        if (rc) return rc;
    }
    return launch_shell4_assemble(ctx, s, d_loadInt, d_intLoad, build, nullptr, nullptr, sync);
}

int elem_update_external_rhs(astro_ctx *ctx, const double *d_intVec, double *d_extInt) {
    if (!ctx->P.intVecSize) return ASTRO_OK;
    return ctx->hasShell ? shell4_update_external_rhs(ctx, d_intVec, d_extInt)
                         : hex81_update_external_rhs(ctx, d_intVec, d_extInt);
}
int elem_update_internal_soln(astro_ctx *ctx, const double *d_extInt, double *d_intSoln, const double *d_intRhs) {
    if (!ctx->P.intVecSize) return ASTRO_OK;
    return ctx->hasShell ? shell4_update_internal_soln(ctx, d_extInt, d_intSoln, d_intRhs)
                         : hex81_update_internal_soln(ctx, d_extInt, d_intSoln, d_intRhs);
}

// updateExternalRHS (Working/AStrO_commandFunctions.f90:568-607) with the loop over the internal
// rows (nodalDof+1 .. totalDof, the evident intent of its empty loop bound): for every element
// with internal DOF (shell4, brickIM) ext_vec(nodal DOF) -= K_ni K_ii^-1 int_vec(its internal DOF).
extern "C" int astro_update_external_rhs(astro_ctx *ctx, double *ext_vec, const double *int_vec) {
    if (!ctx || !ext_vec || !int_vec) return ASTRO_ERR_ARG;
    if (!ctx->P.intVecSize) return ASTRO_OK;  // no internal DOF: nothing to condense
    if (!ctx->haveIntMat) return set_err(ctx, ASTRO_ERR_STATE, "needs the internal rows of astro_el_soln_load(build_mat = 1)");
    const int n = ctx->P.n;
    int rc;
    if ((rc = ensure_io(ctx, false))) return rc;
    DevBuf iv;
    if ((rc = upload(ctx, iv, int_vec, sizeof(double) * ctx->P.intVecSize))) return rc;
    double *dRef = dptr<double>(ctx->d_ioRef), *dInt = dptr<double>(ctx->d_ioInt);
    cudaError_t e = cudaMemcpyAsync(dRef, ext_vec, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess && !(rc = ref_to_int_vec(ctx, dRef, dInt, n)) &&
        !(rc = elem_update_external_rhs(ctx, dptr<double>(iv), dInt)) && !(rc = int_to_ref_vec(ctx, dInt, dRef, n))) {
        e = cudaMemcpyAsync(ext_vec, dRef, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    }
    dev_free(iv);
    if (rc) return rc;
    return cuda_check(ctx, e, "update_external_rhs");
}

// updateInternalSoln (:609-651), loop bound resolved likewise: for every element with internal DOF
// int_soln += K_ii^-1 (int_rhs - K_in ext_soln); int_rhs may be NULL (zeros).
extern "C" int astro_update_internal_soln(astro_ctx *ctx, const double *ext_soln, double *int_soln,
                                          const double *int_rhs) {
    if (!ctx || !ext_soln || !int_soln) return ASTRO_ERR_ARG;
    if (!ctx->P.intVecSize) return ASTRO_OK;
    if (!ctx->haveIntMat) return set_err(ctx, ASTRO_ERR_STATE, "needs the internal rows of astro_el_soln_load(build_mat = 1)");
    const int n = ctx->P.n, ni = ctx->P.intVecSize;
    int rc;
    if ((rc = ensure_io(ctx, false))) return rc;
    DevBuf is, ir;
    if ((rc = upload(ctx, is, int_soln, sizeof(double) * ni))) return rc;
    if (int_rhs && (rc = upload(ctx, ir, int_rhs, sizeof(double) * ni))) {
        dev_free(is);
        return rc;
    }
    double *dRef = dptr<double>(ctx->d_ioRef), *dInt = dptr<double>(ctx->d_ioInt);
    cudaError_t e = cudaMemcpyAsync(dRef, ext_soln, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess && !(rc = ref_to_int_vec(ctx, dRef, dInt, n)) &&
        !(rc = elem_update_internal_soln(ctx, dInt, dptr<double>(is), ir.p ? dptr<double>(ir) : nullptr))) {
        e = cudaMemcpyAsync(int_soln, is.p, sizeof(double) * ni, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    }
    dev_free(is);
    dev_free(ir);
    if (rc) return rc;
    return cuda_check(ctx, e, "update_internal_soln");
}

// The time loop of astro_newmark_run with every history optional (astro_newmark_run_states).
static int newmark_run_impl(astro_ctx *ctx, const astro_newmark_opts *o, const double *load_pattern,
                            const double *load_amplitude, double *disp, double *vel, double *acc, double *int_disp,
                            double *disp_history, double *vel_history, double *acc_history, double *int_disp_history,
                            astro_solve_stats *stats) {
    if (!ctx || !o || !disp || !vel || !acc || o->num_steps < 0 || !(o->del_t > 0.0) || !(o->nm_beta > 0.0) ||
        (load_pattern && !load_amplitude))
        return ASTRO_ERR_ARG;
    const AstroPrep &P = ctx->P;
    const int n = P.n, ni = P.intVecSize;
    int rc;
    struct Bufs {
        DevBuf u, up, vp, ap, iu, iup, pat, hist, vhist, ahist, ihist;
        ~Bufs() {
            DevBuf *b[] = {&u, &up, &vp, &ap, &iu, &iup, &pat, &hist, &vhist, &ahist, &ihist};
            for (auto *x : b) dev_free(*x);
        }
    } B;
    // loadInitialState: the previous state is the initial one, the previous internal DOF zero
    if ((rc = state_vec_up(ctx, disp, B.u, false))) return rc;
    if ((rc = state_vec_up(ctx, vel, B.vp, false))) return rc;
    if ((rc = state_vec_up(ctx, acc, B.ap, false))) return rc;
    if ((rc = dev_alloc(ctx, B.up, sizeof(double) * n))) return rc;
    CK(cudaMemcpyAsync(B.up.p, B.u.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->stream));
    if (ni) {
        if ((rc = dev_alloc(ctx, B.iu, sizeof(double) * ni))) return rc;
        if ((rc = dev_alloc(ctx, B.iup, sizeof(double) * ni))) return rc;
        CK(cudaMemsetAsync(B.iup.p, 0, sizeof(double) * ni, ctx->stream));
        if (int_disp) CK(cudaMemcpyAsync(B.iu.p, int_disp, sizeof(double) * ni, cudaMemcpyHostToDevice, ctx->stream));
        else CK(cudaMemsetAsync(B.iu.p, 0, sizeof(double) * ni, ctx->stream));
    }
    if (load_pattern && (rc = state_vec_up(ctx, load_pattern, B.pat, false))) return rc;
    if (disp_history && o->num_steps > 0 && (rc = dev_alloc(ctx, B.hist, sizeof(double) * n * (size_t)o->num_steps)))
        return rc;
    if (vel_history && o->num_steps > 0 && (rc = dev_alloc(ctx, B.vhist, sizeof(double) * n * (size_t)o->num_steps)))
        return rc;
    if (acc_history && o->num_steps > 0 && (rc = dev_alloc(ctx, B.ahist, sizeof(double) * n * (size_t)o->num_steps)))
        return rc;
    if (int_disp_history && ni && o->num_steps > 0 &&
        (rc = dev_alloc(ctx, B.ihist, sizeof(double) * ni * (size_t)o->num_steps)))
        return rc;
    // K_eff = K + c1 c2 M at the initial state (getElasticSolnLoad(1) with the dynamic flag), then
    // scaleElasticMPC
    ElemDevState ds;
    ds.disp = dptr<double>(B.u);
    ds.pdisp = dptr<double>(B.up);
    ds.pvel = dptr<double>(B.vp);
    ds.pacc = dptr<double>(B.ap);
    ds.idisp = ni ? dptr<double>(B.iu) : nullptr;
    ds.pidisp = ni ? dptr<double>(B.iup) : nullptr;
    ds.dynamic = 1;
    ds.beta = o->nm_beta;
    ds.gamma = o->nm_gamma;
    ds.delT = o->del_t;
    if ((rc = ensure_K(ctx, 2))) return rc;
    if ((rc = elem_soln_load_dev(ctx, ds, nullptr, nullptr, 1, true))) return rc;
    ctx->haveK64 = 1;
    ctx->k64Version++;
    ctx->haveIntMat = ni > 0;
    ctx->haveLT = 0;
    ctx->ltFactored = 0;
    if ((rc = astro_scale_mpc(ctx, nullptr, nullptr))) return rc;
    NewmarkHist H;
    H.disp = B.hist.p ? dptr<double>(B.hist) : nullptr;
    H.vel = B.vhist.p ? dptr<double>(B.vhist) : nullptr;
    H.acc = B.ahist.p ? dptr<double>(B.ahist) : nullptr;
    H.intDisp = B.ihist.p ? dptr<double>(B.ihist) : nullptr;
    rc = krylov_newmark(ctx, o, B.pat.p ? dptr<double>(B.pat) : nullptr, load_amplitude, dptr<double>(B.u),
                        dptr<double>(B.up), dptr<double>(B.vp), dptr<double>(B.ap), ni ? dptr<double>(B.iu) : nullptr,
                        ni ? dptr<double>(B.iup) : nullptr, H, stats);
    if (rc) return rc;
    // final state (after the swap the previous values are the current ones)
    if ((rc = ensure_io(ctx, false))) return rc;
    double *dRef = dptr<double>(ctx->d_ioRef);
    const double *src[3] = {dptr<double>(B.u), dptr<double>(B.vp), dptr<double>(B.ap)};
    double *dst[3] = {disp, vel, acc};
    for (int q = 0; q < 3; ++q) {
        if ((rc = int_to_ref_vec(ctx, src[q], dRef, n))) return rc;
        CK(cudaMemcpyAsync(dst[q], dRef, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
    }
    if (ni && int_disp) CK(cudaMemcpyAsync(int_disp, B.iu.p, sizeof(double) * ni, cudaMemcpyDeviceToHost, ctx->stream));
    const struct {
        DevBuf *d;
        double *h;
        size_t len;
    } outs[4] = {{&B.hist, disp_history, (size_t)n}, {&B.vhist, vel_history, (size_t)n},
                 {&B.ahist, acc_history, (size_t)n}, {&B.ihist, int_disp_history, (size_t)ni}};
    for (const auto &x : outs)
        if (x.d->p)
            CK(cudaMemcpyAsync(x.h, x.d->p, sizeof(double) * x.len * (size_t)o->num_steps, cudaMemcpyDeviceToHost,
                               ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return ASTRO_OK;
}

extern "C" int astro_newmark_run(astro_ctx *ctx, const astro_newmark_opts *o, const double *load_pattern,
                                 const double *load_amplitude, double *disp, double *vel, double *acc, double *int_disp,
                                 double *disp_history, astro_solve_stats *stats) {
    return newmark_run_impl(ctx, o, load_pattern, load_amplitude, disp, vel, acc, int_disp, disp_history, nullptr,
                            nullptr, nullptr, stats);
}

extern "C" int astro_newmark_run_states(astro_ctx *ctx, const astro_newmark_opts *o, const double *load_pattern,
                                        const double *load_amplitude, double *disp, double *vel, double *acc,
                                        double *int_disp, double *disp_history, double *vel_history,
                                        double *acc_history, double *int_disp_history, astro_solve_stats *stats) {
    return newmark_run_impl(ctx, o, load_pattern, load_amplitude, disp, vel, acc, int_disp, disp_history, vel_history,
                            acc_history, int_disp_history, stats);
}

extern "C" int astro_assemble_fp32(astro_ctx *ctx) {
    if (!ctx) return ASTRO_ERR_ARG;
    if (!ctx->hasSolid || ctx->has81)
        return set_err(ctx, ASTRO_ERR_UNSUPPORTED, "FP32 assembly is implemented for brick8 meshes");
    int rc;
    if ((rc = ensure_K(ctx, 1))) return rc;
    // every block is written first by its first-touching element: no zeroing pass
    if ((rc = launch_hex8_assemble(ctx, 32, 1))) return rc;
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->haveK32 = 1;
    ctx->k32Version++;
    return ASTRO_OK;
}

// Timed-path variant used by the benchmark: assembly only, no synchronisation.
extern "C" int astro_assemble_fp32_async(astro_ctx *ctx) {
    if (!ctx || !ctx->d_K32.p) return ASTRO_ERR_STATE;
    ctx->k32Version++;
    if (!ctx->hasSolid || ctx->hasShell) return launch_hex8_assemble(ctx, 32, 1);
    // the colour launches of a pass depend on one another only through the stream order; as a
    // graph they are issued together, without a host launch per colour
    if (!ctx->asmExec) {
        int rc;
        CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
        rc = launch_hex8_assemble(ctx, 32, 1);
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        CK(e);
        e = cudaGraphInstantiate(&ctx->asmExec, g, 0);
        if (e != cudaSuccess) {
            cudaGraphDestroy(g);
            ctx->asmExec = nullptr;
            return cuda_check(ctx, e, "assembly graph");
        }
        ctx->asmGraph = g;
    }
    return cuda_check(ctx, cudaGraphLaunch(ctx->asmExec, ctx->stream), "assembly graph launch");
}

void dvar_elements_by_colour(const astro_ctx *ctx, int dvar, std::vector<int> &list, std::vector<int> &ptr) {
    const AstroPrep &P = ctx->P;
    list.clear();
    ptr.assign(1, 0);
    for (int col = 0; col < P.ncolors; ++col) {
        for (int k = P.colorPtr[col]; k < P.colorPtr[col + 1]; ++k) {
            const int e = P.colorEls[k];
            bool dep = false;
            for (int q = ctx->e2dRange[e]; q < ctx->e2dRange[e + 1]; ++q) dep = dep || ctx->e2d[q] == dvar;
            if (dep) list.push_back(e);
        }
        ptr.push_back((int)list.size());
    }
}

__global__ void k_scale_neg(int n, const double *x, double s, double *y) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = s * -x[i];
}

// getdRelasticdD, element part (Working/AStrO_commandFunctions.f90:1172-1250).  The elements that
// depend on dvar contribute Im(Ru(d + i h)) / h.  Ru is linear in the element's material or
// section stiffness (and section mass) at a real state, so Im(Ru) is the real residual evaluated
// with the imaginary parts of the complex-step properties; the element kernels run in FP64 with
// those properties and the complex path's constants (Gauss points +-0.577350269189626 as a
// single-precision literal), and only the property evaluation is complex.
// Device state of a complex-step evaluation, uploaded once for any number of design variables.
struct DrddState {
    DevState S;
    ElemDevState ds;
};
static int drdd_state(astro_ctx *ctx, const astro_state *state, DrddState &D) {
    int rc;
    if (!state) return ASTRO_OK;
    if ((rc = state_vec_up(ctx, state->node_disp, D.S.disp))) return rc;
    if (ctx->hasShell || state->dynamic) {
        if ((rc = state_vec_up(ctx, state->prev_disp, D.S.pdisp))) return rc;
        if ((rc = state_vec_up(ctx, state->prev_vel, D.S.pvel))) return rc;
        if ((rc = state_vec_up(ctx, state->prev_acc, D.S.pacc))) return rc;
    }
    return elem_state(ctx, state, D.S, D.ds);
}

// dRu/dd of design variable dvar into d_acc (n, internal layout) and d_iacc (internal DOF, may be
// null): the complex step's -sum Im(Ru) scaled by -1/h (getdRelasticdD's compStepInv).
static int drdd_device(astro_ctx *ctx, int dvar, double h, DrddState &D, double *d_acc, double *d_iacc) {
    const int n = ctx->P.n, ni = ctx->P.intVecSize;
    int rc;
    CK(cudaMemsetAsync(d_acc, 0, sizeof(double) * n, ctx->stream));
    if (ni > 0 && d_iacc) CK(cudaMemsetAsync(d_iacc, 0, sizeof(double) * ni, ctx->stream));
    if (ctx->hasSolid) {
        rc = solid_drdd(ctx, dvar, h, D.ds, d_acc, ni > 0 ? d_iacc : nullptr);
    } else {
        rc = shell4_drdd(ctx, dvar, h, D.ds, d_acc, ni > 0 ? d_iacc : nullptr);
    }
    if (rc) return rc;
    const double hInv = 1.0 / h;
    k_scale_neg<<<(n + 255) / 256, 256, 0, ctx->stream>>>(n, d_acc, hInv, d_acc);
    if (ni > 0 && d_iacc) k_scale_neg<<<(ni + 255) / 256, 256, 0, ctx->stream>>>(ni, d_iacc, hInv, d_iacc);
    return cuda_check(ctx, cudaGetLastError(), "drdd");
}

extern "C" int astro_drdd_complex(astro_ctx *ctx, int32_t dvar, double h, const astro_state *state, double *drudd,
                                  double *int_drudd) {
    if (!ctx || !drudd) return ASTRO_ERR_ARG;
    if (dvar < 1 || dvar > ctx->numDvars)
        return set_err(ctx, ASTRO_ERR_ARG, "design variable " + std::to_string(dvar) + " out of range");
    if (!(h > 0.0)) return set_err(ctx, ASTRO_ERR_ARG, "complex step h must be positive");
    const AstroPrep &P = ctx->P;
    const int n = P.n;
    int rc;
    DrddState D;
    if ((rc = drdd_state(ctx, state, D))) return rc;
    struct Tmp {
        DevBuf acc, iacc, out;
        ~Tmp() {
            dev_free(acc);
            dev_free(iacc);
            dev_free(out);
        }
    } T;
    DevBuf &acc = T.acc, &iacc = T.iacc, &out = T.out;
    if ((rc = dev_alloc(ctx, acc, sizeof(double) * n))) return rc;
    if ((rc = dev_alloc(ctx, out, sizeof(double) * n))) return rc;
    const int ni = P.intVecSize;
    if (ni > 0 && (rc = dev_alloc(ctx, iacc, sizeof(double) * ni))) return rc;
    if ((rc = drdd_device(ctx, dvar, h, D, dptr<double>(acc), ni > 0 ? dptr<double>(iacc) : nullptr))) return rc;
    if ((rc = int_to_ref_vec(ctx, dptr<double>(acc), dptr<double>(out), n))) return rc;
    CK(cudaMemcpyAsync(drudd, out.p, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    if (ni > 0 && int_drudd)
        CK(cudaMemcpyAsync(int_drudd, iacc.p, sizeof(double) * ni, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return ASTRO_OK;
}

extern "C" int astro_drdd_complex_condensed(astro_ctx *ctx, int32_t num, const int32_t *dvars, double h,
                                            const astro_state *state, double *drudd) {
    if (!ctx || num < 0 || (num > 0 && (!dvars || !drudd))) return ASTRO_ERR_ARG;
    for (int k = 0; k < num; ++k)
        if (dvars[k] < 1 || dvars[k] > ctx->numDvars)
            return set_err(ctx, ASTRO_ERR_ARG, "design variable " + std::to_string(dvars[k]) + " out of range");
    if (!(h > 0.0)) return set_err(ctx, ASTRO_ERR_ARG, "complex step h must be positive");
    const AstroPrep &P = ctx->P;
    const int n = P.n, ni = P.intVecSize;
    const bool condense = ni > 0;
    if (condense && !ctx->haveIntMat)
        return set_err(ctx, ASTRO_ERR_STATE, "needs the internal rows of astro_el_soln_load(build_mat = 1)");
    if (num == 0) return ASTRO_OK;
    int rc;
    DrddState D;
    if ((rc = drdd_state(ctx, state, D))) return rc;
    struct Tmp {
        DevBuf acc, iacc, out;
        ~Tmp() {
            dev_free(acc);
            dev_free(iacc);
            dev_free(out);
        }
    } T;
    if ((rc = dev_alloc(ctx, T.acc, sizeof(double) * n)) ||
        (rc = dev_alloc(ctx, T.out, sizeof(double) * (size_t)n * num)))
        return rc;
    if (ni > 0 && (rc = dev_alloc(ctx, T.iacc, sizeof(double) * ni))) return rc;
    for (int k = 0; k < num; ++k) {
        if ((rc = drdd_device(ctx, dvars[k], h, D, dptr<double>(T.acc), ni > 0 ? dptr<double>(T.iacc) : nullptr)))
            return rc;
        if (condense && (rc = elem_update_external_rhs(ctx, dptr<double>(T.iacc), dptr<double>(T.acc)))) return rc;
        if ((rc = int_to_ref_vec(ctx, dptr<double>(T.acc), dptr<double>(T.out) + (size_t)k * n, n))) return rc;
    }
    CK(cudaMemcpyAsync(drudd, T.out.p, sizeof(double) * (size_t)n * num, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return ASTRO_OK;
}

// Per-CTA partial sums of a . b (256 threads per CTA); the host adds them in CTA order.
__global__ void k_dot_part(const double *__restrict__ a, const double *__restrict__ b, int n, double *part) {
    __shared__ double sp[8];
    double s = 0.0;
    for (int i = blockIdx.x * 256 + threadIdx.x; i < n; i += gridDim.x * 256) s += a[i] * b[i];
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sp[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int q = 0; q < 8; ++q) t += sp[q];
        part[blockIdx.x] = t;
    }
}

static int dev_dot(astro_ctx *ctx, const double *a, const double *b, int n, DevBuf &part, double *out) {
    constexpr int kCtas = 152;
    if (!part.p) {
        int rc = dev_alloc(ctx, part, sizeof(double) * kCtas);
        if (rc) return rc;
    }
    k_dot_part<<<kCtas, 256, 0, ctx->stream>>>(a, b, n, dptr<double>(part));
    double h[kCtas];
    CK(cudaMemcpyAsync(h, part.p, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    double s = 0.0;
    for (int q = 0; q < kCtas; ++q) s += h[q];
    *out = s;
    return ASTRO_OK;
}

extern "C" int astro_element_matrices(astro_ctx *ctx, int32_t precision, const astro_state *state, double *ke_out,
                                      double *ru_out) {
    if (!ctx || !ke_out || (precision != 64 && precision != 32)) return ASTRO_ERR_ARG;
    const AstroPrep &P = ctx->P;
    DevBuf dk, dr;
    int rc;
    if ((rc = dev_alloc(ctx, dk, sizeof(double) * 576 * (size_t)P.E))) return rc;
    if (ru_out && (rc = dev_alloc(ctx, dr, sizeof(double) * 24 * (size_t)P.E))) return rc;
    DevState S;
    if (state && state->node_disp && (rc = state_vec_up(ctx, state->node_disp, S.disp))) return rc;
    // the previous step's state, as the global load does: the shell kinematics and the Newmark
    // inertia of either element family read it
    if (state && (ctx->hasShell || state->dynamic) &&
        ((rc = state_vec_up(ctx, state->prev_disp, S.pdisp)) || (rc = state_vec_up(ctx, state->prev_vel, S.pvel)) ||
         (rc = state_vec_up(ctx, state->prev_acc, S.pacc))))
        return rc;
    if (ctx->hasSolid) {
        ElemDevState ds;
        if ((rc = elem_state(ctx, state, S, ds))) return rc;
        if (precision == 32) {
            if (S.disp.p || ds.dynamic || ctx->has81)
                return set_err(ctx, ASTRO_ERR_UNSUPPORTED,
                               "the FP32 element kernel evaluates brick8 elements at the zero state only");
            rc = launch_hex8_element_mats(ctx, 32, dptr<double>(dk));
        } else {
            rc = solid_soln_load(ctx, 1, ds, nullptr, nullptr, dptr<double>(dk), dr.p ? dptr<double>(dr) : nullptr);
        }
    } else {
        if (precision == 32) return set_err(ctx, ASTRO_ERR_UNSUPPORTED, "FP32 shell kernel not provided");
        ElemDevState ds;
        if ((rc = elem_state(ctx, state, S, ds))) return rc;
        rc = launch_shell4_assemble(ctx, ds, nullptr, nullptr, 1, dptr<double>(dk), dr.p ? dptr<double>(dr) : nullptr);
    }
    if (rc) return rc;
    CK(cudaMemcpyAsync(ke_out, dk.p, sizeof(double) * 576 * (size_t)P.E, cudaMemcpyDeviceToHost, ctx->stream));
    if (ru_out) CK(cudaMemcpyAsync(ru_out, dr.p, sizeof(double) * 24 * (size_t)P.E, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    dev_free(dk);
    dev_free(dr);
    return ASTRO_OK;
}

// Penalty matrix C^T C in internal numbering, grouped by block row.
static int build_penalty(astro_ctx *ctx) {
    const AstroPrep &P = ctx->P;
    std::map<std::pair<int, int>, double> pen;
    for (int r = 0; r < P.mpcDim; ++r)
        for (int a = P.mpcRange[r]; a < P.mpcRange[r + 1]; ++a) {
            if (!P.mpcCols[a]) continue;
            const int ia = ref2int(P, P.mpcCols[a]);
            for (int b = P.mpcRange[r]; b < P.mpcRange[r + 1]; ++b) {
                if (!P.mpcCols[b]) continue;
                const int ib = ref2int(P, P.mpcCols[b]);
                pen[{ia, ib}] += ctx->mpcScaledHost[a] * ctx->mpcScaledHost[b];
            }
        }
    std::vector<int> ptr(P.N + 1, 0), prow, pcol;
    std::vector<double> pval;
    for (auto &kv : pen) ptr[kv.first.first / P.dpn + 1]++;
    for (int r = 0; r < P.N; ++r) ptr[r + 1] += ptr[r];
    prow.resize(pen.size());
    pcol.resize(pen.size());
    pval.resize(pen.size());
    std::vector<int> fill(ptr.begin(), ptr.end() - 1);
    ctx->penI.clear();
    ctx->penJ.clear();
    ctx->penV.clear();
    for (auto &kv : pen) {
        ctx->penI.push_back(kv.first.first);
        ctx->penJ.push_back(kv.first.second);
        ctx->penV.push_back(kv.second);
    }
    for (auto &kv : pen) {
        int br = kv.first.first / P.dpn;
        int t = fill[br]++;
        prow[t] = kv.first.first % P.dpn;
        pcol[t] = kv.first.second;
        pval[t] = kv.second;
    }
    int rc;
    ctx->penRows = (int)pen.size();
    if ((rc = upload(ctx, ctx->d_penPtr, ptr.data(), sizeof(int) * ptr.size()))) return rc;
    if ((rc = upload(ctx, ctx->d_penRow, prow.data(), sizeof(int) * prow.size()))) return rc;
    if ((rc = upload(ctx, ctx->d_penCol, pcol.data(), sizeof(int) * pcol.size()))) return rc;
    if ((rc = upload(ctx, ctx->d_penVal, pval.data(), sizeof(double) * pval.size()))) return rc;
    ctx->penVersion++;
    return ASTRO_OK;
}

extern "C" int astro_scale_mpc(astro_ctx *ctx, double *mpc_mat, double *mpc_rhs) {
    if (!ctx) return ASTRO_ERR_ARG;
    const AstroPrep &P = ctx->P;
    double maxMat = 0.0;
    int st = ASTRO_OK;
    if (ctx->haveK64) {
        maxMat = bsr_absmax(ctx, &st, 64);
    } else if (ctx->haveK32) {
        maxMat = bsr_absmax(ctx, &st, 32);
    } else {
        return set_err(ctx, ASTRO_ERR_STATE, "scale_mpc called before the stiffness was assembled");
    }
    if (st) return st;
    ctx->mpcScaledHost = P.mpcMat;
    ctx->mpcRhsScaledHost = P.mpcRhs;
    for (int r = 0; r < P.mpcDim; ++r) {
        double mag = 0.0;
        for (int k = P.mpcRange[r]; k < P.mpcRange[r + 1]; ++k) mag += ctx->mpcScaledHost[k] * ctx->mpcScaledHost[k];
        mag = std::sqrt(mag);
        for (int k = P.mpcRange[r]; k < P.mpcRange[r + 1]; ++k) ctx->mpcScaledHost[k] = (1.0 / mag) * ctx->mpcScaledHost[k];
        ctx->mpcRhsScaledHost[r] = (1.0 / mag) * ctx->mpcRhsScaledHost[r];
    }
    for (auto &v : ctx->mpcScaledHost) v = 100.0 * maxMat * v;
    for (auto &v : ctx->mpcRhsScaledHost) v = 100.0 * maxMat * v;
    int rc = build_penalty(ctx);
    if (rc) return rc;
    // the scaled constraints in internal numbering, for the device constraint load
    if (P.mpcDim > 0) {
        std::vector<int> colInt(P.mpcCols.size());
        for (size_t k = 0; k < colInt.size(); ++k) {
            const int d = P.mpcCols[k];  // 1-based reference DOF (component-major), 0 = empty
            colInt[k] = d ? ((d - 1) % P.N) * P.dpn + (d - 1) / P.N : -1;
        }
        if ((rc = upload(ctx, ctx->d_mpcRange, P.mpcRange.data(), sizeof(int) * P.mpcRange.size()))) return rc;
        if ((rc = upload(ctx, ctx->d_mpcCol, colInt.data(), sizeof(int) * colInt.size()))) return rc;
        if ((rc = upload(ctx, ctx->d_mpcVal, ctx->mpcScaledHost.data(), sizeof(double) * ctx->mpcScaledHost.size())))
            return rc;
        if ((rc = upload(ctx, ctx->d_mpcRhs, ctx->mpcRhsScaledHost.data(), sizeof(double) * ctx->mpcRhsScaledHost.size())))
            return rc;
        if ((rc = dev_alloc(ctx, ctx->d_mpcT, sizeof(double) * P.mpcDim))) return rc;
        // gather lists of the constraint load: the terms of every constrained DOF in row order
        std::vector<int> termRow(colInt.size()), order;
        for (int r = 0; r < P.mpcDim; ++r)
            for (int k = P.mpcRange[r]; k < P.mpcRange[r + 1]; ++k) {
                termRow[k] = r;
                if (colInt[k] >= 0) order.push_back(k);
            }
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return colInt[a] < colInt[b]; });
        std::vector<int> gptr(1, 0), grow;
        for (size_t q = 0; q < order.size(); ++q)
            if (q == 0 || colInt[order[q]] != colInt[order[q - 1]]) {
                if (q) gptr.push_back((int)q);
                grow.push_back(colInt[order[q]]);
            }
        gptr.push_back((int)order.size());
        ctx->mpcTargets = (int)grow.size();
        if ((rc = upload(ctx, ctx->d_mpcGPtr, gptr.data(), sizeof(int) * gptr.size()))) return rc;
        if (order.empty()) {
            order.push_back(0);  // placeholders, never read (no target)
            grow.push_back(0);
        }
        if ((rc = upload(ctx, ctx->d_mpcGTerm, order.data(), sizeof(int) * order.size()))) return rc;
        if ((rc = upload(ctx, ctx->d_mpcGRow, grow.data(), sizeof(int) * grow.size()))) return rc;
        if ((rc = upload(ctx, ctx->d_mpcTermRow, termRow.data(), sizeof(int) * termRow.size()))) return rc;
    }
    ctx->mpcScaled = 1;
    if (mpc_mat) std::copy(ctx->mpcScaledHost.begin(), ctx->mpcScaledHost.end(), mpc_mat);
    if (mpc_rhs) std::copy(ctx->mpcRhsScaledHost.begin(), ctx->mpcRhsScaledHost.end(), mpc_rhs);
    return ASTRO_OK;
}

extern "C" int astro_constraint_load(astro_ctx *ctx, const double *node_disp, double *elastic_load) {
    if (!ctx || !elastic_load) return ASTRO_ERR_ARG;
    const AstroPrep &P = ctx->P;
    if (P.mpcDim == 0) return ASTRO_OK;
    if (!ctx->mpcScaled) return set_err(ctx, ASTRO_ERR_STATE, "astro_scale_mpc must run first");
    const int n = P.n;
    int rc;
    if ((rc = ensure_io(ctx, false))) return rc;
    DevState S;
    if ((rc = state_vec_up(ctx, node_disp, S.disp))) return rc;
    double *dRef = dptr<double>(ctx->d_ioRef), *dInt = dptr<double>(ctx->d_ioInt);
    CK(cudaMemcpyAsync(dRef, elastic_load, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
    if ((rc = ref_to_int_vec(ctx, dRef, dInt, n))) return rc;
    if ((rc = constraint_load_dev(ctx, S.disp.p ? dptr<double>(S.disp) : nullptr, dInt))) return rc;
    if ((rc = int_to_ref_vec(ctx, dInt, dRef, n))) return rc;
    CK(cudaMemcpyAsync(elastic_load, dRef, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return ASTRO_OK;
}

extern "C" int astro_surface_load(astro_ctx *ctx, int32_t nfaces, const int32_t *face_el, const int32_t *face_num,
                                  const double *traction, double pressure, double *elastic_load) {
    if (!ctx || !elastic_load || nfaces < 0 || (nfaces && (!face_el || !face_num))) return ASTRO_ERR_ARG;
    const AstroPrep &P = ctx->P;
    for (int f = 0; f < nfaces; ++f) {
        int e = face_el[f], fn = face_num[f];
        if (e < 1 || e > P.E) return set_err(ctx, ASTRO_ERR_ARG, "face element out of range");
        int nfmax = (ctx->etype[e - 1] == 8 || ctx->etype[e - 1] == 81) ? 6 : 2;
        if (fn < 1 || fn > nfmax) return set_err(ctx, ASTRO_ERR_ARG, "face number out of range");
    }
    double tr[3] = {0, 0, 0};
    if (traction) std::copy(traction, traction + 3, tr);
    DevBuf dfe, dfn, dl, dref;
    int rc;
    if ((rc = upload(ctx, dfe, face_el, sizeof(int) * nfaces))) return rc;
    if ((rc = upload(ctx, dfn, face_num, sizeof(int) * nfaces))) return rc;
    if ((rc = state_vec_up(ctx, elastic_load, dl, false))) return rc;
    if ((rc = surface_load_dev(ctx, nfaces, dptr<int>(dfe), dptr<int>(dfn), tr, pressure, dptr<double>(dl)))) return rc;
    if ((rc = dev_alloc(ctx, dref, sizeof(double) * P.n))) return rc;
    if ((rc = int_to_ref_vec(ctx, dptr<double>(dl), dptr<double>(dref), P.n))) return rc;
    CK(cudaMemcpyAsync(elastic_load, dref.p, sizeof(double) * P.n, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    dev_free(dfe);
    dev_free(dfn);
    dev_free(dl);
    dev_free(dref);
    return ASTRO_OK;
}

int krylov_solve_static(astro_ctx *ctx, const double *d_b, double *d_x, const astro_solve_opts *o, astro_solve_stats *st);
int krylov_apply(astro_ctx *ctx, int kind, const double *d_x, double *d_y);

extern "C" int astro_solve_static(astro_ctx *ctx, const double *f, double *u, const astro_solve_opts *opts,
                                  astro_solve_stats *stats) {
    if (!ctx || !f || !u || !opts) return ASTRO_ERR_ARG;
    if (opts->rtol <= 0) return set_err(ctx, ASTRO_ERR_ARG, "rtol must be positive");
    if (!ctx->mpcScaled && ctx->P.mpcDim > 0)
        return set_err(ctx, ASTRO_ERR_STATE, "astro_scale_mpc must run before the solve");
    if (opts->method < ASTRO_SOLVER_GMRES_JACOBI_FP64 || opts->method > ASTRO_SOLVER_FGMRES_LEARNED)
        return set_err(ctx, ASTRO_ERR_ARG, "unknown solver method");
    const int n = ctx->P.n;
    DevBuf db, dx;
    int rc;
    if ((rc = state_vec_up(ctx, f, db, false))) return rc;
    if ((rc = state_vec_up(ctx, u, dx, false))) return rc;
    rc = krylov_solve_static(ctx, dptr<double>(db), dptr<double>(dx), opts, stats);
    if (rc && rc != ASTRO_ERR_MAXIT) {
        dev_free(db);
        dev_free(dx);
        return rc;
    }
    DevBuf dref;
    int rc2;
    if ((rc2 = dev_alloc(ctx, dref, sizeof(double) * n))) return rc2;
    if ((rc2 = int_to_ref_vec(ctx, dptr<double>(dx), dptr<double>(dref), n))) return rc2;
    CK(cudaMemcpyAsync(u, dref.p, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    dev_free(dref);
    dev_free(db);
    dev_free(dx);
    return rc;
}

// y = (K + C^T C) x for host vectors in reference numbering (kind 64: FP64 K, 32: FP32 K).
extern "C" int astro_apply_operator(astro_ctx *ctx, int32_t kind, const double *x, double *y) {
    if (!ctx || !x || !y) return ASTRO_ERR_ARG;
    if ((kind == 64 && !ctx->haveK64) || (kind == 32 && !ctx->haveK32)) return set_err(ctx, ASTRO_ERR_STATE, "no matrix");
    const int n = ctx->P.n;
    DevBuf dx, dy, dref;
    int rc;
    if ((rc = state_vec_up(ctx, x, dx, false))) return rc;
    if ((rc = dev_alloc(ctx, dy, sizeof(double) * n))) return rc;
    if ((rc = krylov_apply(ctx, kind, dptr<double>(dx), dptr<double>(dy)))) return rc;
    if ((rc = dev_alloc(ctx, dref, sizeof(double) * n))) return rc;
    if ((rc = int_to_ref_vec(ctx, dptr<double>(dy), dptr<double>(dref), n))) return rc;
    CK(cudaMemcpyAsync(y, dref.p, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    for (int i = 0; i < n; ++i) y[i] = -y[i];  // the residual kernel returned 0 - A x
    dev_free(dx);
    dev_free(dy);
    dev_free(dref);
    return ASTRO_OK;
}

// Host-only analysis preparation, callable without a GPU: the integer set-up of
// astro_ctx_create.  Pass NULL arrays to obtain only the sizes.  el_mat_cols receives the
// column numbers that astro_el_soln_load exports (the reference's find-or-insert order).
extern "C" int astro_prep_host(const astro_model *m, astro_dims *dims, int32_t *current_rank, int32_t *n_dof_index,
                               int32_t *el_mat_range, int32_t *el_mat_lt_range, int32_t *el_mat_cols,
                               int32_t *num_colors) {
    if (!m || !dims) return set_err(nullptr, ASTRO_ERR_ARG, "null argument");
    astro_ctx tmp;
    int rc = astro_prep_build(&tmp, m);
    if (rc) return set_err(nullptr, rc, tmp.err);
    const AstroPrep &P = tmp.P;
    dims->el_mat_dim = P.n;
    dims->el_mat_size = P.elMatSize;
    dims->el_mat_lt_size = P.ltSize;
    dims->el_mpc_dim = P.mpcDim;
    dims->el_mpc_size = P.mpcSize;
    dims->int_vec_size = P.intVecSize;
    dims->int_mat_size = P.intMatSize;
    dims->solver_max_bw = P.solverMaxBW;
    dims->dof_per_node = P.dpn;
    dims->num_blocks = P.nb;
    dims->num_colors = P.ncolors;
    if (num_colors) *num_colors = P.ncolors;
    if (current_rank) std::copy(P.currentRank.begin() + 1, P.currentRank.end(), current_rank);
    if (n_dof_index) std::copy(P.nDofIndex.begin(), P.nDofIndex.end(), n_dof_index);
    if (el_mat_range) std::copy(P.elMatRange.begin(), P.elMatRange.end(), el_mat_range);
    if (el_mat_lt_range) std::copy(P.elMatLTRange.begin(), P.elMatLTRange.end(), el_mat_lt_range);
    if (el_mat_cols) {
        for (int r = 0; r < P.N; ++r)
            for (int k = P.bRowPtr[r]; k < P.bRowPtr[r + 1]; ++k)
                for (int i = 0; i < P.dpn; ++i)
                    for (int j = 0; j < P.dpn; ++j) {
                        const int dofRow = r + 1 + i * P.N;
                        const long long idx = (long long)P.elMatRange[dofRow - 1] + P.csrPosInRow[(size_t)k * P.dpn + j];
                        el_mat_cols[idx] = P.bCol[k] + 1 + j * P.N;
                    }
    }
    return ASTRO_OK;
}

int shell_kernel_attrs(char *buf, int len);
// Kernel resource attributes and runtime limits (diagnostics; launches nothing).
extern "C" int astro_debug_info(char *buf, int32_t len) {
    if (!buf || len <= 0) return ASTRO_ERR_ARG;
    return shell_kernel_attrs(buf, len);
}

// Status word written by bounds-checked builds (0 = no violation, else the site number).
extern "C" int astro_debug_status(astro_ctx *ctx, int32_t *status) {
    if (!ctx || !status) return ASTRO_ERR_ARG;
    CK(cudaStreamSynchronize(ctx->stream));
    CK(cudaMemcpy(status, ctx->d_status.p, sizeof(int32_t), cudaMemcpyDeviceToHost));
    return ASTRO_OK;
}

extern "C" int astro_set_option(astro_ctx *ctx, int32_t option, int32_t value) {
    if (!ctx) return ASTRO_ERR_ARG;
    if (option == ASTRO_OPT_SHELL_MEAN_ROT_TERM) {
        ctx->quirkShellMeanRot = value ? 1 : 0;
        return ASTRO_OK;
    }
    if (option == ASTRO_OPT_UNROLLED_CYCLES) {
        ctx->unrolledCycles = value ? 1 : 0;
        krylov_release(ctx);  // recapture the cycles in the chosen form
        return ASTRO_OK;
    }
    if (option == ASTRO_OPT_CASES_TWIST) {
        if (value < 0 || value > 2) return set_err(ctx, ASTRO_ERR_ARG, "ASTRO_OPT_CASES_TWIST: 0, 1 or 2");
        ctx->casesTwist = value;
        return ASTRO_OK;
    }
    if (option == ASTRO_OPT_PANELS_SOLVE) {
        if (value < 0 || value > 2) return set_err(ctx, ASTRO_ERR_ARG, "ASTRO_OPT_PANELS_SOLVE: 0, 1 or 2");
        ctx->panelsSolve = value;
        return ASTRO_OK;
    }
    if (option == ASTRO_OPT_BAND_FP64_UPDATE) {
        if (value < 0 || value > 3) return set_err(ctx, ASTRO_ERR_ARG, "ASTRO_OPT_BAND_FP64_UPDATE: 0 .. 3");
        ctx->bandFp64Update = value;
        return ASTRO_OK;
    }
    if (option == ASTRO_OPT_BRICK_WARPS || option == ASTRO_OPT_PANEL_CLUSTER || option == ASTRO_OPT_CASES_CLUSTER) {
        const bool ok = option == ASTRO_OPT_BRICK_WARPS ? (value == 0 || value == 1 || value == 2 || value == 4)
                                                        : (value == 0 || value == 2 || value == 4 || value == 8);
        if (!ok) return set_err(ctx, ASTRO_ERR_ARG, "launch shape not among the candidates");
        if (option == ASTRO_OPT_BRICK_WARPS) {
            ctx->tuneHex8Warps = value;
            if (ctx->asmExec) cudaGraphExecDestroy(ctx->asmExec);  // the captured pass holds the old shape
            if (ctx->asmGraph) cudaGraphDestroy(ctx->asmGraph);
            ctx->asmExec = nullptr;
            ctx->asmGraph = nullptr;
        } else if (option == ASTRO_OPT_PANEL_CLUSTER) {
            ctx->tunePanelCluster = value;
        } else {
            ctx->tuneCasesCluster = value;
        }
        return ASTRO_OK;
    }
    return set_err(ctx, ASTRO_ERR_ARG, "unknown option");
}

// getTotaldLdD, static branch (Working/AStrO_commandFunctions.f90:1384-1410), with the elastic
// branch of solveDynamicAdjoint (:932-956; with dLdv = dLda = 0 its accAdj vanishes): the adjoint
// lambda solves K lambda = dLdu after updateExternalRHS(dLdu, intdLdu) (K is symmetric, and the
// reference solves with K itself), updateInternalSoln gives the internal lambda, and each design
// variable d adds -lambda . dRudD(d) - lambda_int . intdRudD(d) to dLdD(d), dRudD by the complex
// step at the given state.  All vectors stay on the device; the dot products reduce in a fixed order.
extern "C" int astro_total_dldd(astro_ctx *ctx, const astro_state *state, double h, const double *dldu,
                                const double *int_dldu, const double *dldd_explicit, const astro_solve_opts *opts,
                                double *dldd, double *disp_adj, double *int_disp_adj, astro_solve_stats *stats) {
    if (!ctx || !dldu || !opts || !dldd) return ASTRO_ERR_ARG;
    if (!(h > 0.0)) return set_err(ctx, ASTRO_ERR_ARG, "complex step h must be positive");
    if (!ctx->haveK64) return set_err(ctx, ASTRO_ERR_STATE, "needs the FP64 stiffness of astro_el_soln_load(build_mat = 1)");
    if (!ctx->mpcScaled && ctx->P.mpcDim > 0) return set_err(ctx, ASTRO_ERR_STATE, "astro_scale_mpc must run before the adjoint");
    const int n = ctx->P.n, ni = ctx->P.intVecSize, nd = ctx->numDvars;
    const bool hasInt = ni > 0;
    if (hasInt && !ctx->haveIntMat) return set_err(ctx, ASTRO_ERR_STATE, "needs the internal rows of astro_el_soln_load(build_mat = 1)");
    struct Tmp {
        DevBuf b, x, il, ir, acc, iacc, part, ref;
        ~Tmp() {
            DevBuf *v[] = {&b, &x, &il, &ir, &acc, &iacc, &part, &ref};
            for (DevBuf *p : v) dev_free(*p);
        }
    } T;
    int rc;
    if ((rc = state_vec_up(ctx, dldu, T.b, false))) return rc;
    if ((rc = dev_alloc(ctx, T.x, sizeof(double) * n))) return rc;
    CK(cudaMemsetAsync(T.x.p, 0, sizeof(double) * n, ctx->stream));
    if (hasInt) {
        if ((rc = dev_alloc(ctx, T.il, sizeof(double) * ni))) return rc;
        CK(cudaMemsetAsync(T.il.p, 0, sizeof(double) * ni, ctx->stream));
        if (int_dldu) {
            if ((rc = upload(ctx, T.ir, int_dldu, sizeof(double) * ni))) return rc;
            if ((rc = elem_update_external_rhs(ctx, dptr<double>(T.ir), dptr<double>(T.b)))) return rc;
        }
    }
    astro_solve_stats st{};
    rc = krylov_solve_static(ctx, dptr<double>(T.b), dptr<double>(T.x), opts, &st);
    if (stats) *stats = st;
    if (rc) return rc;
    if (hasInt && (rc = elem_update_internal_soln(ctx, dptr<double>(T.x), dptr<double>(T.il),
                                                    T.ir.p ? dptr<double>(T.ir) : nullptr)))
        return rc;
    // dLdD = explicit part - lambda . dRudD for every design variable
    if (nd > 0) {
        DrddState D;
        if ((rc = drdd_state(ctx, state, D))) return rc;
        if ((rc = dev_alloc(ctx, T.acc, sizeof(double) * n))) return rc;
        if (hasInt && (rc = dev_alloc(ctx, T.iacc, sizeof(double) * ni))) return rc;
        if (ctx->hasSolid) {
            // solids: up to kBatch variables per pass of the complex-step kernels, one launch per
            // colour over all of them (the per-variable launches cover a few SMs each)
            constexpr int kBatch = 16;
            const int nb = std::min(nd, kBatch);
            if ((rc = dev_alloc(ctx, T.acc, sizeof(double) * (size_t)n * nb))) return rc;
            if (hasInt && (rc = dev_alloc(ctx, T.iacc, sizeof(double) * (size_t)ni * nb))) return rc;
            for (int d0 = 1; d0 <= nd; d0 += nb) {
                const int cnt = std::min(nb, nd - d0 + 1);
                CK(cudaMemsetAsync(T.acc.p, 0, sizeof(double) * (size_t)n * cnt, ctx->stream));
                if (hasInt) CK(cudaMemsetAsync(T.iacc.p, 0, sizeof(double) * (size_t)ni * cnt, ctx->stream));
                if ((rc = solid_drdd_batch(ctx, d0, cnt, h, D.ds, dptr<double>(T.acc),
                                           hasInt ? dptr<double>(T.iacc) : nullptr)))
                    return rc;
                for (int k = 0; k < cnt; ++k) {
                    // dR/dd = -(sum of -Im Ru) / h: the dot with lambda scaled once
                    double s = 0.0, si = 0.0;
                    if ((rc = dev_dot(ctx, dptr<double>(T.x), dptr<double>(T.acc) + (size_t)k * n, n, T.part, &s)))
                        return rc;
                    if (hasInt && (rc = dev_dot(ctx, dptr<double>(T.il), dptr<double>(T.iacc) + (size_t)k * ni, ni,
                                                T.part, &si)))
                        return rc;
                    const int d = d0 + k;
                    dldd[d - 1] = (dldd_explicit ? dldd_explicit[d - 1] : 0.0) + (s + si) / h;
                }
            }
        } else {
            for (int d = 1; d <= nd; ++d) {
                if ((rc = drdd_device(ctx, d, h, D, dptr<double>(T.acc), hasInt ? dptr<double>(T.iacc) : nullptr)))
                    return rc;
                double s = 0.0, si = 0.0;
                if ((rc = dev_dot(ctx, dptr<double>(T.x), dptr<double>(T.acc), n, T.part, &s))) return rc;
                if (hasInt && (rc = dev_dot(ctx, dptr<double>(T.il), dptr<double>(T.iacc), ni, T.part, &si))) return rc;
                dldd[d - 1] = (dldd_explicit ? dldd_explicit[d - 1] : 0.0) - s - si;
            }
        }
    }
    if (disp_adj) {
        if ((rc = dev_alloc(ctx, T.ref, sizeof(double) * n))) return rc;
        if ((rc = int_to_ref_vec(ctx, dptr<double>(T.x), dptr<double>(T.ref), n))) return rc;
        CK(cudaMemcpyAsync(disp_adj, T.ref.p, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    }
    if (int_disp_adj && hasInt)
        CK(cudaMemcpyAsync(int_disp_adj, T.il.p, sizeof(double) * ni, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return ASTRO_OK;
}

// Per-CTA maxima of |x| (256 threads per CTA); the host takes the maximum.
__global__ void k_absmax_part(const double *__restrict__ x, int n, double *part) {
    __shared__ double sp[8];
    double m = 0.0;
    for (int i = blockIdx.x * 256 + threadIdx.x; i < n; i += gridDim.x * 256) m = fmax(m, fabs(x[i]));
    for (int o = 16; o; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) sp[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int q = 0; q < 8; ++q) t = fmax(t, sp[q]);
        part[blockIdx.x] = t;
    }
}

__global__ void k_axpy_d(int n, double a, const double *__restrict__ x, double *__restrict__ y) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] += a * x[i];
}

// stepSolve, elastic static branch (Working/AStrO_commandFunctions.f90:681-749): up to 1 (linear
// geometry) or 20 (nonlinear) iterations, while max|delDisp| > 1e-12 (a single-precision literal in
// the reference): residual at the current state (and, for nonlinear geometry, the tangent; the
// constraint penalty keeps the scaling it had, as scaleElasticMPC is not repeated), plus the
// applied load and the constraint load, condensation, the solve warm-started from the previous
// increment, internal-DOF recovery, u += delDisp.  The state stays on the device for all
// iterations.
extern "C" int astro_step_solve(astro_ctx *ctx, const astro_step_opts *o, const double *applied_load, double *node_disp,
                                double *internal_disp, int32_t *iterations, astro_solve_stats *stats) {
    if (!ctx || !o || !node_disp) return ASTRO_ERR_ARG;
    if (!ctx->haveK64) return set_err(ctx, ASTRO_ERR_STATE, "needs the stiffness of astro_el_soln_load(build_mat = 1)");
    if (ctx->P.mpcDim > 0 && !ctx->penRows && !ctx->mpcScaled)
        return set_err(ctx, ASTRO_ERR_STATE, "astro_scale_mpc must run before the step");
    const AstroPrep &P = ctx->P;
    const int n = P.n, ni = P.intVecSize;
    const bool hasInt = ni > 0;
    if (hasInt && !ctx->haveIntMat) return set_err(ctx, ASTRO_ERR_STATE, "needs the internal rows of astro_el_soln_load");
    const int maxNLIt = o->nl_geom ? 20 : 1;
    const double tol = (double)1e-12f;
    struct Tmp {
        DevBuf u, iu, f, load, iload, du, part, ref;
        ~Tmp() {
            DevBuf *v[] = {&u, &iu, &f, &load, &iload, &du, &part, &ref};
            for (DevBuf *p : v) dev_free(*p);
        }
    } T;
    int rc;
    if ((rc = state_vec_up(ctx, node_disp, T.u, false))) return rc;
    if (applied_load && (rc = state_vec_up(ctx, applied_load, T.f, false))) return rc;
    if ((rc = dev_alloc(ctx, T.load, sizeof(double) * n)) || (rc = dev_alloc(ctx, T.du, sizeof(double) * n)) ||
        (rc = dev_alloc(ctx, T.part, sizeof(double) * 152)))
        return rc;
    CK(cudaMemsetAsync(T.du.p, 0, sizeof(double) * n, ctx->stream));
    if (hasInt) {
        if ((rc = dev_alloc(ctx, T.iload, sizeof(double) * ni))) return rc;
        if (internal_disp) {
            if ((rc = upload(ctx, T.iu, internal_disp, sizeof(double) * ni))) return rc;
        } else {
            if ((rc = dev_alloc(ctx, T.iu, sizeof(double) * ni))) return rc;
            CK(cudaMemsetAsync(T.iu.p, 0, sizeof(double) * ni, ctx->stream));
        }
    }
    astro_solve_stats acc{};
    double delUNorm = 1.0;
    int it = 0;
    const unsigned g = (n + 255) / 256;
    while (it < maxNLIt && delUNorm > tol) {
        CK(cudaMemsetAsync(T.load.p, 0, sizeof(double) * n, ctx->stream));
        if (hasInt) CK(cudaMemsetAsync(T.iload.p, 0, sizeof(double) * ni, ctx->stream));
        const int build = o->nl_geom ? 1 : 0;
        if (build) {
            if ((rc = ensure_K(ctx, 2))) return rc;
            if (ctx->hasShell && (rc = bsr_zero(ctx, 2))) return rc;
        }
        ElemDevState ds;
        ds.disp = dptr<double>(T.u);
        ds.idisp = hasInt ? dptr<double>(T.iu) : nullptr;
        if (ctx->hasSolid)
            rc = solid_soln_load(ctx, build, ds, dptr<double>(T.load), hasInt ? dptr<double>(T.iload) : nullptr, nullptr,
                                 nullptr);
        else
            rc = launch_shell4_assemble(ctx, ds, dptr<double>(T.load), hasInt ? dptr<double>(T.iload) : nullptr, build,
                                        nullptr, nullptr);
        if (rc) return rc;
        if (build) {
            ctx->k64Version++;
            ctx->haveIntMat = hasInt;
        }
        if (T.f.p) k_axpy_d<<<g, 256, 0, ctx->stream>>>(n, 1.0, dptr<double>(T.f), dptr<double>(T.load));
        if ((rc = constraint_load_dev(ctx, dptr<double>(T.u), dptr<double>(T.load)))) return rc;
        if (hasInt && (rc = elem_update_external_rhs(ctx, dptr<double>(T.iload), dptr<double>(T.load)))) return rc;
        astro_solve_stats s{};
        rc = krylov_solve_static(ctx, dptr<double>(T.load), dptr<double>(T.du), &o->solve, &s);
        acc.iterations += s.iterations;
        acc.restarts += s.restarts;
        acc.refinements += s.refinements;
        acc.seconds += s.seconds;
        acc.rel_residual = std::max(acc.rel_residual, s.rel_residual);
        acc.conditional_graph = s.conditional_graph;
        acc.fallback |= s.fallback;
        acc.residual_kind = s.residual_kind;
        if (rc && rc != ASTRO_ERR_MAXIT) return rc;
        if (rc == ASTRO_ERR_MAXIT) acc.status = rc;
        if (hasInt && (rc = elem_update_internal_soln(ctx, dptr<double>(T.du), dptr<double>(T.iu), dptr<double>(T.iload))))
            return rc;
        k_axpy_d<<<g, 256, 0, ctx->stream>>>(n, 1.0, dptr<double>(T.du), dptr<double>(T.u));
        k_absmax_part<<<152, 256, 0, ctx->stream>>>(dptr<double>(T.du), n, dptr<double>(T.part));
        double hp[152];
        CK(cudaMemcpyAsync(hp, T.part.p, sizeof(hp), cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
        delUNorm = 0.0;
        for (double v : hp) delUNorm = std::max(delUNorm, v);
        ++it;
    }
    if (iterations) *iterations = it;
    if ((rc = dev_alloc(ctx, T.ref, sizeof(double) * n))) return rc;
    if ((rc = int_to_ref_vec(ctx, dptr<double>(T.u), dptr<double>(T.ref), n))) return rc;
    CK(cudaMemcpyAsync(node_disp, T.ref.p, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    if (hasInt && internal_disp) CK(cudaMemcpyAsync(internal_disp, T.iu.p, sizeof(double) * ni, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (stats) *stats = acc;
    return acc.status ? acc.status : ASTRO_OK;
}
