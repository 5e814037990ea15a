// shell4 (reference type 41) element residual/tangent, static condensation and colour-ordered
// assembly, on the GPU in FP64 (and complex FP64 for the complex step).
//
// Algorithm (Working/AStrO_r_elementEqns.f90 r_getElRuk :2206-2533, r_getElRum :2535-2657,
// r_getElRu :2659-2720, r_condenseMat :2722-2743): a co-rotational Reissner-Mindlin quad with
// four Gauss points and eight incompatible internal DOF.  The instantaneous element frame is the
// section frame rotated by the mean nodal rotation (r_getInstOrient); local translations are
// instOri (u + X) - orient X and local rotations drIdrG (theta - mean) to second order
// (r_getInstDof).  The deformation vector (membrane, curvature, transverse shear, drilling,
// r_getShellDef) and its first/second derivatives with respect to the 32 element DOF give
//   Ru_i  = sum_gp w detJ (ABD def) . d def/d u_i
//   K_ij  = sum_gp w detJ [ d def_i^T ABD d def_j + (ABD def) . d2 def/d u_i d u_j ].
// The derivatives are evaluated exactly as the reference defines them, including its rotation
// derivative, which moves only the differentiated node's relative rotation and not the element
// mean (so the reference's tangent is not invariant under rigid rotations; the switch
// quirkShellMeanRot adds the mean-rotation term for the consistent variant).  The point
// rotation of the derivative terms uses the element's own nodes (the reference's loop reads a
// stale column offset there; its evident intent is kept).
//
// Mapping: the evaluation is a pipeline of one-thread-per-item kernels (elem_shell4_pipe.cuh)
// over per-element global scratch, run one element colour at a time; elements of a colour share
// no node, so their 6x6 block updates never collide (no atomics, deterministic).
#include <algorithm>
#include <functional>

#include "astro_internal.h"
#include "bounds.cuh"
#include "elem_shell4_pipe.cuh"

// Resource attributes of the shell kernels (no launch), for diagnostics.
int shell_kernel_attrs(char *buf, int len) {
    cudaFuncAttributes a{}, b{};
    size_t stack = 0;
    cudaError_t e1 = cudaFuncGetAttributes(&a, k_shell_kcol);
    cudaError_t e2 = cudaFuncGetAttributes(&b, k_shell_frame);
    cudaError_t e3 = cudaDeviceGetLimit(&stack, cudaLimitStackSize);
    snprintf(buf, len, "k_shell_kcol: err=%d regs=%d local=%zu | k_shell_frame: err=%d regs=%d local=%zu | stackLimit=%zu (err=%d)",
             (int)e1, a.numRegs, a.localSizeBytes, (int)e2, b.numRegs, b.localSizeBytes, stack, (int)e3);
    return ASTRO_OK;
}

// Per-element section properties on the device (computed once per context).
int shell_sections_prepare(astro_ctx *ctx, const astro_model *m) {
    const int S = m->num_sections, E = ctx->P.E;
    std::vector<int> lr(S + 1);
    for (int s = 0; s <= S; ++s) lr[s] = m->sec_layup_range[s];
    // the layer loops of the section properties run over lr[s] .. lr[s+1]: a prefix sum from 0
    if (lr[0] != 0) return set_err(ctx, ASTRO_ERR_ARG, "sec_layup_range must start at 0");
    for (int s = 0; s < S; ++s)
        if (lr[s + 1] < lr[s]) return set_err(ctx, ASTRO_ERR_ARG, "sec_layup_range must be nondecreasing");
    const int NL = lr[S];
    std::vector<LayerDev> lay(std::max(NL, 1));
    ctx->layMat.assign(m->layup_mat_id, m->layup_mat_id + NL);
    for (int l = 0; l < NL; ++l) {
        const int mat = m->layup_mat_id[l];
        if (mat < 1 || mat > m->num_materials) return set_err(ctx, ASTRO_ERR_ARG, "layup material out of range");
        const double *me = m->material_elastic + 9 * (size_t)(mat - 1);
        lay[l] = {me[0], me[1], me[3], me[6], m->layup_thickness[l], m->layup_angle[l],
                  m->material_density ? m->material_density[mat - 1] : 0.0};
    }
    std::vector<double> zo(S);
    for (int s = 0; s < S; ++s) zo[s] = m->section_z_offset ? m->section_z_offset[s] : 0.0;
    // the section inputs stay on the device for the complex-step property evaluation
    DevBuf &dlr = ctx->d_shLayRange, &dlay = ctx->d_shLay, &dzo = ctx->d_shZoff, &de2dR = ctx->d_e2dR,
           &de2d = ctx->d_e2d, &de2c = ctx->d_e2c, &dcat = ctx->d_dCat, &dlayer = ctx->d_dLayer, &dval = ctx->d_dVal;
    int rc;
    if ((rc = upload(ctx, dlr, lr.data(), sizeof(int) * lr.size()))) return rc;
    if ((rc = upload(ctx, dlay, lay.data(), sizeof(LayerDev) * lay.size()))) return rc;
    if ((rc = upload(ctx, dzo, zo.data(), sizeof(double) * zo.size()))) return rc;
    const bool dv = m->num_dvars > 0 && m->el_to_d_range;
    if (dv) {
        const int nE2D = m->el_to_d_range[E];
        std::vector<int> dl(m->num_dvars, 0);
        if (m->d_layer) dl.assign(m->d_layer, m->d_layer + m->num_dvars);
        if ((rc = upload(ctx, de2dR, m->el_to_d_range, sizeof(int) * (E + 1)))) return rc;
        if ((rc = upload(ctx, de2d, m->el_to_d, sizeof(int) * std::max(nE2D, 1)))) return rc;
        if ((rc = upload(ctx, de2c, m->el_to_coef, sizeof(double) * std::max(nE2D, 1)))) return rc;
        if ((rc = upload(ctx, dcat, m->d_category, sizeof(int) * m->num_dvars))) return rc;
        if ((rc = upload(ctx, dlayer, dl.data(), sizeof(int) * m->num_dvars))) return rc;
        if ((rc = upload(ctx, dval, m->d_value, sizeof(double) * m->num_dvars))) return rc;
        std::vector<int> dc(m->num_dvars, 0);
        if (m->d_component) dc.assign(m->d_component, m->d_component + m->num_dvars);
        if ((rc = upload(ctx, ctx->d_dComp, dc.data(), sizeof(int) * m->num_dvars))) return rc;
    }
    if ((rc = upload(ctx, ctx->d_secOrient, m->section_orient, sizeof(double) * 9 * S))) return rc;
    if ((rc = dev_alloc(ctx, ctx->d_secABD, sizeof(ShellProps) * (size_t)E))) return rc;
    shell_props_kernel<<<(E + 127) / 128, 128, 0, ctx->stream>>>(
        E, dptr<double>(ctx->d_nodes), dptr<int>(ctx->d_elist), dptr<int>(ctx->d_esec), dptr<double>(ctx->d_secOrient),
        dptr<int>(dlr), dptr<LayerDev>(dlay), dptr<double>(dzo), dv ? dptr<int>(de2dR) : nullptr,
        dv ? dptr<int>(de2d) : nullptr, dv ? dptr<double>(de2c) : nullptr, dv ? dptr<int>(dcat) : nullptr,
        dv ? dptr<int>(dlayer) : nullptr, dv ? dptr<int>(ctx->d_dComp) : nullptr, dv ? dptr<double>(dval) : nullptr,
        dptr<ShellProps>(ctx->d_secABD));
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (!ctx->d_intMat.p && (rc = dev_alloc(ctx, ctx->d_intMat, sizeof(double) * 256 * (size_t)E))) return rc;
    return cuda_check(ctx, e, "shell properties");
}

// The five pipeline kernels over the elements of each colour in turn: colour c covers
// els[ptr[c] .. ptr[c+1]) (device list).
static int shell_pipeline(astro_ctx *ctx, const ElemDevState &st, const int *d_els, const std::vector<int> &ptr,
                          const ShellProps *props, double gpc, double *d_loadInt, double *d_intLoad, int buildMat,
                          double *d_K, double *d_intMat, double *d_ke, double *d_ru, bool sync = true) {
    int maxc = 0;
    for (size_t c = 0; c + 1 < ptr.size(); ++c) maxc = std::max(maxc, ptr[c + 1] - ptr[c]);
    if (!maxc) return ASTRO_OK;
    // per-element scratch of the pipeline, kept in the context (grown on demand)
    DevBuf &fr = ctx->d_shFr, &gp = ctx->d_shGp, &de = ctx->d_shDe, &kf = ctx->d_shKf;
    int rc;
    if (maxc > ctx->shScratchEls) {
        if ((rc = dev_alloc(ctx, fr, sizeof(ShellFrame) * (size_t)maxc))) return rc;
        if ((rc = dev_alloc(ctx, gp, sizeof(ShellGP) * 4 * (size_t)maxc))) return rc;
        if ((rc = dev_alloc(ctx, de, sizeof(double) * 4 * 32 * 9 * (size_t)maxc))) return rc;
        if ((rc = dev_alloc(ctx, kf, sizeof(double) * 32 * 33 * (size_t)maxc))) return rc;
        ctx->shScratchEls = maxc;
    }
    ShellPipe A = {};
    A.nodes = dptr<double>(ctx->d_nodes);
    A.elist = dptr<int>(ctx->d_elist);
    A.rank = dptr<int>(ctx->d_rank);
    A.elBlk = dptr<int>(ctx->d_elBlk);
    A.props = props;
    A.disp = st.disp;
    A.pdisp = st.pdisp;
    A.pvel = st.pvel;
    A.pacc = st.pacc;
    A.idisp = st.idisp;
    A.dynamic = st.dynamic;
    A.massOnly = st.massOnly;
    A.beta = st.beta;
    A.gamma = st.gamma;
    A.delT = st.delT;
    A.buildMat = buildMat;
    A.quirk = ctx->quirkShellMeanRot;
    A.gpc = gpc;
    A.fr = dptr<ShellFrame>(fr);
    A.gp = dptr<ShellGP>(gp);
    A.dedU = dptr<double>(de);
    A.Kf = dptr<double>(kf);
    A.K = d_K;
    A.load = d_loadInt;
    A.intLoad = d_intLoad;
    A.intMat = d_intMat;
    A.keOut = d_ke;
    A.ruOut = d_ru;
    A.nNodes = ctx->P.N;
    A.nEls = ctx->P.E;
    A.nBlocks = ctx->P.nb;
    A.scratchEls = ctx->shScratchEls;
    A.status = ASTRO_CHECKED ? dptr<int>(ctx->d_guard) : nullptr;
    cudaStream_t s = ctx->stream;
    for (size_t col = 0; col + 1 < ptr.size(); ++col) {
        const int cnt = ptr[col + 1] - ptr[col];
        if (!cnt) continue;
        A.els = d_els + ptr[col];
        A.count = cnt;
        k_shell_frame<<<(cnt + 63) / 64, 64, 0, s>>>(A);
        k_shell_frame_rot<<<(10 * cnt + 63) / 64, 64, 0, s>>>(A);
        k_shell_frame_rest<<<(cnt + 63) / 64, 64, 0, s>>>(A);
        if (A.dynamic) k_shell_inam<<<(4 * cnt + 127) / 128, 128, 0, s>>>(A);
        k_shell_gauss<<<(4 * cnt + 127) / 128, 128, 0, s>>>(A);
        k_shell_dedu<<<(128 * cnt + 127) / 128, 128, 0, s>>>(A);
        k_shell_kcol<<<(32 * cnt + 127) / 128, 128, 0, s>>>(A);
        if (A.buildMat) {
            k_shell_cond_lu<<<(cnt + 63) / 64, 64, 0, s>>>(A);
            k_shell_cond_col<<<(24 * cnt + 127) / 128, 128, 0, s>>>(A);
        }
        k_shell_scatter<<<(32 * cnt + 127) / 128, 128, 0, s>>>(A);
    }
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && (sync || ASTRO_CHECKED)) e = cudaStreamSynchronize(s);
    if (e == cudaSuccess && ASTRO_CHECKED) return guard_status(ctx, "shell pipeline");
    return cuda_check(ctx, e, "shell pipeline");
}

// The pipeline over a colour-grouped element list (device list d_els, colour c covering
// ptr[c] .. ptr[c+1]), residual only, into d_loadInt (load -= Ru).
int shell4_residual_list(astro_ctx *ctx, const ElemDevState &st, const int *d_els, const std::vector<int> &ptr,
                         double *d_loadInt) {
    return shell_pipeline(ctx, st, d_els, ptr, dptr<ShellProps>(ctx->d_secABD), kShellRt3, d_loadInt, nullptr, 0,
                          nullptr, nullptr, nullptr, nullptr);
}

int launch_shell4_assemble(astro_ctx *ctx, const ElemDevState &st, double *d_loadInt, double *d_intLoad, int buildMat,
                           double *d_ke, double *d_ru, bool sync) {
    const bool toK = buildMat && !d_ke;
    return shell_pipeline(ctx, st, dptr<int>(ctx->d_colorEls), ctx->P.colorPtr, dptr<ShellProps>(ctx->d_secABD), kShellRt3,
                          d_loadInt, d_intLoad, buildMat, toK ? dptr<double>(ctx->d_K64) : nullptr,
                          toK ? dptr<double>(ctx->d_intMat) : nullptr, d_ke, d_ru, sync);
}

// Complex-step properties of the listed elements: orientation (real part), imaginary parts of
// ABD and of the section mass, written over a copy of the per-element properties.
__global__ void k_shell_props_im(int count, const int *els, const double *nodes, const int *elist, const int *esec,
                                 const double *secOrient, const int *layRange, const LayerDev *lay, const double *zoff,
                                 const int *e2dR, const int *e2d, const double *e2c, const int *dcat, const int *dlay,
                                 const int *dcomp, const double *dval, int dvar, double h, ShellProps *out) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= count) return;
    const int e = els[q];
    cplx o[3][3], ABD[9][9], M[6][6];
    shell_props<cplx>(nodes, elist + 8 * (size_t)e, secOrient, esec[e], layRange, lay, zoff, e2dR, e2d, e2c, dcat, dlay,
                      dcomp, dval, e, dvar, h, o, ABD, M);
    ShellProps &P = out[e];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) P.orient[3 * i + j] = o[i][j].re;
    for (int i = 0; i < 9; ++i)
        for (int j = 0; j < 9; ++j) P.ABD[9 * i + j] = ABD[i][j].im;
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) P.M[6 * i + j] = M[i][j].im;
}

// Complex step of the pipeline's residual over a colour-grouped element list (colour c covering
// list[ptr[c] .. ptr[c+1])): d_acc -= Im(Ru(d + i h)) (unscaled).  hook, when given, runs before
// each colour (with that colour's device list and count) and the colours then launch one by one.
int shell4_drdd_list(astro_ctx *ctx, int dvar, double h, const ElemDevState &st, const std::vector<int> &list,
                     const std::vector<int> &ptr, double *d_acc, double *d_intAcc,
                     const std::function<int(const int *, int)> &hook) {
    const int cnt = (int)list.size();
    if (!cnt) return ASTRO_OK;
    const int E = ctx->P.E;
    DevBuf dl, props;
    int rc;
    if ((rc = upload(ctx, dl, list.data(), sizeof(int) * cnt))) return rc;
    if ((rc = dev_alloc(ctx, props, sizeof(ShellProps) * (size_t)E))) {
        dev_free(dl);
        return rc;
    }
    cudaError_t e = cudaMemcpyAsync(props.p, ctx->d_secABD.p, sizeof(ShellProps) * (size_t)E, cudaMemcpyDeviceToDevice,
                                    ctx->stream);
    if (e == cudaSuccess) {
        k_shell_props_im<<<(cnt + 63) / 64, 64, 0, ctx->stream>>>(
            cnt, dptr<int>(dl), dptr<double>(ctx->d_nodes), dptr<int>(ctx->d_elist), dptr<int>(ctx->d_esec),
            dptr<double>(ctx->d_secOrient), dptr<int>(ctx->d_shLayRange), dptr<LayerDev>(ctx->d_shLay),
            dptr<double>(ctx->d_shZoff), dptr<int>(ctx->d_e2dR), dptr<int>(ctx->d_e2d), dptr<double>(ctx->d_e2c),
            dptr<int>(ctx->d_dCat), dptr<int>(ctx->d_dLayer), dptr<int>(ctx->d_dComp), dptr<double>(ctx->d_dVal), dvar, h,
            dptr<ShellProps>(props));
        e = cudaGetLastError();
    }
    rc = cuda_check(ctx, e, "shell complex-step properties");
    if (!rc && !hook)
        rc = shell_pipeline(ctx, st, dptr<int>(dl), ptr, dptr<ShellProps>(props), kShellRt3c, d_acc, d_intAcc, 0, nullptr,
                            nullptr, nullptr, nullptr);
    for (size_t c = 0; !rc && hook && c + 1 < ptr.size(); ++c) {
        const int n = ptr[c + 1] - ptr[c];
        if (!n) continue;
        rc = hook(dptr<int>(dl) + ptr[c], n);
        const std::vector<int> one = {ptr[c], ptr[c + 1]};
        if (!rc)
            rc = shell_pipeline(ctx, st, dptr<int>(dl), one, dptr<ShellProps>(props), kShellRt3c, d_acc, d_intAcc, 0,
                                nullptr, nullptr, nullptr, nullptr);
    }
    dev_free(dl);
    dev_free(props);
    return rc;
}

int shell4_drdd(astro_ctx *ctx, int dvar, double h, const ElemDevState &st, double *d_acc, double *d_intAcc) {
    const int cat = ctx->dCat[dvar - 1];
    if (cat == ASTRO_DCAT_ORIENTATION || cat == ASTRO_DCAT_NODE_COORD)
        return set_err(ctx, ASTRO_ERR_UNSUPPORTED,
                       "complex step of shell orientation or node-coordinate design variables (they enter the shell "
                       "kinematics, which run in real arithmetic) is not provided");
    std::vector<int> list, ptr;
    dvar_elements_by_colour(ctx, dvar, list, ptr);
    return shell4_drdd_list(ctx, dvar, h, st, list, ptr, d_acc, d_intAcc, nullptr);
}

// ---- internal-DOF recovery (updateExternalRHS / updateInternalSoln) ------------------------------
// The condensed internal rows of each shell element (8 rows x 32 columns: the coupling K_in to the
// 24 nodal DOF and the LU factors of K_ii, column-major as intElasticMat) stay on the device
// after the last assembly.

// ext -= K_ni K_ii^-1 int for the shells of one colour (they share no node, so the nodal
// updates of a launch never collide).
__global__ void k_shell_ext_rhs(int count, const int *__restrict__ els, const int *__restrict__ elist,
                                const int *__restrict__ rank, const double *__restrict__ intMat,
                                const double *__restrict__ intVec, double *__restrict__ extInt) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= count) return;
    const int e = els[q];
    const double *M = intMat + 256 * (size_t)e;
    double L[8][8], b[8], x[8];
    for (int r = 0; r < 8; ++r)
        for (int c = 0; c < 8; ++c) L[r][c] = M[8 * (24 + c) + r];
    for (int k = 0; k < 8; ++k) b[k] = intVec[8 * (size_t)e + k];
    a_lu_solve<double, 8>(&L[0][0], b, x, 8);
    const int *el = elist + 8 * (size_t)e;
    for (int i = 0; i < 24; ++i) {  // component-major element DOF: i = 4 (var) + node
        const int var = i / 4, a = i % 4;
        double s = 0.0;
        for (int k = 0; k < 8; ++k) s += M[8 * i + k] * x[k];
        extInt[6 * (size_t)(rank[el[a] - 1] - 1) + var] -= s;
    }
}

// int += K_ii^-1 (rhs - K_in ext), one thread per shell element.
__global__ void k_shell_int_soln(int E, const int *__restrict__ elist, const int *__restrict__ rank,
                                 const double *__restrict__ intMat, const double *__restrict__ extInt,
                                 const double *__restrict__ intRhs, double *__restrict__ intSoln) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    const double *M = intMat + 256 * (size_t)e;
    const int *el = elist + 8 * (size_t)e;
    double L[8][8], b[8], x[8];
    for (int r = 0; r < 8; ++r)
        for (int c = 0; c < 8; ++c) L[r][c] = M[8 * (24 + c) + r];
    for (int k = 0; k < 8; ++k) b[k] = intRhs ? intRhs[8 * (size_t)e + k] : 0.0;
    for (int i = 0; i < 24; ++i) {
        const int var = i / 4, a = i % 4;
        const double u = extInt[6 * (size_t)(rank[el[a] - 1] - 1) + var];
        for (int k = 0; k < 8; ++k) b[k] -= M[8 * i + k] * u;
    }
    a_lu_solve<double, 8>(&L[0][0], b, x, 8);
    for (int k = 0; k < 8; ++k) intSoln[8 * (size_t)e + k] += x[k];
}

int shell4_update_external_rhs(astro_ctx *ctx, const double *d_intVec, double *d_extInt) {
    const AstroPrep &P = ctx->P;
    for (int col = 0; col < P.ncolors; ++col) {
        const int cnt = P.colorPtr[col + 1] - P.colorPtr[col];
        if (!cnt) continue;
        k_shell_ext_rhs<<<(cnt + 127) / 128, 128, 0, ctx->stream>>>(
            cnt, dptr<int>(ctx->d_colorEls) + P.colorPtr[col], dptr<int>(ctx->d_elist), dptr<int>(ctx->d_rank),
            dptr<double>(ctx->d_intMat), d_intVec, d_extInt);
    }
    return cuda_check(ctx, cudaGetLastError(), "shell external rhs");
}

int shell4_update_internal_soln(astro_ctx *ctx, const double *d_extInt, double *d_intSoln, const double *d_intRhs) {
    const int E = ctx->P.E;
    k_shell_int_soln<<<(E + 127) / 128, 128, 0, ctx->stream>>>(E, dptr<int>(ctx->d_elist), dptr<int>(ctx->d_rank),
                                                               dptr<double>(ctx->d_intMat), d_extInt, d_intRhs,
                                                               d_intSoln);
    return cuda_check(ctx, cudaGetLastError(), "shell internal solution");
}
