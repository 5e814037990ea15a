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

#include "astro_internal.h"
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
    const int NL = lr[S];
    std::vector<LayerDev> lay(std::max(NL, 1));
    for (int l = 0; l < NL; ++l) {
        const int mat = m->layup_mat_id[l];
        if (mat < 1 || mat > m->num_materials) return set_err(ctx, ASTRO_ERR_ARG, "layup material out of range");
        const double *me = m->material_elastic + 9 * (size_t)(mat - 1);
        lay[l] = {me[0], me[1], me[3], me[6], m->layup_thickness[l], m->layup_angle[l],
                  m->material_density ? m->material_density[mat - 1] : 0.0};
    }
    std::vector<double> zo(S);
    for (int s = 0; s < S; ++s) zo[s] = m->section_z_offset ? m->section_z_offset[s] : 0.0;
    DevBuf dlr, dlay, dzo, de2dR, de2d, de2c, dcat, dlayer, dval;
    int rc;
    if ((rc = upload(ctx, dlr, lr.data(), sizeof(int) * lr.size()))) return rc;
    if ((rc = upload(ctx, dlay, lay.data(), sizeof(LayerDev) * lay.size()))) return rc;
    if ((rc = upload(ctx, dzo, zo.data(), sizeof(double) * zo.size()))) return rc;
    const bool dv = m->num_dvars > 0 && m->el_to_d_range;
    if (dv) {
        const int nE2D = m->el_to_d_range[E];
        if ((rc = upload(ctx, de2dR, m->el_to_d_range, sizeof(int) * (E + 1)))) return rc;
        if ((rc = upload(ctx, de2d, m->el_to_d, sizeof(int) * std::max(nE2D, 1)))) return rc;
        if ((rc = upload(ctx, de2c, m->el_to_coef, sizeof(double) * std::max(nE2D, 1)))) return rc;
        if ((rc = upload(ctx, dcat, m->d_category, sizeof(int) * m->num_dvars))) return rc;
        if ((rc = upload(ctx, dlayer, m->d_layer, sizeof(int) * m->num_dvars))) return rc;
        if ((rc = upload(ctx, dval, m->d_value, sizeof(double) * m->num_dvars))) return rc;
    }
    if ((rc = upload(ctx, ctx->d_secOrient, m->section_orient, sizeof(double) * 9 * S))) return rc;
    if ((rc = dev_alloc(ctx, ctx->d_secABD, sizeof(ShellProps) * (size_t)E))) return rc;
    shell_props_kernel<<<(E + 127) / 128, 128, 0, ctx->stream>>>(
        E, dptr<double>(ctx->d_nodes), dptr<int>(ctx->d_elist), dptr<int>(ctx->d_esec), dptr<double>(ctx->d_secOrient),
        dptr<int>(dlr), dptr<LayerDev>(dlay), dptr<double>(dzo), dv ? dptr<int>(de2dR) : nullptr,
        dv ? dptr<int>(de2d) : nullptr, dv ? dptr<double>(de2c) : nullptr, dv ? dptr<int>(dcat) : nullptr,
        dv ? dptr<int>(dlayer) : nullptr, dv ? dptr<double>(dval) : nullptr, dptr<ShellProps>(ctx->d_secABD));
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    DevBuf *bufs[] = {&dlr, &dlay, &dzo, &de2dR, &de2d, &de2c, &dcat, &dlayer, &dval};
    for (auto *b : bufs) dev_free(*b);
    if (!ctx->d_intMat.p && (rc = dev_alloc(ctx, ctx->d_intMat, sizeof(double) * 256 * (size_t)E))) return rc;
    return cuda_check(ctx, e, "shell properties");
}

int launch_shell4_assemble(astro_ctx *ctx, const ShellDevState &st, double *d_loadInt, double *d_intLoad, int buildMat,
                           double *d_ke, double *d_ru) {
    const AstroPrep &P = ctx->P;
    int maxc = 0;
    for (int col = 0; col < P.ncolors; ++col) maxc = std::max(maxc, P.colorPtr[col + 1] - P.colorPtr[col]);
    DevBuf fr, gp, de, kf;
    int rc;
    if ((rc = dev_alloc(ctx, fr, sizeof(ShellFrame) * (size_t)maxc))) return rc;
    if ((rc = dev_alloc(ctx, gp, sizeof(ShellGP) * 4 * (size_t)maxc))) return rc;
    if ((rc = dev_alloc(ctx, de, sizeof(double) * 4 * 32 * 9 * (size_t)maxc))) return rc;
    if ((rc = dev_alloc(ctx, kf, sizeof(double) * 32 * 33 * (size_t)maxc))) return rc;
    ShellPipe A = {};
    A.nodes = dptr<double>(ctx->d_nodes);
    A.elist = dptr<int>(ctx->d_elist);
    A.rank = dptr<int>(ctx->d_rank);
    A.elBlk = dptr<int>(ctx->d_elBlk);
    A.props = dptr<ShellProps>(ctx->d_secABD);
    A.disp = st.disp;
    A.pdisp = st.pdisp;
    A.pvel = st.pvel;
    A.pacc = st.pacc;
    A.idisp = st.idisp;
    A.dynamic = st.dynamic;
    A.beta = st.beta;
    A.gamma = st.gamma;
    A.delT = st.delT;
    A.buildMat = buildMat;
    A.quirk = ctx->quirkShellMeanRot;
    A.fr = dptr<ShellFrame>(fr);
    A.gp = dptr<ShellGP>(gp);
    A.dedU = dptr<double>(de);
    A.Kf = dptr<double>(kf);
    A.K = (buildMat && !d_ke) ? dptr<double>(ctx->d_K64) : nullptr;
    A.load = d_loadInt;
    A.intLoad = d_intLoad;
    A.intMat = (buildMat && !d_ke) ? dptr<double>(ctx->d_intMat) : nullptr;
    A.keOut = d_ke;
    A.ruOut = d_ru;
    cudaStream_t s = ctx->stream;
    for (int col = 0; col < P.ncolors; ++col) {
        const int cnt = P.colorPtr[col + 1] - P.colorPtr[col];
        if (!cnt) continue;
        A.els = dptr<int>(ctx->d_colorEls) + P.colorPtr[col];
        A.count = cnt;
        k_shell_frame<<<(cnt + 63) / 64, 64, 0, s>>>(A);
        k_shell_gauss<<<(4 * cnt + 127) / 128, 128, 0, s>>>(A);
        k_shell_dedu<<<(128 * cnt + 127) / 128, 128, 0, s>>>(A);
        k_shell_kcol<<<(32 * cnt + 127) / 128, 128, 0, s>>>(A);
        k_shell_condense<<<(cnt + 63) / 64, 64, 0, s>>>(A);
    }
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    dev_free(fr);
    dev_free(gp);
    dev_free(de);
    dev_free(kf);
    return cuda_check(ctx, e, "shell pipeline");
}
