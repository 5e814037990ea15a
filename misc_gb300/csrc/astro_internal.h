// Internal state of the GB300 library behind include/astro_gpu.h.
//
// Data layout in HBM (one context = one model on one GPU):
//   * nodes are renumbered by the reference's breadth-first ordering (currentRank); all device
//     vectors are node-major by rank: x[(rank-1)*dpn + c], dpn = DOF per node (3 solid, 6 shell);
//   * the stiffness lives as a block-CSR (BSR) matrix over node ranks with dpn x dpn row-major
//     blocks, block columns sorted by rank; FP64 values (faithful path) and/or FP32 values
//     (mixed-precision path);
//   * elements are stored in colour-major order: elements of one colour share no node, so a
//     colour's element matrices are added into the BSR without atomics (deterministic);
//   * the reference's scalar CSR (component-major DOF numbering, find-or-insert column order) is
//     produced only on export through a per-block position table.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <functional>
#include <string>
#include <vector>

#include "../../include/astro_gpu.h"

#define ASTRO_MAX_COLORS 64

struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
};

template <class T> static inline T *dptr(DevBuf &b) { return reinterpret_cast<T *>(b.p); }

struct AstroPrep {
    // reference analysisPrep outputs (1-based values, as the Fortran)
    int N = 0, E = 0, dpn = 0, n = 0;
    int solverMaxBW = 0;
    std::vector<int> currentRank, originalRank, nDofIndex;  // nDofIndex(6,N)
    std::vector<int> elMatRange, elMatLTRange;
    int elMatSize = 0, ltSize = 0;
    std::vector<int> intVecRange, intMatRange;
    int intVecSize = 0, intMatSize = 0;
    // node adjacency in the reference's first-seen order (nodalConn without empty slots)
    std::vector<int> adjPtr, adj;  // 1-based node ids
    // block CSR over ranks (0-based)
    std::vector<int> bRowPtr, bCol;
    int nb = 0;
    // per element: block index of local node pair (a,b), npe x npe
    int npe = 0;
    std::vector<int> elBlk;
    // colouring
    int ncolors = 0;
    std::vector<int> colorPtr, colorEls;  // colorEls: 0-based element ids grouped by colour
    // bit (a*npe+b) of elFirst[e]: element e is the first (in colour order) to touch block (a,b)
    std::vector<unsigned long long> elFirst;
    // reference CSR position of each (block, column component): elMatRange(dof-1) excluded, i.e.
    // position within the row, 0-based; size nb*dpn
    std::vector<int> csrPosInRow;
    // constraints (reference DOF numbering, 1-based columns, 0 = empty slot)
    int mpcDim = 0, mpcSize = 0;
    std::vector<int> mpcRange, mpcCols;
    std::vector<double> mpcMat, mpcRhs;
};

struct HostStage;  // hostcopy.cu: page-locked staging of large pageable copies

struct astro_ctx {
    std::string err;
    // workspaces of the static solvers (FP64, mixed, learned), kept with their restart-cycle graphs
    // across solves; owned by the Krylov unit (krylov_release)
    void *solveWork[3] = {nullptr, nullptr, nullptr};
    int unrolledCycles = 0;  // ASTRO_OPT_UNROLLED_CYCLES
    cudaStream_t stream = nullptr;
    cudaStream_t stream2 = nullptr;  // copies that overlap the element kernels
    // the FP32 assembly pass (one launch per colour) captured once as a graph and replayed
    cudaGraph_t asmGraph = nullptr;
    cudaGraphExec_t asmExec = nullptr;
    int device = 0;
    AstroPrep P;
    // host model copy
    std::vector<double> nodes;  // (N,3)
    std::vector<int> elist;     // (E,8)
    std::vector<int> etype, esec;
    std::vector<double> elMat;  // per element materialElastic(9) (solids)
    std::vector<double> elDensity;  // per element materialDensity (solids)
    std::vector<int> elMatId;       // per element material (solids, 1-based)
    std::vector<int> layMat;        // per layup layer material (shells, 1-based)
    // thermal path (thermal.cu), opaque
    void *thermal = nullptr;
    std::vector<double> secABD, secMass;  // per section ABD(9,9), sMass(6,6) (shells)
    std::vector<double> secOrient;        // per section 3x3 column-major
    std::vector<double> elThickness;      // per element total shell thickness (complex step / loads)
    int hasShell = 0, hasSolid = 0;
    int orientIdentity = 1;
    // device model
    DevBuf d_nodes, d_elist, d_elMat, d_esec, d_secABD, d_secOrient, d_colorEls, d_elBlk;
    DevBuf d_elC;           // per brick element the orthotropic C (C11 C12 C13 C22 C23 C33 C44 C55 C66)
    DevBuf d_elXdf, d_elCdf;  // per brick element: node coordinates (section frame) and C in double-float
    DevBuf d_rank;          // currentRank (N) 1-based
    DevBuf d_bRowPtr, d_bCol, d_bRow, d_etype, d_elFirst;
    DevBuf d_K64, d_K32;    // BSR values
    int haveK64 = 0, haveK32 = 0;
    int haveIntMat = 0;      // d_intMat holds the condensed internal rows of the last FP64 assembly
    // solver copies in slot-major block-ELL layout: entry q of the s-th block of block row r at
    // (s*dpn*dpn + q)*ellLd + r, its block column at d_ellCol[s*ellLd + r] (empty slots: the row
    // itself with zero values)
    DevBuf d_K64p, d_K32p, d_ellCol;
    int ellSlots = 0, ellLd = 0;
    int k64Version = 0, k32Version = 0, k64PlanesVersion = -1, k32PlanesVersion = -1;
    DevBuf d_csrPos, d_elMatRangeRank;  // export tables
    DevBuf d_intMat;        // condensed internal rows (shell), E*256 doubles
    DevBuf d_shFr, d_shGp, d_shDe, d_shKf;  // shell pipeline scratch for shScratchEls elements
    int shScratchEls = 0;
    // constraints on device (internal DOF numbering)
    DevBuf d_mpcRange, d_mpcCol, d_mpcVal, d_mpcRhs, d_mpcT;  // scaled, after astro_scale_mpc
    DevBuf d_mpcGPtr, d_mpcGTerm, d_mpcGRow, d_mpcTermRow;      // constraint load gather lists
    int mpcTargets = 0;
    int mpcScaled = 0;
    // penalty C^T C as CSR over internal rows (host-built after scaling)
    DevBuf d_penRow, d_penPtr, d_penCol, d_penVal;
    int penRows = 0;
    int penVersion = 0;  // incremented whenever the penalty lists are rebuilt (astro_scale_mpc)
    std::vector<int> penI, penJ;  // the same entries on the host (internal row, internal column)
    std::vector<double> penV;
    // batched panel factorisation (panels.cu), opaque
    void *panels = nullptr;
    std::vector<double> mpcScaledHost, mpcRhsScaledHost;
    // skyline (reference DOF numbering) on device
    DevBuf d_ltRange, d_lt;
    int haveLT = 0, ltFactored = 0;
    // design variables (host copies of the model's maps) and, for shells, the section inputs kept
    // on the device for the complex-step property evaluation
    int numDvars = 0;
    std::vector<int> e2dRange, e2d, dCat, dComp, dLayer;
    std::vector<double> e2c, dVal;
    DevBuf d_shLayRange, d_shLay, d_shZoff, d_e2dR, d_e2d, d_e2c, d_dCat, d_dLayer, d_dVal;
    // persistent buffers of the getElasticSolnLoad boundary: load vector in both numberings,
    // exported CSR values and column numbers
    DevBuf d_ioRef, d_ioInt, d_exMat, d_exCols;
    HostStage *stage = nullptr;
    DevBuf d_sky[5];  // grow-only scratch of the host-buffer skyline entry points
    // scratch
    DevBuf d_scratch;
    DevBuf d_status;  // int status words written by kernels
    DevBuf d_guard;   // checked build: site of the first failed index guard (bounds.cuh), else 0
    // solid meshes: the colour-grouped element lists split by type (brick8, brickIM), the
    // internal-DOF offsets (intVecRange, intMatRange) and the per-element density on the device
    std::vector<int> c8Els, c8Ptr, c81Els, c81Ptr;
    DevBuf d_c8Els, d_c81Els, d_intVecOff, d_intMatOff, d_elRho;
    int has81 = 0;
    // node design-variable maps (ndToD) and the activity windows of nodeLoad variables; the
    // section orientations as given (the complex step rotates them itself)
    std::vector<int> n2dRange, n2d;
    std::vector<double> n2c, dActTime;
    DevBuf d_n2dR, d_n2d, d_n2c, d_dComp, d_secOrig;
    int quirkShellMeanRot = 0;
    int bandFp64Update = 1;  // ASTRO_OPT_BAND_FP64_UPDATE
    // launch shapes picked by astro_autotune (0: the default)
    int tuneHex8Warps = 0;   // zero-state brick kernel: warps per CTA (1, 2, 4)
    int tuneCasesCluster = 0;  // many-column band solve: CTAs per cluster (2, 4, 8)
    int casesTwist = 1;        // ASTRO_OPT_CASES_TWIST
    int panelsSolve = 0;       // ASTRO_OPT_PANELS_SOLVE
    int tunePanelCluster = 0;  // band factorisation: CTAs per cluster (2, 4, 8)
};

// error helpers
int set_err(astro_ctx *c, int code, const std::string &msg);
int cuda_check(astro_ctx *c, cudaError_t e, const char *what);
int guard_status(astro_ctx *c, const char *what);
#define CK(call)                                                  \
    do {                                                          \
        cudaError_t e__ = (call);                                 \
        if (e__ != cudaSuccess) return cuda_check(ctx, e__, #call); \
    } while (0)

int dev_alloc(astro_ctx *c, DevBuf &b, size_t bytes);
void dev_free(DevBuf &b);
int upload(astro_ctx *c, DevBuf &b, const void *h, size_t bytes);

// host analysis preparation (prep.cpp)
int astro_prep_build(astro_ctx *c, const astro_model *m);

// kernels' host entry points
int launch_hex8_assemble(astro_ctx *ctx, int precision, int store);           // elem_hex8.cu
int hex8_prepare(astro_ctx *ctx);  // per-element material stiffness, once per context (elem_hex8.cu)
int launch_hex8_element_mats(astro_ctx *ctx, int precision, double *ke_host); // elem_hex8.cu
// device state of an element evaluation (internal layout: nodal vectors rank-major, dpn per node;
// internal-DOF vectors in intVecRange order; any pointer may be null = zeros)
struct ElemDevState {
    const double *disp = nullptr, *pdisp = nullptr, *pvel = nullptr, *pacc = nullptr;
    const double *idisp = nullptr, *pidisp = nullptr;
    int dynamic = 0;
    double beta = 0.25, gamma = 0.5, delT = 0.0;
    int massOnly = 0;  // residual = the Newmark mass term alone (needs dynamic, no matrix)
};
int launch_shell4_assemble(astro_ctx *ctx, const ElemDevState &s, double *d_loadInt, double *d_intLoad,
                           int buildMat, double *d_ke, double *d_ru, bool sync = true);  // elem_shell4.cu
int shell_sections_prepare(astro_ctx *ctx, const astro_model *m);          // elem_shell4.cu
int shell4_residual_list(astro_ctx *ctx, const ElemDevState &st, const int *d_els, const std::vector<int> &ptr,
                         double *d_loadInt);                                 // elem_shell4.cu
int shell4_drdd_list(astro_ctx *ctx, int dvar, double h, const ElemDevState &st, const std::vector<int> &list,
                     const std::vector<int> &ptr, double *d_acc, double *d_intAcc,
                     const std::function<int(const int *, int)> &hook);     // elem_shell4.cu
int shell4_update_external_rhs(astro_ctx *ctx, const double *d_intVec, double *d_extInt);          // elem_shell4.cu
int shell4_update_internal_soln(astro_ctx *ctx, const double *d_extInt, double *d_intSoln,
                                const double *d_intRhs);                                           // elem_shell4.cu
void panels_release(astro_ctx *ctx);                                         // panels.cu
int panels_cases_prepare(astro_ctx *ctx, int ncols, size_t *bytes);         // panels.cu
int precond_node_features(astro_ctx *ctx, int kind, double *dF, DevBuf &L, DevBuf &pd, DevBuf &part,
                          cudaStream_t s);                                  // precond.cu
int precond_mlp_check(astro_ctx *ctx, const astro_precond_mlp *m, int degree);
int precond_mlp_scales_f32(astro_ctx *ctx, const astro_precond_mlp *m, const double *dF, DevBuf &prm, float *a,
                           cudaStream_t s);
int ensure_K(astro_ctx *ctx, int which);          // device BSR value arrays (ctx.cu)
int ensure_io(astro_ctx *ctx, bool exportMat);    // host-vector staging buffers (ctx.cu)
int panels_cases_solve(astro_ctx *ctx, double *d_vec, cudaStream_t s);      // panels.cu
int panels_cases_columns(astro_ctx *ctx);
int panels_cases_launches(astro_ctx *ctx);                                   // panels.cu
int panels_cases_would_twist(astro_ctx *ctx);                                // panels.cu
int panels_factor_impl(astro_ctx *ctx, int32_t cluster_size, astro_panels_info *info, int factor);  // panels.cu
void panels_shape(astro_ctx *ctx, int *np, int *bw, long long *bandBytes, double *factorSeconds);
void thermal_release(astro_ctx *ctx);                                        // thermal.cu
int bsr_zero(astro_ctx *ctx, int which);                                    // assemble.cu
int export_csr_dev(astro_ctx *ctx, cudaStream_t s, double *d_mat, int *d_cols);  // assemble.cu
double bsr_absmax(astro_ctx *ctx, int *status, int kind);                   // assemble.cu
int constraint_load_dev(astro_ctx *ctx, const double *d_u, double *d_loadInt);  // assemble.cu
int ref_to_int_vec(astro_ctx *ctx, const double *d_ref, double *d_int, int n); // assemble.cu
int int_to_ref_vec(astro_ctx *ctx, const double *d_int, double *d_ref, int n); // assemble.cu
// hostcopy.cu: large pageable copies through page-locked staging, complete on return
int copy_to_device(astro_ctx *ctx, void *dst, const void *src, size_t bytes, const char *what);
int copy_to_host(astro_ctx *ctx, void *dst, const void *src, size_t bytes, const char *what);
void host_stage_release(astro_ctx *ctx);
int krylov_residual64(astro_ctx *ctx, const double *d_x, const double *d_b, double *d_r);  // krylov.cu
int surface_load_dev(astro_ctx *ctx, int nf, const int *d_faceEl, const int *d_faceNum, const double *tr,
                     double pressure, double *d_loadInt);                   // assemble.cu
// Solid elements (brick8 and brickIM), colour by colour, at state s: load -= Ru into d_loadInt
// (nodal, internal layout) and d_intLoad (internal DOF); with build = 1 the tangent (K, plus
// c1 c2 M when s.dynamic) goes into the FP64 block-CSR matrix and the condensed internal rows of
// the brickIM elements into d_intMat, or, when d_ke is given, the condensed element matrices
// into d_ke (E x 24 x 24) instead; d_ru receives the element residuals (E x 24).
int solid_soln_load(astro_ctx *ctx, int build, const ElemDevState &s, double *d_loadInt, double *d_intLoad,
                    double *d_ke, double *d_ru);                                                   // elem_hex8.cu
int hex81_run(astro_ctx *ctx, const int *d_list, const std::vector<int> &ptr, int build, double *K,
              const ElemDevState &st, const double *CItem, double gpc, double *d_loadInt, double *d_intLoad,
              double *d_intMat, double *d_ke, double *d_ru);                                       // elem_hex81.cu
int hex81_update_external_rhs(astro_ctx *ctx, const double *d_intVec, double *d_extInt);          // elem_hex81.cu
int hex81_update_internal_soln(astro_ctx *ctx, const double *d_extInt, double *d_intSoln,
                               const double *d_intRhs);                                            // elem_hex81.cu
// getElasticSolnLoad on device vectors for any mesh (ctx.cu): load -= Ru, and with build = 1 the
// FP64 block-CSR tangent (zeroed first for shells; the solid kernels write every block first)
int elem_soln_load_dev(astro_ctx *ctx, const ElemDevState &s, double *d_loadInt, double *d_intLoad, int build,
                       bool sync);
// updateExternalRHS / updateInternalSoln of the context's elements with internal DOF (shell4 or
// brickIM), device vectors in internal layout (ctx.cu)
int elem_update_external_rhs(astro_ctx *ctx, const double *d_intVec, double *d_extInt);
int elem_update_internal_soln(astro_ctx *ctx, const double *d_extInt, double *d_intSoln, const double *d_intRhs);
// Complex-step residual sensitivity of the elements that depend on design variable dvar:
// d_acc -= Im(Ru(d + i h)) accumulated in colour order (internal layout; shells also d_intAcc).
int solid_drdd(astro_ctx *ctx, int dvar, double h, const ElemDevState &s, double *d_acc,
               double *d_intAcc);                                                                   // elem_solid_cstep.cu
// design variables d0 .. d0+nd-1 into d_acc + (d-d0) n, d_intAcc + (d-d0) ni
int solid_drdd_batch(astro_ctx *ctx, int d0, int nd, double h, const ElemDevState &s, double *d_acc,
                     double *d_intAcc);  // elem_solid_cstep.cu
// per-element orientation of solid meshes with orientation design variables (r_getOrientation's
// rotation of the section frame by their real values), into d_secOrient (elem_solid_cstep.cu)
int solid_orient_prepare(astro_ctx *ctx);
int shell4_drdd(astro_ctx *ctx, int dvar, double h, const ElemDevState &s, double *d_acc,
                double *d_intAcc);                                                              // elem_shell4.cu
void krylov_release(astro_ctx *ctx);
// per-step device histories of the time loop (reference numbering; any may be null)
struct NewmarkHist {
    double *disp = nullptr, *vel = nullptr, *acc = nullptr, *intDisp = nullptr;
};
int krylov_newmark(astro_ctx *ctx, const astro_newmark_opts *o, const double *d_pattern, const double *h_amp,
                   double *d_u, double *d_up, double *d_vp, double *d_ap, double *d_iu, double *d_iup,
                   const NewmarkHist &hist, astro_solve_stats *st);  // krylov.cu
// host: elements depending on dvar, grouped by colour (colour c: list[ptr[c] .. ptr[c+1]))
void dvar_elements_by_colour(const astro_ctx *ctx, int dvar, std::vector<int> &list, std::vector<int> &ptr);
