/*
 * astro_gpu.h -- C ABI of the GB300 (sm_103a) implementation of AStrO's structural hot path:
 * element stiffness/residual evaluation (brick8 solids, shell4 shells, real and complex-step),
 * global assembly, and the linear solve (row-skyline LDL^T factor/solve, restarted GMRES).
 *
 * The entry points mirror the Fortran subroutines that AStrO_runJob drives, so a thin
 * iso_c_binding shim can route those subroutines here.  Conventions follow the reference:
 *   - node, element, section, material and DOF numbers are 1-based, as in the Fortran;
 *   - "range" arrays are prefix sums with lower bound 0 (Fortran ARange(0:n)), passed as a
 *     pointer to element 0;
 *   - 2-D arrays are column-major (nodeList(3,N) is x1,y1,z1,x2,...);
 *   - a CSR column index of 0 marks an unused slot and is skipped;
 *   - the global DOF numbering is the reference's component-major nDofIndex.
 * Every function returns ASTRO_OK (0) or a positive ASTRO_ERR_* code; astro_last_error() gives
 * the message.  One host thread per context; calls are synchronous at return.
 */
#ifndef ASTRO_GPU_H
#define ASTRO_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ASTRO_OK 0
#define ASTRO_ERR_ARG 1          /* bad argument or size */
#define ASTRO_ERR_CUDA 2         /* CUDA runtime error (message has the CUDA error string) */
#define ASTRO_ERR_UNSUPPORTED 3  /* element type / mesh mix not handled by this library */
#define ASTRO_ERR_PIVOT 4        /* zero or non-finite pivot in an LDL^T or LU factorisation */
#define ASTRO_ERR_NAN 5          /* non-finite value in a vector or residual */
#define ASTRO_ERR_BREAKDOWN 6    /* Krylov breakdown (zero Arnoldi vector norm) */
#define ASTRO_ERR_MAXIT 7        /* iteration limit reached before the tolerance */
#define ASTRO_ERR_STATE 8        /* call out of order (e.g. solve before factorisation) */
#define ASTRO_ERR_NOMEM 9        /* device allocation failed */
#define ASTRO_ERR_BOUNDS 10      /* library built with ASTRO_BOUNDS_CHECK only: a device index guard
                                    found an index outside its buffer and skipped the access */

/* Design-variable categories (reference dCategory / dSubCat, Working/AStrO_r_designPropertyFunctions.f90).
 * Element categories enter through el_to_d, node categories through nd_to_d. */
#define ASTRO_DCAT_LAYUP_THICKNESS 1   /* 'layup' / 'thickness' of layer d_layer (:242, :299) */
#define ASTRO_DCAT_ELASTIC_MODULUS 2   /* 'elastic' / 'modulus': materialElastic entry d_component (1..9) (:46) */
#define ASTRO_DCAT_DENSITY 3           /* 'density': solid material density (r_getMaterialDensity, :98) */
#define ASTRO_DCAT_ORIENTATION 4       /* 'orientation': component d_component (1..3) of the local rotation
                                          vector applied to the section orientation (r_getOrientation, :203) */
#define ASTRO_DCAT_LAYUP_ZOFFSET 5     /* 'layup' / 'zOffset' of the section (r_getElThickOffset, :252) */
#define ASTRO_DCAT_LAYUP_ANGLE 6       /* 'layup' / 'angle' of layer d_layer, radians (:301) */
#define ASTRO_DCAT_LAYUP_DENSITY 7     /* 'layup' / 'density' of layer d_layer (r_getShellMass, :505) */
#define ASTRO_DCAT_NODE_COORD 8        /* 'nodeCoord': coordinate d_component (1..3) of the nodes of nd_to_d
                                          (r_getNodeCoord, :945-968) */
#define ASTRO_DCAT_NODE_LOAD 9         /* 'nodeLoad' / 'elastic': nodal load component d_component (1..6) at the
                                          nodes of nd_to_d while d_act_time[0] < t < d_act_time[1]
                                          (r_getNodeDLoad, :970-994); d_component 7 = 'nodeLoad' / 'thermal',
                                          the nodal heat input ndLd(7) */
#define ASTRO_DCAT_THERMAL_COND 10     /* 'thermalCond': materialThermCond entry d_component (1..6: k11 k22 k33
                                          k12 k13 k23) of a solid (r_getMaterialThermCond, :129-161) */
#define ASTRO_DCAT_SPEC_HEAT 11        /* 'specHeat': solid specific heat (r_getMaterialSpecHeat, :164-186) */
#define ASTRO_DCAT_LAYUP_THERMAL_COND 12 /* 'layup' / 'thermalCond': conductivity entry d_component (1..6) of layer
                                            d_layer (r_getShellThermCond, :556) */
#define ASTRO_DCAT_LAYUP_SPEC_HEAT 13  /* 'layup' / 'specHeat' of layer d_layer (r_getShellSpecHeat, :630) */
#define ASTRO_DCAT_LAYUP_MODULUS 14    /* 'layup' / 'modulus', 'poissonRatio', 'shearModulus' of layer d_layer
                                          (r_getShellStiffness, :289-303): d_component indexes the layer's
                                          (E1, E2, nu12, G12), 1..4; poissonRatio is component 3 and
                                          shearModulus component 4, as the reference maps them */

/* Model arrays: the reference's module globals (Working/AStrO_globalData.f90) as flat arrays.
 * Element types: 8 = brick8 (2x2x2 Gauss), 81 = brickIM (brick8 plus three incompatible bubbles,
 * 9 condensed internal DOF), 41 = shell4 (4 Gauss points, 8 condensed incompatible-mode DOF);
 * solid (8, 81) and shell elements are not mixed in one model.  Constraints are given as expanded equations: equation k has terms
 * mpc_range[k-1]..mpc_range[k]-1 (0-based term index), each term (node, dof, coef). */
typedef struct astro_model {
    int32_t num_nodes;
    int32_t num_els;
    const double *node_list;        /* nodeList(3,num_nodes) */
    const int32_t *element_list;    /* elementList(8,num_els), 0 = unused slot */
    const int32_t *element_type;    /* elementType(num_els) */
    const int32_t *element_section; /* elementSection(num_els) */
    int32_t num_sections;
    const int32_t *section_mat_id;  /* sectionMatId(num_sections): solid sections */
    const double *section_orient;   /* sectionOrient(3,3*num_sections): rows are local axes */
    const int32_t *sec_layup_range; /* secLayupRange(0:num_sections) */
    const int32_t *layup_mat_id;    /* layupMatId(num_layers) */
    const double *layup_thickness;  /* layupThickness(num_layers) */
    const double *layup_angle;      /* layupAngle(num_layers), radians */
    const double *section_z_offset; /* sectionZOffset(num_sections) */
    int32_t num_materials;
    const double *material_elastic; /* materialElastic(9,num_materials): E1 E2 E3 nu12 nu13 nu23 G12 G13 G23 */
    const double *material_density; /* materialDensity(num_materials) */
    int32_t num_mpc;                /* number of constraint equations (elMPCDim) */
    const int32_t *mpc_range;       /* (0:num_mpc) prefix sums over terms */
    const int32_t *mpc_node;        /* node per term */
    const int32_t *mpc_dof;         /* DOF component 1..6 per term */
    const double *mpc_coef;         /* coefficient per term */
    const double *mpc_rhs;          /* right-hand side per equation */
    int32_t num_dvars;              /* design variables (0 if none) */
    const int32_t *el_to_d_range;   /* elToDRange(0:num_els) */
    const int32_t *el_to_d;         /* elToD: design variable per entry */
    const double *el_to_coef;       /* elToCoef */
    const int32_t *d_category;      /* ASTRO_DCAT_* per design variable */
    const int32_t *d_component;     /* dComponent */
    const int32_t *d_layer;         /* dLayer */
    const double *d_value;          /* r_dVec */
    const int32_t *nd_to_d_range;   /* ndToDRange(0:num_nodes), or NULL (no node design variables) */
    const int32_t *nd_to_d;         /* ndToD: design variable per entry */
    const double *nd_to_coef;       /* ndToCoef */
    const double *d_act_time;       /* dActTime(2, num_dvars): activity window of nodeLoad variables, or NULL
                                       (always active) */
} astro_model;

/* Sizes produced by analysis preparation (reference analysisPrep, Working/AStrO_bookKeeping.f90:794). */
typedef struct astro_dims {
    int32_t el_mat_dim;      /* elMatDim: number of global DOF */
    int32_t el_mat_size;     /* elMatSize: CSR slots of the stiffness matrix */
    int32_t el_mat_lt_size;  /* elMatLTSize: row-skyline size */
    int32_t el_mpc_dim;      /* constraint equations */
    int32_t el_mpc_size;     /* constraint terms */
    int32_t int_vec_size;    /* intVecSize: condensed internal DOF */
    int32_t int_mat_size;    /* intMatSize */
    int32_t solver_max_bw;   /* solverMaxBW (node-rank bandwidth cap of the skyline profile) */
    int32_t dof_per_node;    /* 3 (solid mesh) or 6 (shell mesh) */
    int32_t num_blocks;      /* node-block nonzeros of the internal block-CSR matrix */
    int32_t num_colors;      /* element colours (launches per assembly pass) */
} astro_dims;

/* Nodal state in global DOF numbering (length el_mat_dim) and internal-DOF state (int_vec_size).
 * Any pointer may be NULL (= zeros). */
typedef struct astro_state {
    const double *node_disp, *node_vel, *node_acc;
    const double *prev_disp, *prev_vel, *prev_acc;
    const double *internal_disp, *prev_int_disp;
    int32_t dynamic;         /* 1: add Newmark inertia (r_getElRu dynamic branch) */
    double nm_beta, nm_gamma, del_t;
} astro_state;

/* Polynomial graph-convolution preconditioner of the learned solver (no counterpart in the
 * reference, whose gMRes is preconditioned by a diagonal).  With D the diagonal of
 * A = K + C^T C, lambda = lambda_scale times a power-iteration estimate of the largest
 * eigenvalue of D^-1 A, and xi(mu) = (2 mu / lambda - (1 + 1/ratio)) / (1 - 1/ratio) the map
 * of [lambda/ratio, lambda] onto [-1, 1], the preconditioner is
 *     P v = (1/lambda) sum_{k=0..degree} W_k T_k(xi(D^-1 A)) D^-1 v
 * with T_k the Chebyshev polynomials (one sparse matrix-vector product per hop) and W_k one
 * dpn x dpn weight per hop, shared by all nodes: a linear graph network on the mesh whose node
 * features are the DOF of a node.  weights[(k * dpn + i) * dpn + j] = W_k[i][j]. */
#define ASTRO_PRECOND_MAX_DEGREE 32
typedef struct astro_precond {
    int32_t degree;          /* 1..ASTRO_PRECOND_MAX_DEGREE */
    int32_t dpn;             /* DOF per node of the model the weights are for (3 or 6) */
    double ratio;            /* lambda_max / lambda_min of the fitted interval (> 1) */
    double lambda_scale;     /* safety factor on the eigenvalue estimate (>= 1) */
    double weights[(ASTRO_PRECOND_MAX_DEGREE + 1) * 36];
} astro_precond;

/* Per-node modulation of the polynomial network: the learned part that sees the model.
 * Node features f(r), ASTRO_NODE_FEATURES per node, from the assembled A = K + C^T C (no element
 * data, so any element family): with d_r the mean diagonal entry of node r's diagonal block of K,
 * l_r = ln d_r and lbar the mean of l over the nodes,
 *   f0 = l_r - lbar                               (the node's stiffness level)
 *   f1 = mean over the neighbours c of (l_c - l_r)  (local contrast, e.g. of log E)
 *   f2 = max over the neighbours of |l_c - l_r|
 *   f3 = (neighbours + 1) / (most blocks of a row)  (interior, face, edge, corner)
 *   f4 = ln(1 + p_r / d_r), p_r the mean penalty diagonal of the node's DOF (constraints)
 *   f5 = ln(sum_{c != r} ||K_rc||_F / ||K_rr||_F)  (diagonal dominance)
 * A two-layer perceptron maps them to per-node hop scales
 *   a_k(r) = 1 + b2[k] + sum_h w2[k * hidden + h] tanh(b1[h] + sum_f w1[h * F + f] f_f(r))
 * and the preconditioner becomes P v = (1/lambda) sum_k a_k(r) (W_k y_k)(r) at every node r.
 * With w2 = b2 = 0 it is the polynomial network unchanged.  hidden = 0: no modulation.
 * No counterpart in the reference (whose gMRes is preconditioned by a diagonal). */
#define ASTRO_NODE_FEATURES 6
#define ASTRO_MLP_MAX_HIDDEN 32
typedef struct astro_precond_mlp {
    int32_t hidden;   /* 0..ASTRO_MLP_MAX_HIDDEN */
    int32_t outputs;  /* degree + 1 of the network it modulates */
    double w1[ASTRO_MLP_MAX_HIDDEN * ASTRO_NODE_FEATURES];
    double b1[ASTRO_MLP_MAX_HIDDEN];
    double w2[(ASTRO_PRECOND_MAX_DEGREE + 1) * ASTRO_MLP_MAX_HIDDEN];
    double b2[ASTRO_PRECOND_MAX_DEGREE + 1];
} astro_precond_mlp;

/* Options and statistics of the spec solvers (astro_solve_static). */
#define ASTRO_SOLVER_GMRES_JACOBI_FP64 0   /* plain FP64 Jacobi-GMRES(m): the comparator */
#define ASTRO_SOLVER_FGMRES_MIXED 1        /* FP32 inner Jacobi-GMRES, FP64 refinement */
#define ASTRO_SOLVER_FGMRES_LEARNED 2      /* FP32 inner GMRES right-preconditioned by the
                                              polynomial network, FP64 refinement */
typedef struct astro_solve_opts {
    int32_t method;          /* ASTRO_SOLVER_* */
    int32_t restart;         /* Krylov basis size m (50) */
    int32_t max_iters;       /* total inner iterations cap */
    double rtol;             /* target ||b - A x||_2 / ||b||_2 in FP64 with A = K + C^T C */
    double inner_rtol;       /* inner relative tolerance for the refinement methods */
    const astro_precond *precond;  /* ASTRO_SOLVER_FGMRES_LEARNED: the network (NULL: the
                                      Chebyshev initialisation of degree 24, ratio 3000) */
    const astro_precond_mlp *mlp;  /* ASTRO_SOLVER_FGMRES_LEARNED: its per-node modulation (NULL:
                                      none); outputs must equal the network's degree + 1 */
} astro_solve_opts;

typedef struct astro_solve_stats {
    int32_t iterations;      /* total inner (Arnoldi) iterations */
    int32_t restarts;        /* restart cycles */
    int32_t refinements;     /* FP64 refinement steps */
    int32_t status;          /* ASTRO_OK or error code */
    double rel_residual;     /* final FP64 true relative residual */
    double seconds;          /* device time of the solve, CUDA events */
    int32_t conditional_graph;  /* 1: the restart cycles ran as CUDA graphs whose Arnoldi steps sit
                                   behind conditional nodes (skipped after convergence); 0: the
                                   unrolled graph (the driver refused conditional nodes) */
    int32_t fallback;        /* learned solver: 1 when it ended in a non-finite value, a breakdown or
                                the iteration cap and the FP32 Jacobi solver finished the solve from
                                the initial guess (the counts and seconds then cover both) */
    int32_t residual_kind;   /* the matrix values rel_residual was formed with: 64 = the FP64
                                assembly (astro_el_soln_load), the system the tolerance refers to;
                                32 = only the FP32 assembly was resident (astro_assemble_fp32 alone),
                                so rel_residual is that of the FP32-rounded system, computed in FP64
                                arithmetic; 0 = no solve ran */
} astro_solve_stats;

typedef struct astro_ctx astro_ctx;

/* ---- context ------------------------------------------------------------------------------ */

/* Builds the context: uploads the model, runs analysis preparation (node reordering, DOF map,
 * CSR/skyline structure, constraint matrix, element colouring and scatter maps) and keeps all
 * device mirrors until astro_ctx_destroy.  Replaces analysisPrep
 * (Working/AStrO_bookKeeping.f90:794-1039) together with the model upload. */
int astro_ctx_create(const astro_model *model, astro_ctx **out);
int astro_ctx_destroy(astro_ctx *ctx);
/* Copies the last error message of ctx (or of the last failed astro_ctx_create when ctx is
 * NULL) into buf (NUL-terminated, at most len bytes). */
int astro_last_error(const astro_ctx *ctx, char *buf, int32_t len);

/* Host-only variant of the analysis preparation (no GPU needed), for inspection and tests:
 * fills dims and, when non-NULL, currentRank(num_nodes), nDofIndex(6,num_nodes),
 * elMatRange(0:n), elMatLTRange(0:n), the exported CSR column numbers el_mat_cols[el_mat_size]
 * (the order astro_el_soln_load produces) and the number of element colours.  No counterpart in
 * the reference beyond analysisPrep itself (Working/AStrO_bookKeeping.f90:794-1039). */
int astro_prep_host(const astro_model *model, astro_dims *dims, int32_t *current_rank,
                    int32_t *n_dof_index, int32_t *el_mat_range, int32_t *el_mat_lt_range,
                    int32_t *el_mat_cols, int32_t *num_colors);

int astro_get_dims(const astro_ctx *ctx, astro_dims *out);
/* Behaviour switches.  ASTRO_OPT_SHELL_MEAN_ROT_TERM (default 0 = the reference): when 1, the
 * shell4 rotation derivative also carries the dependence of the element mean rotation on each
 * nodal rotation, which r_getInstDof (Working/AStrO_r_elementEqns.f90:835-858) omits; with it the
 * tangent is invariant under rigid rotations.  No counterpart in the reference. */
#define ASTRO_OPT_SHELL_MEAN_ROT_TERM 1
/* ASTRO_OPT_UNROLLED_CYCLES (default 0): when 1, the static solvers capture their restart cycles
 * as m unrolled Arnoldi steps (kernels that return at once after convergence) instead of
 * conditional graph nodes; the same kernels in the same order, so the results are identical.
 * For profilers that do not look inside conditional nodes, and for drivers without them. */
#define ASTRO_OPT_UNROLLED_CYCLES 2
/* ASTRO_OPT_BAND_FP64_UPDATE (default 1): the band LDL^T of astro_panels_factor (and of
 * astro_newmark_cases) runs its trailing tile updates in FP64 arithmetic; 0 selects the
 * tensor-core emulation on tcgen05 (BF16 slices of the Ozaki error-free splitting, summed exactly
 * in FP32 per level in tensor memory and combined in FP64; 56 bits relative to each row's largest
 * entry), 2 the same emulation on mma.sync (identical results), 3 the whole factorisation in
 * double-float arithmetic on the FP32 pipe (the band converted in place to float pairs and back;
 * about 48 significant bits per operation): a factor of lower precision for solves that refine
 * against the FP64 operator (astro_panels_solve's default mode). */
#define ASTRO_OPT_BAND_FP64_UPDATE 3
/* The launch shapes astro_autotune picks, set directly (0 = the default): the zero-state brick
 * kernel's warps per CTA (1, 2, 4), the band factorisation's and the many-column band solve's
 * CTAs per cluster (2, 4, 8). */
#define ASTRO_OPT_BRICK_WARPS 4
#define ASTRO_OPT_PANEL_CLUSTER 5
#define ASTRO_OPT_CASES_CLUSTER 6
/* ASTRO_OPT_CASES_TWIST (default 1): the many-column band solve of astro_newmark_cases on a
 * single panel runs twisted: the band split into a top and a reversed bottom half that meet in a
 * window of bandwidth-many block rows, both halves swept at once towards the window and back, so
 * the sequential chain is about half as long.  0: off; 1: when the panel has at least 8 windows
 * of block rows; 2: whenever the split is possible (for tests on small models). */
#define ASTRO_OPT_CASES_TWIST 7
/* ASTRO_OPT_PANELS_SOLVE (default 0): astro_panels_solve runs its forward and backward sweeps in
 * double-float arithmetic on the FP32 pipe (about 48 significant bits per operation) from
 * double-float copies of the FP64 factor, made once per factorisation, then one refinement pass:
 * the residual b - A x with the FP64 operator (K and the scaled constraints) and a second
 * double-float solve added to x.  1: the sweeps in FP64 from the factor itself (no copies, half
 * the device memory); 2: the double-float sweeps without the refinement pass. */
#define ASTRO_OPT_PANELS_SOLVE 8
int astro_set_option(astro_ctx *ctx, int32_t option, int32_t value);

/* The CUDA stream (cudaStream_t) the context launches on, for callers that order their own work
 * or record timing events around the library's kernels. */
void *astro_ctx_stream(const astro_ctx *ctx);
/* Reference analysisPrep outputs: currentRank(num_nodes), nDofIndex(6,num_nodes),
 * elMatRange(0:n), elMatLTRange(0:n), and the unscaled constraint matrix
 * elMPCMatRange(0:m), elMPCMatCols, elMPCMat, elMPCRHS.  NULL pointers are skipped. */
int astro_get_prep(const astro_ctx *ctx, int32_t *current_rank, int32_t *n_dof_index,
                   int32_t *el_mat_range, int32_t *el_mat_lt_range,
                   int32_t *mpc_range, int32_t *mpc_cols, double *mpc_mat, double *mpc_rhs);

/* ---- element evaluation and assembly ------------------------------------------------------ */

/* getElasticSolnLoad(buildMat) (Working/AStrO_commandFunctions.f90:260-351).
 * Evaluates every element at `state` on the GPU in FP64.  elastic_load[n] and
 * int_elastic_load[int_vec_size] are accumulated in place: load(dof) -= Ru (as the reference).
 * If build_mat == 1 the stiffness is assembled on the device (kept for the solvers) and, when
 * the pointers are non-NULL, exported in the reference CSR layout: elastic_mat[el_mat_size],
 * el_mat_cols[el_mat_size] (same column order as the reference's find-or-insert), and the
 * condensed internal rows int_elastic_mat[int_mat_size]. */
int astro_el_soln_load(astro_ctx *ctx, int32_t build_mat, const astro_state *state,
                       double *elastic_load, double *int_elastic_load,
                       double *elastic_mat, int32_t *el_mat_cols, double *int_elastic_mat);

/* updateExternalRHS (Working/AStrO_commandFunctions.f90:568-607), loop over the internal rows
 * as intended: ext_vec[el_mat_dim] -= K_ni K_ii^-1 int_vec for every element with internal DOF,
 * using the condensed internal rows of the last astro_el_soln_load(build_mat = 1). */
int astro_update_external_rhs(astro_ctx *ctx, double *ext_vec, const double *int_vec);
/* updateInternalSoln (:609-651), same resolution: int_soln[int_vec_size] +=
 * K_ii^-1 (int_rhs - K_in ext_soln) per element; int_rhs may be NULL (zeros). */
int astro_update_internal_soln(astro_ctx *ctx, const double *ext_soln, double *int_soln,
                               const double *int_rhs);

/* Mixed-precision assembly used by the refinement solvers: element matrices evaluated in FP32
 * (isotropic/orthotropic sparse-B formulation) and assembled at zero state into the device
 * block-CSR matrix in both FP32 and FP64 storage.  The FP64 copy is the system matrix A. */
int astro_assemble_fp32(astro_ctx *ctx);
/* Same as astro_assemble_fp32 without the final stream synchronisation (for timing loops);
 * requires a prior astro_assemble_fp32 on the context. */
int astro_assemble_fp32_async(astro_ctx *ctx);

/* Per-element matrices, for parity tests.  precision 64 or 32.  ke_out holds num_els blocks of
 * nd x nd column-major doubles (nd = 24 for brick8/shell4 after condensation), ru_out num_els
 * blocks of nd (may be NULL).  Evaluated at `state` (NULL = zero state). */
int astro_element_matrices(astro_ctx *ctx, int32_t precision, const astro_state *state,
                           double *ke_out, double *ru_out);

/* Complex-step residual sensitivity dRu/dd for design variable dvar (1-based), at the nodal
 * state `state` (getdRelasticdD, Working/AStrO_commandFunctions.f90:1172-1250, element part):
 * the elements that depend on dvar are evaluated at d_value[dvar] + i*h and
 * drudd[el_mat_dim] = Im(Ru) * (1/h) is summed at their global DOF, int_drudd[int_vec_size]
 * (may be NULL) at their internal DOF.  Both outputs are zeroed first, as the reference does.
 * The reference uses h = 1e-14 (compStep). */
int astro_drdd_complex(astro_ctx *ctx, int32_t dvar, double h, const astro_state *state,
                       double *drudd, double *int_drudd);

/* The complex-step dRu/dd of num design variables (1-based numbers in dvars) at the state, each
 * condensed to the nodal DOF as updateExternalRHS does (shells; needs the internal rows of the
 * last astro_el_soln_load(build_mat = 1)), into drudd (num x el_mat_dim, variable k at
 * drudd + k * el_mat_dim): the right-hand sides of the direct sensitivity solves, formed on the
 * device and copied out once. */
int astro_drdd_complex_condensed(astro_ctx *ctx, int32_t num, const int32_t *dvars, double h,
                                 const astro_state *state, double *drudd);

/* ---- constraints and loads ---------------------------------------------------------------- */

/* scaleElasticMPC (Working/AStrO_commandFunctions.f90:537-566): rows of C normalised to unit
 * 2-norm, then scaled by 100*max|K| of the last assembled stiffness.  Device copy updated;
 * scaled values exported when the pointers are non-NULL. */
int astro_scale_mpc(astro_ctx *ctx, double *mpc_mat, double *mpc_rhs);
/* getElasticConstraintLoad (:506-535): elastic_load += C^T (rhs - C u). */
int astro_constraint_load(astro_ctx *ctx, const double *node_disp, double *elastic_load);
/* Consistent surface load (intended semantics of getElasticAppliedLoad surface branch,
 * :353-504 / r_getElSurfaceTraction, Working/AStrO_r_elementEqns.f90:1923-2018):
 * for each (element, face) pair, elastic_load += integral of N^T t dA over the true face area,
 * with t = traction[3] + (-pressure) * outward face normal. */
int astro_surface_load(astro_ctx *ctx, int32_t nfaces, const int32_t *face_el,
                       const int32_t *face_num, const double *traction, double pressure,
                       double *elastic_load);

/* Body loads: the bodyForce / gravitational / centrifugal branch of getElasticAppliedLoad
 * (Working/AStrO_commandFunctions.f90:393-441) with r_getElBodyForce and r_getElCentAcc
 * (Working/AStrO_r_elementEqns.f90:1801-1921), added into elastic_load[n] (reference numbering).
 *   kind ASTRO_BODY_FORCE (0): vals[0..5] = force per unit volume (per unit volume of the section
 *        for shells: times the section thickness);
 *   kind ASTRO_BODY_GRAVITY (1): vals[0..5] = acceleration (translational, then rotational), the
 *        load being the element mass residual for that acceleration at every node;
 *   kind ASTRO_BODY_CENTRIFUGAL (2): vals = axis point(3), axis direction(3), angular velocity,
 *        the acceleration evaluated at each element's displaced centroid.
 * Bricks and shells, any element list.  elements: 1-based element numbers (count of them; an
 * element listed twice adds twice), or NULL for every element.  state: the displacement
 * (centrifugal centroid; shell frame), may be NULL.  Meshes mixing shells and bricks return
 * ASTRO_ERR_UNSUPPORTED. */
/* The load branch of getdRelasticdD for body loads (Working/AStrO_commandFunctions.f90:1250-1300):
 * drudd[n] -= d(body load)/d(design variable dvar) for the listed elements that depend on it
 * (arguments as astro_body_load; h the complex step).  Together with astro_drdd_complex it gives
 * the reference's dRudD when such loads act.  Brick body loads depend on none of the supported
 * design-variable categories (the call leaves drudd unchanged); for shells the layup-thickness
 * variables move the body force (linearly) and the mass of the gravitational and centrifugal
 * loads (complex step of the mass term). */
int astro_body_load_drdd(astro_ctx *ctx, int32_t dvar, double h, int32_t kind, const double *vals,
                         const int32_t *elements, int32_t count, const astro_state *state, double *drudd);
#define ASTRO_BODY_FORCE 0
#define ASTRO_BODY_GRAVITY 1
#define ASTRO_BODY_CENTRIFUGAL 2
int astro_body_load(astro_ctx *ctx, int32_t kind, const double *vals, const int32_t *elements, int32_t count,
                    const astro_state *state, double *elastic_load);

/* getElasticAppliedLoad's nodal design loads (Working/AStrO_commandFunctions.f90:494-502 with
 * r_getNodeDLoad, Working/AStrO_r_designPropertyFunctions.f90:970-994): elastic_load[n] (reference
 * numbering) += the nodal loads of the ASTRO_DCAT_NODE_LOAD variables active at `time`. */
int astro_design_node_load(astro_ctx *ctx, double time, double *elastic_load);
/* The nodal-load branch of getdRelasticdD (Working/AStrO_commandFunctions.f90:1364-1373): drudd[n]
 * -= d(nodal design load)/d(dvar) at `time`.  With astro_drdd_complex (element part) and
 * astro_body_load_drdd it gives the reference's dRudD. */
int astro_node_load_drdd(astro_ctx *ctx, int32_t dvar, double time, double *drudd);

/* ---- thermal path --------------------------------------------------------------------------- */

/* Thermal material data (not part of astro_model) and the thermal constraints: equations whose
 * terms are temperature DOF (reference DOF 7), expanded per node like astro_model's constraints
 * (buildThermalMPC, Working/AStrO_bookKeeping.f90:614-752). */
typedef struct astro_thermal_props {
    int32_t num_materials;
    const double *material_therm_cond;  /* materialThermCond(6, num_materials): k11 k22 k33 k12 k13 k23 */
    const double *material_spec_heat;   /* materialSpecHeat(num_materials) */
    int32_t num_mpc;                    /* thermal constraint equations */
    const int32_t *mpc_range;           /* (0:num_mpc) prefix sums over terms */
    const int32_t *mpc_node;            /* node per term */
    const double *mpc_coef;             /* coefficient per term */
    const double *mpc_rhs;              /* right-hand side per equation */
} astro_thermal_props;

/* Thermal state, node vectors in rank order (nodeTemp(currentRank(node)), as the reference);
 * NULL = zeros.  dynamic: add the capacitance term with Tdot from the generalised trapezoid rule
 * (r_getElRt, Working/AStrO_r_elementEqns.f90:2176-2204). */
typedef struct astro_thermal_state {
    const double *node_temp, *prev_temp, *prev_tdot;
    int32_t dynamic;
    double nm_gamma, del_t;
} astro_thermal_state;

/* Per-element thermal properties (r_getMaterialThermCond / r_getShellThermCond and the specific
 * heats, Working/AStrO_r_designPropertyFunctions.f90:129-186, 527-644), the thermal CSR layout
 * (allocateThermalMat, bookKeeping :413-472: rows by rank, 1 + neighbours) and the constraint
 * rows.  Outputs thermMatSize and thermMPCDim.  Brick or shell meshes. */
int astro_thermal_setup(astro_ctx *ctx, const astro_thermal_props *props, int32_t *therm_mat_size,
                        int32_t *therm_mpc_dim);
/* getThermalSolnLoad(buildMat) (Working/AStrO_commandFunctions.f90:16-72): thermal_load[N] -= Rt
 * (rank order); for build_mat = 1 the conductivity (+ capacitance / (gamma dt)) matrix stays on
 * the device and, when therm_mat / therm_cols are non-NULL, is exported as the reference's CSR
 * (thermMat, thermMatCols: 1-based rank columns in find-or-insert order). */
int astro_thermal_soln_load(astro_ctx *ctx, int32_t build_mat, const astro_thermal_state *state,
                            double *thermal_load, double *therm_mat, int32_t *therm_cols);
/* scaleThermalMPC (:230-258): rows to unit length, times 100 max|thermMat|; the scaled rows out
 * (may be NULL) and C^T C kept for the solve. */
int astro_thermal_scale_mpc(astro_ctx *ctx, double *mpc_mat, double *mpc_rhs);
/* getThermalConstraintLoad (:197-228): thermal_load += C^T (c - C T). */
int astro_thermal_constraint_load(astro_ctx *ctx, const double *node_temp, double *thermal_load);
/* getThermalAppliedLoad's bodyHeatGen branch (:96-139): heat generation q per unit volume on the
 * listed elements (1-based; NULL = all), integral of N (times the thickness for shells). */
int astro_thermal_heat_gen(astro_ctx *ctx, double q, const int32_t *elements, int32_t count, double *thermal_load);
/* getThermalAppliedLoad's surfaceFlux branch (:140-176): the flux as the first component of a
 * surface traction on the given element faces (as astro_surface_load), thermal_load -= the
 * component-1 nodal values (rank order). */
int astro_thermal_surface_flux(astro_ctx *ctx, int32_t nfaces, const int32_t *face_el, const int32_t *face_num,
                               double flux, double *thermal_load);
/* (K_T + C^T C) dtemp = rhs by Jacobi-preconditioned conjugate gradients in FP64 on the device,
 * from dtemp's input value, to ||r|| <= rtol ||rhs|| (in place of the reference's gMRes with
 * its skyline LDL^T preconditioner on the thermal system, stepSolve :689-703). */
int astro_thermal_solve(astro_ctx *ctx, const double *rhs, double *dtemp, double rtol, int32_t max_iters,
                        astro_solve_stats *stats);

/* Thermal design sensitivities: getdRthermaldD (Working/AStrO_commandFunctions.f90:1016-1170).
 * The design variables act on the thermal properties as the property routines apply them
 * (Working/AStrO_r_designPropertyFunctions.f90): solids take 'thermalCond' (ASTRO_DCAT_THERMAL_COND),
 * 'specHeat' and 'density' (the heat capacity is density x specific heat); shells take the
 * layer's 'layup' thermalCond, specHeat, density, thickness and angle; node coordinates and
 * solid orientation variables move the element geometry.  The real values d_value enter
 * astro_thermal_setup's properties.
 *
 * Element part (:1040-1059): drtdd[N] (rank order) is zeroed, then for every element that depends
 * on dvar (its el_to_d terms, or a nodeCoord term of one of its nodes) Rt is evaluated in complex
 * FP64 with d_value(dvar) + i h at the given thermal state (capacitance included when dynamic)
 * and Im(Rt) / h is added at the element's nodes: properties, section frame (orientation
 * variables; correctAlpha for shells) and node coordinates all in complex arithmetic. */
int astro_thermal_drdd(astro_ctx *ctx, int32_t dvar, double h, const astro_thermal_state *state, double *drtdd);
/* bodyHeatGen branch (:1065-1108): drtdd -= d(heat-generation load)/d(dvar) for the listed
 * elements (1-based, NULL = all; an element listed twice counts twice) that depend on dvar,
 * by the complex step of the load (shell thickness, node coordinates). */
int astro_thermal_heat_gen_drdd(astro_ctx *ctx, int32_t dvar, double h, double q, const int32_t *elements,
                                int32_t count, double *drtdd);
/* surfaceFlux branch (:1109-1152): drtdd += d(component-1 face load)/d(dvar) for the given faces
 * whose element depends on dvar (node coordinates move the face). */
int astro_thermal_surface_flux_drdd(astro_ctx *ctx, int32_t dvar, double h, int32_t nfaces, const int32_t *face_el,
                                    const int32_t *face_num, double flux, double *drtdd);
/* Nodal thermal design loads ('nodeLoad' / 'thermal', ASTRO_DCAT_NODE_LOAD with d_component 7):
 * getThermalAppliedLoad's closing loop (:182-186) thermal_load[rank] += the active variables'
 * coef x d, and getdRthermaldD's node branch (:1162-1167) drtdd[rank] -= coef for dvar. */
int astro_thermal_design_node_load(astro_ctx *ctx, double time, double *thermal_load);
int astro_thermal_node_load_drdd(astro_ctx *ctx, int32_t dvar, double time, double *drtdd);

/* ---- batched panels ----------------------------------------------------------------------- */

/* A model made of many independent panels (the connected components of its mesh; constraints
 * may not couple two of them), each solved with a direct LDL^T factorisation of K + C^T C as the
 * reference solves one model with getSparseLDLFact / solveSparseLDLFact
 * (Working/AStrO_solvers.f90:10-126), all panels in one persistent launch: a blocked band LDL^T
 * in FP64 with one thread-block cluster per panel, panels ordered along their longest extent.
 * The FP64 stiffness must be assembled (astro_el_soln_load) and the constraints scaled
 * (astro_scale_mpc).  cluster_size: CTAs per panel (1, 2, 4 or 8; 0 = 8). */
typedef struct astro_panels_info {
    int32_t num_panels;
    int32_t max_bandwidth;   /* largest lower bandwidth in DOF */
    int64_t band_bytes;      /* device storage of the band factors */
    int32_t cluster_size;
    int32_t workers;         /* clusters of the factor launch */
    double factor_seconds;   /* band fill + factorisation, wall clock */
    double solve_seconds;    /* the last astro_panels_solve, wall clock with the copies */
} astro_panels_info;
int astro_panels_factor(astro_ctx *ctx, int32_t cluster_size, astro_panels_info *info);
/* X = (K + C^T C)^-1 B for num_rhs right-hand sides: rhs and x are num_rhs x el_mat_dim (column
 * k at rhs + k * el_mat_dim), global DOF numbering.  Needs a current astro_panels_factor. */
int astro_panels_solve(astro_ctx *ctx, int32_t num_rhs, const double *rhs, double *x, astro_panels_info *info);
/* Factor (when the stiffness or the constraints changed since the last factorisation) and solve. */
int astro_panels_solve_batched(astro_ctx *ctx, int32_t num_rhs, const double *rhs, double *x,
                               astro_panels_info *info);

/* ---- linear solve ------------------------------------------------------------------------- */

/* convertToLTri (Working/AStrO_bookKeeping.f90:754-792): row-skyline lTri = (K inside the
 * profile) + C^T C inside the profile, from the device-resident K and scaled C.  Exported to
 * l_tri[el_mat_lt_size] when non-NULL; the device copy stays for astro_ldl_fact_resident. */
int astro_convert_to_ltri(astro_ctx *ctx, double *l_tri);

/* getSparseLDLFact (Working/AStrO_solvers.f90:10-78), same arguments: LDL^T of the row-skyline
 * matrix ALTri (ASize values, row ranges ARange(0:n)) overwritten in place, on the GPU. */
int astro_ldl_fact(astro_ctx *ctx, double *a_l_tri, int32_t a_size, const int32_t *a_range,
                   int32_t n);
/* Factorises the device-resident skyline built by astro_convert_to_ltri, in place. */
int astro_ldl_fact_resident(astro_ctx *ctx);

/* solveSparseLDLFact (Working/AStrO_solvers.f90:83-126), same arguments: solves
 * L D L^T soln = rhs with a factor from getSparseLDLFact.  z_vec (Ldim) is scratch. */
int astro_ldl_solve(astro_ctx *ctx, double *soln, const double *rhs, const double *l_mat,
                    int32_t l_size, const int32_t *l_range, int32_t l_dim, double *z_vec);

/* No counterpart in the reference.  The same solve as astro_ldl_solve for callers that must not
 * allocate device memory during a solve: loops that have already filled HBM with the matrix,
 * factor and Krylov basis, and callers with work on other streams that cudaFree would stall.
 * All operands are the caller's DEVICE buffers (soln, rhs: l_dim; l_mat: the factor;
 * l_range: l_dim+1 row ranges); the forward-sweep scratch is a fixed 2 MiB array in the
 * library, so l_dim is limited to ASTRO_LDL_NOALLOC_MAX_DIM (larger sizes return
 * ASTRO_ERR_ARG without touching the GPU).  Every call looks up the scratch's device address
 * with the context's device current; the first lookup on a device may load the library's module,
 * so make the first call before any stream capture begins.  The scratch is shared by all contexts
 * on a device and keeps the last call's values: overlapping calls on one device race and must be
 * serialised.  Runs on the context's stream and returns after it completes. */
#define ASTRO_LDL_NOALLOC_MAX_DIM 262144
int astro_ldl_solve_device_noalloc(astro_ctx *ctx, double *d_soln, const double *d_rhs,
                                   const double *d_l_mat, const int32_t *d_l_range, int32_t l_dim);

/* gMRes (Working/AStrO_solvers.f90:128-297), same arguments: restarted, left-preconditioned
 * GMRES(numVecs) on A = Amat + Cmat^T Cmat with the skyline LDL^T factor Pmat as
 * preconditioner, convergence when the preconditioned residual norm is <= 1e-12 (single
 * precision literal, as the reference) or after maxIt/numVecs+1 restarts.  x_vec is the
 * initial guess on entry and the solution on exit. */
int astro_gmres(astro_ctx *ctx, double *x_vec, const double *a_mat, const int32_t *a_cols,
                const int32_t *a_range, int32_t a_size, int32_t a_dim, const double *c_mat,
                const int32_t *c_cols, const int32_t *c_range, int32_t c_size, int32_t c_dim,
                const double *p_mat, const int32_t *p_range, int32_t p_size,
                const double *b_vec, int32_t num_vecs, int32_t max_it);

/* North-star static solve of (K + C^T C) u = f with device-resident K (from astro_el_soln_load
 * or astro_assemble_fp32) and scaled C.  f and u are host arrays in global DOF numbering;
 * u is the initial guess on entry.  Convergence is judged by the FP64 true relative residual. */
int astro_solve_static(astro_ctx *ctx, const double *f, double *u, const astro_solve_opts *opts,
                       astro_solve_stats *stats);

/* Implicit Newmark time stepping: the dynamic branch of solve (Working/AStrO_commandFunctions.f90:
 * 751-815) with stepSolve (:681-749) for linear geometry.  K_eff = K + c1 c2 M (c1 = 0.5/beta,
 * c2 = 2/del_t^2) is assembled at the initial state and the constraints scaled; then every step
 * t = k del_t forms the residual with the Newmark inertia, adds load_amplitude[k] * load_pattern
 * (load_pattern: el_mat_dim, may be NULL) and the constraint load, condenses the internal DOF,
 * solves K_eff du = r by FP64 Jacobi-GMRES (restart, max_iters per step, relative tolerance rtol)
 * warm-started from the previous increment, recovers the internal DOF and updates the state
 * (acc, vel, previous values).  disp/vel/acc (el_mat_dim) and int_disp (int_vec_size, may be
 * NULL) hold the initial state on entry (loadInitialState) and the final state on exit;
 * disp_history (num_steps x el_mat_dim, may be NULL) receives the displacement of every step.
 * Shell and solid meshes (r_getElRum's shell and solid branches). */
typedef struct astro_newmark_opts {
    int32_t num_steps;
    double del_t, nm_beta, nm_gamma;
    int32_t restart, max_iters;  /* GMRES per step */
    double rtol;
    int32_t method;                /* ASTRO_SOLVER_*: 0 FP64 Jacobi-GMRES (the default, as above);
                                      1 mixed or 2 learned FGMRES on K_eff, FP32 copy converted
                                      from the FP64 K_eff, FP64 refinement */
    const astro_precond *precond;  /* method 2: the network (NULL: the default network) */
} astro_newmark_opts;
int astro_newmark_run(astro_ctx *ctx, const astro_newmark_opts *opts, const double *load_pattern,
                      const double *load_amplitude, double *disp, double *vel, double *acc,
                      double *int_disp, double *disp_history, astro_solve_stats *stats);
/* The same loop returning the state of every step, the records writeBinarySolution writes after
 * each step (Working/AStrO_commandFunctions.f90:808-811, Working/AStrO_output.f90:761-784):
 * disp, vel, acc histories (num_steps x el_mat_dim, global DOF numbering) and int_disp_history
 * (num_steps x int_vec_size); any may be NULL. */
int astro_newmark_run_states(astro_ctx *ctx, const astro_newmark_opts *opts, const double *load_pattern,
                             const double *load_amplitude, double *disp, double *vel, double *acc, double *int_disp,
                             double *disp_history, double *vel_history, double *acc_history,
                             double *int_disp_history, astro_solve_stats *stats);

/* ---- autotuner of the launch shapes (no counterpart in the reference) ----------------------
 * Times the candidate launch shapes of the selected tunables on this context's model (CUDA events)
 * and keeps the fastest for the context:
 *   ASTRO_TUNE_BRICK_WARPS    the zero-state brick kernel's warps per CTA (1, 2, 4): FP32 assembly
 *                             passes (brick8 meshes; leaves the FP32 assembly resident);
 *   ASTRO_TUNE_PANEL_CLUSTER  the band factorisation's CTAs per cluster (2, 4, 8): one
 *                             astro_panels_factor each (needs the FP64 assembly and the scaled
 *                             constraints); astro_panels_factor with cluster_size 0 then uses it;
 *   ASTRO_TUNE_CASES_CLUSTER  the many-column band solve's CTAs per cluster (2, 4, 8): solves of
 *                             the factorisation prepared by the last astro_newmark_cases.
 * cache_path (may be NULL): a text file of lines "<key> <choice> <seconds>", the key naming the
 * GPU, the tunable and the model's size; a cached choice is applied without timing, and new
 * results are appended.  choices (3, may be NULL) receives the context's choices (0 = default). */
#define ASTRO_TUNE_BRICK_WARPS 1
#define ASTRO_TUNE_PANEL_CLUSTER 2
#define ASTRO_TUNE_CASES_CLUSTER 4
int astro_autotune(astro_ctx *ctx, int32_t what, const char *cache_path, int32_t *choices);

/* ---- batched linear Newmark: many load cases through one factorisation ------------------
 * The dynamic branch of solve with linear geometry (Working/AStrO_commandFunctions.f90:770-812:
 * getElasticSolnLoad(1) with the dynamic flag, scaleElasticMPC, getSparseLDLFact of K_eff once,
 * then per step stepSolve and the Newmark update of :796-799) for num_cases load histories
 * f_k(t_j) = amplitudes[k * num_steps + j] * patterns[k * n + :] at once.  K (static) and
 * K_eff = K + c1 c2 M (dynamic) are assembled at the zero state, condensed over the internal DOF;
 * K_eff + C^T C is factored once by the band LDL^T (astro_panels_factor's kernels, tensor-core
 * trailing updates), and every step solves all cases in one launch, the step captured as a CUDA
 * graph and launched num_steps times without a host round trip.  The residual of a step is that
 * of the linearised element equations, r = f - K u - M a_pred - C^T (C u - rhs) (a_pred: the
 * acceleration at the start of the step); the reference's elements carry Green-Lagrange strain
 * and finite rotations at every state, so the two loops differ by the geometric nonlinearity of
 * the motion (and, for shells, only with the consistent tangent ASTRO_OPT_SHELL_MEAN_ROT_TERM do
 * they agree).  disp, vel, acc: num_cases x n, the initial state in, the final state out;
 * disp_history: num_steps x num_cases x n or NULL.  Leaves K_eff in the context's FP64 matrix
 * and its factorisation in the panel plan. */
#define ASTRO_NMC_FACTORED 0
typedef struct astro_newmark_cases_opts {
    int32_t num_steps, num_cases;
    double del_t, nm_beta, nm_gamma;
    int32_t method;    /* ASTRO_NMC_FACTORED */
    int32_t no_graph;  /* 1: launch the step's kernels directly every step (no CUDA graph) */
    int32_t refine;    /* FP64 refinement passes per step (0..4): du -= A^-1 (A du - r) with the
                          residual over the FP64 assembly; the many-column solve runs in
                          double-float (about 48 bits), so ill-conditioned K_eff may want one */
    int32_t autotune;  /* 1: pick the many-column solve's cluster size by timing (astro_autotune's
                          ASTRO_TUNE_CASES_CLUSTER) unless the context already holds a choice */
} astro_newmark_cases_opts;
typedef struct astro_newmark_cases_info {
    double factor_seconds;     /* band fill + LDL^T (host clock around the launch) */
    double prepare_seconds;    /* uploads, both assemblies, scaling, factorisation, band copies */
    double step_seconds;       /* CUDA events around the num_steps step launches */
    double last_rel_residual;  /* max over cases of ||(K_eff + C^T C) du - r|| / ||r||, last step, FP64 */
    int64_t band_bytes;        /* FP64 band of the factor */
    int64_t df_band_bytes;     /* double-float band copies of the many-column solve */
    int32_t bandwidth;         /* lower bandwidth (DOF) of the ordering */
    int32_t panels;            /* connected components */
    int32_t graph_nodes;       /* nodes of the captured step */
    int32_t kernels_per_step;  /* kernel launches of one step */
    int32_t cluster_size;      /* CTAs per case of the many-column solve */
} astro_newmark_cases_info;
int astro_newmark_cases(astro_ctx *ctx, const astro_newmark_cases_opts *opts, const double *patterns,
                        const double *amplitudes, double *disp, double *vel, double *acc, double *disp_history,
                        astro_newmark_cases_info *info);

/* y = (K + C^T C) x for host vectors in global DOF numbering, with the device-resident K
 * (kind 64: FP64 values from astro_el_soln_load, 32: FP32 values from astro_assemble_fp32) and
 * the scaled constraints; the operator of the gMRes matvec (Working/AStrO_solvers.f90:143-169). */
int astro_apply_operator(astro_ctx *ctx, int32_t kind, const double *x, double *y);

/* ---- polynomial preconditioner: initialisation, eigenvalue estimate, training -------------- */

/* Host only: the untrained network, W_k = c_k I with c the least-squares fit of
 * nu sum_k c_k T_k(x(nu)) = 1 over 400 Chebyshev nodes of nu in [1/ratio, 1]; lambda_scale 1.05. */
int astro_precond_init(int32_t degree, double ratio, int32_t dpn, astro_precond *p);

/* Largest eigenvalue of D^-1 A by 50 power iterations on the device from a fixed start vector
 * (deterministic), with the FP64 (kind 64) or FP32 (kind 32) device-resident K. */
int astro_precond_lambda(astro_ctx *ctx, int32_t kind, double *lambda);

/* Training loss of the network on num_samples vectors v_s (host, num_samples x el_mat_dim, global
 * DOF numbering; each is normalised to unit length first) with the FP64 device-resident K:
 *     loss = (1/S) sum_s || v_s - A P v_s ||^2
 * and its gradient with respect to the weights (same layout as astro_precond.weights; A is
 * symmetric).  Everything in FP64 on the device; lambda from astro_precond_lambda(kind 64). */
int astro_precond_loss_grad(astro_ctx *ctx, const astro_precond *p, const double *samples, int32_t num_samples,
                            double *loss, double *grad);

/* Trains the weights of p in place on the samples: iters steps of conjugate gradients
 * (Polak-Ribiere+) with an exact line search (the loss is quadratic in the weights), each step
 * one gradient and one line-search evaluation on the device.  loss_history (iters + 1, may be
 * NULL) receives the loss before every step and after the last. */
int astro_precond_train(astro_ctx *ctx, astro_precond *p, const double *samples, int32_t num_samples, int32_t iters,
                        double *loss_history);

/* Node features (num_nodes x ASTRO_NODE_FEATURES, row = node id - 1) of the device-resident
 * assembly (kind 64: FP64 values, 32: FP32 values) with the scaled constraints. */
int astro_node_features(astro_ctx *ctx, int32_t kind, double *features);

/* The per-node hop scales a_k(r) of mlp (num_nodes x mlp->outputs, row = node id - 1). */
int astro_precond_mlp_scales(astro_ctx *ctx, int32_t kind, const astro_precond_mlp *mlp, double *scales);

/* Training loss of the modulated network (the loss of astro_precond_loss_grad with
 * P v = (1/lambda) sum_k a_k (W_k y_k)) and its gradients: grad_weights with respect to the hop
 * weights (layout of astro_precond.weights, may be NULL) and grad_mlp with respect to the
 * perceptron (layout of astro_precond_mlp; hidden and outputs copied from mlp; may be NULL).
 * Forward and backward passes on the device in FP64; the node features from the FP64 assembly. */
int astro_precond_mlp_loss_grad(astro_ctx *ctx, const astro_precond *p, const astro_precond_mlp *mlp,
                                const double *samples, int32_t num_samples, double *loss, double *grad_weights,
                                astro_precond_mlp *grad_mlp);

/* stepSolve, elastic static branch (Working/AStrO_commandFunctions.f90:681-749): from node_disp
 * (el_mat_dim, global DOF numbering, in/out) and internal_disp (int_vec_size, in/out, may be NULL),
 * iterate while fewer than 1 (nl_geom = 0) or 20 (nl_geom = 1) iterations have run and
 * max|delDisp| > 1e-12 (the reference's single-precision literal): residual at the state (the
 * tangent too when nl_geom = 1; the constraint penalty keeps the scaling of the last
 * astro_scale_mpc), plus applied_load (getElasticAppliedLoad(time), el_mat_dim, may be NULL) and
 * the constraint load, condensation, the solve of opts->solve warm-started from the previous
 * increment, internal-DOF recovery, u += delDisp.  Needs astro_el_soln_load(build_mat = 1) and
 * astro_scale_mpc first.  *iterations (may be NULL) receives the Newton iterations run. */
typedef struct astro_step_opts {
    int32_t nl_geom;            /* nLGeom */
    astro_solve_opts solve;     /* the step's linear solves */
} astro_step_opts;
int astro_step_solve(astro_ctx *ctx, const astro_step_opts *o, const double *applied_load, double *node_disp,
                     double *internal_disp, int32_t *iterations, astro_solve_stats *stats);

/* getTotaldLdD for a static analysis (Working/AStrO_commandFunctions.f90:1377-1410) with the elastic
 * branch of solveDynamicAdjoint (:917-966; dLdv = dLda = 0): the adjoint K lambda = dLdu after
 * updateExternalRHS with int_dldu, the internal lambda by updateInternalSoln, then for every design
 * variable d = 1..num_dvars
 *     dldd[d-1] = dldd_explicit[d-1] - lambda . dRudD(d) - lambda_int . intdRudD(d)
 * with dRudD by the complex step of step h at state (getdRelasticdD).  The objective's partials come
 * from the caller (getdObjdU / getdObjdD): dldu (el_mat_dim, global DOF numbering), int_dldu
 * (int_vec_size, may be NULL), dldd_explicit (num_dvars, may be NULL).  K (astro_el_soln_load with
 * build_mat = 1 at the same state) and the scaled constraints must be resident; the adjoint solve
 * runs the GPU solver of opts instead of the reference's LDL-preconditioned gMRes, converged on the
 * FP64 true residual.  disp_adj (el_mat_dim) and int_disp_adj (int_vec_size) may be NULL. */
int astro_total_dldd(astro_ctx *ctx, const astro_state *state, double h, const double *dldu, const double *int_dldu,
                     const double *dldd_explicit, const astro_solve_opts *opts, double *dldd, double *disp_adj,
                     double *int_disp_adj, astro_solve_stats *stats);

/* getTotaldLdD for a Newmark analysis (Working/AStrO_commandFunctions.f90:1411-1465): the backward
 * sweep i = num_steps..1 over the stored states, each step augmentdLdu (:819-915; i < num_steps),
 * the objective's partials at t_i, solveDynamicAdjoint's elastic branch (:917-966) with K_eff at
 * (state i, previous state i-1) and the complex-step dRu/dD at that state:
 *     dldd[d-1] = dldd_explicit[d-1] - sum_i (lambda_i . dRudD_i(d) + lambda_int_i . intdRudD_i(d)).
 * The states are the records of SolutionHistory<i> (i = 0..num_steps): disp, vel, acc
 * ((num_steps + 1) x el_mat_dim) and int_disp ((num_steps + 1) x int_vec_size, may be NULL).  The
 * objective's partials per step are rows i-1 of dldu, dldv, dlda (num_steps x el_mat_dim) and
 * int_dldu (num_steps x int_vec_size); any may be NULL (zero).  Faithful to the reference: the
 * 1e-20 scaling round trip around augmentdLdu, the warm start of each adjoint solve from the
 * previous one, and the internal adjoint accumulated across steps (updateInternalSoln adds).
 * Shell and solid meshes.  disp_adj (el_mat_dim, may be NULL)
 * receives the adjoint of step 1; stats sums the solves. */
typedef struct astro_transient_adjoint {
    int32_t num_steps;
    double del_t, nm_beta, nm_gamma;
    double h;                               /* complex step of getdRelasticdD */
    const double *disp, *vel, *acc, *int_disp;
    const double *dldu, *dldv, *dlda, *int_dldu;
    const double *dldd_explicit;            /* num_dvars (getdObjdD summed over the steps), may be NULL */
    astro_solve_opts solve;                 /* the adjoint solves */
} astro_transient_adjoint;
int astro_total_dldd_transient(astro_ctx *ctx, const astro_transient_adjoint *a, double *dldd, double *disp_adj,
                               astro_solve_stats *stats);

/* Solution-history step file of the reference (writeBinarySolution / readBinarySolution,
 * Working/AStrO_output.f90:761-784, Working/AStrO_input.f90:1740-1768): Fortran unformatted
 * sequential records (4-byte length markers before and after each record) of prevTemp
 * (num_nodes), prevTdot (num_nodes), prevDisp (el_mat_dim), prevIntDisp (int_vec_size; written when
 * int_vec_size >= 1, read when int_vec_size > 1, as the reference does), prevVel, prevAcc.  Host
 * only.  NULL temperature arrays write zeros / skip the values on reading.  The reader returns
 * ASTRO_ERR_ARG when the file cannot be opened or is short (the reference's errFlag). */
int astro_write_step_file(const char *path, int32_t num_nodes, int32_t el_mat_dim, int32_t int_vec_size,
                          const double *prev_temp, const double *prev_tdot, const double *prev_disp,
                          const double *prev_int_disp, const double *prev_vel, const double *prev_acc);
int astro_read_step_file(const char *path, int32_t num_nodes, int32_t el_mat_dim, int32_t int_vec_size,
                         double *prev_temp, double *prev_tdot, double *prev_disp, double *prev_int_disp,
                         double *prev_vel, double *prev_acc);

/* Measurement hook: the average device time (CUDA events, reps launches after five warm-up
 * launches) of one preconditioner hop on the operator of the last learned solve of this context,
 * and the bytes one hop moves (FP16 block planes, columns, and the hop's vector loads and stores).
 * No counterpart in the reference. */
int astro_precond_time_hop(astro_ctx *ctx, int32_t reps, double *us_per_hop, double *bytes_per_hop);

#ifdef __cplusplus
}
#endif

#endif /* ASTRO_GPU_H */
