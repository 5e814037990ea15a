"""Host-side mirror of AStrO's hot-path subroutines over the GB300 C ABI (include/astro_gpu.h).

Method names follow the Fortran subroutines they replace (Working/AStrO_commandFunctions.f90,
Working/AStrO_solvers.f90, Working/AStrO_bookKeeping.f90); arrays use the reference's numbering
(1-based DOF numbers, range arrays with lower bound 0, CSR column 0 = empty slot).  Everything
runs in libastro_gpu.so on the GPU; there is no CPU fallback: a missing library or device raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .model import AstroStateC, Model, make_state

I32P = C.POINTER(C.c_int32)
F64P = C.POINTER(C.c_double)

ASTRO_OK = 0
ERRORS = {1: "ASTRO_ERR_ARG", 2: "ASTRO_ERR_CUDA", 3: "ASTRO_ERR_UNSUPPORTED", 4: "ASTRO_ERR_PIVOT",
          5: "ASTRO_ERR_NAN", 6: "ASTRO_ERR_BREAKDOWN", 7: "ASTRO_ERR_MAXIT", 8: "ASTRO_ERR_STATE",
          9: "ASTRO_ERR_NOMEM", 10: "ASTRO_ERR_BOUNDS"}
SOLVER_GMRES_JACOBI_FP64 = 0
SOLVER_FGMRES_MIXED = 1
SOLVER_FGMRES_LEARNED = 2
OPT_BAND_FP64_UPDATE = 3
OPT_BRICK_WARPS, OPT_PANEL_CLUSTER, OPT_CASES_CLUSTER = 4, 5, 6
OPT_CASES_TWIST = 7
OPT_PANELS_SOLVE = 8

_LIB = None


class AstroError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class ThermalPropsC(C.Structure):
    _fields_ = [("num_materials", C.c_int32), ("material_therm_cond", F64P), ("material_spec_heat", F64P),
                ("num_mpc", C.c_int32), ("mpc_range", I32P), ("mpc_node", I32P), ("mpc_coef", F64P),
                ("mpc_rhs", F64P)]


class ThermalStateC(C.Structure):
    _fields_ = [("node_temp", F64P), ("prev_temp", F64P), ("prev_tdot", F64P), ("dynamic", C.c_int32),
                ("nm_gamma", C.c_double), ("del_t", C.c_double)]


def thermal_props(cond, spec_heat, mpc=None):
    """astro_thermal_props over float64/int32 arrays: cond (M, 6), spec_heat (M,), mpc =
    (range, node, coef, rhs) of the temperature constraints or None."""
    keep = {"c": _f64(np.asarray(cond).reshape(-1)), "s": _f64(spec_heat)}
    p = ThermalPropsC()
    p.num_materials = len(keep["s"])
    p.material_therm_cond = _d(keep["c"])
    p.material_spec_heat = _d(keep["s"])
    if mpc is not None:
        keep.update(r=_i32(mpc[0]), n=_i32(mpc[1]), k=_f64(mpc[2]), h=_f64(mpc[3]))
        p.num_mpc = len(keep["r"]) - 1
        p.mpc_range, p.mpc_node, p.mpc_coef, p.mpc_rhs = _i(keep["r"]), _i(keep["n"]), _d(keep["k"]), _d(keep["h"])
    p._keep = keep
    return p


def thermal_state(temp=None, prev_temp=None, prev_tdot=None, dynamic=0, gamma=0.5, del_t=0.0):
    keep = {}
    s = ThermalStateC()
    for name, arr in (("node_temp", temp), ("prev_temp", prev_temp), ("prev_tdot", prev_tdot)):
        if arr is not None:
            keep[name] = _f64(arr)
            setattr(s, name, _d(keep[name]))
    s.dynamic, s.nm_gamma, s.del_t = dynamic, gamma, del_t
    s._keep = keep
    return s


class PanelsInfoC(C.Structure):
    _fields_ = [("num_panels", C.c_int32), ("max_bandwidth", C.c_int32), ("band_bytes", C.c_int64),
                ("cluster_size", C.c_int32), ("workers", C.c_int32), ("factor_seconds", C.c_double),
                ("solve_seconds", C.c_double)]


class DimsC(C.Structure):
    _fields_ = [(k, C.c_int32) for k in ("el_mat_dim", "el_mat_size", "el_mat_lt_size", "el_mpc_dim", "el_mpc_size",
                                         "int_vec_size", "int_mat_size", "solver_max_bw", "dof_per_node",
                                         "num_blocks", "num_colors")]


PRECOND_MAX_DEGREE = 32


class PrecondC(C.Structure):
    """astro_precond: polynomial graph-convolution preconditioner (degree, dpn, interval, weights)."""
    _fields_ = [("degree", C.c_int32), ("dpn", C.c_int32), ("ratio", C.c_double), ("lambda_scale", C.c_double),
                ("weights", C.c_double * ((PRECOND_MAX_DEGREE + 1) * 36))]

    def weight_array(self):
        """W as an array (degree + 1, dpn, dpn) (a copy)."""
        k, d = self.degree + 1, self.dpn
        return np.array(self.weights[:k * d * d]).reshape(k, d, d)

    def set_weights(self, w):
        w = np.asarray(w, dtype=np.float64).reshape(-1)
        assert w.size == (self.degree + 1) * self.dpn * self.dpn
        for i, x in enumerate(w):
            self.weights[i] = float(x)


NODE_FEATURES = 6
MLP_MAX_HIDDEN = 32


class PrecondMlpC(C.Structure):
    """astro_precond_mlp: per-node modulation of the polynomial network (node features -> hop
    scales a_k = 1 + b2 + w2 tanh(w1 f + b1))."""
    _fields_ = [("hidden", C.c_int32), ("outputs", C.c_int32),
                ("w1", C.c_double * (MLP_MAX_HIDDEN * NODE_FEATURES)), ("b1", C.c_double * MLP_MAX_HIDDEN),
                ("w2", C.c_double * ((PRECOND_MAX_DEGREE + 1) * MLP_MAX_HIDDEN)),
                ("b2", C.c_double * (PRECOND_MAX_DEGREE + 1))]

    def params(self):
        """(w1 (H, F), b1 (H), w2 (K, H), b2 (K)) as arrays (copies)."""
        H, K = self.hidden, self.outputs
        return (np.array(self.w1[:H * NODE_FEATURES]).reshape(H, NODE_FEATURES), np.array(self.b1[:H]),
                np.array(self.w2[:K * H]).reshape(K, H), np.array(self.b2[:K]))

    def set_params(self, w1, b1, w2, b2):
        H, K = self.hidden, self.outputs
        for dst, src, cnt in ((self.w1, w1, H * NODE_FEATURES), (self.b1, b1, H), (self.w2, w2, K * H),
                              (self.b2, b2, K)):
            a = np.asarray(src, dtype=np.float64).reshape(-1)
            assert a.size == cnt
            for i in range(cnt):
                dst[i] = float(a[i])

    def vector(self):
        return np.concatenate([x.reshape(-1) for x in self.params()])

    def set_vector(self, v):
        H, K, F = self.hidden, self.outputs, NODE_FEATURES
        v = np.asarray(v, dtype=np.float64)
        o = [0, H * F, H * F + H, H * F + H + K * H, H * F + H + K * H + K]
        self.set_params(v[o[0]:o[1]], v[o[1]:o[2]], v[o[2]:o[3]], v[o[3]:o[4]])


def mlp_init(hidden, outputs, seed=0, scale=None):
    """A perceptron whose output layer is zero (a_k = 1: the unmodulated network) and whose first
    layer is drawn N(0, 1/F) from seed."""
    m = PrecondMlpC()
    m.hidden, m.outputs = hidden, outputs
    rng = np.random.default_rng(seed)
    sc = (1.0 / np.sqrt(NODE_FEATURES)) if scale is None else scale
    m.set_params(sc * rng.standard_normal((hidden, NODE_FEATURES)), np.zeros(hidden), np.zeros((outputs, hidden)),
                 np.zeros(outputs))
    return m


class SolveOptsC(C.Structure):
    _fields_ = [("method", C.c_int32), ("restart", C.c_int32), ("max_iters", C.c_int32), ("rtol", C.c_double),
                ("inner_rtol", C.c_double), ("precond", C.POINTER(PrecondC)), ("mlp", C.POINTER(PrecondMlpC))]


class StepOptsC(C.Structure):
    _fields_ = [("nl_geom", C.c_int32), ("solve", SolveOptsC)]


class TransientAdjointC(C.Structure):
    _fields_ = [("num_steps", C.c_int32), ("del_t", C.c_double), ("nm_beta", C.c_double), ("nm_gamma", C.c_double),
                ("h", C.c_double), ("disp", F64P), ("vel", F64P), ("acc", F64P), ("int_disp", F64P),
                ("dldu", F64P), ("dldv", F64P), ("dlda", F64P), ("int_dldu", F64P), ("dldd_explicit", F64P),
                ("solve", SolveOptsC)]


class SolveStatsC(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("restarts", C.c_int32), ("refinements", C.c_int32),
                ("status", C.c_int32), ("rel_residual", C.c_double), ("seconds", C.c_double),
                ("conditional_graph", C.c_int32), ("fallback", C.c_int32), ("residual_kind", C.c_int32)]


class NewmarkOptsC(C.Structure):
    _fields_ = [("num_steps", C.c_int32), ("del_t", C.c_double), ("nm_beta", C.c_double), ("nm_gamma", C.c_double),
                ("restart", C.c_int32), ("max_iters", C.c_int32), ("rtol", C.c_double), ("method", C.c_int32),
                ("precond", C.POINTER(PrecondC))]


class NewmarkCasesOptsC(C.Structure):
    _fields_ = [("num_steps", C.c_int32), ("num_cases", C.c_int32), ("del_t", C.c_double), ("nm_beta", C.c_double),
                ("nm_gamma", C.c_double), ("method", C.c_int32), ("no_graph", C.c_int32), ("refine", C.c_int32),
                ("autotune", C.c_int32)]


class NewmarkCasesInfoC(C.Structure):
    _fields_ = [("factor_seconds", C.c_double), ("prepare_seconds", C.c_double), ("step_seconds", C.c_double),
                ("last_rel_residual", C.c_double), ("band_bytes", C.c_int64), ("df_band_bytes", C.c_int64),
                ("bandwidth", C.c_int32), ("panels", C.c_int32), ("graph_nodes", C.c_int32),
                ("kernels_per_step", C.c_int32), ("cluster_size", C.c_int32)]


NMC_FACTORED = 0
TUNE_BRICK_WARPS, TUNE_PANEL_CLUSTER, TUNE_CASES_CLUSTER = 1, 2, 4


def lib_path():
    """The in-tree library; with ASTRO_BOUNDS_CHECK=1 in the environment, the checked build
    (device index guards that return ASTRO_ERR_BOUNDS instead of touching memory out of bounds)."""
    name = "libastro_gpu_checked.so" if os.environ.get("ASTRO_BOUNDS_CHECK") else "libastro_gpu.so"
    return os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", name)


def load_library():
    """Loads the in-tree libastro_gpu.so (built by misc_gb300/build.py or __graft_entry__.build())."""
    global _LIB
    if _LIB is not None:
        return _LIB
    p = lib_path()
    if not os.path.exists(p):
        raise RuntimeError(f"libastro_gpu.so not built ({p}); run __graft_entry__.build()")
    L = C.CDLL(p)
    vp = C.c_void_p
    sig = {
        "astro_ctx_create": ([vp, C.POINTER(vp)], C.c_int),
        "astro_ctx_destroy": ([vp], C.c_int),
        "astro_last_error": ([vp, C.c_char_p, C.c_int32], C.c_int),
        "astro_get_dims": ([vp, C.POINTER(DimsC)], C.c_int),
        "astro_get_prep": ([vp, I32P, I32P, I32P, I32P, I32P, I32P, F64P, F64P], C.c_int),
        "astro_el_soln_load": ([vp, C.c_int32, vp, F64P, F64P, F64P, I32P, F64P], C.c_int),
        "astro_assemble_fp32": ([vp], C.c_int),
        "astro_assemble_fp32_async": ([vp], C.c_int),
        "astro_element_matrices": ([vp, C.c_int32, vp, F64P, F64P], C.c_int),
        "astro_drdd_complex": ([vp, C.c_int32, C.c_double, vp, F64P, F64P], C.c_int),
        "astro_design_node_load": ([vp, C.c_double, F64P], C.c_int),
        "astro_node_load_drdd": ([vp, C.c_int32, C.c_double, F64P], C.c_int),
        "astro_scale_mpc": ([vp, F64P, F64P], C.c_int),
        "astro_constraint_load": ([vp, F64P, F64P], C.c_int),
        "astro_surface_load": ([vp, C.c_int32, I32P, I32P, F64P, C.c_double, F64P], C.c_int),
        "astro_body_load": ([vp, C.c_int32, F64P, I32P, C.c_int32, C.c_void_p, F64P], C.c_int),
        "astro_body_load_drdd": ([vp, C.c_int32, C.c_double, C.c_int32, F64P, I32P, C.c_int32, C.c_void_p, F64P],
                                 C.c_int),
        "astro_drdd_complex_condensed": ([vp, C.c_int32, I32P, C.c_double, vp, F64P], C.c_int),
        "astro_thermal_setup": ([vp, C.POINTER(ThermalPropsC), I32P, I32P], C.c_int),
        "astro_thermal_soln_load": ([vp, C.c_int32, C.POINTER(ThermalStateC), F64P, F64P, I32P], C.c_int),
        "astro_thermal_scale_mpc": ([vp, F64P, F64P], C.c_int),
        "astro_thermal_constraint_load": ([vp, F64P, F64P], C.c_int),
        "astro_thermal_heat_gen": ([vp, C.c_double, I32P, C.c_int32, F64P], C.c_int),
        "astro_thermal_surface_flux": ([vp, C.c_int32, I32P, I32P, C.c_double, F64P], C.c_int),
        "astro_thermal_solve": ([vp, F64P, F64P, C.c_double, C.c_int32, C.POINTER(SolveStatsC)], C.c_int),
        "astro_thermal_drdd": ([vp, C.c_int32, C.c_double, C.POINTER(ThermalStateC), F64P], C.c_int),
        "astro_thermal_heat_gen_drdd": ([vp, C.c_int32, C.c_double, C.c_double, I32P, C.c_int32, F64P], C.c_int),
        "astro_thermal_surface_flux_drdd": ([vp, C.c_int32, C.c_double, C.c_int32, I32P, I32P, C.c_double, F64P],
                                            C.c_int),
        "astro_thermal_design_node_load": ([vp, C.c_double, F64P], C.c_int),
        "astro_thermal_node_load_drdd": ([vp, C.c_int32, C.c_double, F64P], C.c_int),
        "astro_panels_factor": ([vp, C.c_int32, C.POINTER(PanelsInfoC)], C.c_int),
        "astro_panels_solve": ([vp, C.c_int32, F64P, F64P, C.POINTER(PanelsInfoC)], C.c_int),
        "astro_panels_solve_batched": ([vp, C.c_int32, F64P, F64P, C.POINTER(PanelsInfoC)], C.c_int),
        "astro_convert_to_ltri": ([vp, F64P], C.c_int),
        "astro_ldl_fact": ([vp, F64P, C.c_int32, I32P, C.c_int32], C.c_int),
        "astro_ldl_fact_resident": ([vp], C.c_int),
        "astro_ldl_solve": ([vp, F64P, F64P, F64P, C.c_int32, I32P, C.c_int32, F64P], C.c_int),
        "astro_gmres": ([vp, F64P, F64P, I32P, I32P, C.c_int32, C.c_int32, F64P, I32P, I32P, C.c_int32, C.c_int32,
                         F64P, I32P, C.c_int32, F64P, C.c_int32, C.c_int32], C.c_int),
        "astro_solve_static": ([vp, F64P, F64P, C.POINTER(SolveOptsC), C.POINTER(SolveStatsC)], C.c_int),
        "astro_apply_operator": ([vp, C.c_int32, F64P, F64P], C.c_int),
        "astro_ctx_stream": ([vp], C.c_void_p),
        "astro_update_external_rhs": ([vp, F64P, F64P], C.c_int),
        "astro_newmark_run": ([vp, C.POINTER(NewmarkOptsC), F64P, F64P, F64P, F64P, F64P, F64P, F64P,
                               C.POINTER(SolveStatsC)], C.c_int),
        "astro_node_features": ([vp, C.c_int32, F64P], C.c_int),
        "astro_precond_mlp_scales": ([vp, C.c_int32, C.POINTER(PrecondMlpC), F64P], C.c_int),
        "astro_precond_mlp_loss_grad": ([vp, C.POINTER(PrecondC), C.POINTER(PrecondMlpC), F64P, C.c_int32, F64P, F64P,
                                         C.POINTER(PrecondMlpC)], C.c_int),
        "astro_newmark_run_states": ([vp, C.POINTER(NewmarkOptsC), F64P, F64P, F64P, F64P, F64P, F64P, F64P, F64P,
                                      F64P, F64P, C.POINTER(SolveStatsC)], C.c_int),
        "astro_autotune": ([vp, C.c_int32, C.c_char_p, C.POINTER(C.c_int32)], C.c_int),
        "astro_newmark_cases": ([vp, C.POINTER(NewmarkCasesOptsC), F64P, F64P, F64P, F64P, F64P, F64P,
                                 C.POINTER(NewmarkCasesInfoC)], C.c_int),
        "astro_update_internal_soln": ([vp, F64P, F64P, F64P], C.c_int),
        "astro_precond_init": ([C.c_int32, C.c_double, C.c_int32, C.POINTER(PrecondC)], C.c_int),
        "astro_precond_lambda": ([vp, C.c_int32, F64P], C.c_int),
        "astro_precond_loss_grad": ([vp, C.POINTER(PrecondC), F64P, C.c_int32, F64P, F64P], C.c_int),
        "astro_precond_train": ([vp, C.POINTER(PrecondC), F64P, C.c_int32, C.c_int32, F64P], C.c_int),
        "astro_precond_time_hop": ([vp, C.c_int32, F64P, F64P], C.c_int),
        "astro_total_dldd_transient": ([vp, C.POINTER(TransientAdjointC), F64P, F64P, C.POINTER(SolveStatsC)],
                                       C.c_int),
        "astro_write_step_file": ([C.c_char_p, C.c_int32, C.c_int32, C.c_int32, F64P, F64P, F64P, F64P, F64P, F64P],
                                  C.c_int),
        "astro_read_step_file": ([C.c_char_p, C.c_int32, C.c_int32, C.c_int32, F64P, F64P, F64P, F64P, F64P, F64P],
                                 C.c_int),
        "astro_step_solve": ([vp, C.POINTER(StepOptsC), F64P, F64P, F64P, I32P, C.POINTER(SolveStatsC)], C.c_int),
        "astro_total_dldd": ([vp, vp, C.c_double, F64P, F64P, F64P, C.POINTER(SolveOptsC), F64P, F64P, F64P,
                              C.POINTER(SolveStatsC)], C.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _LIB = L
    return L


def _p(a, t):
    return C.cast(None, t) if a is None else a.ctypes.data_as(t)


def _d(a):
    return _p(a, F64P)


def _i(a):
    return _p(a, I32P)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def write_step_file(path, num_nodes, disp, vel, acc, int_disp=None, temp=None, tdot=None):
    """SolutionHistory<i>.out in the reference's record layout (writeBinarySolution)."""
    disp, vel, acc = _f64(disp), _f64(vel), _f64(acc)
    ni = 0 if int_disp is None else len(int_disp)
    rc = load_library().astro_write_step_file(str(path).encode(), num_nodes, len(disp), ni,
                                              None if temp is None else _d(_f64(temp)),
                                              None if tdot is None else _d(_f64(tdot)), _d(disp),
                                              None if int_disp is None else _d(_f64(int_disp)), _d(vel), _d(acc))
    if rc != ASTRO_OK:
        raise AstroError(rc, f"cannot write {path}")


def read_step_file(path, num_nodes, el_mat_dim, int_vec_size=0):
    """(temp, tdot, disp, int_disp, vel, acc) of a SolutionHistory<i>.out file (readBinarySolution)."""
    t, td = np.zeros(max(num_nodes, 1)), np.zeros(max(num_nodes, 1))
    u, v, a = np.zeros(el_mat_dim), np.zeros(el_mat_dim), np.zeros(el_mat_dim)
    iu = np.zeros(max(int_vec_size, 1))
    rc = load_library().astro_read_step_file(str(path).encode(), num_nodes, el_mat_dim, int_vec_size, _d(t), _d(td),
                                             _d(u), _d(iu), _d(v), _d(a))
    if rc != ASTRO_OK:
        raise AstroError(rc, f"cannot read {path}")
    return t[:num_nodes], td[:num_nodes], u, iu[:int_vec_size], v, a


def precond_init(degree=24, ratio=3000.0, dpn=3):
    """Untrained polynomial preconditioner: W_k = c_k I from the Chebyshev least-squares fit of 1/nu."""
    p = PrecondC()
    rc = load_library().astro_precond_init(degree, ratio, dpn, C.byref(p))
    if rc != ASTRO_OK:
        raise AstroError(rc, "astro_precond_init: bad degree, ratio or dpn")
    return p


class AstroGPU:
    """One model resident on the GPU (astro_ctx).  Construction runs analysisPrep."""

    def __init__(self, model: Model):
        self.L = load_library()
        self.model = model
        self._mc = model.as_c()
        h = C.c_void_p()
        rc = self.L.astro_ctx_create(C.byref(self._mc), C.byref(h))
        if rc != ASTRO_OK:
            raise AstroError(rc, self._err(None))
        self.h = h
        d = DimsC()
        self._check(self.L.astro_get_dims(self.h, C.byref(d)))
        self.dims = d
        self.n = d.el_mat_dim
        self.el_mat_size = d.el_mat_size
        self.lt_size = d.el_mat_lt_size
        self.mpc_dim = d.el_mpc_dim
        self.mpc_size = d.el_mpc_size
        self.int_vec_size = d.int_vec_size
        self.int_mat_size = d.int_mat_size
        self.solver_max_bw = d.solver_max_bw
        N = model.num_nodes
        self.current_rank = np.zeros(N, np.int32)
        self.n_dof_index = np.zeros((N, 6), np.int32)
        self.el_mat_range = np.zeros(self.n + 1, np.int32)
        self.lt_range = np.zeros(self.n + 1, np.int32)
        self.mpc_range = np.zeros(self.mpc_dim + 1, np.int32)
        self.mpc_cols = np.zeros(max(self.mpc_size, 1), np.int32)
        self.mpc_mat = np.zeros(max(self.mpc_size, 1))
        self.mpc_rhs = np.zeros(max(self.mpc_dim, 1))
        self._check(self.L.astro_get_prep(self.h, _i(self.current_rank), _i(self.n_dof_index), _i(self.el_mat_range),
                                          _i(self.lt_range), _i(self.mpc_range), _i(self.mpc_cols),
                                          _d(self.mpc_mat), _d(self.mpc_rhs)))

    # -- plumbing -------------------------------------------------------------------------------
    def _err(self, h):
        buf = C.create_string_buffer(512)
        self.L.astro_last_error(h, buf, 512)
        return buf.value.decode(errors="replace")

    def _check(self, rc, allow=()):
        if rc != ASTRO_OK and rc not in allow:
            raise AstroError(rc, self._err(self.h))
        return rc

    def close(self):
        if getattr(self, "h", None):
            self.L.astro_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- getElasticSolnLoad -----------------------------------------------------------------------
    def getElasticSolnLoad(self, buildMat=1, state=None, elastic_load=None, int_elastic_load=None, export=True):
        """Working/AStrO_commandFunctions.f90:260.  Returns (elasticLoad, intElasticLoad, elasticMat,
        elMatCols, intElasticMat); loads are accumulated (-= Ru) into the given arrays."""
        load = np.zeros(self.n) if elastic_load is None else elastic_load
        iload = np.zeros(max(self.int_vec_size, 1)) if int_elastic_load is None else int_elastic_load
        mat = cols = imat = None
        if buildMat == 1 and export:
            mat = np.zeros(self.el_mat_size)
            cols = np.zeros(self.el_mat_size, np.int32)
            imat = np.zeros(max(self.int_mat_size, 1))
        self._check(self.L.astro_el_soln_load(self.h, buildMat, C.byref(state) if state is not None else None,
                                              _d(load), _d(iload), _d(mat), _i(cols), _d(imat)))
        return load, iload, mat, cols, imat

    def assemble_fp32(self):
        self._check(self.L.astro_assemble_fp32(self.h))

    def element_matrices(self, precision=64, state=None, with_residual=False):
        E = self.model.num_els
        ke = np.zeros((E, 24, 24))
        ru = np.zeros((E, 24)) if with_residual else None
        self._check(self.L.astro_element_matrices(self.h, precision, C.byref(state) if state is not None else None,
                                                  _d(ke), _d(ru)))
        ke = np.transpose(ke, (0, 2, 1)).copy()  # column-major per element
        return (ke, ru) if with_residual else ke

    # -- constraints and loads ------------------------------------------------------------------
    def scaleElasticMPC(self):
        mm = np.zeros(max(self.mpc_size, 1))
        mr = np.zeros(max(self.mpc_dim, 1))
        self._check(self.L.astro_scale_mpc(self.h, _d(mm), _d(mr)))
        return mm[:self.mpc_size], mr[:self.mpc_dim]

    def getElasticConstraintLoad(self, node_disp, elastic_load):
        self._check(self.L.astro_constraint_load(self.h, _d(_f64(node_disp)) if node_disp is not None else None,
                                                 _d(elastic_load)))
        return elastic_load

    def surface_load(self, face_el, face_num, traction=(0.0, 0.0, 0.0), pressure=0.0, elastic_load=None):
        load = np.zeros(self.n) if elastic_load is None else elastic_load
        fe, fn = _i32(face_el), _i32(face_num)
        tr = _f64(traction)
        self._check(self.L.astro_surface_load(self.h, len(fe), _i(fe), _i(fn), _d(tr), float(pressure), _d(load)))
        return load

    def body_load(self, kind, vals, elements=None, state=None, elastic_load=None):
        """getElasticAppliedLoad body-force branch: kind 0 bodyForce, 1 gravitational, 2 centrifugal
        (vals = axis point, axis direction, angular velocity) over the listed 1-based elements
        (None = every element), added into elastic_load."""
        load = np.zeros(self.n) if elastic_load is None else elastic_load
        v = np.zeros(7)
        v[:len(vals)] = vals
        els = None if elements is None else _i32(elements)
        self._check(self.L.astro_body_load(self.h, int(kind), _d(v), None if els is None else _i(els),
                                           0 if els is None else len(els),
                                           C.byref(state) if state is not None else None, _d(load)))
        return load

    def body_load_drdd(self, dvar, kind, vals, elements=None, state=None, drudd=None, h=1e-14):
        """drudd -= d(body load)/d(design variable dvar) (the load branch of getdRelasticdD)."""
        out = np.zeros(self.n) if drudd is None else drudd
        v = np.zeros(7)
        v[:len(vals)] = vals
        els = None if elements is None else _i32(elements)
        self._check(self.L.astro_body_load_drdd(self.h, int(dvar), float(h), int(kind), _d(v),
                                                None if els is None else _i(els), 0 if els is None else len(els),
                                                C.byref(state) if state is not None else None, _d(out)))
        return out

    def applied_load(self, load=None):
        """Consistent surface load of the model's faces plus its point loads (getElasticAppliedLoad)."""
        m = self.model
        load = np.zeros(self.n) if load is None else load
        if len(m.face_el):
            self.surface_load(m.face_el, m.face_num, m.traction, m.pressure, load)
        for nd, dof, v in m.point_loads:
            load[self.n_dof_index[nd - 1, dof - 1] - 1] += v
        return load

    # -- solves ---------------------------------------------------------------------------------
    def solve_static(self, f, u0=None, method=SOLVER_GMRES_JACOBI_FP64, restart=50, rtol=1e-10, max_iters=200000,
                     inner_rtol=1e-4, allow_maxit=False, precond=None, mlp=None):
        u = np.zeros(self.n) if u0 is None else _f64(u0).copy()
        o = SolveOptsC(method, restart, max_iters, rtol, inner_rtol,
                       C.pointer(precond) if precond is not None else C.POINTER(PrecondC)(),
                       C.pointer(mlp) if mlp is not None else C.POINTER(PrecondMlpC)())
        st = SolveStatsC()
        rc = self.L.astro_solve_static(self.h, _d(_f64(f)), _d(u), C.byref(o), C.byref(st))
        self._check(rc, allow=(7,) if allow_maxit else ())
        return u, st

    # -- thermal path ---------------------------------------------------------------------------
    def thermal_setup(self, props):
        ms, md = C.c_int32(), C.c_int32()
        self._thermal_props = props
        self._check(self.L.astro_thermal_setup(self.h, C.byref(props), C.byref(ms), C.byref(md)))
        self.therm_mat_size, self.therm_mpc_dim = ms.value, md.value
        return ms.value, md.value

    def getThermalSolnLoad(self, buildMat=1, state=None, thermal_load=None, export=True):
        """(thermal load in rank order, CSR values, CSR columns) of getThermalSolnLoad."""
        N = self.model.num_nodes
        load = np.zeros(N) if thermal_load is None else thermal_load
        mat = cols = None
        if buildMat == 1 and export:
            mat, cols = np.zeros(self.therm_mat_size), np.zeros(self.therm_mat_size, np.int32)
        self._check(self.L.astro_thermal_soln_load(self.h, int(buildMat), C.byref(state) if state is not None else None,
                                                   _d(load), _d(mat) if mat is not None else None,
                                                   _i(cols) if cols is not None else None))
        return load, mat, cols

    def scaleThermalMPC(self):
        k = max(self._thermal_props.num_mpc, 1)
        mm = np.zeros(max(int(self._thermal_props.mpc_range[k]) if self._thermal_props.num_mpc else 1, 1))
        mr = np.zeros(k)
        self._check(self.L.astro_thermal_scale_mpc(self.h, _d(mm), _d(mr)))
        return mm, mr

    def getThermalConstraintLoad(self, node_temp=None, thermal_load=None):
        load = np.zeros(self.model.num_nodes) if thermal_load is None else thermal_load
        self._check(self.L.astro_thermal_constraint_load(self.h, None if node_temp is None else _d(_f64(node_temp)),
                                                         _d(load)))
        return load

    def thermal_heat_gen(self, q, elements=None, thermal_load=None):
        load = np.zeros(self.model.num_nodes) if thermal_load is None else thermal_load
        els = None if elements is None else _i32(elements)
        self._check(self.L.astro_thermal_heat_gen(self.h, float(q), None if els is None else _i(els),
                                                  0 if els is None else len(els), _d(load)))
        return load

    def thermal_surface_flux(self, face_el, face_num, flux, thermal_load=None):
        load = np.zeros(self.model.num_nodes) if thermal_load is None else thermal_load
        fe, fn = _i32(face_el), _i32(face_num)
        self._check(self.L.astro_thermal_surface_flux(self.h, len(fe), _i(fe), _i(fn), float(flux), _d(load)))
        return load

    def thermal_solve(self, rhs, dtemp0=None, rtol=1e-12, max_iters=100000):
        x = np.zeros(self.model.num_nodes) if dtemp0 is None else _f64(dtemp0).copy()
        st = SolveStatsC()
        self._check(self.L.astro_thermal_solve(self.h, _d(_f64(rhs)), _d(x), float(rtol), int(max_iters),
                                               C.byref(st)))
        return x, st

    def thermal_drdd(self, dvar, h=1e-14, state=None):
        """getdRthermaldD element part: dRt/d(dvar) in rank order by the device complex step."""
        out = np.zeros(self.model.num_nodes)
        self._check(self.L.astro_thermal_drdd(self.h, int(dvar), float(h), C.byref(state) if state is not None else None,
                                              _d(out)))
        return out

    def thermal_heat_gen_drdd(self, dvar, q, elements=None, h=1e-14, drtdd=None):
        drtdd = np.zeros(self.model.num_nodes) if drtdd is None else drtdd
        els = None if elements is None else _i32(elements)
        self._check(self.L.astro_thermal_heat_gen_drdd(self.h, int(dvar), float(h), float(q),
                                                       None if els is None else _i(els), 0 if els is None else len(els),
                                                       _d(drtdd)))
        return drtdd

    def thermal_surface_flux_drdd(self, dvar, face_el, face_num, flux, h=1e-14, drtdd=None):
        drtdd = np.zeros(self.model.num_nodes) if drtdd is None else drtdd
        fe, fn = _i32(face_el), _i32(face_num)
        self._check(self.L.astro_thermal_surface_flux_drdd(self.h, int(dvar), float(h), len(fe), _i(fe), _i(fn),
                                                           float(flux), _d(drtdd)))
        return drtdd

    def thermal_design_node_load(self, t, thermal_load=None):
        load = np.zeros(self.model.num_nodes) if thermal_load is None else thermal_load
        self._check(self.L.astro_thermal_design_node_load(self.h, float(t), _d(load)))
        return load

    def thermal_node_load_drdd(self, dvar, t, drtdd=None):
        drtdd = np.zeros(self.model.num_nodes) if drtdd is None else drtdd
        self._check(self.L.astro_thermal_node_load_drdd(self.h, int(dvar), float(t), _d(drtdd)))
        return drtdd

    def panels_factor(self, cluster_size=0):
        """Band LDL^T of K + C^T C of every panel (connected component) in one launch."""
        info = PanelsInfoC()
        self._check(self.L.astro_panels_factor(self.h, int(cluster_size), C.byref(info)))
        return info

    def panels_solve(self, B, batched=False):
        """X = (K + C^T C)^-1 B for the columns of B (n x k or n), with the panel factors."""
        one = np.ndim(B) == 1
        # column k of B contiguous (Fortran order) is the C ABI's layout: no copy when B has it
        Bf = np.asfortranarray(np.asarray(B, dtype=np.float64).reshape(self.n, -1))
        X = np.empty(Bf.shape, dtype=np.float64, order="F")
        info = PanelsInfoC()
        fn = self.L.astro_panels_solve_batched if batched else self.L.astro_panels_solve
        self._check(fn(self.h, Bf.shape[1], _d(Bf), _d(X), C.byref(info)))
        return (X[:, 0] if one else X), info

    def apply_operator(self, x, kind=64):
        y = np.zeros(self.n)
        self._check(self.L.astro_apply_operator(self.h, kind, _d(_f64(x)), _d(y)))
        return y

    def convertToLTri(self):
        lt = np.zeros(self.lt_size)
        self._check(self.L.astro_convert_to_ltri(self.h, _d(lt)))
        return lt

    def getSparseLDLFact(self, a_l_tri, a_range):
        a = _f64(a_l_tri).copy()
        r = _i32(a_range)
        self._check(self.L.astro_ldl_fact(self.h, _d(a), len(a), _i(r), len(r) - 1))
        return a

    def solveSparseLDLFact(self, rhs, l_mat, l_range):
        n = len(l_range) - 1
        x = np.zeros(n)
        z = np.zeros(n)
        lm = _f64(l_mat)
        self._check(self.L.astro_ldl_solve(self.h, _d(x), _d(_f64(rhs)), _d(lm), len(lm), _i(_i32(l_range)), n, _d(z)))
        return x

    def gMRes(self, x_vec, a_mat, a_cols, a_range, c_mat, c_cols, c_range, p_mat, p_range, b_vec, num_vecs, max_it):
        x = _f64(x_vec).copy()
        am, ac, ar = _f64(a_mat), _i32(a_cols), _i32(a_range)
        cm, cc, cr = _f64(c_mat), _i32(c_cols), _i32(c_range)
        pm, pr = _f64(p_mat), _i32(p_range)
        self._check(self.L.astro_gmres(self.h, _d(x), _d(am), _i(ac), _i(ar), len(am), len(ar) - 1, _d(cm), _i(cc),
                                       _i(cr), len(cm), len(cr) - 1, _d(pm), _i(pr), len(pm), _d(_f64(b_vec)),
                                       num_vecs, max_it))
        return x

    def updateExternalRHS(self, ext_vec, int_vec):
        """ext_vec -= K_ni K_ii^-1 int_vec over the elements with internal DOF (returns a new array)."""
        out = _f64(ext_vec).copy()
        self._check(self.L.astro_update_external_rhs(self.h, _d(out), _d(_f64(int_vec))))
        return out

    def updateInternalSoln(self, ext_soln, int_soln, int_rhs=None):
        """int_soln + K_ii^-1 (int_rhs - K_in ext_soln) over the elements with internal DOF (new array)."""
        out = _f64(int_soln).copy()
        rhs = None if int_rhs is None else _d(_f64(int_rhs))
        self._check(self.L.astro_update_internal_soln(self.h, _d(_f64(ext_soln)), _d(out), rhs))
        return out

    def newmark_run(self, num_steps, del_t, beta=0.25, gamma=0.5, load_pattern=None, load_amplitude=None, disp=None,
                    vel=None, acc=None, int_disp=None, restart=50, max_iters=2000, rtol=1e-12, history=True,
                    method=SOLVER_GMRES_JACOBI_FP64, precond=None):
        """solve() dynamic branch on the device: returns (disp, vel, acc, int_disp, history, stats)."""
        n, ni = self.n, self.int_vec_size
        u = np.zeros(n) if disp is None else _f64(disp).copy()
        v = np.zeros(n) if vel is None else _f64(vel).copy()
        a = np.zeros(n) if acc is None else _f64(acc).copy()
        iu = np.zeros(max(ni, 1)) if int_disp is None else _f64(int_disp).copy()
        hist = np.zeros((num_steps, n)) if history else None
        o = NewmarkOptsC(num_steps, del_t, beta, gamma, restart, max_iters, rtol, method,
                         C.pointer(precond) if precond is not None else C.POINTER(PrecondC)())
        st = SolveStatsC()
        pat = None if load_pattern is None else _d(_f64(load_pattern))
        amp = None if load_amplitude is None else _d(_f64(load_amplitude))
        self._check(self.L.astro_newmark_run(self.h, C.byref(o), pat, amp, _d(u), _d(v), _d(a), _d(iu),
                                             _d(hist) if history else None, C.byref(st)))
        return u, v, a, iu[:ni], hist, st

    def newmark_cases(self, del_t, patterns, amplitudes, beta=0.25, gamma=0.5, disp=None, vel=None, acc=None,
                      history=False, graph=True, method=NMC_FACTORED, refine=0, autotune=False):
        """Batched linear Newmark (astro_newmark_cases): patterns (cases, n), amplitudes (cases,
        steps) in global DOF numbering; returns (disp, vel, acc, history or None, info), states
        (cases, n), history (steps, cases, n)."""
        P = np.ascontiguousarray(patterns, dtype=np.float64)
        Am = np.ascontiguousarray(amplitudes, dtype=np.float64)
        nc, n = P.shape
        steps = Am.shape[1]
        assert n == self.n and Am.shape[0] == nc
        u = np.zeros((nc, n)) if disp is None else np.ascontiguousarray(disp, dtype=np.float64).copy()
        v = np.zeros((nc, n)) if vel is None else np.ascontiguousarray(vel, dtype=np.float64).copy()
        a = np.zeros((nc, n)) if acc is None else np.ascontiguousarray(acc, dtype=np.float64).copy()
        hist = np.zeros((steps, nc, n)) if history else None
        o = NewmarkCasesOptsC(steps, nc, del_t, beta, gamma, method, 0 if graph else 1, refine, 1 if autotune else 0)
        info = NewmarkCasesInfoC()
        self._check(self.L.astro_newmark_cases(self.h, C.byref(o), _d(P), _d(Am), _d(u), _d(v), _d(a),
                                               _d(hist) if history else None, C.byref(info)))
        return u, v, a, hist, info

    def newmark_run_states(self, num_steps, del_t, beta=0.25, gamma=0.5, load_pattern=None, load_amplitude=None,
                           disp=None, vel=None, acc=None, int_disp=None, restart=50, max_iters=2000, rtol=1e-12,
                           method=SOLVER_GMRES_JACOBI_FP64, precond=None):
        """newmark_run returning every step's state (astro_newmark_run_states): (disp, vel, acc,
        int_disp, histories {disp, vel, acc (steps, n), int_disp (steps, int_vec_size)}, stats)."""
        n, ni = self.n, self.int_vec_size
        u = np.zeros(n) if disp is None else _f64(disp).copy()
        v = np.zeros(n) if vel is None else _f64(vel).copy()
        a = np.zeros(n) if acc is None else _f64(acc).copy()
        iu = np.zeros(max(ni, 1)) if int_disp is None else _f64(int_disp).copy()
        H = {"disp": np.zeros((num_steps, n)), "vel": np.zeros((num_steps, n)), "acc": np.zeros((num_steps, n)),
             "int_disp": np.zeros((num_steps, max(ni, 1)))}
        o = NewmarkOptsC(num_steps, del_t, beta, gamma, restart, max_iters, rtol, method,
                         C.pointer(precond) if precond is not None else C.POINTER(PrecondC)())
        st = SolveStatsC()
        pat = None if load_pattern is None else _d(_f64(load_pattern))
        amp = None if load_amplitude is None else _d(_f64(load_amplitude))
        self._check(self.L.astro_newmark_run_states(self.h, C.byref(o), pat, amp, _d(u), _d(v), _d(a), _d(iu),
                                                    _d(H["disp"]), _d(H["vel"]), _d(H["acc"]),
                                                    _d(H["int_disp"]) if ni else None, C.byref(st)))
        H["int_disp"] = H["int_disp"][:, :ni]
        return u, v, a, iu[:ni], H, st

    def autotune(self, what, cache_path=None):
        """astro_autotune: what = a sum of TUNE_* flags; returns the context's choices (brick warps
        per CTA, panel cluster size, many-column solve cluster size; 0 = default)."""
        ch = (C.c_int32 * 3)()
        self._check(self.L.astro_autotune(self.h, int(what), None if cache_path is None else str(cache_path).encode(),
                                          ch))
        return tuple(int(x) for x in ch)

    def getdRelasticdD(self, dvar, h=1e-14, state=None):
        """Complex-step dRu/dd of design variable dvar: (global DOF vector, internal-DOF vector)."""
        out = np.zeros(self.n)
        iout = np.zeros(max(self.int_vec_size, 1))
        self._check(self.L.astro_drdd_complex(self.h, dvar, h, C.byref(state) if state is not None else None,
                                              _d(out), _d(iout)))
        return out, iout[:self.int_vec_size]

    def design_node_load(self, time, elastic_load=None):
        """The nodal design loads active at time, added to elastic_load (returns a new array)."""
        out = np.zeros(self.n) if elastic_load is None else _f64(elastic_load).copy()
        self._check(self.L.astro_design_node_load(self.h, float(time), _d(out)))
        return out

    def node_load_drdd(self, dvar, time, drudd=None):
        """drudd - d(nodal design load)/d(dvar) at time (returns a new array)."""
        out = np.zeros(self.n) if drudd is None else _f64(drudd).copy()
        self._check(self.L.astro_node_load_drdd(self.h, int(dvar), float(time), _d(out)))
        return out

    def drdd_condensed(self, dvars, h=1e-14, state=None):
        """Condensed complex-step dRu/dd of the listed design variables: (n, len(dvars)), Fortran
        order (the right-hand-side layout of panels_solve)."""
        dv = _i32(dvars)
        out = np.empty((self.n, len(dv)), dtype=np.float64, order="F")
        self._check(self.L.astro_drdd_complex_condensed(self.h, len(dv), _i(dv), float(h),
                                                        C.byref(state) if state is not None else None, _d(out)))
        return out

    def stepSolve(self, applied_load, node_disp=None, internal_disp=None, nl_geom=0, method=SOLVER_GMRES_JACOBI_FP64,
                  rtol=1e-12, restart=50, max_iters=200000, precond=None):
        """stepSolve on the device (needs getElasticSolnLoad(1) and scaleElasticMPC first):
        (node_disp, internal_disp, Newton iterations, stats)."""
        u = np.zeros(self.n) if node_disp is None else _f64(node_disp).copy()
        iu = np.zeros(max(self.int_vec_size, 1)) if internal_disp is None else _f64(internal_disp).copy()
        o = StepOptsC(nl_geom, SolveOptsC(method, restart, max_iters, rtol, 1e-4,
                                          C.pointer(precond) if precond is not None else C.POINTER(PrecondC)()))
        its = np.zeros(1, np.int32)
        st = SolveStatsC()
        self._check(self.L.astro_step_solve(self.h, C.byref(o), None if applied_load is None else _d(_f64(applied_load)),
                                            _d(u), _d(iu), _i(its), C.byref(st)))
        return u, iu[:self.int_vec_size], int(its[0]), st

    def getTotaldLdD(self, dldu, int_dldu=None, dldd_explicit=None, state=None, h=1e-14,
                     method=SOLVER_GMRES_JACOBI_FP64, rtol=1e-12, restart=50, max_iters=200000, precond=None):
        """Static design gradient: (dLdD, dispAdj, intDispAdj, stats) with the adjoint solved on the
        device (needs getElasticSolnLoad(1) at the state and scaleElasticMPC first)."""
        nd = len(self.model.d_value) if getattr(self.model, "d_value", None) is not None else 0
        dldd = np.zeros(max(nd, 1))
        lam = np.zeros(self.n)
        ilam = np.zeros(max(self.int_vec_size, 1))
        o = SolveOptsC(method, restart, max_iters, rtol, 1e-4,
                       C.pointer(precond) if precond is not None else C.POINTER(PrecondC)())
        st = SolveStatsC()
        self._check(self.L.astro_total_dldd(self.h, C.byref(state) if state is not None else None, h, _d(_f64(dldu)),
                                            None if int_dldu is None else _d(_f64(int_dldu)),
                                            None if dldd_explicit is None else _d(_f64(dldd_explicit)),
                                            C.byref(o), _d(dldd), _d(lam), _d(ilam), C.byref(st)))
        return dldd[:nd], lam, ilam[:self.int_vec_size], st

    def getTotaldLdD_transient(self, disp, vel, acc, int_disp, del_t, beta=0.25, gamma=0.5, dldu=None, dldv=None,
                               dlda=None, int_dldu=None, dldd_explicit=None, h=1e-14,
                               method=SOLVER_GMRES_JACOBI_FP64, rtol=1e-12, restart=50, max_iters=200000):
        """Transient design gradient over stored Newmark states (rows 0..N of disp/vel/acc/int_disp)
        and per-step objective partials (rows 0..N-1 for t_1..t_N): (dLdD, adjoint of step 1, stats)."""
        N = np.asarray(disp).shape[0] - 1
        nd = len(self.model.d_value) if getattr(self.model, "d_value", None) is not None else 0
        keep = []

        def arr(x):
            if x is None:
                return None
            a = np.ascontiguousarray(x, np.float64)
            keep.append(a)
            return _d(a)

        a = TransientAdjointC(N, del_t, beta, gamma, h, arr(disp), arr(vel), arr(acc), arr(int_disp), arr(dldu),
                              arr(dldv), arr(dlda), arr(int_dldu), arr(dldd_explicit),
                              SolveOptsC(method, restart, max_iters, rtol, 1e-4, C.POINTER(PrecondC)()))
        dldd = np.zeros(max(nd, 1))
        lam = np.zeros(self.n)
        st = SolveStatsC()
        self._check(self.L.astro_total_dldd_transient(self.h, C.byref(a), _d(dldd), _d(lam), C.byref(st)))
        return dldd[:nd], lam, st

    # -- polynomial preconditioner ----------------------------------------------------------------
    def precond_lambda(self, kind=64):
        lam = np.zeros(1)
        self._check(self.L.astro_precond_lambda(self.h, kind, _d(lam)))
        return float(lam[0])

    def precond_loss_grad(self, p, samples):
        """(loss, gradient (degree + 1, dpn, dpn)) of the network p on samples (S x el_mat_dim)."""
        S = _f64(samples).reshape(-1, self.n)
        loss = np.zeros(1)
        g = np.zeros((p.degree + 1) * p.dpn * p.dpn)
        self._check(self.L.astro_precond_loss_grad(self.h, C.byref(p), _d(S), S.shape[0], _d(loss), _d(g)))
        return float(loss[0]), g.reshape(p.degree + 1, p.dpn, p.dpn)

    def node_features(self, kind=64):
        """Node features (num_nodes x NODE_FEATURES, row = node id - 1) of the resident assembly."""
        F = np.zeros((self.model.num_nodes, NODE_FEATURES))
        self._check(self.L.astro_node_features(self.h, kind, _d(F)))
        return F

    def mlp_scales(self, mlp, kind=64):
        """Per-node hop scales (num_nodes x outputs) of the perceptron."""
        A = np.zeros((self.model.num_nodes, mlp.outputs))
        self._check(self.L.astro_precond_mlp_scales(self.h, kind, C.byref(mlp), _d(A)))
        return A

    def mlp_loss_grad(self, p, mlp, samples):
        """(loss, gradient of the hop weights (degree + 1, dpn, dpn), gradient of the perceptron as
        a PrecondMlpC) of the modulated network on samples (S x el_mat_dim)."""
        S = _f64(samples).reshape(-1, self.n)
        loss = np.zeros(1)
        gw = np.zeros((p.degree + 1) * p.dpn * p.dpn)
        gm = PrecondMlpC()
        self._check(self.L.astro_precond_mlp_loss_grad(self.h, C.byref(p), C.byref(mlp), _d(S), S.shape[0], _d(loss),
                                                       _d(gw), C.byref(gm)))
        return float(loss[0]), gw.reshape(p.degree + 1, p.dpn, p.dpn), gm

    def precond_train(self, p, samples, iters=50):
        """Trains p in place; returns the loss history (iters + 1)."""
        S = _f64(samples).reshape(-1, self.n)
        hist = np.zeros(iters + 1)
        self._check(self.L.astro_precond_train(self.h, C.byref(p), _d(S), S.shape[0], iters, _d(hist)))
        return hist

    def precond_time_hop(self, reps=200):
        """(microseconds per hop, bytes per hop) on the operator of the last learned solve."""
        us, by = np.zeros(1), np.zeros(1)
        self._check(self.L.astro_precond_time_hop(self.h, reps, _d(us), _d(by)))
        return float(us[0]), float(by[0])

    def precond_train_validated(self, p, samples, iters=20, rhs=None, rtol=1e-8):
        """Trains a copy of p on samples, then solves this model (right-hand side rhs, default the
        static load; needs the FP32 assembly) with the learned solver under both weight sets and
        keeps the trained weights only when they need fewer Krylov iterations.  The quadratic
        training loss weights the spectrum by the samples, and a lower loss does not always mean
        faster GMRES convergence; the validation solve guards against that.
        Returns (network, info)."""
        q = PrecondC()
        C.memmove(C.byref(q), C.byref(p), C.sizeof(PrecondC))
        hist = self.precond_train(q, samples, iters)
        b = self.static_rhs() if rhs is None else rhs
        _, s0 = self.solve_static(b, method=SOLVER_FGMRES_LEARNED, rtol=rtol, precond=p, allow_maxit=True)
        _, s1 = self.solve_static(b, method=SOLVER_FGMRES_LEARNED, rtol=rtol, precond=q, allow_maxit=True)
        ok = s1.status == ASTRO_OK and (s0.status != ASTRO_OK or s1.iterations < s0.iterations)
        info = {"loss": [float(hist[0]), float(hist[-1])], "val_iters_initial": int(s0.iterations),
                "val_iters_trained": int(s1.iterations), "selected": "trained" if ok else "initial"}
        return (q if ok else p), info

    # -- convenience ----------------------------------------------------------------------------
    def static_rhs(self, mpc_rhs_scaled=True):
        """b = constraint load (zero displacement) + applied load, after scaleElasticMPC."""
        b = np.zeros(self.n)
        self.getElasticConstraintLoad(np.zeros(self.n), b)
        self.applied_load(b)
        return b


__all__ = ["AstroGPU", "AstroError", "load_library", "make_state", "AstroStateC", "SOLVER_GMRES_JACOBI_FP64",
           "thermal_props", "thermal_state",
           "SOLVER_FGMRES_MIXED", "SOLVER_FGMRES_LEARNED", "PrecondC", "precond_init", "PRECOND_MAX_DEGREE"]


def _set_option(self, option, value):
    self.L.astro_set_option.argtypes = [C.c_void_p, C.c_int32, C.c_int32]
    self.L.astro_set_option.restype = C.c_int
    self._check(self.L.astro_set_option(self.h, option, value))


AstroGPU.set_option = _set_option
OPT_SHELL_MEAN_ROT_TERM = 1
