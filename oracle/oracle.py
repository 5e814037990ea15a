"""ctypes wrapper of the oracle library (test infrastructure only)."""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

I32P = C.POINTER(C.c_int32)
F64P = C.POINTER(C.c_double)


def lib_path():
    return os.path.join(_HERE, "_build", "liborc.so")


def build(force=False):
    """Compiles the oracle with its Makefile (a few seconds)."""
    srcs = ["oracle_api.cpp", "oracle_elements.hpp", "oracle_element_driver.hpp"]
    out = lib_path()
    if not force and os.path.exists(out):
        t = os.path.getmtime(out)
        if all(os.path.getmtime(os.path.join(_HERE, s)) <= t for s in srcs):
            return out
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return out


def _lib():
    global _LIB
    if _LIB is None:
        build()
        L = C.CDLL(lib_path())
        L.orc_create.restype = C.c_void_p
        L.orc_create.argtypes = [C.c_void_p]
        L.orc_destroy.argtypes = [C.c_void_p]
        L.orc_dims.argtypes = [C.c_void_p, I32P]
        L.orc_get_prep.argtypes = [C.c_void_p, I32P, I32P, I32P, I32P, I32P, I32P, F64P, F64P]
        L.orc_element.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, F64P, F64P]
        L.orc_element_c.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_double,
                                    F64P, F64P, F64P, F64P]
        L.orc_element_matrices.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, F64P]
        L.orc_drdd_complex.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_void_p, F64P, F64P]
        L.orc_design_node_load.argtypes = [C.c_void_p, C.c_double, F64P]
        L.orc_node_load_drdd.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_double, F64P]
        L.orc_update_external_rhs.argtypes = [C.c_void_p, F64P, F64P, F64P]
        L.orc_update_internal_soln.argtypes = [C.c_void_p, F64P, F64P, F64P, F64P]
        L.orc_el_soln_load.argtypes = [C.c_void_p, C.c_int, C.c_void_p, F64P, F64P, F64P, I32P, F64P]
        L.orc_scale_mpc.argtypes = [F64P, C.c_int, F64P, F64P, I32P, C.c_int]
        L.orc_constraint_load.argtypes = [F64P, I32P, I32P, F64P, C.c_int, F64P, F64P]
        L.orc_convert_to_ltri.argtypes = [F64P, I32P, C.c_int, F64P, I32P, I32P, C.c_int, C.c_int,
                                          F64P, I32P, I32P, C.c_int, C.c_int]
        L.orc_ldl_fact.argtypes = [F64P, C.c_int, I32P, C.c_int]
        L.orc_ldl_solve.argtypes = [F64P, F64P, F64P, C.c_int, I32P, C.c_int, F64P]
        L.orc_gmres.restype = C.c_int
        L.orc_gmres.argtypes = [F64P, F64P, I32P, I32P, C.c_int, C.c_int, F64P, I32P, I32P, C.c_int, C.c_int,
                                F64P, I32P, C.c_int, F64P, C.c_int, C.c_int]
        L.orc_update_external_rhs.argtypes = [C.c_void_p, F64P, F64P, F64P]
        L.orc_update_internal_soln.argtypes = [C.c_void_p, F64P, F64P, F64P, F64P]
        L.orc_surface_load.argtypes = [C.c_void_p, C.c_int, I32P, I32P, F64P, C.c_double, F64P]
        L.orc_thermal_soln_load.restype = C.c_int
        L.orc_thermal_soln_load.argtypes = [C.c_void_p, F64P, F64P, C.c_int, F64P, F64P, F64P, C.c_int, C.c_double,
                                            C.c_double, F64P, F64P, I32P, I32P]
        L.orc_body_load.restype = C.c_int
        L.orc_body_load.argtypes = [C.c_void_p, C.c_int, F64P, C.c_int, I32P, C.c_void_p, F64P]
        L.orc_thermal_drdd.restype = C.c_int
        L.orc_thermal_drdd.argtypes = [C.c_void_p, F64P, F64P, C.c_int, C.c_double, F64P, F64P, F64P, C.c_int,
                                       C.c_double, C.c_double, F64P]
        L.orc_thermal_heat_gen_drdd.restype = C.c_int
        L.orc_thermal_heat_gen_drdd.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_int, I32P, F64P]
        L.orc_thermal_surface_flux_drdd.restype = C.c_int
        L.orc_thermal_surface_flux_drdd.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_int, I32P, I32P, C.c_double,
                                                    F64P]
        L.orc_thermal_design_node_load.argtypes = [C.c_void_p, C.c_double, F64P]
        L.orc_thermal_node_load_drdd.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_double, F64P]
        _LIB = L
    return _LIB


def _p(a, t):
    return C.cast(None, t) if a is None else a.ctypes.data_as(t)


def _i(a):
    return _p(a, I32P)


def _d(a):
    return _p(a, F64P)


class Oracle:
    """Analysis-prepared model on the CPU (reference analysisPrep) plus the hot-path routines."""

    def __init__(self, model):
        self.model = model
        self.mc = model.as_c()
        self.L = _lib()
        self.h = self.L.orc_create(C.byref(self.mc))
        if not self.h:
            raise ValueError("oracle: unsupported model")
        d = np.zeros(8, np.int32)
        self.L.orc_dims(self.h, _i(d))
        (self.n, self.el_mat_size, self.lt_size, self.mpc_dim, self.mpc_size, self.int_vec_size,
         self.int_mat_size, self.solver_max_bw) = [int(x) for x in d]
        N = model.num_nodes
        self.current_rank = np.zeros(N, np.int32)
        self.n_dof_index = np.zeros((N, 6), np.int32)
        self.el_mat_range = np.zeros(self.n + 1, np.int32)
        self.lt_range = np.zeros(self.n + 1, np.int32)
        self.mpc_range = np.zeros(self.mpc_dim + 1, np.int32)
        self.mpc_cols = np.zeros(self.mpc_size, np.int32)
        self.mpc_mat = np.zeros(self.mpc_size)
        self.mpc_rhs = np.zeros(self.mpc_dim)
        self.L.orc_get_prep(self.h, _i(self.current_rank), _i(self.n_dof_index), _i(self.el_mat_range),
                            _i(self.lt_range), _i(self.mpc_range), _i(self.mpc_cols), _d(self.mpc_mat),
                            _d(self.mpc_rhs))

    def __del__(self):
        try:
            if getattr(self, "h", None):
                self.L.orc_destroy(self.h)
        except Exception:
            pass

    # -- elements -------------------------------------------------------------------------------
    def element(self, el, build_mat=1, state=None):
        ru = np.zeros(33)
        k = np.zeros((33, 33), order="F")
        rc = self.L.orc_element(self.h, el, build_mat, C.byref(state) if state is not None else None, _d(ru),
                                k.ctypes.data_as(F64P))
        assert rc == 0
        return ru, k

    def element_c(self, el, dvar, h, build_mat=0, state=None):
        rr, ri = np.zeros(33), np.zeros(33)
        kr, ki = np.zeros((33, 33), order="F"), np.zeros((33, 33), order="F")
        rc = self.L.orc_element_c(self.h, el, build_mat, C.byref(state) if state is not None else None, dvar, h,
                                  _d(rr), _d(ri), kr.ctypes.data_as(F64P), ki.ctypes.data_as(F64P))
        assert rc == 0
        return rr + 1j * ri, kr + 1j * ki

    def update_external_rhs(self, ext_vec, int_vec, int_mat):
        out = np.ascontiguousarray(ext_vec, np.float64).copy()
        self.L.orc_update_external_rhs(self.h, _d(out), _d(np.ascontiguousarray(int_vec, np.float64)),
                                       _d(np.ascontiguousarray(int_mat, np.float64)))
        return out

    def update_internal_soln(self, ext_soln, int_soln, int_rhs, int_mat):
        out = np.ascontiguousarray(int_soln, np.float64).copy()
        rhs = None if int_rhs is None else _d(np.ascontiguousarray(int_rhs, np.float64))
        self.L.orc_update_internal_soln(self.h, _d(np.ascontiguousarray(ext_soln, np.float64)), _d(out), rhs,
                                        _d(np.ascontiguousarray(int_mat, np.float64)))
        return out

    def drdd_complex(self, dvar, h=1e-14, state=None):
        """getdRelasticdD element part: (dRu/dd in global DOF, dRu/dd at the internal DOF)."""
        out = np.zeros(self.n)
        iout = np.zeros(max(self.int_vec_size, 1))
        rc = self.L.orc_drdd_complex(self.h, dvar, h, C.byref(state) if state is not None else None, _d(out),
                                     _d(iout))
        assert rc == 0
        return out, iout[:self.int_vec_size]

    def design_node_load(self, t, load=None):
        """getElasticAppliedLoad's nodal design loads at time t, added to load."""
        load = np.zeros(self.n) if load is None else load
        self.L.orc_design_node_load(self.h, float(t), _d(load))
        return load

    def node_load_drdd(self, dvar, t, h=1e-14, drudd=None):
        """getdRelasticdD's nodal-load branch: drudd -= d(nodal design load)/d(dvar) at time t."""
        drudd = np.zeros(self.n) if drudd is None else drudd
        self.L.orc_node_load_drdd(self.h, int(dvar), float(t), float(h), _d(drudd))
        return drudd

    def element_matrices(self, el0=1, el1=None, state=None):
        """Condensed nodal element matrices (24x24) of elements el0..el1 (1-based, inclusive)."""
        if el1 is None:
            el1 = self.model.num_els
        out = np.zeros((el1 - el0 + 1, 24, 24))
        rc = self.L.orc_element_matrices(self.h, el0, el1, C.byref(state) if state is not None else None,
                                         _d(out))
        assert rc == 0
        return np.transpose(out, (0, 2, 1)).copy()   # stored column-major per element

    def el_soln_load(self, build_mat=1, state=None, elastic_load=None, int_elastic_load=None):
        n = self.n
        load = np.zeros(n) if elastic_load is None else elastic_load
        iload = np.zeros(max(self.int_vec_size, 1)) if int_elastic_load is None else int_elastic_load
        mat = np.zeros(self.el_mat_size)
        cols = np.zeros(self.el_mat_size, np.int32)
        imat = np.zeros(max(self.int_mat_size, 1))
        rc = self.L.orc_el_soln_load(self.h, build_mat, C.byref(state) if state is not None else None, _d(load),
                                     _d(iload), _d(mat), _i(cols), _d(imat))
        assert rc == 0
        return load, iload, mat, cols, imat

    # -- constraints, loads ---------------------------------------------------------------------
    def scale_mpc(self, elastic_mat):
        mm = self.mpc_mat.copy()
        mr = self.mpc_rhs.copy()
        self.L.orc_scale_mpc(_d(elastic_mat), len(elastic_mat), _d(mm), _d(mr), _i(self.mpc_range), self.mpc_dim)
        return mm, mr

    def constraint_load(self, mpc_mat, mpc_rhs, node_disp, elastic_load):
        self.L.orc_constraint_load(_d(mpc_mat), _i(self.mpc_cols), _i(self.mpc_range), _d(mpc_rhs), self.mpc_dim,
                                   _d(node_disp), _d(elastic_load))

    def body_load(self, kind, vals, elements=None, state=None, load=None):
        """getElasticAppliedLoad body-force branch: kind 0 bodyForce, 1 gravitational,
        2 centrifugal (vals = center, axis, angVel) over the listed elements (1-based; None = all)."""
        load = np.zeros(self.n) if load is None else load
        els = None if elements is None else np.ascontiguousarray(elements, np.int32)
        v = np.zeros(7)
        v[:len(vals)] = vals
        rc = self.L.orc_body_load(self.h, kind, _d(v), 0 if els is None else len(els), None if els is None else _i(els),
                                  C.byref(state) if state is not None else None, _d(load))
        assert rc == 0
        return load

    # -- thermal path (restated in oracle_api.cpp: orc_thermal_soln_load; the constraint
    #    bookkeeping below in numpy) ----------------------------------------------------------
    def thermal_soln_load(self, cond, spec_heat, build_mat=1, temp=None, prev_temp=None, prev_tdot=None, dynamic=0,
                          gamma=0.5, del_t=0.0, load=None):
        """getThermalSolnLoad: (thermal load in rank order, thermMat, thermMatCols, thermMatRange)."""
        N = self.model.num_nodes
        load = np.zeros(N) if load is None else load
        cond = np.ascontiguousarray(cond, np.float64).reshape(-1)
        sh = np.ascontiguousarray(spec_heat, np.float64)
        rng = np.zeros(N + 1, np.int32)
        scratch = np.zeros(N)
        opt = lambda a: None if a is None else _d(np.ascontiguousarray(a, np.float64))
        keep = [np.ascontiguousarray(a, np.float64) if a is not None else None for a in (temp, prev_temp, prev_tdot)]
        rc = self.L.orc_thermal_soln_load(self.h, _d(cond), _d(sh), 0, opt(keep[0]), opt(keep[1]), opt(keep[2]), 0,
                                          gamma, del_t, _d(scratch), None, None, _i(rng))
        assert rc == 0
        mat = np.zeros(max(int(rng[N]), 1))
        cols = np.zeros(max(int(rng[N]), 1), np.int32)
        rc = self.L.orc_thermal_soln_load(self.h, _d(cond), _d(sh), build_mat, opt(keep[0]), opt(keep[1]),
                                          opt(keep[2]), dynamic, gamma, del_t, _d(load), _d(mat), _i(cols), None)
        assert rc == 0
        return load, mat[:rng[N]], cols[:rng[N]], rng

    def thermal_drdd(self, cond, spec_heat, dvar, h=1e-14, temp=None, prev_temp=None, prev_tdot=None, dynamic=0,
                     gamma=0.5, del_t=0.0):
        """getdRthermaldD element part: dRt/dd in rank order (complex step)."""
        N = self.model.num_nodes
        out = np.zeros(N)
        keep = [None if a is None else np.ascontiguousarray(a, np.float64) for a in (temp, prev_temp, prev_tdot)]
        rc = self.L.orc_thermal_drdd(self.h, _d(np.ascontiguousarray(cond, np.float64).reshape(-1)),
                                     _d(np.ascontiguousarray(spec_heat, np.float64)), int(dvar), float(h),
                                     *[None if a is None else _d(a) for a in keep], int(dynamic), float(gamma),
                                     float(del_t), _d(out))
        assert rc == 0
        return out

    def thermal_heat_gen_drdd(self, dvar, q, elements=None, h=1e-14, drtdd=None):
        """getdRthermaldD's bodyHeatGen branch: drtdd -= d(heat-generation load)/d(dvar)."""
        drtdd = np.zeros(self.model.num_nodes) if drtdd is None else drtdd
        els = None if elements is None else np.ascontiguousarray(elements, np.int32)
        rc = self.L.orc_thermal_heat_gen_drdd(self.h, int(dvar), float(h), float(q), 0 if els is None else len(els),
                                              None if els is None else _i(els), _d(drtdd))
        assert rc == 0
        return drtdd

    def thermal_surface_flux_drdd(self, dvar, face_el, face_num, flux, h=1e-14, drtdd=None):
        """getdRthermaldD's surfaceFlux branch: drtdd += d(flux face load)/d(dvar)."""
        drtdd = np.zeros(self.model.num_nodes) if drtdd is None else drtdd
        fe = np.ascontiguousarray(face_el, np.int32)
        fn = np.ascontiguousarray(face_num, np.int32)
        rc = self.L.orc_thermal_surface_flux_drdd(self.h, int(dvar), float(h), len(fe), _i(fe), _i(fn), float(flux),
                                                  _d(drtdd))
        assert rc == 0
        return drtdd

    def thermal_design_node_load(self, t, load=None):
        """getThermalAppliedLoad's nodal design heat inputs at time t, added to load (rank order)."""
        load = np.zeros(self.model.num_nodes) if load is None else load
        self.L.orc_thermal_design_node_load(self.h, float(t), _d(load))
        return load

    def thermal_node_load_drdd(self, dvar, t, h=1e-14, drtdd=None):
        """getdRthermaldD's node branch: drtdd -= d(nodal heat input)/d(dvar) at time t."""
        drtdd = np.zeros(self.model.num_nodes) if drtdd is None else drtdd
        self.L.orc_thermal_node_load_drdd(self.h, int(dvar), float(t), float(h), _d(drtdd))
        return drtdd

    def thermal_mpc(self, mpc_range, mpc_node, mpc_coef, mpc_rhs):
        """buildThermalMPC (Working/AStrO_bookKeeping.f90:614-752) for expanded equations: rows of
        (1-based rank column, coefficient), duplicate columns skipped (slot stays 0)."""
        rows = []
        for r in range(len(mpc_range) - 1):
            t0, t1 = mpc_range[r], mpc_range[r + 1]
            cols, vals = [0] * (t1 - t0), [0.0] * (t1 - t0)
            for t in range(t0, t1):
                c = int(self.current_rank[mpc_node[t] - 1])
                for s_ in range(t1 - t0):
                    if cols[s_] == 0:
                        cols[s_], vals[s_] = c, float(mpc_coef[t])
                        break
                    if cols[s_] == c:
                        break
            rows.append((cols, vals, float(mpc_rhs[r])))
        return rows

    @staticmethod
    def scale_thermal_mpc(therm_mat, rows):
        """scaleThermalMPC (Working/AStrO_commandFunctions.f90:230-258)."""
        mx = float(np.abs(therm_mat).max()) if len(therm_mat) else 0.0
        out = []
        for cols, vals, rhs in rows:
            mag = np.sqrt(sum(v * v for v in vals))
            out.append((cols, [100.0 * mx * ((1.0 / mag) * v) for v in vals], 100.0 * mx * ((1.0 / mag) * rhs)))
        return out

    @staticmethod
    def thermal_constraint_load(rows, temp, load):
        """getThermalConstraintLoad (:197-228), node vectors in rank order."""
        for cols, vals, rhs in rows:
            v = rhs
            for c, k in zip(cols, vals):
                if c:
                    v = v - k * temp[c - 1]
            for c, k in zip(cols, vals):
                if c:
                    load[c - 1] += k * v
        return load

    def thermal_heat_gen(self, q, elements=None, load=None):
        """getThermalAppliedLoad's bodyHeatGen branch (:96-139): r_getElBodyForce with the heat
        generation as the first body-force component; component-1 entries to the element nodes'
        thermal DOF (rank order)."""
        N = self.model.num_nodes
        load = np.zeros(N) if load is None else load
        el = self.body_load(0, [q, 0, 0, 0, 0, 0], elements=elements)
        for nd in range(1, N + 1):
            load[self.current_rank[nd - 1] - 1] += el[self.n_dof_index[nd - 1, 0] - 1]
        return load

    def thermal_surface_flux(self, face_el, face_num, flux, load=None):
        """getThermalAppliedLoad's surfaceFlux branch: r_getElSurfaceTraction with the flux as
        the first traction component; thermalLoad -= the component-1 nodal values."""
        N = self.model.num_nodes
        load = np.zeros(N) if load is None else load
        el = np.zeros(self.n)
        fe = np.ascontiguousarray(face_el, np.int32)
        fn = np.ascontiguousarray(face_num, np.int32)
        self.L.orc_surface_load(self.h, len(fe), _i(fe), _i(fn), _d(np.array([flux, 0.0, 0.0])), 0.0, _d(el))
        for nd in range(1, N + 1):
            load[self.current_rank[nd - 1] - 1] -= el[self.n_dof_index[nd - 1, 0] - 1]
        return load

    def thermal_system(self, cond, spec_heat, mpc=None):
        """(A = K_T + C^T C over ranks, b = constraint load at zero temperature, rows) of a steady
        thermal step from the zero state."""
        import scipy.sparse as sp
        N = self.model.num_nodes
        load, mat, cols, rng = self.thermal_soln_load(cond, spec_heat, 1)
        K = sp.csr_matrix((mat, cols - 1, rng), shape=(N, N))
        b = np.zeros(N)
        rows = []
        if mpc is not None:
            rows = self.scale_thermal_mpc(mat, self.thermal_mpc(*mpc))
            r_, c_, v_ = [], [], []
            for i, (cols_, vals, _) in enumerate(rows):
                for c, k in zip(cols_, vals):
                    if c:
                        r_.append(i)
                        c_.append(c - 1)
                        v_.append(k)
            Cm = sp.csr_matrix((v_, (r_, c_)), shape=(len(rows), N))
            K = K + Cm.T @ Cm
            self.thermal_constraint_load(rows, np.zeros(N), b)
        return K.tocsr(), b, rows

    def applied_load(self, load=None):
        """Consistent surface load of the model's faces plus its point loads."""
        m = self.model
        load = np.zeros(self.n) if load is None else load
        if len(m.face_el):
            fe = np.ascontiguousarray(m.face_el, np.int32)
            fn = np.ascontiguousarray(m.face_num, np.int32)
            tr = np.ascontiguousarray(m.traction, np.float64)
            self.L.orc_surface_load(self.h, len(fe), _i(fe), _i(fn), _d(tr), float(m.pressure), _d(load))
        for nd, dof, v in m.point_loads:
            load[self.n_dof_index[nd - 1, dof - 1] - 1] += v
        return load

    def convert_to_ltri(self, mat, cols, mpc_mat):
        lt = np.zeros(self.lt_size)
        self.L.orc_convert_to_ltri(_d(lt), _i(self.lt_range), self.lt_size, _d(mat), _i(cols),
                                   _i(self.el_mat_range), len(mat), self.n, _d(mpc_mat), _i(self.mpc_cols),
                                   _i(self.mpc_range), self.mpc_size, self.mpc_dim)
        return lt

    # -- solvers (pure functions of their arguments) ----------------------------------------------
    @staticmethod
    def ldl_fact(lt, lt_range):
        a = lt.copy()
        _lib().orc_ldl_fact(_d(a), len(a), _i(lt_range), len(lt_range) - 1)
        return a

    @staticmethod
    def ldl_solve(fac, lt_range, rhs):
        n = len(lt_range) - 1
        x = np.zeros(n)
        z = np.zeros(n)
        _lib().orc_ldl_solve(_d(x), _d(np.ascontiguousarray(rhs, np.float64)), _d(fac), len(fac), _i(lt_range), n,
                             _d(z))
        return x

    def gmres(self, mat, cols, mpc_mat, fac, b, x0=None, num_vecs=None, max_it=None):
        n = self.n
        x = np.zeros(n) if x0 is None else x0.copy()
        if num_vecs is None:
            num_vecs = n // 2 if n < 200 else 100
        if max_it is None:
            max_it = n
        cyc = self.L.orc_gmres(_d(x), _d(mat), _i(cols), _i(self.el_mat_range), len(mat), n, _d(mpc_mat),
                               _i(self.mpc_cols), _i(self.mpc_range), self.mpc_size, self.mpc_dim, _d(fac),
                               _i(self.lt_range), len(fac), _d(np.ascontiguousarray(b, np.float64)), num_vecs,
                               max_it)
        return x, cyc

    # -- helpers for tests ----------------------------------------------------------------------
    def csr_scipy(self, mat, cols):
        import scipy.sparse as sp
        n = self.n
        rows = np.repeat(np.arange(n), np.diff(self.el_mat_range))
        keep = cols > 0
        return sp.csr_matrix((mat[keep], (rows[keep], cols[keep] - 1)), shape=(n, n))

    def mpc_scipy(self, mpc_mat):
        import scipy.sparse as sp
        rows = np.repeat(np.arange(self.mpc_dim), np.diff(self.mpc_range))
        keep = self.mpc_cols > 0
        return sp.csr_matrix((mpc_mat[keep], (rows[keep], self.mpc_cols[keep] - 1)), shape=(self.mpc_dim, self.n))

    def total_dldd(self, dldu, int_dldu=None, dldd_explicit=None, state=None, h=1e-14):
        """getTotaldLdD, static branch (Working/AStrO_commandFunctions.f90:1377-1410) with the elastic
        branch of solveDynamicAdjoint (:917-966, dLdv = dLda = 0): tangent and scaled constraints at
        the state, condensation of (dldu, int_dldu), the adjoint by a direct solve of
        (K + C^T C) lambda = b, the internal lambda, then dLdD(d) = explicit(d) - lambda . dRudD(d)
        - lambda_int . intdRudD(d).  Returns (dLdD, lambda, lambda_int)."""
        import scipy.sparse.linalg as spla
        _, _, mat, cols, imat = self.el_soln_load(1, state=state)
        mm, _ = self.scale_mpc(mat)
        A = (self.csr_scipy(mat, cols) + self.mpc_scipy(mm).T @ self.mpc_scipy(mm)).tocsc()
        b = np.asarray(dldu, np.float64).copy()
        ni = self.int_vec_size
        if ni and int_dldu is not None:
            b = self.update_external_rhs(b, int_dldu, imat)
        lam = spla.spsolve(A, b)
        lam_i = np.zeros(ni)
        if ni:
            lam_i = self.update_internal_soln(lam, np.zeros(ni), int_dldu, imat)[:ni]
        nd = len(self.model.d_value)
        out = np.zeros(nd) if dldd_explicit is None else np.asarray(dldd_explicit, np.float64).copy()
        for d in range(1, nd + 1):
            dr, dri = self.drdd_complex(d, h, state=state)
            out[d - 1] -= lam @ dr + (lam_i @ dri[:ni] if ni else 0.0)
        return out, lam, lam_i

    def total_dldd_transient(self, disp, vel, acc, int_disp, del_t, beta, gamma, dldu=None, dldv=None, dlda=None,
                             int_dldu=None, dldd_explicit=None, h=1e-14, accumulate_internal=True):
        """getTotaldLdD, dynamic branch (Working/AStrO_commandFunctions.f90:1411-1465): the backward
        sweep over the stored states (rows 0..N), augmentdLdu (:819-915) with the 1e-20 scaling round
        trip, solveDynamicAdjoint's elastic branch (:917-966) by direct solves of K_eff at (state i,
        state i-1), the internal adjoint accumulated as updateInternalSoln does, and the complex-step
        dRu/dD at each state.  Returns (dLdD, adjoint of step 1)."""
        import scipy.sparse.linalg as spla
        from misc_gb300 import model as M
        n, ni = self.n, self.int_vec_size
        N = len(disp) - 1
        nd = len(self.model.d_value)
        f = 1e-20
        rt = lambda x: (np.asarray(x, np.float64) * f) * (1.0 / f)
        iud = (lambda i: np.asarray(int_disp[i], np.float64)) if int_disp is not None else (lambda i: np.zeros(ni))
        lam, ilam = np.zeros(n), np.zeros(ni)
        velAdj, accAdj = np.zeros(n), np.zeros(n)
        out = np.zeros(nd) if dldd_explicit is None else np.asarray(dldd_explicit, np.float64).copy()

        def st(u, v, a, iu, pu, pv, pa, piu):
            return M.make_state(n, disp=u, vel=v, acc=a, internal_disp=iu, prev_disp=pu, prev_vel=pv, prev_acc=pa,
                                prev_int_disp=piu, dynamic=1, beta=beta, gamma=gamma, del_t=del_t)

        for i in range(N, 0, -1):
            dLdu, dLdv, dLda, idLdu = np.zeros(n), np.zeros(n), np.zeros(n), np.zeros(ni)
            u, v, a, iu = (np.asarray(disp[i], np.float64), np.asarray(vel[i], np.float64),
                           np.asarray(acc[i], np.float64), iud(i))
            if i < N:
                nu, nv, na, niu = (np.asarray(disp[i + 1]) * f, np.asarray(vel[i + 1]) * f,
                                   np.asarray(acc[i + 1]) * f, iud(i + 1) * f)
                pu, pv, pa, piu = u * f, v * f, a * f, iu * f
                load, iload, *_ = self.el_soln_load(0, state=st(nu, nv, na, niu, lam, pv, pa, ilam))
                dLdu += load + accAdj
                idLdu += iload[:ni]
                load, *_ = self.el_soln_load(0, state=st(nu, nv, na, niu, pu, pv, lam, piu))
                dLda += load + 0.5 * del_t * del_t * (1 - 2 * beta) * accAdj + del_t * (1 - gamma) * velAdj
                load, *_ = self.el_soln_load(0, state=st(nu, nv, na, niu, pu, lam, pa, piu))
                dLdv += load + del_t * accAdj + velAdj
                u, v, a, iu = rt(u), rt(v), rt(a), rt(iu)
            if dldu is not None:
                dLdu += dldu[i - 1]
            if dldv is not None:
                dLdv += dldv[i - 1]
            if dlda is not None:
                dLda += dlda[i - 1]
            if int_dldu is not None:
                idLdu += int_dldu[i - 1]
            velAdj = dLdv.copy()
            accAdj = (-1.0 / (del_t * del_t * beta)) * (dLda + del_t * gamma * velAdj)
            dLdu = dLdu - accAdj
            s = st(u, v, a, iu, np.asarray(disp[i - 1], np.float64), np.asarray(vel[i - 1], np.float64),
                   np.asarray(acc[i - 1], np.float64), iud(i - 1))
            _, _, mat, cols, imat = self.el_soln_load(1, state=s)
            mm, _ = self.scale_mpc(mat)
            A = (self.csr_scipy(mat, cols) + self.mpc_scipy(mm).T @ self.mpc_scipy(mm)).tocsc()
            if ni:
                dLdu = self.update_external_rhs(dLdu, idLdu, imat)
            lam = spla.spsolve(A, dLdu)
            if ni:
                ilam = self.update_internal_soln(lam, ilam if accumulate_internal else np.zeros(ni), idLdu, imat)[:ni]
            for d in range(1, nd + 1):
                dr, dri = self.drdd_complex(d, h, state=s)
                out[d - 1] -= lam @ dr + (ilam @ dri[:ni] if ni else 0.0)
        return out, lam

    def static_system(self):
        """(A = K + C^T C, b) of the linear static step from zero state with the scaled constraints."""
        load, iload, mat, cols, imat = self.el_soln_load(1)
        mm, mr = self.scale_mpc(mat)
        b = np.zeros(self.n)
        self.constraint_load(mm, mr, np.zeros(self.n), b)
        self.applied_load(b)
        K = self.csr_scipy(mat, cols)
        Cm = self.mpc_scipy(mm)
        return (K + (Cm.T @ Cm)).tocsr(), b, mat, cols, mm, mr
