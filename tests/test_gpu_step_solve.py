"""stepSolve on the device (astro_step_solve) against a Newton loop built from the oracle: the
geometrically nonlinear brick (tangent rebuilt every iteration, the constraint penalty scaled once,
stop at max|delDisp| <= 1e-12 as a single-precision literal) and the linear step."""
import numpy as np
import pytest
import scipy.sparse.linalg as spla

from misc_gb300 import model as M
from misc_gb300.astro import SOLVER_FGMRES_LEARNED, AstroGPU
from oracle import Oracle

pytestmark = pytest.mark.gpu


def _oracle_step(o, f, nl_geom):
    n, ni = o.n, o.int_vec_size
    u, iu = np.zeros(n), np.zeros(ni)
    _, _, mat0, _, _ = o.el_soln_load(1)
    mm, mr = o.scale_mpc(mat0)           # scaleElasticMPC, once, before the step
    Cm = o.mpc_scipy(mm)
    K0 = None
    tol = float(np.float32(1e-12))
    it, dmax = 0, 1.0
    while it < (20 if nl_geom else 1) and dmax > tol:
        st = M.make_state(n, disp=u, internal_disp=iu)
        load, iload, mat, cols, imat = o.el_soln_load(1, state=st)
        if nl_geom or K0 is None:
            K0 = (o.csr_scipy(mat, cols) + Cm.T @ Cm).tocsc()
            imat0 = imat
        load = load + f
        o.constraint_load(mm, mr, u, load)
        rhs = o.update_external_rhs(load, iload[:ni], imat0) if ni else load
        du = spla.spsolve(K0, rhs)
        if ni:
            iu = o.update_internal_soln(du, iu, iload[:ni], imat0)[:ni]
        u = u + du
        dmax = np.abs(du).max()
        it += 1
    return u, iu, it


def test_nonlinear_brick_newton_matches_oracle():
    m = M.hex_block(nx=4, ny=2, nz=2, jitter=0.1, seed=2, traction=5e9)
    o, g = Oracle(m), AstroGPU(m)
    f = o.applied_load()
    uo, _, ito = _oracle_step(o, f, 1)
    g.getElasticSolnLoad(1, export=False)
    g.scaleElasticMPC()
    u, _, it, st = g.stepSolve(g.applied_load(), nl_geom=1, rtol=1e-14)
    assert it == ito and 3 <= it < 20, (it, ito)
    assert np.linalg.norm(u - uo) <= 1e-9 * np.linalg.norm(uo)


def test_linear_step_is_one_solve():
    m = M.hex_block(nx=4, ny=2, nz=2, jitter=0.1, seed=2)
    g = AstroGPU(m)
    g.getElasticSolnLoad(1, export=False)
    g.scaleElasticMPC()
    u1, _, it, st = g.stepSolve(g.applied_load(), nl_geom=0, rtol=1e-12)
    u2, s2 = g.solve_static(g.static_rhs(), rtol=1e-12)
    assert it == 1
    assert np.linalg.norm(u1 - u2) <= 1e-9 * np.linalg.norm(u2)


def test_linear_shell_step_with_internal_dof():
    m = M.plate_shell(nx=6, ny=3, lx=2.0, ly=1.0, t=0.05, E=7e10, nu=0.33, pressure=1e3)
    o, g = Oracle(m), AstroGPU(m)
    uo, iuo, _ = _oracle_step(o, o.applied_load(), 0)
    g.getElasticSolnLoad(1, export=False)
    g.scaleElasticMPC()
    # Jacobi-GMRES stalls on the shell (drilling DOF): the step's solves use the learned solver
    u, iu, it, st = g.stepSolve(g.applied_load(), nl_geom=0, rtol=1e-11, method=SOLVER_FGMRES_LEARNED)
    assert it == 1 and st.fallback == 0
    assert np.linalg.norm(u - uo) <= 1e-6 * np.linalg.norm(uo)
    assert np.linalg.norm(iu - iuo) <= 1e-6 * np.linalg.norm(iuo)
