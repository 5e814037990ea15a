"""GPU parity of the shell4 path (co-rotational element, static condensation, assembly) against
the oracle through the C ABI.  Element matrices 1e-12 relative (Frobenius per element),
displacements 1e-10 relative."""
import ctypes

import numpy as np
import pytest
import scipy.sparse.linalg as spla

from misc_gb300 import model as M
from misc_gb300.astro import OPT_SHELL_MEAN_ROT_TERM, SOLVER_GMRES_JACOBI_FP64, AstroGPU
from oracle import Oracle
from oracle.oracle import _lib

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.linalg.norm(a - b, axis=(1, 2)) / np.linalg.norm(b, axis=(1, 2))


def _skewed_plate():
    m = M.plate_shell(nx=5, ny=4, lx=2.0, ly=1.0, t=0.03, E=7e10, nu=0.33)
    rng = np.random.default_rng(5)
    X = m.node_list.copy()
    X[:, :2] += 0.05 * rng.uniform(-1, 1, (len(X), 2))
    X[:, 2] += 0.02 * rng.uniform(-1, 1, len(X))   # warped: exercises correctAlpha
    m.node_list = X
    m.layup_angle = np.array([0.3])
    return m


@pytest.fixture(scope="module")
def plate():
    m = _skewed_plate()
    return m, AstroGPU(m), Oracle(m)


def test_shell_element_matrices_zero_state(plate):
    m, g, o = plate
    assert _rel(g.element_matrices(64), o.element_matrices()).max() < 1e-12


def test_shell_residual_tangent_at_displaced_state(plate):
    """Nonzero state: co-rotational frame, second derivatives (stress stiffness), residual."""
    m, g, o = plate
    rng = np.random.default_rng(3)
    u = 1e-3 * rng.standard_normal(o.n)
    iv = 1e-4 * rng.standard_normal(o.int_vec_size)
    st = M.make_state(o.n, disp=u, internal_disp=iv)
    ke, ru = g.element_matrices(64, state=st, with_residual=True)
    ko = o.element_matrices(state=st)
    assert _rel(ke, ko).max() < 1e-11
    for el in (1, 7, m.num_els):
        r_o, _ = o.element(el, 1, st)
        assert np.linalg.norm(ru[el - 1] - r_o[:24]) <= 1e-11 * np.linalg.norm(r_o[:24])
    load, iload, mat, cols, imat = g.getElasticSolnLoad(1, state=st)
    oload, oiload, omat, ocols, oimat = o.el_soln_load(1, state=st)
    assert np.linalg.norm(load - oload) <= 1e-11 * np.linalg.norm(oload)
    assert np.linalg.norm(iload - oiload) <= 1e-11 * np.linalg.norm(oiload)
    assert np.array_equal(cols, ocols)
    assert np.abs(mat - omat).max() <= 1e-11 * np.abs(omat).max()
    assert np.abs(imat - oimat).max() <= 1e-11 * np.abs(oimat).max()


def test_shell_consistent_mean_rotation_option(plate):
    m, g, o = plate
    L = _lib()
    L.orc_set_quirk.argtypes = [ctypes.c_int, ctypes.c_int]
    try:
        L.orc_set_quirk(1, 1)
        g.set_option(OPT_SHELL_MEAN_ROT_TERM, 1)
        o2 = Oracle(m)
        assert _rel(g.element_matrices(64), o2.element_matrices()).max() < 1e-12
    finally:
        L.orc_set_quirk(1, 0)
        g.set_option(OPT_SHELL_MEAN_ROT_TERM, 0)


@pytest.mark.parametrize("model", ["cfg1", "shell_beam"])
def test_shell_static_system(model):
    """Right-hand side (constraint + pressure/point loads) and the operator K + C^T C of the
    linear static step match the oracle's assembled system."""
    m = M.config1() if model == "cfg1" else M.shell_beam()
    g, o = AstroGPU(m), Oracle(m)
    g.getElasticSolnLoad(1, export=False)
    g.scaleElasticMPC()
    b = g.static_rhs()
    A, bo, *_ = o.static_system()
    assert np.linalg.norm(b - bo) <= 1e-13 * np.linalg.norm(bo)
    x = np.random.default_rng(2).standard_normal(o.n)
    y = g.apply_operator(x, 64)
    assert np.linalg.norm(y - A @ x) <= 1e-13 * np.linalg.norm(A @ x)


def test_shell_newmark_dynamic_state(plate):
    """Newmark step (r_getElRu with r_getElRum): acceleration from disp/prev state, inertial
    residual and K + c1 c2 M, against the oracle."""
    m, g, o = plate
    rng = np.random.default_rng(8)
    n = o.n
    st = M.make_state(n, disp=1e-3 * rng.standard_normal(n), prev_disp=1e-3 * rng.standard_normal(n),
                      prev_vel=1e-1 * rng.standard_normal(n), prev_acc=10.0 * rng.standard_normal(n),
                      internal_disp=1e-4 * rng.standard_normal(o.int_vec_size), dynamic=1, beta=0.25, gamma=0.5,
                      del_t=1e-3)
    load, iload, mat, cols, imat = g.getElasticSolnLoad(1, state=st)
    oload, oiload, omat, ocols, oimat = o.el_soln_load(1, state=st)
    assert np.linalg.norm(load - oload) <= 1e-11 * np.linalg.norm(oload)
    assert np.linalg.norm(iload - oiload) <= 1e-11 * np.linalg.norm(oiload)
    assert np.array_equal(cols, ocols)
    assert np.abs(mat - omat).max() <= 1e-11 * np.abs(omat).max()


def test_internal_dof_recovery(plate):
    """updateExternalRHS / updateInternalSoln on the GPU against the oracle, from the condensed
    internal rows of the last assembly (1e-11 relative)."""
    m, g, o = plate
    g.getElasticSolnLoad(1)
    _, _, _, _, imat = o.el_soln_load(1)
    rng = np.random.default_rng(12)
    ext, iv = rng.standard_normal(o.n), rng.standard_normal(o.int_vec_size)
    e_g = g.updateExternalRHS(ext, iv)
    e_o = o.update_external_rhs(ext, iv, imat)
    assert np.linalg.norm(e_g - e_o) <= 1e-11 * np.linalg.norm(e_o)
    i0, rhs = rng.standard_normal(o.int_vec_size), rng.standard_normal(o.int_vec_size)
    s_g = g.updateInternalSoln(ext, i0, rhs)
    s_o = o.update_internal_soln(ext, i0, rhs, imat)
    assert np.linalg.norm(s_g - s_o) <= 1e-11 * np.linalg.norm(s_o)
    s_g0 = g.updateInternalSoln(ext, i0)
    s_o0 = o.update_internal_soln(ext, i0, None, imat)
    assert np.linalg.norm(s_g0 - s_o0) <= 1e-11 * np.linalg.norm(s_o0)
