"""GPU parity of the brickIM element (type 81: brick8 plus three incompatible bubbles, nine
condensed internal DOF) and of the solid Newmark inertia (brick8 and brickIM), against the
oracle, through the C ABI.  Tolerances as the other element tests: element matrices, residuals,
assembled CSR values, internal rows and loads 1e-12 relative; the Newmark time loop 1e-8 per
step against the oracle's loop with a direct solve of K_eff."""
import numpy as np
import pytest
import scipy.sparse.linalg as spla

from misc_gb300 import model as M
from misc_gb300.astro import AstroGPU
from oracle import Oracle

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.linalg.norm(a - b, axis=(1, 2)) / np.linalg.norm(b, axis=(1, 2))


def _im(m, every=1):
    """brickIM on every element (every = 1) or on every second one (a mixed brick8 / brickIM mesh)."""
    t = np.full(m.num_els, 8, np.int32)
    t[::every] = 81
    m.element_type = t
    return m


@pytest.fixture(scope="module", params=[1, 2], ids=["brickIM", "mixed"])
def block(request):
    m = _im(M.hex_block(5, 3, 3, lx=1.25, ly=0.75, lz=0.75, seed=4), request.param)
    return m, AstroGPU(m), Oracle(m)


def _state(o, rng, scale=1e-3, internal=True):
    u = scale * rng.standard_normal(o.n)
    iu = scale * rng.standard_normal(o.int_vec_size) if internal else None
    return M.make_state(o.n, disp=u, internal_disp=iu)


def test_element_matrices_zero_state(block):
    m, g, o = block
    assert g.int_vec_size == o.int_vec_size and g.dims.int_mat_size == o.int_mat_size
    assert _rel(g.element_matrices(64), o.element_matrices()).max() < 1e-12


def test_element_matrices_and_residual_displaced(block):
    """Green-Lagrange strain over the eleven shape functions (nodal and bubble displacements),
    stress stiffness, condensation."""
    m, g, o = block
    st = _state(o, np.random.default_rng(1))
    ke, ru = g.element_matrices(64, state=st, with_residual=True)
    ko = o.element_matrices(state=st)
    assert _rel(ke, ko).max() < 1e-12
    for el in range(1, m.num_els + 1):
        r_o, _ = o.element(el, 1, st)
        assert np.linalg.norm(ru[el - 1] - r_o[:24]) <= 1e-12 * np.linalg.norm(r_o[:24]), el


def test_soln_load_and_internal_rows(block):
    m, g, o = block
    st = _state(o, np.random.default_rng(2))
    load, iload, mat, cols, imat = g.getElasticSolnLoad(1, state=st)
    oload, oiload, omat, ocols, oimat = o.el_soln_load(1, state=st)
    assert np.array_equal(cols, ocols)
    assert np.abs(mat - omat).max() <= 1e-12 * np.abs(omat).max()
    assert np.linalg.norm(load - oload) <= 1e-12 * np.linalg.norm(oload)
    assert np.linalg.norm(iload - oiload[:o.int_vec_size]) <= 1e-12 * np.linalg.norm(oiload[:o.int_vec_size])
    assert np.abs(imat - oimat[:o.int_mat_size]).max() <= 1e-12 * np.abs(oimat[:o.int_mat_size]).max()
    # condensation of an internal vector into the nodal one, and the recovery
    rng = np.random.default_rng(3)
    ext, iv = rng.standard_normal(o.n), rng.standard_normal(o.int_vec_size)
    e1 = g.updateExternalRHS(ext.copy(), iv)
    e2 = o.update_external_rhs(ext.copy(), iv, oimat)
    assert np.linalg.norm(e1 - e2) <= 1e-12 * np.linalg.norm(e2)
    u = rng.standard_normal(o.n)
    i1 = g.updateInternalSoln(u, np.zeros(o.int_vec_size), iv)
    i2 = o.update_internal_soln(u, np.zeros(o.int_vec_size), iv, oimat)
    assert np.linalg.norm(i1 - i2[:o.int_vec_size]) <= 1e-11 * np.linalg.norm(i2[:o.int_vec_size])


def test_static_step_with_internal_dof(block):
    """A linear static step (stepSolve: condensation, solve, internal recovery) against a direct
    solve of the oracle's condensed system and its recovery."""
    m, g, o = block
    n, ni = o.n, o.int_vec_size
    f = o.applied_load()
    load, iload, mat, cols, imat = o.el_soln_load(1)
    mm, mr = o.scale_mpc(mat)
    Cm = o.mpc_scipy(mm)
    A = (o.csr_scipy(mat, cols) + Cm.T @ Cm).tocsc()
    b = load + f
    o.constraint_load(mm, mr, np.zeros(n), b)
    rhs = o.update_external_rhs(b, iload[:ni], imat)
    uo = spla.spsolve(A, rhs)
    iuo = o.update_internal_soln(uo, np.zeros(ni), iload[:ni], imat)[:ni]
    g.getElasticSolnLoad(1, export=False)
    g.scaleElasticMPC()
    u, iu, it, st = g.stepSolve(g.applied_load(), nl_geom=0, rtol=1e-13)
    assert it == 1 and st.status == 0
    assert np.linalg.norm(u - uo) <= 1e-9 * np.linalg.norm(uo)
    assert np.linalg.norm(iu - iuo) <= 1e-8 * np.linalg.norm(iuo)


@pytest.mark.parametrize("eltype", [8, 81])
def test_solid_newmark_matches_oracle_loop(eltype):
    """The solid branch of r_getElRum: consistent mass in K_eff and the inertial residual, five
    steps of a tip-loaded brick cantilever against the oracle's loop (direct K_eff solve)."""
    from newmark_ref import newmark_states
    m = M.hex_block(6, 2, 2, lx=3.0, ly=0.5, lz=0.5, seed=6, jitter=0.1, sigma=0.3)
    m.element_type = np.full(m.num_els, eltype, np.int32)
    o, g = Oracle(m), AstroGPU(m)
    tip = [a for a in range(m.num_nodes) if abs(m.node_list[a, 0] - 3.0) < 1e-9]
    pattern = np.zeros(o.n)
    for a in tip:
        pattern[o.n_dof_index[a, 2] - 1] = 1.0 / len(tip)
    dt, beta, gamma, steps = 2e-5, 0.25, 0.5, 5
    amp = 1e6 * np.sin(2 * np.pi * 2000.0 * dt * np.arange(1, steps + 1))
    D, V, A, I = newmark_states(o, pattern, amp, dt, beta, gamma, steps)
    u, v, a, iu, hist, st = g.newmark_run(steps, dt, beta, gamma, pattern, amp, rtol=1e-13)
    assert st.status == 0
    for k in range(steps):
        assert np.linalg.norm(hist[k] - D[k + 1]) <= 1e-8 * np.linalg.norm(D[k + 1]), k
    assert np.linalg.norm(v - V[-1]) <= 1e-7 * np.linalg.norm(V[-1])
    if eltype == 81:
        assert np.linalg.norm(iu - I[-1]) <= 1e-7 * np.linalg.norm(I[-1])


def test_brick_dynamic_element_matrices():
    """K + c1 c2 M and Ru with the Newmark inertia at a displaced dynamic state, element by
    element, brick8 (double-float kernel) and brickIM."""
    for eltype in (8, 81):
        m = M.hex_block(3, 2, 2, lx=1.0, ly=0.6, lz=0.6, seed=8)
        m.element_type = np.full(m.num_els, eltype, np.int32)
        g, o = AstroGPU(m), Oracle(m)
        rng = np.random.default_rng(9)
        n, ni = o.n, o.int_vec_size
        st = M.make_state(n, disp=1e-3 * rng.standard_normal(n), prev_disp=1e-3 * rng.standard_normal(n),
                          prev_vel=rng.standard_normal(n), prev_acc=1e3 * rng.standard_normal(n),
                          internal_disp=1e-3 * rng.standard_normal(ni) if ni else None,
                          prev_int_disp=1e-3 * rng.standard_normal(ni) if ni else None,
                          dynamic=1, beta=0.25, gamma=0.5, del_t=1e-4)
        ke, ru = g.element_matrices(64, state=st, with_residual=True)
        assert _rel(ke, o.element_matrices(state=st)).max() < 1e-12, eltype
        for el in range(1, m.num_els + 1):
            r_o, _ = o.element(el, 1, st)
            assert np.linalg.norm(ru[el - 1] - r_o[:24]) <= 1e-12 * np.linalg.norm(r_o[:24]), (eltype, el)


def test_brickim_modulus_complex_step():
    """getdRelasticdD for elastic-modulus design variables on brickIM elements (nodal and internal
    residual sensitivities) against the oracle's complex twin."""
    m = _im(M.hex_block(4, 2, 2, lx=1.0, ly=0.5, lz=0.5, seed=10), 2)
    M.add_design_variables(m, 3, 2, component=1)
    g, o = AstroGPU(m), Oracle(m)
    st = _state(o, np.random.default_rng(11))
    for d in (1, 2, 3):
        dr, idr = g.getdRelasticdD(d, h=1e-30, state=st)
        odr, oidr = o.drdd_complex(d, h=1e-30, state=st)
        assert np.linalg.norm(dr - odr) <= 1e-10 * np.linalg.norm(odr), d
        assert np.linalg.norm(idr - oidr[:o.int_vec_size]) <= 1e-10 * np.linalg.norm(oidr[:o.int_vec_size]), d


def test_design_gradient_batched_complex_steps():
    """astro_total_dldd on solids runs the complex-step kernels for up to 16 design variables per
    pass (one launch per colour over all of them): 20 modulus variables on a mixed brick8 /
    brickIM block (two passes, internal DOF), each gradient entry against explicit - lambda .
    dR/dd - lambda_int . dR_int/dd from the per-variable getdRelasticdD, 1e-12."""
    m = _im(M.hex_block(6, 3, 3, lx=1.5, ly=0.75, lz=0.75, seed=12), 2)
    M.add_design_variables(m, 20, M.DCAT_ELASTIC_MODULUS, component=1)
    g, o = AstroGPU(m), Oracle(m)
    st = _state(o, np.random.default_rng(13))
    g.getElasticSolnLoad(1, state=st, export=False)
    g.scaleElasticMPC()
    rng = np.random.default_rng(14)
    dldu, idldu, expl = rng.standard_normal(g.n), rng.standard_normal(g.int_vec_size), rng.standard_normal(20)
    dldd, lam, ilam, s = g.getTotaldLdD(dldu, int_dldu=idldu, dldd_explicit=expl, state=st, rtol=1e-10)
    assert s.status == 0
    for d in range(1, 21):
        dr, idr = g.getdRelasticdD(d, state=st)
        ref = expl[d - 1] - lam @ dr - ilam @ idr
        assert abs(dldd[d - 1] - ref) <= 1e-12 * max(abs(ref), np.linalg.norm(lam) * np.linalg.norm(dr)), d
