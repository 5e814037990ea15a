"""GPU parity of the static design gradient (getTotaldLdD with solveDynamicAdjoint's elastic
branch) against the oracle through the C ABI: the adjoint displacement and dL/dD for brick modulus
variables at a solved state and for shell thickness variables at a displaced state with internal
DOF (condensed int_dLdu)."""
import numpy as np
import pytest
import scipy.sparse.linalg as spla

from misc_gb300 import model as M
from misc_gb300.astro import SOLVER_FGMRES_LEARNED, AstroError, AstroGPU
from oracle import Oracle

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def test_adjoint_gradient_brick_at_solution():
    m = M.add_design_variables(M.hex_block(nx=6, ny=3, nz=3, jitter=0.1, seed=5), 3, M.DCAT_ELASTIC_MODULUS,
                               component=1)
    o, g = Oracle(m), AstroGPU(m)
    A, b, *_ = o.static_system()
    u = spla.spsolve(A.tocsc(), b)
    st = M.make_state(o.n, disp=u)
    g.getElasticSolnLoad(1, state=st, export=False)
    g.scaleElasticMPC()
    expl = np.array([1.0, -2.0, 0.5])
    dldd, lam, _, s = g.getTotaldLdD(b, dldd_explicit=expl, state=st, rtol=1e-13)
    od, olam, _ = o.total_dldd(b, dldd_explicit=expl, state=st)
    assert s.status == 0
    assert _rel(lam, olam) < 1e-9
    assert _rel(dldd - expl, od - expl) < 1e-8


def test_adjoint_gradient_shell_internal_dof():
    m = M.plate_shell(nx=6, ny=4, lx=2.0, ly=1.0, t=0.03, E=7e10, nu=0.33)
    rng = np.random.default_rng(5)
    X = m.node_list.copy()
    X[:, 2] += 0.02 * rng.uniform(-1, 1, len(X))
    m.node_list = X
    m = M.add_design_variables(m, 4, M.DCAT_LAYUP_THICKNESS)
    o, g = Oracle(m), AstroGPU(m)
    n, ni = o.n, o.int_vec_size
    st = M.make_state(n, disp=1e-4 * rng.standard_normal(n), internal_disp=1e-5 * rng.standard_normal(ni))
    g.getElasticSolnLoad(1, state=st, export=False)
    g.scaleElasticMPC()
    dldu = rng.standard_normal(n)
    idldu = rng.standard_normal(ni)
    # the learned solver: plain FP64 Jacobi-GMRES stalls near 1e-12 on this shell system (its
    # last digits move with the rounding of the element kernels)
    dldd, lam, ilam, s = g.getTotaldLdD(dldu, int_dldu=idldu, state=st, rtol=1e-12, method=SOLVER_FGMRES_LEARNED)
    od, olam, oilam = o.total_dldd(dldu, int_dldu=idldu, state=st)
    assert s.status == 0
    # the shell system is ill-conditioned (drilling DOF): its element matrices agree with the
    # oracle's to ~1e-11, so the GPU adjoint's residual in the oracle's condensed system is
    # ~1e-11 x cond; the adjoint and the gradient are compared at that conditioning
    _, _, mat, cols, imat = o.el_soln_load(1, state=st)
    mm, _ = o.scale_mpc(mat)
    A = o.csr_scipy(mat, cols) + o.mpc_scipy(mm).T @ o.mpc_scipy(mm)
    b = o.update_external_rhs(dldu, idldu, imat)
    assert np.linalg.norm(A @ lam - b) <= 1e-7 * np.linalg.norm(b)
    assert _rel(lam, olam) < 1e-6
    assert _rel(ilam, oilam) < 1e-6
    assert _rel(dldd, od) < 1e-6


def test_adjoint_needs_assembly():
    m = M.add_design_variables(M.hex_block(nx=3, ny=2, nz=2, seed=1), 2, M.DCAT_ELASTIC_MODULUS)
    g = AstroGPU(m)
    with pytest.raises(AstroError):
        g.getTotaldLdD(np.ones(g.n))


def test_transient_adjoint_matches_oracle():
    """The Newmark backward sweep (astro_total_dldd_transient) against the oracle's restatement on
    the same stored states: dL/dD and the adjoint of step 1, with objective partials in u, v, a and
    at the internal DOF."""
    import newmark_ref as NR

    m = M.plate_shell(nx=6, ny=4, lx=1.0, ly=0.5, t=0.01, E=7e10, nu=0.33, rho=2700.0, pressure=0.0)
    m = M.add_design_variables(m, 3, M.DCAT_LAYUP_THICKNESS)
    o, g = Oracle(m), AstroGPU(m)
    n, ni = o.n, o.int_vec_size
    dt, beta, gamma, steps = 1e-4, 0.25, 0.5, 4
    pattern = np.zeros(n)
    pattern[o.n_dof_index[m.num_nodes - 1, 2] - 1] = 1.0
    amp = 50.0 * np.sin(2 * np.pi * 500.0 * dt * np.arange(1, steps + 1))
    D, V, A, I = NR.newmark_states(o, pattern, amp, dt, beta, gamma, steps)
    rng = np.random.default_rng(8)
    w = rng.standard_normal((steps, n))
    wv = 1e-3 * rng.standard_normal((steps, n))
    wa = 1e-7 * rng.standard_normal((steps, n))
    wi = rng.standard_normal((steps, ni))
    dldd, lam, st = g.getTotaldLdD_transient(D, V, A, I, dt, beta, gamma, dldu=w, dldv=wv, dlda=wa, int_dldu=wi,
                                             rtol=1e-13)
    od, olam = o.total_dldd_transient(D, V, A, I, dt, beta, gamma, dldu=w, dldv=wv, dlda=wa, int_dldu=wi)
    assert st.status == 0
    assert _rel(lam, olam) < 1e-6
    assert _rel(dldd, od) < 1e-6
