"""Known-answer tests of the CPU oracle (mechanics, not reference outputs: the reference ships
none).  They pin the restatement: rigid-body modes, symmetry, patch test, beam theory, the
skyline LDL^T and the reference GMRES."""
import ctypes

import numpy as np
import pytest
import scipy.sparse.linalg as spla

from misc_gb300 import model as M
from oracle import Oracle
from oracle.oracle import _lib


def _rigid_modes_hex(X):
    modes = []
    for c in range(3):
        u = np.zeros((3, 8)); u[c, :] = 1; modes.append(u.ravel())
    for a, b in [(0, 1), (1, 2), (0, 2)]:
        u = np.zeros((3, 8)); u[a, :] = -X[:, b]; u[b, :] = X[:, a]; modes.append(u.ravel())
    return modes


def test_hex8_rigid_symmetric_psd():
    m = M.hex_block(3, 2, 2, lx=1.0, ly=0.7, lz=0.6, seed=3)
    o = Oracle(m)
    for el in (1, 5, 12):
        _, k = o.element(el)
        K = k[:24, :24]
        s = np.abs(K).max()
        assert np.abs(K - K.T).max() <= 1e-14 * s
        X = m.node_list[m.element_list[el - 1] - 1]
        for u in _rigid_modes_hex(X):
            assert np.abs(K @ u).max() <= 1e-12 * s
        ev = np.linalg.eigvalsh(K)
        assert ev[6] > 1e-6 * ev[-1] and ev[0] > -1e-12 * ev[-1]


def test_hex8_patch_test_linear_field():
    """A linear displacement field produces no internal force at interior nodes."""
    m = M.hex_block(3, 3, 3, lx=1.0, ly=1.0, lz=1.0, seed=5, jitter=0.2, sigma=0.0)
    o = Oracle(m)
    load, _, mat, cols, _ = o.el_soln_load(1)
    K = o.csr_scipy(mat, cols)
    G = np.array([[1e-3, 2e-4, -3e-4], [5e-4, -1e-3, 1e-4], [2e-4, 3e-4, 7e-4]])
    X = m.node_list
    U = X @ G.T
    u = np.zeros(o.n)
    for a in range(m.num_nodes):
        for c in range(3):
            u[o.n_dof_index[a, c] - 1] = U[a, c]
    f = K @ u
    interior = [a for a in range(m.num_nodes) if np.all((X[a] > 1e-9) & (X[a] < 1 - 1e-9))]
    assert interior
    fi = np.array([f[o.n_dof_index[a, c] - 1] for a in interior for c in range(3)])
    assert np.abs(fi).max() <= 1e-9 * np.abs(f).max()


def test_shell_reference_tangent_omits_mean_rotation_term():
    """The reference's shell tangent (r_getInstDof rotation derivative) omits the dependence of
    the element mean rotation on each nodal rotation; rigid rotations then load the element.
    The oracle keeps that behaviour by default; the diagnostic switch restores invariance."""
    L = _lib()
    L.orc_set_quirk.argtypes = [ctypes.c_int, ctypes.c_int]
    m = M.plate_shell(nx=1, ny=1, lx=1.0, ly=1.0, t=0.1, E=1e6, nu=0.0, clamp=None, y0=0.0)
    X = m.node_list[m.element_list[0, :4] - 1]
    u = np.zeros((6, 4)); u[2] = X[:, 1]; u[3] = 1.0   # rigid rotation about x
    v = np.zeros(33); v[:24] = u.ravel()
    try:
        for q, expect_zero in ((0, False), (1, True)):
            L.orc_set_quirk(1, q)
            _, k = Oracle(m).element(1)
            r = np.abs(k @ v).max() / np.abs(k).max()
            assert (r < 1e-12) == expect_zero
    finally:
        L.orc_set_quirk(1, 0)


def test_shell_cantilever_beam_theory_with_consistent_tangent():
    """shellBeam fixture (Working/shellBeamModelInput.yaml): tip load 2, L = 10, t = 0.1, E = 1e6.
    With the consistent tangent the tip deflection lies between the plate-strip (7.28) and
    Euler-Bernoulli (8.0) values; the reference's own tangent gives about 31.6."""
    L = _lib()
    L.orc_set_quirk.argtypes = [ctypes.c_int, ctypes.c_int]
    m = M.shell_beam()
    try:
        L.orc_set_quirk(1, 1)
        o = Oracle(m)
        A, b, *_ = o.static_system()
        x = spla.spsolve(A.tocsc(), b)
        w = x[o.n_dof_index[10, 2] - 1]
        assert 7.2 < w < 8.05
    finally:
        L.orc_set_quirk(1, 0)
    o = Oracle(m)
    A, b, *_ = o.static_system()
    w_ref = spla.spsolve(A.tocsc(), b)[o.n_dof_index[10, 2] - 1]
    assert 30.0 < w_ref < 33.0


def test_skyline_ldl_and_reference_gmres():
    m = M.hex_block(4, 2, 2, lx=1.0, ly=0.5, lz=0.5, seed=1)
    o = Oracle(m)
    A, b, mat, cols, mm, mr = o.static_system()
    lt = o.convert_to_ltri(mat, cols, mm)
    fac = o.ldl_fact(lt, o.lt_range)
    # the factor solves the skyline matrix itself exactly
    n = o.n
    S = np.zeros((n, n))
    for i in range(n):
        r0, r1 = o.lt_range[i], o.lt_range[i + 1]
        S[i, i - (r1 - r0) + 1:i + 1] = lt[r0:r1]
    S = np.tril(S) + np.tril(S, -1).T
    y = np.random.default_rng(0).standard_normal(n)
    x = o.ldl_solve(fac, o.lt_range, S @ y)
    assert np.linalg.norm(x - y) <= 1e-8 * np.linalg.norm(y)
    xd = spla.spsolve(A.tocsc(), b)
    xg, cyc = o.gmres(mat, cols, mm, fac, b)
    assert np.linalg.norm(xg - xd) <= 1e-6 * np.linalg.norm(xd)


def test_solver_max_bw_wraps_like_fortran_integers():
    """solverMaxBW = min b with b^3 >= 27*numNodes^2 in 32-bit wrapping integers
    (Working/AStrO_runJob.f90:106-114): 155 for 369 nodes, 1289 for 70,785 nodes (wrapped)."""
    m = M.config1()
    assert Oracle(m).solver_max_bw == 155
    nn = 70785
    t = np.int64(27) * nn * nn
    t32 = np.int64(((t + 2**31) % 2**32) - 2**31)
    b = 1
    while b**3 < t32:
        b += 1
    assert b == 1289


def _fd_drdd(model_fn, dvar, state_fn, rel=1e-6):
    """Central difference of the residual (-elastic_load) with respect to design variable dvar."""
    m0 = model_fn()
    step = rel * max(1.0, abs(m0.d_value[dvar - 1]))
    if m0.d_category[dvar - 1] == M.DCAT_LAYUP_THICKNESS:
        step = rel * float(m0.layup_thickness[0])
    elif m0.d_category[dvar - 1] == M.DCAT_ELASTIC_MODULUS:
        step = rel * float(m0.material_elastic[0, m0.d_component[dvar - 1] - 1])
    out = []
    for sgn in (1.0, -1.0):
        m = model_fn()
        m.d_value = m.d_value.copy()
        m.d_value[dvar - 1] += sgn * step
        o = Oracle(m)
        load, iload, *_ = o.el_soln_load(0, state=state_fn(o))
        out.append((-load, -iload[:o.int_vec_size]))
    return (out[0][0] - out[1][0]) / (2 * step), (out[0][1] - out[1][1]) / (2 * step)


@pytest.mark.parametrize("kind", ["shell_thickness", "brick_modulus"])
def test_complex_step_matches_central_difference(kind):
    """The oracle's complex twin (getdRelasticdD) against a central difference of the real
    residual.  The complex path's Gauss points are the single-precision 1/sqrt(3), so the two
    differ at the 1e-8 level; the check is 1e-5 relative."""
    if kind == "shell_thickness":
        def model_fn():
            m = M.plate_shell(nx=4, ny=3, lx=2.0, ly=1.0, t=0.03, E=7e10, nu=0.33)
            return M.add_design_variables(m, 3, M.DCAT_LAYUP_THICKNESS)
    else:
        def model_fn():
            m = M.hex_block(nx=3, ny=2, nz=2, jitter=0.1, seed=3)
            return M.add_design_variables(m, 2, M.DCAT_ELASTIC_MODULUS, component=1)

    def state_fn(o):
        rng = np.random.default_rng(7)
        return M.make_state(o.n, disp=1e-3 * rng.standard_normal(o.n),
                            internal_disp=1e-4 * rng.standard_normal(max(o.int_vec_size, 1)))

    o = Oracle(model_fn())
    for dvar in (1, 2):
        cs, ics = o.drdd_complex(dvar, 1e-14, state=state_fn(o))
        fd, ifd = _fd_drdd(model_fn, dvar, state_fn)
        assert np.linalg.norm(cs) > 0
        assert np.linalg.norm(cs - fd) <= 1e-5 * np.linalg.norm(fd)
        if o.int_vec_size:
            assert np.linalg.norm(ics - ifd) <= 1e-5 * np.linalg.norm(ifd)


def test_static_condensation_round_trip():
    """Condensed solve + internal-DOF recovery (updateExternalRHS / updateInternalSoln with the
    intended loop bounds) equals the solve of the full nodal + incompatible-mode system assembled
    from the uncondensed element matrices."""
    import scipy.sparse as sp
    m = M.plate_shell(nx=4, ny=3, lx=2.0, ly=1.0, t=0.03, E=7e10, nu=0.33)
    o = Oracle(m)
    n, ni = o.n, o.int_vec_size
    load, iload, mat, cols, imat = o.el_soln_load(1)
    mm, mr = o.scale_mpc(mat)
    Cm = o.mpc_scipy(mm)
    rows, cls, vals = [], [], []
    for el in range(1, m.num_els + 1):
        _, K = o.element(el, 1)
        dofs = []
        for i in range(24):
            comp, lnd = i // 4 + 1, i % 4 + 1
            nd = int(m.element_list[el - 1, lnd - 1])
            dofs.append(int(o.n_dof_index[nd - 1, comp - 1]) - 1)
        dofs += [n + 8 * (el - 1) + k for k in range(8)]   # intVecRange: 8 incompatible modes per shell
        for a in range(32):
            for b in range(32):
                rows.append(dofs[a]); cls.append(dofs[b]); vals.append(K[a, b])
    Kf = sp.csr_matrix((vals, (rows, cls)), shape=(n + ni, n + ni))
    P = sp.bmat([[Cm.T @ Cm, None], [None, sp.csr_matrix((ni, ni))]])
    rng = np.random.default_rng(6)
    f, g = rng.standard_normal(n), rng.standard_normal(ni)
    full = spla.spsolve((Kf + P).tocsc(), np.concatenate([f, g]))
    rhs = o.update_external_rhs(f, g, imat)
    A = (o.csr_scipy(mat, cols) + Cm.T @ Cm).tocsc()
    u = spla.spsolve(A, rhs)
    a = o.update_internal_soln(u, np.zeros(ni), g, imat)
    assert np.linalg.norm(u - full[:n]) <= 1e-8 * np.linalg.norm(full[:n])
    assert np.linalg.norm(a - full[n:]) <= 1e-8 * np.linalg.norm(full[n:])


def test_static_adjoint_gradient_matches_central_difference():
    """getTotaldLdD (static) for the compliance L(d) = b . u(d): the adjoint gradient at the solved
    state equals central differences of L over re-assembled systems (modulus design variables,
    relative step 1e-4 of E).  The adjoint uses the tangent at the solved state, whose stress
    stiffness is of the order of the strain: a 1e2 Pa traction keeps it near 1e-9."""
    import scipy.sparse.linalg as spla

    def build(dv):
        m = M.hex_block(nx=4, ny=2, nz=2, jitter=0.1, seed=3, traction=1.0e2)
        m = M.add_design_variables(m, 2, M.DCAT_ELASTIC_MODULUS, component=1)
        m.d_value = np.asarray(dv, np.float64)
        return m

    def compliance(dv):
        o = Oracle(build(dv))
        A, b, *_ = o.static_system()
        u = spla.spsolve(A.tocsc(), b)
        return b @ u, u, b, o

    d0 = np.zeros(2)
    L0, u, b, o = compliance(d0)
    st = M.make_state(o.n, disp=u)
    g, lam, _ = o.total_dldd(b, state=st)
    step = 1e-4 * 2.0e11
    for k in range(2):
        e = np.zeros(2)
        e[k] = step
        fd = (compliance(d0 + e)[0] - compliance(d0 - e)[0]) / (2 * step)
        assert abs(g[k] - fd) <= 1e-5 * abs(fd), (k, g[k], fd)


def test_transient_adjoint_gradient_matches_central_difference():
    """getTotaldLdD (Newmark) for L = sum_i w_i . u_i over a shell plate's time loop: the backward
    sweep (augmentdLdu, per-step adjoints, complex-step dRu/dD) equals central differences of L over
    re-run forward loops (thickness variables, step 1e-4 of t; a 1e-3 N load keeps the geometry
    linear to ~1e-9).  With the consistent shell tangent: the reference's default tangent is not the
    derivative of its residual (a quirk), and an adjoint gradient needs K = dRu/du; with the default
    tangent the same comparison fails by O(1), for the static shell gradient too."""
    import newmark_ref as NR

    def build(dv):
        m = M.plate_shell(nx=4, ny=2, lx=1.0, ly=0.5, t=0.01, E=7e10, nu=0.33, rho=2700.0, pressure=0.0)
        m = M.add_design_variables(m, 2, M.DCAT_LAYUP_THICKNESS)
        m.d_value = np.asarray(dv, np.float64)
        return m

    dt, beta, gamma, steps = 1e-4, 0.25, 0.5, 3
    rng = np.random.default_rng(4)
    m0 = build(np.zeros(2))
    o0 = Oracle(m0)
    o0.L.orc_set_quirk(1, 1)
    try:
        _transient_fd_check(o0, m0, build, NR, dt, beta, gamma, steps, rng)
    finally:
        o0.L.orc_set_quirk(1, 0)


def _transient_fd_check(o0, m0, build, NR, dt, beta, gamma, steps, rng):
    w = rng.standard_normal((steps, o0.n))
    pattern = np.zeros(o0.n)
    pattern[o0.n_dof_index[m0.num_nodes - 1, 2] - 1] = 1.0
    amp = 1e-3 * np.array([1.0, 0.6, -0.4])

    def objective(dv):
        o = Oracle(build(dv))
        D, *_ = NR.newmark_states(o, pattern, amp, dt, beta, gamma, steps)
        return float(sum(w[i] @ D[i + 1] for i in range(steps)))

    D, V, A, I = NR.newmark_states(o0, pattern, amp, dt, beta, gamma, steps)
    g, _ = o0.total_dldd_transient(D, V, A, I, dt, beta, gamma, dldu=w)
    step = 1e-6
    for k in range(2):
        e = np.zeros(2)
        e[k] = step
        fd = (objective(e) - objective(-e)) / (2 * step)
        assert abs(g[k] - fd) <= 1e-5 * abs(fd), (k, g[k], fd)


def test_static_adjoint_shell_matches_central_difference_with_consistent_tangent():
    """The static design gradient for shell thickness variables (internal DOF condensed) against
    central differences of L = w . u(d); with the consistent tangent (see the transient test)."""
    import scipy.sparse.linalg as spla

    def build(dv):
        m = M.plate_shell(nx=4, ny=2, lx=1.0, ly=0.5, t=0.01, E=7e10, nu=0.33, rho=2700.0, pressure=1e-3)
        m = M.add_design_variables(m, 2, M.DCAT_LAYUP_THICKNESS)
        m.d_value = np.asarray(dv, np.float64)
        return m

    def solve(dv):
        o = Oracle(build(dv))
        _, iload, mat, cols, imat = o.el_soln_load(1)
        mm, mr = o.scale_mpc(mat)
        A = (o.csr_scipy(mat, cols) + o.mpc_scipy(mm).T @ o.mpc_scipy(mm)).tocsc()
        b = np.zeros(o.n)
        o.constraint_load(mm, mr, np.zeros(o.n), b)
        o.applied_load(b)
        ni = o.int_vec_size
        u = spla.spsolve(A, o.update_external_rhs(b, iload[:ni], imat))
        return u, o.update_internal_soln(u, np.zeros(ni), iload[:ni], imat)[:ni], o

    u, iu, o0 = solve(np.zeros(2))
    o0.L.orc_set_quirk(1, 1)
    try:
        u, iu, o0 = solve(np.zeros(2))
        w = np.random.default_rng(4).standard_normal(o0.n)
        g, _, _ = o0.total_dldd(w, state=M.make_state(o0.n, disp=u, internal_disp=iu))
        step = 1e-6
        for k in range(2):
            e = np.zeros(2)
            e[k] = step
            fd = (w @ solve(e)[0] - w @ solve(-e)[0]) / (2 * step)
            assert abs(g[k] - fd) <= 1e-5 * abs(fd), (k, g[k], fd)
    finally:
        o0.L.orc_set_quirk(1, 0)


def test_body_load_totals():
    """Body loads: the nodal forces add up to the resultant (the shape functions' partition of
    unity): b V for a body force, rho V a for gravity, rho w^2 sum(V_e r_e) for the centrifugal
    load about the z axis (r_e = element centroid's distance from the axis), rho t A a for the
    shell's gravitational load."""
    lx, ly, lz, rho = 1.5, 1.0, 0.75, 7800.0
    m = M.hex_block(6, 4, 3, lx=lx, ly=ly, lz=lz, jitter=0.0, rho=rho)
    o = Oracle(m)
    V = lx * ly * lz
    tot = lambda v: v.reshape(3, -1).sum(axis=1)
    assert np.allclose(tot(o.body_load(0, [1.5, -2.0, 3.0])), np.array([1.5, -2.0, 3.0]) * V, rtol=1e-12)
    assert np.allclose(tot(o.body_load(1, [0.0, 0.0, -9.81])), [0.0, 0.0, -9.81 * rho * V], rtol=1e-12, atol=1e-9)
    w = 12.0
    c = tot(o.body_load(2, [0.0, 0.0, 0.0, 0.0, 0.0, 2.0, w]))
    assert np.allclose(c, [rho * w * w * V * lx / 2, rho * w * w * V * ly / 2, 0.0], rtol=1e-12, atol=1e-6)
    # a subset: the elements of the first x layer only
    els = [e + 1 for e in range(m.num_els) if e % 6 == 0]
    assert np.allclose(tot(o.body_load(0, [0.0, 1.0, 0.0], elements=els)), [0.0, V / 6, 0.0], rtol=1e-12, atol=1e-12)
    p = M.plate_shell(nx=5, ny=4, lx=2.0, ly=1.0, t=0.03, rho=2700.0)
    op = Oracle(p)
    s = op.body_load(1, [0.0, 0.0, -9.81, 0.0, 0.0, 0.0]).reshape(6, -1).sum(axis=1)
    assert np.isclose(s[2], -9.81 * 2700.0 * 0.03 * 2.0, rtol=1e-12)
    assert np.allclose(s[[0, 1, 3, 4, 5]], 0.0, atol=1e-9)


def test_thermal_conduction_kats():
    """Thermal path of the oracle: steady conduction through a brick bar with the end faces held
    at 20 and 80 gives the linear profile (penalty constraints: 1e-4) and the heat flux k A dT/dx
    through the end; uniform heating of the capacitance term gives rho c V Tdot; heat generation
    integrates to q V (bricks) and q t A (shells); the shell conductivity matrix annihilates a
    uniform temperature."""
    import scipy.sparse.linalg as spla
    m = M.hex_block(6, 2, 2, lx=3.0, ly=1.0, lz=1.0, jitter=0.0)
    o = Oracle(m)
    nm = len(m.material_density)
    k = 45.0
    cond, sh = np.tile([k, k, k, 0, 0, 0], (nm, 1)), np.full(nm, 460.0)
    X = m.node_list
    left = np.nonzero(X[:, 0] == 0)[0] + 1
    right = np.nonzero(np.isclose(X[:, 0], 3.0))[0] + 1
    nodes = np.concatenate([left, right])
    rhs = np.concatenate([np.full(len(left), 20.0), np.full(len(right), 80.0)])
    mpc = (np.arange(len(nodes) + 1), nodes, np.ones(len(nodes)), rhs)
    A, b, _ = o.thermal_system(cond, sh, mpc)
    T = spla.spsolve(A.tocsc(), b)
    assert np.abs(T[o.current_rank - 1] - (20 + 60 * X[:, 0] / 3.0)).max() < 1e-4
    load, *_ = o.thermal_soln_load(cond, sh, 0, temp=T)
    assert abs(load[o.current_rank[left - 1] - 1].sum() - k * 1.0 * 20.0) < 1e-3
    N = m.num_nodes
    load2, *_ = o.thermal_soln_load(cond, sh, 0, temp=np.ones(N), prev_temp=np.zeros(N), prev_tdot=np.zeros(N),
                                    dynamic=1, gamma=0.5, del_t=0.1)
    assert np.isclose(-load2.sum(), 7800.0 * 460.0 * 3.0 * (1 / 0.5) * (1 / 0.1), rtol=1e-12)
    assert np.isclose(o.thermal_heat_gen(5.0).sum(), 15.0, rtol=1e-12)
    # surface flux on the x = L faces (area 1): the nodal values sum to -flux * area
    xf = [e + 1 for e in range(m.num_els) if e % 6 == 5]
    assert np.isclose(o.thermal_surface_flux(xf, [4] * len(xf), 2.0).sum(), -2.0, rtol=1e-12)
    p = M.plate_shell(nx=4, ny=2, lx=2.0, ly=1.0, t=0.02)
    op = Oracle(p)
    assert np.isclose(op.thermal_heat_gen(3.0).sum(), 3.0 * 2.0 * 0.02, rtol=1e-12)
    Ap, _, _ = op.thermal_system([[k, k, k, 0, 0, 0]], [900.0])
    assert np.abs(Ap @ np.ones(p.num_nodes)).max() < 1e-12 * abs(Ap).max()


def _brick_im(m):
    m.element_type = np.full(m.num_els, 81, np.int32)
    return m


def test_hex81_condensed_rigid_symmetric_psd():
    """brickIM (type 81: brick8 plus the three incompatible bubbles, 9 internal DOF condensed):
    the condensed 24x24 stiffness is symmetric, annihilates the rigid-body modes and has exactly
    six zero eigenvalues."""
    m = _brick_im(M.hex_block(3, 2, 2, lx=1.0, ly=0.7, lz=0.6, seed=3))
    o = Oracle(m)
    assert o.int_vec_size == 9 * m.num_els and o.int_mat_size == 297 * m.num_els
    ke = o.element_matrices()
    for el in (1, 5, 12):
        K = ke[el - 1]
        s = np.abs(K).max()
        assert np.abs(K - K.T).max() <= 1e-13 * s
        X = m.node_list[m.element_list[el - 1] - 1]
        for u in _rigid_modes_hex(X):
            assert np.abs(K @ u).max() <= 1e-11 * s
        ev = np.linalg.eigvalsh(K)
        assert ev[6] > 1e-6 * ev[-1] and ev[0] > -1e-12 * ev[-1]


def test_hex81_patch_test_parallelepiped():
    """On undistorted elements the incompatible modes vanish under a linear displacement field:
    the condensed assembly leaves no force at the interior nodes (the reference integrates the
    bubbles with the point Jacobian, without the centroid-Jacobian correction, so distorted meshes
    do not pass this test and none is claimed here)."""
    m = _brick_im(M.hex_block(3, 3, 3, lx=1.0, ly=1.0, lz=1.0, seed=5, jitter=0.0, sigma=0.0))
    o = Oracle(m)
    load, iload, mat, cols, imat = o.el_soln_load(1)
    K = o.csr_scipy(mat, cols)
    G = np.array([[1e-3, 2e-4, -3e-4], [5e-4, -1e-3, 1e-4], [2e-4, 3e-4, 7e-4]])
    X = m.node_list
    U = X @ G.T
    u = np.zeros(o.n)
    for a in range(m.num_nodes):
        for c in range(3):
            u[o.n_dof_index[a, c] - 1] = U[a, c]
    f = K @ u
    interior = [a for a in range(m.num_nodes) if np.all((X[a] > 1e-9) & (X[a] < 1 - 1e-9))]
    fi = np.array([f[o.n_dof_index[a, c] - 1] for a in interior for c in range(3)])
    assert np.abs(fi).max() <= 1e-9 * np.abs(f).max()
    # and the recovered incompatible modes of the field are zero
    a = o.update_internal_soln(u, np.zeros(o.int_vec_size), None, imat)
    assert np.abs(a).max() <= 1e-12 * np.abs(u).max()


def _cantilever(eltype, nx=10):
    """Cantilever of nx x 1 x 1 bricks (length 10, square section 1 x 1, E = 1e7, nu = 0), x = 0
    clamped, a transverse tip force of 1 split over the four tip nodes (z direction)."""
    m = M.hex_block(nx, 1, 1, lx=10.0, ly=1.0, lz=1.0, jitter=0.0, sigma=0.0, E_med=1.0e7, nu=0.0)
    m.element_type = np.full(m.num_els, eltype, np.int32)
    m.face_el = np.zeros(0, np.int32)
    m.face_num = np.zeros(0, np.int32)
    tip = [a + 1 for a in range(m.num_nodes) if abs(m.node_list[a, 0] - 10.0) < 1e-9]
    m.point_loads = [(nd, 3, 0.25) for nd in tip]
    o = Oracle(m)
    A, b, *_ = o.static_system()
    u = spla.spsolve(A.tocsc(), b)
    return np.mean([u[o.n_dof_index[nd - 1, 2] - 1] for nd in tip])


def test_hex81_bending_without_shear_locking():
    """The incompatible modes remove the parasitic shear of the fully integrated brick8 in
    bending: on a 10 x 1 x 1 cantilever the brickIM tip deflection is within 3 % of Timoshenko
    beam theory (P L^3 / 3EI + P L / kGA), while the brick8 one is more than 20 % too stiff."""
    E, G, L, I, A = 1.0e7, 0.5e7, 10.0, 1.0 / 12.0, 1.0
    exact = L ** 3 / (3 * E * I) + L / (5.0 / 6.0 * G * A)
    d81, d8 = _cantilever(81), _cantilever(8)
    assert abs(d81 - exact) <= 0.03 * exact, (d81, exact)
    assert d8 < 0.8 * exact, (d8, exact)


def _orthotropic(m):
    me = m.material_elastic.copy()
    me[:, 1] *= 0.5
    me[:, 2] *= 0.3
    me[:, 7] *= 0.7
    m.material_elastic = me
    return m


def _brick(eltype=8):
    m = _orthotropic(M.hex_block(nx=3, ny=2, nz=2, jitter=0.1, seed=3))
    m.element_type = np.full(m.num_els, eltype, np.int32)
    return m


_CAT_CASES = {
    # name: (model builder, step, dynamic state)
    "brick_density": (lambda: M.add_design_variables(_brick(), 2, M.DCAT_DENSITY), 1e-6 * 7800.0, True),
    "brick_orientation": (lambda: M.add_design_variables(_brick(), 2, M.DCAT_ORIENTATION, component=3), 1e-6, False),
    "brickIM_orientation": (lambda: M.add_design_variables(_brick(81), 2, M.DCAT_ORIENTATION, component=1), 1e-6,
                            False),
    "brick_node_coord": (lambda: M.add_node_design_variables(_brick(), [[6, 7, 18], [11, 23]], M.DCAT_NODE_COORD,
                                                             component=2), 1e-7, False),
    "brickIM_node_coord": (lambda: M.add_node_design_variables(_brick(81), [[6, 7, 18], [11, 23]],
                                                               M.DCAT_NODE_COORD, component=1), 1e-7, True),
    "shell_zoffset": (lambda: M.add_design_variables(M.plate_shell(nx=4, ny=3, lx=2.0, ly=1.0, t=0.03), 2,
                                                     M.DCAT_LAYUP_ZOFFSET), 1e-6, False),
    "shell_layup_angle": (lambda: M.add_design_variables(_layered_plate(), 2, M.DCAT_LAYUP_ANGLE, layer=2), 1e-6,
                          False),
    "shell_layup_density": (lambda: M.add_design_variables(_layered_plate(), 2, M.DCAT_LAYUP_DENSITY, layer=1),
                            1e-6 * 2700.0, True),
    "shell_layup_modulus": (lambda: M.add_design_variables(_layered_plate(), 2, M.DCAT_LAYUP_MODULUS, layer=2,
                                                           component=1), 1e-6 * 7e10, False),
    "shell_layup_poisson": (lambda: M.add_design_variables(_layered_plate(), 2, M.DCAT_LAYUP_MODULUS, layer=1,
                                                           component=3), 1e-6, False),
    "shell_layup_shear_modulus": (lambda: M.add_design_variables(_layered_plate(), 2, M.DCAT_LAYUP_MODULUS,
                                                                 layer=2, component=4), 1e-6 * 1e10, False),
}


def _layered_plate():
    """shell4 plate with a two-layer orthotropic laminate (0 and 0.4 rad): the layer angle moves
    the in-plane and bending stiffness."""
    m = M.plate_shell(nx=4, ny=3, lx=2.0, ly=1.0, t=0.03, E=7e10, nu=0.33)
    me = m.material_elastic.copy()
    me[0, 1] *= 0.4
    me[0, 6] *= 0.6
    m.material_elastic = me
    m.sec_layup_range = np.array([0, 2], np.int32)
    m.layup_mat_id = np.array([1, 1], np.int32)
    m.layup_thickness = np.array([0.012, 0.018])
    m.layup_angle = np.array([0.0, 0.4])
    return m


@pytest.mark.parametrize("case", sorted(_CAT_CASES))
def test_design_categories_complex_step_matches_central_difference(case):
    """Every design-variable category the oracle restates (density, orientation, node
    coordinates, layup zOffset, layer angle, layer density and the layer's elastic constants)
    against a central difference of
    its real residual; 1e-5 relative (the complex path's single-precision Gauss points)."""
    build, step, dyn = _CAT_CASES[case]

    def state_fn(o):
        rng = np.random.default_rng(7)
        n, ni = o.n, max(o.int_vec_size, 1)
        kw = {}
        if dyn:
            kw = dict(prev_disp=1e-3 * rng.standard_normal(n), prev_vel=1e-1 * rng.standard_normal(n),
                      prev_acc=10.0 * rng.standard_normal(n), prev_int_disp=1e-4 * rng.standard_normal(ni),
                      dynamic=1, beta=0.25, gamma=0.5, del_t=1e-3)
        return M.make_state(n, disp=1e-3 * rng.standard_normal(n), internal_disp=1e-4 * rng.standard_normal(ni),
                            **kw)

    o = Oracle(build())
    for dvar in (1, 2):
        cs, ics = o.drdd_complex(dvar, 1e-14, state=state_fn(o))
        out = []
        for sgn in (1.0, -1.0):
            m = build()
            m.d_value = m.d_value.copy()
            m.d_value[dvar - 1] += sgn * step
            oo = Oracle(m)
            load, iload, *_ = oo.el_soln_load(0, state=state_fn(oo))
            out.append((-load, -iload[:oo.int_vec_size]))
        fd, ifd = (out[0][0] - out[1][0]) / (2 * step), (out[0][1] - out[1][1]) / (2 * step)
        assert np.linalg.norm(cs) > 0, case
        assert np.linalg.norm(cs - fd) <= 1e-5 * np.linalg.norm(fd), (case, dvar)
        if o.int_vec_size and np.linalg.norm(ifd) > 0:
            assert np.linalg.norm(ics - ifd) <= 1e-5 * np.linalg.norm(ifd), (case, dvar)


def test_node_load_design_variables():
    """nodeLoad variables: the applied nodal load is linear in them inside their activity window
    and absent outside it; getdRelasticdD's load branch is minus the load per unit variable."""
    m = M.add_node_design_variables(M.hex_block(nx=3, ny=2, nz=2, seed=3), [[5, 9], [12]], M.DCAT_NODE_LOAD,
                                    component=2, value=3.0, act_time=(0.5, 2.0))
    o = Oracle(m)
    f = o.design_node_load(1.0)
    expect = np.zeros(o.n)
    for nd, d in ((5, 0), (9, 0), (12, 1)):
        expect[o.n_dof_index[nd - 1, 1] - 1] += m.d_value[d]
    assert np.array_equal(f, expect)
    assert not np.any(o.design_node_load(3.0))
    dr = o.node_load_drdd(1, 1.0)
    assert np.allclose(dr, -expect / 3.0 * (np.arange(o.n) != o.n_dof_index[11, 1] - 1), rtol=0, atol=1e-12)
    assert not np.any(o.node_load_drdd(1, 0.2))
