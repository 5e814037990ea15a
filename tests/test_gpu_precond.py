"""Polynomial graph-convolution preconditioner on the GPU, through the C ABI:
eigenvalue estimate, training loss and gradient against the numpy restatement (FP64, 1e-9) and
against central differences of the device loss, monotone training, and the learned solver
(FP32 inner GMRES right-preconditioned by the network, FP64 refinement) against the direct
solution and against the Jacobi-preconditioned mixed solver on a held-out mesh."""
import numpy as np
import pytest
import scipy.sparse.linalg as spla

from misc_gb300 import model as M
from misc_gb300.astro import (SOLVER_FGMRES_LEARNED, SOLVER_FGMRES_MIXED, AstroError, AstroGPU, precond_init)
from oracle import Oracle
import poly_ref as R

pytestmark = pytest.mark.gpu


def _system(m, fp32=False):
    g, o = AstroGPU(m), Oracle(m)
    g.getElasticSolnLoad(1, export=False)
    if fp32:
        g.assemble_fp32()
    g.scaleElasticMPC()
    A, b, *_ = o.static_system()
    return g, o, A.tocsr(), b


def _samples(A, S, seed, smooth=(0, 2, 8)):
    """white noise and Jacobi-smoothed vectors (the low end of the spectrum)"""
    rng = np.random.default_rng(seed)
    dinv = 1.0 / A.diagonal()
    out = []
    for s in range(S):
        v = rng.standard_normal(A.shape[0])
        for _ in range(smooth[s % len(smooth)]):
            v = v - 0.3 * dinv * (A @ v)
        out.append(v)
    return np.array(out)


def _shell():
    m = M.plate_shell(nx=8, ny=4, lx=2.0, ly=1.0, t=0.03, E=7e10, nu=0.33)
    rng = np.random.default_rng(2)
    X = m.node_list.copy()
    X[:, 2] += 0.02 * rng.uniform(-1, 1, len(X))
    m.node_list = X
    return m


CASES = {"brick": (lambda: M.config2(nx=6, ny=4, nz=4, seed=3), 3),
         "shell": (_shell, 6)}


@pytest.mark.parametrize("case", list(CASES))
def test_lambda_bounds(case):
    mk, dpn = CASES[case]
    g, o, A, _ = _system(mk(), fp32=(dpn == 3))  # the FP32 assembly covers brick8 meshes
    d = np.sqrt(1.0 / A.diagonal())
    lam_true = spla.eigsh((A.multiply(d[:, None]).multiply(d[None, :])).tocsr(), k=1, which="LA",
                          return_eigenvectors=False)[0]
    lam64 = g.precond_lambda(64)
    # power iteration approaches the largest eigenvalue from below
    assert 0.7 * lam_true <= lam64 <= lam_true * (1 + 1e-9), (lam64, lam_true)
    if dpn == 3:
        lam32 = g.precond_lambda(32)
        assert abs(lam32 - lam64) <= 1e-3 * lam64
    assert g.precond_lambda(64) == lam64  # deterministic


@pytest.mark.parametrize("case", list(CASES))
def test_loss_grad_matches_numpy(case):
    mk, dpn = CASES[case]
    g, o, A, _ = _system(mk())
    p = precond_init(4, 50.0, dpn)
    rng = np.random.default_rng(7)
    W = p.weight_array() + 0.1 * rng.standard_normal((5, dpn, dpn))
    p.set_weights(W)
    S = _samples(A, 4, 11)
    L, G = g.precond_loss_grad(p, S)
    lam = g.precond_lambda(64) * p.lambda_scale
    Lr, Gr = R.loss_grad(A, 1.0 / A.diagonal(), lam, p.ratio, W, S, R.node_index(o, dpn))
    assert abs(L - Lr) <= 1e-9 * Lr, (L, Lr)
    assert np.linalg.norm(G - Gr) <= 1e-9 * np.linalg.norm(Gr)


def test_gradient_central_difference():
    m, dpn = CASES["brick"][0](), 3
    g, o, A, _ = _system(m)
    p = precond_init(3, 30.0, dpn)
    S = _samples(A, 3, 5)
    L0, G = g.precond_loss_grad(p, S)
    W = p.weight_array()
    rng = np.random.default_rng(3)
    D = rng.standard_normal(W.shape)
    h = 1e-4
    p.set_weights(W + h * D)
    Lp, _ = g.precond_loss_grad(p, S)
    p.set_weights(W - h * D)
    Lm, _ = g.precond_loss_grad(p, S)
    fd = (Lp - Lm) / (2 * h)
    # the loss is quadratic in W: the central difference is exact up to rounding
    assert abs(fd - np.sum(G * D)) <= 1e-6 * max(abs(fd), 1e-12), (fd, np.sum(G * D))


def test_training_decreases_loss():
    g, o, A, _ = _system(M.config2(nx=8, ny=4, nz=4, seed=1))
    p = precond_init(6, 100.0, 3)
    S = _samples(A, 8, 21)
    hist = g.precond_train(p, S, iters=25)
    assert np.all(np.diff(hist) <= 1e-12 * hist[0]), hist
    assert hist[-1] < hist[0]
    L, _ = g.precond_loss_grad(p, S)
    assert abs(L - hist[-1]) <= 1e-10 * hist[-1]


def test_validated_training_is_never_worse():
    g, o, A, _ = _system(M.config2(nx=8, ny=4, nz=4, seed=1), fp32=True)
    for deg, ratio in ((8, 100.0), (16, 1000.0)):
        p0 = precond_init(deg, ratio, 3)
        p, info = g.precond_train_validated(p0, _samples(A, 8, 4), iters=20)
        assert info["loss"][1] < info["loss"][0]
        if info["selected"] == "trained":
            assert info["val_iters_trained"] < info["val_iters_initial"]
            assert p is not p0
        else:
            assert p is p0


def test_learned_solver_converges_with_fewer_iterations():
    """The network trained on one mesh, applied to a held-out mesh of the same family: the
    solution matches the direct solve and the Krylov iterations drop against Jacobi."""
    gt, ot, At, _ = _system(M.config2(nx=8, ny=4, nz=4, seed=1))
    p = precond_init(8, 100.0, 3)
    gt.precond_train(p, _samples(At, 8, 4), iters=20)
    m = M.config2(nx=16, ny=8, nz=8, seed=9)
    g, o, A, bo = _system(m, fp32=True)
    b = g.static_rhs()
    ul, stl = g.solve_static(b, method=SOLVER_FGMRES_LEARNED, rtol=1e-10, precond=p)
    um, stm = g.solve_static(b, method=SOLVER_FGMRES_MIXED, rtol=1e-10)
    ud, std_ = g.solve_static(b, method=SOLVER_FGMRES_LEARNED, rtol=1e-10)  # untrained default network
    assert stl.status == 0 and stl.rel_residual <= 1e-10
    assert std_.status == 0 and std_.rel_residual <= 1e-10
    assert stl.conditional_graph == 1 and stm.conditional_graph == 1
    ur = spla.spsolve(A.tocsc(), bo)
    for u in (ul, ud):
        # FP32 element matrices: the system differs from the FP64 one at ~1e-7 x conditioning
        assert np.linalg.norm(u - ur) <= 5e-5 * np.linalg.norm(ur)
    assert np.linalg.norm(ul - um) <= 1e-8 * np.linalg.norm(um)
    assert stl.iterations * 5 < stm.iterations, (stl.iterations, stm.iterations)


def test_precond_errors():
    g, o, A, _ = _system(M.config2(nx=4, ny=2, nz=2), fp32=True)
    b = g.static_rhs()
    p6 = precond_init(4, 100.0, 6)
    with pytest.raises(AstroError):
        g.solve_static(b, method=SOLVER_FGMRES_LEARNED, precond=p6)  # DOF per node differs
    p = precond_init(4, 100.0, 3)
    p.degree = 0
    with pytest.raises(AstroError):
        g.solve_static(b, method=SOLVER_FGMRES_LEARNED, precond=p)
    p = precond_init(4, 100.0, 3)
    with pytest.raises(AstroError):
        g.precond_loss_grad(p, np.zeros((1, g.n)))  # zero sample


@pytest.mark.parametrize("method", [SOLVER_FGMRES_LEARNED, SOLVER_FGMRES_MIXED, 0])
def test_repeated_solves_reuse_workspace(method):
    """The workspace and the captured restart-cycle graph stay on the context: a repeated solve
    gives the same bits, and a new right-hand side (2 b) flows through the reused graph."""
    g, o, A, bo = _system(M.config2(nx=8, ny=4, nz=4, seed=2), fp32=True)
    b = g.static_rhs()
    u1, s1 = g.solve_static(b, method=method, rtol=1e-10)
    u2, s2 = g.solve_static(2 * b, method=method, rtol=1e-10)
    u3, s3 = g.solve_static(b, method=method, rtol=1e-10)
    assert s1.status == s2.status == s3.status == 0
    assert np.array_equal(u1, u3) and s1.iterations == s3.iterations
    assert np.linalg.norm(u2 - 2 * u1) <= 1e-8 * np.linalg.norm(u2)


@pytest.mark.parametrize("method", [SOLVER_FGMRES_LEARNED, 0])
def test_unrolled_cycles_match_conditional(method):
    """ASTRO_OPT_UNROLLED_CYCLES captures the same kernels without conditional nodes: identical
    iterations and bits."""
    g, o, A, bo = _system(M.config2(nx=8, ny=4, nz=4, seed=2), fp32=True)
    b = g.static_rhs()
    u1, s1 = g.solve_static(b, method=method, rtol=1e-10)
    g.set_option(2, 1)
    u2, s2 = g.solve_static(b, method=method, rtol=1e-10)
    g.set_option(2, 0)
    assert s1.conditional_graph == 1 and s2.conditional_graph == 0
    assert s1.iterations == s2.iterations and np.array_equal(u1, u2)


def test_learned_solver_falls_back_on_non_finite():
    """Weights that overflow FP32 in the hops make the inner Arnoldi values non-finite: the solve
    restarts from the initial guess with the FP32 Jacobi solver and still converges, flagged."""
    g, o, A, bo = _system(M.config2(nx=8, ny=4, nz=4, seed=2), fp32=True)
    b = g.static_rhs()
    p = precond_init(8, 100.0, 3)
    p.set_weights(p.weight_array() * 1e37)
    u, st = g.solve_static(b, method=SOLVER_FGMRES_LEARNED, rtol=1e-10, precond=p)
    assert st.status == 0 and st.fallback == 1 and st.rel_residual <= 1e-10
    um, sm = g.solve_static(b, method=SOLVER_FGMRES_MIXED, rtol=1e-10)
    assert sm.fallback == 0
    assert np.linalg.norm(u - um) <= 1e-7 * np.linalg.norm(um)
    ul, sl = g.solve_static(b, method=SOLVER_FGMRES_LEARNED, rtol=1e-10)
    assert sl.fallback == 0


def test_learned_solver_shell_from_fp64_matrix():
    """Shells have no FP32 element kernels: the learned solver runs on an FP32 copy of the FP64
    matrix, refined against the FP64 matrix, with a 6x6-block network."""
    g, o, A, bo = _system(_shell())
    b = g.static_rhs()
    p = precond_init(16, 1000.0, 6)
    u, st = g.solve_static(b, method=SOLVER_FGMRES_LEARNED, rtol=1e-10, precond=p)
    # Jacobi-GMRES(50) stalls on this shell (drilling DOF) before 1e-10: allowed to stop at its cap
    um, sm = g.solve_static(b, method=SOLVER_FGMRES_MIXED, rtol=1e-10, max_iters=20000, allow_maxit=True)
    ur = spla.spsolve(A.tocsc(), bo)
    assert st.status == 0 and st.fallback == 0 and st.rel_residual <= 1e-10
    assert np.linalg.norm(A @ u - bo) <= 1e-9 * np.linalg.norm(bo)
    assert np.linalg.norm(u - ur) <= 1e-6 * np.linalg.norm(ur)
    assert st.iterations < sm.iterations


def test_learned_newmark_matches_fp64_newmark():
    import newmark_ref as NR  # noqa: F401  (the FP64 run is the reference here)
    m = M.plate_shell(nx=8, ny=6, lx=1.0, ly=0.75, t=0.01, E=7e10, nu=0.33, rho=2700.0, pressure=0.0, clamp="ss",
                      y0=0.0)
    g = AstroGPU(m)
    pattern = np.zeros(g.n)
    pattern[g.n_dof_index[(3 * 9 + 4), 2] - 1] = 1.0
    dt, steps = 1e-5, 8
    amp = 100.0 * np.sin(2 * np.pi * 500.0 * dt * np.arange(1, steps + 1))
    _, _, _, _, h64, s64 = g.newmark_run(steps, dt, 0.25, 0.5, pattern, amp, rtol=1e-12)
    _, _, _, _, hl, sl = g.newmark_run(steps, dt, 0.25, 0.5, pattern, amp, rtol=1e-12, method=SOLVER_FGMRES_LEARNED,
                                       precond=precond_init(16, 1000.0, 6))
    assert s64.status == 0 and sl.status == 0
    for k in range(steps):
        assert np.linalg.norm(hl[k] - h64[k]) <= 1e-7 * np.linalg.norm(h64[k]), k
