"""GPU parity of the batched linear Newmark (astro_newmark_cases: K_eff + C^T C factored once by
the band LDL^T, every load case solved per step by the cluster band solve, the step launched as a
CUDA graph) against the oracle, through the C ABI.

* Against the oracle's batched linear loop (the same equations with the oracle's assembled K,
  K_eff and constraints and a sparse direct solve): 1e-9 relative per step and case.  The
  many-column solve runs in double-float (about 48 bits), so each step's solve is within about
  1e-12 of the FP64 direct one; the bound leaves room for the steps' accumulation.
* Against the oracle's element-residual loop (the reference's stepSolve with K_eff factored once):
  the linear loop differs by the geometric nonlinearity of the motion, 1e-6 for the small loads
  here (shell with the consistent tangent, brick8).
* Graph and direct launches give identical results; the last step's solve residual is reported.
"""
import numpy as np
import pytest

from misc_gb300 import model as M
from misc_gb300.astro import OPT_SHELL_MEAN_ROT_TERM, AstroGPU
from oracle import Oracle
from oracle import oracle as OO

pytestmark = pytest.mark.gpu


_QUIRK = [0]  # the oracle's shell-tangent switch as this module last set it


def _quirk(v):
    import ctypes
    L = OO._lib()
    L.orc_set_quirk.argtypes = [ctypes.c_int, ctypes.c_int]
    L.orc_set_quirk(1, v)
    _QUIRK[0] = v


def _cases(o, nodes_dofs, steps, dt, seed):
    """One pattern per (node, dof) pair, a seeded random amplitude history each."""
    rng = np.random.default_rng(seed)
    P = np.zeros((len(nodes_dofs), o.n))
    for c, (nd, d) in enumerate(nodes_dofs):
        P[c, o.n_dof_index[nd - 1, d] - 1] = 1.0
    t = dt * np.arange(1, steps + 1)
    A = np.array([rng.uniform(0.5, 1.5) * np.sin(2 * np.pi * rng.uniform(200, 800) * t + rng.uniform(0, 1))
                  for _ in range(len(nodes_dofs))])
    return P, A


def _check(H, Ho, tol):
    for k in range(H.shape[0]):
        for c in range(H.shape[1]):
            assert np.linalg.norm(H[k, c] - Ho[k, c]) <= tol * np.linalg.norm(Ho[k, c]), (k, c)


def test_brick_cases_match_oracle_linear_loop():
    from newmark_cases_ref import newmark_cases
    m = M.hex_block(6, 2, 2, lx=3.0, ly=0.5, lz=0.5, seed=6, jitter=0.1, sigma=0.3)
    o, g = Oracle(m), AstroGPU(m)
    tip = [a + 1 for a in range(m.num_nodes) if abs(m.node_list[a, 0] - 3.0) < 1e-9]
    P, A = _cases(o, [(tip[0], 2), (tip[-1], 1), (tip[1], 0)], 8, 2e-5, 3)
    A *= 1e5
    u, v, a, H, info = g.newmark_cases(2e-5, P, A, history=True)
    Ho, Uo, Vo, Ao = newmark_cases(o, P, A, 2e-5, 0.25, 0.5, 8)
    _check(H, Ho, 1e-9)
    assert np.linalg.norm(v - Vo) <= 1e-8 * np.linalg.norm(Vo)
    assert np.linalg.norm(a - Ao) <= 1e-8 * np.linalg.norm(Ao)
    assert info.last_rel_residual < 1e-10 and info.panels == 1 and info.kernels_per_step == 6


def test_brick_cases_near_element_loop():
    """The linear loop against the reference's loop (element residual at every state) for one
    case: the difference is the geometric nonlinearity of the small motion."""
    from newmark_ref import newmark_states
    m = M.hex_block(6, 2, 2, lx=3.0, ly=0.5, lz=0.5, seed=6, jitter=0.1, sigma=0.3)
    o, g = Oracle(m), AstroGPU(m)
    tip = [a for a in range(m.num_nodes) if abs(m.node_list[a, 0] - 3.0) < 1e-9]
    pattern = np.zeros(o.n)
    for a in tip:
        pattern[o.n_dof_index[a, 2] - 1] = 1.0 / len(tip)
    dt, steps = 2e-5, 5
    amp = 1e3 * np.sin(2 * np.pi * 2000.0 * dt * np.arange(1, steps + 1))
    D, V, A, I = newmark_states(o, pattern, amp, dt, 0.25, 0.5, steps)
    u, v, a, H, info = g.newmark_cases(dt, pattern[None], amp[None], history=True)
    for k in range(steps):
        assert np.linalg.norm(H[k, 0] - D[k + 1]) <= 1e-6 * np.linalg.norm(D[k + 1]), k


@pytest.fixture(scope="module")
def shell():
    _quirk(1)
    try:
        nx = 8
        m = M.plate_shell(nx=nx, ny=nx, lx=1.0, ly=1.0, t=0.01, E=7e10, nu=0.33, rho=2700.0, pressure=0.0,
                          clamp="ss", y0=0.0)
        o = Oracle(m)
        yield nx, m, o
    finally:
        _quirk(0)


def test_shell_cases_match_oracle_linear_loop(shell):
    """Simply supported plate (constraints, eight condensed internal DOF per element), three
    point-load cases, graph and direct launches."""
    from newmark_cases_ref import newmark_cases
    nx, m, o = shell
    _quirk(1)
    g = AstroGPU(m)
    g.set_option(OPT_SHELL_MEAN_ROT_TERM, 1)
    centre = (nx // 2) * (nx + 1) + nx // 2 + 1
    P, A = _cases(o, [(centre, 2), (centre + 2, 2), (centre - nx, 0)], 10, 1e-5, 5)
    A *= 100.0
    u, v, a, H, info = g.newmark_cases(1e-5, P, A, history=True)
    u2, v2, a2, H2, _ = g.newmark_cases(1e-5, P, A, history=True, graph=False)
    assert np.array_equal(H, H2) and np.array_equal(v, v2)
    Ho, Uo, Vo, Ao = newmark_cases(o, P, A, 1e-5, 0.25, 0.5, 10)
    _check(H, Ho, 1e-9)
    assert info.last_rel_residual < 1e-10 and info.graph_nodes >= 6


def test_twisted_solve_matches_oracle(shell):
    """The twisted many-column solve (top and reversed bottom halves meeting in a window, forced
    on this small plate) and the plain one against the oracle's batched loop, 1e-9 each."""
    from misc_gb300.astro import OPT_CASES_TWIST
    from newmark_cases_ref import newmark_cases
    nx, m, o = shell
    _quirk(1)
    centre = (nx // 2) * (nx + 1) + nx // 2 + 1
    P, A = _cases(o, [(centre, 2), (centre + 2, 2), (centre - nx, 0)], 10, 1e-5, 5)
    A *= 100.0
    Ho, *_ = newmark_cases(o, P, A, 1e-5, 0.25, 0.5, 10)
    for twist, kernels in ((2, 10), (0, 6)):
        g = AstroGPU(m)
        g.set_option(OPT_SHELL_MEAN_ROT_TERM, 1)
        g.set_option(OPT_CASES_TWIST, twist)
        u, v, a, H, info = g.newmark_cases(1e-5, P, A, history=True)
        _check(H, Ho, 1e-9)
        assert info.kernels_per_step == kernels and info.last_rel_residual < 1e-10, twist


def test_shell_cases_near_element_loop(shell):
    """The centre-load case against the reference's loop with the consistent shell tangent."""
    from newmark_ref import newmark_states
    nx, m, o = shell
    _quirk(1)
    g = AstroGPU(m)
    g.set_option(OPT_SHELL_MEAN_ROT_TERM, 1)
    centre = (nx // 2) * (nx + 1) + nx // 2 + 1
    pattern = np.zeros(o.n)
    pattern[o.n_dof_index[centre - 1, 2] - 1] = 1.0
    dt, steps = 1e-5, 6
    amp = 100.0 * np.sin(2 * np.pi * 500.0 * dt * np.arange(1, steps + 1))
    D, V, A, I = newmark_states(o, pattern, amp, dt, 0.25, 0.5, steps)
    u, v, a, H, info = g.newmark_cases(dt, pattern[None], amp[None], history=True)
    for k in range(steps):
        assert np.linalg.norm(H[k, 0] - D[k + 1]) <= 1e-6 * np.linalg.norm(D[k + 1]), k


def test_cases_over_several_panels():
    """Two disconnected clamped panels (two band factors, one cluster per panel and case), with
    and without an FP64 refinement pass; the oracle and the device use the same (default) shell
    tangent."""
    from newmark_cases_ref import newmark_cases
    prev = _QUIRK[0]
    _quirk(0)
    try:
        m = M.panel_batch(num_panels=8, indices=[0, 3], n_range=(4, 9), n_dvars=0)
        o, g = Oracle(m), AstroGPU(m)
        last = m.num_nodes
        P, A = _cases(o, [(last, 2), (last // 3, 2)], 6, 1e-5, 8)
        A *= 50.0
        Ho, *_ = newmark_cases(o, P, A, 1e-5, 0.25, 0.5, 6)
        u, v, a, H, info = g.newmark_cases(1e-5, P, A, history=True)
        assert info.panels == 2 and info.kernels_per_step == 6
        _check(H, Ho, 1e-9)
        u, v, a, H, info = g.newmark_cases(1e-5, P, A, history=True, refine=1)
        _check(H, Ho, 1e-9)
        assert info.kernels_per_step == 11
    finally:
        _quirk(prev)


def test_cfg5_plate_seventeen_cases():
    """The 128x128 plate (99,846 DOF) with the centre force and 16 seeded random point loads,
    five steps against the oracle's batched linear loop (sparse direct solve)."""
    from newmark_cases_ref import newmark_cases
    _quirk(1)
    try:
        nx = 128
        m = M.plate_shell(nx=nx, ny=nx, lx=1.0, ly=1.0, t=0.01, E=7e10, nu=0.33, rho=2700.0, pressure=0.0,
                          clamp="ss", y0=0.0)
        o, g = Oracle(m), AstroGPU(m)
        g.set_option(OPT_SHELL_MEAN_ROT_TERM, 1)
        P, A = M.config5_cases(m, g.n_dof_index, 5, 1e-5)
        u, v, a, H, info = g.newmark_cases(1e-5, P, A, history=True)
        Ho, *_ = newmark_cases(o, P, A, 1e-5, 0.25, 0.5, 5)
        _check(H, Ho, 1e-9)
        assert info.last_rel_residual < 1e-10
    finally:
        _quirk(0)
