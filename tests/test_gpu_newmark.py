"""GPU Newmark time stepping (the dynamic branch of solve with stepSolve) against a time loop
built from the oracle: residual with the Newmark inertia, applied point load F(t), constraint
load, static condensation, direct solve of K_eff, internal-DOF recovery and the Newmark update.
Displacement history to 1e-8 relative per step (GMRES to 1e-12 against a direct solve)."""
import numpy as np
import pytest
import scipy.sparse.linalg as spla

from misc_gb300 import model as M
from misc_gb300.astro import AstroGPU
from oracle import Oracle

pytestmark = pytest.mark.gpu


def _oracle_newmark(o, pattern, amp, dt, beta, gamma, steps):
    n, ni = o.n, o.int_vec_size
    c1, c2 = 0.5 / beta, 2.0 / (dt * dt)
    u, up, vp, ap = (np.zeros(n) for _ in range(4))
    iu, iup = np.zeros(ni), np.zeros(ni)

    def state():
        return M.make_state(n, disp=u, prev_disp=up, prev_vel=vp, prev_acc=ap, internal_disp=iu, prev_int_disp=iup,
                            dynamic=1, beta=beta, gamma=gamma, del_t=dt)

    _, _, mat, cols, imat = o.el_soln_load(1, state=state())
    mm, mr = o.scale_mpc(mat)
    Cm = o.mpc_scipy(mm)
    lu = spla.splu((o.csr_scipy(mat, cols) + Cm.T @ Cm).tocsc())
    hist = []
    for k in range(steps):
        load, iload, *_ = o.el_soln_load(0, state=state())
        load = load + amp[k] * pattern
        o.constraint_load(mm, mr, u, load)
        rhs = o.update_external_rhs(load, iload[:ni], imat)
        du = lu.solve(rhs)
        iu = o.update_internal_soln(du, iu, iload[:ni], imat)
        u = u + du
        acc = c1 * (c2 * (u - up - dt * vp) - (1.0 - 2.0 * beta) * ap)
        vel = vp + dt * ((1.0 - gamma) * ap + gamma * acc)
        up, vp, ap, iup = u.copy(), vel, acc, iu.copy()
        hist.append(u.copy())
    return np.array(hist), vp, ap


def test_newmark_matches_oracle_loop():
    m = M.plate_shell(nx=6, ny=4, lx=1.0, ly=0.5, t=0.01, E=7e10, nu=0.33, rho=2700.0, pressure=0.0)
    o, g = Oracle(m), AstroGPU(m)
    corner = m.num_nodes   # free corner (x = lx)
    pattern = np.zeros(o.n)
    pattern[o.n_dof_index[corner - 1, 2] - 1] = 1.0
    dt, beta, gamma, steps = 1e-4, 0.25, 0.5, 6
    amp = 100.0 * np.sin(2 * np.pi * 500.0 * dt * np.arange(1, steps + 1))
    hist_o, v_o, a_o = _oracle_newmark(o, pattern, amp, dt, beta, gamma, steps)
    u, v, a, iu, hist, st = g.newmark_run(steps, dt, beta, gamma, pattern, amp, rtol=1e-13)
    assert st.status == 0
    for k in range(steps):
        assert np.linalg.norm(hist[k] - hist_o[k]) <= 1e-8 * np.linalg.norm(hist_o[k]), k
    assert np.linalg.norm(v - v_o) <= 1e-7 * np.linalg.norm(v_o)
    assert np.linalg.norm(a - a_o) <= 1e-6 * np.linalg.norm(a_o)
