"""Forward Newmark time loop built from the oracle (test infrastructure): the dynamic branch of
solve with stepSolve for linear geometry (K_eff factored once at the initial state, the residual
with the Newmark inertia at each state, applied load amp[k] * pattern, constraint load,
condensation, direct solve, internal-DOF recovery, Newmark update).  Returns the stored states of
every step, rows 0..N (the records of SolutionHistory<i>)."""
import numpy as np
import scipy.sparse.linalg as spla

from misc_gb300 import model as M


def newmark_states(o, pattern, amp, dt, beta, gamma, steps):
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
    D, V, A, I = [u.copy()], [vp.copy()], [ap.copy()], [iu.copy()]
    for k in range(steps):
        load, iload, *_ = o.el_soln_load(0, state=state())
        load = load + amp[k] * pattern
        o.constraint_load(mm, mr, u, load)
        rhs = o.update_external_rhs(load, iload[:ni], imat)
        du = lu.solve(rhs)
        iu = o.update_internal_soln(du, iu, iload[:ni], imat)[:ni]
        u = u + du
        acc = c1 * (c2 * (u - up - dt * vp) - (1.0 - 2.0 * beta) * ap)
        vel = vp + dt * ((1.0 - gamma) * ap + gamma * acc)
        up, vp, ap, iup = u.copy(), vel, acc, iu.copy()
        D.append(u.copy())
        V.append(vel.copy())
        A.append(acc.copy())
        I.append(iu.copy())
    return np.array(D), np.array(V), np.array(A), np.array(I)
