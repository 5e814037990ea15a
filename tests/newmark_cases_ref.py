"""Batched linear Newmark built from the oracle (test infrastructure): the dynamic branch of
solve with linear geometry (Working/AStrO_commandFunctions.f90:770-812: getElasticSolnLoad(1)
with the dynamic flag, scaleElasticMPC, getSparseLDLFact of K_eff once, then stepSolve and the
Newmark update per step) for several load cases at once, with the residual of the linear element
equations written through the assembled matrices: K (static, zero state) and K_eff = K + c1 c2 M
(dynamic, zero state), both condensed over the internal DOF,

    r = amp_k p + C^T rhs - K (u - w) - K_eff w - C^T C u,   w = -(dt v + (1 - 2 beta) a / c2),

that is r = f - K u - M a_pred - C^T (C u - rhs) with a_pred = c1 c2 w the acceleration at the
start of the step; du = (K_eff + C^T C)^-1 r, then the reference's acceleration and velocity
update.  Returns the displacement history (steps x cases x n) and the final u, v, a."""
import numpy as np
import scipy.sparse.linalg as spla

from misc_gb300 import model as M


def linear_matrices(o, dt, beta, gamma):
    n = o.n
    _, _, mat0, cols, _ = o.el_soln_load(1, state=M.make_state(n))
    _, _, mat1, cols1, _ = o.el_soln_load(1, state=M.make_state(n, dynamic=1, beta=beta, gamma=gamma, del_t=dt))
    assert np.array_equal(cols, cols1)
    mm, mr = o.scale_mpc(mat1)
    Cm = o.mpc_scipy(mm)
    g = np.zeros(n)
    o.constraint_load(mm, mr, np.zeros(n), g)
    K, Keff = o.csr_scipy(mat0, cols), o.csr_scipy(mat1, cols)
    return K, Keff, (Cm.T @ Cm).tocsr(), g


def newmark_cases(o, patterns, amps, dt, beta, gamma, steps, u0=None, v0=None, a0=None):
    nc, n = patterns.shape
    c2 = 2.0 / (dt * dt)
    c1 = 0.5 / beta
    K, Keff, CtC, g = linear_matrices(o, dt, beta, gamma)
    lu = spla.splu((Keff + CtC).tocsc())
    U = np.zeros((nc, n)) if u0 is None else u0.copy()
    V = np.zeros((nc, n)) if v0 is None else v0.copy()
    A = np.zeros((nc, n)) if a0 is None else a0.copy()
    H = np.zeros((steps, nc, n))
    for k in range(steps):
        for c in range(nc):
            w = -(dt * V[c] + (1.0 - 2.0 * beta) * A[c] / c2)
            r = amps[c, k] * patterns[c] + g - K @ (U[c] - w) - Keff @ w - CtC @ U[c]
            du = lu.solve(r)
            an = c1 * (c2 * (du - dt * V[c]) - (1.0 - 2.0 * beta) * A[c])
            V[c] = V[c] + dt * ((1.0 - gamma) * A[c] + gamma * an)
            A[c] = an
            U[c] = U[c] + du
            H[k, c] = U[c]
    return H, U, V, A
