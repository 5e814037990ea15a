"""numpy restatement of the polynomial graph-convolution preconditioner (test infrastructure).

P v = (1/lam) sum_k W_k y_k,  y_0 = D^-1 v,  y_1 = (D^-1 A y_0 - theta y_0) / delta,
y_{k+1} = 2 (D^-1 A y_k - theta y_k) / delta - y_{k-1},
theta = lam (1 + 1/ratio) / 2, delta = lam (1 - 1/ratio) / 2, W_k a dpn x dpn weight applied to the
DOF of every node.  Vectors are in the global DOF numbering of the oracle (component-major), so
the per-node mixing gathers each node's DOF through n_dof_index.
"""
import numpy as np


def node_index(o, dpn):
    """(num_nodes, dpn) global DOF indices (0-based) of every node's components."""
    return np.asarray(o.n_dof_index)[:, :dpn] - 1


def cheb_init(degree, ratio, nodes=400):
    """c with nu sum_k c_k T_k(x(nu)) ~ 1 on [1/ratio, 1] in the least-squares sense."""
    x = np.cos(np.pi * (np.arange(nodes) + 0.5) / nodes)
    nu = 0.5 * (x + 1.0) * (1.0 - 1.0 / ratio) + 1.0 / ratio
    T = np.polynomial.chebyshev.chebvander(x, degree)
    c, *_ = np.linalg.lstsq(nu[:, None] * T, np.ones(nodes), rcond=None)
    return c


def features(A, dinv, lam, ratio, degree, v):
    theta = 0.5 * lam * (1.0 + 1.0 / ratio)
    delta = 0.5 * lam * (1.0 - 1.0 / ratio)
    ys = [dinv * v]
    for k in range(degree):
        u = dinv * (A @ ys[k]) - theta * ys[k]
        y = (1.0 if k == 0 else 2.0) / delta * u
        if k > 0:
            y = y - ys[k - 1]
        ys.append(y)
    return ys


def mix(W, y, idx):
    """per-node y -> W y (W: dpn x dpn) in global numbering"""
    out = np.zeros_like(y)
    out[idx] = y[idx] @ W.T
    return out


def apply(A, dinv, lam, ratio, W, v, idx):
    ys = features(A, dinv, lam, ratio, len(W) - 1, v)
    return sum(mix(W[k], y, idx) for k, y in enumerate(ys)) / lam


def loss_grad(A, dinv, lam, ratio, W, samples, idx):
    """mean_s ||v_s - A P v_s||^2 over unit samples and its gradient d/dW (A symmetric)."""
    L = 0.0
    G = np.zeros_like(W)
    for v in samples:
        v = v / np.linalg.norm(v)
        ys = features(A, dinv, lam, ratio, len(W) - 1, v)
        z = sum(mix(W[k], y, idx) for k, y in enumerate(ys)) / lam
        e = v - A @ z
        L += e @ e
        t = (A @ e)[idx]
        for k, y in enumerate(ys):
            G[k] += -2.0 / lam * (t.T @ y[idx])
    return L / len(samples), G / len(samples)
