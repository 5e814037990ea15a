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


# ---- per-node modulation (astro_precond_mlp) ------------------------------------------------

def node_adjacency(model):
    """Per node (0-based) the set of other nodes sharing an element with it."""
    adj = [set() for _ in range(model.num_nodes)]
    for row in np.asarray(model.element_list):
        nds = [int(x) - 1 for x in row if x > 0]
        for a in nds:
            adj[a].update(b for b in nds if b != a)
    return adj


def node_features(K, CtC, idx, adj):
    """The six features of every node from K (global numbering, without the penalty) and the
    penalty C^T C: l = ln(mean diagonal of the node's block), f0 = l - mean(l), f1 = mean over
    neighbours of (l_c - l_r), f2 = max |l_c - l_r|, f3 = (neighbours + 1) / most blocks of a row,
    f4 = ln(1 + mean penalty diagonal / d), f5 = ln(sum ||K_rc||_F / ||K_rr||_F)."""
    K = K.tocsr()
    N = idx.shape[0]
    kd = K.diagonal()
    pdg = CtC.diagonal()
    d = np.array([kd[idx[r]].mean() for r in range(N)])
    p = np.array([pdg[idx[r]].mean() for r in range(N)])
    L = np.log(np.abs(d))
    maxB = max(len(a) + 1 for a in adj)
    F = np.zeros((N, 6))
    for r in range(N):
        nb = sorted(adj[r])
        dl = L[nb] - L[r] if nb else np.zeros(0)
        rows = K[idx[r]]
        dia = np.linalg.norm(rows[:, idx[r]].toarray())
        off = sum(np.linalg.norm(rows[:, idx[c]].toarray()) for c in nb)
        F[r] = [L[r] - L.mean(), dl.mean() if nb else 0.0, np.abs(dl).max() if nb else 0.0, (len(nb) + 1) / maxB,
                np.log1p(p[r] / d[r]), np.log(off / dia) if off > 0 and dia > 0 else 0.0]
    return F


def mlp_forward(F, w1, b1, w2, b2):
    """(hidden activations (N, H), scales a (N, K)) of the perceptron."""
    h = np.tanh(F @ w1.T + b1)
    return h, 1.0 + h @ w2.T + b2


def loss_grad_mod(A, dinv, lam, ratio, W, samples, idx, F, w1, b1, w2, b2):
    """Loss of the modulated network P v = (1/lam) sum_k a_k (W_k y_k) per node, its gradient
    with respect to W and the perceptron's parameters (A symmetric)."""
    h, a = mlp_forward(F, w1, b1, w2, b2)
    L = 0.0
    GW = np.zeros_like(W)
    Ga = np.zeros_like(a)
    S = len(samples)
    for v in samples:
        v = v / np.linalg.norm(v)
        ys = features(A, dinv, lam, ratio, len(W) - 1, v)
        z = np.zeros_like(v)
        for k, y in enumerate(ys):
            m = np.zeros_like(v)
            m[idx] = (y[idx] @ W[k].T) * a[:, k:k + 1]
            z += m
        z /= lam
        e = v - A @ z
        L += e @ e
        T = (A @ e)[idx]
        for k, y in enumerate(ys):
            Y = y[idx]
            GW[k] += -2.0 / (S * lam) * ((T * a[:, k:k + 1]).T @ Y)
            Ga[:, k] += -2.0 / (S * lam) * np.sum(T * (Y @ W[k].T), axis=1)
    gw2 = Ga.T @ h
    gb2 = Ga.sum(0)
    gpre = (Ga @ w2) * (1.0 - h * h)
    gw1 = gpre.T @ F
    gb1 = gpre.sum(0)
    return L / S, GW, (gw1, gb1, gw2, gb2)
