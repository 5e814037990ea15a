"""Host side of the polynomial preconditioner (no GPU): the C initialisation against the numpy
least-squares Chebyshev fit, argument checks, and the numpy restatement's gradient against
central differences of its loss (the restatement checks the device kernels in the GPU tests)."""
import numpy as np

from misc_gb300 import model as M
from misc_gb300.astro import AstroError, precond_init
from oracle import Oracle
import poly_ref as R


def test_init_is_chebyshev_fit():
    for deg, ratio, dpn in ((8, 100.0, 3), (3, 10.0, 6), (16, 1000.0, 3)):
        p = precond_init(deg, ratio, dpn)
        c = R.cheb_init(deg, ratio)
        W = p.weight_array()
        assert W.shape == (deg + 1, dpn, dpn)
        assert np.allclose(W, c[:, None, None] * np.eye(dpn)[None], rtol=1e-8, atol=1e-9 * np.abs(c).max())
        assert p.lambda_scale == 1.05 and p.ratio == ratio


def test_init_rejects_bad_arguments():
    for args in ((0, 100.0, 3), (33, 100.0, 3), (8, 1.0, 3), (8, 100.0, 4)):
        try:
            precond_init(*args)
        except AstroError:
            continue
        raise AssertionError(args)


def test_init_polynomial_maps_spectrum_near_one():
    """nu p(nu) stays within the fit's band on the interval: the preconditioned spectrum is
    clustered around 1 and positive (no indefinite preconditioner)."""
    p = precond_init(8, 100.0, 3)
    c = p.weight_array()[:, 0, 0]
    nu = np.linspace(1 / 100, 1.0, 2001)
    x = (2 * nu - (1 + 1 / 100)) / (1 - 1 / 100)
    q = nu * np.polynomial.chebyshev.chebval(x, c)
    assert q.min() > 0.0 and q.max() < 2.0


def test_reference_gradient_central_difference():
    m = M.hex_block(nx=3, ny=2, nz=2, jitter=0.1, seed=0)
    o = Oracle(m)
    A, *_ = o.static_system()
    A = A.tocsr()
    dinv = 1.0 / A.diagonal()
    rng = np.random.default_rng(0)
    W = rng.standard_normal((4, 3, 3))
    S = rng.standard_normal((2, A.shape[0]))
    idx = R.node_index(o, 3)
    L, G = R.loss_grad(A, dinv, 3.0, 20.0, W, S, idx)
    D = rng.standard_normal(W.shape)
    h = 1e-5
    Lp, _ = R.loss_grad(A, dinv, 3.0, 20.0, W + h * D, S, idx)
    Lm, _ = R.loss_grad(A, dinv, 3.0, 20.0, W - h * D, S, idx)
    assert abs((Lp - Lm) / (2 * h) - np.sum(G * D)) <= 1e-6 * abs(np.sum(G * D))


def test_reference_modulated_gradient_central_difference():
    """The restatement of the per-node modulation: its gradients with respect to the hop weights
    and to every perceptron parameter against central differences of its loss."""
    m = M.hex_block(nx=3, ny=2, nz=2, jitter=0.1, seed=0, sigma=0.6)
    o = Oracle(m)
    A, *_ = o.static_system()
    A = A.tocsr()
    dinv = 1.0 / A.diagonal()
    rng = np.random.default_rng(1)
    W = rng.standard_normal((4, 3, 3))
    S = rng.standard_normal((2, A.shape[0]))
    idx = R.node_index(o, 3)
    F = rng.standard_normal((m.num_nodes, 6))
    prm = [0.5 * rng.standard_normal((5, 6)), 0.2 * rng.standard_normal(5), 0.3 * rng.standard_normal((4, 5)),
           0.1 * rng.standard_normal(4)]
    L, GW, GM = R.loss_grad_mod(A, dinv, 3.0, 20.0, W, S, idx, F, *prm)
    h = 1e-6
    D = rng.standard_normal(W.shape)
    Lp = R.loss_grad_mod(A, dinv, 3.0, 20.0, W + h * D, S, idx, F, *prm)[0]
    Lm = R.loss_grad_mod(A, dinv, 3.0, 20.0, W - h * D, S, idx, F, *prm)[0]
    assert abs((Lp - Lm) / (2 * h) - np.sum(GW * D)) <= 1e-6 * abs(np.sum(GW * D))
    for q in range(4):
        Dq = rng.standard_normal(prm[q].shape)
        pp = [x.copy() for x in prm]
        pm = [x.copy() for x in prm]
        pp[q] = pp[q] + h * Dq
        pm[q] = pm[q] - h * Dq
        fd = (R.loss_grad_mod(A, dinv, 3.0, 20.0, W, S, idx, F, *pp)[0] -
              R.loss_grad_mod(A, dinv, 3.0, 20.0, W, S, idx, F, *pm)[0]) / (2 * h)
        an = np.sum(GM[q] * Dq)
        assert abs(fd - an) <= 1e-5 * abs(an), (q, fd, an)
    # with a zero output layer the modulated loss is the plain network's
    z = [prm[0], prm[1], np.zeros((4, 5)), np.zeros(4)]
    assert abs(R.loss_grad_mod(A, dinv, 3.0, 20.0, W, S, idx, F, *z)[0] -
               R.loss_grad(A, dinv, 3.0, 20.0, W, S, idx)[0]) <= 1e-13 * L
