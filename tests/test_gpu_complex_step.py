"""GPU parity of the complex-step residual sensitivity (getdRelasticdD element part) against the
oracle's complex twin, through the C ABI: dRu/dd in global DOF and at the shell internal DOF,
1e-10 relative (norm), for layer-thickness design variables of shells (static and Newmark
states) and elastic-modulus design variables of bricks."""
import numpy as np
import pytest

from misc_gb300 import model as M
from misc_gb300.astro import AstroError, AstroGPU
from oracle import Oracle

pytestmark = pytest.mark.gpu

TOL = 1e-10


def _shell():
    m = M.plate_shell(nx=6, ny=4, lx=2.0, ly=1.0, t=0.03, E=7e10, nu=0.33)
    rng = np.random.default_rng(5)
    X = m.node_list.copy()
    X[:, :2] += 0.05 * rng.uniform(-1, 1, (len(X), 2))
    X[:, 2] += 0.02 * rng.uniform(-1, 1, len(X))
    m.node_list = X
    return M.add_design_variables(m, 4, M.DCAT_LAYUP_THICKNESS)


def _brick():
    m = M.hex_block(nx=5, ny=3, nz=3, jitter=0.1, seed=4)
    return M.add_design_variables(m, 3, M.DCAT_ELASTIC_MODULUS, component=1)


def _state(o, dynamic=False):
    rng = np.random.default_rng(9)
    n, ni = o.n, max(o.int_vec_size, 1)
    kw = dict(disp=1e-3 * rng.standard_normal(n), internal_disp=1e-4 * rng.standard_normal(ni))
    if dynamic:
        kw.update(prev_disp=1e-3 * rng.standard_normal(n), prev_vel=1e-1 * rng.standard_normal(n),
                  prev_acc=10.0 * rng.standard_normal(n), dynamic=1, beta=0.25, gamma=0.5, del_t=1e-3)
    return M.make_state(n, **kw)


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("case", ["shell_static", "shell_newmark", "brick"])
def test_drdd_matches_oracle(case):
    m = _brick() if case == "brick" else _shell()
    o, g = Oracle(m), AstroGPU(m)
    st = _state(o, dynamic=(case == "shell_newmark"))
    for dvar in range(1, len(m.d_value) + 1):
        d, di = g.getdRelasticdD(dvar, 1e-14, state=st)
        do, dio = o.drdd_complex(dvar, 1e-14, state=st)
        assert np.linalg.norm(do) > 0
        assert _rel(d, do) < TOL, dvar
        if o.int_vec_size:
            assert _rel(di, dio) < TOL, dvar


def test_drdd_tiny_step_and_zero_state():
    """h = 1e-30 gives the same derivative as the reference's 1e-14 (the complex step has no
    subtractive cancellation); at the zero state the residual, and so its sensitivity, vanishes
    up to rounding."""
    m = _shell()
    o, g = Oracle(m), AstroGPU(m)
    st = _state(o)
    d14, _ = g.getdRelasticdD(2, 1e-14, state=st)
    d30, _ = g.getdRelasticdD(2, 1e-30, state=st)
    assert _rel(d30, d14) < 1e-9
    z, zi = g.getdRelasticdD(2, 1e-14)
    assert np.abs(z).max() <= 1e-8 * np.abs(d14).max()


def test_drdd_bad_design_variable():
    g = AstroGPU(_brick())
    with pytest.raises(AstroError):
        g.getdRelasticdD(99, 1e-14)
