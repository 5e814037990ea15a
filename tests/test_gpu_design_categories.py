"""GPU parity of the design-variable categories against the oracle, through the C ABI.

* The complex step of the element residual (getdRelasticdD's element part) for every category the
  device evaluates: solid density, orientation and node coordinates (brick8 and brickIM, the
  complex element kernel) and shell layup zOffset, layer angle, layer density and the layer's
  elastic constants (the complex section properties), at displaced (and, where density enters,
  dynamic) states: 1e-10 relative.
* Models carrying nonzero real values of those variables: element matrices 1e-12 relative.
* nodeLoad variables: the applied nodal design load and its derivative, exact.
* The complex step of shell orientation / node-coordinate variables is refused
  (ASTRO_ERR_UNSUPPORTED): those enter the shell kinematics, which run in real arithmetic.
"""
import numpy as np
import pytest

from misc_gb300 import model as M
from misc_gb300.astro import AstroError, AstroGPU
from oracle import Oracle
from test_oracle_kat import _CAT_CASES, _brick, _layered_plate

pytestmark = pytest.mark.gpu


def _state(o, dyn, seed=7):
    rng = np.random.default_rng(seed)
    n, ni = o.n, max(o.int_vec_size, 1)
    kw = {}
    if dyn:
        kw = dict(prev_disp=1e-3 * rng.standard_normal(n), prev_vel=1e-1 * rng.standard_normal(n),
                  prev_acc=10.0 * rng.standard_normal(n), prev_int_disp=1e-4 * rng.standard_normal(ni),
                  dynamic=1, beta=0.25, gamma=0.5, del_t=1e-3)
    return M.make_state(n, disp=1e-3 * rng.standard_normal(n), internal_disp=1e-4 * rng.standard_normal(ni), **kw)


@pytest.mark.parametrize("case", sorted(_CAT_CASES))
def test_complex_step_matches_oracle(case):
    build, _, dyn = _CAT_CASES[case]
    m = build()
    g, o = AstroGPU(m), Oracle(m)
    st = _state(o, dyn)
    for dvar in (1, 2):
        dr, idr = g.getdRelasticdD(dvar, h=1e-30, state=st)
        odr, oidr = o.drdd_complex(dvar, h=1e-30, state=st)
        assert np.linalg.norm(odr) > 0
        assert np.linalg.norm(dr - odr) <= 1e-10 * np.linalg.norm(odr), (case, dvar)
        if o.int_vec_size and np.linalg.norm(oidr) > 0:
            assert np.linalg.norm(idr - oidr) <= 1e-10 * np.linalg.norm(oidr), (case, dvar)


def _rel(a, b):
    return np.linalg.norm(a - b, axis=(1, 2)) / np.linalg.norm(b, axis=(1, 2))


@pytest.mark.parametrize("case", ["brick_orientation", "brickIM_node_coord", "brick_density", "shell_zoffset",
                                  "shell_layup_angle", "shell_layup_density", "shell_layup_modulus",
                                  "shell_layup_poisson"])
def test_real_design_values_enter_the_element(case):
    """Nonzero design values: rotated frames, moved nodes, changed density / offset / layer angle,
    layer density and layer elastic constants, element matrices (with the Newmark mass where
    density enters)."""
    build, _, dyn = _CAT_CASES[case]
    m = build()
    scale = {"brick_orientation": 0.3, "brickIM_node_coord": 0.02, "brick_density": 500.0, "shell_zoffset": 0.4,
             "shell_layup_angle": 0.5, "shell_layup_density": 900.0, "shell_layup_modulus": 2.0e10,
             "shell_layup_poisson": 0.05}[case]
    m.d_value = np.array([scale, -0.5 * scale])
    g, o = AstroGPU(m), Oracle(m)
    st = _state(o, dyn, seed=3)
    ke, ru = g.element_matrices(64, state=st, with_residual=True)
    assert _rel(ke, o.element_matrices(state=st)).max() < 1e-11, case
    for el in range(1, m.num_els + 1):
        r_o, _ = o.element(el, 1, st)
        assert np.linalg.norm(ru[el - 1] - r_o[:24]) <= 1e-11 * np.linalg.norm(r_o[:24]), (case, el)


def test_node_load_variables():
    m = M.add_node_design_variables(M.hex_block(nx=3, ny=2, nz=2, seed=3), [[5, 9], [12]], M.DCAT_NODE_LOAD,
                                    component=2, value=3.0, act_time=(0.5, 2.0))
    g, o = AstroGPU(m), Oracle(m)
    for t in (0.2, 1.0, 3.0):
        assert np.array_equal(g.design_node_load(t), o.design_node_load(t)), t
        for d in (1, 2):
            assert np.array_equal(g.node_load_drdd(d, t), o.node_load_drdd(d, t)), (t, d)


def test_shell_kinematic_categories_are_refused():
    for cat, comp in ((M.DCAT_ORIENTATION, 3), (M.DCAT_NODE_COORD, 1)):
        m = M.plate_shell(nx=3, ny=2, lx=1.0, ly=0.5, t=0.02)
        if cat == M.DCAT_NODE_COORD:
            M.add_node_design_variables(m, [[2, 3]], cat, component=comp)
        else:
            M.add_design_variables(m, 1, cat, component=comp)
        g = AstroGPU(m)
        with pytest.raises(AstroError) as e:
            g.getdRelasticdD(1)
        assert e.value.code == 3
