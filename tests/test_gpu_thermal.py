"""GPU parity of the thermal path against the oracle through the C ABI: conductivity and
capacitance (rank-ordered thermal load, the reference's CSR values and columns) for bricks with
rotated sections and anisotropic conductivity and for warped shells with rotated layers, static
and transient states; thermal constraints (scaling, constraint load); heat generation; the device
conjugate-gradient solve against a direct solve.  1e-12 relative for element quantities, 1e-10 for
solutions."""
import numpy as np
import pytest
import scipy.sparse.linalg as spla

from misc_gb300 import model as M
from misc_gb300.astro import AstroError, AstroGPU, thermal_props, thermal_state
from oracle import Oracle

pytestmark = pytest.mark.gpu


def _close(a, b, tol):
    assert np.linalg.norm(np.asarray(a) - np.asarray(b)) <= tol * np.linalg.norm(b), np.abs(np.asarray(a) - b).max()


def _materials(nm, seed):
    rng = np.random.default_rng(seed)
    k = rng.uniform(10.0, 60.0, (nm, 3))
    off = rng.uniform(-2.0, 2.0, (nm, 3))
    return np.hstack([k, off]), rng.uniform(400.0, 900.0, nm)


def _rotation(a, b, c):
    ca, sa, cb, sb, cc, sc = np.cos(a), np.sin(a), np.cos(b), np.sin(b), np.cos(c), np.sin(c)
    Rz = np.array([[ca, -sa, 0], [sa, ca, 0], [0, 0, 1]])
    Ry = np.array([[cb, 0, sb], [0, 1, 0], [-sb, 0, cb]])
    Rx = np.array([[1, 0, 0], [0, cc, -sc], [0, sc, cc]])
    return Rz @ Ry @ Rx


def _brick():
    m = M.hex_block(5, 4, 3, lx=1.5, ly=1.0, lz=0.75, seed=2)
    m.section_orient = np.broadcast_to(_rotation(0.3, -0.2, 0.5), m.section_orient.shape).copy()
    return m


def _shell():
    m = M.plate_shell(nx=5, ny=4, lx=2.0, ly=1.0, t=0.03)
    rng = np.random.default_rng(5)
    X = m.node_list.copy()
    X[:, :2] += 0.05 * rng.uniform(-1, 1, (len(X), 2))
    X[:, 2] += 0.02 * rng.uniform(-1, 1, len(X))
    m.node_list = X
    m.layup_angle = np.array([0.3])
    return m


@pytest.fixture(scope="module", params=["brick", "shell"])
def case(request):
    m = _brick() if request.param == "brick" else _shell()
    nm = len(m.material_density)
    cond, sh = _materials(nm, 3)
    X = m.node_list
    nodes = np.nonzero(X[:, 0] <= 1e-9 + X[:, 0].min())[0] + 1
    mpc = (np.arange(len(nodes) + 1), nodes, np.ones(len(nodes)), np.full(len(nodes), 25.0))
    g, o = AstroGPU(m), Oracle(m)
    g.thermal_setup(thermal_props(cond, sh, mpc))
    return m, g, o, cond, sh, mpc


def test_thermal_soln_load_static_and_transient(case):
    m, g, o, cond, sh, mpc = case
    N = m.num_nodes
    rng = np.random.default_rng(7)
    T, pT, pTd = rng.uniform(0, 100, N), rng.uniform(0, 100, N), rng.uniform(-5, 5, N)
    for dyn in (0, 1):
        kw = dict(temp=T, prev_temp=pT, prev_tdot=pTd, dynamic=dyn, gamma=0.6, del_t=0.05)
        lg, mg, cg = g.getThermalSolnLoad(1, state=thermal_state(T, pT, pTd, dyn, 0.6, 0.05))
        lo, mo, co, ro = o.thermal_soln_load(cond, sh, 1, **kw)
        assert np.array_equal(cg, co)
        _close(mg, mo, 1e-12)
        _close(lg, lo, 1e-12)
    assert g.therm_mat_size == len(mo)


def test_thermal_constraints_heat_gen_and_solve(case):
    m, g, o, cond, sh, mpc = case
    N = m.num_nodes
    g.getThermalSolnLoad(1, export=False)
    mm, mr = g.scaleThermalMPC()
    A, b, rows = o.thermal_system(cond, sh, mpc)
    _close(mm, np.concatenate([r[1] for r in rows]), 1e-13)
    _close(mr, [r[2] for r in rows], 1e-13)
    T = np.random.default_rng(3).uniform(0, 50, N)
    _close(g.getThermalConstraintLoad(T), o.thermal_constraint_load(rows, T, np.zeros(N)), 1e-12)
    els = np.array([1, 3, 3, m.num_els])
    _close(g.thermal_heat_gen(7.0, elements=els), o.thermal_heat_gen(7.0, elements=els), 1e-12)
    fe = np.array([1, 2, m.num_els], np.int32)
    fn = np.array([4, 2, 1], np.int32) if m.element_type[0] == 8 else np.array([1, 2, 1], np.int32)
    _close(g.thermal_surface_flux(fe, fn, 3.5), o.thermal_surface_flux(fe, fn, 3.5), 1e-12)
    q = g.thermal_heat_gen(7.0)
    _close(q, o.thermal_heat_gen(7.0), 1e-12)
    rhs = g.getThermalConstraintLoad(None, q.copy())
    x, st = g.thermal_solve(rhs, rtol=1e-12)
    assert st.status == 0
    xr = spla.spsolve(A.tocsc(), rhs)
    _close(x, xr, 1e-9)


def test_thermal_errors():
    m = _brick()
    g = AstroGPU(m)
    with pytest.raises(AstroError):
        g.thermal_setup(thermal_props(np.ones((1, 6)), np.ones(1)))  # fewer materials than the mesh uses
    nm = len(m.material_density)
    cond, sh = _materials(nm, 1)
    g.thermal_setup(thermal_props(cond, sh))
    with pytest.raises(AstroError) as e:
        g.thermal_solve(np.ones(m.num_nodes))
    assert e.value.code == 8
