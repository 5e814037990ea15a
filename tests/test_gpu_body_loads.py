"""GPU parity of the body loads (getElasticAppliedLoad's bodyForce / gravitational / centrifugal
branch) against the oracle through the C ABI: bricks and shells, all three kinds, whole meshes
and element subsets (repeated elements), zero and displaced states.  Loads agree to 1e-12
relative (bricks) and 1e-11 relative (shells)."""
import numpy as np
import pytest

from misc_gb300 import model as M
from misc_gb300.astro import AstroError, AstroGPU
from oracle import Oracle

pytestmark = pytest.mark.gpu


def _close(a, b, tol):
    assert np.linalg.norm(a - b) <= tol * np.linalg.norm(b), np.abs(a - b).max()


@pytest.fixture(scope="module")
def block():
    m = M.hex_block(6, 4, 3, lx=1.5, ly=1.0, lz=0.75, seed=4)
    m.material_density = np.random.default_rng(8).uniform(1000.0, 9000.0, m.num_els)
    return m, AstroGPU(m), Oracle(m)


@pytest.mark.parametrize("kind,vals", [
    (0, [1.5, -2.0, 3.0, 0.0, 0.0, 0.0]),
    (1, [0.0, 0.0, -9.81, 0.0, 0.0, 0.0]),
    (1, [3.0, 1.0, -2.0, 0.0, 0.0, 0.0]),
    (2, [0.2, -0.1, 0.3, 0.3, 1.0, 0.2, 40.0]),
])
def test_brick_body_loads_whole_mesh(block, kind, vals):
    m, g, o = block
    _close(g.body_load(kind, vals), o.body_load(kind, vals), 1e-12)


def test_brick_body_force_total(block):
    """Sum of the nodal body forces = force per volume x total volume (the partition of unity)."""
    m, g, o = block
    b = np.array([1.5, -2.0, 3.0])
    load = g.body_load(0, list(b) + [0.0, 0.0, 0.0])
    tot = load.reshape(3, -1).sum(axis=1)   # reference numbering: component-major
    assert np.allclose(tot, b * 1.5 * 1.0 * 0.75, rtol=1e-12)


def test_brick_body_loads_subset_and_state(block):
    """Element subsets (ragged, unordered, repeated elements add twice), accumulation into an
    existing load, and the centrifugal load at a displaced state (centroids move)."""
    m, g, o = block
    rng = np.random.default_rng(2)
    els = rng.choice(np.arange(1, m.num_els + 1), 17, replace=False)
    els = np.concatenate([els, els[:3]])
    u = 1e-2 * rng.standard_normal(o.n)
    st = M.make_state(o.n, disp=u)
    base = rng.standard_normal(o.n)
    for kind, vals in ((0, [1.0, 2.0, 3.0, 0, 0, 0]), (1, [0.5, 0.0, -9.81, 0, 0, 0]),
                       (2, [0.0, 0.5, 0.0, 1.0, 0.0, 0.0, 25.0])):
        lg = g.body_load(kind, vals, elements=els, state=st, elastic_load=base.copy())
        lo = o.body_load(kind, vals, elements=els, state=st, load=base.copy())
        _close(lg - base, lo - base, 1e-12)
    # the displaced centroids matter for the centrifugal load
    c0 = g.body_load(2, [0.0, 0.5, 0.0, 1.0, 0.0, 0.0, 25.0], elements=els)
    c1 = g.body_load(2, [0.0, 0.5, 0.0, 1.0, 0.0, 0.0, 25.0], elements=els, state=st)
    assert np.linalg.norm(c1 - c0) > 1e-6 * np.linalg.norm(c0)
    # an empty list adds nothing
    assert np.array_equal(g.body_load(1, [0, 0, -9.81], elements=[], elastic_load=base.copy()), base)


def test_brick_body_loads_config4_block():
    """Per-element moduli and densities of the correlated log-normal family."""
    m = M.config4_block(8, 4, 4, seed=3)
    m.material_density = np.random.default_rng(1).uniform(2000.0, 8000.0, m.num_els)
    g, o = AstroGPU(m), Oracle(m)
    for kind, vals in ((1, [0.0, -9.81, 0.0]), (2, [1.0, 0.0, 0.0, 0.0, 0.0, 1.0, 10.0])):
        _close(g.body_load(kind, vals), o.body_load(kind, vals), 1e-12)


def _plate():
    m = M.plate_shell(nx=5, ny=4, lx=2.0, ly=1.0, t=0.03, E=7e10, nu=0.33)
    rng = np.random.default_rng(5)
    X = m.node_list.copy()
    X[:, :2] += 0.05 * rng.uniform(-1, 1, (len(X), 2))
    X[:, 2] += 0.02 * rng.uniform(-1, 1, len(X))
    m.node_list = X
    m.layup_angle = np.array([0.3])
    return m


@pytest.fixture(scope="module")
def plate():
    m = _plate()
    return m, AstroGPU(m), Oracle(m)


@pytest.mark.parametrize("vals", [[0.0, 0.0, -9.81, 0.0, 0.0, 0.0], [1.0, -2.0, 0.5, 0.3, -0.2, 0.1]])
def test_shell_gravity_zero_state(plate, vals):
    m, g, o = plate
    _close(g.body_load(1, vals), o.body_load(1, vals), 1e-11)


def test_shell_gravity_displaced_state(plate):
    """Rotated nodes: the load uses the static orientation of the element's mean rotation, which
    moves the rotational rows (rotary inertia); those rows are checked on their own scale."""
    m, g, o = plate
    rng = np.random.default_rng(3)
    u = 1e-1 * rng.standard_normal(o.n)
    iv = 1e-4 * rng.standard_normal(o.int_vec_size)
    st = M.make_state(o.n, disp=u, internal_disp=iv)
    vals = [1.0, -2.0, 0.5, 0.3, -0.2, 0.1]
    z = o.body_load(1, vals).reshape(6, -1)
    lo = o.body_load(1, vals, state=st)
    rot = lambda v: v.reshape(6, -1)[3:]
    assert np.linalg.norm(rot(lo) - z[3:]) > 1e-5 * np.linalg.norm(z[3:])
    lg = g.body_load(1, vals, state=st)
    _close(lg, lo, 1e-11)
    _close(rot(lg), rot(lo), 1e-9)
    # the whole mesh listed explicitly, in any order, is the whole mesh
    els = np.random.default_rng(4).permutation(np.arange(1, m.num_els + 1))
    _close(g.body_load(1, vals, elements=els, state=st), lo, 1e-11)


@pytest.mark.parametrize("kind,vals", [
    (0, [1.0, -2.0, 0.5, 0.3, -0.2, 0.1]),
    (1, [0.5, 0.0, -9.81, 0.0, 0.0, 0.0]),
    (2, [0.3, 0.2, 0.0, 0.0, 0.2, 1.0, 30.0]),
])
def test_shell_loads_subsets_and_states(plate, kind, vals):
    """Shell body force, gravity and centrifugal loads over element subsets (repeats add twice)
    and the whole mesh, at the zero and a displaced state, accumulated into a load."""
    m, g, o = plate
    rng = np.random.default_rng(11)
    u = 1e-2 * rng.standard_normal(o.n)
    iv = 1e-4 * rng.standard_normal(o.int_vec_size)
    st = M.make_state(o.n, disp=u, internal_disp=iv)
    els = np.array([3, 1, 7, 7, m.num_els, 12])
    base = rng.standard_normal(o.n)
    for e_, s_ in ((None, None), (els, None), (els, st), (None, st)):
        lg = g.body_load(kind, vals, elements=e_, state=s_, elastic_load=base.copy())
        lo = o.body_load(kind, vals, elements=e_, state=s_, load=base.copy())
        _close(lg - base, lo - base, 1e-11)


def test_shell_bad_arguments(plate):
    m, g, o = plate
    with pytest.raises(AstroError):
        g.body_load(1, [0.0, 0.0, -9.81], elements=[m.num_els + 1])
    with pytest.raises(AstroError):
        g.body_load(5, [0.0, 0.0, -9.81])
    assert np.array_equal(g.body_load(0, [1.0, 0, 0], elements=[]), np.zeros(o.n))


@pytest.mark.parametrize("kind,vals", [
    (0, [1.0, -2.0, 0.5, 0.3, -0.2, 0.1]),
    (1, [0.5, 0.0, -9.81, 0.1, 0.0, 0.0]),
    (2, [0.3, 0.2, 0.0, 0.0, 0.2, 1.0, 30.0]),
])
def test_shell_body_load_design_derivative(kind, vals):
    """d(load)/d(thickness group) for shell body loads (getdRelasticdD's load branch) against
    central differences of the oracle's body load over the design variable's value; element
    subsets with repeats, a displaced state; bricks add nothing."""
    def mk(dv=None):
        m = M.add_design_variables(_plate(), 3, M.DCAT_LAYUP_THICKNESS)
        if dv is not None:
            m.d_value = np.asarray(dv, np.float64)
        return m
    m = mk()
    g = AstroGPU(m)
    rng = np.random.default_rng(2)
    st = M.make_state(g.n, disp=1e-3 * rng.standard_normal(g.n), internal_disp=1e-5 * rng.standard_normal(g.int_vec_size))
    for els in (None, np.array([1, 2, 2, 9, m.num_els])):
        for d in (1, 3):
            got = g.body_load_drdd(d, kind, vals, elements=els, state=st)
            step = 1e-6
            e = np.zeros(3)
            e[d - 1] = step
            fp = Oracle(mk(e)).body_load(kind, vals, elements=els, state=st)
            fm = Oracle(mk(-e)).body_load(kind, vals, elements=els, state=st)
            fd = -(fp - fm) / (2 * step)
            if np.linalg.norm(fd) == 0.0:
                assert np.linalg.norm(got) == 0.0
            else:
                _close(got, fd, 1e-6)
    b = M.add_design_variables(M.hex_block(3, 2, 2, seed=1), 2, M.DCAT_ELASTIC_MODULUS)
    gb = AstroGPU(b)
    assert np.array_equal(gb.body_load_drdd(1, 1, [0, 0, -9.81]), np.zeros(gb.n))
