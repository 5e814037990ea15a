"""Model arrays in the reference's layout and seeded synthetic meshes.

A ``Model`` holds the module globals that ``readModelInput`` fills in the reference
(Working/AStrO_globalData.f90; storage conventions Working/AStrO_input.f90:431-452, 703-734,
1072-1095): ``nodeList(3,N)``, ``elementList(8,e)`` (1-based, 0-padded), ``elementType``,
sections, layups, materials, and constraints expanded to one equation per constrained node
DOF (the node-set expansion of buildElasticMPC, Working/AStrO_bookKeeping.f90:474-612).
``Model.as_c()`` returns the ``astro_model`` C struct of include/astro_gpu.h.

The generators build the benchmark workloads as seeded synthetic meshes (no reference input
deck exists for them):
  * ``plate_shell``      shell4 cantilever plate (40x8 on [0,10]x[-1,1], t=0.05, clamped x=0);
  * ``hex_block``        brick8 block (64x32x32 on [0,4]x[0,2]x[0,2], jittered interior nodes,
                         log-normal per-element modulus, clamped x=0, traction on x=4);
  * ``shell_beam``       the 10-element shell4 strip of Working/shellBeamModelInput.yaml.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

I32P = C.POINTER(C.c_int32)
F64P = C.POINTER(C.c_double)


class AstroModelC(C.Structure):
    _fields_ = [
        ("num_nodes", C.c_int32), ("num_els", C.c_int32),
        ("node_list", F64P), ("element_list", I32P), ("element_type", I32P), ("element_section", I32P),
        ("num_sections", C.c_int32), ("section_mat_id", I32P), ("section_orient", F64P),
        ("sec_layup_range", I32P), ("layup_mat_id", I32P), ("layup_thickness", F64P),
        ("layup_angle", F64P), ("section_z_offset", F64P),
        ("num_materials", C.c_int32), ("material_elastic", F64P), ("material_density", F64P),
        ("num_mpc", C.c_int32), ("mpc_range", I32P), ("mpc_node", I32P), ("mpc_dof", I32P),
        ("mpc_coef", F64P), ("mpc_rhs", F64P),
        ("num_dvars", C.c_int32), ("el_to_d_range", I32P), ("el_to_d", I32P), ("el_to_coef", F64P),
        ("d_category", I32P), ("d_component", I32P), ("d_layer", I32P), ("d_value", F64P),
        ("nd_to_d_range", I32P), ("nd_to_d", I32P), ("nd_to_coef", F64P), ("d_act_time", F64P),
    ]


class AstroStateC(C.Structure):
    _fields_ = [
        ("node_disp", F64P), ("node_vel", F64P), ("node_acc", F64P),
        ("prev_disp", F64P), ("prev_vel", F64P), ("prev_acc", F64P),
        ("internal_disp", F64P), ("prev_int_disp", F64P),
        ("dynamic", C.c_int32), ("nm_beta", C.c_double), ("nm_gamma", C.c_double), ("del_t", C.c_double),
    ]


DCAT_LAYUP_THICKNESS = 1
DCAT_ELASTIC_MODULUS = 2
DCAT_DENSITY = 3
DCAT_ORIENTATION = 4
DCAT_LAYUP_ZOFFSET = 5
DCAT_LAYUP_ANGLE = 6
DCAT_LAYUP_DENSITY = 7
DCAT_NODE_COORD = 8
DCAT_NODE_LOAD = 9
DCAT_THERMAL_COND = 10
DCAT_SPEC_HEAT = 11
DCAT_LAYUP_THERMAL_COND = 12
DCAT_LAYUP_SPEC_HEAT = 13
DCAT_LAYUP_MODULUS = 14


def _p(a, typ):
    if a is None:
        return C.cast(None, typ)
    return a.ctypes.data_as(typ)


def _i32(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.int32))


def _f64(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64))


@dataclass
class Model:
    node_list: np.ndarray            # (N,3) float64 -> stored as nodeList(3,N)
    element_list: np.ndarray         # (e,8) int32, 1-based, 0-padded
    element_type: np.ndarray         # (e,)
    element_section: np.ndarray      # (e,) 1-based
    section_mat_id: np.ndarray       # (S,)
    section_orient: np.ndarray       # (S,3,3): rows are the local axes
    sec_layup_range: np.ndarray      # (S+1,)
    layup_mat_id: np.ndarray
    layup_thickness: np.ndarray
    layup_angle: np.ndarray
    section_z_offset: np.ndarray     # (S,)
    material_elastic: np.ndarray     # (M,9)
    material_density: np.ndarray     # (M,)
    mpc_range: np.ndarray = field(default_factory=lambda: np.zeros(1, np.int32))
    mpc_node: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    mpc_dof: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    mpc_coef: np.ndarray = field(default_factory=lambda: np.zeros(0))
    mpc_rhs: np.ndarray = field(default_factory=lambda: np.zeros(0))
    el_to_d_range: np.ndarray | None = None
    el_to_d: np.ndarray | None = None
    el_to_coef: np.ndarray | None = None
    d_category: np.ndarray | None = None
    d_component: np.ndarray | None = None
    d_layer: np.ndarray | None = None
    d_value: np.ndarray | None = None
    nd_to_d_range: np.ndarray | None = None   # (N+1,) node -> design variable map (ndToD)
    nd_to_d: np.ndarray | None = None
    nd_to_coef: np.ndarray | None = None
    d_act_time: np.ndarray | None = None      # (num_dvars, 2): activity window of nodeLoad variables
    # loads (not part of the C model struct): faces carrying traction/pressure, point loads
    face_el: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    face_num: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    traction: np.ndarray = field(default_factory=lambda: np.zeros(3))
    pressure: float = 0.0
    point_loads: list = field(default_factory=list)   # (node, dof, value)
    name: str = "model"

    @property
    def num_nodes(self):
        return int(self.node_list.shape[0])

    @property
    def num_els(self):
        return int(self.element_list.shape[0])

    @property
    def dof_per_node(self):
        return 6 if int(self.element_type[0]) == 41 else 3

    def as_c(self) -> AstroModelC:
        """The astro_model struct; the arrays it points to are kept alive on the struct."""
        keep = {}

        def k(name, arr):
            keep[name] = arr
            return arr

        nl = k("nl", _f64(self.node_list))          # (N,3) row-major == nodeList(3,N) column-major
        el = k("el", _i32(self.element_list))
        so = k("so", _f64(np.transpose(self.section_orient, (0, 2, 1))))  # column-major 3x3 per section
        me = k("me", _f64(self.material_elastic))
        m = AstroModelC()
        m.num_nodes = self.num_nodes
        m.num_els = self.num_els
        m.node_list = _p(nl, F64P)
        m.element_list = _p(el, I32P)
        m.element_type = _p(k("et", _i32(self.element_type)), I32P)
        m.element_section = _p(k("es", _i32(self.element_section)), I32P)
        m.num_sections = len(self.section_mat_id)
        m.section_mat_id = _p(k("sm", _i32(self.section_mat_id)), I32P)
        m.section_orient = _p(so, F64P)
        m.sec_layup_range = _p(k("slr", _i32(self.sec_layup_range)), I32P)
        m.layup_mat_id = _p(k("lm", _i32(self.layup_mat_id)), I32P)
        m.layup_thickness = _p(k("lt", _f64(self.layup_thickness)), F64P)
        m.layup_angle = _p(k("la", _f64(self.layup_angle)), F64P)
        m.section_z_offset = _p(k("sz", _f64(self.section_z_offset)), F64P)
        m.num_materials = int(me.shape[0])
        m.material_elastic = _p(me, F64P)
        m.material_density = _p(k("md", _f64(self.material_density)), F64P)
        m.num_mpc = int(len(self.mpc_range) - 1)
        m.mpc_range = _p(k("mr", _i32(self.mpc_range)), I32P)
        m.mpc_node = _p(k("mn", _i32(self.mpc_node)), I32P)
        m.mpc_dof = _p(k("mdf", _i32(self.mpc_dof)), I32P)
        m.mpc_coef = _p(k("mc", _f64(self.mpc_coef)), F64P)
        m.mpc_rhs = _p(k("mrh", _f64(self.mpc_rhs)), F64P)
        if self.d_value is not None and len(self.d_value) > 0:
            m.num_dvars = len(self.d_value)
            if self.el_to_d_range is not None:
                m.el_to_d_range = _p(k("edr", _i32(self.el_to_d_range)), I32P)
                m.el_to_d = _p(k("ed", _i32(self.el_to_d)), I32P)
                m.el_to_coef = _p(k("ec", _f64(self.el_to_coef)), F64P)
            m.d_category = _p(k("dc", _i32(self.d_category)), I32P)
            m.d_component = _p(k("dco", _i32(self.d_component)), I32P)
            m.d_layer = _p(k("dl", _i32(self.d_layer)), I32P)
            m.d_value = _p(k("dv", _f64(self.d_value)), F64P)
            if self.el_to_d_range is None:   # node design variables only
                m.el_to_d_range = _p(k("edr", np.zeros(self.num_els + 1, np.int32)), I32P)
                m.el_to_d = _p(k("ed", np.zeros(1, np.int32)), I32P)
                m.el_to_coef = _p(k("ec", np.zeros(1)), F64P)
            if self.nd_to_d_range is not None:
                m.nd_to_d_range = _p(k("ndr", _i32(self.nd_to_d_range)), I32P)
                m.nd_to_d = _p(k("nd", _i32(self.nd_to_d)), I32P)
                m.nd_to_coef = _p(k("nc", _f64(self.nd_to_coef)), F64P)
            if self.d_act_time is not None:
                m.d_act_time = _p(k("dat", _f64(self.d_act_time)), F64P)
        else:
            m.num_dvars = 0
        m._keep = keep
        return m


def make_state(n, n_int=0, disp=None, vel=None, acc=None, prev_disp=None, prev_vel=None, prev_acc=None,
               internal_disp=None, prev_int_disp=None, dynamic=0, beta=0.25, gamma=0.5, del_t=0.0):
    """astro_state struct over float64 arrays (None = zeros)."""
    s = AstroStateC()
    keep = {}
    for name, arr in (("node_disp", disp), ("node_vel", vel), ("node_acc", acc), ("prev_disp", prev_disp),
                      ("prev_vel", prev_vel), ("prev_acc", prev_acc), ("internal_disp", internal_disp),
                      ("prev_int_disp", prev_int_disp)):
        if arr is not None:
            a = _f64(arr)
            keep[name] = a
            setattr(s, name, _p(a, F64P))
    s.dynamic = dynamic
    s.nm_beta = beta
    s.nm_gamma = gamma
    s.del_t = del_t
    s._keep = keep
    return s


def add_design_variables(m: Model, n_groups: int, category: int, layer: int = 1, component: int = 1,
                         value: float = 0.0) -> Model:
    """Attaches n_groups design variables of one category to m, one per contiguous group of
    elements (element e belongs to group e * n_groups // num_els), each entering its elements
    with coefficient 1: thickness of layer `layer` (+ d) or materialElastic entry `component`
    (+ d).  The reference's dVec / elToD maps (Working/AStrO_input.f90 design-variable input)."""
    E = m.num_els
    grp = (np.arange(E) * n_groups) // E + 1
    m.el_to_d_range = np.arange(E + 1, dtype=np.int32)
    m.el_to_d = grp.astype(np.int32)
    m.el_to_coef = np.ones(E)
    m.d_category = np.full(n_groups, category, np.int32)
    m.d_component = np.full(n_groups, component, np.int32)
    m.d_layer = np.full(n_groups, layer, np.int32)
    m.d_value = np.full(n_groups, float(value))
    return m


def add_node_design_variables(m: Model, node_groups, category: int, component: int = 1, value: float = 0.0,
                              act_time=None) -> Model:
    """Attaches one design variable of a node category (nodeCoord, nodeLoad) per group of nodes
    (1-based node numbers), each entering its nodes with coefficient 1 (the reference's ndToD
    maps); act_time (start, end) is the activity window of nodeLoad variables.  Replaces any
    design variables m already has."""
    N = m.num_nodes
    lists = [[] for _ in range(N)]
    for g, nodes in enumerate(node_groups):
        for nd in nodes:
            lists[nd - 1].append(g + 1)
    m.nd_to_d_range = np.concatenate([[0], np.cumsum([len(x) for x in lists])]).astype(np.int32)
    m.nd_to_d = np.array([d for x in lists for d in x], np.int32)
    m.nd_to_coef = np.ones(len(m.nd_to_d))
    nd = len(node_groups)
    m.el_to_d_range = np.zeros(m.num_els + 1, np.int32)
    m.el_to_d = np.zeros(0, np.int32)
    m.el_to_coef = np.zeros(0)
    m.d_category = np.full(nd, category, np.int32)
    m.d_component = np.full(nd, component, np.int32)
    m.d_layer = np.ones(nd, np.int32)
    m.d_value = np.full(nd, float(value))
    if act_time is not None:
        m.d_act_time = np.tile(np.asarray(act_time, np.float64), (nd, 1))
    return m


def _iso(E, nu, G=None):
    """materialElastic(9) for an isotropic material; G = E/(2(1+nu)) when not given
    (Working/AStrO_input.f90:807-809)."""
    if G is None:
        G = E / (2.0 * (1.0 + nu))
    return [E, E, E, nu, nu, nu, G, G, G]


def _clamp_mpc(nodes, dofs):
    """One equation per (node, dof): 1.0 * u = 0 (reference 'constraints: matrix' rows applied to a
    node set, expanded per node as buildElasticMPC does)."""
    nodes = np.asarray(nodes, dtype=np.int32)
    terms_n, terms_d = [], []
    for nd in nodes:
        for d in dofs:
            terms_n.append(nd)
            terms_d.append(d)
    m = len(terms_n)
    return (np.arange(m + 1, dtype=np.int32), np.array(terms_n, np.int32), np.array(terms_d, np.int32),
            np.ones(m), np.zeros(m))


def plate_shell(nx=40, ny=8, lx=10.0, ly=2.0, t=0.05, E=7.0e10, nu=0.33, rho=2700.0, pressure=1.0e3,
                clamp="x0", y0=None, name="plate"):
    """shell4 plate on [0,lx] x [y0, y0+ly] at z = 0, nodes numbered x-fastest, elements
    counter-clockwise (normal +z).  clamp: "x0" clamps all 6 DOF on x = 0, "ss" simply supports
    all edges (w = 0)."""
    if y0 is None:
        y0 = -0.5 * ly
    xs = np.linspace(0.0, lx, nx + 1)
    ys = np.linspace(y0, y0 + ly, ny + 1)
    X, Y = np.meshgrid(xs, ys, indexing="xy")
    nodes = np.stack([X.ravel(), Y.ravel(), np.zeros(X.size)], axis=1)
    nid = lambda i, j: j * (nx + 1) + i + 1
    els = np.zeros((nx * ny, 8), np.int32)
    k = 0
    for j in range(ny):
        for i in range(nx):
            els[k, :4] = [nid(i, j), nid(i + 1, j), nid(i + 1, j + 1), nid(i, j + 1)]
            k += 1
    ne = nx * ny
    m = Model(
        node_list=nodes, element_list=els, element_type=np.full(ne, 41, np.int32),
        element_section=np.ones(ne, np.int32), section_mat_id=np.ones(1, np.int32),
        section_orient=np.eye(3)[None], sec_layup_range=np.array([0, 1], np.int32),
        layup_mat_id=np.ones(1, np.int32), layup_thickness=np.array([t]), layup_angle=np.zeros(1),
        section_z_offset=np.zeros(1), material_elastic=np.array([_iso(E, nu)]),
        material_density=np.array([rho]), name=name)
    if clamp == "x0":
        cn = [nid(0, j) for j in range(ny + 1)]
        m.mpc_range, m.mpc_node, m.mpc_dof, m.mpc_coef, m.mpc_rhs = _clamp_mpc(cn, range(1, 7))
    elif clamp == "ss":
        cn = sorted({nid(i, j) for i in range(nx + 1) for j in range(ny + 1)
                     if i in (0, nx) or j in (0, ny)})
        m.mpc_range, m.mpc_node, m.mpc_dof, m.mpc_coef, m.mpc_rhs = _clamp_mpc(cn, [3])
    m.face_el = np.arange(1, ne + 1, dtype=np.int32)
    m.face_num = np.ones(ne, np.int32)
    m.pressure = pressure
    return m


def config5_cases(m, n_dof_index, steps, dt, num_random=16, seed0=5000, force=100.0):
    """Load cases of the Newmark benchmark plate (a square shell4 plate from plate_shell with
    nx = ny): case 0 the centre force force * sin(2 pi 500 t) on w; cases 1 .. num_random a point
    force on w at an interior node drawn uniformly (generator seed0 + k), amplitude
    force * U(0.5, 1.5) * sin(2 pi f t + phi) with f ~ U(200, 800) Hz and phi ~ U(0, 2 pi).
    Returns patterns (cases, n) and amplitudes (cases, steps), t = dt, 2 dt, ..."""
    nx = int(round(np.sqrt(m.num_nodes))) - 1
    n = int(n_dof_index.max())
    t = dt * np.arange(1, steps + 1)
    P = np.zeros((num_random + 1, n))
    A = np.zeros((num_random + 1, steps))
    centre = (nx // 2) * (nx + 1) + nx // 2 + 1
    P[0, n_dof_index[centre - 1, 2] - 1] = 1.0
    A[0] = force * np.sin(2 * np.pi * 500.0 * t)
    for k in range(1, num_random + 1):
        rng = np.random.default_rng(seed0 + k)
        i, j = (int(v) for v in rng.integers(1, nx, 2))
        nd = j * (nx + 1) + i + 1
        P[k, n_dof_index[nd - 1, 2] - 1] = 1.0
        A[k] = force * rng.uniform(0.5, 1.5) * np.sin(2 * np.pi * rng.uniform(200.0, 800.0) * t +
                                                     rng.uniform(0.0, 2 * np.pi))
    return P, A


def panel_batch(num_panels=512, seed0=1000, n_range=(8, 96), t_range=(0.01, 0.1), p_range=(1.0e2, 1.0e4),
                n_dvars=32, h=0.1, E=7.0e10, nu=0.33, rho=2700.0, name="panels", indices=None):
    """Batch of independent shell4 panels as one model (its connected components): panel p has
    n_x, n_y ~ U{n_range} elements of size h (its own generator, seed seed0 + p), thickness
    t ~ U(t_range) (one section per panel), all six DOF clamped on its x = 0 edge, and a pressure
    ~ U(p_range) on all its elements.  n_dvars design variables: layup thickness groups of equal
    element count within every panel (element k of a panel with e elements is in group
    k * n_dvars // e); design variable g covers group g of every panel.  The panels lie side by
    side in z (disconnected).  indices: the panels of the num_panels-panel batch to build (default
    all), each identical to its copy in the whole batch.  Extra attributes: panel_el_ptr,
    panel_node_ptr (per panel first element / node, 0-based, plus the totals), panel_pressure,
    panel_thickness, panel_n."""
    nodes, els, sec, thick, pres, nxy = [], [], [], [], [], []
    mpc_nodes, el_ptr, nd_ptr = [], [0], [0]
    grp = []
    nn = 0
    for p in (range(num_panels) if indices is None else indices):
        rng = np.random.default_rng(seed0 + p)
        nx, ny = (int(v) for v in rng.integers(n_range[0], n_range[1] + 1, 2))
        t = float(rng.uniform(*t_range))
        pr = float(rng.uniform(*p_range))
        xs = np.arange(nx + 1) * h
        ys = np.arange(ny + 1) * h
        X, Y = np.meshgrid(xs, ys, indexing="xy")
        nodes.append(np.stack([X.ravel(), Y.ravel(), np.full(X.size, float(p))], axis=1))
        nid = lambda i, j: nn + j * (nx + 1) + i + 1
        e = np.zeros((nx * ny, 8), np.int32)
        jj, ii = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
        ii, jj = ii.ravel(), jj.ravel()
        e[:, 0], e[:, 1], e[:, 2], e[:, 3] = nid(ii, jj), nid(ii + 1, jj), nid(ii + 1, jj + 1), nid(ii, jj + 1)
        els.append(e)
        ne = nx * ny
        sec.append(np.full(ne, len(thick) + 1, np.int32))
        grp.append((np.arange(ne) * n_dvars) // ne + 1)
        mpc_nodes += [nid(0, j) for j in range(ny + 1)]
        thick.append(t)
        pres.append(pr)
        nxy.append((nx, ny))
        nn += (nx + 1) * (ny + 1)
        el_ptr.append(el_ptr[-1] + ne)
        nd_ptr.append(nn)
    nodes = np.vstack(nodes)
    els = np.vstack(els)
    E_ = els.shape[0]
    S = len(thick)
    m = Model(
        node_list=nodes, element_list=els, element_type=np.full(E_, 41, np.int32),
        element_section=np.concatenate(sec), section_mat_id=np.ones(S, np.int32),
        section_orient=np.broadcast_to(np.eye(3), (S, 3, 3)).copy(),
        sec_layup_range=np.arange(S + 1, dtype=np.int32), layup_mat_id=np.ones(S, np.int32),
        layup_thickness=np.array(thick), layup_angle=np.zeros(S), section_z_offset=np.zeros(S),
        material_elastic=np.array([_iso(E, nu)]), material_density=np.array([rho]), name=name)
    m.mpc_range, m.mpc_node, m.mpc_dof, m.mpc_coef, m.mpc_rhs = _clamp_mpc(mpc_nodes, range(1, 7))
    m.face_el = np.arange(1, E_ + 1, dtype=np.int32)
    m.face_num = np.ones(E_, np.int32)
    m.pressure = 0.0
    if n_dvars:
        m.el_to_d_range = np.arange(E_ + 1, dtype=np.int32)
        m.el_to_d = np.concatenate(grp).astype(np.int32)
        m.el_to_coef = np.ones(E_)
        m.d_category = np.full(n_dvars, 1, np.int32)
        m.d_component = np.ones(n_dvars, np.int32)
        m.d_layer = np.ones(n_dvars, np.int32)
        m.d_value = np.zeros(n_dvars)
    m.panel_el_ptr = np.array(el_ptr)
    m.panel_node_ptr = np.array(nd_ptr)
    m.panel_pressure = np.array(pres)
    m.panel_thickness = np.array(thick)
    m.panel_n = np.array(nxy)
    return m


def hex_block(nx=64, ny=32, nz=32, lx=4.0, ly=2.0, lz=2.0, jitter=0.1, seed=0, E_med=2.0e11, sigma=0.5,
              nu=0.3, rho=7800.0, traction=1.0e6, E_field=None, name="block"):
    """brick8 block; interior nodes jittered U(-jitter*h, +jitter*h) per axis; per-element modulus
    E = E_med*exp(sigma*z), z ~ N(0,1) (or E_field given per element, shape (nz,ny,nx) or (e,)).
    x = 0 clamped (3 DOF), traction +x on the x = lx face.  One section and one material per
    element so that every element carries its own modulus."""
    rng = np.random.default_rng(seed)
    xs = np.linspace(0.0, lx, nx + 1)
    ys = np.linspace(0.0, ly, ny + 1)
    zs = np.linspace(0.0, lz, nz + 1)
    Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
    nodes = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    h = np.array([lx / nx, ly / ny, lz / nz])
    ii, jj, kk = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), np.arange(nz + 1), indexing="xy")
    # node index order: k (z) slowest, j, i fastest
    I = np.broadcast_to(np.arange(nx + 1)[None, None, :], (nz + 1, ny + 1, nx + 1)).ravel()
    J = np.broadcast_to(np.arange(ny + 1)[None, :, None], (nz + 1, ny + 1, nx + 1)).ravel()
    K = np.broadcast_to(np.arange(nz + 1)[:, None, None], (nz + 1, ny + 1, nx + 1)).ravel()
    interior = (I > 0) & (I < nx) & (J > 0) & (J < ny) & (K > 0) & (K < nz)
    if jitter > 0:
        d = rng.uniform(-jitter, jitter, size=(nodes.shape[0], 3)) * h[None, :]
        nodes = nodes + d * interior[:, None]
    nid = lambda i, j, k: (k * (ny + 1) + j) * (nx + 1) + i + 1
    ne = nx * ny * nz
    els = np.zeros((ne, 8), np.int32)
    e = 0
    ex = np.zeros(ne, np.int32)
    for k in range(nz):
        for j in range(ny):
            i = np.arange(nx)
            base = slice(e, e + nx)
            els[base, 0] = nid(i, j, k)
            els[base, 1] = nid(i + 1, j, k)
            els[base, 2] = nid(i + 1, j + 1, k)
            els[base, 3] = nid(i, j + 1, k)
            els[base, 4] = nid(i, j, k + 1)
            els[base, 5] = nid(i + 1, j, k + 1)
            els[base, 6] = nid(i + 1, j + 1, k + 1)
            els[base, 7] = nid(i, j + 1, k + 1)
            ex[base] = i
            e += nx
    if E_field is None:
        Ee = E_med * np.exp(sigma * rng.standard_normal(ne))
    else:
        Ee = np.asarray(E_field, dtype=np.float64).reshape(ne)
    mat = np.zeros((ne, 9))
    G = Ee / (2.0 * (1.0 + nu))
    mat[:, 0:3] = Ee[:, None]
    mat[:, 3:6] = nu
    mat[:, 6:9] = G[:, None]
    m = Model(
        node_list=nodes, element_list=els, element_type=np.full(ne, 8, np.int32),
        element_section=np.arange(1, ne + 1, dtype=np.int32), section_mat_id=np.arange(1, ne + 1, dtype=np.int32),
        section_orient=np.broadcast_to(np.eye(3), (ne, 3, 3)).copy(),
        sec_layup_range=np.zeros(ne + 1, np.int32), layup_mat_id=np.zeros(0, np.int32),
        layup_thickness=np.zeros(0), layup_angle=np.zeros(0), section_z_offset=np.zeros(ne),
        material_elastic=mat, material_density=np.full(ne, rho), name=name)
    cn = [nid(0, j, k) for k in range(nz + 1) for j in range(ny + 1)]
    m.mpc_range, m.mpc_node, m.mpc_dof, m.mpc_coef, m.mpc_rhs = _clamp_mpc(cn, [1, 2, 3])
    # face 4 of brick8 = local nodes (2,3,7,6): the +x face of an element
    last = np.nonzero(ex == nx - 1)[0] + 1
    m.face_el = last.astype(np.int32)
    m.face_num = np.full(len(last), 4, np.int32)
    m.traction = np.array([traction, 0.0, 0.0])
    return m


def correlated_log_normal(nx, ny, nz, h, corr_len, sigma, E_med=2.0e11, seed=0):
    """Per-element modulus field E = E_med * exp(sigma * z) with z a Gaussian-correlated,
    unit-variance field on the (nz, ny, nx) element grid: white noise filtered in Fourier space by
    exp(-(k * corr_len)^2 / 2) (k in rad per unit length, element spacing h = (hx, hy, hz)), then
    standardised.  Returns shape (nz, ny, nx)."""
    rng = np.random.default_rng(seed)
    w = rng.standard_normal((nz, ny, nx))
    kz = 2 * np.pi * np.fft.fftfreq(nz, d=h[2])
    ky = 2 * np.pi * np.fft.fftfreq(ny, d=h[1])
    kx = 2 * np.pi * np.fft.rfftfreq(nx, d=h[0])
    k2 = kz[:, None, None] ** 2 + ky[None, :, None] ** 2 + kx[None, None, :] ** 2
    z = np.fft.irfftn(np.fft.rfftn(w) * np.exp(-0.5 * k2 * corr_len ** 2), s=(nz, ny, nx), axes=(0, 1, 2))
    z = (z - z.mean()) / max(z.std(), 1e-300)
    return E_med * np.exp(sigma * z)


def config4_block(nx, ny, nz, seed, corr_len=None, sigma=None):
    """Learned-preconditioner family: a brick8 block with the element size of the 64x32x32 block
    (box (nx, ny, nz) / 16), interior jitter 10 %, nu = 0.3, x = 0 clamped, traction 1e6 Pa on the
    far x face, and a Gaussian-correlated log-normal modulus (median 2e11) whose correlation
    length (a fraction U[0.2, 1.0] of the box width) and sigma (U[0.3, 1.0]) are drawn from the
    seed unless given.  Training blocks are 32x16x16, the evaluation block 96x48x48."""
    rng = np.random.default_rng(seed)
    lx, ly, lz = nx / 16.0, ny / 16.0, nz / 16.0
    frac = rng.uniform(0.2, 1.0) if corr_len is None else corr_len
    sig = rng.uniform(0.3, 1.0) if sigma is None else sigma
    E = correlated_log_normal(nx, ny, nz, (lx / nx, ly / ny, lz / nz), frac * ly, sig, seed=seed + 1)
    m = hex_block(nx=nx, ny=ny, nz=nz, lx=lx, ly=ly, lz=lz, seed=seed, E_field=E,
                  name=f"cfg4_block_{nx}x{ny}x{nz}_seed{seed}")
    m.field = {"corr_len_frac": float(frac), "sigma": float(sig)}
    return m


def shell_beam():
    """Working/shellBeamModelInput.yaml: 10 shell4 elements on [0,10]x[-0.5,0.5], t = 0.1,
    E = 1e6, nu = 0.3, G = 384615; root nodes (1, 12) clamped in all 6 DOF; unit z load on each
    tip node (11, 22)."""
    m = plate_shell(nx=10, ny=1, lx=10.0, ly=1.0, t=0.1, E=1.0e6, nu=0.3, rho=1.0, pressure=0.0, y0=-0.5,
                    name="shellBeam")
    m.material_elastic = np.array([[1.0e6, 1.0e6, 1.0e6, 0.3, 0.3, 0.3, 384615.0, 384615.0, 384615.0]])
    m.face_el = np.zeros(0, np.int32)
    m.face_num = np.zeros(0, np.int32)
    m.point_loads = [(11, 3, 1.0), (22, 3, 1.0)]
    return m


def config1():
    """Cantilever plate: 40x8 shell4, length 10, width 2, t = 0.05, E = 7e10, nu = 0.33,
    clamped x = 0, uniform pressure 1e3 Pa on all elements."""
    return plate_shell(name="cfg1_plate_40x8")


def config2(seed=0, nx=64, ny=32, nz=32):
    """Heterogeneous solid block: 64x32x32 brick8 on 4x2x2, interior jitter 10 %, log-normal E
    (median 2e11, sigma 0.5), nu = 0.3, x = 0 clamped, traction 1e6 Pa on x = 4."""
    return hex_block(nx=nx, ny=ny, nz=nz, lx=4.0 * nx / 64, ly=2.0 * ny / 32, lz=2.0 * nz / 32, seed=seed,
                     name=f"cfg2_block_{nx}x{ny}x{nz}")
