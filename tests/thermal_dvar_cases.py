"""Models with thermal design variables, shared by the oracle and device tests.

Each case is a small brick or shell model with two design variables of one category (or a node
category) on the thermal path: conductivity, specific heat and density of solids; the layer's
conductivity, specific heat, density, thickness and angle of shells; node coordinates and solid
orientation, which move the element geometry.  The conductivities are anisotropic so that frame
rotations and layer angles change the conduction.
"""
import numpy as np

from misc_gb300 import model as M


def with_element_dvars(m, dvars):
    """dvars: list of (category, component, layer, value, elements (1-based)); coefficient 1.
    Replaces m's design variables (the reference's elToD maps, one term per element and variable
    in variable order)."""
    per = [[] for _ in range(m.num_els)]
    for j, (_, _, _, _, els) in enumerate(dvars):
        for e in els:
            per[e - 1].append(j + 1)
    m.el_to_d_range = np.concatenate([[0], np.cumsum([len(p) for p in per])]).astype(np.int32)
    m.el_to_d = np.array([d for p in per for d in p], np.int32)
    m.el_to_coef = np.ones(len(m.el_to_d))
    m.d_category = np.array([d[0] for d in dvars], np.int32)
    m.d_component = np.array([max(d[1], 1) for d in dvars], np.int32)
    m.d_layer = np.array([max(d[2], 1) for d in dvars], np.int32)
    m.d_value = np.array([float(d[3]) for d in dvars])
    return m


def brick():
    return M.hex_block(nx=3, ny=2, nz=2, jitter=0.1, seed=3)


def layered_plate():
    """shell4 plate with a two-layer laminate (0 and 0.4 rad) of one material."""
    m = M.plate_shell(nx=4, ny=3, lx=2.0, ly=1.0, t=0.03, E=7e10, nu=0.33)
    m.sec_layup_range = np.array([0, 2], np.int32)
    m.layup_mat_id = np.array([1, 1], np.int32)
    m.layup_thickness = np.array([0.012, 0.018])
    m.layup_angle = np.array([0.0, 0.4])
    return m


def thermal_tables(m):
    """(conductivity (M, 6), specific heat (M,)) per material: anisotropic, varying by material."""
    nm = len(m.material_density)
    base = np.array([45.0, 30.0, 20.0, 6.0, 3.0, 2.0])
    cond = np.array([base * (1.0 + 0.01 * k) for k in range(nm)])
    sh = 460.0 + 2.0 * np.arange(nm)
    return cond, sh


def _halves(n):
    return [list(range(1, n // 2 + 1)), list(range(n // 2 + 1, n + 1))]


def _elem_case(builder, cat, comp=0, layer=0, values=(0.0, 0.0)):
    def build():
        m = builder()
        a, b = _halves(m.num_els)
        return with_element_dvars(m, [(cat, comp, layer, values[0], a), (cat, comp, layer, values[1], b)])
    return build


def _node_case(builder, nodes, cat, comp, value=0.0, act_time=None):
    def build():
        return M.add_node_design_variables(builder(), nodes, cat, component=comp, value=value, act_time=act_time)
    return build


# name: (builder, central-difference step, dynamic)
CASES = {
    "brick_thermal_cond_k11": (_elem_case(brick, M.DCAT_THERMAL_COND, comp=1, values=(2.0, -1.0)), 1e-3, False),
    "brick_thermal_cond_k12": (_elem_case(brick, M.DCAT_THERMAL_COND, comp=4, values=(0.5, 0.0)), 1e-3, False),
    "brick_spec_heat": (_elem_case(brick, M.DCAT_SPEC_HEAT, values=(10.0, 0.0)), 1e-2, True),
    "brick_density": (_elem_case(brick, M.DCAT_DENSITY, values=(50.0, 0.0)), 1e-2, True),
    "brick_orientation": (_elem_case(brick, M.DCAT_ORIENTATION, comp=3, values=(0.1, 0.0)), 1e-6, False),
    "brick_node_coord": (_node_case(brick, [[7, 8, 18], [20, 23]], M.DCAT_NODE_COORD, 2), 1e-7, True),
    "shell_layup_thermal_cond": (_elem_case(layered_plate, M.DCAT_LAYUP_THERMAL_COND, comp=2, layer=2,
                                            values=(3.0, 0.0)), 1e-3, False),
    "shell_layup_spec_heat": (_elem_case(layered_plate, M.DCAT_LAYUP_SPEC_HEAT, layer=1, values=(5.0, 0.0)), 1e-2,
                              True),
    "shell_layup_density": (_elem_case(layered_plate, M.DCAT_LAYUP_DENSITY, layer=2, values=(20.0, 0.0)), 1e-2,
                            True),
    "shell_layup_thickness": (_elem_case(layered_plate, M.DCAT_LAYUP_THICKNESS, layer=1, values=(0.002, 0.0)), 1e-7,
                              True),
    "shell_layup_angle": (_elem_case(layered_plate, M.DCAT_LAYUP_ANGLE, layer=2, values=(0.1, 0.0)), 1e-6, False),
    "shell_node_coord": (_node_case(layered_plate, [[7, 8], [13]], M.DCAT_NODE_COORD, 1), 1e-7, True),
}


def thermal_state(n, dynamic, seed=7):
    """A temperature field (and the previous step's for a transient step), rank order."""
    rng = np.random.default_rng(seed)
    st = dict(temp=20.0 + 5.0 * rng.standard_normal(n))
    if dynamic:
        st.update(prev_temp=20.0 + 5.0 * rng.standard_normal(n), prev_tdot=rng.standard_normal(n), dynamic=1,
                  gamma=0.5, del_t=0.1)
    return st


def heat_gen_elements(m):
    """An element list with a repeat (the load lists it twice)."""
    return [1, 2, 2, m.num_els]


def flux_faces(m):
    """Faces for the surface flux: x = max faces of the bricks (face 4), top faces of the shells
    (face 1), element numbers 1-based."""
    if m.element_type[0] == 41:
        return list(range(1, m.num_els + 1)), [1] * m.num_els
    X = m.node_list
    xmax = X[:, 0].max()
    els = [e + 1 for e in range(m.num_els)
           if np.isclose(X[m.element_list[e, [1, 2, 5, 6]] - 1, 0], xmax).all()]
    return els, [4] * len(els)
