"""The model input reader (readModelInput's keyword scanner, Working/AStrO_input.f90:27-1091)
against the reference's example model file (tests/golden/shell_beam_model_input.yaml, a verbatim
copy made by tests/golden/make_shell_beam_input.py), a written-and-read-back config-1 plate,
and the scanner's rules for sets, materials and constraint expansion.  CPU only, except the last
test (the read model solved on the GPU)."""
import ctypes
from pathlib import Path

import numpy as np
import pytest
import scipy.sparse.linalg as spla

from misc_gb300 import inputfile as IF
from misc_gb300 import model as M
from oracle import Oracle
from oracle.oracle import _lib

FIX = Path(__file__).parent / "golden" / "shell_beam_model_input.yaml"


def _eqset(m):
    return sorted((tuple((int(m.mpc_node[t]), int(m.mpc_dof[t]), float(m.mpc_coef[t]))
                         for t in range(m.mpc_range[r], m.mpc_range[r + 1])), float(m.mpc_rhs[r]))
                  for r in range(len(m.mpc_range) - 1))


def test_shell_beam_fixture():
    mi = IF.read_model_input(FIX)
    m, ref = mi.model(), M.shell_beam()
    assert mi.num_nodes == 22 and mi.num_els == 10
    assert np.array_equal(m.node_list, ref.node_list)
    assert np.array_equal(m.element_list, ref.element_list)
    assert np.array_equal(m.element_type, ref.element_type) and np.all(m.element_section == 1)
    assert np.array_equal(m.layup_thickness, ref.layup_thickness) and m.layup_angle[0] == 0.0
    assert np.array_equal(m.material_elastic, ref.material_elastic)
    assert np.array_equal(m.section_orient[0], np.eye(3))
    assert mi.node_sets == {"root": [1, 12], "tip": [11, 22]} and mi.element_sets["allEls"] == list(range(1, 11))
    assert _eqset(m) == _eqset(ref)
    assert sorted(mi.nodal_loads()) == sorted(ref.point_loads)
    assert np.array_equal(mi.initial["displacement"][10], [0, 0, 1.0, 0, 0, 0])


def test_shell_beam_fixture_solves_to_beam_theory():
    """The read model, solved by the oracle with the consistent shell tangent, bends like the
    cantilever strip it describes (tip load 2, L = 10, t = 0.1, E = 1e6: 7.28 .. 8.0)."""
    mi = IF.read_model_input(FIX)
    m = mi.model()
    m.point_loads = mi.nodal_loads()
    L = _lib()
    L.orc_set_quirk.argtypes = [ctypes.c_int, ctypes.c_int]
    L.orc_set_quirk(1, 1)
    try:
        o = Oracle(m)
        A, b, *_ = o.static_system()
        w = spla.spsolve(A.tocsc(), b)[o.n_dof_index[10, 2] - 1]
        assert 7.2 < w < 8.05
    finally:
        L.orc_set_quirk(1, 0)


def test_write_read_round_trip(tmp_path):
    ref = M.config1()
    ref.layup_angle = np.array([0.25])
    ref.section_orient = np.array([[[0.6, 0.8, 0.0], [-0.8, 0.6, 0.0], [0.0, 0.0, 1.0]]])
    p = tmp_path / "cfg1.yaml"
    IF.write_model_input(ref, p, node_sets={"tipNodes": [41, 82]}, point_loads=[(41, 3, 5.0)])
    mi = IF.read_model_input(p)
    m = mi.model()
    assert np.array_equal(m.node_list, ref.node_list)
    assert np.array_equal(m.element_list, ref.element_list)
    assert np.array_equal(m.element_section, ref.element_section)
    assert np.array_equal(m.layup_thickness, ref.layup_thickness) and np.array_equal(m.layup_angle, ref.layup_angle)
    assert np.allclose(m.section_orient, ref.section_orient, atol=1e-15)
    assert np.array_equal(m.material_elastic, ref.material_elastic)
    assert _eqset(m) == _eqset(ref)
    assert mi.node_sets["tipNodes"] == [41, 82] and mi.nodal_loads() == [(41, 3, 5.0)]


def test_scanner_rules(tmp_path):
    """Label ranges with steps, a single-node term repeated in every equation of a set-expanded
    block, DOF-7 terms kept apart, G derived for the last material only, the reference's nu
    formula, 'specificHeat:' read and 'specHeat:' not, scalar conductivity."""
    txt = """nodes:
    - [1, 0.0, 0.0, 0.0]
    - [2, 1.0, 0.0, 0.0]
    - [3, 1.0, 1.0, 0.0]
    - [4, 0.0, 1.0, 0.0]
    - [5, 2.0, 0.0, 0.0]
    - [6, 2.0, 1.0, 0.0]
elements:
    - type: shell4
      connectivity:
          - [1, 1, 2, 3, 4]
          - [2, 2, 5, 6, 3]
sets:
    node:
        - name: odd
          labels:
              - [1, 5, 2]
        - name: pair
          labels:
              - 2
              - 3
    element:
        - name: all2
          labels: all
sections:
    - type: shell
      orientation: [0.0, 0.0, 0.0, 0.0, 1.0, 0.0]
      layup:
          zOffset: 0.5
          layers:
              - [alu, 0.01, 0.0]
              - [steel, 0.02, 0.7]
      elementSet: all2
materials:
    - name: alu
      density: 2700
      elastic:
          E: 7e10
          nu: 0.33
          G: 2.6e10
      thermal:
          conductivity: 150
          specHeat: 900
    - name: steel
      density: 7800
      elastic:
          E: [2e11, 2.1e11, 2.2e11]
          nu: 0.3
      thermal:
          conductivity: [40, 41, 42, 1, 2, 3]
          specificHeat: 460
constraints:
    matrix:
        - [1, pair, 3, 1.0]
        - [1, 6, 3, -1.0]
        - [2, odd, 7, 1.0]
    rhs:
        - 0.5
        - 20.0
"""
    p = tmp_path / "t.yaml"
    p.write_text(txt)
    mi = IF.read_model_input(p)
    assert mi.node_sets["odd"] == [1, 3, 5]
    m = mi.model()
    # G was given in the block (for 'alu'), so the last material's G stays 0; nu scalar fills 3
    assert np.array_equal(m.material_elastic[1], [2e11, 2.1e11, 2.2e11, 0.3, 0.3, 0.3, 0, 0, 0])
    assert np.array_equal(m.material_elastic[0][6:], [2.6e10] * 3)
    assert m.sec_layup_range.tolist() == [0, 2] and m.layup_mat_id.tolist() == [1, 2]
    assert np.allclose(m.section_orient[0], np.eye(3)) and m.section_z_offset[0] == 0.5
    assert _eqset(m) == sorted([(((2, 3, 1.0), (6, 3, -1.0)), 0.5), (((3, 3, 1.0), (6, 3, -1.0)), 0.5)])
    cond, sh, (rng, nd, cf, rh) = mi.thermal()
    assert np.array_equal(cond[0], [150, 150, 150, 0, 0, 0]) and np.array_equal(cond[1], [40, 41, 42, 1, 2, 3])
    assert sh.tolist() == [0.0, 460.0]
    assert rng.tolist() == [0, 1, 2, 3] and nd.tolist() == [1, 3, 5] and rh.tolist() == [20.0] * 3
    # no G anywhere in the block: derived for the last material only; G without nu: 0.5 E/G + 1
    p.write_text(txt.replace("          G: 2.6e10\n", ""))
    e = IF.read_model_input(p).model().material_elastic
    assert e[0][6] == 0.0 and np.isclose(e[1][6], 0.5 * 2e11 / 1.3)
    p.write_text(txt.replace("          nu: 0.33\n", "").replace("          nu: 0.3\n", "          G: 8e10\n"))
    e = IF.read_model_input(p).model().material_elastic
    assert np.isclose(e[1][3], 0.5 * 2e11 / 8e10 + 1.0)


@pytest.mark.gpu
def test_read_model_solves_on_the_gpu():
    """The fixture's model through the C ABI: the static system matches the oracle's."""
    from misc_gb300.astro import AstroGPU
    mi = IF.read_model_input(FIX)
    m = mi.model()
    m.point_loads = mi.nodal_loads()
    g, o = AstroGPU(m), Oracle(m)
    g.getElasticSolnLoad(1, export=False)
    g.scaleElasticMPC()
    b = g.static_rhs()
    A, bo, *_ = o.static_system()
    assert np.linalg.norm(b - bo) <= 1e-13 * np.linalg.norm(bo)
    x = np.random.default_rng(0).standard_normal(o.n)
    assert np.linalg.norm(g.apply_operator(x, 64) - A @ x) <= 1e-12 * np.linalg.norm(A @ x)


def test_design_variable_input():
    """The reference's example design-variable file: a layup thickness variable and a layup
    modulus variable (E1 of layer 1, coefficient 2).  Both map to element categories; with values
    they move the oracle's element stiffness like a thicker, stiffer layer.  A category the
    library does not evaluate (thermal expansion) is refused in strict mode and left out
    otherwise."""
    mi = IF.read_model_input(FIX)
    dvs = IF.read_design_var_input(FIX.with_name("shell_beam_dvar_input.yaml"), mi)
    assert [(d["category"], d["subCategory"], d["layer"], d["component"]) for d in dvs] == \
        [("layup", "thickness", 1, 0), ("layup", "modulus", 1, 1)]
    assert dvs[0]["elements"] == list(range(1, 11)) and dvs[1]["coefficients"] == [2.0] * 10
    m = mi.model()
    kept = IF.apply_design_vars(m, dvs, values=[0.01, 5.0e9])
    assert kept == [1, 2]
    assert m.d_category.tolist() == [M.DCAT_LAYUP_THICKNESS, M.DCAT_LAYUP_MODULUS]
    assert m.d_component.tolist() == [1, 1] and m.d_layer.tolist() == [1, 1]
    assert m.el_to_d_range.tolist() == list(range(0, 21, 2)) and m.el_to_d.tolist() == [1, 2] * 10
    assert m.el_to_coef.tolist() == [1.0, 2.0] * 10
    ke = Oracle(m).element_matrices()
    m2 = mi.model()
    m2.layup_thickness = m2.layup_thickness + 0.01
    me = m2.material_elastic.copy()
    me[m2.layup_mat_id[0] - 1, 0] += 1.0e10
    m2.material_elastic = me
    assert np.allclose(ke, Oracle(m2).element_matrices(), rtol=1e-12, atol=1e-9 * np.abs(ke).max())
    extra = dict(category="thermalExp", subCategory="", component=1, layer=0, activeTime=[0.0, 0.0], elements=[1],
                 nodes=[], coefficients=[1.0])
    with pytest.raises(ValueError):
        IF.apply_design_vars(mi.model(), dvs + [extra])
    assert IF.apply_design_vars(mi.model(), dvs + [extra], strict=False) == [1, 2]


def test_node_design_variable_input(tmp_path):
    """nodeCoord and nodeLoad (elastic and thermal) variables over node sets, with the activity
    window of activeTime, become ndToD terms."""
    mi = IF.read_model_input(FIX)
    m = mi.model()
    name, nodes = next(iter(mi.node_sets.items()))
    f = tmp_path / "dv.yaml"
    f.write_text("designVariables:\n"
                 f"    - category: nodeCoord\n      component: 2\n      nodeSet: {name}\n      coefficients: 1.0\n"
                 f"    - category: nodeLoad\n      subCategory: thermal\n      activeTime: [0.5, 2.0]\n"
                 f"      nodeSet: {name}\n      coefficients: 3.0\n")
    dvs = IF.read_design_var_input(f, mi)
    assert IF.apply_design_vars(m, dvs, values=[0.0, 1.0]) == [1, 2]
    assert m.d_category.tolist() == [M.DCAT_NODE_COORD, M.DCAT_NODE_LOAD] and m.d_component.tolist() == [2, 7]
    assert m.d_act_time[1].tolist() == [0.5, 2.0]
    per = {nd: m.nd_to_d[m.nd_to_d_range[nd - 1]:m.nd_to_d_range[nd]].tolist() for nd in nodes}
    assert all(v == [1, 2] for v in per.values())
    o = Oracle(m)
    q = o.thermal_design_node_load(1.0)
    assert np.isclose(q.sum(), 3.0 * len(set(nodes)))
