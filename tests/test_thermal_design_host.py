"""Thermal design variables in the CPU oracle (getdRthermaldD, Working/AStrO_commandFunctions.f90:
1016-1170): the complex-step derivatives of the element residual, of the heat-generation and
surface-flux loads and of the nodal heat inputs against central differences of the oracle's own
real loads (1e-5 relative: the complex path's single-precision Gauss points), and the real values
of the property variables against the same model with its material table changed."""
import numpy as np
import pytest

from misc_gb300 import model as M
from oracle import Oracle
from thermal_dvar_cases import CASES, flux_faces, heat_gen_elements, thermal_state, thermal_tables


def _fd(build, dvar, step, fn):
    out = []
    for sgn in (1.0, -1.0):
        m = build()
        m.d_value = m.d_value.copy()
        m.d_value[dvar - 1] += sgn * step
        out.append(fn(Oracle(m), m))
    return (out[0] - out[1]) / (2 * step)


def _close(cs, fd, tol, what, scale):
    """cs against fd at tol relative; a derivative below 1e-6 of the load's own norm (scale) is a
    zero one (a rotation does not change a volume), where both sides must stay below that floor."""
    if np.linalg.norm(fd) <= 1e-6 * scale:
        assert np.linalg.norm(cs) <= 1e-6 * scale, what
        return
    assert np.linalg.norm(cs - fd) <= tol * np.linalg.norm(fd), (what, np.linalg.norm(cs - fd) / np.linalg.norm(fd))


@pytest.mark.parametrize("case", sorted(CASES))
def test_thermal_complex_step_matches_central_difference(case):
    build, step, dyn = CASES[case]
    m0 = build()
    o = Oracle(m0)
    cond, sh = thermal_tables(m0)
    st = thermal_state(m0.num_nodes, dyn)
    els = heat_gen_elements(m0)
    fe, fn = flux_faces(m0)
    nonzero = 0
    for dvar in (1, 2):
        cs = o.thermal_drdd(cond, sh, dvar, 1e-14, **st)
        fd = -_fd(build, dvar, step, lambda oo, m: oo.thermal_soln_load(cond, sh, 0, **st)[0])
        scale = np.linalg.norm(o.thermal_soln_load(cond, sh, 0, **st)[0])
        _close(cs, fd, 1e-5, (case, dvar, "element"), scale)
        nonzero += np.linalg.norm(fd) > 1e-6 * scale
        cs = o.thermal_heat_gen_drdd(dvar, 7.0, els)
        fd = -_fd(build, dvar, step, lambda oo, m: oo.thermal_heat_gen(7.0, els))
        _close(cs, fd, 1e-5, (case, dvar, "heat generation"), np.linalg.norm(o.thermal_heat_gen(7.0, els)))
        cs = o.thermal_surface_flux_drdd(dvar, fe, fn, 3.0)
        fd = -_fd(build, dvar, step, lambda oo, m: oo.thermal_surface_flux(fe, fn, 3.0))
        _close(cs, fd, 1e-5, (case, dvar, "surface flux"), np.linalg.norm(o.thermal_surface_flux(fe, fn, 3.0)))
    assert nonzero, case


def test_thermal_property_values_match_material_table():
    """Real values of conductivity, specific-heat and density variables are the material table
    changed by them (each brick of the block has its own material): identical loads."""
    from thermal_dvar_cases import brick, with_element_dvars
    m = brick()
    E = m.num_els
    a, b = list(range(1, E // 2 + 1)), list(range(E // 2 + 1, E + 1))
    with_element_dvars(m, [(M.DCAT_THERMAL_COND, 1, 0, 2.0, a), (M.DCAT_THERMAL_COND, 4, 0, 0.5, b),
                           (M.DCAT_SPEC_HEAT, 0, 0, 10.0, a), (M.DCAT_DENSITY, 0, 0, 50.0, b)])
    cond, sh = thermal_tables(m)
    st = thermal_state(m.num_nodes, True)
    load, mat, cols, _ = Oracle(m).thermal_soln_load(cond, sh, 1, **st)
    m2 = brick()
    c2, s2, rho2 = cond.copy(), sh.copy(), m2.material_density.copy()
    mat_of = m2.section_mat_id[m2.element_section - 1]
    for e in a:
        c2[mat_of[e - 1] - 1, 0] += 2.0
        s2[mat_of[e - 1] - 1] += 10.0
    for e in b:
        c2[mat_of[e - 1] - 1, 3] += 0.5
        rho2[mat_of[e - 1] - 1] += 50.0
    m2.material_density = rho2
    load2, mat2, cols2, _ = Oracle(m2).thermal_soln_load(c2, s2, 1, **st)
    assert np.array_equal(cols, cols2)
    assert np.allclose(load, load2, rtol=1e-14, atol=1e-12 * np.abs(load2).max())
    assert np.allclose(mat, mat2, rtol=1e-14, atol=1e-14 * np.abs(mat2).max())


def test_thermal_node_load_design_variables():
    """'nodeLoad' / 'thermal' variables (component 7): the nodal heat input is linear in them
    inside their window and absent outside it; the derivative branch is minus the input per unit
    variable; elastic nodal loads ignore them."""
    m = M.add_node_design_variables(M.hex_block(nx=3, ny=2, nz=2, seed=3), [[5, 9], [12]], M.DCAT_NODE_LOAD,
                                    component=7, value=3.0, act_time=(0.5, 2.0))
    o = Oracle(m)
    q = o.thermal_design_node_load(1.0)
    expect = np.zeros(m.num_nodes)
    for nd in (5, 9, 12):
        expect[o.current_rank[nd - 1] - 1] += 3.0
    assert np.array_equal(q, expect)
    assert not np.any(o.thermal_design_node_load(3.0))
    dr = o.thermal_node_load_drdd(1, 1.0)
    e1 = np.zeros(m.num_nodes)
    for nd in (5, 9):
        e1[o.current_rank[nd - 1] - 1] = -1.0
    assert np.allclose(dr, e1, rtol=0, atol=1e-12)
    assert not np.any(o.design_node_load(1.0))
