"""GPU parity of the thermal design variables against the oracle, through the C ABI
(getdRthermaldD, Working/AStrO_commandFunctions.f90:1016-1170).

For every category on the thermal path (solid conductivity, specific heat, density, orientation
and node coordinates; shell layer conductivity, specific heat, density, thickness and angle, and
node coordinates), with nonzero real values of the variables:
* the thermal load and the reference CSR matrix at a (transient where the capacity enters) state:
  1e-12 relative;
* the complex step of the element residual, of the heat-generation load and of the surface-flux
  load: 1e-10 relative (the oracle's complex twin, pinned against central differences by the host
  tests);
* nodal 'nodeLoad' / 'thermal' variables: the applied heat input and its derivative, exact;
* the elastic residual's complex step of a thermal-only variable is zero.
"""
import numpy as np
import pytest

from misc_gb300 import model as M
from misc_gb300.astro import AstroGPU, thermal_props, thermal_state
from oracle import Oracle
from thermal_dvar_cases import CASES, flux_faces, heat_gen_elements, thermal_state as tstate, thermal_tables

pytestmark = pytest.mark.gpu

# nonzero real values per case (the variables' own values in the case builders are small or zero)
_VALUES = {"brick_node_coord": (0.02, -0.01), "shell_node_coord": (0.03, -0.02), "brick_orientation": (0.3, -0.2),
           "shell_layup_angle": (0.2, 0.1), "shell_layup_thickness": (0.003, 0.001)}


def _close(a, b, tol, what):
    nb = np.linalg.norm(b)
    assert np.linalg.norm(np.asarray(a) - b) <= tol * max(nb, 1e-300), (what, np.linalg.norm(np.asarray(a) - b), nb)


@pytest.mark.parametrize("case", sorted(CASES))
def test_thermal_design_matches_oracle(case):
    build, _, dyn = CASES[case]
    m = build()
    if case in _VALUES:
        m.d_value = np.array(_VALUES[case], np.float64)
    g, o = AstroGPU(m), Oracle(m)
    cond, sh = thermal_tables(m)
    g.thermal_setup(thermal_props(cond, sh))
    st = tstate(m.num_nodes, dyn)
    gst = thermal_state(st["temp"], st.get("prev_temp"), st.get("prev_tdot"), st.get("dynamic", 0), st.get("gamma", 0.5),
                        st.get("del_t", 0.0))
    load, mat, cols = g.getThermalSolnLoad(1, state=gst)
    oload, omat, ocols, _ = o.thermal_soln_load(cond, sh, 1, **st)
    assert np.array_equal(cols, ocols)
    _close(load, oload, 1e-12, "load")
    _close(mat, omat, 1e-12, "matrix")
    els = heat_gen_elements(m)
    fe, fn = flux_faces(m)
    scale = np.linalg.norm(oload)
    for dvar in (1, 2):
        d = g.thermal_drdd(dvar, 1e-14, state=gst)
        od = o.thermal_drdd(cond, sh, dvar, 1e-14, **st)
        assert np.linalg.norm(od) > 1e-6 * scale, (case, dvar)
        _close(d, od, 1e-10, (case, dvar, "element"))
        hg = g.thermal_heat_gen_drdd(dvar, 7.0, els)
        ohg = o.thermal_heat_gen_drdd(dvar, 7.0, els)
        # a load that does not depend on the variable (a rotation leaves a volume unchanged): both
        # sides at the rounding level of the load itself, 1e-12 of its norm
        assert np.linalg.norm(hg - ohg) <= max(1e-10 * np.linalg.norm(ohg),
                                               1e-12 * np.linalg.norm(o.thermal_heat_gen(7.0, els))), \
            (case, dvar, "heat generation")
        fl = g.thermal_surface_flux_drdd(dvar, fe, fn, 3.0)
        ofl = o.thermal_surface_flux_drdd(dvar, fe, fn, 3.0)
        assert np.linalg.norm(fl - ofl) <= max(1e-10 * np.linalg.norm(ofl),
                                               1e-12 * np.linalg.norm(o.thermal_surface_flux(fe, fn, 3.0))), \
            (case, dvar, "surface flux")


def test_thermal_node_loads_match_oracle():
    m = M.add_node_design_variables(M.hex_block(nx=3, ny=2, nz=2, seed=3), [[5, 9], [12]], M.DCAT_NODE_LOAD,
                                    component=7, value=3.0, act_time=(0.5, 2.0))
    g, o = AstroGPU(m), Oracle(m)
    cond, sh = thermal_tables(m)
    g.thermal_setup(thermal_props(cond, sh))
    for t in (0.2, 1.0, 3.0):
        assert np.array_equal(g.thermal_design_node_load(t), o.thermal_design_node_load(t)), t
        for d in (1, 2):
            assert np.array_equal(g.thermal_node_load_drdd(d, t), o.thermal_node_load_drdd(d, t)), (t, d)
    assert not np.any(g.design_node_load(1.0))


def test_elastic_complex_step_of_thermal_variable_is_zero():
    build, _, _ = CASES["brick_thermal_cond_k11"]
    m = build()
    g = AstroGPU(m)
    dr, _ = g.getdRelasticdD(1, h=1e-30, state=M.make_state(g.n, disp=1e-3 * np.ones(g.n)))
    assert not np.any(dr)
