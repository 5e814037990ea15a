"""Model input reader: AStrO's YAML-subset model files (readModelInput,
Working/AStrO_input.f90:27-1091) into the arrays of the C ABI's astro_model, plus the parts of
the file the model struct does not carry (sets, loads, initial state, thermal material data).

The reference does not parse YAML: it scans the file line by line and recognises a field by the
keyword that ends at the line's colon ('nodes:', 'type:', 'labels:', ...), reading list entries
from the text between '[' and ']' or after '-'.  This reader follows that scanner's rules,
including what it does with input the template describes but the scanner never reads:
  * labels index the arrays directly (node and element labels are 1..count);
  * a set's 'labels:' is 'all', a list of labels, or ranges [first, last(, step)];
  * materials: scalar E / nu / G fill all three components; when G (or nu) is missing it is
    derived after the whole 'materials:' block, for the last material only, as E/(2(1+nu)) (or
    0.5 E/G + 1, the reference's formula); 'specificHeat:' is read ('specHeat:' is not);
  * section orientation [x1 x2 x3 xy1 xy2 xy3]: rows x = x/|x|, z = x cross xy / |.|, y = z cross x
    (identity when |x| < 1e-12); layer angles are taken as written;
  * constraints: terms [eqn, node-or-set, dof, coef]; an equation whose terms name sets expands to
    one equation per set member (a one-node set or a single node repeats in every one), for the
    structural DOF 1..6 (buildElasticMPC) and separately for the temperature DOF 7
    (buildThermalMPC, Working/AStrO_bookKeeping.f90:474-752).
"""
from __future__ import annotations

import re
from dataclasses import dataclass, field

import numpy as np

from .model import Model

_TOP = ("nodes:", "elements:", "sets:", "sections:", "materials:", "constraints:", "loads:", "initialState:")
_ELTYPES = (("tet4", 4, 4), ("wedge6", 6, 6), ("brick8", 8, 8), ("brickIM", 8, 81), ("shell3", 3, 3),
            ("shell4", 4, 41), ("beam2", 2, 2))
# setLoads values read per load type (the rest take 7)
_LOAD_NVALS = {"gravitational": 3, "surfacePressure": 5, "bodyHeatGen": 1, "surfaceFlux": 5}


def _key(line):
    """The keyword ending at the line's first colon ('' when there is none)."""
    i = line.find(":")
    if i < 0:
        return ""
    m = re.search(r"([A-Za-z0-9_]+)$", line[:i])
    return (m.group(1) + ":") if m else ":"


def _after(line):
    return line[line.find(":") + 1:].strip()


def _bracket(line):
    i, j = line.find("["), line.find("]")
    if i < 0 or j < 0:
        return None
    return [t for t in re.split(r"[,\s]+", line[i + 1:j].strip()) if t]


def _num(t):
    return float(t.replace("d", "e").replace("D", "e"))


@dataclass
class ModelInput:
    num_nodes: int = 0
    num_els: int = 0
    nodes: np.ndarray = None                 # (N, 3)
    elements: np.ndarray = None              # (E, 8), 0-padded
    element_type: np.ndarray = None          # (E,)
    node_sets: dict = field(default_factory=dict)     # name -> 1-based labels
    element_sets: dict = field(default_factory=dict)
    sections: list = field(default_factory=list)      # dicts: type, material, orientation, zOffset, layers, elementSet
    element_section: np.ndarray = None
    materials: list = field(default_factory=list)     # dicts: name, density, elastic(9), stiffness(21),
                                                      # conductivity(6), expansion(6), specHeat
    mpc_terms: list = field(default_factory=list)     # (eqn, node-or-set, dof, coef)
    mpc_rhs: list = field(default_factory=list)
    loads: list = field(default_factory=list)         # dicts: type, activeTime(2), rows [(target, values)]
    initial: dict = field(default_factory=dict)       # displacement/velocity/acceleration (N,6), temperature, tdot (N,)

    # -- derived arrays ----------------------------------------------------------------------
    def _material_id(self, name):
        ids = [k + 1 for k, m in enumerate(self.materials) if m["name"] == name]
        return ids[-1] if ids else 0

    def _node_list_of(self, target):
        """Nodes named by a constraint or load target: a label or a node set."""
        try:
            return [int(float(target))], True
        except ValueError:
            return list(self.node_sets.get(target, [])), False

    def expanded_equations(self, dofs):
        """Equations over the given DOF set expanded per set member: [(terms [(node, dof, coef)], rhs)]."""
        neq = max([t[0] for t in self.mpc_terms], default=0)
        out = []
        for e in range(1, neq + 1):
            terms = [t for t in self.mpc_terms if t[0] == e and t[2] in dofs]
            if not terms:
                continue
            lists = [self._node_list_of(t[1]) for t in terms]
            n_eq = max([1 if single else len(nl) for nl, single in lists], default=0)
            rows = [[] for _ in range(n_eq)]
            for (eq, tgt, dof, coef), (nl, single) in zip(terms, lists):
                if single or len(nl) == 1:
                    for r in rows:
                        r.append((nl[0], dof, coef))
                else:
                    for i, nd in enumerate(nl[:n_eq]):
                        rows[i].append((nd, dof, coef))
            rhs = self.mpc_rhs[e - 1] if e - 1 < len(self.mpc_rhs) else 0.0
            out += [(r, rhs) for r in rows]
        return out

    def model(self, name="input") -> Model:
        """astro_model arrays (structural constraints expanded; solid sections take their
        material, shell sections their layup)."""
        S = len(self.sections)
        orient = np.zeros((max(S, 1), 3, 3))
        lay_range, lay_mat, lay_t, lay_a, zoff, sec_mat = [0], [], [], [], np.zeros(max(S, 1)), np.zeros(max(S, 1), np.int32)
        for s, sec in enumerate(self.sections):
            orient[s] = _orient(sec.get("orientation"))
            zoff[s] = sec.get("zOffset", 0.0)
            sec_mat[s] = self._material_id(sec.get("material", ""))
            for mat, t, a in sec.get("layers", []):
                lay_mat.append(self._material_id(mat))
                lay_t.append(t)
                lay_a.append(a)
            lay_range.append(len(lay_mat))
        mats = self.materials or [dict(elastic=np.zeros(9), density=0.0)]
        m = Model(node_list=self.nodes.copy(), element_list=self.elements.copy(),
                  element_type=self.element_type.copy(), element_section=self.element_section.copy(),
                  section_mat_id=sec_mat, section_orient=orient, sec_layup_range=np.array(lay_range, np.int32),
                  layup_mat_id=np.array(lay_mat, np.int32), layup_thickness=np.array(lay_t, np.float64),
                  layup_angle=np.array(lay_a, np.float64), section_z_offset=zoff,
                  material_elastic=np.array([mt["elastic"] for mt in mats], np.float64),
                  material_density=np.array([mt["density"] for mt in mats], np.float64), name=name)
        eqs = self.expanded_equations(range(1, 7))
        rng, nd, df, cf, rh = [0], [], [], [], []
        for terms, rhs in eqs:
            for (n_, d_, c_) in terms:
                nd.append(n_)
                df.append(d_)
                cf.append(c_)
            rng.append(len(nd))
            rh.append(rhs)
        m.mpc_range, m.mpc_node = np.array(rng, np.int32), np.array(nd, np.int32)
        m.mpc_dof, m.mpc_coef, m.mpc_rhs = np.array(df, np.int32), np.array(cf, np.float64), np.array(rh, np.float64)
        m.face_el = np.zeros(0, np.int32)
        m.face_num = np.zeros(0, np.int32)
        return m

    def thermal(self):
        """(conductivity (M, 6), specific heat (M,), temperature constraints (range, node, coef,
        rhs)) for astro_thermal_props."""
        mats = self.materials
        cond = np.array([mt["conductivity"] for mt in mats], np.float64)
        sh = np.array([mt["specHeat"] for mt in mats], np.float64)
        eqs = self.expanded_equations((7,))
        rng, nd, cf, rh = [0], [], [], []
        for terms, rhs in eqs:
            for (n_, d_, c_) in terms:
                nd.append(n_)
                cf.append(c_)
            rng.append(len(nd))
            rh.append(rhs)
        return cond, sh, (np.array(rng, np.int32), np.array(nd, np.int32), np.array(cf), np.array(rh))

    def nodal_loads(self, time=0.0):
        """'nodal' loads active at time: [(node, dof 1..7, value)] (dof 7 = heat)."""
        out = []
        for ld in self.loads:
            if ld["type"] != "nodal" or not (ld["activeTime"][0] <= time <= ld["activeTime"][1]):
                continue
            for tgt, vals in ld["rows"]:
                nl, _ = self._node_list_of(tgt)
                for nd in nl:
                    for k in range(7):
                        if vals[k] != 0.0:
                            out.append((nd, k + 1, vals[k]))
        return out


def _orient(v):
    if v is None:
        return np.eye(3)
    v1, v2 = np.array(v[:3], np.float64), np.array(v[3:6], np.float64)
    mag = np.sqrt(v1 @ v1)
    if mag < 1e-12:
        return np.eye(3)
    v1 = (1.0 / mag) * v1
    v3 = np.cross(v1, v2)
    v3 = (1.0 / np.sqrt(v3 @ v3)) * v3
    v2 = np.cross(v3, v1)
    return np.array([v1, v2, v3])


def _labels(lines, i, total):
    """A set's labels starting after its 'labels:' line i: (labels, next line index)."""
    head = _after(lines[i])
    if "all" in head:
        return list(range(1, total + 1)), i + 1
    out = []
    i += 1
    while i < len(lines) and ":" not in lines[i]:
        b = _bracket(lines[i])
        if b is not None:
            # [first, last(, step)] over the defaults (1, 0, 1), as a Fortran DO loop
            v = [1, 0, 1]
            for j, x in enumerate(b[:3]):
                v[j] = int(float(x))
            first, last, step = v
            if step:
                out += list(range(first, last + (1 if step > 0 else -1), step))
        elif "-" in lines[i]:
            out.append(int(float(lines[i].split("-", 1)[1].split()[0])))
        i += 1
    return out, i


def read_model_input(path) -> ModelInput:
    with open(path) as f:
        lines = [ln.rstrip("\n").replace("\t", "    ") for ln in f]
    lines = [ln.split("#", 1)[0] for ln in lines]
    mi = ModelInput()
    # first pass: counts (the reference sizes its arrays from the entries it finds)
    nn = ne = 0
    block = ""
    for ln in lines:
        k = _key(ln)
        if k in _TOP:
            block = k
        elif block == "nodes:" and not k and "[" in ln:
            nn = max(nn, int(float(_bracket(ln)[0])))
        elif block == "elements:" and not k and "[" in ln:
            ne = max(ne, int(float(_bracket(ln)[0])))
    mi.num_nodes, mi.num_els = nn, ne
    mi.nodes = np.zeros((nn, 3))
    mi.elements = np.zeros((ne, 8), np.int32)
    mi.element_type = np.zeros(ne, np.int32)
    mi.element_section = np.zeros(ne, np.int32)
    mi.initial = {k: np.zeros((nn, 6)) for k in ("displacement", "velocity", "acceleration")}
    mi.initial.update(temperature=np.zeros(nn), tdot=np.zeros(nn))
    i = 0
    block = ""
    nnd, etype = 0, 0
    in_el_set = False
    set_name = None
    mat = None
    mat_g = mat_nu = False
    load = None
    ini = None
    while i < len(lines):
        ln = lines[i]
        k = _key(ln)
        if k in _TOP:
            if block == "materials:" and mi.materials:
                _finish_materials(mi.materials[-1], mat_g, mat_nu)
            block, i = k, i + 1
            mat_g = mat_nu = False
            continue
        if block == "nodes:":
            b = _bracket(ln) if not k else None
            if b and "-" in ln:
                lab = int(float(b[0]))
                if lab <= nn:
                    mi.nodes[lab - 1] = [_num(x) for x in b[1:4]]
        elif block == "elements:":
            if k == "type:":
                t = _after(ln)
                for name, cnt, code in _ELTYPES:
                    if name in t:
                        nnd, etype = cnt, code
                        break
            elif not k and "[" in ln:
                b = [int(float(x)) for x in _bracket(ln)]
                if b[0] <= ne:
                    mi.elements[b[0] - 1, :nnd] = b[1:nnd + 1]
                    mi.element_type[b[0] - 1] = etype
        elif block == "sets:":
            if k == "node:":
                in_el_set = False
            elif k == "element:":
                in_el_set = True
            elif k == "name:":
                set_name = _after(ln).split()[0]
            elif k == "labels:":
                labs, i = _labels(lines, i, ne if in_el_set else nn)
                (mi.element_sets if in_el_set else mi.node_sets)[set_name] = labs
                continue
        elif block == "sections:":
            if k == "type:":
                mi.sections.append(dict(type=_after(ln).split()[0], layers=[]))
            elif mi.sections:
                sec = mi.sections[-1]
                if k == "material:":
                    sec["material"] = _after(ln).split()[0]
                elif k == "orientation:":
                    sec["orientation"] = [_num(x) for x in _bracket(ln)[:6]]
                elif k == "zOffset:":
                    sec["zOffset"] = _num(_after(ln).split()[0])
                elif k == "layers:":
                    i += 1
                    while i < len(lines) and ":" not in lines[i]:
                        b = _bracket(lines[i])
                        if b:
                            sec["layers"].append((b[0], _num(b[1]), _num(b[2])))
                        i += 1
                    continue
                elif k == "elementSet:":
                    nm = _after(ln).split()[0]
                    sec["elementSet"] = nm
                    for e in mi.element_sets.get(nm, []):
                        mi.element_section[e - 1] = len(mi.sections)
        elif block == "materials:":
            if k == "name:":
                mi.materials.append(dict(name=_after(ln).split()[0], density=0.0, elastic=np.zeros(9),
                                         stiffness=np.zeros(21), conductivity=np.zeros(6), expansion=np.zeros(6),
                                         specHeat=0.0))
            elif mi.materials:
                mt = mi.materials[-1]
                b = _bracket(ln)
                if k == "density:":
                    mt["density"] = _num(_after(ln).split()[0])
                elif k in ("E:", "nu:", "G:"):
                    o = {"E:": 0, "nu:": 3, "G:": 6}[k]
                    vals = [_num(x) for x in b[:3]] if b else [_num(_after(ln).split()[0])] * 3
                    mt["elastic"][o:o + 3] = vals
                    mat_nu |= k == "nu:"
                    mat_g |= k == "G:"
                elif k == "stiffness:":
                    mt["stiffness"][:] = [_num(x) for x in b[:21]]
                elif k in ("conductivity:", "expansion:"):
                    key = k[:-1]
                    if b:
                        mt[key][:] = [_num(x) for x in b[:6]]
                    else:
                        v = _num(_after(ln).split()[0])
                        mt[key][:] = [v, v, v, 0.0, 0.0, 0.0]
                elif k == "specificHeat:":
                    mt["specHeat"] = _num(_after(ln).split()[0])
        elif block == "constraints:":
            if k == "matrix:":
                i += 1
                while i < len(lines) and ":" not in lines[i]:
                    b = _bracket(lines[i])
                    if b:
                        mi.mpc_terms.append((int(float(b[0])), b[1], int(float(b[2])), _num(b[3])))
                    i += 1
                continue
            if k == "rhs:":
                i += 1
                while i < len(lines) and ":" not in lines[i]:
                    if "-" in lines[i]:
                        mi.mpc_rhs.append(_num(lines[i].split("-", 1)[1].split()[0]))
                    i += 1
                continue
        elif block == "loads:":
            if k == "type:":
                load = dict(type=_after(ln).split()[0], activeTime=[0.0, 0.0], rows=[])
                mi.loads.append(load)
            elif load is not None and k == "activeTime:":
                b = _bracket(ln)
                load["activeTime"] = [_num(b[0]), _num(b[1])] if b else [_num(_after(ln).split()[0]), 1e100]
            elif load is not None and k == "setLoads:":
                nv = _LOAD_NVALS.get(load["type"], 7)
                i += 1
                while i < len(lines) and ":" not in lines[i]:
                    b = _bracket(lines[i])
                    if b:
                        vals = np.zeros(7)
                        vals[:nv] = [_num(x) for x in b[1:nv + 1]]
                        load["rows"].append((b[0], vals))
                    i += 1
                continue
        elif block == "initialState:":
            if k in ("displacement:", "velocity:", "acceleration:", "temperature:", "tempChangeRate:"):
                ini = {"tempChangeRate:": "tdot"}.get(k, k[:-1])
                i += 1
                while i < len(lines) and ":" not in lines[i]:
                    b = _bracket(lines[i])
                    if b:
                        nl, _ = mi._node_list_of(b[0])
                        for nd in nl:
                            if ini in ("temperature", "tdot"):
                                mi.initial[ini][nd - 1] = _num(b[1])
                            else:
                                mi.initial[ini][nd - 1] = [_num(x) for x in b[1:7]]
                    i += 1
                continue
        i += 1
    if block == "materials:" and mi.materials:
        _finish_materials(mi.materials[-1], mat_g, mat_nu)
    return mi


def _finish_materials(mt, g_set, nu_set):
    """After the 'materials:' block, for its last material (the reference's flags are per block)."""
    e = mt["elastic"]
    if not g_set:
        e[6] = 0.5 * e[0] / (1.0 + e[3])
        e[7:9] = e[6]
    elif not nu_set:
        e[3] = 0.5 * e[0] / e[6] + 1.0
        e[4:6] = e[3]


def write_model_input(m: Model, path, node_sets=None, point_loads=None):
    """Writes a model in the reference's input layout (the inverse of read_model_input for what
    astro_model holds): nodes, elements by type, one element set and one section per model
    section, materials (E, nu, G as given), single-node constraint terms, nodal loads."""
    _r = lambda v: repr(float(v))
    names = {4: "tet4", 6: "wedge6", 8: "brick8", 81: "brickIM", 3: "shell3", 41: "shell4", 2: "beam2"}
    counts = {4: 4, 6: 6, 8: 8, 81: 8, 3: 3, 41: 4, 2: 2}
    out = ["nodes:"]
    for i, x in enumerate(m.node_list):
        out.append(f"    - [{i + 1}, {_r(x[0])}, {_r(x[1])}, {_r(x[2])}]")
    out.append("elements:")
    for t in sorted(set(int(v) for v in m.element_type)):
        out += [f"    - type: {names[t]}", "      connectivity:"]
        for e in np.nonzero(m.element_type == t)[0]:
            nd = ", ".join(str(int(v)) for v in m.element_list[e, :counts[t]])
            out.append(f"          - [{e + 1}, {nd}]")
    out += ["sets:", "    node:"]
    for nm, labs in (node_sets or {}).items():
        out += [f"        - name: {nm}", "          labels:"] + [f"              - {int(v)}" for v in labs]
    out.append("    element:")
    S = len(m.section_mat_id)
    for s in range(S):
        els = np.nonzero(m.element_section == s + 1)[0] + 1
        out += [f"        - name: sec{s + 1}Els", "          labels:"] + [f"              - {int(v)}" for v in els]
    out.append("sections:")
    shell = bool(np.any(m.element_type == 41))
    for s in range(S):
        o = np.asarray(m.section_orient[s])
        out += [f"    - type: {'shell' if shell else 'solid'}"]
        if not shell:
            out.append(f"      material: mat{int(m.section_mat_id[s])}")
        out.append(f"      orientation: [{_r(o[0, 0])}, {_r(o[0, 1])}, {_r(o[0, 2])}, {_r(o[1, 0])}, {_r(o[1, 1])}, {_r(o[1, 2])}]")
        if shell:
            out += ["      layup:", f"          zOffset: {_r(float(m.section_z_offset[s]))}", "          layers:"]
            for li in range(m.sec_layup_range[s], m.sec_layup_range[s + 1]):
                out.append(f"              - [mat{int(m.layup_mat_id[li])}, {_r(float(m.layup_thickness[li]))}, "
                           f"{_r(float(m.layup_angle[li]))}]")
        out.append(f"      elementSet: sec{s + 1}Els")
    out.append("materials:")
    for k, e in enumerate(m.material_elastic):
        out += [f"    - name: mat{k + 1}", f"      density: {_r(float(m.material_density[k]))}", "      elastic:",
                f"          E: [{_r(e[0])}, {_r(e[1])}, {_r(e[2])}]", f"          nu: [{_r(e[3])}, {_r(e[4])}, {_r(e[5])}]",
                f"          G: [{_r(e[6])}, {_r(e[7])}, {_r(e[8])}]"]
    if len(m.mpc_range) > 1:
        out += ["constraints:", "    matrix:"]
        for r in range(len(m.mpc_range) - 1):
            for t in range(m.mpc_range[r], m.mpc_range[r + 1]):
                out.append(f"        - [{r + 1}, {int(m.mpc_node[t])}, {int(m.mpc_dof[t])}, {_r(float(m.mpc_coef[t]))}]")
        out.append("    rhs:")
        out += [f"        - {_r(float(v))}" for v in m.mpc_rhs]
    if point_loads:
        out += ["loads:", "    - type: nodal", "      activeTime: 0.0", "      setLoads:"]
        for nd, dof, v in point_loads:
            vals = [0.0] * 7
            vals[dof - 1] = float(v)
            out.append(f"          - [{int(nd)}, " + ", ".join(_r(x) for x in vals) + "]")
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")


# design-variable categories (astro_model d_category): (category, subCategory) -> (d_category,
# component offset, node category).  The reference's property routines
# (Working/AStrO_r_designPropertyFunctions.f90) select on these names: 'elastic' modulus /
# poissonRatio / shearModulus index eProps (component, + 3, + 6; :46-53), the shell layer's
# modulus / poissonRatio / shearModulus index layerProps (component, 3, 4; :292-298), and
# 'nodeLoad' / 'thermal' is ndLd(7) (:986-987).
_DCAT = {
    ("layup", "thickness"): (1, 0, False), ("elastic", "modulus"): (2, 0, False),
    ("elastic", "poissonRatio"): (2, 3, False), ("elastic", "shearModulus"): (2, 6, False),
    ("density", ""): (3, 0, False), ("orientation", ""): (4, 0, False), ("layup", "zOffset"): (5, 0, False),
    ("layup", "angle"): (6, 0, False), ("layup", "density"): (7, 0, False), ("nodeCoord", ""): (8, 0, True),
    ("nodeLoad", "elastic"): (9, 0, True), ("nodeLoad", "thermal"): (9, None, True),
    ("thermalCond", ""): (10, 0, False), ("specHeat", ""): (11, 0, False), ("layup", "thermalCond"): (12, 0, False),
    ("layup", "specHeat"): (13, 0, False), ("layup", "modulus"): (14, 0, False),
    ("layup", "poissonRatio"): (14, None, False), ("layup", "shearModulus"): (14, None, False),
}
# fixed components of the entries marked None above
_FIXED_COMP = {("nodeLoad", "thermal"): 7, ("layup", "poissonRatio"): 3, ("layup", "shearModulus"): 4}


def _dcat(dv):
    """(d_category, d_component, node category) of one design variable, or None."""
    key = (dv["category"], dv["subCategory"])
    if key not in _DCAT:
        return None
    cat, off, node = _DCAT[key]
    comp = _FIXED_COMP[key] if off is None else max(dv["component"], 1) + off
    return cat, comp, node


def read_design_var_input(path, mi: ModelInput):
    """readDesignVarInput (Working/AStrO_input.f90:1099-1408): one entry per 'category:' with its
    subCategory, component, layer, activeTime, the element (or node) set it acts on and its
    coefficients (one value for every member, or a list).  Returns a list of dicts."""
    with open(path) as f:
        lines = [ln.rstrip("\n").replace("\t", "    ").split("#", 1)[0] for ln in f]
    dvs = []
    i = 0
    while i < len(lines):
        ln = lines[i]
        k = _key(ln)
        dv = dvs[-1] if dvs else None
        if k == "category:":
            dvs.append(dict(category=_after(ln).split()[0], subCategory="", component=0, layer=0,
                            activeTime=[0.0, 0.0], elements=[], nodes=[], coefficients=None))
        elif dv is not None and k == "subCategory:":
            dv["subCategory"] = _after(ln).split()[0]
        elif dv is not None and k in ("component:", "layer:"):
            dv[k[:-1]] = int(float(_after(ln).split()[0]))
        elif dv is not None and k == "activeTime:":
            b = _bracket(ln)
            dv["activeTime"] = [_num(b[0]), _num(b[1])] if b else [_num(_after(ln).split()[0]), 1e100]
        elif dv is not None and k == "elementSet:":
            dv["elements"] += list(mi.element_sets.get(_after(ln).split()[0], []))
        elif dv is not None and k == "nodeSet:":
            dv["nodes"] += list(mi.node_sets.get(_after(ln).split()[0], []))
        elif dv is not None and k == "coefficients:":
            head = _after(ln)
            members = len(dv["elements"]) or len(dv["nodes"])
            if head:
                dv["coefficients"] = [_num(head.split()[0])] * members
            else:
                cs = []
                i += 1
                while i < len(lines) and ":" not in lines[i]:
                    if "-" in lines[i]:
                        cs.append(_num(lines[i].split("-", 1)[1].split()[0]))
                    i += 1
                dv["coefficients"] = (cs + [1.0] * members)[:members]
                continue
        i += 1
    for dv in dvs:
        if dv["coefficients"] is None:
            dv["coefficients"] = [1.0] * (len(dv["elements"]) or len(dv["nodes"]))
    return dvs


def apply_design_vars(m: Model, dvs, values=None, strict=True):
    """Attaches the design variables to m: element categories as elToD / elToCoef (per element,
    the variables in input order, an element listed twice for one variable kept once), node
    categories (nodeCoord, nodeLoad) as ndToD / ndToCoef over their node sets, with the activity
    window of activeTime.  Categories the library does not evaluate raise (strict) or are left
    out; returns the input numbers (1-based) of the variables kept."""
    keep, cats = [], []
    for k, dv in enumerate(dvs):
        c = _dcat(dv)
        if c is None:
            if strict:
                raise ValueError(f"design variable {k + 1}: {dv['category']}/{dv['subCategory']} is not evaluated "
                                 f"by the device complex step")
            continue
        keep.append(k)
        cats.append(c)
    E, N = m.num_els, m.num_nodes
    per_el = [[] for _ in range(E)]
    per_nd = [[] for _ in range(N)]
    for j, (k, (_, _, node)) in enumerate(zip(keep, cats)):
        dv = dvs[k]
        members, lists = (dv["nodes"], per_nd) if node else (dv["elements"], per_el)
        for x, c in zip(members, dv["coefficients"]):
            if all(d != j + 1 for d, _ in lists[x - 1]):
                lists[x - 1].append((j + 1, c))
    m.el_to_d_range = np.cumsum([0] + [len(p) for p in per_el]).astype(np.int32)
    m.el_to_d = np.array([d for p in per_el for d, _ in p], np.int32)
    m.el_to_coef = np.array([c for p in per_el for _, c in p], np.float64)
    if any(node for _, _, node in cats):
        m.nd_to_d_range = np.cumsum([0] + [len(p) for p in per_nd]).astype(np.int32)
        m.nd_to_d = np.array([d for p in per_nd for d, _ in p], np.int32)
        m.nd_to_coef = np.array([c for p in per_nd for _, c in p], np.float64)
        m.d_act_time = np.array([dvs[k]["activeTime"] for k in keep], np.float64).reshape(-1, 2)
    m.d_category = np.array([c[0] for c in cats], np.int32)
    m.d_component = np.array([c[1] for c in cats], np.int32)
    m.d_layer = np.array([max(dvs[k]["layer"], 1) for k in keep], np.int32)
    m.d_value = np.zeros(len(keep)) if values is None else np.asarray(values, np.float64)[keep]
    return [k + 1 for k in keep]
