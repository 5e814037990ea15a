"""Job scripts: AStrO_runJob (Working/AStrO_runJob.f90) on the device.

A job script is a list of '*command' blocks with 'key: value' lines (Working/ScriptCommands.txt).
This runner reads the model (and design-variable) inputs with misc_gb300.inputfile, builds the
loads of the model file with the device entry points, runs the solves of '*solve' through the C
ABI and writes '*writeNodeResults' files in the reference's layout (writeNodeResults,
Working/AStrO_output.f90:10-152: 'time:', 'timeStep:', then per field '    - [node, values]').

Supported: *readModelInput, *readDesignVarInput (the categories the device complex step
evaluates), *solve (elastic static, linear or nonlinear geometry; elastic Newmark dynamics;
steady and transient thermal), *writeNodeResults (temperature, tdot, displacement, velocity,
acceleration, reactionForce, reactionHeatGen).  Other commands (*modalAnalysis, objectives, element results)
are logged as not run.

Loads of the model file, at a time t (a load acts when activeTime[0] <= t <= activeTime[1]):
nodal forces and heat, bodyForce / gravitational / centrifugal (astro_body_load), surfacePressure
/ surfaceTraction / surfaceFlux on the element faces whose outward normal lies within thetaTol
degrees of the given direction (r_getElSurfaceTraction's test, Working/AStrO_r_elementEqns.f90:
1923-2018; faces of r_getElementFaces, exterior faces only for bricks, both faces of a shell) and
bodyHeatGen (astro_thermal_heat_gen).  Solvers: the FP64 Jacobi-GMRES for bricks and the learned
FGMRES for shells, each to 1e-10 relative FP64 residual, inside the device Newton loop of
stepSolve; the Newmark loop runs on the device, split into segments where the set of active loads
changes.
"""
from __future__ import annotations

import math
from pathlib import Path

import numpy as np

from . import inputfile as IF
from .astro import (SOLVER_FGMRES_LEARNED, SOLVER_GMRES_JACOBI_FP64, AstroGPU, make_state, thermal_props,
                    thermal_state, write_step_file)

# element faces, local node numbers (r_getElementFaces)
HEX_FACES = ((4, 3, 2, 1), (5, 6, 7, 8), (1, 2, 6, 5), (2, 3, 7, 6), (3, 4, 8, 7), (4, 1, 5, 8))
SHELL_FACES = ((1, 2, 3, 4), (1, 4, 3, 2))


def _blocks(path):
    """'*command' blocks of a job script: [(command, {key: value or [list entries]})]."""
    out = []
    cur = None
    key = None
    for raw in Path(path).read_text().replace("\t", "    ").splitlines():
        ln = raw.split("#", 1)[0].rstrip()
        if not ln.strip():
            continue
        s = ln.strip()
        if s.startswith("*"):
            cur = (s.split(":")[0], {})
            out.append(cur)
            key = None
        elif cur is not None and ":" in s:
            key, val = s.split(":", 1)
            key = key.strip()
            cur[1][key] = val.strip()
        elif cur is not None and s.startswith("-") and key is not None:
            v = cur[1].get(key)
            if not isinstance(v, list):
                v = [] if not v else [v]
            v.append(s[1:].strip())
            cur[1][key] = v
    return out


class Job:
    def __init__(self, workdir="."):
        self.dir = Path(workdir)
        self.mi = None
        self.model = None
        self.g = None
        self.log = []
        self.time = 0.0
        self.step = 0
        self.u = self.iu = self.v = self.a = None
        self.temp = None
        self.tdot = None
        self.save_hist = False
        self.therm_load = None
        self.reaction = None
        self.thermal_ready = False

    # -- model ----------------------------------------------------------------------------------
    def _gpu(self):
        if self.g is None:
            m = self.model
            self.g = AstroGPU(m)
            n, ni = self.g.n, self.g.int_vec_size
            self.u, self.v, self.a = np.zeros(n), np.zeros(n), np.zeros(n)
            self.iu = np.zeros(ni)
            ini = self.mi.initial
            idx = self.g.n_dof_index[:, :self.g.dims.dof_per_node] - 1
            for key, vec in (("displacement", self.u), ("velocity", self.v), ("acceleration", self.a)):
                vec[idx] = ini[key][:, :self.g.dims.dof_per_node]
            rank = self.g.current_rank - 1
            self.temp = np.zeros(m.num_nodes)
            self.temp[rank] = ini["temperature"]
            self.tdot = np.zeros(m.num_nodes)
            self.tdot[rank] = ini["tdot"]
        return self.g

    def _shell(self):
        return bool(np.any(self.model.element_type == 41))

    def _method(self):
        return SOLVER_FGMRES_LEARNED if self._shell() else SOLVER_GMRES_JACOBI_FP64

    # -- loads ----------------------------------------------------------------------------------
    def _active(self, ld, t):
        return ld["activeTime"][0] <= t <= ld["activeTime"][1]

    def _elements(self, target):
        try:
            return [int(float(target))]
        except ValueError:
            return list(self.mi.element_sets.get(target, []))

    def _faces(self, els, ndir, tol_deg):
        """(element, face) pairs of the listed elements whose outward normal (face diagonals'
        cross product, r_getElSurfaceNormal) is within tol_deg of ndir; bricks: exterior faces."""
        m = self.model
        X = m.node_list
        if not hasattr(self, "_exterior"):
            count = {}
            for e in range(m.num_els):
                if m.element_type[e] == 8:
                    for f in HEX_FACES:
                        key = tuple(sorted(int(m.element_list[e, k - 1]) for k in f))
                        count[key] = count.get(key, 0) + 1
            self._exterior = count
        u = np.asarray(ndir, np.float64)
        u = u / math.sqrt(u @ u)
        c = math.cos(math.pi / 180.0 * tol_deg)
        out = []
        for e in els:
            shell = m.element_type[e - 1] == 41
            for fn, f in enumerate(SHELL_FACES if shell else HEX_FACES, start=1):
                nd = [int(m.element_list[e - 1, k - 1]) for k in f]
                if not shell and self._exterior[tuple(sorted(nd))] != 1:
                    continue
                v1, v2 = X[nd[2] - 1] - X[nd[0] - 1], X[nd[3] - 1] - X[nd[1] - 1]
                nv = np.cross(v1, v2)
                nv = nv / math.sqrt(nv @ nv)
                if nv @ u > c:
                    out.append((e, fn))
        return out

    def elastic_load(self, t):
        g = self._gpu()
        load = np.zeros(g.n)
        for nd, dof, val in self.mi.nodal_loads(t):
            if dof <= g.dims.dof_per_node:
                load[g.n_dof_index[nd - 1, dof - 1] - 1] += val
        kinds = {"bodyForce": 0, "gravitational": 1, "centrifugal": 2}
        for ld in self.mi.loads:
            if not self._active(ld, t):
                continue
            if ld["type"] in kinds:
                for tgt, vals in ld["rows"]:
                    g.body_load(kinds[ld["type"]], list(vals), elements=self._elements(tgt),
                                state=make_state(g.n, disp=self.u, internal_disp=self.iu), elastic_load=load)
            elif ld["type"] in ("surfacePressure", "surfaceTraction"):
                for tgt, vals in ld["rows"]:
                    faces = self._faces(self._elements(tgt), vals[:3], vals[3])
                    if not faces:
                        continue
                    fe, fn = zip(*faces)
                    if ld["type"] == "surfacePressure":
                        g.surface_load(fe, fn, pressure=vals[4], elastic_load=load)
                    else:
                        g.surface_load(fe, fn, traction=vals[4:7], elastic_load=load)
        return load

    def thermal_load(self, t):
        g = self._gpu()
        load = np.zeros(self.model.num_nodes)
        for nd, dof, val in self.mi.nodal_loads(t):
            if dof == 7:
                load[g.current_rank[nd - 1] - 1] += val
        for ld in self.mi.loads:
            if not self._active(ld, t):
                continue
            if ld["type"] == "bodyHeatGen":
                for tgt, vals in ld["rows"]:
                    g.thermal_heat_gen(vals[0], elements=self._elements(tgt), thermal_load=load)
            elif ld["type"] == "surfaceFlux":
                for tgt, vals in ld["rows"]:
                    faces = self._faces(self._elements(tgt), vals[:3], vals[3])
                    if faces:
                        fe, fn = zip(*faces)
                        g.thermal_surface_flux(fe, fn, vals[4], thermal_load=load)
        return load

    # -- commands -------------------------------------------------------------------------------
    def run(self, script):
        for cmd, kv in _blocks(script):
            name = cmd.lstrip("*")
            fn = getattr(self, "cmd_" + name, None)
            if fn is None:
                self.log.append(f"{cmd}: not run by this runner")
                continue
            fn(kv)
        return self

    def cmd_readModelInput(self, kv):
        self.mi = IF.read_model_input(self.dir / kv["fileName"])
        self.model = self.mi.model(name=Path(kv["fileName"]).stem)
        self.g = None
        self.thermal_ready = False
        if hasattr(self, "_exterior"):
            del self._exterior
        self.log.append(f"read model {kv['fileName']}: {self.mi.num_nodes} nodes, {self.mi.num_els} elements")

    def cmd_readDesignVarInput(self, kv):
        dvs = IF.read_design_var_input(self.dir / kv["fileName"], self.mi)
        kept = IF.apply_design_vars(self.model, dvs, strict=False)
        self.g = None
        self.log.append(f"read design variables {kv['fileName']}: kept {kept} of {len(dvs)}")

    def cmd_solve(self, kv):
        yes = lambda k, d: (kv.get(k, d) or d).strip().lower().startswith("y")
        elastic, thermal = yes("elastic", "yes"), yes("thermal", "no")
        nl = 1 if yes("nonLinearGeom", "no") else 0
        dynamic = yes("dynamic", "no")
        # saveSolnHist (Working/AStrO_runJob.f90:183-186): the step files of the time loop
        self.save_hist = yes("saveSolnHist", "no")
        t_load = float(kv.get("staticLoadTime") or 0.0)
        g = self._gpu()
        if thermal and dynamic:
            self._thermal_dynamic(float(kv["timeStep"]), float(kv.get("simPeriod") or 0.0),
                                  float(kv.get("newmarkGamma") or 0.5))
        elif thermal:
            self._thermal_solve(t_load)
        if elastic and not dynamic:
            g.getElasticSolnLoad(1, export=False)
            g.scaleElasticMPC()
            f = self.elastic_load(t_load)
            u0, iu0 = self.u.copy(), self.iu.copy()
            # 1e-12 FP64 relative residual: the shell models of job files are slender (the
            # reference's example beam, E = 1e6), so 1e-10 leaves the displacement near 1e-6
            self.u, self.iu, its, st = g.stepSolve(f, node_disp=self.u, internal_disp=self.iu, nl_geom=nl,
                                                   method=self._method(), rtol=1e-12)
            self.time, self.step = t_load, 0
            # reactionForce is -elasticLoad as the step left it: the load of its last Newton
            # iteration, formed before that iteration's solve (the step's start for a linear step)
            self.reaction = -(self._residual_load(f, u0, iu0) if not nl else self._residual_load(f, self.u, self.iu))
            self.log.append(f"static step: {its} Newton iteration(s), status {st.status}")
        elif elastic and dynamic:
            self._newmark(float(kv["timeStep"]), float(kv.get("simPeriod") or 0.0),
                          float(kv.get("newmarkBeta") or 0.25), float(kv.get("newmarkGamma") or 0.5))

    def _residual_load(self, f, u, iu):
        """applied - Ru at the state (u, iu): the elastic load of a Newton iteration at that state."""
        g = self.g
        load = f.copy()
        g.getElasticSolnLoad(0, state=make_state(g.n, disp=u, internal_disp=iu), elastic_load=load, export=False)
        return load

    def _write_step(self, i, u, v, a, iu):
        """SolutionHistory<i>.out (writeBinarySolution, Working/AStrO_output.f90:761-784)."""
        write_step_file(self.dir / f"SolutionHistory{i}.out", self.model.num_nodes, u, v, a,
                        int_disp=iu if len(iu) else None, temp=self.temp, tdot=self.tdot)

    def _newmark(self, dt, period, beta, gamma):
        g = self.g
        nsteps = int(round(period / dt)) if period > 0 else 0
        g.getElasticSolnLoad(1, state=make_state(g.n, disp=self.u, internal_disp=self.iu), export=False)
        g.scaleElasticMPC()
        if self.save_hist:
            # step 0: the initial state, as loadInitialState leaves it (previous internal DOF zero)
            self._write_step(0, self.u, self.v, self.a, np.zeros(g.int_vec_size))
        times = [(k + 1) * dt for k in range(nsteps)]
        k = 0
        while k < nsteps:
            act = tuple(self._active(ld, times[k]) for ld in self.mi.loads)
            j = k
            while j < nsteps and tuple(self._active(ld, times[j]) for ld in self.mi.loads) == act:
                j += 1
            pattern = self.elastic_load(times[k])
            kw = dict(disp=self.u, vel=self.v, acc=self.a, int_disp=self.iu, rtol=1e-10, method=self._method())
            if self.save_hist:
                self.u, self.v, self.a, self.iu, H, st = g.newmark_run_states(j - k, dt, beta, gamma, pattern,
                                                                              np.ones(j - k), **kw)
                for q in range(j - k):
                    self._write_step(k + q + 1, H["disp"][q], H["vel"][q], H["acc"][q], H["int_disp"][q])
            else:
                self.u, self.v, self.a, self.iu, _, st = g.newmark_run(j - k, dt, beta, gamma, pattern,
                                                                       np.ones(j - k), history=False, **kw)
            self.log.append(f"Newmark steps {k + 1}..{j}: status {st.status}")
            k = j
        self.time, self.step = nsteps * dt, nsteps

    def _thermal_solve(self, t):
        g = self.g
        self._thermal_setup()
        st = thermal_state(self.temp)
        load = self.thermal_load(t)
        f = load.copy()
        g.getThermalSolnLoad(1, state=st, thermal_load=load, export=False)
        g.scaleThermalMPC()
        g.getThermalConstraintLoad(self.temp, load)
        dT, stats = g.thermal_solve(load, rtol=1e-12)
        self.temp = self.temp + dT
        after = f.copy()
        g.getThermalSolnLoad(0, state=thermal_state(self.temp), thermal_load=after, export=False)
        self.therm_load = after
        self.log.append(f"thermal step: {stats.iterations} CG iterations, status {stats.status}")

    def _thermal_setup(self):
        if not self.thermal_ready:
            cond, sh, mpc = self.mi.thermal()
            self.g.thermal_setup(thermal_props(cond, sh, mpc if len(mpc[0]) > 1 else None))
            self.thermal_ready = True

    def _thermal_dynamic(self, dt, period, gamma):
        """The thermal branch of solve's time loop (Working/AStrO_commandFunctions.f90:751-817 with
        stepSolve :689-703): the conductivity + capacitance / (gamma dt) matrix built once at the
        initial state, then per step the residual at the current temperature, the applied and
        constraint loads, one solve, and the rate update of the generalised trapezoid rule."""
        g = self.g
        self._thermal_setup()
        N = self.model.num_nodes
        T = self.temp.copy()
        pT = T.copy()
        pTd = self.tdot.copy() if getattr(self, "tdot", None) is not None else np.zeros(N)
        g.getThermalSolnLoad(1, state=thermal_state(T, pT, pTd, 1, gamma, dt), thermal_load=np.zeros(N), export=False)
        g.scaleThermalMPC()
        nsteps = int(round(period / dt)) if period > 0 else 0
        for k in range(1, nsteps + 1):
            load = self.thermal_load(k * dt)
            g.getThermalSolnLoad(0, state=thermal_state(T, pT, pTd, 1, gamma, dt), thermal_load=load, export=False)
            g.getThermalConstraintLoad(T, load)
            dT, st = g.thermal_solve(load, rtol=1e-12)
            T = T + dT
            Td = (1.0 / gamma) * ((1.0 / dt) * (T - pT) - (1.0 - gamma) * pTd)
            pT, pTd = T.copy(), Td
        self.temp, self.tdot = T, pTd
        self.time, self.step = nsteps * dt, nsteps
        self.log.append(f"thermal time loop: {nsteps} steps")

    def cmd_writeNodeResults(self, kv):
        g = self.g
        m = self.model
        ns = kv.get("nodeSet")
        nodes = self.mi.node_sets.get(ns, None) if ns else None
        nodes = list(range(1, m.num_nodes + 1)) if nodes is None else nodes
        fields = kv.get("fields", [])
        fields = fields if isinstance(fields, list) else [fields]
        fmt = lambda v: f"{float(v):.12G}"
        out = [f" time: {fmt(self.time)}", f" timeStep: {self.step}"]
        for fld in fields:
            if fld in ("temperature", "tdot", "reactionHeatGen"):
                if fld == "temperature":
                    vec = self.temp
                elif fld == "tdot":
                    vec = getattr(self, "tdot", None)
                    vec = np.zeros(m.num_nodes) if vec is None else vec
                else:
                    vec = -(self.therm_load if self.therm_load is not None else np.zeros(m.num_nodes))
                out.append(f" {fld}:")
                for nd in nodes:
                    out.append(f"     - [{nd}, {fmt(vec[g.current_rank[nd - 1] - 1])}]")
            elif fld in ("displacement", "velocity", "acceleration", "reactionForce"):
                vec = {"displacement": self.u, "velocity": self.v, "acceleration": self.a,
                       "reactionForce": self.reaction if self.reaction is not None else np.zeros(g.n)}[fld]
                out.append(f" {fld}:")
                for nd in nodes:
                    vals = [vec[g.n_dof_index[nd - 1, k] - 1] if k < g.dims.dof_per_node else 0.0 for k in range(6)]
                    out.append(f"     - [{nd}, " + ", ".join(fmt(v) for v in vals) + "]")
            else:
                self.log.append(f"*writeNodeResults: field {fld} not written")
        (self.dir / kv["fileName"]).write_text("\n".join(out) + "\n")


def read_node_results(path):
    """Fields of a node-results file: {field: {node: values}}."""
    res, cur = {}, None
    for ln in Path(path).read_text().splitlines():
        s = ln.strip()
        if s.endswith(":") and not s.startswith("-"):
            cur = s[:-1]
            res[cur] = {}
        elif s.startswith("- [") and cur is not None:
            vals = [float(x) for x in s[3:s.index("]")].split(",")]
            res[cur][int(vals[0])] = np.array(vals[1:])
    return res


def main():
    import argparse
    ap = argparse.ArgumentParser(description="Run an AStrO job script on the GPU")
    ap.add_argument("script")
    a = ap.parse_args()
    job = Job(Path(a.script).parent).run(a.script)
    print("\n".join(job.log))


if __name__ == "__main__":
    main()
