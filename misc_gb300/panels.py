"""Batched panels with complex-step sensitivities: many independent shell panels solved for
their pressure load and for the complex-step design sensitivities of their thickness groups.

For every panel the reference would run one model: assembly (getElasticSolnLoad), the
constraint scaling, the applied pressure load, getdRelasticdD per design variable
(Working/AStrO_commandFunctions.f90:1172-1375) and a linear solve per right-hand side.  Here the
panels are one model (its connected components) and every step runs once for all of them: the
FP64 assembly, the complex-step dR/dd of each thickness group (a design variable covers its group
in every panel), and one batched LDL^T factorisation plus one multi-right-hand-side solve
(astro_panels_factor / astro_panels_solve)."""
from __future__ import annotations

import time

import numpy as np

from .astro import AstroGPU
from .model import make_state


def pressure_load(g: AstroGPU, m) -> np.ndarray:
    """Consistent load of each panel's own pressure (the unit-pressure load of all faces scaled
    panel by panel: the load is linear in the pressure and local to the panel)."""
    unit = g.surface_load(m.face_el, m.face_num, pressure=1.0)
    node_p = np.repeat(m.panel_pressure, np.diff(m.panel_node_ptr))
    scale = np.zeros(g.n)
    idx = g.n_dof_index[:, :g.dims.dof_per_node] - 1
    scale[idx] = node_p[:, None]
    return unit * scale


def sensitivity_rhs(g: AstroGPU, n_dvars: int, state=None, h: float = 1e-14) -> np.ndarray:
    """Columns dRu/dd of design variables 1..n_dvars (complex step at the given state), condensed
    to the nodal DOF (updateExternalRHS) on the device: the right-hand sides of the sensitivity
    solves."""
    return g.drdd_condensed(np.arange(1, n_dvars + 1), h, state=state)


def solve_batch(g: AstroGPU, m, n_dvars: int, cluster_size: int = 0, load_scale: float = 1.0):
    """Assembly, pressure load, batched factorisation and displacement solve, the complex-step
    dRu/dd of every thickness group at the solved state, and one batched solve of all of them:
    returns (u, du_dd, timings) with du_dd[:, k] = -(K + C^T C)^-1 dRu/dd_k, the direct design
    sensitivity of the displacement (exact for the linear response; at a large displacement the
    complex step differentiates the element's nonlinear residual at that state)."""
    t = {}
    t0 = time.perf_counter()
    g.getElasticSolnLoad(1, export=False)
    g.scaleElasticMPC()
    f = load_scale * pressure_load(g, m)
    t["assembly_s"] = time.perf_counter() - t0
    info = g.panels_factor(cluster_size)
    t["factor_s"] = info.factor_seconds
    u, s1 = g.panels_solve(f)
    t["solve_u_s"] = s1.solve_seconds
    t0 = time.perf_counter()
    iu = g.updateInternalSoln(u, np.zeros(g.int_vec_size)) if g.int_vec_size else None
    st = make_state(g.n, disp=u, internal_disp=iu)
    R = sensitivity_rhs(g, n_dvars, state=st)
    t["rhs_s"] = time.perf_counter() - t0
    dU, s2 = g.panels_solve(R)
    t["solve_dU_s"] = s2.solve_seconds
    t["info"] = info
    t["f"], t["R"], t["state"] = f, R, st
    return u, -dU, t


def _main(argv=None):
    """Factor a generated batch with the trailing-update variants in turn and print each factor
    time (ASTRO_OPT_BAND_FP64_UPDATE: 1 FP64, 2 emulation on mma.sync, 0 emulation on tcgen05, 3
    double-float factorisation); with --rhs, then solve a seeded random block of that many columns
    in each ASTRO_OPT_PANELS_SOLVE mode (0 double-float + FP64 refinement, 1 FP64 sweeps, 2
    double-float alone), twice each, and print the host-clock times and the distance to the first
    mode's solution."""
    import argparse

    from . import model as M
    from .astro import OPT_BAND_FP64_UPDATE, OPT_PANELS_SOLVE
    p = argparse.ArgumentParser(description=_main.__doc__)
    p.add_argument("--panels", type=int, default=64)
    p.add_argument("--cluster", type=int, default=4, help="CTAs per cluster (2, 4, 8)")
    p.add_argument("--updates", default="1,2,0", help="option values, in launch order")
    p.add_argument("--rhs", type=int, default=0, help="right-hand-side columns of the solves (0: no solve)")
    p.add_argument("--solves", default="1,2,0", help="ASTRO_OPT_PANELS_SOLVE values, in order")
    p.add_argument("--solve-update", type=int, default=1, help="the trailing-update option of the solves' factor")
    a = p.parse_args(argv)
    m = M.panel_batch(num_panels=a.panels)
    g = AstroGPU(m)
    g.getElasticSolnLoad(1, export=False)
    g.scaleElasticMPC()
    for mode in (int(x) for x in a.updates.split(",")):
        g.set_option(OPT_BAND_FP64_UPDATE, mode)
        for _ in range(2):
            info = g.panels_factor(a.cluster)
            print(f"update {mode}: factor {info.factor_seconds:.4f} s, {info.workers} clusters of "
                  f"{info.cluster_size}", flush=True)
    if a.rhs > 0:
        g.set_option(OPT_BAND_FP64_UPDATE, a.solve_update)
        g.panels_factor(a.cluster)
        B = np.asfortranarray(np.random.default_rng(1).standard_normal((g.n, a.rhs)))
        first = None
        for mode in (int(x) for x in a.solves.split(",")):
            g.set_option(OPT_PANELS_SOLVE, mode)
            for rep in range(2):
                t0 = time.perf_counter()
                X, si = g.panels_solve(B)
                print(f"solve mode {mode} rep {rep}: {time.perf_counter() - t0:.4f} s "
                      f"(call {si.solve_seconds:.4f} s)", flush=True)
            if first is None:
                first = X
            else:
                print(f"  distance to the first mode's solution {np.linalg.norm(X - first) / np.linalg.norm(first):.3e}")
        g.set_option(OPT_PANELS_SOLVE, 0)
    g.set_option(OPT_BAND_FP64_UPDATE, 1)


if __name__ == "__main__":
    _main()
