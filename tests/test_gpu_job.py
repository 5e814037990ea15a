"""Job scripts on the device (misc_gb300.job): the reference's example model solved statically
through a '*solve' block and written by '*writeNodeResults' (against the oracle's direct solve),
a steady thermal job on a brick bar with end temperatures given as DOF-7 constraints (linear
profile, heat flux), and a Newmark job whose load switches off half way (split into segments,
against one device time loop with the same load history)."""
import shutil
from pathlib import Path

import numpy as np
import pytest
import scipy.sparse.linalg as spla

from misc_gb300 import inputfile as IF
from misc_gb300 import job as J
from misc_gb300 import model as M
from misc_gb300.astro import SOLVER_FGMRES_LEARNED, AstroGPU
from oracle import Oracle

pytestmark = pytest.mark.gpu
FIX = Path(__file__).parent / "golden" / "shell_beam_model_input.yaml"


def test_static_job_on_the_reference_example(tmp_path):
    shutil.copyfile(FIX, tmp_path / "model.yaml")
    (tmp_path / "job.txt").write_text(
        "*readModelInput:\n    fileName: model.yaml\n*solve:\n    elastic: yes\n    thermal: no\n"
        "*writeNodeResults:\n    fileName: out.txt\n    nodeSet: tip\n    fields:\n        - displacement\n"
        "        - reactionForce\n*modalAnalysis:\n    type: buckling\n")
    job = J.Job(tmp_path).run(tmp_path / "job.txt")
    assert any("not run" in s for s in job.log)
    res = J.read_node_results(tmp_path / "out.txt")
    mi = IF.read_model_input(FIX)
    m = mi.model()
    m.point_loads = mi.nodal_loads()
    o = Oracle(m)
    A, b, *_ = o.static_system()
    u = spla.spsolve(A.tocsc(), b)
    # the step starts from the file's initial state (loadInitialState); the linear step from there
    # lands on the oracle's solution from zero (the tip displacement is a rigid-body-free
    # translation of two nodes, inside the linear range of the element residual)
    for nd in (11, 22):
        ref = np.array([u[o.n_dof_index[nd - 1, k] - 1] for k in range(6)])
        assert np.linalg.norm(res["displacement"][nd] - ref) <= 1e-7 * np.linalg.norm(ref)
    # reactionForce = -elasticLoad of the step's (only) iteration: -(f - Ru(u0)), u0 the file's
    # initial displacement (w = 1 at the tip nodes)
    u0 = np.zeros(o.n)
    for nd in range(1, m.num_nodes + 1):
        for k in range(6):
            u0[o.n_dof_index[nd - 1, k] - 1] = mi.initial["displacement"][nd - 1, k]
    f = o.applied_load(np.zeros(o.n))
    lo = o.el_soln_load(0, state=M.make_state(o.n, disp=u0), elastic_load=f.copy())[0]
    for nd in (11, 22):
        ref = -np.array([lo[o.n_dof_index[nd - 1, k] - 1] for k in range(6)])
        assert np.linalg.norm(res["reactionForce"][nd] - ref) <= 1e-9 * np.linalg.norm(ref)


def test_thermal_job_on_a_brick_bar(tmp_path):
    m = M.hex_block(6, 2, 2, lx=3.0, ly=1.0, lz=1.0, jitter=0.0)
    X = m.node_list
    left = list(np.nonzero(X[:, 0] == 0)[0] + 1)
    right = list(np.nonzero(np.isclose(X[:, 0], 3.0))[0] + 1)
    IF.write_model_input(m, tmp_path / "bar.yaml", node_sets={"left": left, "right": right})
    txt = (tmp_path / "bar.yaml").read_text()
    # thermal data and the end temperatures (constraint terms on DOF 7), replacing the clamp
    txt = txt[:txt.index("constraints:")]
    txt = txt.replace("      elastic:\n", "      thermal:\n          conductivity: 45.0\n          specificHeat: 460.0\n"
                                         "      elastic:\n")
    txt += "constraints:\n    matrix:\n        - [1, left, 7, 1.0]\n        - [2, right, 7, 1.0]\n" \
           "    rhs:\n        - 20.0\n        - 80.0\n"
    (tmp_path / "bar.yaml").write_text(txt)
    (tmp_path / "job.txt").write_text(
        "*readModelInput:\n    fileName: bar.yaml\n*solve:\n    elastic: no\n    thermal: yes\n"
        "*writeNodeResults:\n    fileName: temp.txt\n    fields:\n        - temperature\n        - reactionHeatGen\n")
    job = J.Job(tmp_path).run(tmp_path / "job.txt")
    res = J.read_node_results(tmp_path / "temp.txt")
    T = np.array([res["temperature"][nd][0] for nd in range(1, m.num_nodes + 1)])
    assert np.abs(T - (20.0 + 60.0 * X[:, 0] / 3.0)).max() < 1e-3
    q_left = sum(res["reactionHeatGen"][nd][0] for nd in left)
    assert abs(abs(q_left) - 45.0 * 1.0 * 20.0) < 0.05


def test_newmark_job_segments(tmp_path):
    m = M.plate_shell(nx=6, ny=6, lx=1.0, ly=1.0, t=0.01, E=7e10, nu=0.33, rho=2700.0, pressure=0.0, clamp="ss",
                      y0=0.0)
    centre = 3 * 7 + 3 + 1
    IF.write_model_input(m, tmp_path / "plate.yaml", node_sets={"c": [centre]})
    txt = (tmp_path / "plate.yaml").read_text()
    txt = txt[:txt.index("loads:")] if "loads:" in txt else txt
    txt += "loads:\n    - type: nodal\n      activeTime: [0.0, 5.5e-5]\n      setLoads:\n" \
           "          - [c, 0.0, 0.0, 100.0, 0.0, 0.0, 0.0, 0.0]\n"
    (tmp_path / "plate.yaml").write_text(txt)
    (tmp_path / "job.txt").write_text(
        "*readModelInput:\n    fileName: plate.yaml\n*solve:\n    elastic: yes\n    dynamic: yes\n"
        "    timeStep: 1e-5\n    simPeriod: 1e-4\n    newmarkBeta: 0.25\n    newmarkGamma: 0.5\n"
        "*writeNodeResults:\n    fileName: dyn.txt\n    fields:\n        - displacement\n        - velocity\n")
    job = J.Job(tmp_path).run(tmp_path / "job.txt")
    assert sum("Newmark steps" in s for s in job.log) == 2
    res = J.read_node_results(tmp_path / "dyn.txt")
    mi = IF.read_model_input(tmp_path / "plate.yaml")
    g = AstroGPU(mi.model())
    g.getElasticSolnLoad(1, export=False)
    g.scaleElasticMPC()
    pat = np.zeros(g.n)
    pat[g.n_dof_index[centre - 1, 2] - 1] = 100.0
    amp = np.array([1.0] * 5 + [0.0] * 5)
    u, v, a, iu, _, st = g.newmark_run(10, 1e-5, 0.25, 0.5, pat, amp, rtol=1e-10, history=False,
                                       method=SOLVER_FGMRES_LEARNED)
    ug = np.array([[u[g.n_dof_index[nd - 1, k] - 1] for k in range(6)] for nd in range(1, m.num_nodes + 1)])
    uj = np.array([res["displacement"][nd] for nd in range(1, m.num_nodes + 1)])
    assert np.linalg.norm(uj - ug) <= 1e-6 * np.linalg.norm(ug)


def test_transient_thermal_job(tmp_path):
    """solve's thermal time loop: a brick bar at 0 with its left end held at 100, five steps of
    the generalised trapezoid rule, against the same loop on the oracle's matrices."""
    m = M.hex_block(6, 2, 2, lx=3.0, ly=1.0, lz=1.0, jitter=0.0)
    X = m.node_list
    left = list(np.nonzero(X[:, 0] == 0)[0] + 1)
    IF.write_model_input(m, tmp_path / "bar.yaml", node_sets={"left": left})
    txt = (tmp_path / "bar.yaml").read_text()
    txt = txt[:txt.index("constraints:")]
    txt = txt.replace("      elastic:\n", "      thermal:\n          conductivity: 45.0\n          specificHeat: 460.0\n"
                                         "      elastic:\n")
    txt += "constraints:\n    matrix:\n        - [1, left, 7, 1.0]\n    rhs:\n        - 100.0\n"
    (tmp_path / "bar.yaml").write_text(txt)
    (tmp_path / "job.txt").write_text(
        "*readModelInput:\n    fileName: bar.yaml\n*solve:\n    elastic: no\n    thermal: yes\n    dynamic: yes\n"
        "    timeStep: 50.0\n    simPeriod: 250.0\n    newmarkGamma: 0.6\n"
        "*writeNodeResults:\n    fileName: temp.txt\n    fields:\n        - temperature\n        - tdot\n")
    J.Job(tmp_path).run(tmp_path / "job.txt")
    res = J.read_node_results(tmp_path / "temp.txt")
    Tj = np.array([res["temperature"][nd][0] for nd in range(1, m.num_nodes + 1)])
    # the oracle's loop (rank order)
    mi = IF.read_model_input(tmp_path / "bar.yaml")
    o = Oracle(mi.model())
    cond, sh, mpc = mi.thermal()
    N, dt, gm = m.num_nodes, 50.0, 0.6
    T, pT, pTd = np.zeros(N), np.zeros(N), np.zeros(N)
    _, mat, cols, rng = o.thermal_soln_load(cond, sh, 1, temp=T, prev_temp=pT, prev_tdot=pTd, dynamic=1, gamma=gm,
                                            del_t=dt)
    import scipy.sparse as sp
    K = sp.csr_matrix((mat, cols - 1, rng), shape=(N, N))
    rows = o.scale_thermal_mpc(mat, o.thermal_mpc(*mpc))
    r_, c_, v_ = zip(*[(i, c - 1, k) for i, (cs, vs, _) in enumerate(rows) for c, k in zip(cs, vs) if c])
    Cm = sp.csr_matrix((v_, (r_, c_)), shape=(len(rows), N))
    A = (K + Cm.T @ Cm).tocsc()
    for _ in range(5):
        load = np.zeros(N)
        o.thermal_soln_load(cond, sh, 0, temp=T, prev_temp=pT, prev_tdot=pTd, dynamic=1, gamma=gm, del_t=dt, load=load)
        o.thermal_constraint_load(rows, T, load)
        T = T + spla.spsolve(A, load)
        Td = (1 / gm) * ((1 / dt) * (T - pT) - (1 - gm) * pTd)
        pT, pTd = T.copy(), Td
    To = T[o.current_rank - 1]
    assert np.linalg.norm(Tj - To) <= 1e-8 * np.linalg.norm(To)
    assert To.max() > 50.0 and To.min() < 10.0   # heat has entered from the left end, not reached the right


def test_newmark_job_writes_solution_history(tmp_path):
    """saveSolnHist: yes writes SolutionHistory0..N.out (writeBinarySolution's records after each
    step of solve's time loop): the initial state, then each step's displacement, internal DOF,
    velocity and acceleration, equal to the device loop's states."""
    from misc_gb300.astro import read_step_file
    m = M.plate_shell(nx=4, ny=4, lx=1.0, ly=1.0, t=0.01, E=7e10, nu=0.33, rho=2700.0, pressure=0.0, clamp="ss",
                      y0=0.0)
    centre = 2 * 5 + 2 + 1
    IF.write_model_input(m, tmp_path / "plate.yaml", node_sets={"c": [centre]})
    txt = (tmp_path / "plate.yaml").read_text()
    txt = txt[:txt.index("loads:")] if "loads:" in txt else txt
    txt += "loads:\n    - type: nodal\n      activeTime: [0.0, 1.0]\n      setLoads:\n" \
           "          - [c, 0.0, 0.0, 100.0, 0.0, 0.0, 0.0, 0.0]\n"
    (tmp_path / "plate.yaml").write_text(txt)
    (tmp_path / "job.txt").write_text(
        "*readModelInput:\n    fileName: plate.yaml\n*solve:\n    elastic: yes\n    dynamic: yes\n"
        "    timeStep: 1e-5\n    simPeriod: 4e-5\n    saveSolnHist: yes\n")
    job = J.Job(tmp_path).run(tmp_path / "job.txt")
    g = job.g
    n, ni, N = g.n, g.int_vec_size, m.num_nodes
    files = sorted(tmp_path.glob("SolutionHistory*.out"))
    assert len(files) == 5
    _, _, u0, iu0, v0, a0 = read_step_file(tmp_path / "SolutionHistory0.out", N, n, ni)
    assert not u0.any() and not iu0.any()
    mi = IF.read_model_input(tmp_path / "plate.yaml")
    g2 = AstroGPU(mi.model())
    g2.getElasticSolnLoad(1, export=False)
    g2.scaleElasticMPC()
    pat = job.elastic_load(1e-5)
    u, v, a, iu, H, st = g2.newmark_run_states(4, 1e-5, 0.25, 0.5, pat, np.ones(4), rtol=1e-10,
                                               method=SOLVER_FGMRES_LEARNED)
    for i in range(1, 5):
        _, _, ui, iui, vi, ai = read_step_file(tmp_path / f"SolutionHistory{i}.out", N, n, ni)
        for x, y in ((ui, H["disp"][i - 1]), (vi, H["vel"][i - 1]), (ai, H["acc"][i - 1]), (iui, H["int_disp"][i - 1])):
            assert np.linalg.norm(x - y) <= 1e-9 * max(np.linalg.norm(y), 1e-300), i
    assert np.array_equal(H["disp"][-1], u) and np.array_equal(H["vel"][-1], v) and np.array_equal(H["acc"][-1], a)
