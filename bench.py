"""Benchmark of the AStrO hot path on one GB300 (config: 64x32x32 brick8 heterogeneous block).

Metric: element matrices per second (the element-evaluation + global-assembly pass), plus the
static solve to 1e-10 FP64 relative residual reported in the "solve" object.
  value   FP32 element kernels (sparse-B, orthotropic C) assembled into the device block-CSR
          matrix, inputs resident in HBM; one step = one pass over all 65,536 elements
          (8 colour launches).  L2 is flushed between timed steps.
  e2e     getElasticSolnLoad(buildMat=1) through the C ABI (astro_el_soln_load) with host
          buffers: state/load upload, FP64 element kernels, assembly, and the export of the
          reference CSR matrix (values + columns) and the residual load to host memory.
  solve   to 1e-10, seconds each (CUDA events): the learned solver (FP32 inner GMRES(50)
          right-preconditioned by the polynomial graph network, trained on the device on a smaller
          block of the same family, FP64 residual refinement), the mixed-precision Jacobi solver
          (FP32 inner, FP64 refinement) and the plain FP64 Jacobi-GMRES(50) comparator.
`--impl reference` times the CPU restatement of the reference (the oracle) on a bounded sample of
the same workload with all host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

TRAFFIC_PER_PASS = 286490112  # bytes, see the roofline comment in run_ours
METRIC = "element mats/s (64x32x32 brick8 block: element eval + assembly); s to 1e-10 FP64 rel resid"
UNIT = "elements/s"


def _parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--precond-degree", type=int, default=24)
    p.add_argument("--precond-ratio", type=float, default=3000.0)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--nx", type=int, default=64)
    p.add_argument("--ny", type=int, default=32)
    p.add_argument("--nz", type=int, default=32)
    p.add_argument("--no-solve", action="store_true")
    p.add_argument("--solve-max-iters", type=int, default=60000)
    p.add_argument("--no-learned-eval", action="store_true")
    p.add_argument("--learned-only", action="store_true",
                   help="run only the learned-preconditioner evaluation and print its JSON object")
    p.add_argument("--unrolled-cycles", action="store_true",
                   help="capture the restart cycles unrolled (profilers do not look inside conditional nodes)")
    p.add_argument("--no-fp64", action="store_true", help="learned evaluation without the FP64 comparator")
    p.add_argument("--eval-nx", type=int, default=96)
    p.add_argument("--panels", type=int, default=512, help="panels of the batched-panel leg (0: skip it)")
    p.add_argument("--newmark-steps", type=int, default=0,
                   help="time steps of the element-residual Newmark leg (astro_newmark_run; 0: skip it, the default)")
    p.add_argument("--nmc-steps", type=int, default=2000,
                   help="time steps of the batched linear Newmark leg (factored K_eff, 17 cases; 0: skip it)")
    p.add_argument("--nmc-cases", type=int, default=17, help="load cases of the batched Newmark leg")
    p.add_argument("--no-widened", action="store_true", help="skip the thermal / adjoint / body-load leg")
    p.add_argument("--no-cpu-legs", action="store_true", help="skip the CPU baseline legs of configs 1, 2 and 5")
    p.add_argument("--panels-only", action="store_true", help="only the batched-panel leg")
    p.add_argument("--panels-cluster", type=int, default=0, help="cluster size (0: autotuned over 2, 4, 8)")
    return p.parse_args()


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    return rank, ws


def _config(a):
    return {"workload": f"cfg2 heterogeneous block {a.nx}x{a.ny}x{a.nz} brick8 (seed 0)",
            "elements": a.nx * a.ny * a.nz, "dof": 3 * (a.nx + 1) * (a.ny + 1) * (a.nz + 1),
            "l2": "flushed between timed steps (256 MB write)", "parallelism": "replicas only"}


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self):
        self.proc = None
        import tempfile
        self.path = os.path.join(tempfile.gettempdir(), f"misc_gb300_clocks_{os.getpid()}.csv")

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "100"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def _peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return None


def _oracle_rate(model, nel, threads):
    """Oracle (CPU restatement) element matrices per second on elements 1..nel, split over threads."""
    from oracle import Oracle
    o = Oracle(model)
    chunks = np.array_split(np.arange(1, nel + 1), threads)

    def work(c):
        if len(c):
            o.element_matrices(int(c[0]), int(c[-1]))

    t0 = time.perf_counter()
    ths = [threading.Thread(target=work, args=(c,)) for c in chunks]
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    dt = time.perf_counter() - t0
    return nel / dt, dt


def run_reference(a):
    rank, ws = _dist()
    if rank != 0:
        return 0
    from misc_gb300 import model as M
    m = M.config2(nx=a.nx, ny=a.ny, nz=a.nz)
    cores = os.cpu_count() or 1
    sample = min(m.num_els, 512 * cores)
    for _ in range(max(a.warmup, 0)):
        _oracle_rate(m, min(sample, 64 * cores), cores)
    times = []
    for _ in range(a.steps):
        r, dt = _oracle_rate(m, sample, cores)
        times.append(dt)
    tot = sum(times)
    val = a.steps * sample / tot
    line = {"metric": METRIC, "value": val, "unit": UNIT, "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": 1e3 * tot / a.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic", "config": _config(a), "impl": "reference",
            "cpu_baseline": {"value": val, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"brick8 element matrices of elements 1..{sample} per step (oracle restatement "
                                       f"of r_getElRuk, FP64), split over {cores} host threads"},
            "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def run_ours(a):
    rank, ws = _dist()
    import ctypes as C

    import torch
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    from misc_gb300 import model as M
    from misc_gb300.astro import (SOLVER_FGMRES_LEARNED, SOLVER_FGMRES_MIXED, SOLVER_GMRES_JACOBI_FP64, AstroGPU,
                                  load_library, precond_init)
    m = M.config2(nx=a.nx, ny=a.ny, nz=a.nz)
    g = AstroGPU(m)
    L = load_library()
    E = m.num_els
    # device-resident FP32 path
    g.assemble_fp32()
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    stream = C.c_void_p()
    # the library launches on its own stream: time with CUDA events recorded on that stream via
    # the runtime API (torch events would only see torch's stream)
    cudart = C.CDLL("libcudart.so")
    cudart.cudaEventCreate.argtypes = [C.POINTER(C.c_void_p)]
    cudart.cudaEventRecord.argtypes = [C.c_void_p, C.c_void_p]
    cudart.cudaEventElapsedTime.argtypes = [C.POINTER(C.c_float), C.c_void_p, C.c_void_p]
    cudart.cudaEventSynchronize.argtypes = [C.c_void_p]
    cudart.cudaDeviceSynchronize.argtypes = []
    cudart.cudaMemsetAsync.argtypes = [C.c_void_p, C.c_int, C.c_size_t, C.c_void_p]
    s = L.astro_ctx_stream(g.h)
    ev = [C.c_void_p() for _ in range(2 * a.steps)]
    for e in ev:
        cudart.cudaEventCreate(C.byref(e))
    for _ in range(a.warmup):
        L.astro_assemble_fp32_async(g.h)
        flush.fill_(1)
    torch.cuda.synchronize()
    cudart.cudaDeviceSynchronize()
    if ws > 1:
        torch.distributed.barrier()
    clk = Clocks()
    clk.start()
    t0 = time.perf_counter()
    # the L2 flush is queued on the library's stream ahead of each step, and the host does not
    # wait between steps: the events bracket the device work of the pass alone, not the host's
    # launch latency (that latency is in the end-to-end figure)
    for k in range(a.steps):
        assert cudart.cudaMemsetAsync(flush.data_ptr(), k & 0xFF, flush.numel(), s) == 0
        cudart.cudaEventRecord(ev[2 * k], s)
        rc = L.astro_assemble_fp32_async(g.h)
        assert rc == 0
        cudart.cudaEventRecord(ev[2 * k + 1], s)
    cudart.cudaDeviceSynchronize()
    wall = time.perf_counter() - t0
    ms = []
    for k in range(a.steps):
        f = C.c_float()
        cudart.cudaEventElapsedTime(C.byref(f), ev[2 * k], ev[2 * k + 1])
        ms.append(f.value)
    clocks = clk.stop()
    tot_ms = sum(ms)
    if ws > 1:
        t = torch.tensor([tot_ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        tot_ms = float(t.item())
    value = ws * E * a.steps / (tot_ms * 1e-3)
    ms_step = tot_ms / a.steps
    # e2e: FP64 drop-in call with host buffers
    n = g.n

    def pinned(size, dtype):
        # page-locked host buffers: the library's copies to and from them are direct DMA
        return torch.zeros(size, dtype=dtype, pin_memory=True).numpy()

    load = pinned(n, torch.float64)
    mat = pinned(g.el_mat_size, torch.float64)
    cols = pinned(g.el_mat_size, torch.int32)
    disp = np.zeros(n)
    st = M.make_state(n, disp=disp)
    from misc_gb300.astro import _d, _i
    for _ in range(max(1, a.warmup // 2)):
        load[:] = 0
        L.astro_el_soln_load(g.h, 1, C.byref(st), _d(load), None, _d(mat), _i(cols), None)
    e2e_steps = max(3, min(a.steps, 10))
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        load[:] = 0
        rc = L.astro_el_soln_load(g.h, 1, C.byref(st), _d(load), None, _d(mat), _i(cols), None)
        assert rc == 0
    e2e_dt = (time.perf_counter() - t0) / e2e_steps
    # the FP64 path device-resident: the same call without the matrix export (double-float element
    # kernels and assembly; only the load vector comes back), host clock per call
    for _ in range(2):
        load[:] = 0
        L.astro_el_soln_load(g.h, 1, C.byref(st), _d(load), None, None, None, None)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        load[:] = 0
        rc = L.astro_el_soln_load(g.h, 1, C.byref(st), _d(load), None, None, None, None)
        assert rc == 0
    fp64_dt = (time.perf_counter() - t0) / e2e_steps
    # the same two calls at a displaced state (a Newton iteration's getElasticSolnLoad): the
    # general-state kernels (Green-Lagrange strain, stress stiffness, residual); the state is one
    # more host-to-device copy
    disp_nz = pinned(n, torch.float64)
    disp_nz[:] = 1e-4 * np.random.default_rng(17).standard_normal(n)
    st_nz = M.make_state(n, disp=disp_nz)
    for _ in range(2):
        load[:] = 0
        L.astro_el_soln_load(g.h, 1, C.byref(st_nz), _d(load), None, _d(mat), _i(cols), None)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        load[:] = 0
        rc = L.astro_el_soln_load(g.h, 1, C.byref(st_nz), _d(load), None, _d(mat), _i(cols), None)
        assert rc == 0
    e2e_nz_dt = (time.perf_counter() - t0) / e2e_steps
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        load[:] = 0
        rc = L.astro_el_soln_load(g.h, 1, C.byref(st_nz), _d(load), None, None, None, None)
        assert rc == 0
    fp64_nz_dt = (time.perf_counter() - t0) / e2e_steps
    # FP64 device-resident (kernel only) for reference
    g.getElasticSolnLoad(1, export=False)
    # roofline of the assembly pass
    peaks = _peaks()
    hbm = peaks["hbm_gbs"] if peaks else 6800.0
    nnz = g.dims.num_blocks * 9
    alg_bytes = nnz * 4 + m.num_nodes * 24 + E * (8 * 4 + 9 * 8)
    achieved = alg_bytes / (ms_step * 1e-3) / 1e9
    # DRAM bytes (read + write) of the 8 colour launches of one FP32 assembly pass, measured by ncu
    # with the caches flushed before every launch (the assembly kernel's ncu summary under
    # profiles/); only for the default 64x32x32 block
    traffic = TRAFFIC_PER_PASS if (a.nx, a.ny, a.nz) == (64, 32, 32) else None
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic", "config": _config(a),
            "e2e": {"value": E / e2e_dt, "unit": UNIT, "path": "astro_el_soln_load FP64 with pinned host buffers",
                    "h2d_bytes_per_step": n * 8, "d2h_bytes_per_step": n * 8 + g.el_mat_size * 12,
                    "note": "state is the undeformed one (all-zero displacement is not copied); copied per call: "
                            "the load vector in, the load, CSR values and CSR columns out"},
            "e2e_nonzero_state": {"value": E / e2e_nz_dt, "unit": UNIT,
                                  "path": "astro_el_soln_load FP64 at a displaced state (1e-4 N(0,1) per DOF, seed 17): "
                                          "the general-state double-float kernel (Green-Lagrange strain, stress "
                                          "stiffness, residual), pinned host buffers",
                                  "h2d_bytes_per_step": 2 * n * 8, "d2h_bytes_per_step": n * 8 + g.el_mat_size * 12,
                                  "device_resident_value": E / fp64_nz_dt,
                                  "device_resident_path": "the same call without the CSR export (load vector in and "
                                                          "out, state in); host clock"},
            "fp64_assembly": {"value": E / fp64_dt, "unit": UNIT,
                              "path": "astro_el_soln_load(build_mat=1) without the CSR export: FP64 (double-float) "
                                      "element kernels + block-CSR assembly, load vector copied back; host clock"},
            "per_context_staging": "excluded from every timed figure: per element C = S^-1 (the reference's LU of the "
                                   "engineering constants) and the node coordinates in the section frame, split "
                                   "into double-float, are computed once when the context is created (the model is "
                                   "fixed), where the reference recomputes them in every element call",
            "fp64_arithmetic": "the FP64 element paths compute in double-float (pairs of FP32, about 48 significant "
                               "bits; element matrices within 1e-12 of the FP64 oracle) and deliver FP64",
            "gpu_launches": a.steps * g.dims.num_colors,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                         "traffic": traffic, "traffic_note": "ncu, caches flushed before each colour launch",
                         "kernel": "hex8_fast_kernel<float> (8 colour launches = 1 assembly pass)",
                         "algorithmic_bytes": alg_bytes, "peak_source": "measured" if peaks else "fallback"},
            "clocks": clocks, "wall_s": wall}
    if not a.no_solve and rank == 0:
        g.scaleElasticMPC()
        b = g.static_rhs()
        res = {}
        # the network: trained on the device on a 16x8x8 block of the same family (other seed),
        # white-noise samples; the training is a one-off cost outside the solve
        gt = AstroGPU(M.config2(nx=16, ny=8, nz=8, seed=101))
        gt.getElasticSolnLoad(1, export=False)
        gt.assemble_fp32()
        gt.scaleElasticMPC()
        p0 = precond_init(a.precond_degree, a.precond_ratio, 3)
        samples = np.random.default_rng(5).standard_normal((8, gt.n))
        t0 = time.perf_counter()
        p, tinfo = gt.precond_train_validated(p0, samples, iters=20)
        train_s = time.perf_counter() - t0
        del gt
        sols = {}
        for name, meth in (("gmres_fp64", SOLVER_GMRES_JACOBI_FP64), ("fgmres_learned", SOLVER_FGMRES_LEARNED),
                           ("fgmres_mixed", SOLVER_FGMRES_MIXED)):
            # first call: workspace allocation, graph capture and instantiation included; the
            # second call reuses them (the steady state of repeated solves on one model).  Before
            # the second call the FP32 matrix is assembled again (same values), so the learned
            # solve rebuilds its FP16 operator and eigenvalue estimate inside the timed solve
            kw = dict(method=meth, rtol=1e-10, restart=50, max_iters=a.solve_max_iters, allow_maxit=True,
                      precond=p if meth == SOLVER_FGMRES_LEARNED else None)
            u, st1 = g.solve_static(b, **kw)
            g.assemble_fp32()
            u, stt = g.solve_static(b, **kw)
            sols[name] = u
            res[name] = {"seconds": stt.seconds, "first_call_seconds": st1.seconds, "iterations": stt.iterations, "restarts": stt.restarts,
                         "refinements": stt.refinements, "rel_residual": stt.rel_residual, "status": stt.status,
                         "conditional_graph": stt.conditional_graph, "residual_kind": stt.residual_kind}
        # the error of each solution against a tighter FP64 solve of the same system (FP64
        # Jacobi-GMRES to 1e-13 relative residual: the FP64 reference solution on the device)
        uref, _ = g.solve_static(b, method=SOLVER_GMRES_JACOBI_FP64, rtol=1e-13, restart=50,
                                 max_iters=a.solve_max_iters, allow_maxit=True)
        for name, u in sols.items():
            res[name]["err_vs_fp64"] = float(np.linalg.norm(u - uref) / np.linalg.norm(uref))
        res["fgmres_learned"].update({"degree": p.degree, "ratio": p.ratio, "train_seconds": train_s,
                                      "training": tinfo,
                                      "train_mesh": "16x8x8 block, seed 101, 8 white-noise samples, 20 CG steps, "
                                                    "validated by a solve of that block"})
        res["metric"] = ("s to 1e-10 FP64 rel resid (restart 50; the learned solver's seconds include its FP16 "
                         "operator build and eigenvalue estimate); err_vs_fp64 = ||u - u64|| / ||u64|| with u64 "
                         "the FP64 Jacobi-GMRES solution to 1e-13")
        line["solve"] = res
    if not a.no_solve and not a.no_learned_eval and rank == 0:
        del g
        line["learned_solve"] = _learned_eval(a)
    if a.panels > 0 and rank == 0:
        line["batched_panels"] = _panels_eval(a)
    if a.newmark_steps > 0 and rank == 0:
        line["newmark"] = _newmark_eval(a)
    if a.nmc_steps > 0 and rank == 0:
        line["newmark"] = line.get("newmark", {})
        line["newmark"]["factored_cases"] = _newmark_cases_eval(a, line["newmark"])
    if "newmark" in line:
        line["newmark"].pop("_final_disp_gmres", None)
    if not a.no_widened and rank == 0:
        line["widened"] = _widened_eval(a)
    # CPU baseline: oracle, 1 core, bounded sample
    if rank == 0:
        rate, dt = _oracle_rate(m, 1024, 1)
        if not a.no_cpu_legs:
            line["cpu_legs"] = _cpu_legs(a)
        line["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": 1, "kind": "port",
                                "sample": "brick8 element matrices of elements 1..1024 (oracle restatement, FP64, "
                                          "single thread)"}
        print(json.dumps(line))
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


def _learned_eval(a):
    """The learned-preconditioner evaluation: a 96x48x48 brick block (698,691 DOF) with a
    Gaussian-correlated log-normal modulus (correlation length 0.5 of the box width, sigma 0.65,
    seed 4000) solved to 1e-8 relative FP64 residual by the learned solver (the trained network
    shipped with the package when present, else the Chebyshev initialisation) and by the plain
    FP64 Jacobi-GMRES(50), CUDA events, the second call of each (the first also reported)."""
    from misc_gb300 import model as M
    from misc_gb300.astro import SOLVER_FGMRES_LEARNED, SOLVER_GMRES_JACOBI_FP64, precond_init
    from misc_gb300 import learned as LN
    nx = a.eval_nx
    m = M.config4_block(nx, nx // 2, nx // 2, 4000, corr_len=0.5, sigma=0.65)
    t0 = time.perf_counter()
    g, b = LN.block_system(m, fp32=True)
    if a.unrolled_cycles:
        g.set_option(2, 1)
    setup = time.perf_counter() - t0
    path = os.path.join(ROOT, "misc_gb300", "data", "precond_cfg4.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        p, src = LN.from_json(d), {"network": "trained", "training": d.get("meta")}
    else:
        p, src = precond_init(a.precond_degree, a.precond_ratio, 3), {"network": "Chebyshev initialisation"}
    out = {"workload": f"{nx}x{nx // 2}x{nx // 2} brick8, correlated log-normal E (corr 0.5 width, sigma 0.65, "
                       f"seed 4000)", "dof": g.n, "rtol": 1e-8, "setup_seconds": setup}
    # the per-node modulation trained on the config-4 family (committed weights), run beside
    mpath = os.path.join(ROOT, "misc_gb300", "data", "precond_mlp_cfg4.json")
    mlp = None
    if os.path.exists(mpath):
        with open(mpath) as f:
            dm = json.load(f)
        pm, mlp = LN.mlp_from_json(dm)
    runs = [("fgmres_learned", SOLVER_FGMRES_LEARNED, p, None)]
    if mlp is not None:
        runs.append(("fgmres_learned_modulated", SOLVER_FGMRES_LEARNED, pm, mlp))
    if not a.no_fp64:
        runs.append(("gmres_fp64", SOLVER_GMRES_JACOBI_FP64, None, None))
    sols = {}
    for name, meth, pc, ml in runs:
        kw = dict(method=meth, rtol=1e-8, restart=50, max_iters=a.solve_max_iters, allow_maxit=True, precond=pc,
                  mlp=ml)
        _, s1 = g.solve_static(b, **kw)
        # the FP32 matrix assembled again (same values): the second, timed learned solve rebuilds
        # its FP16 operator and eigenvalue estimate; workspace and captured graph are reused
        g.assemble_fp32()
        u, s2 = g.solve_static(b, **kw)
        sols[name] = u
        out[name] = {"seconds": s2.seconds, "first_call_seconds": s1.seconds, "iterations": s2.iterations,
                     "refinements": s2.refinements, "rel_residual": s2.rel_residual, "status": s2.status,
                     "conditional_graph": s2.conditional_graph, "fallback": s2.fallback,
                     "residual_kind": s2.residual_kind}
    out["fgmres_learned"].update({"degree": p.degree, "ratio": p.ratio, **src})
    if "fgmres_learned_modulated" in out:
        out["fgmres_learned_modulated"].update({
            "network": "trained", "hidden": mlp.hidden, "training": {k: dm["meta"].get(k) for k in (
                "family", "training_seeds", "samples_per_block", "optimizer", "loss_unmodulated")},
            "loss_last_epoch": dm["meta"]["loss_per_epoch"][-1],
            "note": "the per-node modulation (astro_precond_mlp) trained on 48 blocks of the family: its objective "
                    "falls 3x, the Krylov step count does not (a recorded negative result)"})
    if "gmres_fp64" in out:
        out["speedup_vs_fp64_gmres"] = out["gmres_fp64"]["seconds"] / out["fgmres_learned"]["seconds"]
        # both solutions against a tighter FP64 solve (Jacobi-GMRES to 1e-12, warm-started from the
        # FP64 solution): the error each result carries against the FP64 system's solution
        uref, sref = g.solve_static(b, u0=sols["gmres_fp64"], method=SOLVER_GMRES_JACOBI_FP64, rtol=1e-12,
                                    restart=50, max_iters=a.solve_max_iters, allow_maxit=True)
        for name, u in sols.items():
            out[name]["err_vs_fp64"] = float(np.linalg.norm(u - uref) / np.linalg.norm(uref))
        out["fp64_reference"] = {"rtol": 1e-12, "rel_residual": sref.rel_residual, "status": sref.status}
    # roofline of the solve's dominant kernel (the preconditioner hop, about 85 % of the learned
    # solve): its bytes per launch over its CUDA-event time; the operator (FP16 planes and columns,
    # about 157 MB at this size) streams from HBM and L2
    us, by = g.precond_time_hop(200)
    peaks = _peaks()
    hbm = peaks["hbm_gbs"] if peaks else 6800.0
    ach = by / (us * 1e-6) / 1e9
    out["hop_roofline"] = {"bound": "hbm", "kernel": "k_poly_hop<OpH,float,3>", "us_per_launch": us,
                           "bytes_per_launch": by, "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
                           "peak_source": "measured" if peaks else "fallback"}
    out["dof_per_second_learned"] = g.n / out["fgmres_learned"]["seconds"]
    return out


def _fp64_peak():
    """FP64 matrix-multiply rate of this GPU (torch.matmul float64 4096^3, cuBLAS DGEMM, best of 5,
    CUDA events): the denominator of the FP64-bound band factorisation."""
    import torch
    a = torch.randn(4096, 4096, dtype=torch.float64, device="cuda")
    b = torch.randn(4096, 4096, dtype=torch.float64, device="cuda")
    best = 1e30
    for _ in range(6):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1) * 1e-3)
    del a, b
    torch.cuda.empty_cache()
    return 2.0 * 4096 ** 3 / best / 1e12


def _panels_eval(a):
    """Batched panels with complex-step sensitivities: a.panels shell4 panels (n_x, n_y ~ U{8..96},
    t ~ U[0.01, 0.1], one clamped edge, pressure ~ U[1e2, 1e4], seeds 1000 + panel) as one model;
    32 thickness-group design variables.  The pipeline (assembly, loads, factorisation,
    displacement solve, 32 complex-step right-hand sides at the solved state, their solve) runs
    once; the cluster size of the factorisation is autotuned over 2, 4 and 8 CTAs per panel on the
    batch itself; then the timed unit, the band LDL^T of every panel plus the 33-right-hand-side
    solve, is repeated three times (median, host clock around synchronous calls)."""
    import gc
    from misc_gb300 import model as M
    from misc_gb300 import panels as PN
    from misc_gb300.astro import AstroGPU
    gc.collect()
    m = M.panel_batch(num_panels=a.panels)
    t0 = time.perf_counter()
    g = AstroGPU(m)
    ctx_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    u, du, t = PN.solve_batch(g, m, 32, cluster_size=8)
    pipe_s = time.perf_counter() - t0
    if a.panels_cluster:
        best, tune = a.panels_cluster, {}
    else:
        tune = {cs: g.panels_factor(cs).factor_seconds for cs in (2, 4, 8)}
        best = min(tune, key=tune.get)
    B = np.asfortranarray(np.column_stack([t["f"], t["R"]]))
    reps = []
    for _ in range(3):
        t0 = time.perf_counter()
        info = g.panels_factor(best)
        X, si = g.panels_solve(B)
        reps.append((time.perf_counter() - t0, info.factor_seconds, si.solve_seconds))
    reps.sort()
    tot, fac, sol = reps[1]
    r = g.apply_operator(X[:, 0], 64) - B[:, 0]
    # the solve's other sweep modes on the same factor: FP64 sweeps, double-float sweeps alone
    from misc_gb300.astro import OPT_PANELS_SOLVE
    sweeps = {}
    for mode, name in ((1, "fp64"), (2, "double_float_alone")):
        g.set_option(OPT_PANELS_SOLVE, mode)
        Xm, sm = g.panels_solve(B)
        rm = g.apply_operator(Xm[:, 0], 64) - B[:, 0]
        sweeps[name] = {"solve_seconds": sm.solve_seconds,
                        "rel_diff_vs_default": float(np.linalg.norm(Xm - X) / np.linalg.norm(X)),
                        "rel_residual_u": float(np.linalg.norm(rm) / np.linalg.norm(B[:, 0]))}
        del Xm
    g.set_option(OPT_PANELS_SOLVE, 0)
    # the same unit with the factorisation in double-float (a 48-bit factor; the default solve
    # refines against the FP64 operator)
    from misc_gb300.astro import OPT_BAND_FP64_UPDATE
    g.set_option(OPT_BAND_FP64_UPDATE, 3)
    reps3 = []
    for _ in range(3):
        t0 = time.perf_counter()
        info3 = g.panels_factor(best)
        X3, si3 = g.panels_solve(B)
        reps3.append((time.perf_counter() - t0, info3.factor_seconds, si3.solve_seconds))
    g.set_option(OPT_BAND_FP64_UPDATE, 1)
    reps3.sort()
    r3 = g.apply_operator(X3[:, 0], 64) - B[:, 0]
    df_update = {"seconds": reps3[1][0], "factor_seconds": reps3[1][1], "solve_seconds": reps3[1][2],
                 "rel_residual_u": float(np.linalg.norm(r3) / np.linalg.norm(B[:, 0])),
                 "rel_diff_vs_fp64_update": float(np.linalg.norm(X3 - X) / np.linalg.norm(X))}
    del X3
    # FP64 multiply-adds of the tile algorithm (32^3 per trailing tile update, the diagonal and
    # panel tiles) and of the two sweeps per right-hand side
    fma_f, fma_s = 0.0, 0.0
    for p in range(len(m.panel_n)):
        nx, ny = m.panel_n[p]
        n = (nx + 1) * (ny + 1) * 6
        bw = (min(nx, ny) + 2) * 6 + 5
        bt, nbc = (bw + 31) // 32, (n + 31) // 32
        fma_f += nbc * (bt * (bt + 1) / 2 * 32 ** 3 + bt * 32 * 32 * 31 / 2 + 32 ** 3 / 6)
        fma_s += 2 * nbc * (bt + 1) * 1024 * B.shape[1]
    # the same factorisation with the trailing tile updates on the tensor cores (FP64-exact BF16
    # slice emulation; the FP64 update is the default), and the two solutions' distance
    from misc_gb300.astro import OPT_BAND_FP64_UPDATE
    g.set_option(OPT_BAND_FP64_UPDATE, 0)
    facTcs = []
    for _ in range(2):
        facTcs.append(g.panels_factor(best).factor_seconds)
    Xtc, _ = g.panels_solve(B)
    # the same emulation on mma.sync (identical factor)
    g.set_option(OPT_BAND_FP64_UPDATE, 2)
    facMma = min(g.panels_factor(best).factor_seconds for _ in range(2))
    g.set_option(OPT_BAND_FP64_UPDATE, 1)
    g.panels_factor(best)
    facTc = min(facTcs)
    diffTc = float(np.linalg.norm(Xtc - X) / np.linalg.norm(X))
    try:
        pk = _fp64_peak()
    except Exception:
        pk = None
    out = {"metric": "s per batch: band LDL^T of every panel + the 33-right-hand-side solve (u and 32 "
                     "complex-step design sensitivities)",
           "trailing_update": "FP64 (the tensor-core emulation measured beside it)",
           "tensor_core_update_factor_seconds": facTc, "tensor_core_rel_diff_vs_fp64_update": diffTc,
           "tensor_core_update_kernel": "tcgen05 (BF16 slices, accumulators in tensor memory)",
           "mma_sync_update_factor_seconds": facMma,
           "seconds": tot, "factor_seconds": fac, "solve_seconds": sol,
           "solve_sweeps": "double-float sweeps from copies of the FP64 factor + one FP64 refinement pass",
           "solve_other_sweeps": sweeps, "double_float_factorisation": df_update, "panels": int(info.num_panels),
           "elements": m.num_els, "dof": g.n, "max_bandwidth": info.max_bandwidth, "band_bytes": info.band_bytes,
           "cluster_size": best, "autotune_factor_seconds": tune, "workers": info.workers,
           "rel_residual_u": float(np.linalg.norm(r) / np.linalg.norm(B[:, 0])),
           "pipeline_first_run": {"ctx_seconds": ctx_s, "total_seconds": pipe_s,
                                  **{k: v for k, v in t.items() if k.endswith("_s")}},
           "dof_rhs_per_second": g.n * B.shape[1] / tot,
           "fp64_roofline": {"bound": "fp64", "kernel": "k_band_ldl", "fma": fma_f,
                             "achieved_tflops": 2 * fma_f / fac / 1e12, "peak_tflops": pk,
                             "frac": (2 * fma_f / fac / 1e12 / pk) if pk else None,
                             "achieved_tflops_tensor_core_update": 2 * fma_f / facTc / 1e12,
                             "achieved_tflops_double_float_factor": 2 * fma_f / df_update["factor_seconds"] / 1e12,
                             "note": "the factor's FP64 multiply-adds over its time; the tensor-core "
                                     "emulation's and the double-float factor's rates are the same count "
                                     "over their own times",
                             "peak_source": "measured: torch.matmul float64 4096^3 (cuBLAS DGEMM) on this GPU",
                             "solve_fma": fma_s, "solve_tflops": 2 * fma_s / sol / 1e12}}
    del g
    gc.collect()
    return out


def _newmark_eval(a):
    """Implicit Newmark dynamics on the config-5 plate: 128x128 shell4 on 1 x 1 m, t = 0.01,
    E = 7e10, nu = 0.33, rho = 2700, simply supported edges (w = 0), beta 0.25, gamma 0.5,
    dt = 1e-5, point force 100 sin(2 pi 500 t) N at the centre; a.newmark_steps steps of the
    device time loop per method (the second run timed; CUDA events), each step solved to 1e-10:
    FP64 Jacobi-GMRES and the learned FGMRES (degree 8, ratio 100)."""
    import gc
    from misc_gb300 import model as M
    from misc_gb300.astro import OPT_SHELL_MEAN_ROT_TERM, SOLVER_FGMRES_LEARNED, AstroGPU, precond_init
    gc.collect()
    nx = 128
    m = M.plate_shell(nx=nx, ny=nx, lx=1.0, ly=1.0, t=0.01, E=7e10, nu=0.33, rho=2700.0, pressure=0.0, clamp="ss",
                      y0=0.0)
    g = AstroGPU(m)
    # the consistent shell tangent: with the reference's default tangent (not the derivative of
    # its residual) this implicit loop diverges (|u| about 1e12 by step 117 at this size)
    g.set_option(OPT_SHELL_MEAN_ROT_TERM, 1)
    centre = (nx // 2) * (nx + 1) + nx // 2 + 1
    pattern = np.zeros(g.n)
    pattern[g.n_dof_index[centre - 1, 2] - 1] = 1.0
    steps, dt = a.newmark_steps, 1e-5
    amp = 100.0 * np.sin(2 * np.pi * 500.0 * dt * np.arange(1, steps + 1))
    out = {"workload": "128x128 shell4 plate (99,846 DOF), simply supported, dt 1e-5, centre point force "
                       "100 sin(2 pi 500 t) N", "steps": steps, "rtol": 1e-10,
           "tangent": "consistent (ASTRO_OPT_SHELL_MEAN_ROT_TERM)"}
    res = {}
    for name, kw in (("gmres_fp64", {}), ("fgmres_learned", dict(method=SOLVER_FGMRES_LEARNED,
                                                                  precond=precond_init(8, 100.0, 6)))):
        for _ in range(2):
            u, v, acc, iu, hist, st = g.newmark_run(steps, dt, 0.25, 0.5, pattern, amp, rtol=1e-10, history=False, **kw)
        res[name] = u
        if name == "gmres_fp64":
            out["_final_disp_gmres"] = u
        out[name] = {"ms_per_step": 1e3 * st.seconds / steps, "seconds": st.seconds, "inner_iterations": st.iterations,
                     "refinements": st.refinements, "status": st.status}
    out["speedup_learned_vs_fp64"] = out["gmres_fp64"]["ms_per_step"] / out["fgmres_learned"]["ms_per_step"]
    out["rel_diff_final_disp"] = float(np.linalg.norm(res["fgmres_learned"] - res["gmres_fp64"]) /
                                       max(np.linalg.norm(res["gmres_fp64"]), 1e-300))
    del g
    gc.collect()
    return out


def _newmark_cases_eval(a, nm):
    """Config 5 as specified: the 128x128 plate's K_eff + C^T C factored once (FP64 band LDL^T,
    tensor-core trailing updates), the centre force and 16 seeded random point-load cases
    (model.config5_cases) stepped together, every step one cluster band solve of all cases, the
    step a CUDA graph launched a.nmc_steps times (CUDA events around the launches).  The
    linearised loop's centre case is also run for the Newmark leg's steps and compared with that
    leg's element-residual FP64 GMRES loop."""
    import gc
    from misc_gb300 import model as M
    from misc_gb300.astro import OPT_SHELL_MEAN_ROT_TERM, AstroGPU
    gc.collect()
    nx, dt = 128, 1e-5
    m = M.plate_shell(nx=nx, ny=nx, lx=1.0, ly=1.0, t=0.01, E=7e10, nu=0.33, rho=2700.0, pressure=0.0, clamp="ss",
                      y0=0.0)
    g = AstroGPU(m)
    g.set_option(OPT_SHELL_MEAN_ROT_TERM, 1)
    steps = a.nmc_steps
    P, A = M.config5_cases(m, g.n_dof_index, steps, dt, num_random=a.nmc_cases - 1)
    # the autotuner picks the solve's CTAs per case (2, 4, 8) on this factorisation: one step to
    # prepare it, then the timed candidates (kept in a scratch cache file, reported below)
    import tempfile
    from misc_gb300.astro import TUNE_CASES_CLUSTER
    g.newmark_cases(dt, P, A[:, :1])
    with tempfile.TemporaryDirectory() as td:
        cache = os.path.join(td, "tune.txt")
        choice = g.autotune(TUNE_CASES_CLUSTER, cache)[2]
        with open(cache) as f:
            tune = [ln.split() for ln in f if ln.strip()]
    u, v, acc, _, info = g.newmark_cases(dt, P, A)
    ms = 1e3 * info.step_seconds / max(steps, 1)
    nbc = (g.n + 31) // 32
    out = {"workload": f"128x128 shell4 plate (99,846 DOF), simply supported, dt 1e-5, {a.nmc_cases} load cases "
                       "(centre force 100 sin(2 pi 500 t) N + seeded random point forces, model.config5_cases)",
           "steps": steps, "cases": a.nmc_cases, "ms_per_step": ms, "ms_per_case_step": ms / a.nmc_cases,
           "step_seconds": info.step_seconds, "factor_seconds": info.factor_seconds,
           "prepare_seconds": info.prepare_seconds, "band_bytes": info.band_bytes,
           "df_band_bytes": info.df_band_bytes, "bandwidth_dof": info.bandwidth,
           "last_step_rel_residual": info.last_rel_residual, "graph_nodes": info.graph_nodes,
           "kernels_per_step": info.kernels_per_step, "cluster_size": info.cluster_size,
           "autotune": {"choice": choice, "cache_lines": tune,
                        "note": "astro_autotune(ASTRO_TUNE_CASES_CLUSTER): the fastest of 2, 4, 8 CTAs per case, "
                                "seconds per solve of all cases"},
           "solve_chain": {"block_rows_per_sweep": nbc, "us_per_block_row": 1e3 * ms / (2 * nbc),
                           "note": "each step solves every case by forward and backward sweeps over the band's "
                                   "32-row block rows; a row waits for the previous one (one cluster barrier per "
                                   "row), so the step time is the chain of 2 x block rows, not HBM traffic"},
           "method": "K_eff + C^T C factored once (FP64 band LDL^T), linearised residual through the assembled "
                     "K and K_eff, cluster band solve of all cases per step (double-float), CUDA graph per step"}
    g2 = g
    if a.newmark_steps > 0 and "gmres_fp64" in nm:
        k = a.newmark_steps
        t = dt * np.arange(1, k + 1)
        u1, *_ = g2.newmark_cases(dt, P[:1], (100.0 * np.sin(2 * np.pi * 500.0 * t))[None])
        ref = nm.get("_final_disp_gmres")
        if ref is not None:
            out["centre_case_vs_element_loop"] = {
                "steps": k, "rel_diff_final_disp": float(np.linalg.norm(u1[0] - ref) / max(np.linalg.norm(ref), 1e-300)),
                "note": "linearised loop against the element-residual loop (FP64 GMRES, consistent tangent)"}
        out["gmres_element_loop_ms_per_step_one_case"] = nm["gmres_fp64"]["ms_per_step"]
    del g, g2
    gc.collect()
    return out


def _cpu_legs(a):
    """The reference path timed on this machine's host cores through the oracle (the C++
    restatement of the reference's algorithms, single thread, built -O2; the reference itself is
    serial Fortran built at -O0 and cannot be compiled here), on bounded samples:
    config 1 (40x8 shell cantilever): element matrices, the assembly (getElasticSolnLoad),
    convertToLTri + the skyline LDL^T factor and solve, the reference gMRes with the skyline
    preconditioner, the tip deflection;
    config 2 (64x32x32 block): the assembly, and FP64 Jacobi-GMRES(50) (scipy, the GPU
    comparator's algorithm) for a bounded number of steps, extrapolated to the GPU comparator's
    step count at 1e-10;
    config 5 (128x128 plate, consistent shell tangent): the factorisation of K_eff (scipy
    SuperLU) and the first steps of the reference's loop (element residual, constraint load,
    condensation, solve, recovery), per step."""
    import gc
    import scipy.sparse.linalg as spla
    from misc_gb300 import model as M
    from oracle import Oracle
    from oracle import oracle as OO
    out = {"kind": "port", "cores": 1, "threads_note": "oracle single thread; scipy SpMV single thread",
           "host": {"nproc": os.cpu_count()}}
    # config 1
    m = M.config1()
    o = Oracle(m)
    t0 = time.perf_counter()
    o.element_matrices()
    t_el = time.perf_counter() - t0
    t0 = time.perf_counter()
    load, iload, mat, cols, imat = o.el_soln_load(1)
    t_as = time.perf_counter() - t0
    mm, mr = o.scale_mpc(mat)
    f = o.applied_load()
    b = load + f
    o.constraint_load(mm, mr, np.zeros(o.n), b)
    rhs = o.update_external_rhs(b, iload[:o.int_vec_size], imat)
    t0 = time.perf_counter()
    lt = o.convert_to_ltri(mat, cols, mm)
    fac = o.ldl_fact(lt, o.lt_range)
    t_fac = time.perf_counter() - t0
    t0 = time.perf_counter()
    u = o.ldl_solve(fac, o.lt_range, rhs)
    t_sol = time.perf_counter() - t0
    t0 = time.perf_counter()
    ug, cyc = o.gmres(mat, cols, mm, fac, rhs)
    t_gm = time.perf_counter() - t0
    tip = [k for k in range(m.num_nodes) if abs(m.node_list[k, 0] - 10.0) < 1e-9]
    w_tip = float(np.mean([u[o.n_dof_index[k, 2] - 1] for k in tip]))
    out["config1"] = {"workload": "40x8 shell4 cantilever (2,214 DOF)", "element_matrices_per_s": m.num_els / t_el,
                      "assembly_s": t_as, "ldl_fact_s": t_fac, "ldl_solve_s": t_sol, "ref_gmres_s": t_gm,
                      "ref_gmres_cycles": int(cyc), "tip_w": w_tip}
    del o
    gc.collect()
    # config 2
    m = M.config2(nx=a.nx, ny=a.ny, nz=a.nz)
    o = Oracle(m)
    t0 = time.perf_counter()
    load, iload, mat, cols, imat = o.el_soln_load(1)
    t_as = time.perf_counter() - t0
    mm, mr = o.scale_mpc(mat)
    Cm = o.mpc_scipy(mm)
    A = (o.csr_scipy(mat, cols) + Cm.T @ Cm).tocsr()
    b = o.applied_load() + load
    o.constraint_load(mm, mr, np.zeros(o.n), b)
    dinv = 1.0 / A.diagonal()
    Mj = spla.LinearOperator(A.shape, matvec=lambda x: dinv * x)
    steps = 300
    it = [0]
    t0 = time.perf_counter()
    spla.gmres(A, b, rtol=1e-10, restart=50, maxiter=steps // 50, M=Mj, callback=lambda r: it.__setitem__(0, it[0] + 1),
               callback_type="pr_norm")
    t_gm = time.perf_counter() - t0
    gpu_steps = 7735
    out["config2"] = {"workload": f"{a.nx}x{a.ny}x{a.nz} brick8 block ({o.n} DOF)", "assembly_s": t_as,
                      "element_matrices_per_s": m.num_els / t_as,
                      "jacobi_gmres50": {"sample_steps": it[0], "sample_s": t_gm, "s_per_step": t_gm / max(it[0], 1),
                                         "extrapolated_s_to_1e-10": t_gm / max(it[0], 1) * gpu_steps,
                                         "extrapolated_at_steps": gpu_steps,
                                         "note": "the step count of the GPU's FP64 Jacobi-GMRES(50) to 1e-10 on this "
                                                 "block"}}
    del o, A
    gc.collect()
    # config 5
    L = OO._lib()
    import ctypes
    L.orc_set_quirk.argtypes = [ctypes.c_int, ctypes.c_int]
    L.orc_set_quirk(1, 1)
    try:
        nx, dt, nsteps = 128, 1e-5, 3
        m = M.plate_shell(nx=nx, ny=nx, lx=1.0, ly=1.0, t=0.01, E=7e10, nu=0.33, rho=2700.0, pressure=0.0, clamp="ss",
                          y0=0.0)
        o = Oracle(m)
        n, ni = o.n, o.int_vec_size
        centre = (nx // 2) * (nx + 1) + nx // 2 + 1
        pattern = np.zeros(n)
        pattern[o.n_dof_index[centre - 1, 2] - 1] = 1.0
        amp = 100.0 * np.sin(2 * np.pi * 500.0 * dt * np.arange(1, nsteps + 1))
        u, up, vp, ap = (np.zeros(n) for _ in range(4))
        iu, iup = np.zeros(ni), np.zeros(ni)
        st = lambda: M.make_state(n, disp=u, prev_disp=up, prev_vel=vp, prev_acc=ap, internal_disp=iu,
                                  prev_int_disp=iup, dynamic=1, beta=0.25, gamma=0.5, del_t=dt)
        t0 = time.perf_counter()
        _, _, mat, cols, imat = o.el_soln_load(1, state=st())
        mm, mr = o.scale_mpc(mat)
        Cm = o.mpc_scipy(mm)
        lu = spla.splu((o.csr_scipy(mat, cols) + Cm.T @ Cm).tocsc())
        t_fac = time.perf_counter() - t0
        c1, c2 = 2.0, 2.0 / (dt * dt)
        t0 = time.perf_counter()
        for k in range(nsteps):
            load, iload, *_ = o.el_soln_load(0, state=st())
            load = load + amp[k] * pattern
            o.constraint_load(mm, mr, u, load)
            r = o.update_external_rhs(load, iload[:ni], imat)
            du = lu.solve(r)
            iu = o.update_internal_soln(du, iu, iload[:ni], imat)[:ni]
            u = u + du
            acc = c1 * (c2 * (u - up - dt * vp) - (1.0 - 2.0 * 0.25) * ap)
            vel = vp + dt * (0.5 * ap + 0.5 * acc)
            up, vp, ap, iup = u.copy(), vel, acc, iu.copy()
        t_steps = time.perf_counter() - t0
        out["config5"] = {"workload": "128x128 shell4 plate (99,846 DOF), one load case, consistent tangent",
                          "assembly_and_factor_s": t_fac, "steps_timed": nsteps, "s_per_step": t_steps / nsteps,
                          "extrapolated_2000_steps_one_case_s": t_steps / nsteps * 2000,
                          "solver": "scipy SuperLU of K_eff + C^T C (the reference's skyline LDL^T of this K_eff "
                                    "would take longer)"}
    finally:
        L.orc_set_quirk(1, 0)
    return out


def _widened_eval(a):
    """Device times of the widened rows on the 64x32x32 brick block (212,355 DOF), CUDA-synchronous
    host clock, best of three: the gravitational body load (astro_body_load), the static design
    gradient for 8 modulus variables (astro_total_dldd: adjoint solve by the learned solver to
    1e-10 plus eight complex-step dR/dd), the thermal conductivity assembly
    (astro_thermal_soln_load) and the thermal CG solve to 1e-10 with the x = 0 face held."""
    import gc
    from misc_gb300 import model as M
    from misc_gb300.astro import SOLVER_FGMRES_LEARNED, AstroGPU, make_state, thermal_props
    gc.collect()
    m = M.add_design_variables(M.config2(), 8, M.DCAT_ELASTIC_MODULUS)
    g = AstroGPU(m)
    g.getElasticSolnLoad(1, export=False)
    g.assemble_fp32()
    g.scaleElasticMPC()
    b = g.static_rhs()
    u, _ = g.solve_static(b, method=SOLVER_FGMRES_LEARNED, rtol=1e-10)
    st = make_state(g.n, disp=u)

    def best(fn, k=3):
        ts = []
        for _ in range(k):
            t0 = time.perf_counter()
            fn()
            ts.append(time.perf_counter() - t0)
        return min(ts)
    out = {"workload": "64x32x32 brick8 block (212,355 DOF), 8 elastic-modulus design variables"}
    out["body_load_gravity_s"] = best(lambda: g.body_load(1, [0.0, 0.0, -9.81]))
    w = np.random.default_rng(3).standard_normal(g.n)
    out["total_dldd_s"] = best(lambda: g.getTotaldLdD(w, state=st, rtol=1e-10, method=SOLVER_FGMRES_LEARNED), k=2)
    nm = len(m.material_density)
    X = m.node_list
    left = np.nonzero(X[:, 0] == 0)[0] + 1
    mpc = (np.arange(len(left) + 1), left, np.ones(len(left)), np.full(len(left), 100.0))
    g.thermal_setup(thermal_props(np.tile([45.0, 45.0, 45.0, 0.0, 0.0, 0.0], (nm, 1)), np.full(nm, 460.0), mpc))
    out["thermal_assembly_s"] = best(lambda: g.getThermalSolnLoad(1, export=False))
    g.scaleThermalMPC()
    q = g.thermal_heat_gen(1.0e3)
    rhs = g.getThermalConstraintLoad(None, q.copy())
    x, ts = g.thermal_solve(rhs, rtol=1e-10)
    out["thermal_solve"] = {"seconds": ts.seconds, "iterations": ts.iterations, "rel_residual": ts.rel_residual,
                            "nodes": m.num_nodes}
    del g
    gc.collect()
    # config 1 (40x8 shell cantilever): the reference's skyline path through the C ABI with host
    # buffers (convertToLTri from the device matrix, getSparseLDLFact, solveSparseLDLFact), and
    # the factor of the device-resident profile
    m1 = M.config1()
    g1 = AstroGPU(m1)
    g1.getElasticSolnLoad(1, export=False)
    g1.scaleElasticMPC()
    lt = g1.convertToLTri()
    fac = g1.getSparseLDLFact(lt, g1.lt_range)
    rhs = np.random.default_rng(5).standard_normal(g1.n)

    def resident():  # the profile is factored in place: a fresh copy before each timed factor
        g1.convertToLTri()
        t0 = time.perf_counter()
        g1._check(g1.L.astro_ldl_fact_resident(g1.h))
        return time.perf_counter() - t0
    out["config1_skyline"] = {
        "workload": f"40x8 shell4 cantilever ({g1.n} DOF, profile {g1.lt_size} entries)",
        "convert_to_ltri_s": best(g1.convertToLTri),
        "ldl_fact_s": best(lambda: g1.getSparseLDLFact(lt, g1.lt_range)),
        "ldl_fact_resident_s": min(resident() for _ in range(3)),
        "ldl_solve_s": best(lambda: g1.solveSparseLDLFact(rhs, fac, g1.lt_range)),
        "path": "one 512-thread CTA sweeping the profile's rows, as the reference's row-sequential algorithm; "
                "host clock, host buffers copied in and out"}
    del g1
    gc.collect()
    return out


def main():
    a = _parse()
    if a.panels_only:
        print(json.dumps(_panels_eval(a)))
        return 0
    if a.learned_only:
        print(json.dumps(_learned_eval(a)))
        return 0
    if a.impl == "reference":
        return run_reference(a)
    return run_ours(a)


if __name__ == "__main__":
    sys.exit(main())
