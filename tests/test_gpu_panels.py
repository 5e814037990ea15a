"""GPU parity of the batched panel solver (astro_panels_factor / astro_panels_solve): the band
LDL^T of K + C^T C of every panel in one launch against a sparse direct solve of the oracle's
assembled system, for several cluster sizes, multi-tile bands, many right-hand sides, bricks
(3 DOF per node) and the complex-step sensitivity pipeline.  Solutions agree to 1e-10 relative
and the FP64 residual ||A X - B|| is within 10x of the sparse direct solve's per column.  The
solves run in the default mode (double-float sweeps and one FP64 refinement pass) unless a test
selects another."""
import numpy as np
import pytest
import scipy.sparse.linalg as spla

from misc_gb300 import model as M
from misc_gb300 import panels as PN
from misc_gb300.astro import AstroError, AstroGPU
from oracle import Oracle

pytestmark = pytest.mark.gpu


def _check(A, X, B, Xref, tol=1e-10):
    X, B, Xref = X.reshape(len(B), -1), B.reshape(len(B), -1), Xref.reshape(len(B), -1)
    for c in range(B.shape[1]):
        assert np.linalg.norm(X[:, c] - Xref[:, c]) <= tol * np.linalg.norm(Xref[:, c]), c
        # backward error no worse than the sparse direct solve's (the scaled penalty rows put
        # 1e20-size entries into A, so the residual is set by their rounding)
        r, r_ref = np.linalg.norm(A @ X[:, c] - B[:, c]), np.linalg.norm(A @ Xref[:, c] - B[:, c])
        assert r <= 10.0 * r_ref + 1e-14 * np.linalg.norm(B[:, c]), (c, r, r_ref)


@pytest.fixture(scope="module")
def batch():
    m = M.panel_batch(num_panels=6, n_range=(2, 9), t_range=(0.05, 0.1), n_dvars=4)
    g, o = AstroGPU(m), Oracle(m)
    g.getElasticSolnLoad(1, export=False)
    g.scaleElasticMPC()
    A, *_ = o.static_system()
    return m, g, o, A.tocsc()


@pytest.mark.parametrize("cs", [1, 2, 8])
def test_panels_match_direct_solve(batch, cs):
    m, g, o, A = batch
    info = g.panels_factor(cs)
    assert info.num_panels == 6 and info.cluster_size == cs
    B = np.random.default_rng(cs).standard_normal((g.n, 11))
    X, sinfo = g.panels_solve(B)
    _check(A, X, B, spla.splu(A).solve(B))


def test_panels_single_rhs_and_refactor(batch):
    """One right-hand side; a new assembly makes the factor stale until refactored (the batched
    entry point refactors by itself)."""
    m, g, o, A = batch
    g.panels_factor()
    b = np.random.default_rng(5).standard_normal(g.n)
    x, _ = g.panels_solve(b)
    _check(A, x, b, spla.spsolve(A, b))
    g.getElasticSolnLoad(1, export=False)
    g.scaleElasticMPC()
    with pytest.raises(AstroError) as e:
        g.panels_solve(b)
    assert e.value.code == 8
    x2, _ = g.panels_solve(b, batched=True)
    _check(A, x2, b, spla.spsolve(A, b))
    with pytest.raises(AstroError):
        g.panels_factor(3)


def test_panels_multi_tile_bands():
    """Panels whose bands span several 32-wide tiles (bt up to 5) and many block columns."""
    m = M.panel_batch(num_panels=3, seed0=7, n_range=(14, 22), t_range=(0.2, 0.25), n_dvars=0)
    g, o = AstroGPU(m), Oracle(m)
    g.getElasticSolnLoad(1, export=False)
    g.scaleElasticMPC()
    A = o.static_system()[0].tocsc()
    info = g.panels_factor(4)
    assert info.max_bandwidth > 96
    B = np.random.default_rng(1).standard_normal((g.n, 17))
    X, _ = g.panels_solve(B)
    _check(A, X, B, spla.splu(A).solve(B))


def test_panels_on_a_brick_block():
    """3 DOF per node, one component, jittered nodes (the ordering is only a band heuristic)."""
    m = M.hex_block(6, 4, 3, lx=1.5, ly=1.0, lz=0.75, seed=4)
    g, o = AstroGPU(m), Oracle(m)
    g.getElasticSolnLoad(1, export=False)
    g.scaleElasticMPC()
    A, b, *_ = o.static_system()
    A = A.tocsc()
    g.panels_factor(2)
    x, _ = g.panels_solve(b)
    _check(A, x, b, spla.spsolve(A, b))


def test_panel_sensitivity_pipeline(batch):
    """Pressure load per panel, the complex-step sensitivity right-hand sides at the solved state
    (against the oracle) and the batched solves of all of them."""
    m, g, o, A = batch
    u, du, t = PN.solve_batch(g, m, 4)
    load, iload, mat, cols, imat = o.el_soln_load(1)
    f = sum(_surface(o, m, m.panel_el_ptr[p], m.panel_el_ptr[p + 1], m.panel_pressure[p]) for p in range(6))
    assert np.linalg.norm(t["f"] - f) <= 1e-12 * np.linalg.norm(f)
    _check(A, u, f, spla.spsolve(A, f))
    st = t["state"]
    for d in range(1, 5):
        dr, idr = o.drdd_complex(d, state=st)
        r = o.update_external_rhs(dr, idr, imat)
        assert np.linalg.norm(t["R"][:, d - 1] - r) <= 1e-9 * np.linalg.norm(r), d
    _check(A, -du, t["R"], spla.splu(A).solve(t["R"]))


def test_panel_sensitivities_match_central_differences():
    """du/dd of the batched pipeline against central differences of the oracle's direct solves
    with a group's thickness perturbed: thin panels, a load small enough for the element's
    nonlinear terms to vanish, and the consistent shell tangent on both sides (the reference's
    default tangent is not the derivative of its residual, so its sensitivities and central
    differences disagree)."""
    import ctypes
    from oracle.oracle import _lib
    from misc_gb300.astro import OPT_SHELL_MEAN_ROT_TERM

    def mk(dv=None):
        m = M.panel_batch(num_panels=4, n_range=(2, 7), t_range=(0.002, 0.004), h=0.01, n_dvars=4)
        if dv is not None:
            m.d_value = np.asarray(dv, np.float64)
        return m

    L = _lib()
    L.orc_set_quirk.argtypes = [ctypes.c_int, ctypes.c_int]
    L.orc_set_quirk(1, 1)
    try:
        m = mk()
        g, o = AstroGPU(m), Oracle(m)
        g.set_option(OPT_SHELL_MEAN_ROT_TERM, 1)
        ls = 1e-6
        u, du, t = PN.solve_batch(g, m, 4, load_scale=ls)
        f = t["f"]
        step = 1e-7
        for d in (1, 3):
            e = np.zeros(4)
            e[d - 1] = step
            us = [spla.spsolve(Oracle(mk(s * e)).static_system()[0].tocsc(), f) for s in (1.0, -1.0)]
            fd = (us[0] - us[1]) / (2 * step)
            assert np.linalg.norm(du[:, d - 1] - fd) <= 3e-5 * np.linalg.norm(fd), d
    finally:
        L.orc_set_quirk(1, 0)


def _surface(o, m, e0, e1, pressure):
    import ctypes as C
    from oracle.oracle import _d, _i
    load = np.zeros(o.n)
    fe = np.ascontiguousarray(m.face_el[e0:e1], np.int32)
    fn = np.ascontiguousarray(m.face_num[e0:e1], np.int32)
    tr = np.zeros(3)
    o.L.orc_surface_load(o.h, len(fe), _i(fe), _i(fn), _d(tr), C.c_double(pressure), _d(load))
    return load


def test_condensed_complex_step_batch(batch):
    """astro_drdd_complex_condensed equals astro_drdd_complex + astro_update_external_rhs per
    design variable, bit for bit."""
    m, g, o, A = batch
    g.getElasticSolnLoad(1, export=False)
    g.scaleElasticMPC()
    rng = np.random.default_rng(9)
    st = M.make_state(g.n, disp=1e-5 * rng.standard_normal(g.n), internal_disp=1e-6 * rng.standard_normal(g.int_vec_size))
    R = g.drdd_condensed([3, 1, 4], state=st)
    for k, d in enumerate((3, 1, 4)):
        dr, idr = g.getdRelasticdD(d, state=st)
        assert np.array_equal(R[:, k], g.updateExternalRHS(dr, idr))
    with pytest.raises(AstroError):
        g.drdd_condensed([5])


def test_tensor_core_update_matches_fp64_update(batch):
    """The band factor's trailing updates on the tensor cores (FP64-exact BF16 slice emulation,
    an option) against the same factorisation with FP64 updates (the default): the two solutions
    agree to 1e-10, and the emulated one matches the sparse direct solve as the FP64 one does.
    The tcgen05 emulation (option value 0) and the mma.sync one (2) sum every level exactly and
    combine the levels in the same order: their factors, hence their solutions, are identical."""
    from misc_gb300.astro import OPT_BAND_FP64_UPDATE
    m, g, o, A = batch
    B = np.random.default_rng(17).standard_normal((g.n, 9))
    Xr = spla.splu(A).solve(B)
    try:
        g.set_option(OPT_BAND_FP64_UPDATE, 0)
        g.panels_factor(4)
        Xtc, _ = g.panels_solve(B)
        g.set_option(OPT_BAND_FP64_UPDATE, 2)
        g.panels_factor(4)
        Xmma, _ = g.panels_solve(B)
    finally:
        g.set_option(OPT_BAND_FP64_UPDATE, 1)
    g.panels_factor(4)
    X64, _ = g.panels_solve(B)
    _check(A, X64, B, Xr)
    _check(A, Xtc, B, Xr)
    assert np.array_equal(Xtc, Xmma)
    assert np.linalg.norm(Xtc - X64) <= 1e-10 * np.linalg.norm(X64)


def test_solve_sweep_arithmetic(batch):
    """astro_panels_solve's three sweep modes on one factor: double-float sweeps with one FP64
    refinement pass (the default), FP64 sweeps, and double-float sweeps alone.  The first two
    meet the sparse direct solve as above and agree to 1e-10; the double-float sweeps alone are
    within 1e-8 of the FP64 ones (about 48 significant bits per operation)."""
    from misc_gb300.astro import OPT_PANELS_SOLVE
    m, g, o, A = batch
    B = np.random.default_rng(23).standard_normal((g.n, 13))
    Xr = spla.splu(A).solve(B)
    g.panels_factor(4)
    X = {}
    try:
        for mode in (0, 1, 2):
            g.set_option(OPT_PANELS_SOLVE, mode)
            X[mode], _ = g.panels_solve(B)
    finally:
        g.set_option(OPT_PANELS_SOLVE, 0)
    _check(A, X[0], B, Xr)
    _check(A, X[1], B, Xr)
    assert np.linalg.norm(X[0] - X[1]) <= 1e-10 * np.linalg.norm(X[1])
    assert np.linalg.norm(X[2] - X[1]) <= 1e-8 * np.linalg.norm(X[1])
    with pytest.raises(AstroError):
        g.set_option(OPT_PANELS_SOLVE, 3)


def test_double_float_factorisation_with_refined_solve(batch):
    """The band factor carried in double-float throughout (option value 3: about 48 significant
    bits per operation) and the default solve (double-float sweeps, one FP64 refinement against the operator):
    the solution meets the sparse direct solve as the FP64 factor's does and agrees with it to
    1e-10; the unrefined double-float sweeps on that factor are within 1e-7."""
    from misc_gb300.astro import OPT_BAND_FP64_UPDATE, OPT_PANELS_SOLVE
    m, g, o, A = batch
    B = np.random.default_rng(29).standard_normal((g.n, 10))
    Xr = spla.splu(A).solve(B)
    g.panels_factor(4)
    X64, _ = g.panels_solve(B)
    try:
        g.set_option(OPT_BAND_FP64_UPDATE, 3)
        g.panels_factor(4)
        Xdf, _ = g.panels_solve(B)
        g.set_option(OPT_PANELS_SOLVE, 2)
        Xraw, _ = g.panels_solve(B)
    finally:
        g.set_option(OPT_PANELS_SOLVE, 0)
        g.set_option(OPT_BAND_FP64_UPDATE, 1)
    _check(A, Xdf, B, Xr)
    assert np.linalg.norm(Xdf - X64) <= 1e-10 * np.linalg.norm(X64)
    assert np.linalg.norm(Xraw - X64) <= 1e-7 * np.linalg.norm(X64)


def test_staged_pageable_copies():
    """A solve whose right-hand sides and solutions pass 64 MB each way goes through the staged
    pageable copies (page-locked slots, host threads): every column equals the same column solved
    alone (small plain copies), bit for bit: each column's sweeps and refinement are independent
    of the others."""
    m = M.panel_batch(num_panels=512, indices=range(0, 512, 32))
    g = AstroGPU(m)
    g.getElasticSolnLoad(1, export=False)
    g.scaleElasticMPC()
    g.panels_factor(4)
    k = max(9, -(-80_000_000 // (8 * g.n)))  # at least 80 MB
    assert 8 * g.n * k >= 64 << 20
    B = np.random.default_rng(31).standard_normal((g.n, k))
    X, _ = g.panels_solve(B)
    for c in sorted({0, 1, k // 2, k - 1}):
        x1, _ = g.panels_solve(B[:, c])
        assert np.array_equal(X[:, c], x1), c
