"""The autotuner of the launch shapes (astro_autotune) on the GPU, through the C ABI: every
candidate gives the same results (bit-identical assembly for the brick kernel's warps per CTA;
the many-column band solve's cluster sizes within 1e-9 of the oracle's batched loop), the
autotuner picks a candidate, writes its cache file and applies a cached choice without timing."""
import numpy as np
import pytest

from misc_gb300 import model as M
from misc_gb300.astro import (OPT_BRICK_WARPS, OPT_CASES_CLUSTER, OPT_PANEL_CLUSTER, TUNE_BRICK_WARPS,
                              TUNE_CASES_CLUSTER, TUNE_PANEL_CLUSTER, AstroError, AstroGPU)
from oracle import Oracle

pytestmark = pytest.mark.gpu


def test_brick_warps_candidates_and_cache(tmp_path):
    m = M.config2(nx=12, ny=6, nz=6, seed=2)
    g = AstroGPU(m)
    outs = []
    for fw in (1, 2, 4):
        g.set_option(OPT_BRICK_WARPS, fw)
        ke = g.element_matrices(32)
        outs.append(ke)
    assert np.array_equal(outs[0], outs[1]) and np.array_equal(outs[1], outs[2])
    cache = tmp_path / "tune.txt"
    ch = g.autotune(TUNE_BRICK_WARPS, cache)
    assert ch[0] in (1, 2, 4)
    lines = cache.read_text().splitlines()
    assert len(lines) == 1 and lines[0].split()[1] == str(ch[0])
    g2 = AstroGPU(m)
    assert g2.autotune(TUNE_BRICK_WARPS, cache)[0] == ch[0]
    assert len(cache.read_text().splitlines()) == 1  # cached: no new timing
    with pytest.raises(AstroError):
        g.set_option(OPT_BRICK_WARPS, 3)


def test_panel_cluster_autotune(tmp_path):
    m = M.panel_batch(num_panels=8, indices=[0, 1, 2, 3], n_range=(6, 12), n_dvars=0)
    g = AstroGPU(m)
    g.getElasticSolnLoad(1, export=False)
    g.scaleElasticMPC()
    ch = g.autotune(TUNE_PANEL_CLUSTER, tmp_path / "t.txt")
    assert ch[1] in (2, 4, 8)
    info = g.panels_factor(0)
    assert info.cluster_size == ch[1]
    g.set_option(OPT_PANEL_CLUSTER, 0)


def test_cases_cluster_sizes_match_oracle():
    from newmark_cases_ref import newmark_cases
    m = M.hex_block(6, 2, 2, lx=3.0, ly=0.5, lz=0.5, seed=6, jitter=0.1, sigma=0.3)
    o = Oracle(m)
    tip = [a + 1 for a in range(m.num_nodes) if abs(m.node_list[a, 0] - 3.0) < 1e-9]
    P = np.zeros((2, o.n))
    P[0, o.n_dof_index[tip[0] - 1, 2] - 1] = 1.0
    P[1, o.n_dof_index[tip[-1] - 1, 1] - 1] = 1.0
    t = 2e-5 * np.arange(1, 7)
    A = 1e5 * np.array([np.sin(2 * np.pi * 800 * t), np.cos(2 * np.pi * 300 * t)])
    Ho, *_ = newmark_cases(o, P, A, 2e-5, 0.25, 0.5, 6)
    for cs in (2, 4, 8):
        g = AstroGPU(m)
        g.set_option(OPT_CASES_CLUSTER, cs)
        u, v, a, H, info = g.newmark_cases(2e-5, P, A, history=True)
        assert info.cluster_size == cs
        for k in range(6):
            for c in range(2):
                assert np.linalg.norm(H[k, c] - Ho[k, c]) <= 1e-9 * np.linalg.norm(Ho[k, c]), (cs, k, c)
    g = AstroGPU(m)
    u, v, a, H, info = g.newmark_cases(2e-5, P, A, history=True, autotune=True)
    assert info.cluster_size in (2, 4, 8)
    assert g.autotune(0)[2] == info.cluster_size  # what = 0: the choices only
