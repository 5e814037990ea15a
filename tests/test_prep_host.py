"""Host logic of the C ABI (no GPU): the library loads, exports every declared symbol, and its
analysis preparation reproduces the reference's integer set-up (node ranks, DOF map, CSR and
skyline structure, and the find-or-insert CSR column order) bit for bit against the oracle."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from misc_gb300 import model as M
from misc_gb300.astro import DimsC, load_library
from oracle import Oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_library_exports_every_declared_symbol():
    L = load_library()
    hdr = open(os.path.join(ROOT, "include", "astro_gpu.h")).read()
    names = sorted(set(re.findall(r"^int (astro_\w+)\(", hdr, flags=re.M)))
    assert len(names) >= 20
    for nm in names:
        assert hasattr(L, nm), nm


def _prep_host(m):
    L = load_library()
    mc = m.as_c()
    d = DimsC()
    nc = C.c_int32(0)
    I = C.POINTER(C.c_int32)
    f = L.astro_prep_host
    f.argtypes = [C.c_void_p, C.POINTER(DimsC), I, I, I, I, I, I]
    rc = f(C.byref(mc), C.byref(d), None, None, None, None, None, None)
    assert rc == 0
    N = m.num_nodes
    rank = np.zeros(N, np.int32); ndi = np.zeros((N, 6), np.int32)
    rng = np.zeros(d.el_mat_dim + 1, np.int32); lt = np.zeros(d.el_mat_dim + 1, np.int32)
    cols = np.zeros(d.el_mat_size, np.int32)
    p = lambda a: a.ctypes.data_as(I)
    rc = f(C.byref(mc), C.byref(d), p(rank), p(ndi), p(rng), p(lt), p(cols), C.byref(nc))
    assert rc == 0
    return d, rank, ndi, rng, lt, cols, nc.value


def _shuffled_block():
    m = M.hex_block(5, 3, 2, lx=1.0, ly=0.6, lz=0.4, seed=11)
    perm = np.random.default_rng(2).permutation(m.num_els)
    m.element_list = m.element_list[perm]
    return m


CASES = {
    "hex_small": lambda: M.hex_block(4, 3, 2, lx=1.0, ly=0.75, lz=0.5, seed=2),
    "hex_shuffled": _shuffled_block,
    "shell_beam": M.shell_beam,
    "plate_cfg1": M.config1,
    "plate_ss": lambda: M.plate_shell(nx=9, ny=7, lx=1.0, ly=1.0, clamp="ss", y0=0.0),
    "block_cfg2_8x4x4": lambda: M.config2(nx=8, ny=4, nz=4),
    "brickIM_mixed": lambda: _mixed_brick_im(),
}


def _mixed_brick_im():
    """brick8 and brickIM (type 81) elements in one block: the same node structure, plus the
    internal-DOF ranges of the incompatible modes."""
    m = M.hex_block(4, 3, 2, lx=1.0, ly=0.75, lz=0.5, seed=3)
    t = np.full(m.num_els, 8, np.int32)
    t[::3] = 81
    m.element_type = t
    return m


@pytest.mark.parametrize("name", sorted(CASES))
def test_prep_matches_oracle(name):
    m = CASES[name]()
    o = Oracle(m)
    d, rank, ndi, rng, lt, cols, ncol = _prep_host(m)
    assert d.el_mat_dim == o.n and d.el_mat_size == o.el_mat_size and d.el_mat_lt_size == o.lt_size
    assert d.solver_max_bw == o.solver_max_bw
    assert d.int_vec_size == o.int_vec_size and d.int_mat_size == o.int_mat_size
    assert np.array_equal(rank, o.current_rank)
    assert np.array_equal(ndi, o.n_dof_index)
    assert np.array_equal(rng, o.el_mat_range)
    assert np.array_equal(lt, o.lt_range)
    _, _, _, ocols, _ = o.el_soln_load(1)
    assert np.array_equal(cols, ocols)
    assert 1 <= ncol <= (8 if m.dof_per_node == 3 else 4) + 4


def test_prep_rejects_unsupported_element_type():
    m = M.hex_block(2, 2, 2)
    m.element_type = m.element_type.copy()
    m.element_type[0] = 4
    L = load_library()
    mc = m.as_c()
    d = DimsC()
    f = L.astro_prep_host
    f.argtypes = [C.c_void_p, C.POINTER(DimsC)] + [C.c_void_p] * 6
    assert f(C.byref(mc), C.byref(d), None, None, None, None, None, None) == 3
