"""The allocation-free skyline triangular solve (astro_ldl_solve_device_noalloc) against the
ordinary one (astro_ldl_solve), through the C ABI, and against the oracle's solveSparseLDLFact
restatement on the CPU (so that a fault in the device sweep the two entry points share cannot pass
unseen).  Tolerance 1e-12 relative; two calls in a row check that the shared scratch carries
nothing from one call into the next.  This file is collected last on purpose: it must pass both in
a fresh process and after every other GPU test has run in the same process."""
import ctypes as C

import numpy as np
import pytest

from misc_gb300 import model as M
from misc_gb300.astro import AstroError, AstroGPU
from oracle import Oracle

pytestmark = pytest.mark.gpu

MAX_DIM = 262144   # ASTRO_LDL_NOALLOC_MAX_DIM in include/astro_gpu.h
F64P, I32P = C.POINTER(C.c_double), C.POINTER(C.c_int32)


def _bind(g):
    f = g.L.astro_ldl_solve_device_noalloc
    f.argtypes = [C.c_void_p, F64P, F64P, F64P, I32P, C.c_int32]
    f.restype = C.c_int
    return f


def _ptr(t, typ):
    return C.cast(C.c_void_p(t.data_ptr()), typ)


@pytest.mark.parametrize("model", ["hex", "shell_beam"])
def test_noalloc_solve_matches_ldl_solve(model):
    torch = pytest.importorskip("torch")
    m = M.hex_block(nx=6, ny=3, nz=3) if model == "hex" else M.shell_beam()
    o, g = Oracle(m), AstroGPU(m)
    A, b, mat, cols, mm, mr = o.static_system()
    fac = o.ldl_fact(o.convert_to_ltri(mat, cols, mm), o.lt_range)
    f = _bind(g)
    dev = torch.device("cuda", 0)
    d_l = torch.tensor(fac, dtype=torch.float64, device=dev)
    d_r = torch.tensor(o.lt_range, dtype=torch.int32, device=dev)
    rng = np.random.default_rng(21)
    rhs = [rng.standard_normal(o.n) for _ in range(2)]
    x_ref = [g.solveSparseLDLFact(r, fac, o.lt_range) for r in rhs]
    x_orc = [o.ldl_solve(fac, o.lt_range, r) for r in rhs]
    d_b = [torch.tensor(r, dtype=torch.float64, device=dev) for r in rhs]
    d_x = [torch.full((o.n,), float("nan"), dtype=torch.float64, device=dev) for _ in rhs]
    torch.cuda.synchronize()
    for call in range(2):   # two calls in a row
        g._check(f(g.h, _ptr(d_x[call], F64P), _ptr(d_b[call], F64P), _ptr(d_l, F64P), _ptr(d_r, I32P), o.n))
    for call in range(2):
        x = d_x[call].cpu().numpy()
        assert np.linalg.norm(x - x_ref[call]) <= 1e-12 * np.linalg.norm(x_ref[call]), call
        assert np.linalg.norm(x - x_orc[call]) <= 1e-12 * np.linalg.norm(x_orc[call]), call


def test_noalloc_solve_rejects_oversize():
    m = M.hex_block(nx=2, ny=1, nz=1)
    g = AstroGPU(m)
    f = _bind(g)
    rc = f(g.h, None, None, None, None, MAX_DIM + 1)
    assert rc == 1
    with pytest.raises(AstroError, match="limit of 262144 rows"):
        g._check(rc)
