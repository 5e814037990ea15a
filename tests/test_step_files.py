"""Solution-history step files (writeBinarySolution / readBinarySolution) on the host: the
Fortran unformatted sequential layout byte for byte, the round trip, and the reader's error on a
missing or short record (the reference's errFlag)."""
import struct

import numpy as np
import pytest

from misc_gb300.astro import AstroError, read_step_file, write_step_file


def _fortran_records(*arrays):
    out = b""
    for a in arrays:
        data = np.asarray(a, np.float64).tobytes()
        out += struct.pack("<I", len(data)) + data + struct.pack("<I", len(data))
    return out


def test_step_file_layout_and_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    nn, n, ni = 5, 30, 16
    u, v, a, iu = rng.standard_normal(n), rng.standard_normal(n), rng.standard_normal(n), rng.standard_normal(ni)
    p = tmp_path / "SolutionHistory3.out"
    write_step_file(p, nn, u, v, a, int_disp=iu)
    assert p.read_bytes() == _fortran_records(np.zeros(nn), np.zeros(nn), u, iu, v, a)
    t, td, u2, iu2, v2, a2 = read_step_file(p, nn, n, ni)
    assert np.array_equal(u2, u) and np.array_equal(v2, v) and np.array_equal(a2, a) and np.array_equal(iu2, iu)
    assert not t.any() and not td.any()


def test_step_file_without_internal_dof(tmp_path):
    rng = np.random.default_rng(1)
    n = 12
    u, v, a = rng.standard_normal(n), rng.standard_normal(n), rng.standard_normal(n)
    p = tmp_path / "SolutionHistory0.out"
    write_step_file(p, 4, u, v, a)
    assert p.read_bytes() == _fortran_records(np.zeros(4), np.zeros(4), u, v, a)
    _, _, u2, _, v2, a2 = read_step_file(p, 4, n, 0)
    assert np.array_equal(u2, u) and np.array_equal(v2, v) and np.array_equal(a2, a)


def test_step_file_errors(tmp_path):
    with pytest.raises(AstroError):
        read_step_file(tmp_path / "missing.out", 4, 12, 0)
    p = tmp_path / "short.out"
    p.write_bytes(_fortran_records(np.zeros(4), np.zeros(4), np.zeros(6)))
    with pytest.raises(AstroError):
        read_step_file(p, 4, 12, 0)
    # one internal DOF: written (>= 1) but not read (> 1), so prevVel meets the short record
    q = tmp_path / "one.out"
    write_step_file(q, 4, np.ones(12), np.ones(12), np.ones(12), int_disp=np.ones(1))
    with pytest.raises(AstroError):
        read_step_file(q, 4, 12, 1)
