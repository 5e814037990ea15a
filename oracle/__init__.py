"""CPU oracle for AStrO's hot path -- TEST INFRASTRUCTURE ONLY.

A C++ restatement (oracle_elements.hpp, oracle_element_driver.hpp, oracle_api.cpp) of the
reference's element, assembly, book-keeping and solver routines, loaded through ctypes.
Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of bench.py use it, and only
as the checker; the GPU product path never imports it.
"""
from .oracle import Oracle, build, lib_path  # noqa: F401
