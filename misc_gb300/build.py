"""Builds libastro_gpu.so in-tree with nvcc for sm_103a (no torch involved).

Each translation unit under csrc/ is compiled in parallel to an object file, then linked into
misc_gb300/_lib/libastro_gpu.so.  Rebuilds only what changed.  With ASTRO_BOUNDS_CHECK=1 in the
environment the checked build (device index guards, csrc/bounds.cuh) goes to
misc_gb300/_lib/libastro_gpu_checked.so instead, which misc_gb300.astro loads under the same
variable.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libastro_gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "nvcc")
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
         "--expt-relaxed-constexpr"]
if os.environ.get("ASTRO_BOUNDS_CHECK"):
    FLAGS += ["-DASTRO_BOUNDS_CHECK"]
    BUILD = BUILD + "_checked"
    LIB = os.path.join(OUT, "libastro_gpu_checked.so")


def lib_path():
    return LIB


def _deps_newer(obj, src):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    hdrs = (glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) +
            [os.path.join(HERE, "..", "include", "astro_gpu.h")])
    return any(os.path.getmtime(p) > t for p in [src] + hdrs)


def _compile(src):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    if not _deps_newer(obj, src):
        return obj, None
    cmd = [NVCC] + ARCH + FLAGS + ["-c", src, "-o", obj]
    if src.endswith(".cpp"):
        cmd = [NVCC] + ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-x", "c++", "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return obj, r.stdout + r.stderr
    return obj, None


def build(verbose=False):
    os.makedirs(OUT, exist_ok=True)
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        res = list(ex.map(_compile, srcs))
    errs = [e for _, e in res if e]
    if errs:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errs))
    objs = [o for o, _ in res]
    if not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
