"""In-tree build of the native libraries (no pip install, no cmake).

* ``liblss.so``     -- the solver: hand-written sm_103a CUDA kernels, the C++
  host library and the C ABI of ``include/lss.h`` (nvcc, one -gencode,
  translation units compiled in parallel, static cudart).
* ``liblss_gen.so`` -- host-only synthetic-system assembler (g++, OpenMP).
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

from . import _paths

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-Xcompiler", "-Wall", "-Xcompiler", "-Wno-unknown-pragmas"]
LIB_SOURCES = ["select.cu", "pcg.cu", "mas.cu", "stiff.cu", "multifrontal.cu", "batch.cu", "noalloc.cu", "solver.cpp",
               "batch.cpp", "capi.cpp", "params.cpp", "postproc.cpp", "partition.cpp", "pattern.cpp", "baddof.cpp",
               "mf_symbolic.cpp"]


def _nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r


def build(force: bool = False, verbose: bool = False) -> dict:
    os.makedirs(_paths.BUILD_DIR, exist_ok=True)
    headers = glob.glob(os.path.join(_paths.CSRC, "*.hpp")) + glob.glob(os.path.join(_paths.CSRC, "*.cuh")) + \
        [os.path.join(_paths.INCLUDE, "lss.h")]
    nvcc = _nvcc()
    objs, jobs = [], []
    for src in LIB_SOURCES:
        s = os.path.join(_paths.CSRC, src)
        o = os.path.join(_paths.BUILD_DIR, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            # host code: no FMA contraction, so that x86 and aarch64 builds (and
            # the oracle, built the same way) round every expression alike
            extra = ["-x", "cu"] if src.endswith(".cu") else ["-Xcompiler", "-ffp-contract=off"]
            jobs.append([nvcc, *ARCH, *NVCC_FLAGS, *extra, "-I", _paths.CSRC, "-I", _paths.INCLUDE, "-c", s,
                         "-o", o])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for f in [ex.submit(_run, j, verbose) for j in jobs]:
                f.result()
    lib = _paths.lib_path()
    if force or jobs or _stale(lib, objs):
        _run([nvcc, *ARCH, "-shared", "-o", lib, *objs, "-lpthread"], verbose)
    glib = build_generator(force, verbose)
    return {"lib": lib, "gen": glib}


def build_generator(force: bool = False, verbose: bool = False) -> str:
    """Host-only assembler of the synthetic elasticity systems (no CUDA)."""
    os.makedirs(_paths.BUILD_DIR, exist_ok=True)
    gsrc = os.path.join(_paths.CSRC, "gen_elasticity.cpp")
    glib = _paths.gen_lib_path()
    if force or _stale(glib, [gsrc]):
        # no FMA contraction: the x86 and aarch64 builds assemble bit-identical matrices
        _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", gsrc, "-o", glib],
             verbose)
    return glib
