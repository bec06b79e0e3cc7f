"""The polysolve adapter (include/lss_polysolve.hpp) through a C++ compiler.

The adapter derives from polysolve::linear::Solver and marks every method
`override`, so it compiles only if its signatures match the interface
(Solver.hpp:85-135 of the reference).  It is compiled against the committed
stand-in of that header (oracle/stubs) and, where a reference checkout has
been staged by oracle/build_ref.py, against the reference's own Solver.hpp and
Types.hpp; Eigen and nlohmann::json are the minimal stand-ins in oracle/stubs.
The program links liblss.so and drives the adapter like polysolve's callers:
without a GPU the constructor must refuse with the library's no-device error;
on a GB300 it solves a stiff 2D Laplacian to 1e-8 (or twice the FP64
rounding floor of the residual, where that is higher)."""
import os
import subprocess

import pytest

from conftest import ROOT

STUBS = os.path.join(ROOT, "oracle", "stubs")
REF_INC = os.path.join(ROOT, "oracle", "_ref", "include")
SRC = os.path.join(ROOT, "tests", "adapter", "adapter_main.cpp")


def _variants():
    out = [pytest.param("stand-in", [STUBS], id="stand-in")]
    out.append(pytest.param("reference", [REF_INC, STUBS], id="reference-header"))
    return out


def _build(tmp_path, incs):
    from lss import _paths
    lib = _paths.lib_path()
    exe = str(tmp_path / "adapter")
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Werror=overloaded-virtual", "-Werror=suggest-override",
           "-I", os.path.join(ROOT, "include")]
    for d in incs:
        cmd += ["-I", d]
    cmd += [SRC, "-o", exe, lib, "-Wl,-rpath," + os.path.dirname(lib), "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


def _need(kind):
    if kind == "reference" and not os.path.exists(os.path.join(REF_INC, "polysolve", "linear", "Solver.hpp")):
        pytest.skip("the reference's Solver.hpp is staged by oracle/build_ref.py from a reference checkout")


@pytest.mark.parametrize("kind,incs", _variants())
def test_adapter_compiles_and_refuses_without_gpu(kind, incs, built, tmp_path):
    _need(kind)
    exe = _build(tmp_path, incs)
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present: the solve itself runs in the gpu test")
    except ImportError:
        pass
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 2 and "no CUDA device" in r.stdout, (r.returncode, r.stdout, r.stderr)


@pytest.mark.gpu
@pytest.mark.parametrize("kind,incs", _variants())
def test_adapter_solves_on_gpu(kind, incs, built, tmp_path):
    _need(kind)
    exe = _build(tmp_path, incs)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, (r.stdout, r.stderr)
    tag, name, iters, rel, floor = r.stdout.split()
    assert tag == "ok" and name == "GPUHybrid" and int(iters) > 0, r.stdout
    assert float(rel) <= max(1e-8, 2 * float(floor)), r.stdout
