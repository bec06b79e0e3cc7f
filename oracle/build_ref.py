"""Recipe: build the reference's own stiff-DOF selection code on the host --
TEST INFRASTRUCTURE ONLY (the product never loads it).

GPUHybrid (src/polysolve/linear/GPUHybrid.cu) as a whole needs hypre, cuDSS,
MPI, Eigen and spdlog, none of which exist here.  Its selection stage does
not: select_bad_dofs (GPUHybrid.cu:737-883) is thrust + std, and the
post-processing (filter_subdomains :885-970, expand_subdomains_to_strongly_
connected :972-991, decompose_subdomains_to_disjoint_subsets :691-735, with
disjointSet from Hybrid.hpp:223-260) is std + Eigen's InnerIterator.  This
script copies those definitions verbatim, located by their signatures and
brace matching, from the reference checkout into oracle/_ref/*.inc (build
output, git-ignored; the polysolve Types.hpp and Solver.hpp headers are staged
there too, for the adapter's compile check) and compiles oracle/ref/harness.cpp
around them with g++
against CCCL's thrust (sequential host backend) and the Eigen stand-in in
oracle/stubs, into oracle/_ref/libgpuhybrid_ref.so.

    python oracle/build_ref.py [reference checkout]     (default /root/reference)

Without the reference checkout, a previously extracted oracle/_ref/*.inc is
compiled again (the .inc files are text and travel with the working tree).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT, "libgpuhybrid_ref.so")
DEFAULT_REFERENCE = "/root/reference"

GPUHYBRID = os.path.join("src", "polysolve", "linear", "GPUHybrid.cu")
HYBRID_HPP = os.path.join("src", "polysolve", "linear", "Hybrid.hpp")
FUNCTIONS = [
    "void GPUHybrid::decompose_subdomains_to_disjoint_subsets(",
    "void GPUHybrid::select_bad_dofs(",
    "void GPUHybrid::filter_subdomains(",
    "void GPUHybrid::expand_subdomains_to_strongly_connected(",
]


def _block_end(src: str, start: int) -> int:
    """Index one past the '}' closing the first '{' at or after `start`,
    skipping string/char literals and comments."""
    i, depth, n = src.index("{", start), 0, len(src)
    while i < n:
        c = src[i]
        if c == "/" and src.startswith("//", i):
            i = src.index("\n", i)
            continue
        if c == "/" and src.startswith("/*", i):
            i = src.index("*/", i) + 2
            continue
        if c in "\"'":
            j = i + 1
            while src[j] != c:
                j += 2 if src[j] == "\\" else 1
            i = j + 1
            continue
        if c == "{":
            depth += 1
        elif c == "}":
            depth -= 1
            if depth == 0:
                return i + 1
        i += 1
    raise ValueError("unbalanced braces")


def _extract(src: str, path: str, signature: str, struct: bool = False) -> str:
    k = src.index(signature)
    k = src.rfind("\n", 0, k) + 1
    end = _block_end(src, k)
    if struct:
        end = src.index(";", end) + 1
    line = src.count("\n", 0, k) + 1
    return f'#line {line} "{path}"\n' + src[k:end] + "\n"


HEADERS = [os.path.join("src", "polysolve", "Types.hpp"), os.path.join("src", "polysolve", "linear", "Solver.hpp")]


def extract(reference: str) -> None:
    os.makedirs(OUT, exist_ok=True)
    # the polysolve interface headers, for the adapter's compile check
    for h in HEADERS:
        dst = os.path.join(OUT, "include", os.path.relpath(h, "src"))
        os.makedirs(os.path.dirname(dst), exist_ok=True)
        shutil.copyfile(os.path.join(reference, h), dst)
    gh = open(os.path.join(reference, GPUHYBRID)).read()
    hy = open(os.path.join(reference, HYBRID_HPP)).read()
    head = f"// generated by oracle/build_ref.py from the reference checkout at {reference}; do not edit\n"
    with open(os.path.join(OUT, "gpuhybrid_disjoint_set.inc"), "w") as f:
        f.write(head + _extract(hy, HYBRID_HPP, "struct disjointSet", struct=True))
    with open(os.path.join(OUT, "gpuhybrid_selection.inc"), "w") as f:
        f.write(head)
        for sig in FUNCTIONS:
            f.write(_extract(gh, GPUHYBRID, sig))


def _cccl_includes() -> list[str]:
    nvcc = shutil.which("nvcc")
    root = os.path.dirname(os.path.dirname(nvcc)) if nvcc else "/usr/local/cuda"
    inc = os.path.join(root, "include")
    out = []
    for d in (os.path.join(inc, "cccl"), inc):
        if os.path.isdir(d):
            out += ["-I", d]
    return out


def build(reference: str | None = None, force: bool = False) -> str | None:
    """Extract (when the reference checkout exists) and compile; returns the
    library path, or None when neither the checkout nor extracted sources exist."""
    ref = reference or DEFAULT_REFERENCE
    have_ref = os.path.exists(os.path.join(ref, GPUHYBRID))
    inc = os.path.join(OUT, "gpuhybrid_selection.inc")
    if have_ref and (force or not os.path.exists(inc)):
        extract(ref)
    if not os.path.exists(inc):
        return None
    srcs = [os.path.join(HERE, "ref", "harness.cpp"), inc, os.path.join(OUT, "gpuhybrid_disjoint_set.inc")]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(s) for s in srcs):
        return LIB
    cmd = (["g++", "-std=gnu++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-w",
            "-DTHRUST_DEVICE_SYSTEM=THRUST_DEVICE_SYSTEM_CPP", "-I", OUT, "-I", os.path.join(HERE, "stubs")]
           + _cccl_includes() + [srcs[0], "-o", LIB + ".tmp"])
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    path = build(sys.argv[1] if len(sys.argv) > 1 else None, force=True)
    print(path or "reference checkout not found and nothing extracted")
