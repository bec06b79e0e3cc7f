"""Locations of the package, its sources and its in-tree build outputs."""
import os

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))  # local-stiff-solver_gb300/
REPO_ROOT = os.path.dirname(PKG_ROOT)
CSRC = os.path.join(PKG_ROOT, "csrc")
INCLUDE = os.path.join(REPO_ROOT, "include")
BUILD_DIR = os.path.join(PKG_ROOT, "_build")


def lib_path():
    return os.path.join(BUILD_DIR, "liblss.so")


def gen_lib_path():
    return os.path.join(BUILD_DIR, "liblss_gen.so")
