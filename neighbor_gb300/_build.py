"""Compile the CUDA library of neighbor_gb300 in-tree (nvcc, sm_103a only)."""
from __future__ import annotations

import os
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
INCLUDE = os.path.join(ROOT, "include")
BUILD_DIR = os.path.join(PKG, "_build")
LIB_NAME = "libneighbor_gb300.so"
LIB_PATH = os.path.join(BUILD_DIR, LIB_NAME)
SOURCES = [os.path.join(PKG, "csrc", "capi.cu"), os.path.join(PKG, "csrc", "noalloc.cu")]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _inputs():
    files = list(SOURCES)
    for d, _, names in os.walk(INCLUDE):
        files += [os.path.join(d, n) for n in names if n.endswith((".h", ".cuh"))]
    return files


def up_to_date() -> bool:
    if not os.path.exists(LIB_PATH):
        return False
    t = os.path.getmtime(LIB_PATH)
    return all(os.path.getmtime(f) <= t for f in _inputs())


def build(force: bool = False, verbose: bool = False) -> str:
    """Build libneighbor_gb300.so unless it is newer than every source and header."""
    if not force and up_to_date():
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    cmd = [_nvcc(), "-std=c++17", "-O3", *ARCH, "-lineinfo", "-Xcompiler", "-fPIC", "-shared",
           "-I" + INCLUDE, "-o", tmp, *SOURCES]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH
