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
SOURCES = [os.path.join(PKG, "csrc", n) for n in ("capi.cu", "noalloc.cu", "learned.cu", "batched.cu")]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _inputs():
    files = list(SOURCES)
    for d, _, names in os.walk(INCLUDE):
        files += [os.path.join(d, n) for n in names if n.endswith((".h", ".cuh"))]
    files += [os.path.join(PKG, "csrc", n) for n in os.listdir(os.path.join(PKG, "csrc")) if n.endswith(".h")]
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
    tag = f".tmp{os.getpid()}"
    # one object per translation unit, compiled in parallel, then one link
    objs, procs = [], []
    for src in SOURCES:
        obj = os.path.join(BUILD_DIR, os.path.basename(src) + tag + ".o")
        cmd = [_nvcc(), "-std=c++17", "-O3", *ARCH, "-lineinfo", "-Xcompiler", "-fPIC", "-c",
               "-I" + INCLUDE, "-o", obj, src]
        if verbose:
            print(" ".join(cmd))
        procs.append((subprocess.Popen(cmd), cmd))
        objs.append(obj)
    failed = [cmd for p, cmd in procs if p.wait() != 0]
    if failed:
        raise subprocess.CalledProcessError(1, failed[0])
    tmp = LIB_PATH + tag
    link = [_nvcc(), *ARCH, "-shared", "-o", tmp, *objs]
    if verbose:
        print(" ".join(link))
    subprocess.run(link, check=True)
    for o in objs:
        os.remove(o)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH
