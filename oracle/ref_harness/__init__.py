"""Reference harness -- TEST AND MEASUREMENT INFRASTRUCTURE ONLY.

Builds and runs the reference's own CUDA kernels (mphowardlab/neighbor v0.3.2) on the GPU:
``ref_kernels.cu`` instantiates them from the reference headers into
``oracle/_ref/ref_kernels.cubin`` (only where the reference sources exist), and
``ref_driver.cu`` -- compiled wherever that cubin exists -- loads it and replays
the reference's build / setup / traverse sequence.  Used by the parity tests (to pin the oracle
and the library against the real reference) and by bench.py (to time the reference on the same
GPU).  The product never touches it.
"""
from __future__ import annotations

import json
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(os.path.dirname(HERE), "_ref")
CUBIN = os.path.join(OUT, "ref_kernels.cubin")
DRIVER = os.path.join(OUT, "ref_driver")
# The reference's headers, where its sources exist (the build machine; never the GPU machine, which
# uses the cubin built there).  NEIGHBOR_REFERENCE_INCLUDE points the recipe elsewhere.
REFERENCE_INCLUDE = os.environ.get("NEIGHBOR_REFERENCE_INCLUDE", "/root/reference/include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def build_cubin(force=False) -> bool:
    """Compile the reference's kernels from its headers (needs the reference sources)."""
    if not os.path.isdir(REFERENCE_INCLUDE):
        return os.path.exists(CUBIN)
    src = os.path.join(HERE, "ref_kernels.cu")
    if not force and os.path.exists(CUBIN) and os.path.getmtime(CUBIN) >= os.path.getmtime(src):
        return True
    os.makedirs(OUT, exist_ok=True)
    subprocess.run([_nvcc(), "-std=c++17", "-cubin", *ARCH, "-I", REFERENCE_INCLUDE, "-I", HERE,
                    "-o", CUBIN, src], check=True)
    return True


def build_driver(force=False) -> bool:
    """Compile the host driver (wherever the cubin exists)."""
    if not os.path.exists(CUBIN):
        return False
    src = os.path.join(HERE, "ref_driver.cu")
    if not force and os.path.exists(DRIVER) and os.path.getmtime(DRIVER) >= os.path.getmtime(src):
        return True
    subprocess.run([_nvcc(), "-std=c++17", "-O3", *ARCH, "-o", DRIVER, src, "-lcuda"], check=True)
    return True


def build_if_available() -> bool:
    return build_cubin() and build_driver()


def available() -> bool:
    return os.path.exists(CUBIN) and os.path.exists(DRIVER)


def _run(args, timeout):
    r = subprocess.run([DRIVER, *[str(a) for a in args]], capture_output=True, text=True, timeout=timeout)
    if r.returncode != 0:
        raise RuntimeError(f"reference driver failed ({r.returncode}): {r.stderr.strip()[-400:]}")
    return json.loads(r.stdout.strip().splitlines()[-1])


def run_bench(n, steps=20, warmup=3, rc=1.3, timeout=900):
    """Time the reference's plain two-pass step (build, setup, count, max, fill) on uniform
    trajectory frames for every block size 32..1024 (step 32); returns the driver's JSON."""
    return _run(["bench", n, steps, warmup, rc], timeout)


def _write_frames(path, frames):
    with open(path, "wb") as f:
        for fr in frames:
            np.ascontiguousarray(fr, np.float32).reshape(-1, 3).tofile(f)


def run_frames(frames, rc, L, steps, warmup, timeout=900):
    """The same plain step on the given frames (a list of [n, 3] float32 arrays, cycled), queries
    in the tree's sorted order, 27 images of the cube of side L, every block size."""
    n = len(frames[0])
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "frames.f32")
        _write_frames(path, frames)
        return _run(["frames", path, n, len(frames), repr(float(rc)), repr(float(L)), steps, warmup], timeout)


def run_frames64(frames, rc, L, steps, warmup, timeout=900):
    """The plain step on the given double-precision frames ([n, 3] float64 arrays, cycled) with the
    harness's double insert op and double exact query op through the reference's kernels, every
    block size; adds the pair total of the last timed frame."""
    n = len(frames[0])
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "frames.f64")
        with open(path, "wb") as f:
            for fr in frames:
                np.ascontiguousarray(fr, np.float64).reshape(-1, 3).tofile(f)
        return _run(["frames64", path, n, len(frames), repr(float(rc)), repr(float(L)), steps, warmup], timeout)


def run_poly(small_frames, large_frames, L, steps, warmup, timeout=900):
    """Two-tree polydisperse step (diameters 1 and 10, cutoff (di+dj)/2 + 0.4, 27 images) on the
    given frames of each species, every block size."""
    with tempfile.TemporaryDirectory() as d:
        sp, lp = os.path.join(d, "small.f32"), os.path.join(d, "large.f32")
        _write_frames(sp, small_frames)
        _write_frames(lp, large_frames)
        return _run(["poly", sp, len(small_frames[0]), lp, len(large_frames[0]), len(small_frames),
                     repr(float(L)), steps, warmup], timeout)


# Row hash of a neighbor list (the driver's k_row_hash): sum over k < count of (entry_k + 1) * C_k
# plus count * C_COUNT, exact in 64-bit integers for rows of up to 64 entries.
HASH_COUNT = 0x2545F491


def hash_coefficients(m):
    k = np.arange(m, dtype=np.uint64)
    return ((((k + 1) * np.uint64(2654435761)) % np.uint64(1 << 32)) & np.uint64(0x7FFFFFFF)) | np.uint64(1)


def run_hash(points, rc, L, timeout=900):
    """Counts and row hashes of the reference's exact neighbor list of the points (queries in
    input order, 27 images of the cube of side L)."""
    P = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
    n = len(P)
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "points.f32")
        P.tofile(src)
        prefix = os.path.join(d, "ref")
        info = _run(["hash", src, n, repr(float(rc)), repr(float(L)), prefix], timeout)
        return (np.fromfile(prefix + ".count", np.uint32), np.fromfile(prefix + ".hash", np.uint64),
                int(info["max_count"]))


def run_dump(points, lo, hi, rc, box, timeout=300, exact_only=False, sphere_radius=None):
    """The reference's tree arrays, compressed nodes, counts (stock and exact query, 27 periodic
    images of `box`, queries = the points in input order) and the exact query's neighbor list
    (stride = the largest count) for the given points.  exact_only: skip the stock query's
    counts and lists; sphere_radius: build with SphereInsertOp of that radius."""
    P = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
    n = len(P)
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "points.f32")
        P.tofile(src)
        prefix = os.path.join(d, "ref")
        args = [DRIVER, "dump", src, str(n), *[repr(float(x)) for x in lo], *[repr(float(x)) for x in hi],
                repr(float(rc)), *[repr(float(x)) for x in box], prefix]
        if exact_only:
            args.append("exact_only")
        elif sphere_radius is not None:
            args += ["sphere", repr(float(sphere_radius))]
        r = subprocess.run(args, capture_output=True, text=True, timeout=timeout)
        if r.returncode != 0:
            raise RuntimeError(f"reference driver failed ({r.returncode}): {r.stderr.strip()[-400:]}")
        out = {}
        for name, dt, shape in [("codes", np.uint32, (n,)), ("primitive", np.uint32, (n,)),
                                ("parent", np.int32, (2 * n - 1,)), ("left", np.int32, (n - 1,)),
                                ("right", np.int32, (n - 1,)), ("lo", np.float32, (2 * n - 1, 3)),
                                ("hi", np.float32, (2 * n - 1, 3)), ("data", np.int32, (2 * n - 1, 4)),
                                ("count_stock", np.uint32, (n,)), ("count_exact", np.uint32, (n,))]:
            path = prefix + "." + name
            if os.path.exists(path):
                out[name] = np.fromfile(path, dt).reshape(shape)
        lpath = prefix + ".list_exact"
        if os.path.exists(lpath) and "count_exact" in out and n:
            stride = max(1, int(out["count_exact"].max()))
            out["list_exact"] = np.fromfile(lpath, np.uint32).reshape(n, stride)
            out["count_list"] = np.fromfile(prefix + ".count_list", np.uint32)
        spath = prefix + ".list_stock"
        if os.path.exists(spath) and "count_stock" in out and n:
            stride = max(1, int(out["count_stock"].max()))
            out["list_stock"] = np.fromfile(spath, np.uint32).reshape(n, stride)
        return out
