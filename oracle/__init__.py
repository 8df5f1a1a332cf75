"""CPU oracle for the neighbor LBVH path -- TEST INFRASTRUCTURE ONLY.

This package is the checker for the CUDA library in ``neighbor_gb300``.  Only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` import it; the product
never does.  The C++ restatement lives in ``oracle/oracle.cpp`` (every function cites the
reference file:line it follows); this module compiles it with g++ and wraps it with ctypes
over numpy arrays.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "liboracle.so")
SOURCES = [os.path.join(HERE, "oracle.cpp"), os.path.join(HERE, "frame_list.cpp")]

SENTINEL = 0x7FFFFFFF
INSERT_POINT, INSERT_SPHERE = 0, 1
QUERY_SPHERE, QUERY_EXACT = 0, 1

_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> str:
    """Compile liboracle.so (g++, OpenMP, IEEE rounding semantics kept)."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    newest = max(os.path.getmtime(s) for s in SOURCES + [os.path.join(HERE, "oracle.h")])
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= newest:
        return LIB_PATH
    tag = f".tmp{os.getpid()}"
    tmp = LIB_PATH + tag
    # oracle.cpp switches the rounding mode (-frounding-math); frame_list.cpp, the timed CPU
    # baseline, rounds to nearest only and is optimised fully.  Neither fuses a*b+c.
    objs = [os.path.join(BUILD_DIR, "oracle.o" + tag), os.path.join(BUILD_DIR, "frame_list.o" + tag)]
    procs = [subprocess.Popen(["g++", "-O2", "-std=c++17", "-fPIC", "-fopenmp", "-frounding-math",
                               "-ffp-contract=off", "-c", "-o", objs[0], SOURCES[0]]),
             subprocess.Popen(["g++", "-O3", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off",
                               "-fno-trapping-math", "-c", "-o", objs[1], SOURCES[1]])]
    if any(p.wait() != 0 for p in procs):
        raise subprocess.CalledProcessError(1, "g++ (oracle)")
    subprocess.run(["g++", "-shared", "-fopenmp", "-o", tmp] + objs, check=True)
    for o in objs:
        os.remove(o)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(LIB_PATH)
            _declare(L)
            _lib = L
    return _lib


_f = ctypes.c_float
_u32 = ctypes.c_uint32
_i32 = ctypes.c_int32
_P = ctypes.c_void_p


def _declare(L):
    for name in ["fadd_rd", "fadd_ru", "fsub_rd", "fsub_ru", "fmul_rd", "fmul_ru", "fdiv_rd",
                 "fdiv_ru"]:
        fn = getattr(L, "orc_" + name)
        fn.argtypes = [_f, _f]
        fn.restype = _f
    for name in ["frcp_rd", "frcp_ru"]:
        fn = getattr(L, "orc_" + name)
        fn.argtypes = [_f]
        fn.restype = _f
    for name in ["fmaf_rd", "fmaf_ru"]:
        fn = getattr(L, "orc_" + name)
        fn.argtypes = [_f, _f, _f]
        fn.restype = _f
    for name in ["double2float_rd", "double2float_ru"]:
        fn = getattr(L, "orc_" + name)
        fn.argtypes = [ctypes.c_double]
        fn.restype = _f
    L.orc_morton_codes.argtypes = [_P, _u32, ctypes.c_int, _f, _P, _P, _P]
    L.orc_build.argtypes = [_P, _u32, ctypes.c_int, _f, _P, _P, _P, _P, _P, _P, _P, _P, _P]
    L.orc_compress_ref10.argtypes = [_u32, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P]
    L.orc_traverse_ref10.argtypes = [_u32, _P, _P, _P, _P, _P, _u32, _P, _u32, ctypes.c_int,
                                     _P, _P, _f, _P, _P, _u32]
    L.orc_exact_pair.argtypes = [_P, _P, _f, _P]
    L.orc_exact_pair.restype = ctypes.c_int
    L.orc_exact_pad.argtypes = [_f, _f]
    L.orc_exact_pad.restype = _f
    L.orc_brute_count.argtypes = [_P, _P, _u32, _P, _u32, _P, _P]
    L.orc_celllist.argtypes = [_P, _P, _f, _u32, _P, _u32, _P, _P, _P, _P, _u32, ctypes.c_int]
    L.orc_celllist.restype = ctypes.c_int
    L.orc_celllist_csr.argtypes = [_P, _P, _f, _u32, _P, _u32, _P, _P, _P, _P, ctypes.c_int]
    L.orc_celllist_csr.restype = ctypes.c_int
    L.orc_frame_list.argtypes = [_P, _u32, _P, _P, _f, ctypes.c_int, _P, _P, _P, ctypes.c_uint64, _P, _P, _P]
    L.orc_frame_list.restype = ctypes.c_int
    L.orc_uniform_points.argtypes = [_P, _u32, _P, _P, ctypes.c_uint64]
    L.orc_gaussian_move.argtypes = [_P, _P, _u32, _P, _P, _f, ctypes.c_uint64]
    L.orc_pair_distance_minus_rc_f64.argtypes = [_P, _P, _f, _P]
    L.orc_pair_distance_minus_rc_f64.restype = ctypes.c_double
    L.orc_fast_nodes.argtypes = [_u32, _u32, _P, _P, _P, _P, _P, _P, _P, _P]
    L.orc_fast_nodes.restype = _u32
    L.orc_fast_frame.argtypes = [_P, _P, _P]
    L.orc_fast_quantize.argtypes = [_P, _P, _P, _P, _P]
    L.orc_gen_validate_points.argtypes = [_u32, _P, _u32, _P]
    L.orc_cap_occupancy.argtypes = [_P, _u32, _u32, _P]
    L.orc_cap_features.argtypes = [_P, _P, _u32, _P, _P, _u32, ctypes.c_int, _P, _P]
    L.orc_cap_forward_backward.argtypes = [_P, _P, _P, _u32, _u32, _u32, _u32, ctypes.c_int, _P, _P, _P]


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _f32(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float32)
    if shape is not None:
        a = a.reshape(shape)
    return a


def rounding(name: str, *args):
    """Directed-rounding op by reference name, e.g. rounding('fadd_rd', 1.0, 1e-12)."""
    return getattr(lib(), "orc_" + name)(*args)


def morton_codes(points, lo, hi, insert=INSERT_POINT, r=0.0):
    p = _f32(points, (-1, 3))
    out = np.empty(len(p), np.uint32)
    lib().orc_morton_codes(_ptr(p), len(p), insert, r, _ptr(_f32(lo)), _ptr(_f32(hi)), _ptr(out))
    return out


def build_tree(points, lo, hi, insert=INSERT_POINT, r=0.0):
    """Reference-layout LBVH: dict of sorted codes, primitives, parent/left/right, lo/hi."""
    p = _f32(points, (-1, 3))
    N = len(p)
    nn = max(2 * N - 1, 0)
    ni = max(N - 1, 0)
    t = dict(N=N, codes=np.zeros(N, np.uint32), primitive=np.zeros(N, np.uint32),
             parent=np.zeros(nn, np.int32), left=np.zeros(ni, np.int32),
             right=np.zeros(ni, np.int32), lo=np.zeros((nn, 3), np.float32),
             hi=np.zeros((nn, 3), np.float32))
    if N:
        lib().orc_build(_ptr(p), N, insert, r, _ptr(_f32(lo)), _ptr(_f32(hi)),
                        _ptr(t["codes"]), _ptr(t["primitive"]), _ptr(t["parent"]),
                        _ptr(t["left"]), _ptr(t["right"]), _ptr(t["lo"]), _ptr(t["hi"]))
    return t


def compress_ref10(tree, mapping=None):
    """Reference 10-bit int4 nodes: (data[nn,4] int32, clo, chi, bins)."""
    N = tree["N"]
    nn = 2 * N - 1
    data = np.zeros((nn, 4), np.int32)
    clo = np.zeros(3, np.float32)
    chi = np.zeros(3, np.float32)
    bins = np.zeros(3, np.float32)
    m = None if mapping is None else np.ascontiguousarray(mapping, np.uint32)
    lib().orc_compress_ref10(N, _ptr(tree["parent"]), _ptr(tree["left"]), _ptr(tree["right"]),
                             _ptr(tree["primitive"]), _ptr(tree["lo"]), _ptr(tree["hi"]),
                             _ptr(m), _ptr(data), _ptr(clo), _ptr(chi), _ptr(bins))
    return data, clo, chi, bins


def traverse_ref10(comp, spheres, images=None, query=QUERY_SPHERE, points=None, box_L=None,
                   pad=0.0, max_neigh=None):
    """Reference rope traversal. Returns nneigh, or (nneigh, list) when max_neigh is given."""
    data, clo, chi, bins = comp
    s = _f32(spheres, (-1, 4))
    Q = len(s)
    nneigh = np.zeros(Q, np.uint32)
    lst = None
    if max_neigh is not None:
        lst = np.full(Q * max(max_neigh, 1), 0xFFFFFFFF, np.uint32)
    img = None if images is None else _f32(images, (-1, 3))
    pts = None if points is None else _f32(points, (-1, 3))
    bl = _f32(box_L if box_L is not None else [0, 0, 0])
    lib().orc_traverse_ref10(len(data), _ptr(data), _ptr(clo), _ptr(chi), _ptr(bins), _ptr(s),
                             Q, _ptr(img), 0 if img is None else len(img), query, _ptr(pts),
                             _ptr(bl), pad, _ptr(nneigh), _ptr(lst),
                             0 if max_neigh is None else max_neigh)
    if max_neigh is None:
        return nneigh
    return nneigh, lst.reshape(Q, max(max_neigh, 1))[:, :max_neigh]


def exact_pair(pi, pj, rc, box_L=(0, 0, 0)):
    return bool(lib().orc_exact_pair(_ptr(_f32(pi)), _ptr(_f32(pj)), rc, _ptr(_f32(box_L))))


def exact_pad(rc, coord_max):
    return float(lib().orc_exact_pad(rc, coord_max))


def brute_count(qpos, qr, points, box_L=(0, 0, 0)):
    q = _f32(qpos, (-1, 3))
    r = _f32(np.broadcast_to(np.asarray(qr, np.float32), (len(q),)))
    p = _f32(points, (-1, 3))
    out = np.zeros(len(q), np.uint32)
    lib().orc_brute_count(_ptr(q), _ptr(r), len(q), _ptr(p), len(p), _ptr(_f32(box_L)), _ptr(out))
    return out


def celllist_counts(qpos, points, rc, box_lo, box_L, qr=None, nthreads=0, max_neigh=None):
    """OpenMP cell list (periodic). Returns (nneigh, threads) or (nneigh, list, threads)."""
    q = _f32(qpos, (-1, 3))
    p = _f32(points, (-1, 3))
    r = None if qr is None else _f32(qr)
    nn = np.zeros(len(q), np.uint32)
    lst = None
    if max_neigh is not None:
        lst = np.full(len(q) * max(max_neigh, 1), 0xFFFFFFFF, np.uint32)
    used = lib().orc_celllist(_ptr(q), _ptr(r), rc, len(q), _ptr(p), len(p), _ptr(_f32(box_lo)),
                              _ptr(_f32(box_L)), _ptr(nn), _ptr(lst),
                              0 if max_neigh is None else max_neigh, nthreads)
    if max_neigh is None:
        return nn, used
    return nn, lst.reshape(len(q), max(max_neigh, 1))[:, :max_neigh], used


def celllist_csr(qpos, points, rc, box_lo, box_L, qr=None, nthreads=0):
    """Exact neighbor sets as CSR (offsets[Q+1] uint64, sorted neighbor ids)."""
    counts, _ = celllist_counts(qpos, points, rc, box_lo, box_L, qr=qr, nthreads=nthreads)
    offsets = np.zeros(len(counts) + 1, np.uint64)
    np.cumsum(counts, out=offsets[1:])
    nbrs = np.zeros(int(offsets[-1]), np.uint32)
    q = _f32(qpos, (-1, 3))
    p = _f32(points, (-1, 3))
    r = None if qr is None else _f32(qr)
    lib().orc_celllist_csr(_ptr(q), _ptr(r), rc, len(q), _ptr(p), len(p), _ptr(_f32(box_lo)),
                           _ptr(_f32(box_L)), _ptr(offsets), _ptr(nbrs), nthreads)
    return offsets, nbrs


def pair_distance_minus_rc_f64(pi, pj, rc, box_L=(0, 0, 0)):
    return lib().orc_pair_distance_minus_rc_f64(_ptr(_f32(pi)), _ptr(_f32(pj)), rc,
                                                _ptr(_f32(box_L)))


def fast_nodes(tree, leaf_size):
    """The project's traversal records restated: (records[n,4] uint32, frame[6])."""
    N = tree["N"]
    nodes = np.zeros((max(2 * N, 1), 4), np.uint32)
    frame = np.zeros(6, np.float32)
    n = lib().orc_fast_nodes(N, leaf_size, _ptr(tree["parent"]), _ptr(tree["left"]),
                             _ptr(tree["right"]), _ptr(tree["primitive"]), _ptr(tree["lo"]),
                             _ptr(tree["hi"]), _ptr(nodes), _ptr(frame))
    return nodes[:n].copy(), frame


def gen_validate_points(N=7500, L=(20.0, 15.0, 25.0), seed=42):
    out = np.zeros((N, 3), np.float32)
    lib().orc_gen_validate_points(N, _ptr(_f32(L)), seed, _ptr(out))
    return out


def images27(L):
    """27 periodic image vectors ordered as the reference's tests build them
    (ix, iy, iz each in -1..1, z fastest; test/lbvh_test.cu:427-440)."""
    L = np.asarray(L, np.float32)
    out = []
    for ix in (-1, 0, 1):
        for iy in (-1, 0, 1):
            for iz in (-1, 0, 1):
                out.append([L[0] * np.float32(ix), L[1] * np.float32(iy), L[2] * np.float32(iz)])
    return np.asarray(out, np.float32)


CAP_PARAMS = 6337
CAP_FEATURES = 32


def cap_occupancy(codes, shift):
    """Points per coarse Morton cell (G^3, G = 1024 >> shift) of the sorted codes."""
    c = np.ascontiguousarray(codes, np.uint32)
    G = 1024 >> shift
    occ = np.zeros(G ** 3, np.uint32)
    lib().orc_cap_occupancy(_ptr(c), len(c), shift, _ptr(occ))
    return occ


def cap_features(codes, points4, lo, ext, shift, periodic):
    """The 32 capacity features of every sorted point (points4: float4 payload)."""
    c = np.ascontiguousarray(codes, np.uint32)
    p = _f32(points4, (-1, 4))
    occ = cap_occupancy(c, shift)
    out = np.zeros((len(c), CAP_FEATURES), np.float32)
    lib().orc_cap_features(_ptr(c), _ptr(p), len(c), _ptr(_f32(lo)), _ptr(_f32(ext)), shift,
                           1 if periodic else 0, _ptr(occ), _ptr(out))
    return out


def cap_forward_backward(params, features, targets, batch, offset, stride, mode=1):
    """Summed gradient, summed loss and outputs of a batch; mode 1 = BF16 rounding as the GPU,
    0 = FP32 without rounding, -1 = float64 without rounding."""
    P = _f32(params)
    F = _f32(features, (-1, CAP_FEATURES))
    T = _f32(targets)
    grad = np.zeros(CAP_PARAMS, np.float64)
    loss = np.zeros(1, np.float64)
    y = np.zeros(batch, np.float32)
    lib().orc_cap_forward_backward(_ptr(P), _ptr(F), _ptr(T), len(T), batch, offset, stride, mode,
                                   _ptr(grad), _ptr(loss), _ptr(y))
    return grad, float(loss[0]), y


class FrameLister:
    """Whole-frame self neighbor list on the host cores (frame_list.cpp): the benchmark's CPU
    baseline.  Keeps its output buffers between frames, so that a timed call allocates nothing
    of the list's size."""

    def __init__(self, n, nthreads=0, slots_per_point=16):
        self.n = int(n)
        self.nthreads = int(nthreads)
        self.counts = np.empty(self.n, np.uint32)
        self.offsets = np.empty(self.n + 1, np.uint64)
        self.order = np.empty(self.n, np.uint32)
        self.list = np.empty(max(1, self.n * slots_per_point), np.uint32)

    def run(self, points, L, rc, lo=(0.0, 0.0, 0.0)):
        """List the frame; returns (total pairs, threads used, seconds of grid/count/scan/fill).
        Rows are in grid order (self.order[k] is the point of row k)."""
        p = _f32(points, (-1, 3))
        assert len(p) == self.n
        total = ctypes.c_uint64()
        secs = np.zeros(4, np.float64)
        used = lib().orc_frame_list(_ptr(p), self.n, _ptr(_f32(lo)), _ptr(_f32(L)), float(rc), self.nthreads,
                                    _ptr(self.counts), _ptr(self.offsets), _ptr(self.list), len(self.list),
                                    _ptr(self.order), ctypes.byref(total), _ptr(secs))
        if used < 0:   # more pairs than the buffer holds: grow it and list again
            self.list = np.empty(int(total.value * 1.25) + 1, np.uint32)
            used = lib().orc_frame_list(_ptr(p), self.n, _ptr(_f32(lo)), _ptr(_f32(L)), float(rc), self.nthreads,
                                        _ptr(self.counts), _ptr(self.offsets), _ptr(self.list), len(self.list),
                                        _ptr(self.order), ctypes.byref(total), _ptr(secs))
        return int(total.value), int(used), secs


def uniform_points(n, L, seed, lo=(0.0, 0.0, 0.0)):
    """n points uniform in [lo, lo+L) (host, counter-based generator)."""
    out = np.empty((int(n), 3), np.float32)
    lib().orc_uniform_points(_ptr(out), int(n), _ptr(_f32(lo)), _ptr(_f32(L)), int(seed))
    return out


def gaussian_move(points, L, sigma, seed, lo=(0.0, 0.0, 0.0), out=None):
    """Every point moved by an i.i.d. Gaussian of `sigma` per axis and wrapped into [lo, lo+L)."""
    p = _f32(points, (-1, 3))
    if out is None:
        out = np.empty_like(p)
    lib().orc_gaussian_move(_ptr(p), _ptr(out), len(p), _ptr(_f32(lo)), _ptr(_f32(L)), float(sigma), int(seed))
    return out
