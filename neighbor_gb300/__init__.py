"""neighbor_gb300: LBVH neighbor search on NVIDIA GB300 (sm_103a).

Python mirror of the library's C ABI (include/neighbor_gb300.h), which exports the C++ template
API in include/neighbor/ (LBVH, LBVHTraverser and the insert / query / output / translate /
transform ops of mphowardlab/neighbor).  Arrays are torch CUDA tensors; every call is enqueued on
the current torch stream unless a stream is passed.

There is no CPU fallback: if the CUDA library has not been built, or no GPU is present, the
calls raise.
"""
from __future__ import annotations

import ctypes
import os
import threading
from typing import Optional, Sequence

from . import _build

__all__ = ["LBVH", "LBVHTraverser", "NeighborError", "load", "build", "exact_pad", "images27",
           "QUERY_SPHERE", "QUERY_EXACT", "SENTINEL"]

QUERY_SPHERE = 0
QUERY_EXACT = 1
SENTINEL = 0x7FFFFFFF

NBR_OK = 0
_ERRORS = {1: "invalid argument", 2: "CUDA error", 3: "allocation failed",
           4: "bounded device wait gave up", 5: "unsupported"}


class NeighborError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{_ERRORS.get(code, 'error')} ({code}): {msg}")
        self.code = code


_lib = None
_lock = threading.Lock()


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile the CUDA library in-tree (nvcc, sm_103a)."""
    return _build.build(force=force, verbose=verbose)


def library_path() -> str:
    return _build.LIB_PATH


def load() -> ctypes.CDLL:
    """Load libneighbor_gb300.so; raises if it is missing (no fallback path exists)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(_build.LIB_PATH):
                raise RuntimeError("neighbor_gb300 CUDA library is not built "
                                   f"({_build.LIB_PATH}); run neighbor_gb300.build()")
            L = ctypes.CDLL(_build.LIB_PATH)
            _declare(L)
            _lib = L
    return _lib


_P = ctypes.c_void_p
_U = ctypes.c_uint
_I = ctypes.c_int
_F = ctypes.c_float
_PP = ctypes.POINTER(ctypes.c_void_p)


def _declare(L):
    def sig(name, args, res=ctypes.c_int):
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    sig("nbr_last_error", [], ctypes.c_char_p)
    sig("nbr_version", [ctypes.POINTER(_I), ctypes.POINTER(_I)])
    sig("nbr_lbvh_create", [_PP])
    sig("nbr_lbvh_destroy", [_P])
    sig("nbr_lbvh_set_leaf_size", [_P, _U])
    sig("nbr_lbvh_set_radix_bits", [_P, _U])
    sig("nbr_lbvh_set_climb_block", [_P, _U])
    sig("nbr_lbvh_build_points", [_P, _P, _U, _P, _P, _U, _P])
    sig("nbr_lbvh_build_spheres", [_P, _P, _F, _U, _P, _P, _U, _P])
    sig("nbr_lbvh_get_sizes", [_P, ctypes.POINTER(_I), ctypes.POINTER(_U), ctypes.POINTER(_U),
                               ctypes.POINTER(_U)])
    sig("nbr_lbvh_get_arrays", [_P, _PP, _PP, _PP, _PP, _PP, _PP])
    sig("nbr_lbvh_get_codes", [_P, _PP])
    sig("nbr_lbvh_get_primitives", [_P, _PP])
    sig("nbr_lbvh_get_fast", [_P, _PP, _PP, _PP, ctypes.POINTER(_U)])
    sig("nbr_lbvh_num_fast_nodes", [_P, ctypes.POINTER(_U), _P])
    sig("nbr_lbvh_check_status", [_P, _P])
    sig("nbr_traverser_create", [_PP])
    sig("nbr_traverser_destroy", [_P])
    sig("nbr_traverser_setup", [_P, _P, _P, _U, _P])
    sig("nbr_traverser_reset", [_P])
    sig("nbr_traverser_set_fast_path", [_P, _I])
    sig("nbr_traverser_set_mode", [_P, _I])
    sig("nbr_traverser_set_stats", [_P, _P])
    sig("nbr_traverser_set_symmetric", [_P, _I])
    sig("nbr_debug_inject_alloc_failures", [_U])
    sig("nbr_traverser_set_work_order", [_P, _I])
    sig("nbr_traverser_set_warp_walk_max", [_P, ctypes.c_uint])
    sig("nbr_traverser_set_pair_cache", [_P, _I])
    sig("nbr_traverser_set_symmetric_min_points", [_P, ctypes.c_uint])
    sig("nbr_traverser_set_walk_lanes", [_P, ctypes.c_uint])
    sig("nbr_traverser_set_half_walk_lanes", [_P, ctypes.c_uint])
    sig("nbr_traverser_get_data", [_P, _PP, _PP, _PP, _PP])
    sig("nbr_traverser_count_summary", [_P, ctypes.POINTER(_U), ctypes.POINTER(ctypes.c_ulonglong),
                                        ctypes.POINTER(_U), _P])
    sig("nbr_traverser_count_summary_device", [_P, _PP])
    sig("nbr_tune_self", [_P, _P, _P, _U, _P, _P, _F, _P, _F, _I, _U, _P, ctypes.POINTER(_U),
                          ctypes.POINTER(_U), ctypes.POINTER(_U), ctypes.POINTER(_F)])
    sig("nbr_tune_self_clear", [])
    sig("nbr_traverse", [_P, _P, _I, _P, _U, _P, _P, _F, _P, _U, _P, _P, _P, _U, _U, _P])
    sig("nbr_traverse_self", [_P, _P, _F, _P, _F, _P, _U, _P, _P, _P, _U, _I, _U, _P])
    sig("nbr_exact_pad", [_F, _F], _F)
    sig("nbr_lbvh_build_points_f64", [_P, _P, _U, _P, _P, _U, _P])
    sig("nbr_traverse_f64", [_P, _P, _P, _U, _P, _P, _F, _P, _U, _P, _P, _P, _U, _U, _P])
    sig("nbr_traverse_self_f64", [_P, _P, _P, ctypes.c_double, _P, _F, _P, _U, _P, _P, _P, _U, _I, _U, _P])
    sig("nbr_debug_wait_timeout", [ctypes.POINTER(_U), _P])
    sig("nbr_morton_sort_noalloc", [_P, _U, _P, _P, _P, _P, _P])
    sig("nbr_morton_sort_noalloc_status", [ctypes.POINTER(_U), _P])
    sig("nbr_debug_noalloc_wait_timeout", [_P, _U, _P, _P, _P, _P, _P])
    _ULL = ctypes.c_ulonglong
    sig("nbr_traverse_self_csr", [_P, _P, _F, _P, _F, _P, _U, _P, _P, _P, _P, _P, _U, _I, _U, _P])
    sig("nbr_traverse_self_subset_csr", [_P, _P, _F, _P, _F, _P, _U, _P, _P, _U, _P, _P, _P, _P, _I, _P])
    sig("nbr_capmodel_create", [_PP, _ULL])
    sig("nbr_capmodel_destroy", [_P])
    sig("nbr_capmodel_get_params", [_P, _P])
    sig("nbr_capmodel_set_params", [_P, _P])
    sig("nbr_capmodel_set_margin", [_P, _F])
    sig("nbr_capmodel_get_margin", [_P, ctypes.POINTER(_F)])
    sig("nbr_capmodel_set_margins", [_P, _P])
    sig("nbr_capmodel_save", [_P, ctypes.c_char_p])
    sig("nbr_capmodel_load", [_P, ctypes.c_char_p])
    sig("nbr_capmodel_get_margins", [_P, _P])
    sig("nbr_capmodel_set_infer_kernel", [_P, _I])
    sig("nbr_capmodel_get_infer_kernel", [_P, ctypes.POINTER(_I)])
    sig("nbr_capmodel_status", [_P, ctypes.POINTER(_U)])
    sig("nbr_capmodel_level", [_F, _P, _P, ctypes.POINTER(_U)])
    sig("nbr_capmodel_features", [_P, _P, _P, _P, _F, _I, _P, _P])
    sig("nbr_capmodel_predict", [_P, _P, _P, _P, _F, _I, _I, _U, _P, _P, _P])
    sig("nbr_capmodel_targets", [_P, _U, _P, _P])
    sig("nbr_capmodel_gradient", [_P, _P, _P, _U, _U, _U, _U, _P, _P, _P])
    sig("nbr_capmodel_train", [_P, _P, _P, _U, _U, _U, _F, _ULL, ctypes.POINTER(_F), _P])
    sig("nbr_onepass_create", [_PP])
    sig("nbr_onepass_destroy", [_P])
    sig("nbr_onepass_capacity", [_P, _U, _PP])
    sig("nbr_onepass_build", [_P, _P, _P, _F, _P, _F, _I, _I, _U, _P, _U, _P,
                              ctypes.POINTER(_ULL), ctypes.POINTER(_U), ctypes.POINTER(_ULL)])
    sig("nbr_onepass_get", [_P, _PP, _PP, _PP, _PP, ctypes.POINTER(_ULL)])
    sig("nbr_batch_create", [_PP])
    sig("nbr_batch_destroy", [_P])
    sig("nbr_batch_setup", [_P, _P, _P, _U, _F, _U])
    sig("nbr_batch_set_config", [_P, _U, _U])
    sig("nbr_batch_get_config", [_P, ctypes.POINTER(_U), ctypes.POINTER(_U)])
    sig("nbr_batch_run", [_P, _P, _P, _P, _P])
    sig("nbr_batch_tune", [_P, _P, _P, _P, _P, ctypes.POINTER(_U), ctypes.POINTER(_U)])
    sig("nbr_batch_capture", [_P, _P, _P, _P, _P])
    sig("nbr_batch_replay", [_P, _P])
    sig("nbr_batch_status", [_P, ctypes.POINTER(_U), ctypes.POINTER(_U), _P])
    sig("nbr_batch_sequential_plain", [_P, _P, _P, _P, _P, _U, _F, _P, _P, _U, _U, _P])
    sig("nbr_onepass_build_learned", [_P, _P, _P, _P, _P, _U, _P, _P, _F, _P, _F, _I, _I, _U, _P, _U, _P,
                                      ctypes.POINTER(_ULL), ctypes.POINTER(_U), ctypes.POINTER(_ULL)])
    sig("nbr_onepass_scan", [_P, _P, _U, _P, ctypes.POINTER(_ULL), _P])


# C-ABI symbols declared in include/neighbor_gb300.h (checked by the CPU tests).
EXPORTED = ["nbr_last_error", "nbr_version", "nbr_lbvh_create", "nbr_lbvh_destroy",
            "nbr_lbvh_set_leaf_size", "nbr_lbvh_set_radix_bits", "nbr_lbvh_set_climb_block",
            "nbr_lbvh_build_points",
            "nbr_lbvh_build_spheres", "nbr_lbvh_get_sizes", "nbr_lbvh_get_arrays",
            "nbr_lbvh_get_codes", "nbr_lbvh_get_primitives", "nbr_lbvh_get_fast", "nbr_lbvh_num_fast_nodes",
            "nbr_lbvh_check_status", "nbr_traverser_create", "nbr_traverser_destroy",
            "nbr_traverser_setup", "nbr_traverser_reset", "nbr_traverser_set_fast_path",
            "nbr_traverser_set_mode", "nbr_traverser_set_stats", "nbr_traverser_set_symmetric",
            "nbr_debug_inject_alloc_failures",
            "nbr_traverser_set_work_order", "nbr_traverser_set_warp_walk_max",
            "nbr_traverser_set_symmetric_min_points", "nbr_traverser_set_walk_lanes",
            "nbr_traverser_set_half_walk_lanes",
            "nbr_traverser_set_pair_cache", "nbr_traverser_count_summary",
            "nbr_traverser_count_summary_device", "nbr_tune_self", "nbr_tune_self_clear",
            "nbr_traverser_get_data", "nbr_traverse", "nbr_traverse_self", "nbr_exact_pad",
            "nbr_debug_wait_timeout", "nbr_morton_sort_noalloc", "nbr_morton_sort_noalloc_status",
            "nbr_debug_noalloc_wait_timeout", "nbr_traverse_self_csr",
            "nbr_traverse_self_subset_csr",
            "nbr_capmodel_create", "nbr_capmodel_destroy", "nbr_capmodel_get_params",
            "nbr_capmodel_set_params", "nbr_capmodel_set_margin", "nbr_capmodel_get_margin",
            "nbr_capmodel_set_margins", "nbr_capmodel_get_margins", "nbr_capmodel_save",
            "nbr_capmodel_load", "nbr_capmodel_set_infer_kernel", "nbr_capmodel_get_infer_kernel",
            "nbr_capmodel_status",
            "nbr_capmodel_level", "nbr_capmodel_features", "nbr_capmodel_predict",
            "nbr_capmodel_targets", "nbr_capmodel_gradient", "nbr_capmodel_train",
            "nbr_onepass_create", "nbr_onepass_destroy", "nbr_onepass_capacity",
            "nbr_onepass_build", "nbr_onepass_get", "nbr_onepass_scan", "nbr_onepass_build_learned",
            "nbr_batch_create", "nbr_batch_destroy", "nbr_batch_setup", "nbr_batch_set_config",
            "nbr_batch_get_config", "nbr_batch_run", "nbr_batch_tune", "nbr_batch_capture",
            "nbr_batch_replay", "nbr_batch_status", "nbr_batch_sequential_plain",
            "nbr_lbvh_build_points_f64", "nbr_traverse_f64", "nbr_traverse_self_f64"]

BATCH_MAX_N = 16384

CAP_PARAMS = 6337
CAP_FEATURES = 32
CAP_MARGIN_BINS = 16
CAP_INFER_WARP_TILES = 0      # mma.sync m16n8k16 warp tiles (k_cap_infer)
CAP_INFER_TENSOR_MEMORY = 1   # tcgen05 128-query tiles, Tensor Memory accumulators (k_cap_infer_tc)

NOALLOC_MAX_POINTS = 1 << 20


def _check(rc: int):
    if rc != NBR_OK:
        msg = load().nbr_last_error()
        raise NeighborError(rc, msg.decode() if msg else "")


def _torch():
    import torch
    return torch


def _stream_ptr(stream) -> Optional[int]:
    torch = _torch()
    if stream is None:
        stream = torch.cuda.current_stream()
    if isinstance(stream, int):
        return stream or None
    return stream.cuda_stream or None


def _dev(t, dtype, shape_last=None):
    """Validate a CUDA tensor argument and return it contiguous."""
    torch = _torch()
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError("expected a CUDA tensor")
    if t.dtype != dtype:
        raise TypeError(f"expected dtype {dtype}, got {t.dtype}")
    if shape_last is not None and (t.dim() != 2 or t.shape[1] != shape_last):
        raise ValueError(f"expected shape [n, {shape_last}], got {tuple(t.shape)}")
    return t.contiguous()


def _ptr(t) -> Optional[int]:
    return None if t is None else t.data_ptr()


def _f3(v) -> ctypes.Array:
    a = (ctypes.c_float * 3)(*[float(x) for x in v])
    return a


class _DeviceView:
    """Non-owning __cuda_array_interface__ over a device or managed pointer."""

    def __init__(self, ptr: int, shape, typestr: str):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr,
                                         "data": (int(ptr), False), "version": 3, "strides": None}


def _view(ptr, shape, typestr, dtype):
    torch = _torch()
    n = 1
    for s in shape:
        n *= s
    if n == 0 or not ptr:
        return torch.empty(shape, dtype=dtype, device="cuda")
    return torch.as_tensor(_DeviceView(ptr, shape, typestr), device="cuda")


def exact_pad(rc: float, coord_max: float) -> float:
    """Radius padding of the exact query (16 ulps of 2*coord_max plus 1e-6*rc)."""
    return float(load().nbr_exact_pad(float(rc), float(coord_max)))


def debug_wait_timeout(stream=None) -> int:
    """Run the scan with a tile that is never published; returns the device status word."""
    st = ctypes.c_uint()
    _check(load().nbr_debug_wait_timeout(ctypes.byref(st), _stream_ptr(stream)))
    return st.value


def _noalloc_args(points, codes_out, order_out):
    torch = _torch()
    p = _dev(points, torch.float32, 3)
    n = p.shape[0]
    for t in (codes_out, order_out):
        if not (isinstance(t, torch.Tensor) and t.is_cuda and t.is_contiguous() and t.numel() >= n
                and t.element_size() == 4):
            raise TypeError("outputs must be contiguous 4-byte CUDA tensors of N elements")
        if t.device != p.device:
            raise ValueError("points and outputs must be on one device")
    return p, n


def morton_sort_noalloc(points, lo, hi, codes_out, order_out, stream=None):
    """Morton codes of the points and their stable order, without any device allocation by the
    library: all working memory is its fixed device array (at most NOALLOC_MAX_POINTS points).
    codes_out / order_out: preallocated CUDA int32 tensors of N elements on the points' device
    (the call runs there).  A look-back wait that gave up is reported by morton_sort_noalloc_status."""
    torch = _torch()
    p, n = _noalloc_args(points, codes_out, order_out)
    with torch.cuda.device(p.device):
        _check(load().nbr_morton_sort_noalloc(_ptr(p), n, _f3(lo), _f3(hi), _ptr(codes_out),
                                              _ptr(order_out), _stream_ptr(stream)))


def morton_sort_noalloc_status(stream=None, device=None) -> int:
    """Status word of the last morton_sort_noalloc call on `device` (synchronises the stream);
    raises NeighborError (bounded device wait gave up) when it is set."""
    torch = _torch()
    st = ctypes.c_uint()
    with torch.cuda.device(device if device is not None else torch.cuda.current_device()):
        _check(load().nbr_morton_sort_noalloc_status(ctypes.byref(st), _stream_ptr(stream)))
    return st.value


def debug_noalloc_wait_timeout(points, lo, hi, codes_out, order_out, stream=None):
    """Test hook: the allocation-free sort with its first tile never run (the next look-back gives
    up); morton_sort_noalloc_status then reports it."""
    torch = _torch()
    p, n = _noalloc_args(points, codes_out, order_out)
    with torch.cuda.device(p.device):
        _check(load().nbr_debug_noalloc_wait_timeout(_ptr(p), n, _f3(lo), _f3(hi), _ptr(codes_out),
                                                     _ptr(order_out), _stream_ptr(stream)))


def tune_self(lbvh, trav, points, lo, hi, rc: float, box, pad: float, periodic: bool = True, reps: int = 3,
              stream=None):
    """Autotune the self neighbor list of `points` (leaf size, sort digit width, climb block) by
    timing the whole two-pass step on them; applies the fastest to `lbvh` and returns it as a
    dict (ms = 0 when the workload's class was cached)."""
    torch = _torch()
    p = _dev(points, torch.float32, 3)
    leaf, bits, climb = ctypes.c_uint(), ctypes.c_uint(), ctypes.c_uint()
    ms = ctypes.c_float()
    _check(load().nbr_tune_self(lbvh.handle, trav._h, _ptr(p), p.shape[0], _f3(lo), _f3(hi), float(rc), _f3(box),
                                float(pad), 1 if periodic else 0, int(reps), _stream_ptr(stream), ctypes.byref(leaf),
                                ctypes.byref(bits), ctypes.byref(climb), ctypes.byref(ms)))
    return {"leaf_size": leaf.value, "radix_bits": bits.value, "climb_block": climb.value, "ms": ms.value}


def tune_self_clear():
    """Forget every configuration tune_self has cached."""
    _check(load().nbr_tune_self_clear())


def inject_alloc_failures(count: int):
    """Test hook: the library's next `count` device allocations fail (NBR_ERR_ALLOC)."""
    _check(load().nbr_debug_inject_alloc_failures(int(count)))


def images27(L: Sequence[float], device="cuda"):
    """27 periodic image vectors, ix/iy/iz in -1..1 with iz fastest."""
    torch = _torch()
    out = []
    for ix in (-1, 0, 1):
        for iy in (-1, 0, 1):
            for iz in (-1, 0, 1):
                out.append([float(L[0]) * ix, float(L[1]) * iy, float(L[2]) * iz])
    return torch.tensor(out, dtype=torch.float32, device=device)


class LBVH:
    """neighbor::LBVH (include/neighbor/LBVH.h) through the C ABI."""

    def __init__(self, leaf_size: Optional[int] = None, radix_bits: Optional[int] = None,
                 climb_block: Optional[int] = None):
        L = load()
        h = ctypes.c_void_p()
        _check(L.nbr_lbvh_create(ctypes.byref(h)))
        self._h = h
        self._L = L
        if leaf_size is not None:
            self.set_leaf_size(leaf_size)
        if radix_bits is not None:
            self.set_radix_bits(radix_bits)
        if climb_block is not None:
            self.set_climb_block(climb_block)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                self._L.nbr_lbvh_destroy(h)
            except Exception:
                pass
            self._h = None

    @property
    def handle(self):
        return self._h

    def set_leaf_size(self, n: int):
        _check(self._L.nbr_lbvh_set_leaf_size(self._h, int(n)))

    def set_radix_bits(self, bits: int):
        _check(self._L.nbr_lbvh_set_radix_bits(self._h, int(bits)))

    def build_f64(self, points, lo, hi, block_size: int = 32, stream=None):
        """LBVH::build with PointInsertOpF64: points is a CUDA float64 [N, 3] tensor."""
        torch = _torch()
        p = _dev(points, torch.float64, 3)
        _check(self._L.nbr_lbvh_build_points_f64(self._h, _ptr(p), p.shape[0], _f3(lo), _f3(hi), block_size,
                                                 _stream_ptr(stream)))

    def set_climb_block(self, leaves: int):
        """Sorted leaves per block of the build's agglomerative climb (128, 256 or 512)."""
        _check(self._L.nbr_lbvh_set_climb_block(self._h, int(leaves)))

    def build(self, points, lo, hi, radius: Optional[float] = None, block_size: int = 32,
              stream=None):
        """LBVH::build with PointInsertOp (radius None) or SphereInsertOp(radius)."""
        p = _dev(points, _torch().float32, 3)
        self._points = p  # keep the input alive while the build is in flight
        n = p.shape[0]
        s = _stream_ptr(stream)
        if radius is None:
            _check(self._L.nbr_lbvh_build_points(self._h, _ptr(p), n, _f3(lo), _f3(hi), block_size, s))
        else:
            _check(self._L.nbr_lbvh_build_spheres(self._h, _ptr(p), float(radius), n, _f3(lo),
                                                  _f3(hi), block_size, s))
        return self

    def sizes(self):
        root, N, ni, nn = ctypes.c_int(), ctypes.c_uint(), ctypes.c_uint(), ctypes.c_uint()
        _check(self._L.nbr_lbvh_get_sizes(self._h, ctypes.byref(root), ctypes.byref(N),
                                          ctypes.byref(ni), ctypes.byref(nn)))
        return root.value, N.value, ni.value, nn.value

    def getRoot(self):
        return self.sizes()[0]

    def getN(self):
        return self.sizes()[1]

    def getNInternal(self):
        return self.sizes()[2]

    def getNNodes(self):
        return self.sizes()[3]

    def _arrays(self):
        ptrs = [ctypes.c_void_p() for _ in range(6)]
        _check(self._L.nbr_lbvh_get_arrays(self._h, *[ctypes.byref(p) for p in ptrs]))
        return [p.value for p in ptrs]

    def arrays(self):
        """Copies of parent, left, right, primitive, lo, hi (reference layout) as CUDA tensors."""
        torch = _torch()
        _, N, ni, nn = self.sizes()
        par, lft, rgt, prim, lo, hi = self._arrays()
        return dict(
            parent=_view(par, (nn,), "<i4", torch.int32).clone(),
            left=_view(lft, (ni,), "<i4", torch.int32).clone(),
            right=_view(rgt, (ni,), "<i4", torch.int32).clone(),
            primitive=_view(prim, (N,), "<u4", torch.int32).clone(),
            lo=_view(lo, (nn, 3), "<f4", torch.float32).clone(),
            hi=_view(hi, (nn, 3), "<f4", torch.float32).clone(),
        )

    def primitives(self):
        """View of the sorted primitive order (getPrimitives())."""
        torch = _torch()
        _, N, _, _ = self.sizes()
        p = ctypes.c_void_p()
        _check(self._L.nbr_lbvh_get_primitives(self._h, ctypes.byref(p)))
        return _view(p.value, (N,), "<u4", torch.int32)

    def codes(self):
        torch = _torch()
        _, N, _, _ = self.sizes()
        p = ctypes.c_void_p()
        _check(self._L.nbr_lbvh_get_codes(self._h, ctypes.byref(p)))
        return _view(p.value, (N,), "<u4", torch.int32).clone()

    def num_fast_nodes(self, stream=None) -> int:
        n = ctypes.c_uint()
        _check(self._L.nbr_lbvh_num_fast_nodes(self._h, ctypes.byref(n), _stream_ptr(stream)))
        return n.value

    def fast(self, stream=None):
        """Copies of the traversal records, the sorted payload and the frame."""
        torch = _torch()
        n = self.num_fast_nodes(stream)
        nodes, pts, frame = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
        ls = ctypes.c_uint()
        _check(self._L.nbr_lbvh_get_fast(self._h, ctypes.byref(nodes), ctypes.byref(pts),
                                         ctypes.byref(frame), ctypes.byref(ls)))
        _, N, _, _ = self.sizes()
        return dict(nodes=_view(nodes.value, (n, 4), "<u4", torch.int32).clone(),
                    points=_view(pts.value, (N, 4), "<f4", torch.float32).clone(),
                    frame=_view(frame.value, (9,), "<f4", torch.float32).clone(),
                    leaf_size=ls.value)

    def check_status(self, stream=None):
        _check(self._L.nbr_lbvh_check_status(self._h, _stream_ptr(stream)))


class LBVHTraverser:
    """neighbor::LBVHTraverser (include/neighbor/LBVHTraverser.h) through the C ABI."""

    def __init__(self):
        L = load()
        h = ctypes.c_void_p()
        _check(L.nbr_traverser_create(ctypes.byref(h)))
        self._h = h
        self._L = L

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                self._L.nbr_traverser_destroy(h)
            except Exception:
                pass
            self._h = None

    def setup(self, lbvh: LBVH, map=None, block_size: int = 32, stream=None):
        m = None if map is None else _dev(map, _torch().int32)
        _check(self._L.nbr_traverser_setup(self._h, lbvh.handle, _ptr(m), block_size,
                                           _stream_ptr(stream)))

    def reset(self):
        _check(self._L.nbr_traverser_reset(self._h))

    def set_fast_path(self, enabled: bool):
        _check(self._L.nbr_traverser_set_fast_path(self._h, 1 if enabled else 0))

    def set_stats(self, counters):
        """counters: CUDA int64 tensor of 3 (node visits, point tests, packets) or None."""
        self._stats = counters
        _check(self._L.nbr_traverser_set_stats(self._h, None if counters is None else counters.data_ptr()))

    def set_symmetric(self, enabled: bool):
        """Self traversals: find each pair once and write both rows (True, default)."""
        _check(self._L.nbr_traverser_set_symmetric(self._h, 1 if enabled else 0))

    def set_work_order(self, enabled: bool):
        """Symmetric fills take each block's queries in order of the walk lengths of the last
        symmetric count over the same tree (True, default)."""
        _check(self._L.nbr_traverser_set_work_order(self._h, 1 if enabled else 0))

    def set_pair_cache(self, enabled: bool):
        """Pair exchange: a symmetric count keeps each point's pairs so that the next fill
        assembles the rows without walking (True, default)."""
        _check(self._L.nbr_traverser_set_pair_cache(self._h, 1 if enabled else 0))

    def count_summary(self, stream=None):
        """(largest count, total of the counts, rows past the pair exchange) of the last counting
        self traversal; synchronises the stream."""
        mx, past = ctypes.c_uint(), ctypes.c_uint()
        tot = ctypes.c_ulonglong()
        _check(self._L.nbr_traverser_count_summary(self._h, ctypes.byref(mx), ctypes.byref(tot),
                                                   ctypes.byref(past), _stream_ptr(stream)))
        return mx.value, tot.value, past.value

    def count_summary_device(self):
        """Device address of the summary words ([0] max, [1] rows past the exchange, [2..3]
        64-bit total), or 0 before the first count."""
        p = ctypes.c_void_p()
        _check(self._L.nbr_traverser_count_summary_device(self._h, ctypes.byref(p)))
        return p.value or 0

    def set_warp_walk_max(self, max_queries: int):
        """Traversals of at most max_queries queries walk one warp per query (0 = never)."""
        _check(self._L.nbr_traverser_set_warp_walk_max(self._h, int(max_queries)))

    def set_symmetric_min_points(self, min_points: int):
        """Self traversals take the symmetric walk only above min_points points (0 = any)."""
        _check(self._L.nbr_traverser_set_symmetric_min_points(self._h, int(min_points)))

    def set_walk_lanes(self, lanes: int):
        """Lanes per query of small traversals: 4, 8, 16 or 32 (0 = by size)."""
        _check(self._L.nbr_traverser_set_walk_lanes(self._h, int(lanes)))

    def set_half_walk_lanes(self, lanes: int):
        """Lanes per query of the exchanging symmetric count: 1, 4, 8, 16 or 32 (0 = by size)."""
        _check(self._L.nbr_traverser_set_half_walk_lanes(self._h, int(lanes)))

    def force_symmetric(self):
        """The symmetric walk for self traversals of every size (no size routing)."""
        self.set_symmetric(True)
        self.set_warp_walk_max(0)
        self.set_symmetric_min_points(0)

    def set_mode(self, mode: int):
        """0 = one thread per query, 1 = one warp per 32 consecutive queries."""
        _check(self._L.nbr_traverser_set_mode(self._h, int(mode)))

    def get_data(self, lbvh: LBVH):
        """Copy of getData() (int4 reference-layout nodes) and the compression frame."""
        torch = _torch()
        d, lo, hi, bins = (ctypes.c_void_p() for _ in range(4))
        _check(self._L.nbr_traverser_get_data(self._h, ctypes.byref(d), ctypes.byref(lo),
                                              ctypes.byref(hi), ctypes.byref(bins)))
        nn = lbvh.getNNodes()
        return dict(data=_view(d.value, (nn, 4), "<i4", torch.int32).clone(),
                    lo=_view(lo.value, (3,), "<f4", torch.float32).clone(),
                    hi=_view(hi.value, (3,), "<f4", torch.float32).clone(),
                    bins=_view(bins.value, (3,), "<f4", torch.float32).clone())

    def traverse(self, lbvh: LBVH, spheres, query: int = QUERY_SPHERE, points=None, box=None,
                 pad: float = 0.0, images=None, map=None, max_neigh: Optional[int] = None,
                 nneigh=None, neigh_list=None, block_size: int = 32, stream=None):
        """LBVHTraverser::traverse with Count (max_neigh None) or NeighborList output.

        images: a CUDA float32 [n, 3] tensor, None (self image only) or "periodic" (the 27 images
        of `box`).  Returns nneigh, or (nneigh, list[Q, max_neigh])."""
        torch = _torch()
        sph = _dev(spheres, torch.float32, 4)
        Q = sph.shape[0]
        pts = None if points is None else _dev(points, torch.float32, 3)
        lattice = isinstance(images, str) and images == "periodic"
        img = None if images is None or lattice else _dev(images, torch.float32, 3)
        m = None if map is None else _dev(map, torch.int32)
        if nneigh is None:
            nneigh = torch.empty(Q, dtype=torch.int32, device=sph.device)
        lst = neigh_list
        if max_neigh is not None and lst is None:
            lst = torch.full((Q, max(max_neigh, 1)), -1, dtype=torch.int32, device=sph.device)
        b = _f3(box if box is not None else (0.0, 0.0, 0.0))
        _check(self._L.nbr_traverse(self._h, lbvh.handle, int(query), _ptr(sph), Q, _ptr(pts), b,
                                    float(pad), _ptr(img),
                                    27 if lattice else (0 if img is None else img.shape[0]),
                                    _ptr(m), _ptr(nneigh), _ptr(lst),
                                    0 if max_neigh is None else int(max_neigh), block_size,
                                    _stream_ptr(stream)))
        if max_neigh is None:
            return nneigh
        return nneigh, lst

    def traverse_f64(self, lbvh: LBVH, spheres, points, box, pad: float, images=None, map=None,
                     max_neigh: Optional[int] = None, nneigh=None, neigh_list=None, block_size: int = 256,
                     stream=None):
        """Exact sphere queries on double positions (ExactSphereQueryOpF64): spheres float64 [Q, 4],
        points float64 [N, 3], box the periodic lengths (0 = open), images as traverse().  On a
        tree of double points this is the double fast walk, one thread per query in blocks of
        block_size."""
        torch = _torch()
        sph = _dev(spheres, torch.float64, 4)
        pts = _dev(points, torch.float64, 3)
        Q = sph.shape[0]
        lattice = isinstance(images, str) and images == "periodic"
        img = None if images is None or lattice else _dev(images, torch.float32, 3)
        m = None if map is None else _dev(map, torch.int32)
        if nneigh is None:
            nneigh = torch.empty(Q, dtype=torch.int32, device=sph.device)
        lst = neigh_list
        if max_neigh is not None and lst is None:
            lst = torch.full((Q, max(max_neigh, 1)), -1, dtype=torch.int32, device=sph.device)
        b = (ctypes.c_double * 3)(*[float(x) for x in box])
        _check(self._L.nbr_traverse_f64(self._h, lbvh.handle, _ptr(sph), Q, _ptr(pts), b, float(pad), _ptr(img),
                                        27 if lattice else (0 if img is None else img.shape[0]), _ptr(m),
                                        _ptr(nneigh), _ptr(lst), 0 if max_neigh is None else int(max_neigh),
                                        block_size, _stream_ptr(stream)))
        if max_neigh is None:
            return nneigh
        return nneigh, lst

    def traverse_self_f64(self, lbvh: LBVH, points, rc: float, box, pad: float, images=None, map=None,
                          max_neigh: Optional[int] = None, rows_sorted: bool = True, nneigh=None,
                          neigh_list=None, block_size: int = 256, stream=None):
        """Every primitive of a tree of double points queries the tree with cutoff rc (exact double
        predicate): points float64 [N, 3] are the tree's own points by primitive id; rows and
        images as traverse_self.  Equals traverse_f64 over the spheres (points[primitives], rc)."""
        torch = _torch()
        pts = _dev(points, torch.float64, 3)
        _, N, _, _ = lbvh.sizes()
        lattice = isinstance(images, str) and images == "periodic"
        img = None if images is None or lattice else _dev(images, torch.float32, 3)
        m = None if map is None else _dev(map, torch.int32)
        if nneigh is None:
            nneigh = torch.empty(N, dtype=torch.int32, device=pts.device)
        lst = neigh_list
        if max_neigh is not None and lst is None:
            lst = torch.full((N, max(max_neigh, 1)), -1, dtype=torch.int32, device=pts.device)
        b = (ctypes.c_double * 3)(*[float(x) for x in box])
        _check(self._L.nbr_traverse_self_f64(self._h, lbvh.handle, _ptr(pts), float(rc), b, float(pad), _ptr(img),
                                             27 if lattice else (0 if img is None else img.shape[0]), _ptr(m),
                                             _ptr(nneigh), _ptr(lst), 0 if max_neigh is None else int(max_neigh),
                                             1 if rows_sorted else 0, block_size, _stream_ptr(stream)))
        if max_neigh is None:
            return nneigh
        return nneigh, lst

    def traverse_self(self, lbvh: LBVH, rc: float, box, pad: float, images=None, map=None,
                      max_neigh: Optional[int] = None, rows_sorted: bool = True, nneigh=None,
                      neigh_list=None, block_size: int = 256, stream=None):
        """Every primitive of a point tree queries the tree (exact predicate, fast path)."""
        torch = _torch()
        _, N, _, _ = lbvh.sizes()
        lattice = isinstance(images, str) and images == "periodic"
        img = None if images is None or lattice else _dev(images, torch.float32, 3)
        m = None if map is None else _dev(map, torch.int32)
        if nneigh is None:
            nneigh = torch.empty(N, dtype=torch.int32, device="cuda")
        lst = neigh_list
        if max_neigh is not None and lst is None:
            lst = torch.full((N, max(max_neigh, 1)), -1, dtype=torch.int32, device="cuda")
        _check(self._L.nbr_traverse_self(self._h, lbvh.handle, float(rc), _f3(box), float(pad),
                                         _ptr(img),
                                         27 if lattice else (0 if img is None else img.shape[0]),
                                         _ptr(m),
                                         _ptr(nneigh), _ptr(lst),
                                         0 if max_neigh is None else int(max_neigh),
                                         1 if rows_sorted else 0, block_size,
                                         _stream_ptr(stream)))
        if max_neigh is None:
            return nneigh
        return nneigh, lst

    def traverse_self_csr(self, lbvh: LBVH, rc: float, box, pad: float, offsets, caps, list_out,
                          max_capacity: int = 0, images=None, map=None, rows_sorted: bool = True,
                          nneigh=None, block_size: int = 256, stream=None):
        """Self traversal into a CSR list: row r at list_out[offsets[r]:offsets[r]+caps[r]].
        offsets: CUDA int64 tensor, caps: int32, list_out: int32.  Returns the counts."""
        torch = _torch()
        _, N, _, _ = lbvh.sizes()
        lattice = isinstance(images, str) and images == "periodic"
        img = None if images is None or lattice else _dev(images, torch.float32, 3)
        m = None if map is None else _dev(map, torch.int32)
        if nneigh is None:
            nneigh = torch.empty(N, dtype=torch.int32, device="cuda")
        _check(self._L.nbr_traverse_self_csr(self._h, lbvh.handle, float(rc), _f3(box), float(pad),
                                             _ptr(img),
                                             27 if lattice else (0 if img is None else img.shape[0]),
                                             _ptr(m), _ptr(nneigh), _ptr(list_out), _ptr(offsets),
                                             _ptr(caps), int(max_capacity), 1 if rows_sorted else 0,
                                             block_size, _stream_ptr(stream)))
        return nneigh

    def traverse_self_subset_csr(self, lbvh: LBVH, rc: float, box, pad: float, subset, offsets, caps, list_out,
                                 images=None, map=None, rows_sorted: bool = True, nneigh=None, stream=None):
        """traverseSelfSubset: only the rows of the sorted positions in `subset` (CUDA int32) are
        written into the CSR list (one warp per row); returns nneigh."""
        torch = _torch()
        _, N, _, _ = lbvh.sizes()
        sub = _dev(subset, torch.int32)
        lattice = isinstance(images, str) and images == "periodic"
        img = None if images is None or lattice else _dev(images, torch.float32, 3)
        m = None if map is None else _dev(map, torch.int32)
        if nneigh is None:
            nneigh = torch.zeros(N, dtype=torch.int32, device="cuda")
        _check(self._L.nbr_traverse_self_subset_csr(self._h, lbvh.handle, float(rc), _f3(box), float(pad), _ptr(img),
                                                     27 if lattice else (0 if img is None else img.shape[0]), _ptr(m),
                                                     _ptr(sub), sub.shape[0], _ptr(nneigh), _ptr(list_out),
                                                     _ptr(offsets), _ptr(caps), 1 if rows_sorted else 0,
                                                     _stream_ptr(stream)))
        return nneigh


class CapacityModel:
    """Capacity network (32 -> 64 -> 64 -> 1, BF16 weights, FP32 accumulation) on the GPU."""

    def __init__(self, seed: int = 1):
        self._L = load()
        h = ctypes.c_void_p()
        _check(self._L.nbr_capmodel_create(ctypes.byref(h), int(seed)))
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None):
            self._L.nbr_capmodel_destroy(self._h)
            self._h = None

    @property
    def handle(self):
        return self._h

    def params(self):
        import numpy as np
        out = np.zeros(CAP_PARAMS, np.float32)
        _check(self._L.nbr_capmodel_get_params(self._h, out.ctypes.data_as(ctypes.c_void_p)))
        return out

    def set_params(self, params):
        import numpy as np
        p = np.ascontiguousarray(params, np.float32)
        if p.size != CAP_PARAMS:
            raise ValueError("expected %d parameters" % CAP_PARAMS)
        _check(self._L.nbr_capmodel_set_params(self._h, p.ctypes.data_as(ctypes.c_void_p)))

    @property
    def margin(self) -> float:
        v = ctypes.c_float()
        _check(self._L.nbr_capmodel_get_margin(self._h, ctypes.byref(v)))
        return v.value

    @margin.setter
    def margin(self, value: float):
        _check(self._L.nbr_capmodel_set_margin(self._h, float(value)))

    @property
    def margins(self):
        """Calibration table: margin of each bin of 0.5 in the output (the last bin open)."""
        t = (ctypes.c_float * CAP_MARGIN_BINS)()
        _check(self._L.nbr_capmodel_get_margins(self._h, ctypes.cast(t, ctypes.c_void_p)))
        return list(t)

    @margins.setter
    def margins(self, table):
        t = (ctypes.c_float * CAP_MARGIN_BINS)(*[float(v) for v in table])
        _check(self._L.nbr_capmodel_set_margins(self._h, ctypes.cast(t, ctypes.c_void_p)))

    @property
    def infer_kernel(self) -> int:
        """CAP_INFER_WARP_TILES or CAP_INFER_TENSOR_MEMORY: the kernel predict() runs."""
        v = ctypes.c_int()
        _check(self._L.nbr_capmodel_get_infer_kernel(self._h, ctypes.byref(v)))
        return v.value

    @infer_kernel.setter
    def infer_kernel(self, kernel: int):
        _check(self._L.nbr_capmodel_set_infer_kernel(self._h, int(kernel)))

    def status(self) -> int:
        """Device status word of the inference, read and cleared (4 = a tensor-core wait gave up)."""
        v = ctypes.c_uint()
        _check(self._L.nbr_capmodel_status(self._h, ctypes.byref(v)))
        return v.value

    def save(self, path: str):
        """Write the weights file (parameters, margin table, shapes, hash)."""
        _check(self._L.nbr_capmodel_save(self._h, os.fsencode(path)))

    def load(self, path: str):
        """Read a weights file written by save(); a damaged or foreign file raises."""
        _check(self._L.nbr_capmodel_load(self._h, os.fsencode(path)))

    def calibrate(self, targets, y, quantile: float = 0.999, min_rows: int = 1000):
        """Set the calibration table from residuals: bin b gets the `quantile` of target - y over the
        rows whose output y falls in bin b (width 0.5, the last bin open, as the inference bins
        it); a bin with fewer than min_rows rows gets the quantile over all rows.  Returns it."""
        torch = _torch()
        t = _dev(targets, torch.float32).reshape(-1)
        yy = _dev(y, torch.float32).reshape(-1)
        r = t - yy
        b = torch.clamp(torch.floor(yy * 2.0), 0, CAP_MARGIN_BINS - 1).to(torch.int64)

        def q(v):
            s, _ = torch.sort(v)
            return float(s[min(s.numel() - 1, int(quantile * s.numel()))].item())

        overall = q(r)
        table = []
        for k in range(CAP_MARGIN_BINS):
            sel = r[b == k]
            table.append(q(sel) if sel.numel() >= min_rows else overall)
        self.margins = table
        return table

    @staticmethod
    def level(rc, lo, hi) -> int:
        v = ctypes.c_uint()
        _check(load().nbr_capmodel_level(float(rc), _f3(lo), _f3(hi), ctypes.byref(v)))
        return v.value

    def features(self, lbvh: "LBVH", lo, hi, rc: float, periodic: bool = True, stream=None):
        torch = _torch()
        _, N, _, _ = lbvh.sizes()
        out = torch.empty((N, CAP_FEATURES), dtype=torch.float32, device="cuda")
        _check(self._L.nbr_capmodel_features(self._h, lbvh.handle, _f3(lo), _f3(hi), float(rc),
                                             1 if periodic else 0, _ptr(out), _stream_ptr(stream)))
        return out

    def predict(self, lbvh: "LBVH", lo, hi, rc: float, periodic: bool = True, rows_sorted: bool = True,
                cap_max: int = 4096, caps=None, want_y: bool = False, stream=None):
        torch = _torch()
        _, N, _, _ = lbvh.sizes()
        if caps is None:
            caps = torch.empty(N, dtype=torch.int32, device="cuda")
        y = torch.empty(N, dtype=torch.float32, device="cuda") if want_y else None
        _check(self._L.nbr_capmodel_predict(self._h, lbvh.handle, _f3(lo), _f3(hi), float(rc),
                                            1 if periodic else 0, 1 if rows_sorted else 0, int(cap_max),
                                            _ptr(caps), _ptr(y), _stream_ptr(stream)))
        return (caps, y) if want_y else caps

    @staticmethod
    def targets(counts, stream=None):
        torch = _torch()
        c = _dev(counts, torch.int32)
        out = torch.empty(c.shape[0], dtype=torch.float32, device="cuda")
        _check(load().nbr_capmodel_targets(_ptr(c), c.shape[0], _ptr(out), _stream_ptr(stream)))
        return out

    def gradient(self, features, targets, batch: int, offset: int, stride: int, stream=None):
        torch = _torch()
        F = _dev(features, torch.float32, CAP_FEATURES)
        T = _dev(targets, torch.float32)
        grad = torch.empty(CAP_PARAMS, dtype=torch.float32, device="cuda")
        loss = torch.empty(1, dtype=torch.float32, device="cuda")
        _check(self._L.nbr_capmodel_gradient(self._h, _ptr(F), _ptr(T), T.shape[0], int(batch),
                                             int(offset), int(stride), _ptr(grad), _ptr(loss),
                                             _stream_ptr(stream)))
        return grad, loss

    def train(self, features, targets, steps: int, batch: int = 8192, lr: float = 3e-3, seed: int = 1,
              stream=None) -> float:
        torch = _torch()
        F = _dev(features, torch.float32, CAP_FEATURES)
        T = _dev(targets, torch.float32)
        loss = ctypes.c_float()
        _check(self._L.nbr_capmodel_train(self._h, _ptr(F), _ptr(T), T.shape[0], int(steps), int(batch),
                                          float(lr), int(seed), ctypes.byref(loss), _stream_ptr(stream)))
        return loss.value


class OnePassList:
    """One-pass self neighbor list in CSR form with per-row capacities."""

    def __init__(self):
        self._L = load()
        h = ctypes.c_void_p()
        _check(self._L.nbr_onepass_create(ctypes.byref(h)))
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None):
            self._L.nbr_onepass_destroy(self._h)
            self._h = None

    def capacity(self, N: int):
        """The device capacity array of N rows (an int32 CUDA view) to fill before build()."""
        torch = _torch()
        p = ctypes.c_void_p()
        _check(self._L.nbr_onepass_capacity(self._h, int(N), ctypes.byref(p)))
        return _view(p.value, (N,), "<u4", torch.int32)

    def build(self, trav: "LBVHTraverser", lbvh: "LBVH", rc: float, box, pad: float, periodic: bool = True,
              rows_sorted: bool = True, cap_max: int = 4096, map=None, block_size: int = 256, stream=None):
        torch = _torch()
        m = None if map is None else _dev(map, torch.int32)
        slots, ovf, ovf_slots = ctypes.c_ulonglong(), ctypes.c_uint(), ctypes.c_ulonglong()
        _check(self._L.nbr_onepass_build(self._h, trav._h, lbvh.handle, float(rc), _f3(box), float(pad),
                                         1 if periodic else 0, 1 if rows_sorted else 0, int(cap_max), _ptr(m),
                                         block_size, _stream_ptr(stream), ctypes.byref(slots),
                                         ctypes.byref(ovf), ctypes.byref(ovf_slots)))
        return dict(slots=slots.value, overflow_rows=ovf.value, overflow_slots=ovf_slots.value)

    def build_learned(self, model: "CapacityModel", trav: "LBVHTraverser", lbvh: "LBVH", points, lo, hi,
                      rc: float, box, pad: float, periodic: bool = True, rows_sorted: bool = True,
                      cap_max: int = 32, map=None, block_size: int = 256, stream=None):
        """Build the tree of `points`, predict capacities with `model` (on a second stream from the
        end of the sort on) and fill the list, in one call."""
        torch = _torch()
        p = _dev(points, torch.float32, 3)
        m = None if map is None else _dev(map, torch.int32)
        slots, ovf, ovf_slots = ctypes.c_ulonglong(), ctypes.c_uint(), ctypes.c_ulonglong()
        _check(self._L.nbr_onepass_build_learned(self._h, model.handle, trav._h, lbvh.handle, _ptr(p), p.shape[0],
                                                 _f3(lo), _f3(hi), float(rc), _f3(box), float(pad),
                                                 1 if periodic else 0, 1 if rows_sorted else 0, int(cap_max),
                                                 _ptr(m), block_size, _stream_ptr(stream), ctypes.byref(slots),
                                                 ctypes.byref(ovf), ctypes.byref(ovf_slots)))
        return dict(slots=slots.value, overflow_rows=ovf.value, overflow_slots=ovf_slots.value)

    def result(self, N: int):
        """Views of (list, offsets, capacities, counts) of the last build."""
        torch = _torch()
        lst, off, caps, nn = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
        total = ctypes.c_ulonglong()
        _check(self._L.nbr_onepass_get(self._h, ctypes.byref(lst), ctypes.byref(off), ctypes.byref(caps),
                                       ctypes.byref(nn), ctypes.byref(total)))
        return dict(list=_view(lst.value, (max(total.value, 1),), "<u4", torch.int32),
                    offsets=_view(off.value, (N,), "<i8", torch.int64),
                    caps=_view(caps.value, (N,), "<u4", torch.int32),
                    nneigh=_view(nn.value, (N,), "<u4", torch.int32),
                    total=total.value)

    def scan(self, counts, stream=None, out=None, read_total: bool = True):
        """Exclusive scan of int32 counts into int64 offsets; returns (offsets, total).  With
        read_total False the scan is only enqueued (no synchronisation) and total is None."""
        torch = _torch()
        c = _dev(counts, torch.int32)
        if out is None:
            out = torch.empty(c.shape[0], dtype=torch.int64, device="cuda")
        total = ctypes.c_ulonglong()
        _check(self._L.nbr_onepass_scan(self._h, _ptr(c), c.shape[0], _ptr(out),
                                        ctypes.byref(total) if read_total else None, _stream_ptr(stream)))
        return out, (total.value if read_total else None)


class BatchedList:
    """Many independent small periodic systems, built and listed in one launch."""

    def __init__(self):
        self._L = load()
        h = ctypes.c_void_p()
        _check(self._L.nbr_batch_create(ctypes.byref(h)))
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None):
            self._L.nbr_batch_destroy(self._h)
            self._h = None

    def setup(self, start, boxes, rc: float, max_neigh: int):
        """start: S + 1 point offsets, boxes: S x 3 periodic lengths (host sequences)."""
        import numpy as np
        st = np.ascontiguousarray(start, np.uint32)
        bx = np.ascontiguousarray(boxes, np.float32).reshape(-1)
        S = len(st) - 1
        self.S, self.T, self.max_neigh = S, int(st[-1]), int(max_neigh)
        self._start, self._boxes = st, bx
        _check(self._L.nbr_batch_setup(self._h, st.ctypes.data_as(ctypes.c_void_p),
                                       bx.ctypes.data_as(ctypes.c_void_p), S, float(rc), int(max_neigh)))

    def outputs(self):
        torch = _torch()
        return (torch.empty(max(self.T, 1), dtype=torch.int32, device="cuda"),
                torch.empty(max(self.T, 1) * max(self.max_neigh, 1), dtype=torch.int32, device="cuda"))

    def set_config(self, leaf_size: int, block: int):
        _check(self._L.nbr_batch_set_config(self._h, int(leaf_size), int(block)))

    def config(self):
        leaf, block = ctypes.c_uint(), ctypes.c_uint()
        _check(self._L.nbr_batch_get_config(self._h, ctypes.byref(leaf), ctypes.byref(block)))
        return leaf.value, block.value

    def run(self, points, nneigh, lst, stream=None):
        _check(self._L.nbr_batch_run(self._h, _ptr(points), _ptr(nneigh), _ptr(lst), _stream_ptr(stream)))

    def tune(self, points, nneigh, lst, stream=None):
        leaf, block = ctypes.c_uint(), ctypes.c_uint()
        _check(self._L.nbr_batch_tune(self._h, _ptr(points), _ptr(nneigh), _ptr(lst), _stream_ptr(stream),
                                      ctypes.byref(leaf), ctypes.byref(block)))
        return leaf.value, block.value

    def capture(self, points, nneigh, lst, stream):
        _check(self._L.nbr_batch_capture(self._h, _ptr(points), _ptr(nneigh), _ptr(lst), _stream_ptr(stream)))

    def replay(self, stream):
        _check(self._L.nbr_batch_replay(self._h, _stream_ptr(stream)))

    def status(self, stream=None):
        bits, largest = ctypes.c_uint(), ctypes.c_uint()
        _check(self._L.nbr_batch_status(self._h, ctypes.byref(bits), ctypes.byref(largest), _stream_ptr(stream)))
        return bits.value, largest.value

    def sequential_plain(self, lbvh: "LBVH", trav: "LBVHTraverser", points, rc: float, nneigh, lst,
                         block_size: int = 256, stream=None):
        """The same lists by one plain two-pass call per system (build, count, max, fill); list
        entries are system-local primitive ids."""
        _check(self._L.nbr_batch_sequential_plain(lbvh.handle, trav._h, _ptr(points),
                                                  self._start.ctypes.data_as(ctypes.c_void_p),
                                                  self._boxes.ctypes.data_as(ctypes.c_void_p), self.S,
                                                  float(rc), _ptr(nneigh), _ptr(lst), self.max_neigh,
                                                  block_size, _stream_ptr(stream)))
