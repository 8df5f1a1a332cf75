"""CPU-side checks of the C-ABI library: it builds for sm_103a, loads, and exports every symbol
declared in include/neighbor_gb300.h.  No compute call is made (there may be no GPU)."""
import ctypes
import os
import re

import pytest

import neighbor_gb300 as nb

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    with open(os.path.join(ROOT, "include", "neighbor_gb300.h")) as f:
        text = f.read()
    return sorted(set(re.findall(r"\b(nbr_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    nb.build()
    return ctypes.CDLL(nb.library_path())


def test_library_exports_every_declared_symbol(lib):
    declared = _declared()
    assert declared, "no declarations found"
    missing = [s for s in declared if not hasattr(lib, s)]
    assert not missing, missing
    assert sorted(nb.EXPORTED) == declared


def test_python_mirror_declares_signatures():
    L = nb.load()
    for s in nb.EXPORTED:
        assert getattr(L, s).argtypes is not None


def test_exact_pad_matches_oracle():
    import oracle as O
    for rc, cm in [(1.3, 270.25), (1.0, 20.0), (5.9, 173.6), (0.5, 1e-3)]:
        assert nb.exact_pad(rc, cm) == pytest.approx(O.exact_pad(rc, cm), rel=0, abs=0)


def test_errors_do_not_cross_the_abi(lib):
    L = nb.load()
    rc = L.nbr_lbvh_set_leaf_size(None, 4)
    assert rc == 1 and b"null" in L.nbr_last_error()
    h = ctypes.c_void_p()
    assert L.nbr_lbvh_create(ctypes.byref(h)) == 0
    assert L.nbr_lbvh_set_leaf_size(h, 0) == 1
    assert b"Leaf size" in L.nbr_last_error()
    assert L.nbr_lbvh_set_radix_bits(h, 7) == 1
    lo = (ctypes.c_float * 3)(0, 0, 0)
    # invalid tunable is rejected before any device work (reference: Tunable.h:110-118)
    assert L.nbr_lbvh_build_points(h, ctypes.c_void_p(8), 10, lo, lo, 33, None) == 1
    assert L.nbr_lbvh_destroy(h) == 0


def test_product_rejects_host_tensors():
    # the product has no CPU path: a host tensor is refused before any library call
    torch = pytest.importorskip("torch")
    lbvh = nb.LBVH()
    with pytest.raises(TypeError):
        lbvh.build(torch.zeros((10, 3)), [0, 0, 0], [1, 1, 1])
    with pytest.raises(TypeError):
        nb.CapacityModel.targets(torch.zeros(4, dtype=torch.int32))
