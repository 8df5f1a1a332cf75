"""The allocation-free Morton sort gives the same arrays as the LBVH build.

nbr_morton_sort_noalloc exists for callers that cannot allocate device memory (a framework that
owns every allocation, a loop that must not touch the allocator, a committed memory budget): it
runs the build's Morton-code and stable-sort stage entirely in one fixed device array.  Its
output must equal, bit for bit, the sorted codes and the primitive order that
nbr_lbvh_build_points produces for the same points -- here on two calls in a row (the second one
reuses the array the first one left behind), one of them at the maximum size.

This file is named so that pytest collects it last.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

import neighbor_gb300 as nb  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _lib():
    nb.build()
    nb.load()


def _points(n, seed, L):
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    return torch.rand((n, 3), generator=g, device="cuda", dtype=torch.float32) * L


def test_noalloc_sort_matches_build_on_two_calls():
    cases = [(300_001, 1, 40.0), (nb.NOALLOC_MAX_POINTS, 2, 107.0)]
    for n, seed, L in cases:
        pts = _points(n, seed, L)
        codes = torch.empty(n, dtype=torch.int32, device="cuda")
        order = torch.empty(n, dtype=torch.int32, device="cuda")
        nb.morton_sort_noalloc(pts, [0, 0, 0], [L, L, L], codes, order)
        lbvh = nb.LBVH()
        lbvh.build(pts, [0, 0, 0], [L, L, L])
        lbvh.check_status()
        want_codes = lbvh.codes()
        want_order = lbvh.primitives().clone()
        torch.cuda.synchronize()
        assert torch.equal(codes.cpu().view(torch.int32), want_codes.cpu().view(torch.int32)), n
        assert torch.equal(order.cpu().view(torch.int32), want_order.cpu().view(torch.int32)), n


def test_noalloc_sort_rejects_oversize_without_work():
    n = nb.NOALLOC_MAX_POINTS + 1
    pts = torch.zeros((n, 3), dtype=torch.float32, device="cuda")
    out = torch.empty(n, dtype=torch.int32, device="cuda")
    with pytest.raises(nb.NeighborError, match="exceed its fixed scratch"):
        nb.morton_sort_noalloc(pts, [0, 0, 0], [1, 1, 1], out, out.clone())
