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


def _build_arrays(pts, L):
    lbvh = nb.LBVH()
    lbvh.build(pts, [0, 0, 0], [L, L, L])
    lbvh.check_status()
    return lbvh.codes().cpu(), lbvh.primitives().clone().cpu()


@pytest.mark.parametrize("n", [1, 4095])
def test_noalloc_sort_small_sizes_on_a_user_stream(n):
    # N = 1 and N below one 4096-key sort tile, on a non-default stream; the expected arrays are
    # the oracle's codes and their stable order (a one-point build sorts nothing)
    import oracle as O
    L = 9.0
    pts = _points(n, 5 + n, L)
    codes_np = O.morton_codes(pts.cpu().numpy(), [0, 0, 0], [L, L, L])
    order_np = np.argsort(codes_np, kind="stable").astype(np.uint32)
    want_codes = torch.from_numpy(codes_np[order_np].view(np.int32))
    want_order = torch.from_numpy(order_np.view(np.int32))
    side = torch.cuda.Stream()
    codes = torch.empty(n, dtype=torch.int32, device="cuda")
    order = torch.empty(n, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    with torch.cuda.stream(side):
        nb.morton_sort_noalloc(pts, [0, 0, 0], [L, L, L], codes, order, stream=side)
        assert nb.morton_sort_noalloc_status(stream=side) == 0
    side.synchronize()
    assert torch.equal(codes.cpu(), want_codes.view(torch.int32))
    assert torch.equal(order.cpu(), want_order.view(torch.int32))


def test_noalloc_sort_two_streams_ordered_by_an_event():
    # the calls share the array: two calls on two streams, the second ordered after the first by
    # an event (the serialisation the array requires), each equal to its build
    out = []
    streams = [torch.cuda.Stream(), torch.cuda.Stream()]
    done = torch.cuda.Event()
    cases = [(200_000, 21, 50.0), (70_001, 22, 30.0)]
    inputs = [(_points(n, seed, L), L) for n, seed, L in cases]
    torch.cuda.synchronize()
    for k, ((pts, L), st) in enumerate(zip(inputs, streams)):
        n = pts.shape[0]
        codes = torch.empty(n, dtype=torch.int32, device="cuda")
        order = torch.empty(n, dtype=torch.int32, device="cuda")
        with torch.cuda.stream(st):
            if k == 1:
                st.wait_event(done)
            nb.morton_sort_noalloc(pts, [0, 0, 0], [L, L, L], codes, order, stream=st)
            if k == 0:
                # copy the first result out before the second call reuses the array
                out.append((codes.clone(), order.clone()))
                done.record(st)
            else:
                out.append((codes, order))
    torch.cuda.synchronize()
    for (pts, L), (codes, order) in zip(inputs, out):
        want_codes, want_order = _build_arrays(pts, L)
        assert torch.equal(codes.cpu(), want_codes.view(torch.int32))
        assert torch.equal(order.cpu(), want_order.view(torch.int32))


def test_noalloc_sort_reports_a_wait_that_gave_up():
    # the test hook never runs the first sort tile: the next tile's bounded look-back gives up,
    # the status says so, and the array and the context stay usable for a correct call after it
    n, L = 50_000, 30.0
    pts = _points(n, 31, L)
    codes = torch.empty(n, dtype=torch.int32, device="cuda")
    order = torch.empty(n, dtype=torch.int32, device="cuda")
    nb.debug_noalloc_wait_timeout(pts, [0, 0, 0], [L, L, L], codes, order)
    with pytest.raises(nb.NeighborError, match="gave up"):
        nb.morton_sort_noalloc_status()
    nb.morton_sort_noalloc(pts, [0, 0, 0], [L, L, L], codes, order)
    assert nb.morton_sort_noalloc_status() == 0
    want_codes, want_order = _build_arrays(pts, L)
    assert torch.equal(codes.cpu(), want_codes.view(torch.int32))
    assert torch.equal(order.cpu(), want_order.view(torch.int32))


def test_noalloc_sort_rejects_host_memory():
    n = 100
    pts = torch.zeros((n, 3), dtype=torch.float32, device="cuda")
    codes = torch.empty(n, dtype=torch.int32, device="cuda")
    host = torch.empty(n, dtype=torch.int32).pin_memory()
    lib = nb.load()
    import ctypes
    lo = (ctypes.c_float * 3)(0, 0, 0)
    hi = (ctypes.c_float * 3)(1, 1, 1)
    rc = lib.nbr_morton_sort_noalloc(pts.data_ptr(), n, lo, hi, codes.data_ptr(), host.data_ptr(), None)
    assert rc == 1 and b"current device" in lib.nbr_last_error()


def test_noalloc_sort_rejects_oversize_without_work():
    n = nb.NOALLOC_MAX_POINTS + 1
    pts = torch.zeros((n, 3), dtype=torch.float32, device="cuda")
    out = torch.empty(n, dtype=torch.int32, device="cuda")
    with pytest.raises(nb.NeighborError, match="exceed its fixed scratch"):
        nb.morton_sort_noalloc(pts, [0, 0, 0], [1, 1, 1], out, out.clone())
