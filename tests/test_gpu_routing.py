"""Routing by size: every traversal kernel gives the same counts and the same rows, in order.

Small traversals walk one group of 4, 8, 16 or 32 lanes per query (LBVHTraverser::setWalkLanes,
chosen by size by default), middle-sized self traversals one thread per query over the whole tree,
large ones the symmetric walk.  Each route is forced here on the same trees, and its counts and
every list row (stride and CSR, with and without a map transform) must equal those of the
one-thread walk; the counts of the larger trees must equal the oracle's cell list.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

import neighbor_gb300 as nb  # noqa: E402
import oracle as O  # noqa: E402

ROUTES = ["thread", "symmetric", "g4", "g8", "g16", "g32"]


@pytest.fixture(scope="module", autouse=True)
def _lib():
    nb.build()
    nb.load()


def _t(a, dtype=torch.float32):
    return torch.tensor(np.asarray(a), dtype=dtype, device="cuda")


def _points(N, seed, clustered=False):
    rng = np.random.default_rng(seed)
    L = float((max(N, 1) / 0.85) ** (1.0 / 3.0))
    P = rng.random((N, 3)) * L
    if clustered and N > 10:
        c = rng.random((max(1, N // 300), 3)) * L
        k = rng.integers(0, len(c), N // 2)
        P[: N // 2] = c[k] + rng.normal(size=(N // 2, 3)) * 0.8
        P = np.mod(P, L)
    return P.astype(np.float32), L


def _traverser(route, N):
    trav = nb.LBVHTraverser()
    if route == "thread":
        trav.set_symmetric(False)
        trav.set_warp_walk_max(0)
    elif route == "symmetric":
        trav.force_symmetric()
    else:
        trav.set_symmetric(False)
        trav.set_warp_walk_max(max(N, 1))
        trav.set_walk_lanes(int(route[1:]))
    return trav


def _rows(cnt, lst):
    cnt = cnt.cpu().numpy().view(np.uint32)
    lst = lst.cpu().numpy().view(np.uint32)
    mask = np.arange(lst.shape[1])[None, :] < cnt[:, None]
    return cnt, np.where(mask, lst, 0xFFFFFFFF)


@pytest.mark.parametrize("images", ["periodic", "self"])
@pytest.mark.parametrize("N,clustered", [(1, False), (37, False), (3000, False), (3000, True), (40000, False)])
def test_routes_give_identical_rows(N, clustered, images):
    P, L = _points(N, 100 + N, clustered)
    rc = 1.3
    box = [L, L, L] if images == "periodic" else [0, 0, 0]
    imgs = "periodic" if images == "periodic" else None
    lbvh = nb.LBVH()
    lbvh.build(_t(P), [0, 0, 0], [L, L, L])
    pad = nb.exact_pad(rc, 2 * L)
    m = _t(np.random.default_rng(N).permutation(N).astype(np.int32), torch.int32)
    out = {}
    for route in ROUTES:
        trav = _traverser(route, N)
        cnt = trav.traverse_self(lbvh, rc, box, pad, images=imgs, rows_sorted=False)
        mx = max(1, int(cnt.max().item()))
        if route == "symmetric":
            mx = min(mx, 32)   # the symmetric fill orders rows of up to 32 entries
        c, lst = _rows(*trav.traverse_self(lbvh, rc, box, pad, images=imgs, rows_sorted=False, max_neigh=mx,
                                           map=m))
        out[route] = (cnt.cpu().numpy().view(np.uint32), c, lst, mx)
    c0, _, l0, mx0 = out["thread"]
    for route, (cnt, c, lst, mx) in out.items():
        assert np.array_equal(cnt, c0), route
        assert np.array_equal(c, c0), route
        if mx == mx0:
            assert np.array_equal(lst, l0), route
    if N >= 3000:
        want, _ = O.celllist_counts(P, P, rc, [0, 0, 0], box)
        assert np.array_equal(c0, want)


@pytest.mark.parametrize("lanes", [4, 8, 16, 32])
def test_lane_groups_csr_and_general_queries(lanes):
    P, L = _points(6000, 7, clustered=True)
    rc = 1.3
    box = [L, L, L]
    lbvh = nb.LBVH()
    lbvh.build(_t(P), [0, 0, 0], box)
    pad = nb.exact_pad(rc, 2 * L)
    ref = _traverser("thread", len(P))
    grp = _traverser(f"g{lanes}", len(P))
    # CSR rows (every row its exact count)
    cnt = ref.traverse_self(lbvh, rc, box, pad, images="periodic", rows_sorted=True)
    op = nb.OnePassList()
    offsets, total = op.scan(cnt)
    lists = []
    for trav in (ref, grp):
        lst = torch.full((total + 1,), -1, dtype=torch.int32, device="cuda")
        nn = trav.traverse_self_csr(lbvh, rc, box, pad, offsets, cnt, lst, max_capacity=int(cnt.max().item()),
                                    images="periodic", rows_sorted=True)
        assert torch.equal(nn, cnt)
        lists.append(lst.cpu().numpy())
    assert np.array_equal(lists[0], lists[1])
    # general sphere queries (query points other than the tree's), exact predicate
    rng = np.random.default_rng(8)
    Qp = (rng.random((5000, 3)) * L).astype(np.float32)
    sph = _t(np.concatenate([Qp, np.full((len(Qp), 1), rc, np.float32)], 1))
    res = []
    for trav in (ref, grp):
        trav.set_warp_walk_max(0 if trav is ref else len(Qp))
        c = trav.traverse(lbvh, sph, query=nb.QUERY_EXACT, points=_t(P), box=box, pad=pad, images="periodic")
        mx = max(1, int(c.max().item()))
        res.append(_rows(*trav.traverse(lbvh, sph, query=nb.QUERY_EXACT, points=_t(P), box=box, pad=pad,
                                        images="periodic", max_neigh=mx)))
    assert np.array_equal(res[0][0], res[1][0])
    assert np.array_equal(res[0][1], res[1][1])
    want, _ = O.celllist_counts(Qp, P, rc, [0, 0, 0], box)
    assert np.array_equal(res[0][0], want)


def test_walk_lanes_rejects_other_widths():
    trav = nb.LBVHTraverser()
    with pytest.raises(nb.NeighborError):
        trav.set_walk_lanes(5)
    trav.set_walk_lanes(0)


@pytest.mark.parametrize("N,clustered,rc", [(3000, True, 1.3), (40000, False, 1.3), (20000, False, 2.6),
                                            (70000, True, 1.3)])
def test_half_walk_lane_groups_give_identical_rows(N, clustered, rc):
    # the exchanging symmetric count with one thread per query and with lane groups of every width:
    # the same counts, the same rows in order (assembled from the exchange, or re-walked past it --
    # the clustered sets and the cutoff of 2.6 put many rows there), and the oracle's counts
    P, L = _points(N, 300 + N, clustered)
    box = [L, L, L]
    lbvh = nb.LBVH()
    lbvh.build(_t(P), [0, 0, 0], box)
    pad = nb.exact_pad(rc, 2 * L)
    out = {}
    for lanes in (1, 4, 8, 16, 32):
        trav = nb.LBVHTraverser()
        trav.force_symmetric()
        trav.set_half_walk_lanes(lanes)
        cnt = trav.traverse_self(lbvh, rc, box, pad, images="periodic", rows_sorted=True)
        c_host = cnt.cpu().numpy().view(np.uint32).copy()
        mx = max(1, int(c_host.max()))
        c, lst = _rows(*trav.traverse_self(lbvh, rc, box, pad, images="periodic", rows_sorted=True, max_neigh=mx))
        out[lanes] = (c_host, c, lst)
    c0, _, l0 = out[1]
    for lanes, (cnt, c, lst) in out.items():
        assert np.array_equal(cnt, c0), lanes
        assert np.array_equal(c, c0), lanes
        assert np.array_equal(lst, l0), lanes
    # rows by sorted slot: the oracle's counts in the tree's order
    want, _ = O.celllist_counts(P, P, rc, [0, 0, 0], box)
    prim = lbvh.primitives().cpu().numpy().view(np.uint32).astype(np.int64)
    assert np.array_equal(c0, want[prim])


def test_half_walk_lanes_rejects_other_widths():
    trav = nb.LBVHTraverser()
    with pytest.raises(nb.NeighborError):
        trav.set_half_walk_lanes(2)
    trav.set_half_walk_lanes(0)
