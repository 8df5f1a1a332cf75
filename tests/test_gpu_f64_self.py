"""Double-precision self queries (traverse_self_f64, nbr_traverse_self_f64).

Every point of a tree of double points queries the tree with one cutoff.  Counts of more than the
symmetric minimum of points with the self image or the 27 periodic images take the symmetric
double walk with the pair exchange (k_traverse_half_f64), and the following fill assembles the
rows from it; image lists and forced routes walk the whole tree per query.  Every route must give
the counts and rows -- entries and their order -- of traverse_f64 over the same points given as
spheres in the tree's sorted order (ExactSphereQueryOpF64, the route that stands for the
reference's traverse with an exact double query), and the float64 brute force on pairs placed
within 1e-12 of the cutoff.
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


def _uniform(n, seed, density=0.85):
    rng = np.random.default_rng(seed)
    L = float((n / density) ** (1.0 / 3.0))
    return rng.random((n, 3)) * L, L, rng


def _images(kind, L):
    if kind == "periodic":
        return "periodic", [L, L, L]
    if kind == "list":
        return nb.images27([L, L, L]), [L, L, L]
    return None, [0.0, 0.0, 0.0]


def _expected(lbvh, P, rc, box, pad, imgs, perm, max_neigh):
    """traverse_f64 over the spheres (P[primitive[s]], rc): counts and rows by sorted slot."""
    prims = lbvh.primitives().cpu().numpy().view(np.uint32).astype(np.int64)
    sph = torch.tensor(np.concatenate([P[prims], np.full((len(P), 1), rc)], 1), device="cuda")
    # traverse_f64 reads positions by the reported id (the mapped id when a map is given)
    Pr = np.empty_like(P)
    if perm is not None:
        Pr[perm] = P
    else:
        Pr = P
    trav = nb.LBVHTraverser()
    m = None if perm is None else torch.tensor(perm, device="cuda")
    cnt = trav.traverse_f64(lbvh, sph, torch.tensor(Pr, device="cuda"), box, pad, images=imgs, map=m)
    c = cnt.cpu().numpy().view(np.uint32).copy()
    mx = max(int(c.max()), 1) if max_neigh is None else max_neigh
    _, lst = trav.traverse_f64(lbvh, sph, torch.tensor(Pr, device="cuda"), box, pad, images=imgs, map=m,
                               max_neigh=mx)
    return c, lst.cpu().numpy().view(np.uint32), prims


def _self(trav, lbvh, pts, rc, box, pad, imgs, perm, rows_sorted, max_neigh=None, read_summary=False):
    m = None if perm is None else torch.tensor(perm, device="cuda")
    cnt = trav.traverse_self_f64(lbvh, pts, rc, box, pad, images=imgs, map=m, rows_sorted=rows_sorted)
    c = cnt.cpu().numpy().view(np.uint32).copy()
    if read_summary:
        mx, total, _ = trav.count_summary()
        assert mx == int(c.max()) and total == int(c.sum())
    mx = max(int(c.max()), 1) if max_neigh is None else max_neigh
    c2, lst = trav.traverse_self_f64(lbvh, pts, rc, box, pad, images=imgs, map=m, rows_sorted=rows_sorted,
                                     max_neigh=mx)
    assert np.array_equal(c2.cpu().numpy().view(np.uint32), c)
    return c, lst.cpu().numpy().view(np.uint32)


def _compare(c_self, l_self, c_want, l_want, prims, rows_sorted):
    """Rows of the self call (by sorted slot, or by primitive id) against traverse_f64's rows."""
    if rows_sorted:
        cs, ls = c_self, l_self
    else:
        cs, ls = c_self[prims], l_self[prims]
    assert np.array_equal(cs, c_want)
    k = min(ls.shape[1], l_want.shape[1])
    valid = np.arange(k)[None, :] < np.minimum(c_want, k)[:, None]
    assert np.array_equal(np.where(valid, ls[:, :k], 0), np.where(valid, l_want[:, :k], 0))


@pytest.mark.parametrize("images", ["periodic", "list", None])
@pytest.mark.parametrize("mapped", [False, True])
@pytest.mark.parametrize("rows_sorted", [True, False])
def test_self_f64_equals_traverse_f64(images, mapped, rows_sorted):
    # 60,000 points: above the symmetric minimum, so the self image and the lattice take the
    # symmetric walk with the exchange and the fill assembles; the image list walks whole
    N, rc = 60000, 1.3
    P, L, rng = _uniform(N, 101 + 2 * mapped + (images is None), 0.85)
    imgs, box = _images(images, L)
    pad = nb.exact_pad(rc, 2 * L)
    pts = torch.tensor(P, device="cuda")
    lbvh = nb.LBVH()
    lbvh.build_f64(pts, [0, 0, 0], [L, L, L])
    perm = rng.permutation(N).astype(np.int32) if mapped else None
    c_want, l_want, prims = _expected(lbvh, P, rc, box, pad, imgs, perm, None)
    trav = nb.LBVHTraverser()
    c, lst = _self(trav, lbvh, pts, rc, box, pad, imgs, perm, rows_sorted, max_neigh=l_want.shape[1])
    _compare(c, lst, c_want, l_want, prims, rows_sorted)


@pytest.mark.parametrize("route", ["symmetric_off", "exchange_off", "below_minimum", "summary_read"])
def test_self_f64_routes(route):
    # the same rows on every route: whole-tree walks (symmetric off, or fewer points than the
    # symmetric minimum), the exchange off (the fill walks whole), and the exchange with the
    # summary read between count and fill (the two-pass pattern)
    N, rc = 40000, 1.3
    P, L, _ = _uniform(N, 7, 0.85)
    box = [L, L, L]
    pad = nb.exact_pad(rc, 2 * L)
    pts = torch.tensor(P, device="cuda")
    lbvh = nb.LBVH()
    lbvh.build_f64(pts, [0, 0, 0], box)
    c_want, l_want, prims = _expected(lbvh, P, rc, box, pad, "periodic", None, None)
    trav = nb.LBVHTraverser()
    if route == "symmetric_off":
        trav.set_symmetric(False)
    elif route == "exchange_off":
        trav.set_pair_cache(False)
    elif route == "below_minimum":
        trav.set_symmetric_min_points(N + 1)
    c, lst = _self(trav, lbvh, pts, rc, box, pad, "periodic", None, True, max_neigh=l_want.shape[1],
                   read_summary=(route == "summary_read"))
    _compare(c, lst, c_want, l_want, prims, True)


def test_self_f64_rows_past_the_exchange():
    # a cutoff of 2.6 at density 0.85 gives about 63 neighbors per point: nearly every row is
    # past the exchange's 16 + 16 slots and is walked whole after the assembly; then a clustered
    # set mixes rows assembled from the exchange with re-walked ones
    N = 30000
    for rc, clustered in ((2.6, False), (1.3, True)):
        P, L, rng = _uniform(N, 55, 0.85)
        if clustered:
            centres = rng.random((40, 3)) * L
            k = N // 2
            P[:k] = np.mod(centres[rng.integers(0, 40, k)] + rng.normal(scale=0.9, size=(k, 3)), L)
        box = [L, L, L]
        pad = nb.exact_pad(rc, 2 * L)
        pts = torch.tensor(P, device="cuda")
        lbvh = nb.LBVH()
        lbvh.build_f64(pts, [0, 0, 0], box)
        c_want, l_want, prims = _expected(lbvh, P, rc, box, pad, "periodic", None, None)
        trav = nb.LBVHTraverser()
        c, lst = _self(trav, lbvh, pts, rc, box, pad, "periodic", None, True, max_neigh=l_want.shape[1])
        _compare(c, lst, c_want, l_want, prims, True)
        assert int(c.max()) > 32


def _brute(P, rc, L):
    counts, rows = [], []
    for i in range(len(P)):
        d = P - P[i]
        h = 0.5 * L
        d = np.where(d >= h, d - L, np.where(d < -h, d + L, d))
        d2 = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]
        nbr = np.nonzero(d2 <= rc * rc)[0]
        counts.append(len(nbr))
        rows.append(nbr)
    return np.asarray(counts, np.uint32), rows


def test_self_f64_near_cutoff_pairs():
    # pairs placed at relative offsets of 1e-12 .. 1e-3 either side of the cutoff along random
    # directions, some across the periodic boundary, in a set large enough for the symmetric walk:
    # the FP32 screen decides the clear pairs, the double predicate the band, on both rows of a pair
    rng = np.random.default_rng(43)
    N, rc = 20000, 1.3
    L = float((N / 0.85) ** (1.0 / 3.0))
    P = rng.random((N, 3)) * L
    offsets = [1e-12, 1e-9, 1e-6, 3e-6, 1e-5, 3e-5, 1e-4, 1e-3]
    k = 0
    for off in offsets:
        for sign in (-1.0, 1.0):
            for rep in range(6):
                i = 2 * k
                u = rng.normal(size=3)
                u /= np.linalg.norm(u)
                base = rng.random(3) * L
                if rep % 3 == 0:
                    base[0] = L - 0.3   # the partner lies across the periodic boundary
                    u[0] = abs(u[0]) + 0.5
                    u /= np.linalg.norm(u)
                P[i] = base
                P[i + 1] = np.mod(base + u * rc * (1.0 + sign * off), L)
                k += 1
    box = [L, L, L]
    pad = nb.exact_pad(rc, 2 * L)
    pts = torch.tensor(P, device="cuda")
    lbvh = nb.LBVH()
    lbvh.build_f64(pts, [0, 0, 0], box)
    want_c, want_rows = _brute(P, rc, L)
    trav = nb.LBVHTraverser()
    c, lst = _self(trav, lbvh, pts, rc, box, pad, "periodic", None, False, max_neigh=int(want_c.max()))
    assert np.array_equal(c, want_c)
    for i in range(N):
        assert np.array_equal(np.sort(lst[i, : c[i]]), want_rows[i]), i


def _round_f32(x, up):
    """float64 -> float32 rounded toward +inf (up) or -inf, elementwise."""
    f = x.astype(np.float32)
    back = f.astype(np.float64)
    if up:
        return np.where(back < x, np.nextafter(f, np.float32(np.inf)), f)
    return np.where(back > x, np.nextafter(f, np.float32(-np.inf)), f)


def test_double_tree_reference_layout_boxes():
    # a double point tree forms its reference-layout boxes on first access from the payload (the
    # point rounded down) and the upper-corner bits: leaf boxes must be the points rounded outward
    # to FP32 -- with coordinates that are floats (multiples of 1/8) and ones that are not -- and
    # every internal box the union of its children's
    rng = np.random.default_rng(61)
    N = 5000
    L = 20.0
    P = rng.random((N, 3)) * L
    exact = rng.random((N, 3)) < 0.4
    P = np.where(exact, np.round(P * 8.0) / 8.0, P)
    lbvh = nb.LBVH()
    lbvh.build_f64(torch.tensor(P, device="cuda"), [0, 0, 0], [L, L, L])
    arr = {k: v.cpu().numpy() for k, v in lbvh.arrays().items()}
    ni = N - 1
    prim = arr["primitive"].view(np.uint32).astype(np.int64)
    lo_leaf, hi_leaf = arr["lo"][ni:], arr["hi"][ni:]
    assert np.array_equal(lo_leaf, _round_f32(P[prim], False))
    assert np.array_equal(hi_leaf, _round_f32(P[prim], True))
    assert np.array_equal(hi_leaf == lo_leaf, exact[prim] | (P[prim] == P[prim].astype(np.float32)))
    left, right = arr["left"], arr["right"]
    assert np.array_equal(arr["lo"][:ni], np.minimum(arr["lo"][left], arr["lo"][right]))
    assert np.array_equal(arr["hi"][:ni], np.maximum(arr["hi"][left], arr["hi"][right]))


@pytest.mark.parametrize("N", [1, 2, 37, 5000])
def test_self_f64_small_sets(N):
    # tiny trees (one point, two, a few dozen: the whole-tree walk) and a set just above the
    # symmetric minimum: the same counts and rows as traverse_f64 over the sorted points
    rc = 1.3
    P, L, _ = _uniform(N, 900 + N, 0.85)
    L = max(L, 3.0)
    box = [L, L, L]
    pad = nb.exact_pad(rc, 2 * L)
    pts = torch.tensor(P, device="cuda")
    lbvh = nb.LBVH()
    lbvh.build_f64(pts, [0, 0, 0], box)
    c_want, l_want, prims = _expected(lbvh, P, rc, box, pad, "periodic", None, None)
    trav = nb.LBVHTraverser()
    c, lst = _self(trav, lbvh, pts, rc, box, pad, "periodic", None, True, max_neigh=l_want.shape[1])
    _compare(c, lst, c_want, l_want, prims, True)
