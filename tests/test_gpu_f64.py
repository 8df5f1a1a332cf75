"""Double-precision inputs: trees of double points and exact double sphere queries.

Positions given in double (as HOOMD-blue built with Scalar = double gives them) are inserted as
boxes rounded outward to FP32, and the query refines with the double minimum-image predicate.
The neighbor sets must equal a float64 brute force with the same operation order, including pairs
placed within 1e-12 of the cutoff, where an FP32 predicate would decide differently.
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


def _brute(P, rc, L):
    counts, rows = [], []
    for i in range(len(P)):
        d = P - P[i]
        if L > 0:
            h = 0.5 * L
            d = np.where(d >= h, d - L, np.where(d < -h, d + L, d))
        d2 = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]
        nbr = np.nonzero(d2 <= rc * rc)[0]
        counts.append(len(nbr))
        rows.append(nbr)
    return np.asarray(counts, np.uint32), rows


@pytest.mark.parametrize("periodic", [True, False])
def test_double_points_exact_sets(periodic):
    rng = np.random.default_rng(21)
    N = 3000
    rc = 1.3
    L = float((N / 0.85) ** (1.0 / 3.0))
    P = rng.random((N, 3)) * L
    # pairs straddling the cutoff by 1e-12 along x (inside the box, away from its faces)
    for k in range(40):
        i = 2 * k
        P[i] = [L / 2 + 0.01 * k, L / 3, L / 4]
        P[i + 1] = P[i] + np.array([rc * (1 + (1e-12 if k % 2 else -1e-12)), 0.0, 0.0])
    lbvh = nb.LBVH()
    lbvh.build_f64(torch.tensor(P, device="cuda"), [0, 0, 0], [L, L, L])
    box = [L, L, L] if periodic else [0.0, 0.0, 0.0]
    sph = torch.tensor(np.concatenate([P, np.full((N, 1), rc)], 1), device="cuda")
    pts = torch.tensor(P, device="cuda")
    pad = nb.exact_pad(rc, 2 * L)
    imgs = "periodic" if periodic else None
    trav = nb.LBVHTraverser()
    cnt = trav.traverse_f64(lbvh, sph, pts, box, pad, images=imgs)
    want_c, want_rows = _brute(P, rc, L if periodic else 0.0)
    got_c = cnt.cpu().numpy().view(np.uint32)
    assert np.array_equal(got_c, want_c)
    cnt2, lst = trav.traverse_f64(lbvh, sph, pts, box, pad, images=imgs, max_neigh=int(want_c.max()))
    lst = lst.cpu().numpy().view(np.uint32)
    for i in range(N):
        assert np.array_equal(np.sort(lst[i, : got_c[i]]), want_rows[i]), i
    # the near-cutoff pairs: inside for even k (rc (1 - 1e-12)), outside for odd k (rc (1 + 1e-12))
    for k in range(40):
        i = 2 * k
        assert ((i + 1) in set(lst[i, : got_c[i]].tolist())) == (k % 2 == 0)


def _routes(lbvh, sph, pts, box, pad, imgs, map_=None, max_neigh=None):
    """(counts, lists) of the double-precision fast walk and of the reference-layout walk."""
    out = []
    for fast in (True, False):
        trav = nb.LBVHTraverser()
        trav.set_fast_path(fast)
        if max_neigh is None:
            out.append((trav.traverse_f64(lbvh, sph, pts, box, pad, images=imgs, map=map_).cpu().numpy(), None))
        else:
            c, lst = trav.traverse_f64(lbvh, sph, pts, box, pad, images=imgs, map=map_, max_neigh=max_neigh,
                                       block_size=256)
            out.append((c.cpu().numpy(), lst.cpu().numpy()))
    return out


@pytest.mark.parametrize("images", ["periodic", "list", None])
@pytest.mark.parametrize("mapped", [False, True])
def test_fast_double_walk_equals_reference_layout_walk(images, mapped):
    # k_traverse_fast_f64 (the route for ExactSphereQueryOpF64 on a tree of double points) and the
    # reference-layout rope walk of the same op: equal counts and every row equal in order
    rng = np.random.default_rng(31 + (images is None) + 2 * mapped)
    N = 60000
    rc = 1.3
    L = float((N / 0.85) ** (1.0 / 3.0))
    P = rng.random((N, 3)) * L
    lbvh = nb.LBVH()
    lbvh.build_f64(torch.tensor(P, device="cuda"), [0, 0, 0], [L, L, L])
    periodic = images is not None
    box = [L, L, L] if periodic else [0.0, 0.0, 0.0]
    if images == "list":
        imgs = nb.images27([L, L, L])
    else:
        imgs = images
    perm = rng.permutation(N).astype(np.int32)
    map_ = torch.tensor(perm, device="cuda") if mapped else None
    # points indexed by the reported id (the mapped id when a map is given)
    Pr = np.empty_like(P)
    if mapped:
        Pr[perm] = P
    else:
        Pr = P
    sph = torch.tensor(np.concatenate([P, np.full((N, 1), rc)], 1), device="cuda")
    pts = torch.tensor(Pr, device="cuda")
    pad = nb.exact_pad(rc, 2 * L)
    (cf, _), (cr, _) = _routes(lbvh, sph, pts, box, pad, imgs, map_)
    assert np.array_equal(cf, cr)
    mx = int(cf.max())
    (cf, lf), (cr, lr) = _routes(lbvh, sph, pts, box, pad, imgs, map_, max_neigh=mx)
    assert np.array_equal(cf, cr)
    valid = np.arange(mx)[None, :] < cf[:, None]
    assert np.array_equal(np.where(valid, lf, 0), np.where(valid, lr, 0))


def test_fast_double_walk_near_cutoff_pairs():
    # lists of the double walk against the float64 brute force, with pairs placed at relative
    # offsets of 1e-12 .. 1e-3 either side of the cutoff along random directions, some across the
    # periodic boundary: the FP32 screen decides the clear ones, the double predicate the band
    rng = np.random.default_rng(41)
    N = 8000
    rc = 1.3
    L = float((N / 0.85) ** (1.0 / 3.0))
    P = rng.random((N, 3)) * L
    offsets = [1e-12, 1e-9, 1e-6, 3e-6, 1e-5, 3e-5, 1e-4, 1e-3]
    want_in = []
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
                want_in.append((i, sign < 0, off))
                k += 1
    lbvh = nb.LBVH()
    lbvh.build_f64(torch.tensor(P, device="cuda"), [0, 0, 0], [L, L, L])
    sph = torch.tensor(np.concatenate([P, np.full((N, 1), rc)], 1), device="cuda")
    pts = torch.tensor(P, device="cuda")
    pad = nb.exact_pad(rc, 2 * L)
    trav = nb.LBVHTraverser()
    want_c, want_rows = _brute(P, rc, L)
    cnt, lst = trav.traverse_f64(lbvh, sph, pts, [L, L, L], pad, images="periodic", max_neigh=int(want_c.max()),
                                 block_size=256)
    c = cnt.cpu().numpy().view(np.uint32)
    assert np.array_equal(c, want_c)
    lst = lst.cpu().numpy().view(np.uint32)
    for i in range(N):
        assert np.array_equal(np.sort(lst[i, : c[i]]), want_rows[i]), i
    # the planted pairs fall on the intended side (beyond the float64 rounding of the placement)
    # and the walk reports exactly the brute force's decision for each
    for i, inside, off in want_in:
        brute = (i + 1) in set(want_rows[i].tolist())
        if off >= 1e-9:
            assert brute == inside, (i, off)
        assert brute == ((i + 1) in set(lst[i, : c[i]].tolist())), (i, off)
