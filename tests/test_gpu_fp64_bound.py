"""The GPU's FP32 neighbor decisions against an FP64 brute force.

The library decides every pair with the FP32 minimum-image predicate (the reference validation
test's, test/lbvh_test.cu:469-482; bit-exact parity with the reference requires it).  An FP64
brute force of the same points (with the same FP32 box length) may decide a pair differently
only where the true distance lies within 1 ulp(rc) of rc -- plus, for a pair across the periodic
boundary, half an ulp of the FP32 difference pj - pi (about L) per wrapped axis, which is rounded
before the wrap subtracts L.  Quantization of the tree's boxes must never drop a pair.  Checked
on adversarial pairs within a few ulp of the cutoff (open box; and across the periodic boundary),
and on the full lists of 20,000 random points (periodic, rc 1.3) from the symmetric self
traversal.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

import neighbor_gb300 as nb  # noqa: E402
import oracle as O  # noqa: E402
from test_oracle_kats import fp32_disagreement_bound  # noqa: E402

RC = np.float32(1.3)
ULP = float(np.spacing(RC))


@pytest.fixture(scope="module", autouse=True)
def _lib():
    nb.build()
    nb.load()


def _f64_dist(pi, pj, L):
    """Exact minimum-image distance of FP32 points with the FP32 box length L (0 = open)."""
    d = pj.astype(np.float64) - pi.astype(np.float64)
    Lf = np.float64(np.float32(L))
    if L > 0:
        d -= Lf * np.round(d / Lf)
    return np.sqrt((d * d).sum(-1))


def _pairs_one_per_query(centers, pts, L, periodic):
    """The GPU's decision for each (centre k, point k) pair: the sphere query of centre k over a
    tree of the points lists point k (pairs are placed so that no other pair meets)."""
    lbvh = nb.LBVH()
    lbvh.build(torch.from_numpy(pts).cuda(), [0, 0, 0], [L, L, L])
    sph = torch.from_numpy(np.concatenate([centers, np.full((len(centers), 1), RC, np.float32)], 1)).cuda()
    trav = nb.LBVHTraverser()
    pad = nb.exact_pad(float(RC), 2 * L)
    box = [L, L, L] if periodic else [0.0, 0.0, 0.0]
    nn, lst = trav.traverse(lbvh, sph, query=nb.QUERY_EXACT, points=torch.from_numpy(pts).cuda(), box=box,
                            pad=pad, images="periodic" if periodic else None, max_neigh=4)
    nn = nn.cpu().numpy().view(np.uint32)
    lst = lst.cpu().numpy().view(np.uint32)
    assert np.all(nn <= 1)   # pairs never meet
    return (nn == 1) & (lst[:, 0] == np.arange(len(centers)))


def test_adversarial_pairs_disagree_only_within_one_ulp():
    # open box: centre k on a grid of spacing 8, its partner at rc + delta (|delta| <= 3 ulp(rc))
    # in a random direction
    rng = np.random.default_rng(4)
    side = 32
    L = float(side * 8)
    g = np.stack(np.meshgrid(*[np.arange(side)] * 3, indexing="ij"), -1).reshape(-1, 3)
    centers = (g * 8.0 + 4.0).astype(np.float32)
    u = rng.normal(size=centers.shape)
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    r = float(RC) + rng.uniform(-3, 3, len(centers)) * ULP
    pts = (centers.astype(np.float64) + u * r[:, None]).astype(np.float32)
    got = _pairs_one_per_query(centers, pts, L, periodic=False)
    rd = _f64_dist(centers, pts, 0.0)
    dis = got != (rd <= float(RC))
    assert dis.sum() > 20   # the pairs do reach the cutoff's rounding
    assert np.all(np.abs(rd[dis] - float(RC)) < ULP)
    for i in np.nonzero(dis)[0][:50]:   # the host's FP32 predicate decides as the GPU
        assert O.exact_pair(centers[i], pts[i], float(RC), [0, 0, 0]) == bool(got[i])


def test_adversarial_pairs_across_the_boundary():
    # periodic: centres next to the x = 0 face (a grid of spacing 8 in y and z), partners across it
    rng = np.random.default_rng(5)
    side = 64
    L = float(side * 8)
    g = np.stack(np.meshgrid(np.arange(side), np.arange(side), indexing="ij"), -1).reshape(-1, 2)
    centers = np.zeros((len(g), 3), np.float32)
    centers[:, 0] = (0.2 + rng.random(len(g)) * 0.8).astype(np.float32)
    centers[:, 1:] = (g * 8.0 + 4.0).astype(np.float32)
    u = rng.normal(size=centers.shape)
    u[:, 0] = -np.abs(u[:, 0]) - 1.0
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    r = float(RC) + rng.uniform(-400, 400, len(centers)) * ULP
    pts = np.mod(centers.astype(np.float64) + u * r[:, None], L).astype(np.float32)
    pts[:, 0] = np.where(pts[:, 0] >= np.float32(L), np.float32(0), pts[:, 0])
    got = _pairs_one_per_query(centers, pts, L, periodic=True)
    rd = _f64_dist(centers, pts, L)
    dis = got != (rd <= float(RC))
    assert dis.sum() > 100
    assert np.all(np.abs(rd[dis] - float(RC)) < fp32_disagreement_bound(centers[dis], pts[dis], RC, [L, L, L]))
    # (and far beyond 1 ulp(rc): the wrap's rounding is what limits these pairs)
    assert np.abs(rd[dis] - float(RC)).max() > 4 * ULP


def test_random_lists_against_fp64_brute_force():
    N = 20000
    rng = np.random.default_rng(33)
    L = float((N / 0.85) ** (1.0 / 3.0))
    P = (rng.random((N, 3)) * L).astype(np.float32)
    box = [L, L, L]
    lbvh = nb.LBVH()
    lbvh.build(torch.from_numpy(P).cuda(), [0, 0, 0], box)
    trav = nb.LBVHTraverser()
    trav.force_symmetric()
    pad = nb.exact_pad(float(RC), 2 * L)
    trav.traverse_self(lbvh, float(RC), box, pad, images="periodic", rows_sorted=False)
    mx = trav.count_summary()[0]
    nn, lst = trav.traverse_self(lbvh, float(RC), box, pad, images="periodic", rows_sorted=False, max_neigh=mx)
    nn = nn.cpu().numpy().view(np.uint32)
    lst = lst.cpu().numpy().view(np.uint32)
    # candidates: every pair within rc + 1e-4 (a wider host cell list), decided in FP64
    off, nbrs = O.celllist_csr(P, P, float(RC) + 1e-4, [0, 0, 0], box)
    qi = np.repeat(np.arange(N), np.diff(off).astype(np.int64))
    qj = nbrs.astype(np.int64)
    rd = _f64_dist(P[qi], P[qj], L)
    want = rd <= float(RC)
    got_sets = [set(lst[i, :nn[i]].tolist()) for i in range(N)]
    got = np.fromiter((int(j) in got_sets[i] for i, j in zip(qi, qj)), bool, count=len(qi))
    # every listed pair is a candidate: nothing farther than rc + 1e-4 was listed
    assert int(nn.astype(np.int64).sum()) == int(got.sum())
    dis = got != want
    assert np.all(np.abs(rd[dis] - float(RC)) < fp32_disagreement_bound(P[qi[dis]], P[qj[dis]], RC, box))
    assert int(dis.sum()) < 5
