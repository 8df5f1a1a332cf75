"""Symmetric (half) self traversal: same counts, same neighbor sets, same row order.

With the self image or the 27-image lattice, a self traversal finds each unordered pair once and
writes it to both rows; the rows are then ordered by (image, sorted position), the order of a
whole-tree walk (and of the reference's rope traversal).  So the full outputs -- counts and every
list row -- must be bit-identical to the whole-tree walk's, and the sets must equal the oracle's
cell list.  With the size routing off (force_symmetric), counts take the symmetric kernel at every
size.  A fill after a count on the same traverser assembles the rows from the count's pair
exchange (rows whose pairs did not fit it are walked again, one warp per row for up to 32,768
such rows, one thread per row above); a fill without such a count walks symmetrically while rows
fit 32 entries and takes the whole-tree walk beyond.  Rows that overflow max_neigh keep their full
count and a subset of their true neighbors.  The whole-tree side keeps the default routing (lane
groups per query up to 32,768 points).
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

import neighbor_gb300 as nb  # noqa: E402
import oracle as O  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _lib():
    nb.build()
    nb.load()


def _t(a, dtype=torch.float32):
    return torch.tensor(np.asarray(a), dtype=dtype, device="cuda")


def _uniform(N, seed, density=0.85):
    rng = np.random.default_rng(seed)
    L = float((N / density) ** (1.0 / 3.0))
    return (rng.random((N, 3)) * L).astype(np.float32), L


def _clustered(N, seed, L, per=200):
    rng = np.random.default_rng(seed)
    nb_ = max(1, N // per)
    centers = rng.random((nb_, 3)) * L
    sig = np.exp(rng.uniform(np.log(0.5), np.log(3.0), nb_))
    k = rng.integers(0, nb_, N)
    p = centers[k] + rng.normal(size=(N, 3)) * sig[k, None]
    n_bg = N * 3 // 10
    p[:n_bg] = rng.random((n_bg, 3)) * L
    return np.mod(p, L).astype(np.float32)


def _both(lbvh, rc, box, pad, images, rows_sorted, max_neigh=None, map=None, travs=None):
    """(symmetric, whole-tree) results; `travs` keeps the two traversers across calls, so that a
    fill follows the count of the same traverser (the fill then reuses that count's results)."""
    out = []
    for k, sym in enumerate((True, False)):
        if travs is not None and len(travs) > k:
            trav = travs[k]
        else:
            trav = nb.LBVHTraverser()
            trav.set_symmetric(sym)
            if sym:
                trav.force_symmetric()   # the symmetric kernels at every size
            if travs is not None:
                travs.append(trav)
        out.append(trav.traverse_self(lbvh, rc, box, pad, images=images, rows_sorted=rows_sorted,
                                      max_neigh=max_neigh, map=map))
    return out


def _rows(cnt, lst):
    cnt = cnt.cpu().numpy().view(np.uint32)
    lst = lst.cpu().numpy().view(np.uint32)
    mask = np.arange(lst.shape[1])[None, :] < cnt[:, None]
    return cnt, np.where(mask, lst, 0xFFFFFFFF)


@pytest.mark.parametrize("rows_sorted", [True, False])
@pytest.mark.parametrize("images", ["periodic", "self"])
@pytest.mark.parametrize("dist", ["uniform", "clustered"])
@pytest.mark.parametrize("leaf", [1, 4])
def test_symmetric_equals_whole_tree_walk(leaf, dist, images, rows_sorted):
    N = 30000
    P, L = _uniform(N, 41)
    if dist == "clustered":
        P = _clustered(N, 42, L)
    box = [L, L, L] if images == "periodic" else [0, 0, 0]
    rc = 1.3
    lbvh = nb.LBVH(leaf_size=leaf)
    lbvh.build(_t(P), [0, 0, 0], [L, L, L])
    pad = nb.exact_pad(rc, 2 * L)
    imgs = "periodic" if images == "periodic" else None
    travs = []
    c_sym, c_full = _both(lbvh, rc, box, pad, imgs, rows_sorted, travs=travs)
    assert torch.equal(c_sym, c_full)
    mx = int(c_full.max().item())
    (cs, ls), (cf, lf) = _both(lbvh, rc, box, pad, imgs, rows_sorted, max_neigh=mx, travs=travs)
    # the same fill without the count's results (a fresh traverser)
    (cs2, ls2), _ = _both(lbvh, rc, box, pad, imgs, rows_sorted, max_neigh=mx)
    cs2, ls2 = _rows(cs2, ls2)
    cs, ls = _rows(cs, ls)
    cf, lf = _rows(cf, lf)
    assert np.array_equal(cs, cf)
    assert np.array_equal(ls, lf)  # same entries in the same order
    assert np.array_equal(cs2, cf)
    assert np.array_equal(ls2, lf)
    if dist == "clustered":
        assert mx > 32  # rows too long for the symmetric fill
    # the sets are the oracle's (open box: a periodic grid three times wider never wraps a pair)
    if images == "periodic":
        off, nbrs = O.celllist_csr(P, P, rc, [0, 0, 0], box)
    else:
        off, nbrs = O.celllist_csr(P, P, rc, [-L, -L, -L], [3 * L, 3 * L, 3 * L])
    prim = lbvh.primitives().cpu().numpy().view(np.uint32)
    row_of = prim if rows_sorted else np.arange(N, dtype=np.uint32)
    want = np.diff(off).astype(np.uint32)
    assert np.array_equal(cs, want[row_of])
    for r in range(0, N, 211):
        got = np.sort(ls[r, : cs[r]])
        assert np.array_equal(got, nbrs[off[row_of[r]]:off[row_of[r] + 1]])


def test_symmetric_overflow_keeps_counts_and_a_subset():
    N = 20000
    P, L = _uniform(N, 43)
    box = [L, L, L]
    rc = 1.3
    lbvh = nb.LBVH()
    lbvh.build(_t(P), [0, 0, 0], box)
    pad = nb.exact_pad(rc, 2 * L)
    trav = nb.LBVHTraverser()
    trav.force_symmetric()
    full = trav.traverse_self(lbvh, rc, box, pad, images="periodic", rows_sorted=False)
    cnt, lst = trav.traverse_self(lbvh, rc, box, pad, images="periodic", rows_sorted=False, max_neigh=5)
    assert torch.equal(cnt, full)
    off, nbrs = O.celllist_csr(P, P, rc, [0, 0, 0], box)
    cnt = cnt.cpu().numpy().view(np.uint32)
    lst = lst.cpu().numpy().view(np.uint32)
    for r in range(N):
        k = min(int(cnt[r]), 5)
        assert set(lst[r, :k].tolist()) <= set(nbrs[off[r]:off[r + 1]].tolist())


def test_symmetric_transform_and_long_rows():
    # dense clusters: rows of several hundred entries (the fill takes the whole-tree walk, the
    # count the symmetric kernel), a map transform on the ids
    N = 20000
    L = 30.0
    P = _clustered(N, 44, L, per=2000)
    box = [L, L, L]
    rc = 1.5
    lbvh = nb.LBVH()
    lbvh.build(_t(P), [0, 0, 0], box)
    pad = nb.exact_pad(rc, 2 * L)
    rng = np.random.default_rng(45)
    m = rng.permutation(N).astype(np.int32)
    c_full = nb.LBVHTraverser().traverse_self(lbvh, rc, box, pad, images="periodic", rows_sorted=True)
    mx = int(c_full.max().item())
    assert 32 < mx <= 4096
    (cs, ls), (cf, lf) = _both(lbvh, rc, box, pad, "periodic", True, max_neigh=mx, map=_t(m, torch.int32))
    cs, ls = _rows(cs, ls)
    cf, lf = _rows(cf, lf)
    assert np.array_equal(cs, cf)
    assert np.array_equal(ls, lf)


@pytest.mark.parametrize("images", ["periodic", "self"])
@pytest.mark.parametrize("N", [1, 37, 300, 20000])
def test_work_order_does_not_change_results(N, images):
    P, L = _uniform(N, 7)
    box = [L, L, L] if images == "periodic" else [0, 0, 0]
    imgs = "periodic" if images == "periodic" else None
    rc = 1.3
    lbvh = nb.LBVH()
    lbvh.build(_t(P), [0, 0, 0], [L, L, L])
    pad = nb.exact_pad(rc, 2 * L)
    out = []
    for ordered in (False, True):
        trav = nb.LBVHTraverser()
        trav.set_work_order(ordered)
        trav.force_symmetric()   # the symmetric kernels at every size
        trav.set_pair_cache(False)   # the fill walks again (in the count's work order)
        cnt = trav.traverse_self(lbvh, rc, box, pad, images=imgs)   # records the walk lengths
        mx = max(1, int(cnt.max().item()))
        out.append(_rows(*trav.traverse_self(lbvh, rc, box, pad, images=imgs, max_neigh=mx)))
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])


@pytest.mark.parametrize("count_rows_sorted,fill_rows_sorted", [(True, True), (False, False), (True, False),
                                                                (False, True)])
def test_fill_after_count_with_map_transform(count_rows_sorted, fill_rows_sorted):
    # the fill reuses the count's row totals only when both ran on the same rows
    N = 30000
    P, L = _uniform(N, 52)
    box = [L, L, L]
    rc = 1.3
    lbvh = nb.LBVH()
    lbvh.build(_t(P), [0, 0, 0], box)
    pad = nb.exact_pad(rc, 2 * L)
    m = _t(np.random.default_rng(53).permutation(N).astype(np.int32), torch.int32)
    whole = nb.LBVHTraverser()
    whole.set_symmetric(False)
    cnt_w = whole.traverse_self(lbvh, rc, box, pad, images="periodic", rows_sorted=fill_rows_sorted)
    mx = int(cnt_w.max().item())
    cf, lf = _rows(*whole.traverse_self(lbvh, rc, box, pad, images="periodic", rows_sorted=fill_rows_sorted,
                                        max_neigh=mx, map=m))
    trav = nb.LBVHTraverser()
    trav.traverse_self(lbvh, rc, box, pad, images="periodic", rows_sorted=count_rows_sorted)
    cs, ls = _rows(*trav.traverse_self(lbvh, rc, box, pad, images="periodic", rows_sorted=fill_rows_sorted,
                                       max_neigh=mx, map=m))
    assert np.array_equal(cs, cf)
    assert np.array_equal(ls, lf)
    # a rebuild invalidates the count's results
    P2 = np.mod(P + np.random.default_rng(54).normal(size=P.shape).astype(np.float32) * 0.3, L).astype(np.float32)
    lbvh.build(_t(P2), [0, 0, 0], box)
    cnt2 = whole.traverse_self(lbvh, rc, box, pad, images="periodic", rows_sorted=fill_rows_sorted)
    mx2 = int(cnt2.max().item())
    cf2, lf2 = _rows(*whole.traverse_self(lbvh, rc, box, pad, images="periodic", rows_sorted=fill_rows_sorted,
                                          max_neigh=mx2))
    cs2, ls2 = _rows(*trav.traverse_self(lbvh, rc, box, pad, images="periodic", rows_sorted=fill_rows_sorted,
                                         max_neigh=mx2))
    assert np.array_equal(cs2, cf2)
    assert np.array_equal(ls2, lf2)


@pytest.mark.parametrize("N", [300, 25000])
def test_noncubic_offset_box(N):
    # periodic box of unequal sides whose corner is not the origin: counts and sets equal the
    # oracle's cell list, and the symmetric count + ordered fill equal the whole-tree walk row by row
    rng = np.random.default_rng(71)
    Lv = np.array([21.0, 14.5, 26.3]) * (N / 25000.0) ** (1.0 / 3.0)
    lo = np.array([-5.0, 2.0, 10.0])
    P = (lo + rng.random((N, 3)) * Lv).astype(np.float32)
    box = [float(v) for v in Lv]
    rc = 1.3
    lbvh = nb.LBVH()
    lbvh.build(_t(P), lo.tolist(), (lo + Lv).tolist())
    pad = nb.exact_pad(rc, 2.0 * float(np.max(np.abs(lo + 2 * Lv))))
    trav = nb.LBVHTraverser()
    trav.force_symmetric()   # the symmetric kernels at every size
    cnt = trav.traverse_self(lbvh, rc, box, pad, images="periodic", rows_sorted=False)
    mx = max(1, int(cnt.max().item()))
    cs, ls = _rows(*trav.traverse_self(lbvh, rc, box, pad, images="periodic", rows_sorted=False, max_neigh=mx))
    whole = nb.LBVHTraverser()
    whole.set_symmetric(False)
    cf, lf = _rows(*whole.traverse_self(lbvh, rc, box, pad, images="periodic", rows_sorted=False, max_neigh=mx))
    assert np.array_equal(cs, cf)
    assert np.array_equal(ls, lf)
    off, nbrs = O.celllist_csr(P, P, rc, lo.tolist(), box)
    assert np.array_equal(cs, np.diff(off).astype(np.uint32))
    for r in range(0, N, max(1, N // 97)):
        assert np.array_equal(np.sort(ls[r, : cs[r]]), nbrs[off[r]:off[r + 1]])


@pytest.mark.parametrize("rows_sorted", [True, False])
def test_pair_exchange_assembles_the_count(rows_sorted):
    # tight clusters of 20 points inside the cutoff: rows of about 20 entries; the first points of
    # a cluster find more than 16 pairs themselves and the last ones receive more than 16 (both
    # are walked again); the assembled fill, the walking fill and the whole-tree walk must agree
    rng = np.random.default_rng(61)
    N, L, rc = 24000, 33.0, 1.0
    # cluster centres on a grid of spacing 3 (clusters do not meet), jittered
    g = np.stack(np.meshgrid(np.arange(11), np.arange(11), np.arange(10), indexing="ij"), -1).reshape(-1, 3)
    centers = (g[: N // 20] * 3.0 + 1.5 + rng.uniform(-0.2, 0.2, (N // 20, 3)))
    P = np.mod(np.repeat(centers, 20, axis=0) + rng.normal(size=(N, 3)) * 0.12, L).astype(np.float32)
    box = [L, L, L]
    lbvh = nb.LBVH()
    lbvh.build(_t(P), [0, 0, 0], box)
    pad = nb.exact_pad(rc, 2 * L)
    out = []
    for mode in ("cache", "walk", "whole"):
        trav = nb.LBVHTraverser()
        if mode == "whole":
            trav.set_symmetric(False)
            trav.set_warp_walk_max(0)
        else:
            trav.force_symmetric()
            trav.set_pair_cache(mode == "cache")
        cnt = trav.traverse_self(lbvh, rc, box, pad, images="periodic", rows_sorted=rows_sorted)
        mx = int(cnt.max().item())
        assert 16 < mx <= 32
        out.append(_rows(*trav.traverse_self(lbvh, rc, box, pad, images="periodic", rows_sorted=rows_sorted,
                                             max_neigh=mx)))
        assert np.array_equal(out[-1][0], cnt.cpu().numpy().view(np.uint32))
    for c, lst in out[1:]:
        assert np.array_equal(c, out[0][0])
        assert np.array_equal(lst, out[0][1])
    # a fill on other rows than the count's does not assemble from its pairs
    trav = nb.LBVHTraverser()
    trav.force_symmetric()
    trav.traverse_self(lbvh, rc, box, pad, images="periodic", rows_sorted=not rows_sorted)
    c, lst = _rows(*trav.traverse_self(lbvh, rc, box, pad, images="periodic", rows_sorted=rows_sorted,
                                       max_neigh=int(out[0][0].max())))
    assert np.array_equal(c, out[0][0])
    assert np.array_equal(lst, out[0][1])


def test_fill_after_a_count_on_another_tree_walks():
    # the count ran on tree A, which is then destroyed; tree B (same size, other points, possibly
    # at A's address) is filled by the same traverser: nothing of A's count may be reused
    N = 20000
    PA, L = _uniform(N, 71)
    PB, _ = _uniform(N, 72)
    box = [L, L, L]
    rc = 1.3
    pad = nb.exact_pad(rc, 2 * L)
    trav = nb.LBVHTraverser()
    trav.force_symmetric()
    a = nb.LBVH()
    a.build(_t(PA), [0, 0, 0], box)
    trav.traverse_self(lbvh=a, rc=rc, box=box, pad=pad, images="periodic", rows_sorted=True)
    torch.cuda.synchronize()
    del a
    b = nb.LBVH()
    b.build(_t(PB), [0, 0, 0], box)
    whole = nb.LBVHTraverser()
    whole.set_symmetric(False)
    whole.set_warp_walk_max(0)
    cnt = whole.traverse_self(b, rc, box, pad, images="periodic", rows_sorted=True)
    mx = int(cnt.max().item())
    want = _rows(*whole.traverse_self(b, rc, box, pad, images="periodic", rows_sorted=True, max_neigh=mx))
    got = _rows(*trav.traverse_self(b, rc, box, pad, images="periodic", rows_sorted=True, max_neigh=mx))
    assert np.array_equal(got[0], want[0])
    assert np.array_equal(got[1], want[1])


def test_pair_cache_csr_fill_equals_whole_walk():
    # count, then a CSR fill (rows sized by the counts) assembled from the count's pairs
    N = 60000
    P, L = _uniform(N, 81)
    box = [L, L, L]
    rc = 1.3
    lbvh = nb.LBVH()
    lbvh.build(_t(P), [0, 0, 0], box)
    pad = nb.exact_pad(rc, 2 * L)
    op = nb.OnePassList()
    out = []
    for mode in ("assembled", "whole"):
        trav = nb.LBVHTraverser()
        if mode == "assembled":
            trav.force_symmetric()
        else:
            trav.set_symmetric(False)
            trav.set_warp_walk_max(0)
        cnt = trav.traverse_self(lbvh, rc, box, pad, images="periodic", rows_sorted=False)
        mx = int(cnt.max().item())
        assert mx <= 32
        offsets, total = op.scan(cnt)
        lst = torch.full((total + 1,), -1, dtype=torch.int32, device="cuda")
        nn = trav.traverse_self_csr(lbvh, rc, box, pad, offsets, cnt, lst, max_capacity=mx, images="periodic",
                                    rows_sorted=False)
        assert torch.equal(nn, cnt)
        out.append(lst.cpu().numpy())
    assert np.array_equal(out[0], out[1])


@pytest.mark.parametrize("per,N", [(30, 24000), (40, 80000)])
def test_rows_past_the_exchange_are_walked(per, N):
    # tight clusters of `per` points inside the cutoff: most rows hold more pairs than the
    # exchange keeps.  24,000 such rows are walked one warp per row, 80,000 one thread per row;
    # rows in both cases equal the whole-tree walk, for a fixed-stride list and a CSR list.
    rng = np.random.default_rng(per)
    n_cl = N // per
    side = int(np.ceil(n_cl ** (1.0 / 3.0)))
    L = side * 3.0
    g = np.stack(np.meshgrid(np.arange(side), np.arange(side), np.arange(side), indexing="ij"), -1).reshape(-1, 3)
    centers = g[:n_cl] * 3.0 + 1.5
    P = np.mod(np.repeat(centers, per, axis=0) + rng.normal(size=(N, 3)) * 0.1, L).astype(np.float32)
    rc = 1.0
    box = [L, L, L]
    lbvh = nb.LBVH()
    lbvh.build(_t(P), [0, 0, 0], box)
    pad = nb.exact_pad(rc, 2 * L)
    trav = nb.LBVHTraverser()
    trav.force_symmetric()
    cnt = trav.traverse_self(lbvh, rc, box, pad, images="periodic", rows_sorted=True)
    # (the largest count from the counts themselves: a summary read on the host would steer these
    # dense fills to the whole-tree walk, and this test is about the assembly and its re-walk)
    c = cnt.cpu().numpy().view(np.uint32)
    mx = int(c.max())
    whole = nb.LBVHTraverser()
    whole.set_symmetric(False)
    whole.set_warp_walk_max(0)
    want = _rows(*whole.traverse_self(lbvh, rc, box, pad, images="periodic", rows_sorted=True, max_neigh=mx))
    got = _rows(*trav.traverse_self(lbvh, rc, box, pad, images="periodic", rows_sorted=True, max_neigh=mx))
    assert np.array_equal(got[0], want[0])
    assert np.array_equal(got[1], want[1])
    op = nb.OnePassList()
    offsets, tot = op.scan(cnt)
    lst = torch.full((tot + 1,), -1, dtype=torch.int32, device="cuda")
    nn = trav.traverse_self_csr(lbvh, rc, box, pad, offsets, cnt, lst, max_capacity=mx, images="periodic",
                                rows_sorted=True)
    assert torch.equal(nn, cnt)
    flat = lst[:tot].cpu().numpy().view(np.uint32)
    off = offsets.cpu().numpy()
    for r in range(0, N, 97):
        assert np.array_equal(flat[off[r]:off[r] + c[r]], want[1][r, : c[r]])
    mx2, total, past = trav.count_summary()
    assert mx2 == mx and total == int(c.astype(np.int64).sum())
    assert past > (20000 if N == 24000 else 60000)
    # With the summary read, the fill walks the whole tree and the next counts skip the exchange
    # (too many rows past it); a count without the exchange reports rows longer than 32, and the
    # lists stay the same through every step of that sequence.
    got = _rows(*trav.traverse_self(lbvh, rc, box, pad, images="periodic", rows_sorted=True, max_neigh=mx))
    assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])
    for k in range(2):
        cnt2 = trav.traverse_self(lbvh, rc, box, pad, images="periodic", rows_sorted=True)
        assert torch.equal(cnt2, cnt)
        m3, t3, rows_past = trav.count_summary()
        assert m3 == mx and t3 == total
        if k == 0:   # the count after the dense summary: no exchange, rows longer than 32 reported
            assert rows_past == int(np.count_nonzero(c > 32))
        got = _rows(*trav.traverse_self(lbvh, rc, box, pad, images="periodic", rows_sorted=True, max_neigh=mx))
        assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])


@pytest.mark.parametrize("symmetric", [True, False])
def test_count_summary(symmetric):
    # the largest count and the total on the device equal the counts' own, on either route
    N = 50000
    P, L = _uniform(N, 91)
    box = [L, L, L]
    rc = 1.3
    lbvh = nb.LBVH()
    lbvh.build(_t(P), [0, 0, 0], box)
    pad = nb.exact_pad(rc, 2 * L)
    trav = nb.LBVHTraverser()
    if symmetric:
        trav.force_symmetric()
    else:
        trav.set_symmetric(False)
        trav.set_warp_walk_max(0)
    for rows_sorted in (True, False):
        cnt = trav.traverse_self(lbvh, rc, box, pad, images="periodic", rows_sorted=rows_sorted)
        mx, total, past = trav.count_summary()
        c = cnt.cpu().numpy().view(np.uint32)
        assert mx == int(c.max())
        assert total == int(c.astype(np.int64).sum())
        assert 0 <= past < N // 100
        assert trav.count_summary_device() != 0
