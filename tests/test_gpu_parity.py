"""Parity of the CUDA path with the CPU oracle on seeded inputs.

Bit-exact for everything integer or index valued (Morton codes, sorted order, hierarchy, node
records, neighbor sets); FP32 boxes compared with ==.
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
    L = float((max(N, 1) / density) ** (1.0 / 3.0))
    return (rng.random((N, 3)) * L).astype(np.float32), L


def _clustered(N, seed, L):
    rng = np.random.default_rng(seed)
    nb_ = max(1, N // 200)
    centers = rng.random((nb_, 3)) * L
    sig = np.exp(rng.uniform(np.log(0.5), np.log(3.0), nb_))
    k = rng.integers(0, nb_, N)
    p = centers[k] + rng.normal(size=(N, 3)) * sig[k, None]
    n_bg = N * 3 // 10
    p[:n_bg] = rng.random((n_bg, 3)) * L
    return np.mod(p, L).astype(np.float32)


def _edge_inputs():
    rng = np.random.default_rng(11)
    cases = []
    for N in [2, 3, 31, 32, 33, 100]:
        cases.append((f"uniform{N}", (rng.random((N, 3)) * 10).astype(np.float32), [0, 0, 0], [10, 10, 10]))
    cases.append(("duplicates", np.tile(np.float32([[1.5, 2.5, 3.5]]), (77, 1)), [0, 0, 0], [4, 4, 4]))
    # points exactly on Morton bin edges: x = k * L / 1023
    g = (np.arange(64, dtype=np.float32) * np.float32(8.0 / 1023.0)).astype(np.float32)
    cases.append(("bin_edges", np.stack([g, g[::-1], np.roll(g, 7)], 1), [0, 0, 0], [8, 8, 8]))
    # everything in one Morton cell (all codes equal: the index tie-break builds the tree)
    cases.append(("same_code", (rng.random((50, 3)) * 1e-4 + 0.5).astype(np.float32), [0, 0, 0], [1024, 1024, 1024]))
    # points outside the scene bounds are clamped to the edge bins
    cases.append(("outside", (rng.random((40, 3)) * 20 - 5).astype(np.float32), [0, 0, 0], [10, 10, 10]))
    # a plane (zero extent in z)
    pl = rng.random((60, 3)).astype(np.float32) * 5
    pl[:, 2] = 1.0
    cases.append(("plane", pl, [0, 0, 0], [5, 5, 5]))
    return cases


def _check_tree(lbvh, P, lo, hi, insert=O.INSERT_POINT, r=0.0):
    T = O.build_tree(P, lo, hi, insert=insert, r=r)
    a = lbvh.arrays()
    N = len(P)
    if N > 1:  # a one-primitive build computes no codes (reference: LBVH.h:252-257)
        assert np.array_equal(lbvh.codes().cpu().numpy().view(np.uint32), T["codes"])
    assert np.array_equal(a["primitive"].cpu().numpy().view(np.uint32), T["primitive"])
    assert np.array_equal(a["parent"].cpu().numpy(), T["parent"])
    if N > 1:
        assert np.array_equal(a["left"].cpu().numpy(), T["left"])
        assert np.array_equal(a["right"].cpu().numpy(), T["right"])
    assert np.array_equal(a["lo"].cpu().numpy(), T["lo"])
    assert np.array_equal(a["hi"].cpu().numpy(), T["hi"])
    return T


@pytest.mark.parametrize("name,P,lo,hi", _edge_inputs(), ids=[c[0] for c in _edge_inputs()])
@pytest.mark.parametrize("leaf", [1, 4])
def test_tree_and_nodes_edge_cases(name, P, lo, hi, leaf):
    lbvh = nb.LBVH(leaf_size=leaf)
    lbvh.build(_t(P), lo, hi)
    lbvh.check_status()
    T = _check_tree(lbvh, P, lo, hi)
    fast = lbvh.fast()
    want_nodes, want_frame = O.fast_nodes(T, leaf)
    assert np.array_equal(fast["frame"].cpu().numpy()[[0, 1, 2, 6, 7, 8]], want_frame)
    assert np.array_equal(fast["nodes"].cpu().numpy().view(np.uint32), want_nodes)
    # reference-layout nodes (getData) after setup
    trav = nb.LBVHTraverser()
    trav.setup(lbvh)
    torch.cuda.synchronize()
    d = trav.get_data(lbvh)
    want = O.compress_ref10(T)
    assert np.array_equal(d["data"].cpu().numpy(), want[0])
    assert np.array_equal(d["bins"].cpu().numpy(), want[3])


@pytest.mark.parametrize("N,seed", [(1000, 1), (33333, 2), (200000, 3)])
@pytest.mark.parametrize("radix_bits", [8, 10])
def test_tree_uniform(N, seed, radix_bits):
    P, L = _uniform(N, seed)
    lbvh = nb.LBVH(radix_bits=radix_bits)
    lbvh.build(_t(P), [0, 0, 0], [L, L, L])
    lbvh.check_status()
    _check_tree(lbvh, P, [0, 0, 0], [L, L, L])


def test_tree_sphere_insert():
    P, L = _uniform(5000, 4)
    lbvh = nb.LBVH()
    lbvh.build(_t(P), [0, 0, 0], [L, L, L], radius=0.37)
    lbvh.check_status()
    _check_tree(lbvh, P, [0, 0, 0], [L, L, L], insert=O.INSERT_SPHERE, r=0.37)


@pytest.mark.parametrize("leaf", [1, 2, 4, 8, 16])
def test_fast_nodes_clustered(leaf):
    L = 40.0
    P = _clustered(30000, 5, L)
    lbvh = nb.LBVH(leaf_size=leaf)
    lbvh.build(_t(P), [0, 0, 0], [L, L, L])
    lbvh.check_status()
    T = O.build_tree(P, [0, 0, 0], [L, L, L])
    fast = lbvh.fast()
    want, _ = O.fast_nodes(T, leaf)
    assert np.array_equal(fast["nodes"].cpu().numpy().view(np.uint32), want)


@pytest.mark.parametrize("climb", [128, 256, 512])
@pytest.mark.parametrize("N", [5000, 70001])
def test_climb_block_sizes_give_the_same_tree(climb, N):
    # the block size of the agglomerative climb changes which splits meet in shared memory and
    # which across blocks, never the tree
    L = 40.0
    P = _clustered(N, 6, L)
    lbvh = nb.LBVH(leaf_size=4, climb_block=climb)
    lbvh.build(_t(P), [0, 0, 0], [L, L, L])
    lbvh.check_status()
    T = _check_tree(lbvh, P, [0, 0, 0], [L, L, L])
    want, _ = O.fast_nodes(T, 4)
    assert np.array_equal(lbvh.fast()["nodes"].cpu().numpy().view(np.uint32), want)


def _csr_rows(off, nbrs, i):
    return nbrs[off[i]:off[i + 1]]


@pytest.mark.parametrize("images", ["list", "periodic"])
@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("leaf", [1, 4, 8])
@pytest.mark.parametrize("dist", ["uniform", "clustered"])
def test_exact_self_lists_match_cell_list(leaf, dist, mode, images):
    N = 40000
    P, L = _uniform(N, 7)
    if dist == "clustered":
        P = _clustered(N, 8, L)
    box = [L, L, L]
    rc = 1.3
    lbvh = nb.LBVH(leaf_size=leaf)
    lbvh.build(_t(P), [0, 0, 0], box)
    trav = nb.LBVHTraverser()
    trav.set_mode(mode)
    pad = nb.exact_pad(rc, 2 * L)
    imgs = nb.images27(box) if images == "list" else "periodic"
    cnt = trav.traverse_self(lbvh, rc, box, pad, images=imgs, rows_sorted=False)
    off, nbrs = O.celllist_csr(P, P, rc, [0, 0, 0], box)
    want = np.diff(off).astype(np.uint32)
    got = cnt.cpu().numpy().view(np.uint32)
    assert np.array_equal(got, want)
    mx = int(want.max())
    cnt2, lst = trav.traverse_self(lbvh, rc, box, pad, images=imgs, rows_sorted=False, max_neigh=mx)
    lst = lst.cpu().numpy().view(np.uint32)
    assert np.array_equal(cnt2.cpu().numpy().view(np.uint32), want)
    got_sorted = np.sort(np.where(np.arange(mx)[None, :] < want[:, None], lst, 0xFFFFFFFF), axis=1)
    flat = got_sorted[got_sorted != 0xFFFFFFFF]
    assert np.array_equal(flat, nbrs)


@pytest.mark.parametrize("mode", [0, 1])
def test_exact_unsorted_queries(mode):
    # queries in random order (packets are not compact) and a small open box
    rng = np.random.default_rng(30)
    P = (rng.random((6000, 3)) * 12).astype(np.float32)
    Qp = (rng.random((3000, 3)) * 14 - 1).astype(np.float32)
    r = rng.uniform(0.3, 1.6, 3000).astype(np.float32)
    lbvh = nb.LBVH(leaf_size=4)
    lbvh.build(_t(P), [0, 0, 0], [12, 12, 12])
    trav = nb.LBVHTraverser()
    trav.set_mode(mode)
    sph = np.concatenate([Qp, r[:, None]], 1)
    got = trav.traverse(lbvh, _t(sph), query=nb.QUERY_EXACT, points=_t(P), box=(0, 0, 0),
                        pad=nb.exact_pad(1.6, 16.0)).cpu().numpy().view(np.uint32)
    want = O.brute_count(Qp, r, P, (0, 0, 0))
    assert np.array_equal(got, want)


def test_exact_query_rows_sorted_and_transform():
    P, L = _uniform(20000, 9)
    box = [L, L, L]
    rc = 1.3
    lbvh = nb.LBVH()
    lbvh.build(_t(P), [0, 0, 0], box)
    prim = lbvh.primitives().cpu().numpy().view(np.uint32).copy()
    trav = nb.LBVHTraverser()
    pad = nb.exact_pad(rc, 2 * L)
    imgs = nb.images27(box)
    cs = trav.traverse_self(lbvh, rc, box, pad, images=imgs, rows_sorted=True).cpu().numpy()
    want, _ = O.celllist_counts(P, P, rc, [0, 0, 0], box)
    assert np.array_equal(cs.view(np.uint32), want[prim])
    # spheres in sorted order through the generic traverse() entry point, map = inverse order
    sph = np.concatenate([P[prim], np.full((len(P), 1), rc, np.float32)], 1)
    inv = np.empty_like(prim)
    inv[prim] = np.arange(len(prim), dtype=np.uint32)
    nn, lst = trav.traverse(lbvh, _t(sph), query=nb.QUERY_EXACT, points=_t(P[prim]), box=box,
                            pad=pad, images=imgs, map=_t(inv.view(np.int32), torch.int32),
                            max_neigh=int(want.max()))
    nn = nn.cpu().numpy().view(np.uint32)
    assert np.array_equal(nn, want[prim])
    off, nbrs = O.celllist_csr(P, P, rc, [0, 0, 0], box)
    lst = lst.cpu().numpy().view(np.uint32)
    for s in range(0, len(P), 997):
        got = np.sort(prim[lst[s, : nn[s]]])
        assert np.array_equal(got, _csr_rows(off, nbrs, prim[s]))


def test_generic_path_matches_fast_path():
    # The same exact query through the reference-layout kernel gives the same sets.
    P, L = _uniform(8000, 10)
    box = [L, L, L]
    rc = 1.3
    lbvh = nb.LBVH()
    lbvh.build(_t(P), [0, 0, 0], box)
    pad = nb.exact_pad(rc, 2 * L)
    imgs = nb.images27(box)
    sph = _t(np.concatenate([P, np.full((len(P), 1), rc, np.float32)], 1))
    fast = nb.LBVHTraverser()
    slow = nb.LBVHTraverser()
    slow.set_fast_path(False)
    a = fast.traverse(lbvh, sph, query=nb.QUERY_EXACT, points=_t(P), box=box, pad=pad, images=imgs)
    b = slow.traverse(lbvh, sph, query=nb.QUERY_EXACT, points=_t(P), box=box, pad=pad, images=imgs)
    assert torch.equal(a, b)


def test_stock_sphere_query_matches_reference_superset():
    # Stock SphereQueryOp (refine() == true): counts equal to the reference's rope traversal
    # over its 10-bit nodes, restated in the oracle.
    P, L = _uniform(20000, 12)
    lbvh = nb.LBVH()
    lbvh.build(_t(P), [0, 0, 0], [L, L, L])
    sph = np.concatenate([P, np.full((len(P), 1), 1.3, np.float32)], 1)
    imgs = O.images27([L, L, L])
    trav = nb.LBVHTraverser()
    got = trav.traverse(lbvh, _t(sph), images=_t(imgs)).cpu().numpy().view(np.uint32)
    comp = O.compress_ref10(O.build_tree(P, [0, 0, 0], [L, L, L]))
    want = O.traverse_ref10(comp, sph, images=imgs)
    assert np.array_equal(got, want)


def test_empty_and_zero_queries():
    lbvh = nb.LBVH()
    lbvh.build(torch.empty((0, 3), dtype=torch.float32, device="cuda"), [0, 0, 0], [1, 1, 1])
    assert lbvh.sizes()[1] == 0
    trav = nb.LBVHTraverser()
    out = trav.traverse(lbvh, torch.zeros((5, 4), device="cuda"))
    assert out.shape[0] == 5  # nothing traversed, nothing written (reference: LBVHTraverser.h:423)


def test_too_many_images_rejected():
    P, L = _uniform(100, 13)
    lbvh = nb.LBVH()
    lbvh.build(_t(P), [0, 0, 0], [L, L, L])
    trav = nb.LBVHTraverser()
    with pytest.raises(nb.NeighborError):
        trav.traverse(lbvh, _t(np.zeros((3, 4), np.float32)), images=torch.zeros((33, 3), device="cuda"))


def test_rebuild_shrink_and_grow():
    # Reusing one LBVH across sizes (allocation grows, never shrinks; results stay exact).
    lbvh = nb.LBVH()
    for N, seed in [(5000, 20), (300, 21), (12000, 22), (1, 23), (7, 24)]:
        P, L = _uniform(N, seed)
        lbvh.build(_t(P), [0, 0, 0], [L, L, L])
        lbvh.check_status()
        _check_tree(lbvh, P, [0, 0, 0], [L, L, L])


def test_periodic_images_op_matches_explicit_list():
    # PeriodicImagesOp must give exactly the explicit 27-image list's results, on the fast path
    # (exact query) and on the reference-layout path (stock query).
    P, L = _uniform(15000, 31)
    box = [L, L, L]
    lbvh = nb.LBVH()
    lbvh.build(_t(P), [0, 0, 0], box)
    sph = _t(np.concatenate([P, np.full((len(P), 1), 1.3, np.float32)], 1))
    trav = nb.LBVHTraverser()
    a = trav.traverse(lbvh, sph, images=nb.images27(box))
    b = trav.traverse(lbvh, sph, images="periodic", box=box)
    assert torch.equal(a, b)
    pad = nb.exact_pad(1.3, 2 * L)
    c = trav.traverse(lbvh, sph, query=nb.QUERY_EXACT, points=_t(P), box=box, pad=pad, images=nb.images27(box))
    d = trav.traverse(lbvh, sph, query=nb.QUERY_EXACT, points=_t(P), box=box, pad=pad, images="periodic")
    assert torch.equal(c, d)
    want, _ = O.celllist_counts(P, P, 1.3, [0, 0, 0], box)
    assert np.array_equal(d.cpu().numpy().view(np.uint32), want)
