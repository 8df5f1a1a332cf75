"""Parity with the reference's own CUDA kernels, run on the same GPU.

The reference harness (oracle/ref_harness) compiles mphowardlab/neighbor's kernels from its
headers and replays its build / setup / traverse sequence.  Its outputs must equal this
library's bit for bit: sorted codes and primitive order, hierarchy, FP32 boxes, the 10-bit int4
nodes of getData(), the stock query's superset counts, the exact query's counts (which also
equal the oracle's cell list), the stock query's neighbor lists, and the exact query's neighbor
lists, row by row in the reference's order, from the general traversal, the whole-tree self walk and the symmetric self
walk.  Skipped where the reference kernels were not built.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

import neighbor_gb300 as nb  # noqa: E402
import oracle as O  # noqa: E402
from oracle import ref_harness  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _setup():
    nb.build()
    nb.load()
    if not ref_harness.build_if_available() or not ref_harness.available():
        pytest.skip("reference kernels not built (needs the reference sources at build time)")


def _t(a, dtype=torch.float32):
    return torch.tensor(np.asarray(a), dtype=dtype, device="cuda")


def _cases():
    rng = np.random.default_rng(5)
    out = []
    L = 24.0
    out.append(("uniform", (rng.random((20000, 3)) * L).astype(np.float32), L, 1.3))
    c = rng.random((60, 3)) * L
    k = rng.integers(0, 60, 15000)
    p = np.mod(c[k] + rng.normal(size=(15000, 3)) * 0.8, L).astype(np.float32)
    out.append(("clustered", p, L, 1.0))
    out.append(("duplicates", np.tile(np.float32([[3.0, 4.0, 5.0]]), (300, 1)), 8.0, 0.7))
    out.append(("small", (rng.random((5, 3)) * 6).astype(np.float32), 6.0, 2.0))
    # the small plain configuration: 32,768 uniform points at density 0.85, cutoff 1.3
    Lc = float((32768 / 0.85) ** (1.0 / 3.0))
    out.append(("uniform32k", (rng.random((32768, 3)) * Lc).astype(np.float32), Lc, 1.3))
    return out


@pytest.mark.parametrize("name,P,L,rc", _cases(), ids=[c[0] for c in _cases()])
def test_library_matches_reference_kernels(name, P, L, rc):
    box = [L, L, L]
    ref = ref_harness.run_dump(P, [0, 0, 0], box, rc, box)
    lbvh = nb.LBVH()
    lbvh.build(_t(P), [0, 0, 0], box)
    lbvh.check_status()
    a = lbvh.arrays()
    assert np.array_equal(lbvh.codes().cpu().numpy().view(np.uint32), ref["codes"])
    assert np.array_equal(a["primitive"].cpu().numpy().view(np.uint32), ref["primitive"])
    assert np.array_equal(a["parent"].cpu().numpy(), ref["parent"])
    assert np.array_equal(a["left"].cpu().numpy(), ref["left"])
    assert np.array_equal(a["right"].cpu().numpy(), ref["right"])
    assert np.array_equal(a["lo"].cpu().numpy(), ref["lo"])
    assert np.array_equal(a["hi"].cpu().numpy(), ref["hi"])
    trav = nb.LBVHTraverser()
    trav.setup(lbvh)
    torch.cuda.synchronize()
    assert np.array_equal(trav.get_data(lbvh)["data"].cpu().numpy(), ref["data"])
    sph = _t(np.concatenate([P, np.full((len(P), 1), rc, np.float32)], 1))
    stock = trav.traverse(lbvh, sph, images=nb.images27(box)).cpu().numpy().view(np.uint32)
    assert np.array_equal(stock, ref["count_stock"])
    # the stock query's lists (the reference's default path): every row equal, in order
    ms = ref["list_stock"].shape[1]
    _, lst_s = trav.traverse(lbvh, sph, images=nb.images27(box), max_neigh=ms)
    vs = np.arange(ms)[None, :] < ref["count_stock"][:, None]
    got_s = lst_s.cpu().numpy().view(np.uint32)
    assert np.array_equal(np.where(vs, got_s, 0), np.where(vs, ref["list_stock"], 0))
    pad = nb.exact_pad(rc, 2 * L)
    exact = trav.traverse(lbvh, sph, query=nb.QUERY_EXACT, points=_t(P), box=box, pad=pad,
                          images="periodic").cpu().numpy().view(np.uint32)
    assert np.array_equal(exact, ref["count_exact"])
    want, _ = O.celllist_counts(P, P, rc, [0, 0, 0], box)
    assert np.array_equal(exact, want)

    # neighbor lists: every row equal to the reference's, entries in the reference's order
    ref_list = ref["list_exact"]
    mx = ref_list.shape[1]
    assert np.array_equal(ref["count_list"], ref["count_exact"])
    valid = np.arange(mx)[None, :] < ref["count_exact"][:, None]
    _, lst = trav.traverse(lbvh, sph, query=nb.QUERY_EXACT, points=_t(P), box=box, pad=pad,
                           images="periodic", max_neigh=mx)
    got = lst.cpu().numpy().view(np.uint32)
    assert np.array_equal(np.where(valid, got, 0), np.where(valid, ref_list, 0))
    # self traversals: whole-tree walk with one thread per query, symmetric walk (a fill on its
    # own), symmetric count + fill assembled from its pair exchange, one warp per query
    for route in ("thread", "symmetric", "exchange", "warp"):
        st = nb.LBVHTraverser()
        if route == "thread":
            st.set_symmetric(False)
            st.set_warp_walk_max(0)
        elif route in ("symmetric", "exchange"):
            st.force_symmetric()
        else:
            st.set_symmetric(False)
            st.set_warp_walk_max(len(P))
        if route == "exchange":
            st.traverse_self(lbvh, rc, box, pad, images="periodic", rows_sorted=False)
        nn, lst = st.traverse_self(lbvh, rc, box, pad, images="periodic", max_neigh=mx, rows_sorted=False)
        assert np.array_equal(nn.cpu().numpy().view(np.uint32), ref["count_exact"]), route
        got = lst.cpu().numpy().view(np.uint32)
        assert np.array_equal(np.where(valid, got, 0), np.where(valid, ref_list, 0)), route


@pytest.mark.parametrize("radius", [0.25, 1.5])
def test_sphere_tree_matches_reference_kernels(radius):
    # SphereInsertOp (include/neighbor/InsertOps.h:57-96): the tree of spheres of one radius --
    # codes of the box centres, primitive order, hierarchy and the FP32 boxes -- and the
    # reference-layout nodes equal the reference kernels' own sphere tree bit for bit, as do the
    # stock query's counts over it
    rng = np.random.default_rng(int(radius * 100))
    L = 20.0
    P = (rng.random((12000, 3)) * L).astype(np.float32)
    box = [L, L, L]
    ref = ref_harness.run_dump(P, [0, 0, 0], box, 1.0, box, sphere_radius=radius)
    lbvh = nb.LBVH()
    lbvh.build(_t(P), [0, 0, 0], box, radius=radius)
    lbvh.check_status()
    a = lbvh.arrays()
    assert np.array_equal(lbvh.codes().cpu().numpy().view(np.uint32), ref["codes"])
    assert np.array_equal(a["primitive"].cpu().numpy().view(np.uint32), ref["primitive"])
    assert np.array_equal(a["parent"].cpu().numpy(), ref["parent"])
    assert np.array_equal(a["left"].cpu().numpy(), ref["left"])
    assert np.array_equal(a["right"].cpu().numpy(), ref["right"])
    assert np.array_equal(a["lo"].cpu().numpy(), ref["lo"])
    assert np.array_equal(a["hi"].cpu().numpy(), ref["hi"])
    trav = nb.LBVHTraverser()
    trav.setup(lbvh)
    torch.cuda.synchronize()
    assert np.array_equal(trav.get_data(lbvh)["data"].cpu().numpy(), ref["data"])
    sph = _t(np.concatenate([P, np.full((len(P), 1), 1.0, np.float32)], 1))
    stock = trav.traverse(lbvh, sph, images=nb.images27(box)).cpu().numpy().view(np.uint32)
    assert np.array_equal(stock, ref["count_stock"])
