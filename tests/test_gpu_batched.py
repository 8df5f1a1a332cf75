"""Batched ensembles: one launch for many small periodic systems, equal to one call per system.

Every system's counts and list rows (global ids) must equal, bit for bit and in order, those of
LBVH.build + traverse_self on that system alone -- which the parity tests pin to the oracle --
for every configuration the autotuner can pick, through a captured CUDA graph, and through the
sequential plain form the bench compares with.  A few systems are also checked against the
oracle's cell list directly.
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


RC = 1.3
MAXN = 64


def _systems(seed, S):
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(64), np.log(16384), S)).astype(np.int64)
    sizes = np.concatenate([sizes, [1, 2, 3, 31, 16384]])
    pts, boxes = [], []
    for n in sizes:
        L = max(float((n / 0.85) ** (1.0 / 3.0)), 3.0)
        pts.append((rng.random((n, 3)) * L).astype(np.float32))
        boxes.append([L, L, L])
    start = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint32)
    return np.concatenate(pts), start, np.asarray(boxes, np.float32)


def _per_system(P, start, boxes):
    """counts and lists (global ids, MAXN per row) by one library call per system."""
    T = int(start[-1])
    cnt = np.zeros(T, np.uint32)
    lst = np.full((T, MAXN), 0xFFFFFFFF, np.uint32)
    trav = nb.LBVHTraverser()
    for s in range(len(start) - 1):
        o, e = int(start[s]), int(start[s + 1])
        L = float(boxes[s][0])
        lbvh = nb.LBVH()
        lbvh.build(torch.tensor(P[o:e], device="cuda"), [0, 0, 0], [L, L, L])
        c, li = trav.traverse_self(lbvh, RC, [L, L, L], nb.exact_pad(RC, 2 * L), images="periodic",
                                   rows_sorted=False, max_neigh=MAXN)
        c = c.cpu().numpy().view(np.uint32)
        li = li.cpu().numpy().view(np.uint32)
        cnt[o:e] = c
        for r in range(e - o):
            lst[o + r, : c[r]] = li[r, : c[r]] + o
    return cnt, lst


def _rows(cnt, lst):
    cnt = cnt.cpu().numpy().view(np.uint32)
    lst = lst.cpu().numpy().view(np.uint32).reshape(len(cnt), -1)
    mask = np.arange(lst.shape[1])[None, :] < cnt[:, None]
    return cnt, np.where(mask, lst, 0xFFFFFFFF)


@pytest.fixture(scope="module")
def batch():
    P, start, boxes = _systems(5, 40)
    want = _per_system(P, start, boxes)
    return P, start, boxes, want


@pytest.mark.parametrize("block", [512, 1024])
@pytest.mark.parametrize("leaf", [1, 4, 8])
def test_batched_equals_one_call_per_system(batch, leaf, block):
    P, start, boxes, (wc, wl) = batch
    b = nb.BatchedList()
    b.setup(start, boxes, RC, MAXN)
    b.set_config(leaf, block)
    pts = torch.tensor(P, device="cuda")
    cnt, lst = b.outputs()
    for _ in range(2):  # twice: the workspace keeps the previous run's contents
        cnt.fill_(-1)
        b.run(pts, cnt, lst)
        c, l = _rows(cnt, lst)
        assert np.array_equal(c, wc)
        assert np.array_equal(l, wl)
    bits, largest = b.status()
    assert bits == 0 and largest == int(wc.max())


def test_batched_tuned_graph_and_sequential(batch):
    P, start, boxes, (wc, wl) = batch
    b = nb.BatchedList()
    b.setup(start, boxes, RC, MAXN)
    pts = torch.tensor(P, device="cuda")
    cnt, lst = b.outputs()
    leaf, block = b.tune(pts, cnt, lst)
    assert (leaf, block) == b.config() and block in (512, 1024)
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        b.capture(pts, cnt, lst, stream)
        for _ in range(2):
            cnt.fill_(-1)
            b.replay(stream)
        stream.synchronize()
    c, l = _rows(cnt, lst)
    assert np.array_equal(c, wc) and np.array_equal(l, wl)
    # one plain call per system: entries are system-local ids
    cnt2, lst2 = b.outputs()
    b.sequential_plain(nb.LBVH(), nb.LBVHTraverser(), pts, RC, cnt2, lst2)
    torch.cuda.synchronize()
    c2, l2 = _rows(cnt2, lst2)
    assert np.array_equal(c2, wc)
    sys_of = np.repeat(np.arange(len(start) - 1), np.diff(start))
    local = np.where(l2 == 0xFFFFFFFF, l2, l2 + start[sys_of][:, None])
    assert np.array_equal(local, wl)


def test_batched_matches_oracle_cell_list(batch):
    P, start, boxes, (wc, wl) = batch
    rng = np.random.default_rng(6)
    for s in rng.choice(len(start) - 1, 4, replace=False):
        o, e = int(start[s]), int(start[s + 1])
        L = float(boxes[s][0])
        if L < 4 * RC:
            continue
        off, nbrs = O.celllist_csr(P[o:e], P[o:e], RC, [0, 0, 0], [L, L, L])
        assert np.array_equal(np.diff(off).astype(np.uint32), wc[o:e])
        for r in range(e - o):
            got = np.sort(wl[o + r, : wc[o + r]] - o)
            assert np.array_equal(got, nbrs[off[r]:off[r + 1]])


def test_batched_rejects_oversized_system():
    b = nb.BatchedList()
    with pytest.raises(nb.NeighborError):
        b.setup([0, nb.BATCH_MAX_N + 1], [[30.0, 30.0, 30.0]], RC, MAXN)
