"""Host-side fault injection and the capacity model's weights file.

A failed device allocation must come back as NBR_ERR_ALLOC (the reference throws for it,
include/neighbor/Memory.h:182-186) and leave the handle usable.  The failure is injected on the
host (the allocator call is replaced by a refusal); nothing faults the GPU.  The weights file must
round-trip a trained model and be refused when damaged.
"""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

import neighbor_gb300 as nb  # noqa: E402
import oracle as O  # noqa: E402

NBR_ERR_INVALID = 1
NBR_ERR_ALLOC = 3


@pytest.fixture(scope="module", autouse=True)
def _lib():
    nb.build()
    nb.load()
    yield
    nb.inject_alloc_failures(0)


def _points(N, seed=3):
    rng = np.random.default_rng(seed)
    L = float((N / 0.85) ** (1.0 / 3.0))
    return (rng.random((N, 3)) * L).astype(np.float32), L


def test_failed_allocation_in_build_is_reported_and_recoverable():
    P, L = _points(20000)
    lbvh = nb.LBVH()
    nb.inject_alloc_failures(1)
    with pytest.raises(nb.NeighborError) as e:
        lbvh.build(torch.tensor(P, device="cuda"), [0, 0, 0], [L, L, L])
    assert e.value.code == NBR_ERR_ALLOC
    nb.inject_alloc_failures(0)
    lbvh.build(torch.tensor(P, device="cuda"), [0, 0, 0], [L, L, L])
    lbvh.check_status()
    trav = nb.LBVHTraverser()
    rc = 1.3
    cnt = trav.traverse_self(lbvh, rc, [L, L, L], nb.exact_pad(rc, 2 * L), images="periodic", rows_sorted=False)
    want, _ = O.celllist_counts(P, P, rc, [0, 0, 0], [L, L, L])
    assert np.array_equal(cnt.cpu().numpy().view(np.uint32), want)


def test_failed_allocation_in_traversal_is_reported_and_recoverable():
    P, L = _points(15000, seed=4)
    lbvh = nb.LBVH()
    lbvh.build(torch.tensor(P, device="cuda"), [0, 0, 0], [L, L, L])
    rc = 1.3
    pad = nb.exact_pad(rc, 2 * L)
    trav = nb.LBVHTraverser()
    trav.force_symmetric()       # the symmetric count, which allocates work buffers
    nb.inject_alloc_failures(1)   # the count's first work buffer
    with pytest.raises(nb.NeighborError) as e:
        trav.traverse_self(lbvh, rc, [L, L, L], pad, images="periodic")
    assert e.value.code == NBR_ERR_ALLOC
    nb.inject_alloc_failures(0)
    cnt = trav.traverse_self(lbvh, rc, [L, L, L], pad, images="periodic")
    mx = int(cnt.max().item())
    c2, lst = trav.traverse_self(lbvh, rc, [L, L, L], pad, images="periodic", max_neigh=mx)
    assert torch.equal(c2, cnt)
    want, _ = O.celllist_counts(P, P, rc, [0, 0, 0], [L, L, L])
    prim = lbvh.primitives().cpu().numpy().view(np.uint32)
    assert np.array_equal(cnt.cpu().numpy().view(np.uint32), want[prim])


def test_model_file_round_trip_and_damage(tmp_path):
    P, L = _points(30000, seed=5)
    lbvh = nb.LBVH()
    lbvh.build(torch.tensor(P, device="cuda"), [0, 0, 0], [L, L, L])
    rc = 1.3
    a = nb.CapacityModel(seed=21)
    rng = np.random.default_rng(22)
    a.set_params(a.params() + (rng.normal(size=nb.CAP_PARAMS) * 0.05).astype(np.float32))
    a.margins = [0.1 * k for k in range(nb.CAP_MARGIN_BINS)]
    path = str(tmp_path / "capacity.nbrcap")
    a.save(path)
    b = nb.CapacityModel(seed=99)
    b.load(path)
    assert np.array_equal(a.params(), b.params())
    assert np.allclose(a.margins, b.margins)
    ca = a.predict(lbvh, [0, 0, 0], [L, L, L], rc, cap_max=4096)
    cb = b.predict(lbvh, [0, 0, 0], [L, L, L], rc, cap_max=4096)
    assert torch.equal(ca, cb)
    raw = bytearray(open(path, "rb").read())
    # one flipped byte in the parameters: the hash no longer matches
    bad = bytearray(raw)
    bad[100] ^= 0x40
    open(path, "wb").write(bytes(bad))
    with pytest.raises(nb.NeighborError) as e:
        b.load(path)
    assert e.value.code == NBR_ERR_INVALID
    # a truncated file and a foreign one
    for data in (bytes(raw[:-9]), b"NOTAMODEL" + bytes(raw[9:])):
        open(path, "wb").write(data)
        with pytest.raises(nb.NeighborError) as e:
            b.load(path)
        assert e.value.code == NBR_ERR_INVALID
    with pytest.raises(nb.NeighborError):
        b.load(os.path.join(str(tmp_path), "missing.nbrcap"))
    # the failed loads left the loaded parameters in place
    assert np.array_equal(a.params(), b.params())
