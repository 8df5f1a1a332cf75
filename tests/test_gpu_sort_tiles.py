"""The build's radix sort runs on tiles of 256 x 4 keys below 2^20 keys and 256 x 16 keys above:
at sizes on either side of the switch and of tile edges, and on one LBVH reused across sizes (its
look-back words sized for the largest tile count any size up to its capacity needs), the sorted
codes are non-decreasing, equal codes keep their input order, and the order is a permutation.
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


def _check_sorted(lbvh, N):
    codes = lbvh.codes().cpu().numpy().view(np.uint32)[:N]
    prim = lbvh.primitives().cpu().numpy().view(np.uint32)[:N]
    assert np.all(codes[1:] >= codes[:-1])
    same = codes[1:] == codes[:-1]
    assert np.all(prim[1:][same] > prim[:-1][same])   # stable: input order among equal codes
    assert np.array_equal(np.sort(prim), np.arange(N, dtype=np.uint32))


@pytest.mark.parametrize("N", [2, 1023, 1024, 1025, 4097, 32768, (1 << 20) - 1, 1 << 20, (1 << 20) + 1])
def test_sort_either_side_of_the_tile_switch(N):
    rng = np.random.default_rng(N)
    L = 40.0
    # a coarse lattice with repeats: many equal codes test the stability
    P = (rng.integers(0, 200, (N, 3)) * (L / 200)).astype(np.float32)
    lbvh = nb.LBVH()
    lbvh.build(torch.tensor(P, device="cuda"), [0, 0, 0], [L, L, L])
    lbvh.check_status()
    _check_sorted(lbvh, N)


def test_one_tree_reused_across_sizes():
    rng = np.random.default_rng(3)
    L = 60.0
    lbvh = nb.LBVH()
    for N in (1_300_000, 900_000, (1 << 20) - 1, 70_000, 1 << 20, 5_000):
        P = (rng.random((N, 3)) * L).astype(np.float32)
        lbvh.build(torch.tensor(P, device="cuda"), [0, 0, 0], [L, L, L])
        lbvh.check_status()
        _check_sorted(lbvh, N)
        fresh = nb.LBVH()
        fresh.build(torch.tensor(P, device="cuda"), [0, 0, 0], [L, L, L])
        assert torch.equal(fresh.primitives()[:N], lbvh.primitives()[:N])
