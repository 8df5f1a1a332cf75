"""Two-species (polydisperse) neighbor lists: one tree per species, every (query species, tree)
pair with cutoff (d_i + d_j) / 2 + skin, equal to the oracle's cell list.

This is the workload of a colloid mixture (small and large spheres): the cross-species pairs use
per-query cutoffs through ExactSphereQueryOp, the same-species pairs the self traversal.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

import neighbor_gb300 as nb  # noqa: E402
import oracle as O  # noqa: E402
import bench  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _lib():
    nb.build()
    nb.load()


def test_two_species_lists_match_cell_list():
    n_small, n_large = 60_000, 60
    L = float(((n_small * np.pi / 6.0 + n_large * np.pi / 6.0 * 1000.0) / 0.2) ** (1.0 / 3.0))
    species = bench.polydisperse_frame(n_small, n_large, L, 5)
    trees = [nb.LBVH(), nb.LBVH()]
    travs = [nb.LBVHTraverser() for _ in range(4)]
    streams = [torch.cuda.Stream() for _ in range(4)]
    out = bench.polydisperse_step(nb, trees, travs, species, L, streams=streams)
    torch.cuda.synchronize()
    for (i, j), (cnt, lst, R) in out.items():
        qp = species[i].cpu().numpy()
        tp = species[j].cpu().numpy()
        off, nbrs = O.celllist_csr(qp, tp, R, [0, 0, 0], [L, L, L])
        c = cnt.cpu().numpy().view(np.uint32)
        assert np.array_equal(c, np.diff(off).astype(np.uint32)), (i, j)
        lst = lst.cpu().numpy().view(np.uint32)
        for r in range(0, len(qp), max(1, len(qp) // 500)):
            assert np.array_equal(np.sort(lst[r, : c[r]]), nbrs[off[r]:off[r + 1]]), (i, j, r)
    # the large-from-small pair lists many neighbors per query
    assert int(out[(1, 0)][0].max().item()) > 50
