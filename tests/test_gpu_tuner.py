"""The single-system autotuner: a valid configuration, cached per workload class, and the same
lists whatever it picks.

nbr_tune_self times the two-pass step (build, count, host read, fill) for every leaf size, sort
digit width and climb block on the caller's points and applies the fastest; a second call for a
workload of the same class reuses the cached choice without timing.  Lists must be bit-identical
under the tuned and the default configuration.
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


def _lists(lbvh, trav, P, L, rc):
    box = [L, L, L]
    pad = nb.exact_pad(rc, 2 * L)
    lbvh.build(P, [0, 0, 0], box)
    trav.traverse_self(lbvh, rc, box, pad, images="periodic", rows_sorted=True)
    mx = trav.count_summary()[0]
    cnt, lst = trav.traverse_self(lbvh, rc, box, pad, images="periodic", rows_sorted=True, max_neigh=mx)
    c = cnt.cpu().numpy().view(np.uint32)
    rows = lst.cpu().numpy().view(np.uint32)
    mask = np.arange(mx)[None, :] < c[:, None]
    return c, np.where(mask, rows, 0xFFFFFFFF), lbvh.primitives().cpu().numpy()


def test_tuned_configuration_changes_nothing_but_speed():
    N, rc = 300_000, 1.3
    L = float((N / 0.85) ** (1.0 / 3.0))
    g = torch.Generator(device="cuda")
    g.manual_seed(3)
    P = torch.rand((N, 3), generator=g, device="cuda") * L
    pad = nb.exact_pad(rc, 2 * L)
    nb.tune_self_clear()
    base = _lists(nb.LBVH(), nb.LBVHTraverser(), P, L, rc)
    lbvh, trav = nb.LBVH(), nb.LBVHTraverser()
    cfg = nb.tune_self(lbvh, trav, P, [0, 0, 0], [L, L, L], rc, [L, L, L], pad, reps=1)
    assert cfg["leaf_size"] in (1, 2, 4, 8) and cfg["radix_bits"] in (8, 10) and cfg["climb_block"] in (256, 512)
    assert cfg["ms"] > 0
    tuned = _lists(lbvh, trav, P, L, rc)
    for a, b in zip(base, tuned):
        assert np.array_equal(a, b)
    # the same class (another frame of the same size and density) is taken from the cache
    lbvh2 = nb.LBVH()
    again = nb.tune_self(lbvh2, nb.LBVHTraverser(), P * 0.999, [0, 0, 0], [L, L, L], rc, [L, L, L], pad)
    assert again["ms"] == 0 and {k: again[k] for k in ("leaf_size", "radix_bits", "climb_block")} == \
        {k: cfg[k] for k in ("leaf_size", "radix_bits", "climb_block")}
    nb.tune_self_clear()
    assert nb.tune_self(lbvh2, nb.LBVHTraverser(), P, [0, 0, 0], [L, L, L], rc, [L, L, L], pad, reps=1)["ms"] > 0
