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
