"""The benchmark's CPU baseline (oracle/frame_list.cpp) lists exactly the oracle's pairs.

The whole-frame host lister (grid, count, scan, fill on all host threads) must give every point
the neighbor set of the oracle's cell list -- the same FP32 minimum-image predicate -- and the
same total, independent of the number of threads; the host trajectory generator keeps points in
the box and moves them by about sigma.
"""
import numpy as np
import pytest

import oracle as O


@pytest.mark.parametrize("n,threads", [(1, 1), (50, 2), (30000, 0), (30000, 3)])
def test_frame_list_equals_cell_list(n, threads):
    L = float((n / 0.85) ** (1.0 / 3.0)) if n > 10 else 4.0
    P = O.uniform_points(n, [L, L, L], seed=11)
    fl = O.FrameLister(n, nthreads=threads, slots_per_point=2)   # small buffer: the list grows once
    total, used, secs = fl.run(P, [L, L, L], 1.3)
    assert used >= 1 and len(secs) == 4
    want, _ = O.celllist_counts(P, P, 1.3, [0, 0, 0], [L, L, L])
    assert total == int(want.astype(np.int64).sum())
    counts = np.empty(n, np.uint32)
    counts[fl.order] = fl.counts
    assert np.array_equal(counts, want)
    assert sorted(fl.order.tolist()) == list(range(n))
    off, nbrs = O.celllist_csr(P, P, 1.3, [0, 0, 0], [L, L, L])
    for k in range(0, n, max(1, n // 300)):
        i = fl.order[k]
        row = np.sort(fl.list[fl.offsets[k]:fl.offsets[k + 1]])
        assert np.array_equal(row, nbrs[off[i]:off[i + 1]])


def test_frame_list_noncubic_offset_box():
    rng = np.random.default_rng(3)
    lo = np.array([-4.0, 1.0, 7.0], np.float32)
    Lv = np.array([17.0, 11.5, 23.0], np.float32)
    P = (lo + rng.random((8000, 3)) * Lv).astype(np.float32)
    fl = O.FrameLister(len(P))
    total, _, _ = fl.run(P, Lv, 1.1, lo=lo)
    want, _ = O.celllist_counts(P, P, 1.1, lo, Lv)
    counts = np.empty(len(P), np.uint32)
    counts[fl.order] = fl.counts
    assert np.array_equal(counts, want) and total == int(want.sum())


def test_trajectory_generator():
    L = [20.0, 30.0, 25.0]
    P = O.uniform_points(100000, L, seed=5)
    assert P.min() >= 0 and np.all(P.max(axis=0) < np.array(L, np.float32))
    Q = O.gaussian_move(P, L, 0.05, seed=6)
    assert np.all(Q >= 0) and np.all(Q.max(axis=0) < np.array(L, np.float32))
    d = Q - P
    d -= np.round(d / np.array(L, np.float32)) * np.array(L, np.float32)
    assert abs(float(d.std()) - 0.05) < 0.002 and abs(float(d.mean())) < 0.001
    assert np.array_equal(O.gaussian_move(P, L, 0.05, seed=6), Q)   # deterministic
