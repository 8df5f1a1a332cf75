"""User-written ops compiled against the C++ headers, as the reference's callers write them.

tests/cpp/user_ops.cu is built with nvcc against include/neighbor/neighbor.h -- no C ABI -- and
drives LBVH::build and LBVHTraverser::traverse with its own ops:

- the reference test's three-point sequence (test/lbvh_test.cu:17-315): two streams, the tree
  getters, getData()'s 10-bit nodes, CountNeighborsOp, NeighborListOp with max_neigh 2 and a
  MapTransformOp -- compared with the reference test's own values (tests/golden);
- the double-precision ParticleInsertOp / ParticleQueryOp of the reference's benchmark
  (benchmark/lbvh_benchmark.cuh:25-92) with 27 double3 images, a user exact query and a user
  output op (count, sum of ids, nearest other particle) -- compared with a float64 brute force
  that applies the same minimum-image predicate;
- the same particles through the library's double self queries (PointInsertOpF64 and
  LBVHTraverser::traverseSelfF64, count, readCountSummary, fill) -- the same brute force.
"""
import json
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "user_ops.cu")
BIN = os.path.join(ROOT, "tests", "cpp", "_build", "user_ops")


@pytest.fixture(scope="module")
def user_ops():
    os.makedirs(os.path.dirname(BIN), exist_ok=True)
    nvcc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    subprocess.run([nvcc if os.path.exists(nvcc) else "nvcc", "-std=c++17", "-O2",
                    "-gencode", "arch=compute_103a,code=sm_103a", "-I", os.path.join(ROOT, "include"),
                    "-o", BIN, SRC], check=True)
    return BIN


def test_three_point_sequence_through_the_templates(user_ops, kats, tmp_path):
    out = tmp_path / "kat.json"
    subprocess.run([user_ops, "kat", str(out)], check=True, timeout=120)
    got = json.loads(out.read_text())
    k = kats["three_point"]
    for b in got["builds"]:   # one build per stream
        assert b["N"] == k["N"] and b["root"] == k["root"]
        assert b["parents"] == k["parents"]
        assert b["left"] == k["left"] and b["right"] == k["right"]
        assert b["primitives"] == k["primitives"]
        for node, v in k["lo_x"].items():
            assert abs(b["lo_x"][int(node)] - v) <= k["box_tol"]
        for node, v in k["hi_x"].items():
            assert abs(b["hi_x"][int(node)] - v) <= k["box_tol"]
    nodes = k["nodes_x_bins"]
    assert got["hits"] == k["hits"]
    assert got["lo_x_bin"] == nodes["lo_x_bin"] and got["hi_x_bin"] == nodes["hi_x_bin"]
    assert got["node_z"] == nodes["z"] and got["node_w"] == nodes["w"]
    m = k["max_neigh"]

    def rows_of(res):
        return [res["list"][m * i: m * i + min(n, m)] for i, n in enumerate(res["nneigh"])]
    for res in got["nlists"]:   # one list per stream
        assert res["nneigh"] == k["nlist"]["nneigh"]
        assert rows_of(res) == k["nlist"]["rows"]
    assert got["mapped"]["nneigh"] == k["nlist_mapped"]["nneigh"]
    assert rows_of(got["mapped"]) == k["nlist_mapped"]["rows"]


def _brute(P, L, r):
    """Count, id sum and nearest other particle per query: float64, the user op's predicate."""
    h = 0.5 * L

    def comp(a):
        d = a[None, :] - a[:, None]
        return np.where(d >= h, d - L, np.where(d < -h, d + L, d))
    dx, dy, dz = comp(P[:, 0]), comp(P[:, 1]), comp(P[:, 2])
    d2 = (dx * dx + dy * dy) + dz * dz
    hit = d2 <= r * r
    n = len(P)
    ids = np.arange(n, dtype=np.uint64)
    count = hit.sum(1).astype(np.uint32)
    idsum = (hit * ids[None, :]).sum(1).astype(np.uint64)
    d2o = np.where(hit & ~np.eye(n, dtype=bool), d2, np.inf)
    nearest = np.where(np.isfinite(d2o.min(1)), d2o.argmin(1), -1).astype(np.int32)
    return count, idsum, nearest


@pytest.mark.parametrize("n,L,r", [(3000, 14.0, 1.1), (2500, 6.0, 2.6), (5000, 16.0, 1.3)])
def test_double_particle_ops_and_user_output_op(user_ops, tmp_path, n, L, r):
    rng = np.random.default_rng(n)
    P = np.zeros((n, 4))
    P[:, :3] = rng.random((n, 3)) * L
    P[:, 3] = rng.integers(0, 3, n)
    src = tmp_path / "particles.f64"
    P.tofile(src)
    prefix = str(tmp_path / "out")
    subprocess.run([user_ops, "ops", str(src), str(n), repr(L), repr(r), prefix], check=True, timeout=120)
    superset = np.fromfile(prefix + ".superset", np.uint32)
    count = np.fromfile(prefix + ".count", np.uint32)
    idsum = np.fromfile(prefix + ".idsum", np.uint64)
    nearest = np.fromfile(prefix + ".nearest", np.int32)
    want_count, want_idsum, want_nearest = _brute(P[:, :3], L, r)
    assert np.array_equal(count, want_count)
    assert np.array_equal(idsum, want_idsum)
    assert np.array_equal(nearest, want_nearest)
    # the stock-style particle query (refine() == true) returns a superset of the exact set
    assert np.all(superset >= count) and superset.sum() > count.sum()
    # the same particles as the library's double self queries from C++ (traverseSelfF64, two
    # passes; above 4,096 points the symmetric double walk): the exact sets by particle index
    assert np.array_equal(np.fromfile(prefix + ".self_count", np.uint32), want_count)
    assert np.array_equal(np.fromfile(prefix + ".self_idsum", np.uint64), want_idsum)
