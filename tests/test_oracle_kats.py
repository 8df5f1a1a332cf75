"""Pin the CPU oracle against the reference's own known-answer tests.

Every value checked here comes from tests/golden/reference_kats.json, which records the
assertions of test/lbvh_test.cu and test/approx_math_test.cu (mphowardlab/neighbor v0.3.2).
"""
import numpy as np
import pytest

import oracle as O


def _f32(x):
    return float(np.float32(x))


def test_approx_math_kats(kats):
    # test/approx_math_test.cu:88-132
    for name, args, rel, thr in kats["approx_math"]["cases"]:
        if name.startswith("double2float"):
            v = O.rounding(name, *args)
            t = _f32(thr)
        else:
            v = O.rounding(name, *[_f32(a) for a in args])
            # division and reciprocal compare against the double 1/3 in the reference
            t = thr if name.startswith(("fdiv", "frcp")) else _f32(thr)
        ok = {"eq": v == t, "lt": v < t, "le": v <= t, "gt": v > t, "ge": v >= t}[rel]
        assert ok, (name, args, rel, thr, v)


def test_three_point_tree(kats):
    # test/lbvh_test.cu:61-117
    k = kats["three_point"]
    T = O.build_tree(k["points"], k["scene_lo"], k["scene_hi"])
    assert T["N"] == k["N"]
    assert T["parent"].tolist() == k["parents"]
    assert T["left"].tolist() == k["left"]
    assert T["right"].tolist() == k["right"]
    assert T["primitive"].tolist() == k["primitives"]
    for node, v in k["lo_x"].items():
        assert abs(T["lo"][int(node), 0] - v) <= k["box_tol"]
    for node, v in k["hi_x"].items():
        assert abs(T["hi"][int(node), 0] - v) <= k["box_tol"]


def test_three_point_compressed_nodes_and_hits(kats):
    # test/lbvh_test.cu:120-199
    k = kats["three_point"]
    T = O.build_tree(k["points"], k["scene_lo"], k["scene_hi"])
    comp = O.compress_ref10(T)
    d = comp[0]
    nb = k["nodes_x_bins"]
    assert (((d[:, 0].view(np.uint32) >> 20) & 0x3FF).tolist()) == nb["lo_x_bin"]
    assert (((d[:, 1].view(np.uint32) >> 20) & 0x3FF).tolist()) == nb["hi_x_bin"]
    assert d[:, 2].tolist() == nb["z"]
    assert d[:, 3].tolist() == nb["w"]
    assert O.traverse_ref10(comp, k["spheres"]).tolist() == k["hits"]


@pytest.mark.parametrize("mapped", [False, True])
def test_three_point_neighbor_list(kats, mapped):
    # test/lbvh_test.cu:202-312
    k = kats["three_point"]
    T = O.build_tree(k["points"], k["scene_lo"], k["scene_hi"])
    comp = O.compress_ref10(T, mapping=k["map"] if mapped else None)
    nn, lst = O.traverse_ref10(comp, k["spheres"], max_neigh=k["max_neigh"])
    exp = k["nlist_mapped"] if mapped else k["nlist"]
    assert nn.tolist() == exp["nneigh"]
    for q, row in enumerate(exp["rows"]):
        assert lst[q, : len(row)].tolist() == row


def test_periodic(kats):
    # test/lbvh_test.cu:318-388
    k = kats["periodic"]
    T = O.build_tree(k["points"], k["scene_lo"], k["scene_hi"])
    comp = O.compress_ref10(T)
    assert O.traverse_ref10(comp, k["spheres"]).tolist() == k["hits_self"]
    imgs = O.images27([k["image_step"]] * 3)
    assert O.traverse_ref10(comp, k["spheres"], images=imgs).tolist() == k["hits_images"]


def test_small(kats):
    # test/lbvh_test.cu:506-582
    k = kats["small"]
    T = O.build_tree(k["points"], k["scene_lo"], k["scene_hi"])
    assert T["parent"].tolist() == k["parents"]
    assert T["primitive"].tolist() == k["primitives"]
    assert len(T["left"]) == 0 and len(T["right"]) == 0
    comp = O.compress_ref10(T)
    assert comp[0][0, 2] == k["node0_z"] and comp[0][0, 3] == k["node0_w"]
    assert O.traverse_ref10(comp, k["spheres"]).tolist() == k["hits"]


def test_validate_superset_and_exact(kats):
    # test/lbvh_test.cu:391-503: the stock query is a superset of brute force; the exact
    # query equals it; the cell list equals it.
    k = kats["validate"]
    L = np.asarray(k["L"], np.float32)
    P = O.gen_validate_points(k["N"], L, k["seed"])
    fx = np.load(O.os.path.join(O.HERE, "..", "tests", "golden", "validate_points.npy"))
    assert np.array_equal(P, fx), "libstdc++ mt19937/uniform_real_distribution drift"
    T = O.build_tree(P, -0.5 * L, 0.5 * L)
    comp = O.compress_ref10(T)
    sph = np.concatenate([P, np.full((len(P), 1), k["rcut"], np.float32)], 1)
    imgs = O.images27(L)
    ref = O.brute_count(P, k["rcut"], P, L)
    hits = O.traverse_ref10(comp, sph, images=imgs)
    assert (hits >= ref).all()
    pad = O.exact_pad(k["rcut"], float(np.abs(P).max() + L.max()))
    ex = O.traverse_ref10(comp, sph, images=imgs, query=O.QUERY_EXACT, points=P, box_L=L, pad=pad)
    assert np.array_equal(ex, ref)
    cl, _ = O.celllist_counts(P, P, k["rcut"], -0.5 * L, L)
    assert np.array_equal(cl, ref)
    import json
    with open(O.os.path.join(O.HERE, "..", "tests", "golden", "validate_fixture.json")) as f:
        fx = json.load(f)
    assert int(ref.sum()) == fx["pairs"]
    w = (ref.astype(np.uint64) * np.arange(1, len(ref) + 1, dtype=np.uint64)).sum()
    assert int(w) == fx["weighted_checksum"]


def test_fp64_disagreements_within_one_ulp():
    # Pairs where FP32 and FP64 decide differently must lie within ~1 ulp of rc.
    rng = np.random.default_rng(7)
    L = np.float32(12.0)
    P = (rng.random((3000, 3)) * L).astype(np.float32)
    rc = np.float32(1.3)
    off, nb = O.celllist_csr(P, P, rc, [0, 0, 0], [L, L, L])
    n_flag = 0
    for i in range(0, len(P), 97):
        s = set(nb[off[i]:off[i + 1]].tolist())
        for j in range(len(P)):
            d = O.pair_distance_minus_rc_f64(P[i], P[j], rc, [L, L, L])
            if (d <= 0) != (j in s):
                n_flag += 1
                assert abs(d) < 4 * np.spacing(rc), (i, j, d)
    assert n_flag < 5
