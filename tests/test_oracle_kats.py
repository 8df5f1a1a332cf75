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


def fp32_disagreement_bound(pi, pj, rc, L):
    """Largest |r - rc| at which the FP32 minimum-image predicate may decide a pair differently
    from FP64: 1 ulp(rc), plus, for every axis on which the pair wraps, half an ulp of the FP32
    difference pj - pi that is rounded before the wrap subtracts L (about L)."""
    rc = np.float32(rc)
    d = np.abs(np.asarray(pj, np.float32) - np.asarray(pi, np.float32))
    Lf = np.asarray(L, np.float32)
    wraps = (Lf > 0) & (d >= np.float32(0.5) * Lf)
    extra = np.sqrt(np.sum(np.where(wraps, (0.5 * np.spacing(np.maximum(d, 1e-30).astype(np.float32))) ** 2, 0.0),
                           axis=-1))
    return float(np.spacing(rc)) + extra


def test_fp64_disagreements_within_one_ulp():
    # Pairs where FP32 and FP64 decide differently must lie within 1 ulp of rc (plus the rounding
    # of a wrapped difference for pairs across the periodic boundary).
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
                assert abs(d) < fp32_disagreement_bound(P[i], P[j], rc, [L, L, L]), (i, j, d)
    assert n_flag < 5


def test_fp32_predicate_disagrees_with_fp64_only_within_one_ulp():
    # Adversarial pairs: distances within 3 ulp of rc in random directions, coordinates up to
    # 270 (the benchmark's box).  The FP32 predicate's operation order (d = pj - pi, squares,
    # ((dx*dx + dy*dy) + dz*dz) <= rc*rc, all rounded to nearest) must agree with the exact
    # FP64 distance on every pair farther than 1 ulp(rc) from the cutoff.
    rng = np.random.default_rng(17)
    rc = np.float32(1.3)
    rc2 = np.float32(rc * rc)
    ulp = np.float64(np.spacing(rc))
    n_dis = 0
    for L in (12.0, 270.25):
        pi = (rng.random((400000, 3)) * L).astype(np.float32)
        u = rng.normal(size=pi.shape)
        u /= np.linalg.norm(u, axis=1, keepdims=True)
        r = np.float64(rc) + rng.uniform(-3, 3, len(pi)) * ulp
        pj = (pi.astype(np.float64) + u * r[:, None]).astype(np.float32)
        d = pj - pi
        f32 = ((d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]) <= rc2
        rd = np.sqrt(((pj.astype(np.float64) - pi.astype(np.float64)) ** 2).sum(1))
        dis = f32 != (rd <= np.float64(rc))
        n_dis += int(dis.sum())
        assert np.all(np.abs(rd[dis] - np.float64(rc)) < ulp)
    assert n_dis > 1000   # the pairs do reach the cutoff's rounding


@pytest.mark.parametrize("L", [12.0, 33.78, 270.25])
def test_wrapped_pairs_disagree_within_the_wrap_bound(L):
    # Pairs across the periodic boundary: the FP32 difference pj - pi (up to about L) is rounded
    # before the wrap, so FP32 and FP64 (with the same FP32 box length) may differ by up to half
    # an ulp of it per wrapped axis on top of 1 ulp(rc) -- and no further.
    rng = np.random.default_rng(int(L * 100))
    rc = np.float32(1.3)
    rc2 = np.float32(rc * rc)
    Lf = np.float32(L)
    h = np.float32(0.5) * Lf
    n = 300000
    pi = (rng.random((n, 3)) * L).astype(np.float32)
    pi[:, 0] = (rng.random(n) * 1.3).astype(np.float32)   # next to the x = 0 face
    u = rng.normal(size=(n, 3))
    u[:, 0] = -np.abs(u[:, 0]) - 0.3                     # partners across it
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    r = np.float64(rc) + rng.uniform(-300, 300, n) * np.spacing(rc)
    pj = np.mod(pi.astype(np.float64) + u * r[:, None], np.float64(Lf)).astype(np.float32)
    pj = np.where(pj >= Lf, np.float32(0), pj)
    d = pj - pi
    d = np.where(d >= h, d - Lf, np.where(d < -h, d + Lf, d))
    f32 = ((d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]) <= rc2
    dd = pj.astype(np.float64) - pi.astype(np.float64)
    dd -= np.float64(Lf) * np.round(dd / np.float64(Lf))
    rd = np.sqrt((dd * dd).sum(1))
    dis = f32 != (rd <= np.float64(rc))
    assert dis.sum() > 100
    bound = fp32_disagreement_bound(pi[dis], pj[dis], rc, [L, L, L])
    assert np.all(np.abs(rd[dis] - np.float64(rc)) < bound)
