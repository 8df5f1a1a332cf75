"""Learned capacity network, CSR lists and one-pass lists on the GPU, against the CPU oracle.

* Features: occupancy grid and the 32 features of every point equal the oracle's restatement.
* Gradients: the GPU forward/backward kernel's summed gradient and loss of a batch match the
  oracle's (same BF16 rounding points, FP32; tolerance 1e-3 relative, from summation order).
* Inference: the fused mma.sync kernel's outputs match the oracle's forward (tolerance in the
  test: FP32 accumulation order and the BF16 rounding of hidden activations can move an output
  by a few 1e-3).
* One-pass lists are exact: every row equals the plain two-pass list's row, including rows that
  overflowed their capacity and were re-run.
* The trained network is worth having: with the same number of list slots as its predictions use,
  one constant capacity overflows many more rows than the learned capacities.
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


def _t(a, dtype=torch.float32):
    return torch.tensor(np.asarray(a), dtype=dtype, device="cuda")


def _clustered(N, seed, density=0.85, blobs_per=2000):
    """70% of the points in Gaussian blobs (sigma log-uniform in [0.5, 3]), 30% uniform."""
    rng = np.random.default_rng(seed)
    L = float((N / density) ** (1.0 / 3.0))
    nb_ = max(1, N // blobs_per)
    centers = rng.random((nb_, 3)) * L
    sig = np.exp(rng.uniform(np.log(0.5), np.log(3.0), nb_))
    n_blob = N * 7 // 10
    k = rng.integers(0, nb_, n_blob)
    p = np.empty((N, 3))
    p[:n_blob] = centers[k] + rng.normal(size=(n_blob, 3)) * sig[k, None]
    p[n_blob:] = rng.random((N - n_blob, 3)) * L
    return np.mod(p, L).astype(np.float32), L


def _tree(P, L, leaf=4):
    lbvh = nb.LBVH(leaf_size=leaf)
    lbvh.build(_t(P), [0, 0, 0], [L, L, L])
    return lbvh


def _plain_rows(lbvh, rc, L, rows_sorted=True):
    trav = nb.LBVHTraverser()
    pad = nb.exact_pad(rc, 2 * L)
    cnt = trav.traverse_self(lbvh, rc, [L, L, L], pad, images="periodic", rows_sorted=rows_sorted)
    mx = int(cnt.max().item())
    cnt2, lst = trav.traverse_self(lbvh, rc, [L, L, L], pad, images="periodic", rows_sorted=rows_sorted,
                                   max_neigh=mx)
    assert torch.equal(cnt, cnt2)
    return cnt.cpu().numpy().view(np.uint32), lst.cpu().numpy().view(np.uint32)


def _csr_equals_rows(res, cnt, lst):
    nn = res["nneigh"].cpu().numpy().view(np.uint32)
    off = res["offsets"].cpu().numpy().astype(np.int64)
    flat = res["list"].cpu().numpy().view(np.uint32)
    assert np.array_equal(nn, cnt)
    for r in range(len(cnt)):
        assert np.array_equal(flat[off[r]:off[r] + cnt[r]], lst[r, :cnt[r]]), r


@pytest.mark.parametrize("periodic", [True, False])
def test_features_match_oracle(periodic):
    P, L = _clustered(60000, 1)
    lbvh = _tree(P, L)
    rc = 1.0
    model = nb.CapacityModel()
    got = model.features(lbvh, [0, 0, 0], [L, L, L], rc, periodic=periodic).cpu().numpy()
    shift = nb.CapacityModel.level(rc, [0, 0, 0], [L, L, L])
    codes = lbvh.codes().cpu().numpy().view(np.uint32)
    pts = lbvh.fast()["points"].cpu().numpy()
    want = O.cap_features(codes, pts, [0, 0, 0], [L, L, L], shift, periodic)
    np.testing.assert_allclose(got, want, rtol=2e-7, atol=2e-7)
    assert got[:, :27].max() > 2.0  # dense cells present


def test_gradient_matches_oracle():
    P, L = _clustered(40000, 2)
    lbvh = _tree(P, L)
    rc = 1.0
    cnt, _ = _plain_rows(lbvh, rc, L)
    model = nb.CapacityModel(seed=5)
    F = model.features(lbvh, [0, 0, 0], [L, L, L], rc)
    T = nb.CapacityModel.targets(_t(cnt.view(np.int32), torch.int32))
    rng = np.random.default_rng(3)
    params = model.params() + (rng.normal(size=nb.CAP_PARAMS) * 0.05).astype(np.float32)
    model.set_params(params)
    for batch, offset, stride in [(1000, 17, 7919), (777, 39000, 1)]:
        g, loss = model.gradient(F, T, batch, offset, stride)
        torch.cuda.synchronize()
        gw, lw, _ = O.cap_forward_backward(model.params(), F.cpu().numpy(), T.cpu().numpy(), batch, offset,
                                           stride, mode=1)
        g = g.cpu().numpy().astype(np.float64)
        rel = np.linalg.norm(g - gw) / np.linalg.norm(gw)
        assert rel < 1e-3, rel
        assert abs(loss.item() - lw) <= 1e-4 * abs(lw)


def test_inference_matches_oracle_forward():
    P, L = _clustered(50000, 4)
    lbvh = _tree(P, L)
    rc = 1.0
    model = nb.CapacityModel(seed=9)
    rng = np.random.default_rng(10)
    model.set_params(model.params() + (rng.normal(size=nb.CAP_PARAMS) * 0.05).astype(np.float32))
    model.margin = 0.25
    caps, y = model.predict(lbvh, [0, 0, 0], [L, L, L], rc, rows_sorted=True, cap_max=4096, want_y=True)
    F = model.features(lbvh, [0, 0, 0], [L, L, L], rc).cpu().numpy()
    N = len(P)
    _, _, yw = O.cap_forward_backward(model.params(), F, np.zeros(N, np.float32), N, 0, 1, mode=1)
    y = y.cpu().numpy()
    d = np.abs(y - yw)
    assert d.max() < 0.05 and d.mean() < 2e-3, (d.max(), d.mean())
    c = caps.cpu().numpy().view(np.uint32)
    want = np.clip(np.ceil(np.expm1(y.astype(np.float64) + np.float32(0.25))), 1, 4096)
    assert np.mean(c == want) > 0.999


def test_csr_two_pass_equals_stride_lists():
    P, L = _clustered(50000, 6)
    lbvh = _tree(P, L)
    rc = 1.0
    cnt, lst = _plain_rows(lbvh, rc, L)
    op = nb.OnePassList()
    caps = _t(cnt.view(np.int32), torch.int32)
    offsets, total = op.scan(caps)
    assert total == int(cnt.sum())
    flat = torch.full((total,), -1, dtype=torch.int32, device="cuda")
    trav = nb.LBVHTraverser()
    trav.force_symmetric()
    pad = nb.exact_pad(rc, 2 * L)
    for max_capacity in (int(cnt.max()), 0):  # symmetric kernels, then the whole-tree walk
        flat.fill_(-1)
        nn = trav.traverse_self_csr(lbvh, rc, [L, L, L], pad, offsets, caps, flat, max_capacity=max_capacity,
                                    images="periodic")
        res = dict(nneigh=nn, offsets=offsets, list=flat)
        _csr_equals_rows(res, cnt, lst)


@pytest.mark.parametrize("symmetric", [False, True])
@pytest.mark.parametrize("rows_sorted", [True, False])
def test_one_pass_with_small_capacities_is_exact(rows_sorted, symmetric):
    P, L = _clustered(30000, 7)
    lbvh = _tree(P, L)
    rc = 1.0
    cnt, lst = _plain_rows(lbvh, rc, L, rows_sorted=rows_sorted)
    op = nb.OnePassList()
    caps = op.capacity(len(P))
    caps.fill_(3)  # most rows overflow and are re-run
    trav = nb.LBVHTraverser()
    if symmetric:
        trav.force_symmetric()
    st = op.build(trav, lbvh, rc, [L, L, L], nb.exact_pad(rc, 2 * L), rows_sorted=rows_sorted, cap_max=4096)
    assert st["overflow_rows"] == int((cnt > 3).sum())
    res = op.result(len(P))
    assert res["total"] == st["slots"] + st["overflow_slots"]
    _csr_equals_rows(res, cnt, lst)


def test_trained_capacities_are_exact_and_beat_a_constant_capacity():
    rc = 1.0
    # training frames: seeds distinct from the evaluation frame
    model = nb.CapacityModel(seed=11)
    feats, targs = [], []
    for seed in (101, 102):
        P, L = _clustered(150000, seed)
        lbvh = _tree(P, L)
        cnt, _ = _plain_rows(lbvh, rc, L)
        feats.append(model.features(lbvh, [0, 0, 0], [L, L, L], rc))
        targs.append(nb.CapacityModel.targets(_t(cnt.view(np.int32), torch.int32)))
    F = torch.cat(feats)
    T = torch.cat(targs)
    model.margin = 0.0
    first = model.train(F, T, steps=1, batch=8192, lr=3e-3, seed=1)
    last = model.train(F, T, steps=600, batch=8192, lr=3e-3, seed=2)
    assert last < 0.25 * first, (first, last)
    # margin: the 99th percentile of the training residuals
    model.margin = 0.0
    resid = []
    for seed in (101, 102):
        P, L = _clustered(150000, seed)
        lbvh = _tree(P, L)
        cnt, _ = _plain_rows(lbvh, rc, L)
        _, y = model.predict(lbvh, [0, 0, 0], [L, L, L], rc, want_y=True)
        resid.append(np.log1p(cnt.astype(np.float64)) - y.cpu().numpy())
    model.margin = float(np.quantile(np.concatenate(resid), 0.99))
    # evaluation frame
    P, L = _clustered(150000, 200)
    lbvh = _tree(P, L)
    cnt, lst = _plain_rows(lbvh, rc, L)
    N = len(P)
    trav = nb.LBVHTraverser()
    pad = nb.exact_pad(rc, 2 * L)
    op = nb.OnePassList()
    model.predict(lbvh, [0, 0, 0], [L, L, L], rc, cap_max=4096, caps=op.capacity(N))
    learned = op.build(trav, lbvh, rc, [L, L, L], pad, cap_max=4096)
    _csr_equals_rows(op.result(N), cnt, lst)
    # the method without the network: one capacity for every row, same number of slots
    const = max(1, learned["slots"] // N)
    op2 = nb.OnePassList()
    op2.capacity(N).fill_(const)
    plain = op2.build(trav, lbvh, rc, [L, L, L], pad, cap_max=4096)
    _csr_equals_rows(op2.result(N), cnt, lst)
    assert plain["slots"] <= learned["slots"]
    assert learned["overflow_rows"] * 5 < plain["overflow_rows"], (learned, plain)
    assert learned["overflow_rows"] < 0.05 * N


@pytest.mark.parametrize("rows_sorted", [True, False])
def test_learned_step_in_one_call_matches_separate_calls(rows_sorted):
    # the one-call form predicts on a second stream from the end of the sort on; capacities,
    # counts and every row must equal those of build + predict + one-pass fill done in sequence
    P, L = _clustered(80000, 12)
    rc = 1.0
    box = [L, L, L]
    pad = nb.exact_pad(rc, 2 * L)
    model = nb.CapacityModel(seed=13)
    rng = np.random.default_rng(14)
    model.set_params(model.params() + (rng.normal(size=nb.CAP_PARAMS) * 0.05).astype(np.float32))
    model.margin = 0.3
    N = len(P)
    trav = nb.LBVHTraverser()
    trav.force_symmetric()   # the path of large trees (the symmetric CSR fill)
    lbvh = _tree(P, L)
    op_a = nb.OnePassList()
    model.predict(lbvh, [0, 0, 0], box, rc, rows_sorted=rows_sorted, cap_max=32, caps=op_a.capacity(N))
    st_a = op_a.build(trav, lbvh, rc, box, pad, rows_sorted=rows_sorted, cap_max=32)
    lbvh_b = nb.LBVH(leaf_size=4)
    op_b = nb.OnePassList()
    for _ in range(2):  # twice: the second call reuses the side stream and buffers
        st_b = op_b.build_learned(model, trav, lbvh_b, _t(P), [0, 0, 0], box, rc, box, pad,
                                  rows_sorted=rows_sorted, cap_max=32)
        assert st_b == st_a
        a, b = op_a.result(N), op_b.result(N)
        assert torch.equal(a["nneigh"], b["nneigh"])
        assert torch.equal(a["offsets"], b["offsets"])
        assert torch.equal(a["caps"], b["caps"])
        cnt, lst = _plain_rows(lbvh, rc, L, rows_sorted=rows_sorted)
        _csr_equals_rows(b, cnt, lst)


def test_csr_fill_work_order_does_not_change_results():
    P, L = _clustered(50000, 16)
    lbvh = _tree(P, L)
    rc = 1.0
    box = [L, L, L]
    pad = nb.exact_pad(rc, 2 * L)
    op = nb.OnePassList()
    out = []
    for ordered in (False, True):
        trav = nb.LBVHTraverser()
        trav.set_work_order(ordered)
        cnt = trav.traverse_self(lbvh, rc, box, pad, images="periodic", rows_sorted=False)
        mx = int(cnt.max().item())
        assert mx > 32  # rows too long for the symmetric fill: the whole-tree walk fills them
        offsets, total = op.scan(cnt)
        lst = torch.full((total + 1,), -1, dtype=torch.int32, device="cuda")
        nn = trav.traverse_self_csr(lbvh, rc, box, pad, offsets, cnt, lst, max_capacity=mx,
                                    images="periodic", rows_sorted=False)
        out.append((nn.cpu().numpy(), lst.cpu().numpy()))
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])


@pytest.mark.parametrize("rows_sorted", [True, False])
def test_subset_rows_equal_full_traversal(rows_sorted):
    P, L = _clustered(40000, 21)
    lbvh = _tree(P, L)
    rc = 1.0
    box = [L, L, L]
    pad = nb.exact_pad(rc, 2 * L)
    trav = nb.LBVHTraverser()
    cnt = trav.traverse_self(lbvh, rc, box, pad, images="periodic", rows_sorted=rows_sorted)
    op = nb.OnePassList()
    offsets, total = op.scan(cnt)
    full = torch.full((total + 1,), -1, dtype=torch.int32, device="cuda")
    nn_full = trav.traverse_self_csr(lbvh, rc, box, pad, offsets, cnt, full, max_capacity=int(cnt.max().item()),
                                     images="periodic", rows_sorted=rows_sorted)
    rng = np.random.default_rng(3)
    sub = np.sort(rng.choice(len(P), 3000, replace=False)).astype(np.int32)
    sub = np.concatenate([sub, np.arange(0, len(P), 997, dtype=np.int32)])
    part = torch.full((total + 1,), -1, dtype=torch.int32, device="cuda")
    nn = trav.traverse_self_subset_csr(lbvh, rc, box, pad, torch.tensor(sub, device="cuda"), offsets, cnt, part,
                                       images="periodic", rows_sorted=rows_sorted)
    prim = lbvh.primitives().cpu().numpy()
    rows = sub if rows_sorted else prim[sub]
    off = offsets.cpu().numpy()
    c = cnt.cpu().numpy()
    f = full.cpu().numpy()
    p = part.cpu().numpy()
    got = nn.cpu().numpy()
    assert np.array_equal(got[rows], nn_full.cpu().numpy()[rows])
    for r in rows:
        assert np.array_equal(p[off[r]:off[r] + c[r]], f[off[r]:off[r] + c[r]])


def test_margin_table_bins_outputs():
    # each row's capacity uses the margin of its output's bin (bins of 0.5, the last open)
    P, L = _clustered(40000, 31)
    lbvh = _tree(P, L)
    rc = 1.0
    model = nb.CapacityModel(seed=11)
    table = [0.05 * k for k in range(nb.CAP_MARGIN_BINS)]
    model.margins = table
    assert np.allclose(model.margins, table)
    assert model.margin == pytest.approx(max(table))
    caps, y = model.predict(lbvh, [0, 0, 0], [L, L, L], rc, cap_max=4096, want_y=True)
    yv = y.cpu().numpy().astype(np.float32)
    b = np.clip(np.floor(yv * np.float32(2.0)), 0, nb.CAP_MARGIN_BINS - 1).astype(int)
    m = np.asarray(table, np.float32)[b]
    want = np.clip(np.ceil(np.expm1((yv + m).astype(np.float64))), 1, 4096)
    assert np.mean(caps.cpu().numpy().view(np.uint32) == want) > 0.999
    # calibration: residuals of a bin land in that bin's margin
    t = torch.tensor((yv + 0.1 + (b >= 4) * 0.5).astype(np.float32), device="cuda")
    got = model.calibrate(t, y, quantile=0.5, min_rows=1)
    for k in range(nb.CAP_MARGIN_BINS):
        if np.any(b == k):
            assert got[k] == pytest.approx(0.1 + (0.5 if k >= 4 else 0.0), abs=1e-3)
