"""Capacity inference on the fifth-generation tensor cores (k_cap_infer_tc) against the oracle.

The tcgen05 kernel takes 128 queries per MMA tile, accumulates in Tensor Memory and reads the
accumulators back with tcgen05.ld.  Its outputs must match the oracle's forward pass of the same
network with the same BF16 rounding points (tolerance in the tests: FP32 summation order and the
BF16 rounding of the first hidden layer can move an output by a few 1e-3), and the warp-tile
mma.sync kernel's outputs on the same trees, for sizes that do not fill the last 128-query tile,
for both row orders, and for periodic and open scenes.  Its status word stays clear.
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


def _points(N, seed, density=0.85, clustered=True):
    rng = np.random.default_rng(seed)
    L = float((N / density) ** (1.0 / 3.0))
    if not clustered:
        return (rng.random((N, 3)) * L).astype(np.float32), L
    nb_ = max(1, N // 2000)
    centers = rng.random((nb_, 3)) * L
    sig = np.exp(rng.uniform(np.log(0.5), np.log(3.0), nb_))
    n_blob = N * 7 // 10
    k = rng.integers(0, nb_, n_blob)
    p = np.empty((N, 3))
    p[:n_blob] = centers[k] + rng.normal(size=(n_blob, 3)) * sig[k, None]
    p[n_blob:] = rng.random((N - n_blob, 3)) * L
    return np.mod(p, L).astype(np.float32), L


def _model(seed):
    model = nb.CapacityModel(seed=seed)
    rng = np.random.default_rng(seed + 1)
    model.set_params(model.params() + (rng.normal(size=nb.CAP_PARAMS) * 0.05).astype(np.float32))
    model.margin = 0.25
    return model


def _predict(model, lbvh, L, rc, kernel, rows_sorted=True, periodic=True):
    model.infer_kernel = kernel
    assert model.infer_kernel == kernel
    caps, y = model.predict(lbvh, [0, 0, 0], [L, L, L], rc, periodic=periodic, rows_sorted=rows_sorted,
                            cap_max=4096, want_y=True)
    torch.cuda.synchronize()
    assert model.status() == 0
    return caps.cpu().numpy().view(np.uint32), y.cpu().numpy()


@pytest.mark.parametrize("periodic", [True, False])
@pytest.mark.parametrize("N", [2, 127, 128, 129, 5000, 50000])
def test_tc_inference_matches_oracle_forward(N, periodic):
    P, L = _points(N, 100 + N)
    lbvh = nb.LBVH(leaf_size=4)
    lbvh.build(_t(P), [0, 0, 0], [L, L, L])
    rc = 1.0
    model = _model(9)
    caps, y = _predict(model, lbvh, L, rc, nb.CAP_INFER_TENSOR_MEMORY, periodic=periodic)
    F = model.features(lbvh, [0, 0, 0], [L, L, L], rc, periodic=periodic).cpu().numpy()
    _, _, yw = O.cap_forward_backward(model.params(), F, np.zeros(N, np.float32), N, 0, 1, mode=1)
    d = np.abs(y - yw)
    assert d.max() < 0.05 and d.mean() < 2e-3, (d.max(), d.mean())
    want = np.clip(np.ceil(np.expm1(y.astype(np.float64) + np.float32(0.25))), 1, 4096)
    assert np.mean(caps == want) > 0.999


@pytest.mark.parametrize("rows_sorted", [True, False])
@pytest.mark.parametrize("clustered", [True, False])
def test_tc_matches_warp_tiles(rows_sorted, clustered):
    N = 300_001
    P, L = _points(N, 7, clustered=clustered)
    lbvh = nb.LBVH(leaf_size=4)
    lbvh.build(_t(P), [0, 0, 0], [L, L, L])
    model = _model(21)
    cw, yw = _predict(model, lbvh, L, 1.3, nb.CAP_INFER_WARP_TILES, rows_sorted=rows_sorted)
    ct, yt = _predict(model, lbvh, L, 1.3, nb.CAP_INFER_TENSOR_MEMORY, rows_sorted=rows_sorted)
    d = np.abs(yt - yw)
    assert d.max() < 0.02 and d.mean() < 1e-4, (d.max(), d.mean())
    assert np.mean(ct == cw) > 0.999
    # every row written (rows_sorted=False scatters through the primitive order)
    assert np.all(np.isfinite(yt))


def test_tc_is_the_one_pass_lists_capacity_source():
    # the one-pass list driven by the tensor-core prediction is exact (rows re-run on overflow)
    P, L = _points(40000, 3)
    lbvh = nb.LBVH(leaf_size=4)
    lbvh.build(_t(P), [0, 0, 0], [L, L, L])
    rc = 1.0
    model = _model(5)
    model.infer_kernel = nb.CAP_INFER_TENSOR_MEMORY
    trav = nb.LBVHTraverser()
    pad = nb.exact_pad(rc, 2 * L)
    cnt = trav.traverse_self(lbvh, rc, [L, L, L], pad, images="periodic",
                             rows_sorted=True).cpu().numpy().view(np.uint32)
    op = nb.OnePassList()
    model.margin = -0.5   # predictions a little short: some rows overflow and are re-run
    caps = model.predict(lbvh, [0, 0, 0], [L, L, L], rc, cap_max=4096, caps=op.capacity(len(P)))
    predicted = caps.cpu().numpy().view(np.uint32).copy()   # (the build rewrites overflowed rows)
    st = op.build(trav, lbvh, rc, [L, L, L], pad, cap_max=4096)
    res = op.result(len(P))
    assert np.array_equal(res["nneigh"].cpu().numpy().view(np.uint32), cnt)
    assert st["overflow_rows"] == int((cnt > predicted).sum()) > 0
    assert model.status() == 0


def test_infer_kernel_rejects_unknown_values():
    model = nb.CapacityModel(seed=1)
    with pytest.raises(Exception):
        model.infer_kernel = 7
