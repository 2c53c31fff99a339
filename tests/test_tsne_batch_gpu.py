"""Batched t-SNE: many instances share every launch. Each instance must come out exactly as it
does alone (same kernels, per-instance grids, reductions and sort keys), and the batch must
reach the single-instance path's KL (within 1%) and local structure."""
import numpy as np
import pytest

import oracle as O
from fastembedr_gb300 import _lib, api, synthetic

pytestmark = pytest.mark.gpu


def _instances(sizes, k=30, seed=0):
    out = []
    for j, n in enumerate(sizes):
        x, _ = synthetic.mixture(n, 12, 4 + j % 5, seed + j, centre_sd=4.0)
        out.append(synthetic.exact_knn_numpy(x, k))
    return out


def test_each_instance_matches_itself_alone():
    """Per-instance grids, reductions and sort keys make an instance's arithmetic independent of
    its batch, and the charge sums are order-independent integers: every instance of a batch
    follows the bits of the same instance run alone, after one iteration and after a schedule."""
    knns = _instances([300, 2500, 9000, 21000, 700])
    with api.TsneBatch(knns, perplexity=10.0, seed=7) as b:
        info = b.info()
        b.iterate(1, 12.0, 1.0 / 12.0)
        one = b.layouts()
        b.run(early_exaggeration_iter=60, n_iter=240)
        after = b.layouts()
        kl_together = [b.kl(j) for j in range(len(knns))]
    assert info["grid_classes"] == 2 and info["points"] == 300 + 2500 + 9000 + 21000 + 700
    assert info["launches_per_iteration"] == 3 + 3 * 2
    for j, knn in enumerate(knns):
        with api.TsneBatch([knn], perplexity=10.0, seed=7) as a:
            a.iterate(1, 12.0, 1.0 / 12.0)
            alone = a.layouts()[0]
            a.run(early_exaggeration_iter=60, n_iter=240)
            alone_after = a.layouts()[0]
            kl_alone = a.kl(0)
        assert np.array_equal(one[j], alone), j
        assert np.array_equal(after[j], alone_after), j
        assert kl_together[j] == kl_alone


def test_mixed_label_bases_and_both_entry_points_agree():
    """Instances may carry 0- or 1-based labels independently (each is detected on the device);
    the concatenated column-major entry point and the per-instance row-major one give the same
    first iteration."""
    import ctypes as C

    knns = _instances([400, 1500, 3000], seed=3)
    mixed = [knns[0], (knns[1][0] + 1, knns[1][1]), knns[2]]
    with api.TsneBatch(knns, perplexity=10.0, seed=7) as a:
        a.iterate(1, 12.0, 1.0 / 12.0)
        base = a.layouts()
    with api.TsneBatch(mixed, perplexity=10.0, seed=7) as b:
        b.iterate(1, 12.0, 1.0 / 12.0)
        got = b.layouts()
    lib = _lib.require_gpu()
    sizes = np.array([i.shape[0] for i, _ in knns], np.int32)
    idx = np.concatenate([np.asfortranarray(i.astype(np.int32)).ravel(order="F") for i, _ in knns])
    dist = np.concatenate([np.asfortranarray(d.astype(np.float32)).ravel(order="F") for _, d in knns])
    h = C.c_void_p()
    _lib.check(lib.fastembedr_tsne_batch_create(3, sizes.ctypes.data, idx.ctypes.data, dist.ctypes.data, None, 30,
                                                10.0, 0, 0, 0, 7, C.byref(h)), "column-major batch")
    _lib.check(lib.fastembedr_tsne_batch_iterate(h, 1, 12.0, 1.0 / 12.0, 0.8, 0.01, 5.0), "iterate")
    out = np.zeros((int(sizes.sum()), 2), np.float32)
    _lib.check(lib.fastembedr_tsne_batch_layout(h, out.ctypes.data), "layout")
    lib.fastembedr_tsne_batch_destroy(h)
    cm = np.split(out, np.cumsum(sizes)[:-1])
    for j in range(3):
        scale = np.abs(base[j]).max()
        assert np.abs(got[j] - base[j]).max() <= 1e-5 * scale
        assert np.abs(cm[j] - base[j]).max() <= 1e-5 * scale


def test_batch_matches_single_instance_path():
    """Against tsne_knn (one instance per call): with the same start, grid policy and the opt-SNE
    rate rounded the same way, every instance of the batch returns tsne_knn's layout bit for bit,
    so KL and 15-NN preservation agree exactly (the KL is also checked against the oracle's)."""
    sizes = [4000, 6000, 8000, 12000]
    knns = _instances(sizes, k=90, seed=20)
    inits = [synthetic.tsne_init(n, seed=30 + j) for j, n in enumerate(sizes)]
    with api.TsneBatch(knns, perplexity=30.0, inits=inits) as b:
        b.run()
        lays = b.layouts()
        kls = [b.kl(j) for j in range(len(sizes))]
    for j, (idx, dist) in enumerate(knns):
        fit = api.tsne_knn(idx, dist, perplexity=30.0, Y_init=inits[j], n_iter=750)
        assert np.array_equal(lays[j], fit.layout), j
        rp, col, val, _ = O.tsne_csr(idx, dist, 30.0)
        assert abs(kls[j] - O.kl(rp, col, val, lays[j])) <= 1e-3 * kls[j]


def test_adaptive_grids_follow_the_layout_and_keep_the_kl():
    """The adaptive box count: at least 256 nodes, so instances below 20,000 points keep the CUDA
    size policy's grid (and its exact trajectory) while their spans stay below ~180; larger
    instances take the smallest grid with node spacing <= 0.7 over the current layout, at a KL no
    more than 1 % above the policy's."""
    sizes = [2000, 9000, 30000]
    knns = _instances(sizes, k=90, seed=50)
    inits = [synthetic.tsne_init(n, seed=60 + j) for j, n in enumerate(sizes)]
    kls, grids = {}, {}
    for policy in ("cuda", "adaptive"):
        with api.TsneBatch(knns, perplexity=30.0, inits=inits, grid_size=policy) as b:
            b.run(early_exaggeration_iter=250, n_iter=0)
            g_early, _ = b.grids()
            b.run(early_exaggeration_iter=0, n_iter=750)
            g_late, regrids = b.grids()
            lays = b.layouts()
            kls[policy] = np.array([b.kl(j) for j in range(len(sizes))])
            grids[policy] = (g_early, g_late)
        if policy == "adaptive":
            assert np.all(g_early == 256) and np.all(g_late >= g_early)
            for lay, g in zip(lays, g_late):
                ext = 1.1 * np.ptp(lay, 0).max()
                assert ext / (g - 1) <= 0.7 * 1.15 or g == 1024  # grown during the last chunk
    ka, kc = kls["adaptive"], kls["cuda"]
    same = (grids["adaptive"][1] == grids["cuda"][1]) & (grids["adaptive"][0] == grids["cuda"][0])
    assert same[0] and same[1], grids
    assert np.array_equal(ka[same], kc[same]), (ka, kc)
    assert np.all(ka <= 1.01 * kc), (ka, kc)


def test_invalid_batches_raise():
    knns = _instances([200, 300])
    with pytest.raises(ValueError):
        api.TsneBatch([])
    bad = [knns[0], (knns[1][0][:, :10], knns[1][1][:, :10])]
    with pytest.raises(ValueError, match="same number"):
        api.TsneBatch(bad)
    idx, dist = knns[0]
    oob = idx.copy()
    oob[0, 0] = 5000
    with pytest.raises(_lib.CudaEmbeddingError, match="out of range"):
        api.TsneBatch([(oob, dist)])
    # a bad instance after a good one fails the whole batch (checked once, before P is built)
    with pytest.raises(_lib.CudaEmbeddingError, match="out of range"):
        api.TsneBatch([knns[1], (oob, dist)])
    neg = dist.copy()
    neg[3, 2] = -1.0
    with pytest.raises(_lib.CudaEmbeddingError, match="finite and non-negative"):
        api.TsneBatch([knns[1], (idx, neg)])
    with api.TsneBatch(knns) as b:
        b.iterate(5, 12.0, 1.0 / 12.0)
        assert all(np.all(np.isfinite(y)) for y in b.layouts())
