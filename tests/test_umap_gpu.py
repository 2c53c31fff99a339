"""GPU parity of the UMAP path: fuzzy graph against the reference CPU builder (golden vectors),
the SGD epochs statistically against the reference CPU SGD on the same graph and init."""
import numpy as np
import pytest

import oracle as O
from fastembedr_gb300 import _lib, api, synthetic

pytestmark = pytest.mark.gpu


def test_fuzzy_graph_matches_reference_golden(golden):
    g = golden("umap_3k")
    out = api.umap_graph(g["idx"], g["dist"])
    np.testing.assert_array_equal(out["offsets"], g["offsets"])
    np.testing.assert_array_equal(out["neighbors"], g["neighbors"])
    w = g["weights"]
    assert np.abs(out["weights"] - w).max() <= 2e-6 * max(1.0, np.abs(w).max())
    np.testing.assert_allclose(out["epochs_per_sample"], g["epochs_per_sample"], rtol=1e-5)
    assert out["max_weight"] == pytest.approx(float(g["max_weight"]), rel=1e-6)


def test_fuzzy_graph_matches_oracle_20k():
    x, _ = synthetic.mixture(20000, 30, 12, 41, centre_sd=3.0, lognormal_sizes=True, anisotropic=True)
    idx, dist = synthetic.exact_knn_numpy(x, 15)
    out = api.umap_graph(idx, dist)
    off, nb, w, e, mw = O.umap_graph(idx, dist)
    np.testing.assert_array_equal(out["offsets"], off)
    np.testing.assert_array_equal(out["neighbors"], nb)
    assert np.abs(out["weights"] - w).max() < 2e-6


def _spread_init(n, seed):
    return np.random.default_rng(seed).uniform(-10, 10, (n, 2)).astype(np.float32)


def _pca_init(x, seed):
    """Data-derived start (the reference feeds a spectral/PCA layout scaled to [-10, 10] to every
    backend): top two principal components, scaled to max |y| = 10, plus a little jitter."""
    xc = x.astype(np.float64) - x.mean(0)
    _, _, vt = np.linalg.svd(xc[:: max(1, x.shape[0] // 4000)], full_matrices=False)
    y = xc @ vt[:2].T
    y *= 10.0 / np.abs(y).max()
    y += np.random.default_rng(seed).normal(0, 1e-4, y.shape)
    return y.astype(np.float32)


def test_sgd_preservation_matches_reference_cpu():
    """Same graph and init: 15-NN preservation of the GPU layout within 0.01 of the reference
    CPU SGD (serial branch of optimize_layout_csr)."""
    x, _ = synthetic.mixture(20000, 30, 12, 42, centre_sd=3.0, lognormal_sizes=True, anisotropic=True)
    idx, dist = synthetic.exact_knn_numpy(x, 15)
    n = idx.shape[0]
    init = _pca_init(x, 5)
    off, nb, w, e, mw = O.umap_graph(idx, dist)
    a, b = O.umap_ab(0.01)
    emb = np.ascontiguousarray(init.T.astype(np.float64)).ravel().copy()
    O.orc().orc_umap_sgd_serial(n, off, nb, w, emb, 200, a, b, 5, 1.0, 1.0, 42)
    cpu = emb.reshape(2, n).T.astype(np.float32)
    fit = api.umap_knn(idx, dist, init, n_epochs=200)
    keep = np.arange(0, n, 4, dtype=np.int32)
    pc = O.knn_preservation(cpu, idx, keep=keep, preserve_k=15)
    pg = O.knn_preservation(fit.layout, idx, keep=keep, preserve_k=15)
    assert np.all(np.isfinite(fit.layout)) and np.abs(fit.layout).max() <= 16.0
    p0 = O.knn_preservation(init, idx, keep=keep, preserve_k=15)
    assert abs(pg - pc) < 0.01, (pg, pc)
    assert pg > p0 + 0.02, (pg, p0)


def test_coo_entry_point_matches_graph_path():
    """The reference C ABI entry on the host-expanded COO graph and the all-GPU path agree
    statistically (same schedule, same Philox streams)."""
    x, _ = synthetic.mixture(8000, 20, 8, 43, centre_sd=3.0, lognormal_sizes=True, anisotropic=True)
    idx, dist = synthetic.exact_knn_numpy(x, 15)
    n = idx.shape[0]
    init = _spread_init(n, 6)
    g = api.umap_graph(idx, dist)
    heads = np.repeat(np.arange(n, dtype=np.int32), np.diff(g["offsets"]))
    a, b = O.umap_ab(0.01)
    y1 = api.umap_optimize_coo(heads, g["neighbors"], g["weights"], g["epochs_per_sample"], init, 200, a, b)
    y2 = api.umap_knn(idx, dist, init, n_epochs=200).layout
    keep = np.arange(0, n, 2, dtype=np.int32)
    p1 = O.knn_preservation(y1, idx, keep=keep)
    p2 = O.knn_preservation(y2, idx, keep=keep)
    assert abs(p1 - p2) < 0.01


def test_umap_invalid_parameters():
    h = np.array([0, 1], np.int32)
    with pytest.raises(_lib.CudaEmbeddingError, match="invalid"):
        api.umap_optimize_coo(h, h[::-1].copy(), np.ones(2), np.ones(2), np.zeros((2, 2)), 0, 1.9, 0.8)


def test_batched_umap_matches_each_instance_alone():
    """Instances in one batched job reach the local structure they reach alone (15-NN
    preservation within 0.01; float atomics make runs differ in rounding only)."""
    knns, inits, xs = [], [], []
    for j, n in enumerate([3000, 12000, 5000]):
        x, _ = synthetic.mixture(n, 20, 6, 300 + j, centre_sd=3.0)
        knns.append(synthetic.exact_knn_numpy(x, 15))
        inits.append(_pca_init(x, 400 + j))
    lays = api.umap_knn_batch(knns, inits, n_epochs=200)
    for (idx, dist), y0, lay in zip(knns, inits, lays):
        alone = api.umap_knn(idx, dist, y0, n_epochs=200).layout
        n = idx.shape[0]
        keep = np.arange(0, n, 2, dtype=np.int32)
        pa = O.knn_preservation(alone, idx, keep=keep, preserve_k=15)
        pb = O.knn_preservation(lay, idx, keep=keep, preserve_k=15)
        assert np.all(np.isfinite(lay)) and np.abs(lay).max() <= 16.0
        assert abs(pa - pb) < 0.01, (n, pa, pb)
