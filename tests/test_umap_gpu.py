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
    """Instances in one batched job reach the local structure they reach alone: mean 15-NN
    preservation of three batched runs within 0.01 of three runs alone. Float atomics (Hogwild)
    make every run differ; single runs of the 3,000-point instance spread over about 0.008, so
    single pairs can differ by twice that while the means of three stay well inside 0.01."""
    knns, inits = [], []
    for j, n in enumerate([3000, 12000, 5000]):
        x, _ = synthetic.mixture(n, 20, 6, 300 + j, centre_sd=3.0)
        knns.append(synthetic.exact_knn_numpy(x, 15))
        inits.append(_pca_init(x, 400 + j))
    keeps = [np.arange(0, idx.shape[0], 2, dtype=np.int32) for idx, _ in knns]
    pb = np.zeros(len(knns))
    for _ in range(3):
        lays = api.umap_knn_batch(knns, inits, n_epochs=200)
        for j, ((idx, dist), lay) in enumerate(zip(knns, lays)):
            assert np.all(np.isfinite(lay)) and np.abs(lay).max() <= 16.0
            pb[j] += O.knn_preservation(lay, idx, keep=keeps[j], preserve_k=15) / 3
    for j, ((idx, dist), y0) in enumerate(zip(knns, inits)):
        pa = np.mean([O.knn_preservation(api.umap_knn(idx, dist, y0, n_epochs=200).layout, idx, keep=keeps[j],
                                         preserve_k=15) for _ in range(3)])
        assert abs(pa - pb[j]) < 0.01, (idx.shape[0], pa, pb[j])


def test_batched_umap_column_major_entry_matches_rows_entry():
    """The concatenated column-major batch entry and the per-instance row-major one run the same
    job: mean 15-NN preservation of two runs each within 0.01 per instance (Hogwild runs differ)."""
    import ctypes as C

    knns, inits = [], []
    for j, n in enumerate([4000, 9000]):
        x, _ = synthetic.mixture(n, 20, 6, 320 + j, centre_sd=3.0)
        knns.append(synthetic.exact_knn_numpy(x, 15))
        inits.append(_pca_init(x, 420 + j))
    sizes = np.array([i.shape[0] for i, _ in knns], np.int32)
    idx, dist = api._concat_knn(knns)
    y0 = np.concatenate([y.ravel() for y in inits]).astype(np.float32)
    lib = _lib.require_gpu()
    keeps = [np.arange(0, s_, 2, dtype=np.int32) for s_ in sizes]
    pc, pr = np.zeros(2), np.zeros(2)
    for _ in range(2):
        out = np.zeros((int(sizes.sum()), 2), np.float32)
        _lib.check(lib.fastembedr_cuda_umap_batch_from_knn(2, sizes.ctypes.data, idx.ctypes.data, dist.ctypes.data,
                                                           y0.ctypes.data, 15, 0, 200, 5, 1.0, 0.01, 1.0, 42,
                                                           out.ctypes.data, C.byref(C.c_float())), "column-major batch")
        cm = np.split(out, np.cumsum(sizes)[:-1])
        rows = api.umap_knn_batch(knns, inits, n_epochs=200)
        for j, (i, _) in enumerate(knns):
            pc[j] += O.knn_preservation(cm[j], i, keep=keeps[j], preserve_k=15) / 2
            pr[j] += O.knn_preservation(rows[j], i, keep=keeps[j], preserve_k=15) / 2
    assert np.all(np.abs(pc - pr) < 0.01), (pc, pr)


def test_batched_umap_rejects_an_invalid_instance():
    """The batch checks every instance's KNN before its SGD: an out-of-range index or a negative
    distance in any one instance fails the whole call with the single-instance message."""
    knns, inits = [], []
    for j, n in enumerate([800, 1200, 900]):
        x, _ = synthetic.mixture(n, 10, 4, 340 + j, centre_sd=3.0)
        knns.append(synthetic.exact_knn_numpy(x, 15))
        inits.append(_pca_init(x, 440 + j))
    idx, dist = knns[1][0].copy(), knns[1][1].copy()
    idx[7, 3] = idx.shape[0] + 5
    with pytest.raises(_lib.CudaEmbeddingError, match="out of range"):
        api.umap_knn_batch([knns[0], (idx, knns[1][1]), knns[2]], inits, n_epochs=5)
    dist[11, 2] = -1.0
    with pytest.raises(_lib.CudaEmbeddingError, match="finite and non-negative"):
        api.umap_knn_batch([knns[0], (knns[1][0], dist), knns[2]], inits, n_epochs=5)
    lays = api.umap_knn_batch(knns, inits, n_epochs=5)
    assert all(np.all(np.isfinite(y)) for y in lays)


@pytest.mark.parametrize("tag", ["3k", "200"])
def test_diffusion_start_matches_reference_golden(golden, tag):
    """fastembedr_cuda_spectral_init_from_knn against the reference's CPU statement of its GPU
    diffusion start (golden), and against the oracle on this build's own graph."""
    g = golden("umap_diffusion")
    idx, dist = g["idx_" + tag], g["dist_" + tag]
    iters, seed = int(g["iters_" + tag]), int(g["seed_" + tag])
    got = api.umap_spectral_init(idx, dist, iters, seed)
    want = g["init_" + tag]
    scale = np.abs(want).max()
    # graph weights agree with the reference builder to 2e-6; averaging keeps that size
    assert np.abs(got - want).max() <= 2e-5 * scale
    gr = api.umap_graph(idx, dist)
    orc = O.umap_diffusion_init(gr["offsets"], gr["neighbors"], gr["weights"], iters, seed)
    # same graph: rows are summed exactly as the restatement; only the whitening moments are
    # reduced in another order
    assert np.abs(got - orc).max() <= 1e-6 * scale
    y = got.astype(np.float64)
    assert np.abs(y.mean(0)).max() < 1e-6
    assert np.linalg.norm(y[:, 0]) == pytest.approx(1.0, rel=1e-5)
    assert np.linalg.norm(y[:, 1]) == pytest.approx(1.0, rel=1e-5)
    assert abs(y[:, 0] @ y[:, 1]) < 1e-5


def test_fused_umap_entry_points_match_reference_cpu_sgd():
    """The three fused entry points (host double, host float, device float KNN) run graph ->
    diffusion start -> SGD on the GPU; from the same start the reference CPU SGD reaches the
    same 15-NN preservation within 0.015."""
    x, _ = synthetic.mixture(20000, 30, 12, 44, centre_sd=3.0, lognormal_sizes=True, anisotropic=True)
    idx, dist = synthetic.exact_knn_numpy(x, 15)
    n, k = idx.shape
    rounds, epochs = 30, 200
    start = api.umap_spectral_init(idx, dist, rounds, 42)
    off, nb, w, e, mw = O.umap_graph(idx, dist)
    a, b = api.umap_ab_params(0.01)
    emb = np.ascontiguousarray(start.T.astype(np.float64)).ravel().copy()
    O.orc().orc_umap_sgd_serial(n, off, nb, w, emb, epochs, a, b, 5, 1.0, 1.0, 42)
    cpu = emb.reshape(2, n).T.astype(np.float32)
    keep = np.arange(0, n, 4, dtype=np.int32)
    pc = O.knn_preservation(cpu, idx, keep=keep, preserve_k=15)
    p0 = O.knn_preservation(start, idx, keep=keep, preserve_k=15)
    lib = _lib.require_gpu()
    icm = np.asfortranarray(idx.astype(np.int32))
    outs = {}
    for tag, dcm in (("double", np.asfortranarray(dist.astype(np.float64))),
                     ("float", np.asfortranarray(dist.astype(np.float32)))):
        out = np.zeros((n, 2), np.float32)
        fn = lib.fastembedr_cuda_umap_from_knn_spectral if tag == "double" else \
            lib.fastembedr_cuda_umap_from_knn_spectral_float
        st = fn(icm.ctypes.data, dcm.ctypes.data, n, k, epochs, 5, 1.0, a, b, 1.0, rounds, 42, 0, 0, out.ctypes.data)
        _lib.check(st, "fused UMAP " + tag)
        outs[tag] = out
    outs["device"] = api.umap_knn(idx, dist, init="diffusion", n_epochs=epochs, spectral_n_iter=rounds, seed=42).layout
    # the reference starts SGD from the whitened start itself (coordinates ~1/sqrt(n)), so the
    # first epochs scatter the layout; both sides do the same
    for tag, y in outs.items():
        assert np.all(np.isfinite(y)) and np.abs(y).max() <= 16.0, tag
        pg = O.knn_preservation(y, idx, keep=keep, preserve_k=15)
        assert abs(pg - pc) < 0.015, (tag, pg, pc, p0)
    binary = api.umap_knn(idx, dist, init="diffusion", n_epochs=epochs, spectral_n_iter=rounds, seed=42,
                          graph_mode="binary").layout
    assert np.all(np.isfinite(binary)) and np.abs(binary).max() <= 16.0


def test_fused_umap_rejects_invalid_arguments():
    x, _ = synthetic.mixture(500, 8, 3, 45, centre_sd=3.0)
    idx, dist = synthetic.exact_knn_numpy(x, 10)
    lib = _lib.require_gpu()
    icm = np.asfortranarray(idx.astype(np.int32))
    dcm = np.asfortranarray(dist.astype(np.float32))
    out = np.zeros((500, 2), np.float32)
    assert lib.fastembedr_cuda_umap_from_knn_spectral_float(icm.ctypes.data, dcm.ctypes.data, 500, 10, 0, 5, 1.0, 1.9,
                                                            0.8, 1.0, 10, 1, 0, 0, out.ctypes.data) != 0
    assert b"invalid fused CUDA UMAP" in lib.fastembedr_cuda_embedding_last_error()
    assert lib.fastembedr_cuda_umap_from_knn_spectral_float(icm.ctypes.data, dcm.ctypes.data, 500, 10, 10, 5, 1.0,
                                                            1.9, 0.8, 1.0, 10, 1, 0, 1, out.ctypes.data) != 0
    assert b"optimizer_mode" in lib.fastembedr_cuda_embedding_last_error()
    with pytest.raises(_lib.CudaEmbeddingError, match="invalid spectral initialization"):
        api.umap_spectral_init(idx, dist, 0)


@pytest.mark.parametrize("tag", ["3k", "40"])
def test_spectral_start_matches_reference_golden(golden, tag):
    """The reference CPU spectral start (spectral_knn_init(backend = "cpu")) computed on the GPU:
    against the reference's own output, and against the oracle on this build's graph."""
    g = golden("umap_spectral")
    idx, dist = g["idx_" + tag], g["dist_" + tag]
    iters, seed = int(g["iters_" + tag]), int(g["seed_" + tag])
    want = g["start_" + tag]
    # on the reference's own graph (the oracle's, bit-identical to it) the GPU start differs from
    # the reference only by the order of the FP64 sums over points. The start is ill-conditioned
    # in the graph (a 1e-7 relative change of the weights moves the 3k start by 0.7 on its scale
    # of 10), so it is compared on the same graph, not on this build's graph (weights within 2e-6)
    off, nb, w, _, _ = O.umap_graph(idx, dist)
    on_ref_graph = api.umap_spectral_start_csr(off, nb, w, iters, seed)
    assert np.abs(on_ref_graph - want).max() <= 1e-4, np.abs(on_ref_graph - want).max()
    # the KNN entry point builds the graph on the GPU: against the oracle on that graph
    got = api.umap_spectral_start(idx, dist, iters, seed)
    gr = api.umap_graph(idx, dist)
    orc = O.umap_spectral_init(gr["offsets"], gr["neighbors"], gr["weights"], iters, seed)
    assert np.abs(got - orc).max() <= 1e-4, np.abs(got - orc).max()
    if tag == "40":
        scaled = api.umap_spectral_start_csr(off, nb, w, 5, 9, init_scale=2.0)
        assert np.abs(scaled - g["start_40_scaled"]).max() <= 1e-4
        assert np.std(scaled, axis=0, ddof=1) == pytest.approx([2.0, 2.0], rel=1e-9)


def test_spectral_start_redraws_vanished_columns_like_the_reference(golden):
    """A graph whose operator has rank 6 (a weighted 6-ring and 34 isolated points): after every
    multiply the block's later columns vanish in Gram-Schmidt and are redrawn from the random
    stream, so the start depends on each redraw landing where the reference's does."""
    g = golden("umap_spectral")
    got = api.umap_spectral_start_csr(g["iso_offsets"], g["iso_neighbors"], g["iso_weights"], 4, 11)
    assert np.abs(got - g["start_iso"]).max() <= 1e-6, np.abs(got - g["start_iso"]).max()


def test_spectral_start_matches_oracle_20k():
    x, _ = synthetic.mixture(20000, 30, 12, 46, centre_sd=3.0, lognormal_sizes=True, anisotropic=True)
    idx, dist = synthetic.exact_knn_numpy(x, 15)
    got = api.umap_spectral_start(idx, dist, 30, 7)
    gr = api.umap_graph(idx, dist)
    orc = O.umap_spectral_init(gr["offsets"], gr["neighbors"], gr["weights"], 30, 7)
    assert np.abs(got - orc).max() <= 1e-4, np.abs(got - orc).max()
    assert np.abs(got).max() == pytest.approx(10.0, abs=1e-3)


def test_umap_knn_with_gpu_spectral_start_matches_reference_cpu():
    """umap_knn's default path (graph -> spectral start -> SGD, all on the GPU) against the
    reference CPU SGD from the same start: 15-NN preservation within 0.01."""
    x, _ = synthetic.mixture(20000, 30, 12, 47, centre_sd=3.0, lognormal_sizes=True, anisotropic=True)
    idx, dist = synthetic.exact_knn_numpy(x, 15)
    n = idx.shape[0]
    off, nb, w, e, mw = O.umap_graph(idx, dist)
    start = api.umap_spectral_start(idx, dist, 30, 42)  # deterministic: the start umap_knn computes
    a, b = O.umap_ab(0.01)
    emb = np.ascontiguousarray(start.T).ravel().copy()
    O.orc().orc_umap_sgd_serial(n, off, nb, w, emb, 200, a, b, 5, 1.0, 1.0, 42)
    cpu = emb.reshape(2, n).T.astype(np.float32)
    fit = api.umap_knn(idx, dist, n_epochs=200, seed=42)
    assert fit.config["init_backend"] == "cuda_spectral_csr" and fit.config["spectral_n_iter"] == 30
    keep = np.arange(0, n, 4, dtype=np.int32)
    pc = O.knn_preservation(cpu, idx, keep=keep, preserve_k=15)
    pg = O.knn_preservation(fit.layout, idx, keep=keep, preserve_k=15)
    p0 = O.knn_preservation(start.astype(np.float32), idx, keep=keep, preserve_k=15)
    assert np.all(np.isfinite(fit.layout)) and np.abs(fit.layout).max() <= 16.0
    assert abs(pg - pc) < 0.01, (pg, pc)
    assert pg > p0 + 0.02, (pg, p0)


def test_sgd_preservation_matches_reference_cpu_at_100k_500_epochs():
    """The plain umap_knn workload at full size (100,000 x 50 mixture of 20 log-normal clusters,
    exact k = 15 KNN, 500 epochs, the package's spectral start): 15-NN preservation of the GPU
    layout within 0.01 of the reference CPU SGD on the same graph and start. At this size the
    package runs the reference's multi-threaded SGD branch (min(4, cores) workers), restated in
    the oracle."""
    import os

    import torch

    x, _ = synthetic.plain_umap_100k()
    i_t, d_t = synthetic.exact_knn_torch(x, 15, device="cuda")
    idx = np.asfortranarray(i_t.cpu().numpy())
    dist = np.asfortranarray(d_t.cpu().numpy())
    del i_t, d_t
    torch.cuda.empty_cache()
    n = idx.shape[0]
    rounds = api.umap_spectral_n_iter(n, 15)
    init = np.ascontiguousarray(api.umap_spectral_start(idx, dist, rounds, 42).astype(np.float32))
    fit = api.umap_knn(idx, dist, init, n_epochs=500)
    off, nb, w, e, mw = O.umap_graph(np.ascontiguousarray(idx), np.ascontiguousarray(dist))
    a, b = O.umap_ab(0.01)
    emb = np.ascontiguousarray(init.T.astype(np.float64)).ravel().copy()
    workers = max(1, min(4, os.cpu_count() or 1))
    if workers > 1:
        O.orc().orc_umap_sgd_threaded(n, off, nb, w, emb, 500, a, b, 5, 1.0, 1.0, 42, workers)
    else:
        O.orc().orc_umap_sgd_serial(n, off, nb, w, emb, 500, a, b, 5, 1.0, 1.0, 42)
    cpu = emb.reshape(2, n).T.astype(np.float32)
    keep = np.arange(0, n, 10, dtype=np.int32)
    pc = O.knn_preservation(cpu, np.ascontiguousarray(idx), keep=keep, preserve_k=15)
    pg = O.knn_preservation(fit.layout, np.ascontiguousarray(idx), keep=keep, preserve_k=15)
    p0 = O.knn_preservation(init, np.ascontiguousarray(idx), keep=keep, preserve_k=15)
    assert np.all(np.isfinite(fit.layout)) and np.abs(fit.layout).max() <= 16.0
    # at this size both layouts keep ~1.3 % of the 15-NN (heavily overlapping clusters), so the
    # absolute bar is complemented by a relative one, and the optimisation must beat its start.
    # CPU runs with different seeds agree to +-0.0002; the GPU's Hogwild epochs (every edge of an
    # epoch in flight at once, updates by atomics, as in the reference's GPU kernel) have kept
    # 0.85-0.92 of the CPU's preservation in repeated runs, hence the 20 % relative bar.
    assert abs(pg - pc) < 0.01, (pg, pc)
    assert abs(pg - pc) <= 0.20 * pc, (pg, pc)
    assert pg > 2.0 * p0, (pg, p0)
