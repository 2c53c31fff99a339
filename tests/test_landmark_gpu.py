"""Landmark t-SNE transform (fastembedr_cuda_landmark_tsne_from_device_knn,
src/embedding_cuda_kernels.cpp:3572-3686): the affine start against a NumPy FP64 restatement of
landmark_affine_projection_kernel (:552-733), the iterations against the fixed-reference
transform from the same start, and the reference's argument checks."""
import numpy as np
import pytest

from fastembedr_gb300 import _lib, api

pytestmark = pytest.mark.gpu

EPS = 1.4901161193847656e-8


def _weighted_mean(L, refs, d, valid, rho, sigma):
    w = np.where(valid, np.exp(-np.maximum(0.0, d - rho) / max(sigma, EPS)), 0.0)
    s = w.sum()
    if not np.isfinite(s) or s <= 0:
        s = 1.0
    return (w[:, None] * L[np.where(valid, refs, 0)]).sum(0) / s


def affine_start(X, Q, L, idx, dist, off, m_req, ridge, max_ext):
    """Test-side restatement of the landmark affine start in float64."""
    nq, k = idx.shape
    n_ref = L.shape[0]
    m = max(3, min(m_req, min(k, 12)))
    out = np.zeros((nq, 2))
    for i in range(nq):
        refs = idx[i].astype(np.int64) - off
        d = dist[i].astype(np.float64)
        inr = (refs >= 0) & (refs < n_ref)
        valid = inr & np.isfinite(d) & (d >= 0)
        rho = d[valid].min() if valid.any() else 0.0
        zero = np.where(valid & (d <= EPS))[0]
        if len(zero):
            out[i] = L[refs[zero[0]]]
            continue
        exc = np.where(valid, np.maximum(0.0, d - rho), np.inf)
        pos = np.sort(exc[np.isfinite(exc) & (exc > EPS)])
        sigma = np.median(pos) if len(pos) else max(rho, EPS)
        if not np.isfinite(sigma) or sigma < EPS:
            sigma = EPS
        r, vm, im = refs[:m], valid[:m], inr[:m]
        ex = np.where(vm, np.maximum(0.0, d[:m] - rho), np.inf)
        w = np.where(im & np.isfinite(ex), np.exp(-ex / sigma), 0.0)
        if not np.isfinite(w.sum()) or w.sum() <= 0:
            out[i] = _weighted_mean(L, refs, d, valid, rho, sigma)
            continue
        w = w / w.sum()
        sw = np.sqrt(w)
        rc = np.where(im, r, 0)
        Lr = np.where(im[:, None], L[rc], 0.0)
        cy = (w[:, None] * Lr).sum(0)
        U = np.where(im[:, None], Lr - cy, 0.0)
        rhs = sw[:, None] * U
        radius2 = (U ** 2).sum(1).max()
        Xr = np.where(im[:, None], X[rc].astype(np.float64), 0.0)
        xc = (w[:, None] * Xr).sum(0)
        C = np.where(im[:, None], Xr - xc, 0.0)
        qc = Q[i].astype(np.float64) - xc
        G = (C @ C.T) * np.outer(sw, sw)
        qv = (C @ qc) * sw
        trace = (w * (C ** 2).sum(1)).sum()
        G += (ridge * max(trace, EPS) + EPS) * np.eye(m)
        Lc = np.zeros_like(G)
        ok = True
        for j in range(m):
            dg = G[j, j] - (Lc[j, :j] ** 2).sum()
            if not np.isfinite(dg) or dg <= EPS:
                ok = False
                break
            Lc[j, j] = np.sqrt(dg)
            for t in range(j + 1, m):
                Lc[t, j] = (G[t, j] - (Lc[t, :j] * Lc[j, :j]).sum()) / Lc[j, j]
        if ok:
            z = np.linalg.solve(Lc.T, np.linalg.solve(Lc, rhs))
            disp = qv @ z
            cap = max_ext * np.sqrt(max(radius2, EPS))
            nd = np.sqrt((disp ** 2).sum())
            if nd * nd > cap * cap:
                disp = disp * cap / (nd + EPS)
            start = cy + disp
            ok = np.all(np.isfinite(start))
        out[i] = start if ok else _weighted_mean(L, refs, d, valid, rho, sigma)
    return out


def _case(seed=3, n_ref=2000, nq=300, nf=10, k=30):
    rng = np.random.default_rng(seed)
    X = rng.normal(size=(n_ref, nf)).astype(np.float32)
    L = (X[:, :2] * 3.0 + 0.3 * X[:, 2:4] ** 2).astype(np.float32)  # a smooth, non-linear map
    Q = (X[:nq] + rng.normal(0, 0.2, (nq, nf))).astype(np.float32)
    Q[5] = X[123]  # a query sitting on a landmark
    d2 = ((Q[:, None, :].astype(np.float64) - X[None, :, :]) ** 2).sum(-1)
    idx = np.argsort(d2, 1)[:, :k]
    dist = np.sqrt(np.take_along_axis(d2, idx, 1)).astype(np.float32)
    return X, Q, L, (idx + 1).astype(np.int32), dist


def test_affine_start_matches_restatement():
    X, Q, L, idx, dist = _case()
    got = api.landmark_tsne_transform(X, Q, L, idx, dist, n_iter=0, affine_neighbors=8, affine_ridge=1e-3,
                                      max_extrapolation=1.5)
    want = affine_start(X, Q, L, idx, dist, 1, 8, 1e-3, 1.5)
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-4 * np.abs(L).max())
    np.testing.assert_array_equal(got[5], L[123])  # distance 0: the landmark itself


def test_exact_iterations_equal_the_fixed_reference_transform():
    """With exact repulsion the landmark path is the fixed-reference transform from the affine
    start (same P from the same float32 distances, same iteration kernel)."""
    X, Q, L, idx, dist = _case(seed=4)
    kw = dict(perplexity=5.0, n_iter=60, early_exaggeration_iter=10, learning_rate=0.1, max_grad_norm=0.25)
    start = api.landmark_tsne_transform(X, Q, L, idx, dist, n_iter=0)
    land = api.landmark_tsne_transform(X, Q, L, idx, dist, n_negatives=4096, exact_repulsion_threshold=4096, **kw)
    ref = api.transform_tsne(L.astype(np.float64), dict(indices=idx, distances=dist.astype(np.float64)),
                             Y_init=start.astype(np.float64), n_negatives=4096, exact_repulsion_threshold=4096,
                             **kw).layout
    np.testing.assert_allclose(land, ref, rtol=0, atol=2e-4 * np.abs(L).max())


def test_sampled_iterations_stay_near_the_exact_result():
    X, Q, L, idx, dist = _case(seed=5)
    exact = api.landmark_tsne_transform(X, Q, L, idx, dist, n_negatives=4096, exact_repulsion_threshold=4096)
    sampled = api.landmark_tsne_transform(X, Q, L, idx, dist, n_negatives=64, exact_repulsion_threshold=10, seed=9)
    assert np.all(np.isfinite(sampled))
    gap = np.sqrt(((sampled - exact) ** 2).sum(1))
    assert np.median(gap) < 0.1 * np.ptp(L, 0).max(), np.median(gap)


def test_invalid_landmark_inputs_raise():
    X, Q, L, idx, dist = _case(nq=20)
    with pytest.raises(_lib.CudaEmbeddingError, match="invalid CUDA landmark"):
        api.landmark_tsne_transform(X, Q, L, np.tile(idx, (1, 5)), np.tile(dist, (1, 5)))  # k = 150 > 128
    with pytest.raises(_lib.CudaEmbeddingError, match="invalid CUDA landmark"):
        api.landmark_tsne_transform(X, Q, L, idx, dist, perplexity=-1.0)
