"""Landmark t-SNE transform (fastembedr_cuda_landmark_tsne_from_device_knn,
src/embedding_cuda_kernels.cpp:3572-3686): the affine start against the reference's CPU
statement of it (golden) and a NumPy FP64 restatement of landmark_affine_projection_kernel
(:552-733, pinned to the same golden on the CPU), the iterations against the fixed-reference
transform from the same start, and the reference's argument checks."""
import numpy as np
import pytest

from affine_restatement import affine_start
from fastembedr_gb300 import _lib, api

pytestmark = pytest.mark.gpu


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


@pytest.mark.parametrize("case", [0, 1, 2])
def test_affine_start_matches_reference_golden(golden, case):
    """The GPU affine start against the reference's CPU statement of it
    (project_embedding_affine_cpp, src/embedding_utils.cpp:2120-2335, golden made under the test
    shim) for three (neighbours, ridge, max extrapolation) settings."""
    g = golden("landmark_affine")
    m, ridge, ext = g["settings"][case]
    got = api.landmark_tsne_transform(g["X"], g["Q"], g["L"], g["idx"] + 1, g["dist"], n_iter=0,
                                      affine_neighbors=int(m), affine_ridge=float(ridge),
                                      max_extrapolation=float(ext))
    want = g["layouts"][case]
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-4 * np.abs(g["L"]).max())
    np.testing.assert_array_equal(got[5], g["L"][123])


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
