"""GPU parity of the fixed-reference t-SNE transform (transform_tsne_cpp,
src/tsne_neighbors.cpp:2124-2373) against the reference's own outputs (golden vectors) and the
FP64 oracle, plus the behaviour tests of tests/testthat/test-transform-tsne.R.

Pair terms run in FP32 on the GPU and in FP64 in the reference, so layouts agree to a stated
tolerance, not bit for bit; the sampled repulsion draws the reference's exact xorshift32 sample
sequence, so sampled runs are compared the same way."""
import math

import numpy as np
import pytest

import oracle as O
from fastembedr_gb300 import _lib, api, synthetic

pytestmark = pytest.mark.gpu

# |GPU - reference| per coordinate after 250 iterations on a layout of spread ~10:
# median <= MED_TOL and 99th percentile <= P99_TOL.
MED_TOL = 1e-3
P99_TOL = 1e-2


def _close(a, b, med=MED_TOL, p99=P99_TOL):
    d = np.abs(np.asarray(a) - np.asarray(b))
    assert np.all(np.isfinite(a))
    assert np.median(d) <= med and np.quantile(d, 0.99) <= p99, (np.median(d), np.quantile(d, 0.99), d.max())


def test_exact_repulsion_matches_reference_golden(golden):
    g = golden("transform_2k")
    fit = api.transform_tsne(g["ref_y"], dict(indices=g["idx"], distances=g["dist"]), perplexity=5.0,
                             n_negatives=256, exact_repulsion_threshold=4096, seed=4)
    assert fit.config["repulsion"] == "exact_reference_cuda"
    _close(fit.layout, g["y_exact"])


def test_sampled_repulsion_matches_reference_golden(golden):
    g = golden("transform_2k")
    fit = api.transform_tsne(g["ref_y"], dict(indices=g["idx"], distances=g["dist"]), perplexity=5.0,
                             n_negatives=64, exact_repulsion_threshold=10, seed=4)
    assert fit.config["repulsion"] == "sampled_reference_cuda"
    assert fit.config["n_negatives"] == 64
    _close(fit.layout, g["y_sampled"])


@pytest.mark.parametrize("init", ["median", "weighted"])
def test_initialisation_matches_oracle(golden, init):
    """One iteration from the median / inverse-distance weighted start: the start is FP64 on
    both sides, so only one FP32 step separates them."""
    g = golden("transform_2k")
    fit = api.transform_tsne(g["ref_y"], dict(indices=g["idx"], distances=g["dist"]), initialization=init,
                             n_iter=1, seed=4)
    cpu = O.transform_tsne(g["ref_y"], g["idx"], g["dist"], init_mode=1 if init == "median" else 2, n_iter=1,
                           n_negatives=4096, exact_threshold=4096, seed=4)
    np.testing.assert_allclose(fit.layout, cpu, rtol=0, atol=1e-5)


def _libstdcxx_normal_pair(seed32):
    """std::mt19937(seed32) followed by two draws of std::normal_distribution<double>(0, 1e-4)
    as libstdc++ implements it (Marsaglia polar method over generate_canonical<double, 53>)."""
    bg = np.random.MT19937()
    bg._legacy_seeding(int(seed32))
    while True:
        w = bg.random_raw(4).astype(np.float64)
        u = (w[0] + w[1] * 2.0 ** 32) / 2.0 ** 64
        v = (w[2] + w[3] * 2.0 ** 32) / 2.0 ** 64
        x, y = 2.0 * u - 1.0, 2.0 * v - 1.0
        r2 = x * x + y * y
        if 0.0 < r2 <= 1.0:
            mult = math.sqrt(-2.0 * math.log(r2) / r2)
            return y * mult * 1e-4, x * mult * 1e-4


def _mix(v):
    v &= 0xFFFFFFFF
    v ^= v >> 16
    v = (v * 0x7FEB352D) & 0xFFFFFFFF
    v ^= v >> 15
    v = (v * 0x846CA68B) & 0xFFFFFFFF
    v ^= v >> 16
    return v if v else 0x6D2B79F5


def test_random_initialisation_matches_reference_stream(golden):
    """initialization = "random": N(0, 1e-4^2) from a per-query std::mt19937 seeded with
    mix_uint32(seed ^ (i + 1) * 0x9e3779b9) (src/tsne_neighbors.cpp:1398-1413)."""
    g = golden("transform_2k")
    seed = 11
    nq = g["idx"].shape[0]
    y0 = np.array([_libstdcxx_normal_pair(_mix(seed ^ (((i + 1) * 0x9E3779B9) & 0xFFFFFFFF))) for i in range(nq)])
    fit = api.transform_tsne(g["ref_y"], dict(indices=g["idx"], distances=g["dist"]), initialization="random",
                             n_iter=1, seed=seed)
    cpu = O.transform_tsne(g["ref_y"], g["idx"], g["dist"], y_init=y0, n_iter=1, n_negatives=4096,
                           exact_threshold=4096, seed=seed)
    np.testing.assert_allclose(fit.layout, cpu, rtol=0, atol=1e-5)


def test_supplied_init_and_early_phase_match_oracle():
    rng = np.random.default_rng(406)
    n_ref, nq, k = 96, 32, 18
    ref = rng.normal(size=(n_ref, 2))
    idx = rng.integers(1, n_ref + 1, (nq, k)).astype(np.int32)
    dist = np.sort(rng.exponential(size=(nq, k)), 1)
    y0 = rng.normal(size=(nq, 2))
    fit = api.transform_tsne(ref, dict(indices=idx, distances=dist), Y_init=y0, n_iter=5, early_exaggeration_iter=3,
                             n_negatives=12, exact_repulsion_threshold=8, seed=406)
    cpu = O.transform_tsne(ref, idx, dist, y_init=y0, n_iter=5, early_iter=3, n_negatives=12, exact_threshold=8,
                           seed=406)
    np.testing.assert_allclose(fit.layout, cpu, rtol=0, atol=1e-5)


def test_each_query_is_the_same_alone_and_in_a_batch():
    """Per-query streams are keyed by the global query row, so transforming a prefix of the
    queries alone gives bit-identical rows (tests/testthat/test-transform-tsne.R:89-149 with
    tolerance 0)."""
    rng = np.random.default_rng(407)
    n_ref, nq, k = 5000, 600, 15
    ref = rng.normal(0, 5, (n_ref, 2))
    idx = rng.integers(1, n_ref + 1, (nq, k)).astype(np.int32)
    dist = np.sort(rng.exponential(size=(nq, k)), 1)
    for thr in (8, 8192):  # sampled, exact
        full = api.transform_tsne(ref, dict(indices=idx, distances=dist), n_iter=20, n_negatives=40,
                                  exact_repulsion_threshold=thr, seed=407).layout
        part = api.transform_tsne(ref, dict(indices=idx[:77], distances=dist[:77]), n_iter=20, n_negatives=40,
                                  exact_repulsion_threshold=thr, seed=407).layout
        np.testing.assert_array_equal(part, full[:77])


def test_mixture_queries_match_oracle_sampled_20k():
    """20k-row reference (sampled repulsion, 256 negatives) with 1000 mixture queries and their
    exact 30-NN, against the FP64 oracle on the same sample streams."""
    x, _ = synthetic.mixture(21000, 20, 10, 77, centre_sd=4.0)
    ref_x, q_x = x[:20000].astype(np.float64), x[20000:].astype(np.float64)
    ref_y = np.random.default_rng(78).normal(0, 15, (20000, 2))
    d2 = (q_x ** 2).sum(1)[:, None] - 2.0 * q_x @ ref_x.T + (ref_x ** 2).sum(1)[None, :]
    qi = np.argsort(d2, 1)[:, :30]
    qd = np.sqrt(np.maximum(np.take_along_axis(d2, qi, 1), 0.0))
    qi = (qi + 1).astype(np.int32)
    fit = api.transform_tsne(ref_y, dict(indices=qi, distances=qd), seed=5)
    cpu = O.transform_tsne(ref_y, qi, qd, n_negatives=256, exact_threshold=4096, seed=5)
    assert fit.config["repulsion"] == "sampled_reference_cuda" and fit.config["n_negatives"] == 256
    _close(fit.layout, cpu)


def test_config_strings_follow_the_cuda_transform():
    rng = np.random.default_rng(403)
    ref = rng.normal(size=(42, 2))
    idx = rng.integers(1, 43, (8, 12)).astype(np.int32)
    dist = np.sort(rng.exponential(size=(8, 12)), 1)
    fit = api.transform_tsne(ref, dict(indices=idx, distances=dist), perplexity=4, n_iter=3, n_negatives=8,
                             exact_repulsion_threshold=1, seed=403)
    assert fit.layout.shape == (8, 2) and np.all(np.isfinite(fit.layout))
    assert fit.config["optimizer"] == "opentsne_style_fixed_reference_transform_cuda"
    assert fit.config["repulsion"] == "sampled_reference_cuda"
    assert fit.config["affinities"] == "precomputed_query_conditional"
    assert fit.config["transform_batches"] == 1


def test_invalid_inputs_raise():
    rng = np.random.default_rng(1)
    ref = rng.normal(size=(50, 2))
    idx = rng.integers(1, 51, (10, 5)).astype(np.int32)
    dist = np.sort(rng.exponential(size=(10, 5)), 1)
    bad = idx.copy()
    bad[3, 2] = 77
    with pytest.raises(_lib.CudaEmbeddingError, match="out of range"):
        api.transform_tsne(ref, dict(indices=bad, distances=dist), n_iter=2)
    neg = dist.copy()
    neg[0, 0] = -1.0
    with pytest.raises(_lib.CudaEmbeddingError, match="finite and non-negative"):
        api.transform_tsne(ref, dict(indices=idx, distances=neg), n_iter=2)
    with pytest.raises(ValueError, match="iteration counts"):
        api.transform_tsne(ref, dict(indices=idx, distances=dist), n_iter=0)
    with pytest.raises(ValueError, match="initialization"):
        api.transform_tsne(ref, dict(indices=idx, distances=dist), initialization="pca")
