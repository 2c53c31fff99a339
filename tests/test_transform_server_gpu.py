"""The transform serving loop: continuous admission against a memory budget, merged launches,
and results that are bit-identical to the one-shot transform whatever else is in flight."""
import threading

import numpy as np
import pytest

from fastembedr_gb300 import _lib, api

pytestmark = pytest.mark.gpu


def _requests(n_ref, sizes, k, seed):
    rng = np.random.default_rng(seed)
    out = []
    for nq in sizes:
        idx = rng.integers(1, n_ref + 1, (nq, k)).astype(np.int32)
        dist = np.sort(rng.exponential(size=(nq, k)), 1).astype(np.float32)
        out.append((idx, dist))
    return out


def _one_shot(ref, idx, dist, **kw):
    return api.transform_tsne(ref, dict(indices=idx, distances=dist.astype(np.float64)), **kw).layout


@pytest.mark.parametrize("n_ref", [20000, 3000])  # sampled, exact
def test_results_equal_one_shot_in_a_mix(n_ref):
    rng = np.random.default_rng(11)
    ref = rng.normal(0, 12, (n_ref, 2))
    reqs = _requests(n_ref, [1, 7, 300, 5000, 2, 1200, 33, 90], 30, 12)
    ids = [None] * len(reqs)
    with api.TransformServer(ref, n_iter=60, seed=21) as sv:
        def submit(part):
            for j in part:
                ids[j] = sv.submit(*reqs[j])
        ts = [threading.Thread(target=submit, args=(range(p, len(reqs), 2),)) for p in (0, 1)]
        for t in ts:
            t.start()
        for t in ts:
            t.join()
        results = [sv.result(i) for i in ids]
        stats = sv.stats()
    assert stats["completed"] == len(reqs) and stats["queries"] == sum(r[0].shape[0] for r in reqs)
    for (idx, dist), (layout, latency) in zip(reqs, results):
        assert latency > 0.0
        np.testing.assert_array_equal(layout, _one_shot(ref, idx, dist, n_iter=60, seed=21))


def test_memory_budget_queues_requests_and_everything_completes():
    n_ref, k = 8000, 30
    ref = np.random.default_rng(3).normal(0, 10, (n_ref, 2))
    reqs = _requests(n_ref, [4000] * 5 + [10] * 5, k, 4)
    per_query = k * 20 + 64  # idx, dist, neighbour coordinates, P; state, options, output
    budget = int(4000 * per_query * 1.5)  # one large request at a time
    with api.TransformServer(ref, n_iter=30, memory_budget_bytes=budget, seed=5) as sv:
        ids = [sv.submit(*r) for r in reqs]
        results = [sv.result(i) for i in ids]
        stats = sv.stats()
    assert stats["budget_bytes"] <= budget and stats["peak_bytes"] <= stats["budget_bytes"]
    assert stats["groups"] >= 5
    for (idx, dist), (layout, _) in zip(reqs, results):
        np.testing.assert_array_equal(layout, _one_shot(ref, idx, dist, n_iter=30, seed=5))


def test_request_larger_than_budget_is_rejected():
    ref = np.random.default_rng(1).normal(size=(500, 2))
    idx, dist = _requests(500, [20000], 15, 2)[0]
    with api.TransformServer(ref, n_iter=5, memory_budget_bytes=1 << 20) as sv:
        with pytest.raises(_lib.CudaEmbeddingError, match="memory budget"):
            sv.submit(idx, dist)
        bad = idx[:10].copy()
        bad[0, 0] = 9999
        with pytest.raises(_lib.CudaEmbeddingError, match="out of range"):
            sv.submit(bad, dist[:10])


def test_random_and_weighted_starts_match_one_shot():
    n_ref = 6000
    ref = np.random.default_rng(8).normal(0, 10, (n_ref, 2))
    reqs = _requests(n_ref, [50, 400], 20, 9)
    for init in ("random", "weighted"):
        with api.TransformServer(ref, initialization=init, n_iter=20, early_exaggeration_iter=5, seed=13) as sv:
            ids = [sv.submit(*r) for r in reqs]
            outs = [sv.result(i)[0] for i in ids]
        for (idx, dist), layout in zip(reqs, outs):
            ref_out = _one_shot(ref, idx, dist, initialization=init, n_iter=20, early_exaggeration_iter=5, seed=13)
            np.testing.assert_array_equal(layout, ref_out)
