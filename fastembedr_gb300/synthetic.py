"""Seeded synthetic inputs with the shapes of the benchmark workloads.

No public dataset is used. Each generator draws a Gaussian mixture and returns exact
Euclidean non-self KNN as the reference expects it: int32 indices (0-based) and float32
distances, both ``(n, k)``; the C ABI takes them column-major (``np.asfortranarray``).

* ``plain_tsne_10k``: 10,000 x 50, 10 equal clusters, centres N(0, 4^2 I), within N(0, I).
* ``plain_umap_100k``: 100,000 x 50, 20 clusters, log-normal(sigma = 1) sizes, centres
  N(0, 3^2 I), per-dimension sd U(0.5, 2).
* ``tsne_1m``: 1,000,000 x 50, 30 anisotropic clusters (diagonal sd U(0.5, 2)), log-normal sizes.
* ``serving_transform``: a 500,000 x 50 reference of 20 clusters and a query pool, 95% drawn
  from the same mixture and 5% uniform in the reference's bounding box.

Points are shuffled so that index order carries no cluster locality.
"""
from __future__ import annotations

import numpy as np


def mixture(n, dim, n_clusters, seed, centre_sd, within_sd=None, lognormal_sizes=False, anisotropic=False):
    rng = np.random.default_rng(seed)
    if lognormal_sizes:
        w = rng.lognormal(0.0, 1.0, n_clusters)
        counts = np.floor(w / w.sum() * n).astype(np.int64)
        counts[: n - counts.sum()] += 1
    else:
        counts = np.full(n_clusters, n // n_clusters, np.int64)
        counts[: n - counts.sum()] += 1
    centres = rng.normal(0.0, centre_sd, (n_clusters, dim))
    labels = np.repeat(np.arange(n_clusters), counts)
    if anisotropic or within_sd is None:
        sd = rng.uniform(0.5, 2.0, (n_clusters, dim))
    else:
        sd = np.full((n_clusters, dim), float(within_sd))
    x = centres[labels] + rng.standard_normal((n, dim)) * sd[labels]
    perm = rng.permutation(n)
    return x[perm].astype(np.float32), labels[perm].astype(np.int32)


def exact_knn_numpy(x, k, chunk=2048):
    """Brute-force exact non-self KNN in float64 (ties broken by index)."""
    x64 = np.asarray(x, np.float64)
    n = x64.shape[0]
    sq = np.einsum("ij,ij->i", x64, x64)
    idx = np.empty((n, k), np.int32)
    dist = np.empty((n, k), np.float32)
    for s in range(0, n, chunk):
        e = min(n, s + chunk)
        d2 = sq[s:e, None] + sq[None, :] - 2.0 * (x64[s:e] @ x64.T)
        np.maximum(d2, 0.0, out=d2)
        d2[np.arange(e - s), np.arange(s, e)] = np.inf
        part = np.argpartition(d2, k - 1, axis=1)[:, :k]
        pd = np.take_along_axis(d2, part, axis=1)
        order = np.lexsort((part, pd), axis=1)
        sel = np.take_along_axis(part, order, axis=1)
        idx[s:e] = sel
        dist[s:e] = np.sqrt(np.take_along_axis(d2, sel, axis=1)).astype(np.float32)
    return idx, dist


def exact_knn_torch(x, k, device="cuda", chunk=4096):
    """Brute-force exact non-self KNN on the GPU with torch (setup plumbing only)."""
    import torch

    xt = torch.as_tensor(np.asarray(x, np.float32), device=device)
    n = xt.shape[0]
    sq = (xt.double() ** 2).sum(1).float()
    idx = torch.empty((n, k), dtype=torch.int32, device=device)
    dist = torch.empty((n, k), dtype=torch.float32, device=device)
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    try:
        for s in range(0, n, chunk):
            e = min(n, s + chunk)
            d2 = sq[s:e, None] + sq[None, :] - 2.0 * (xt[s:e] @ xt.T)
            d2.clamp_(min=0.0)
            d2[torch.arange(e - s, device=device), torch.arange(s, e, device=device)] = float("inf")
            val, sel = torch.topk(d2, k, dim=1, largest=False, sorted=True)
            idx[s:e] = sel.int()
            dist[s:e] = val.sqrt()
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev
    return idx, dist


def exact_knn_query_torch(ref, queries, k, device="cuda", chunk=4096):
    """Brute-force exact KNN of each query row among the reference rows (no self exclusion)."""
    import torch

    rt = torch.as_tensor(np.asarray(ref, np.float32), device=device)
    qt = torch.as_tensor(np.asarray(queries, np.float32), device=device)
    sq_r = (rt.double() ** 2).sum(1).float()
    sq_q = (qt.double() ** 2).sum(1).float()
    nq = qt.shape[0]
    idx = torch.empty((nq, k), dtype=torch.int32, device=device)
    dist = torch.empty((nq, k), dtype=torch.float32, device=device)
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    try:
        for s in range(0, nq, chunk):
            e = min(nq, s + chunk)
            d2 = sq_q[s:e, None] + sq_r[None, :] - 2.0 * (qt[s:e] @ rt.T)
            d2.clamp_(min=0.0)
            val, sel = torch.topk(d2, k, dim=1, largest=False, sorted=True)
            idx[s:e] = sel.int()
            dist[s:e] = val.sqrt()
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev
    return idx, dist


def serving_transform(seed=5, n_ref=500_000, n_pool=100_000, dim=50, n_clusters=20):
    """Reference rows and a query pool for the serving transform: 20 clusters, centres
    N(0, 4^2 I), within N(0, I); 95% of the pool from the same mixture, 5% uniform in the
    reference's bounding box, shuffled."""
    n_mix = int(round(0.95 * n_pool))
    x, _ = mixture(n_ref + n_mix, dim, n_clusters, seed, centre_sd=4.0, within_sd=1.0)
    ref, q_mix = x[:n_ref], x[n_ref:]
    rng = np.random.default_rng(seed + 1)
    q_uni = rng.uniform(ref.min(0), ref.max(0), (n_pool - n_mix, dim)).astype(np.float32)
    pool = np.vstack([q_mix, q_uni])
    return ref, pool[rng.permutation(n_pool)]


def plain_tsne_10k(seed=1, n=10_000, k=90):
    x, lab = mixture(n, 50, 10, seed, centre_sd=4.0, within_sd=1.0)
    return x, lab


def plain_umap_100k(seed=2, n=100_000, k=15):
    x, lab = mixture(n, 50, 20, seed, centre_sd=3.0, lognormal_sizes=True, anisotropic=True)
    return x, lab


def tsne_1m(seed=3, n=1_000_000, k=90):
    x, lab = mixture(n, 50, 30, seed, centre_sd=4.0, lognormal_sizes=True, anisotropic=True)
    return x, lab


def tsne_init(n, seed=4):
    """Y_init ~ N(0, 1e-4^2), centred (the package's default random initialisation)."""
    rng = np.random.default_rng(seed)
    y = rng.normal(0.0, 1e-4, (n, 2))
    y -= y.mean(0)
    return y.astype(np.float32)
