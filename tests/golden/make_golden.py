"""Generate tests/golden/*.npz from the reference's own CPU code.

Runs fastEmbedR's src/tsne_neighbors.cpp, src/fast_knn_umap.cpp and src/embedding_utils.cpp,
compiled where they lie against the test-only Rcpp shim (``make -C oracle ref``), on small seeded
inputs and stores inputs + outputs. The fixtures travel with the repository; the
reference sources do not. Re-run with
    FASTEMBEDR_REFERENCE_SRC=<the reference's src/ directory> python tests/golden/make_golden.py
(or ``... make_golden.py umap_diffusion`` for one case).
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402
from fastembedr_gb300 import synthetic as S  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def cm(a, t):
    return np.ascontiguousarray(np.asarray(a, t).T).ravel()


def force_case(name, x_seed, n, dim, k, perp, grid, layout_sd, layout=None, x=None):
    R = O.ref()
    rng = np.random.default_rng(x_seed)
    if x is None:
        x = rng.standard_normal((n, dim)).astype(np.float32)
    idx, dist = S.exact_knn_numpy(x, k)
    n = idx.shape[0]
    if layout is None:
        layout = (rng.standard_normal((n, 2)) * layout_sd).astype(np.float32)
    cap = 2 * n * k
    att, rex, rff = np.zeros(2 * n), np.zeros(2 * n), np.zeros(2 * n)
    rp = np.zeros(n + 1, np.int32)
    col = np.zeros(cap, np.int32)
    w = np.zeros(cap)
    nnz, sq, kl = C.c_longlong(), C.c_double(), C.c_double()
    st = R.ref_force_diagnostic(cm(idx, np.int32), cm(dist, np.float64), cm(layout, np.float64), n, k,
                                float(perp), 1.0, int(grid), 1, att, rex, rff, rp, col, w, cap, C.byref(nnz),
                                C.byref(sq), C.byref(kl))
    assert st == 0, R.ref_last_error()
    m = nnz.value
    np.savez_compressed(
        os.path.join(OUT, f"force_{name}.npz"), idx=idx, dist=dist, layout=layout, perplexity=perp, grid=grid,
        row_ptr=rp, col=col[:m], weight=w[:m], attractive=att.reshape(2, n).T, rep_exact=rex.reshape(2, n).T,
        rep_fft=rff.reshape(2, n).T, sum_q=sq.value, kl=kl.value)


def tsne_run_case():
    R = O.ref()
    x, _ = S.mixture(2000, 20, 5, 11, centre_sd=4.0, within_sd=1.0)
    idx, dist = S.exact_knn_numpy(x, 30)
    n, k = idx.shape
    init = S.tsne_init(n, 5)
    y = np.zeros(2 * n)
    costs = np.zeros(64)
    nc, g = C.c_int(), C.c_int()
    st = R.ref_tsne_run(cm(idx, np.int32), cm(dist, np.float64), cm(init, np.float64), n, k, 10.0, 250, 750, 12.0,
                        1.0, -1.0, 1, 0.8, 0.8, 0.01, 5.0, b"fft", 1, 4, 1, y, costs, C.byref(nc), C.byref(g))
    assert st == 0, R.ref_last_error()
    np.savez_compressed(os.path.join(OUT, "tsne_run_2k.npz"), idx=idx, dist=dist, init=init, perplexity=10.0,
                        early_iter=250, n_iter=750, y=y.reshape(2, n).T, itercosts=costs[: nc.value],
                        grid=g.value)


def umap_case():
    R = O.ref()
    x, _ = S.mixture(3000, 20, 6, 12, centre_sd=3.0, lognormal_sizes=True, anisotropic=True)
    idx, dist = S.exact_knn_numpy(x, 15)
    n, k = idx.shape
    cap = 2 * n * k
    off = np.zeros(n + 1, np.int32)
    nb = np.zeros(cap, np.int32)
    w, e = np.zeros(cap), np.zeros(cap)
    nnz, mw = C.c_longlong(), C.c_double()
    st = R.ref_umap_graph(cm(idx, np.int32), cm(dist, np.float64), n, k, 1, off, nb, w, e, cap, C.byref(nnz),
                          C.byref(mw))
    assert st == 0, R.ref_last_error()
    m = nnz.value
    init = np.random.default_rng(3).uniform(-10, 10, (n, 2))
    out = np.zeros(2 * n)
    st = R.ref_umap_sgd(off, nb[:m].copy(), w[:m].copy(), cm(init, np.float64), n, m, 200, 0.01, 5, 1.0, 1.0, 1,
                        42, out)
    assert st == 0, R.ref_last_error()
    np.savez_compressed(os.path.join(OUT, "umap_3k.npz"), idx=idx, dist=dist, offsets=off, neighbors=nb[:m],
                        weights=w[:m], epochs_per_sample=e[:m], max_weight=mw.value, init=init,
                        y=out.reshape(2, n).T, n_epochs=200, seed=42)


def umap_diffusion_case():
    """The reference's CPU statement of its GPU diffusion start (umap_cuda_diffusion_init_csr_cpp,
    one worker) over the reference fuzzy graph of the umap_3k workload (20 rounds, the pilot
    default for k <= 15), and over a small two-cluster graph with k = 5 (3 rounds)."""
    R = O.ref()
    out = {}
    cases = (("3k", S.mixture(3000, 20, 6, 12, centre_sd=3.0, lognormal_sizes=True, anisotropic=True)[0], 15, 20, 42),
             ("200", np.vstack([np.random.default_rng(8).normal(-3, 1, (100, 4)),
                                np.random.default_rng(9).normal(3, 1, (100, 4))]).astype(np.float32), 5, 3, 7))
    for tag, x, k, iters, seed in cases:
        idx, dist = S.exact_knn_numpy(x, k)
        n = idx.shape[0]
        cap = 2 * n * k
        off = np.zeros(n + 1, np.int32)
        nb = np.zeros(cap, np.int32)
        w, e = np.zeros(cap), np.zeros(cap)
        nnz, mw = C.c_longlong(), C.c_double()
        st = R.ref_umap_graph(cm(idx, np.int32), cm(dist, np.float64), n, k, 1, off, nb, w, e, cap, C.byref(nnz),
                              C.byref(mw))
        assert st == 0, R.ref_last_error()
        m = nnz.value
        y = np.zeros(2 * n)
        st = R.ref_umap_diffusion_init(off, nb[:m].copy(), w[:m].copy(), n, m, iters, seed, y)
        assert st == 0, R.ref_last_error()
        out.update({f"idx_{tag}": idx, f"dist_{tag}": dist, f"init_{tag}": y.reshape(n, 2),
                    f"iters_{tag}": iters, f"seed_{tag}": seed})
    np.savez_compressed(os.path.join(OUT, "umap_diffusion.npz"), **out)


def umap_spectral_case():
    """spectral_knn_init(backend = "cpu") of the reference (fast_knn_umap_range_cpp with n_epochs = 0,
    one worker) on the umap_3k KNN (30 rounds) and on a 40-point KNN (5 rounds); the second also
    through fast_knn_umap_csr_cpp with init_scale 2 on the reference graph."""
    R = O.ref()
    out = {}
    x3k = S.mixture(3000, 20, 6, 12, centre_sd=3.0, lognormal_sizes=True, anisotropic=True)[0]
    x40 = np.random.default_rng(41).normal(size=(40, 5)).astype(np.float32)
    for tag, x, k, iters, seed in (("3k", x3k, 15, 30, 42), ("40", x40, 8, 5, 9)):
        idx, dist = S.exact_knn_numpy(x, k)
        n = idx.shape[0]
        y = np.zeros(2 * n)
        st = R.ref_umap_spectral_knn(cm(idx, np.int32), cm(dist, np.float64), n, k, iters, seed, y)
        assert st == 0, R.ref_last_error()
        out.update({f"idx_{tag}": idx, f"dist_{tag}": dist, f"start_{tag}": y.reshape(n, 2),
                    f"iters_{tag}": iters, f"seed_{tag}": seed})
    idx, dist = out["idx_40"], out["dist_40"]
    n, k = idx.shape
    cap = 2 * n * k
    off = np.zeros(n + 1, np.int32)
    nb = np.zeros(cap, np.int32)
    w, e = np.zeros(cap), np.zeros(cap)
    nnz, mw = C.c_longlong(), C.c_double()
    st = R.ref_umap_graph(cm(idx, np.int32), cm(dist, np.float64), n, k, 1, off, nb, w, e, cap, C.byref(nnz),
                          C.byref(mw))
    assert st == 0, R.ref_last_error()
    m = nnz.value
    y = np.zeros(2 * n)
    st = R.ref_umap_spectral_init(off, nb[:m].copy(), w[:m].copy(), n, m, 5, 2.0, 9, y)
    assert st == 0, R.ref_last_error()
    out["start_40_scaled"] = y.reshape(n, 2)
    # a graph whose operator has rank 6 (a 6-ring with weights exact in float32, 34 isolated
    # points): after each multiply the block's later columns vanish in Gram-Schmidt and are
    # redrawn from the stream
    n = 40
    ring = 6
    rows = [[] for _ in range(n)]
    for i in range(ring):
        for j, wv in (((i + 1) % ring, 0.5 + 0.125 * i), ((i + 2) % ring, 0.25 + 0.0625 * i)):
            rows[i].append((j, wv))
            rows[j].append((i, wv))
    off = np.zeros(n + 1, np.int32)
    nbl, wl = [], []
    for i in range(n):
        for j, wv in sorted(rows[i]):
            nbl.append(j)
            wl.append(wv)
        off[i + 1] = len(nbl)
    nb, w = np.array(nbl, np.int32), np.array(wl, np.float64)
    y = np.zeros(2 * n)
    st = R.ref_umap_spectral_init(off, nb, w, n, len(nb), 4, float("nan"), 11, y)
    assert st == 0, R.ref_last_error()
    out.update({"iso_offsets": off, "iso_neighbors": nb, "iso_weights": w, "start_iso": y.reshape(n, 2)})
    np.savez_compressed(os.path.join(OUT, "umap_spectral.npz"), **out)


def transform_case():
    R = O.ref()
    xr, _ = S.mixture(2500, 20, 5, 13, centre_sd=4.0, within_sd=1.0)
    xq = xr[:300] + np.random.default_rng(1).normal(0, 0.3, (300, 20)).astype(np.float32)
    ref = xr[300:]
    refy = np.random.default_rng(2).normal(0, 10, (ref.shape[0], 2))
    d2 = ((xq[:, None, :].astype(np.float64) - ref[None, :, :]) ** 2).sum(-1)
    qi = np.argsort(d2, 1)[:, :30].astype(np.int32)
    qd = np.sqrt(np.take_along_axis(d2, qi, 1))
    outs = {}
    for tag, nneg, thr in (("exact", 256, 4096), ("sampled", 64, 10)):
        y = np.zeros(600)
        st = R.ref_transform(cm(refy, np.float64), refy.shape[0], cm(qi, np.int32), cm(qd, np.float64), 300, 30,
                             None, 0, b"median", 5.0, 250, 0, 0.1, 4.0, 1.5, 0.8, 0.8, 0.25, np.inf, nneg, thr, 1, 4,
                             y)
        assert st == 0, R.ref_last_error()
        outs[tag] = y.reshape(2, 300).T
    np.savez_compressed(os.path.join(OUT, "transform_2k.npz"), ref_y=refy, idx=qi, dist=qd,
                        y_exact=outs["exact"], y_sampled=outs["sampled"])


def structure_case():
    """knn_structure_score_cpp (src/embedding_utils.cpp:1386-1579) on 400 points of a 20-d
    mixture against their exact 24-NN: two layouts (two data coordinates, random normal), every
    row or every 7th row, preserve_k 10 and 15. Stores preservation, trustworthiness,
    continuity and the structure score per case."""
    lib = O.ref()
    x, _ = S.mixture(400, 20, 5, 71, centre_sd=3.0)
    idx, _ = S.exact_knn_numpy(x, 24)
    layouts = np.stack([(x[:, :2] * 2.0).astype(np.float32),
                        np.random.default_rng(72).standard_normal((400, 2)).astype(np.float32)])
    keeps = [np.arange(400, dtype=np.int32), np.arange(0, 400, 7, dtype=np.int32)]
    scores = np.zeros((2, 2, 2, 4))
    for a, lay in enumerate(layouts):
        for b, keep in enumerate(keeps):
            keep1 = np.ascontiguousarray(keep + 1, np.int32)
            for c, pk in enumerate((10, 15)):
                r = np.zeros(4)
                st = lib.ref_knn_structure_score(cm(lay, np.float64), 400, cm(idx + 1, np.int32), 24, keep1,
                                                 keep1.size, pk, r)
                assert st == 0, lib.ref_last_error()
                scores[a, b, c] = r
    np.savez_compressed(os.path.join(OUT, "knn_structure.npz"), idx=idx, layouts=layouts, keep_all=keeps[0],
                        keep_sub=keeps[1], preserve_k=np.array([10, 15]), scores=scores)


def affine_case():
    """project_embedding_affine_cpp (src/embedding_utils.cpp:2120-2335), the reference's CPU
    statement of the landmark affine start, on 800 landmarks x 8 features with a smooth
    non-linear 2-d layout and 150 queries (one sitting on a landmark), exact 24-NN; three
    (neighbours, ridge, max extrapolation) settings."""
    lib = O.ref()
    rng = np.random.default_rng(5)
    n_ref, nq, nf, k = 800, 150, 8, 24
    X = rng.normal(size=(n_ref, nf)).astype(np.float32)
    L = (X[:, :2] * 3.0 + 0.3 * X[:, 2:4] ** 2).astype(np.float32)
    Q = (X[:nq] + rng.normal(0, 0.2, (nq, nf))).astype(np.float32)
    Q[5] = X[123]
    d2 = ((Q[:, None, :].astype(np.float64) - X[None, :, :]) ** 2).sum(-1)
    idx = np.argsort(d2, 1, kind="stable")[:, :k].astype(np.int32)
    dist = np.sqrt(np.take_along_axis(d2, idx, 1)).astype(np.float32)
    settings = np.array([[8, 1e-3, 1.5], [12, 1e-2, 2.5], [3, 1e-3, 1.0]])
    layouts = np.zeros((len(settings), nq, 2))
    fallback = np.zeros((len(settings), nq), np.int32)
    for t, (m, ridge, ext) in enumerate(settings):
        out = np.zeros(2 * nq)
        conf = np.zeros(nq)
        fb = np.zeros(nq, np.int32)
        st = lib.ref_project_affine(cm(X, np.float64), n_ref, cm(Q, np.float64), nq, nf, cm(L, np.float64),
                                    cm(idx + 1, np.int32), cm(dist, np.float64), k, int(m), float(ridge),
                                    float(ext), out, conf, fb)
        assert st == 0, lib.ref_last_error()
        layouts[t] = out.reshape(2, nq).T
        fallback[t] = fb
    np.savez_compressed(os.path.join(OUT, "landmark_affine.npz"), X=X, Q=Q, L=L, idx=idx, dist=dist,
                        settings=settings, layouts=layouts, fallback=fallback)


def main():
    O.build(ref=True)
    if len(sys.argv) > 1:
        for name in sys.argv[1:]:
            globals()[name + "_case"]()
        print("golden fixtures written to", OUT)
        return
    force_case("n48", 701, 48, 6, 15, 5.0, 64, 0.3)
    force_case("n300", 7011, 300, 6, 15, 5.0, 64, 0.3)
    # pathological inputs of tests/testthat/test-tsne-numerics.R:120-160
    rng = np.random.default_rng(705)
    dup = np.vstack([np.zeros((8, 4)), np.ones((8, 4)), rng.normal(0, 1e-8, (8, 4))]).astype(np.float32)
    force_case("duplicated", 705, 24, 4, 6, 2.0, 64, 0.1, x=dup)
    force_case("coincident", 705, 24, 4, 6, 2.0, 64, 0.1, x=dup, layout=np.zeros((24, 2), np.float32))
    ext = np.tile(np.array([[-1e4, 1e4]], np.float32), (24, 1))
    force_case("extreme", 705, 24, 4, 6, 2.0, 64, 0.1, x=dup, layout=ext)
    dis = np.vstack([rng.normal(-20, 0.01, (12, 4)), rng.normal(20, 0.01, (12, 4))]).astype(np.float32)
    force_case("disconnected", 7051, 24, 4, 6, 2.0, 64, 0.1, x=dis)
    tsne_run_case()
    umap_case()
    transform_case()
    structure_case()
    affine_case()
    print("golden fixtures written to", OUT)


if __name__ == "__main__":
    main()
