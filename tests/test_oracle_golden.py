"""The CPU oracle against golden vectors produced by the reference's own CPU code.

The fixtures in tests/golden were made by tests/golden/make_golden.py from fastEmbedR
src/tsne_neighbors.cpp and src/fast_knn_umap.cpp (compiled unchanged against the
test-only Rcpp shim). Matching them pins the plain-C restatement that the GPU parity
tests then use as their checker.
"""
import numpy as np
import pytest

import oracle as O


@pytest.mark.parametrize("case", ["n48", "n300", "duplicated", "coincident", "extreme", "disconnected"])
def test_force_diagnostic_matches_reference(golden, case):
    g = golden("force_" + case)
    rp, col, val, _ = O.tsne_csr(g["idx"], g["dist"], float(g["perplexity"]))
    # (a) symmetrised CSR: integer structure bit-exact, values identical
    np.testing.assert_array_equal(rp, g["row_ptr"])
    np.testing.assert_array_equal(col, g["col"])
    np.testing.assert_array_equal(val.astype(np.float64), g["weight"])
    y = g["layout"].astype(np.float32)
    att = O.attractive(rp, col, val, y, 1.0)
    np.testing.assert_array_equal(att.astype(np.float64), g["attractive"])
    rex, sq = O.exact_rep_f32(y)
    np.testing.assert_allclose(rex, g["rep_exact"], rtol=0, atol=1e-6 * max(1e-30, np.abs(g["rep_exact"]).max()))
    rff, _ = O.fft_grid_rep_f32(y, int(g["grid"]))
    np.testing.assert_allclose(rff, g["rep_fft"], rtol=0, atol=1e-6 * max(1e-30, np.abs(g["rep_fft"]).max()))
    assert O.kl(rp, col, val, y) == pytest.approx(float(g["kl"]), rel=1e-12)
    assert np.all(np.isfinite(rff)) and np.all(np.isfinite(rex))


def test_full_tsne_run_matches_reference_bitwise(golden):
    g = golden("tsne_run_2k")
    y, trace, its = O.tsne_run(g["idx"], g["dist"], g["init"], perplexity=float(g["perplexity"]),
                               early_iter=int(g["early_iter"]), n_iter=int(g["n_iter"]), kl_every=True)
    np.testing.assert_array_equal(y.astype(np.float64), g["y"])
    np.testing.assert_allclose(trace, g["itercosts"], rtol=1e-12)


def test_umap_graph_and_serial_sgd_match_reference(golden):
    g = golden("umap_3k")
    off, nb, w, e, mw = O.umap_graph(g["idx"], g["dist"])
    np.testing.assert_array_equal(off, g["offsets"])
    np.testing.assert_array_equal(nb, g["neighbors"])
    np.testing.assert_array_equal(w.astype(np.float64), g["weights"])
    np.testing.assert_array_equal(e.astype(np.float64), g["epochs_per_sample"])
    n = off.size - 1
    emb = np.ascontiguousarray(g["init"].T).ravel().copy()
    a, b = O.umap_ab(0.01)
    O.orc().orc_umap_sgd_serial(n, off, nb, w, emb, int(g["n_epochs"]), a, b, 5, 1.0, 1.0, int(g["seed"]))
    np.testing.assert_array_equal(emb.reshape(2, n).T, g["y"])


@pytest.mark.parametrize("tag", ["3k", "200"])
def test_umap_diffusion_start_matches_reference(golden, tag):
    """initialize_layout_csr_cuda_diffusion (one worker) over the reference fuzzy graph."""
    g = golden("umap_diffusion")
    off, nb, w, _, _ = O.umap_graph(g["idx_" + tag], g["dist_" + tag])
    y = O.umap_diffusion_init(off, nb, w, int(g["iters_" + tag]), int(g["seed_" + tag]))
    np.testing.assert_array_equal(y.astype(np.float64), g["init_" + tag])


@pytest.mark.parametrize("tag", ["3k", "40"])
def test_umap_spectral_start_matches_reference(golden, tag):
    """initialize_layout_csr through spectral_knn_init(backend = "cpu"), one worker."""
    g = golden("umap_spectral")
    off, nb, w, _, _ = O.umap_graph(g["idx_" + tag], g["dist_" + tag])
    y = O.umap_spectral_init(off, nb, w, int(g["iters_" + tag]), int(g["seed_" + tag]))
    np.testing.assert_array_equal(y, g["start_" + tag])
    if tag == "40":
        ys = O.umap_spectral_init(off, nb, w, 5, 9, init_scale=2.0)
        np.testing.assert_array_equal(ys, g["start_40_scaled"])


def test_umap_spectral_start_redraws_like_the_reference(golden):
    """Gram-Schmidt redraws of vanished columns (a rank-6 graph with 34 isolated points)."""
    g = golden("umap_spectral")
    y = O.umap_spectral_init(g["iso_offsets"], g["iso_neighbors"], g["iso_weights"].astype(np.float32), 4, 11)
    np.testing.assert_array_equal(y, g["start_iso"])


@pytest.mark.parametrize("tag,nneg,thr", [("exact", 256, 4096), ("sampled", 64, 10)])
def test_transform_matches_reference(golden, tag, nneg, thr):
    g = golden("transform_2k")
    y = O.transform_tsne(g["ref_y"], g["idx"], g["dist"], init_mode=1, n_negatives=nneg, exact_threshold=thr)
    np.testing.assert_array_equal(y, g["y_" + tag])


def test_umap_ab_policies():
    # CPU policy hard-codes min_dist = 0.01 (src/fast_knn_umap.cpp:437-440); the CUDA host
    # path grid-fits it (src/embedding_cuda_impl.cpp:491-545)
    assert O.umap_ab(0.01) == (1.895605865596314, 0.8006377738365004)
    a, b = O.umap_ab(0.01, cuda_host=True)
    assert abs(a - 1.8956) < 0.05 and abs(b - 0.8006) < 0.01


def test_fp64_probability_oracle_tracks_fp32_reference(golden):
    """The FP64 bisection (the reference's test helper) and the FP32 CPU path agree on the
    symmetric P within the reference's own check: testthat all.equal mean relative
    difference < 2e-6 (tests/testthat/test-tsne-numerics.R:18-22)."""
    g = golden("force_n300")
    p32 = O.row_p_f32(g["dist"], 5.0)
    p64, _ = O.row_p_f64(g["dist"], 5.0)
    _, _, v32, _ = O.csr_from_p(g["idx"], p32)
    _, _, v64, _ = O.csr_from_p(g["idx"], p64.astype(np.float32))
    assert np.abs(v32.astype(np.float64) - v64).sum() / np.abs(v64).sum() < 2e-6


def test_knn_preservation_known_answers():
    """15-NN preservation as knn_structure_score_cpp defines it (src/embedding_utils.cpp:1386-1579:
    the preserve_k nearest layout points by (squared distance, index), counted against the first
    preserve_k high-dimensional neighbours). Known answers: an unchanged embedding scores exactly 1
    (the reference's tests/testthat/test-evaluation-core.R:1-13 and test-cuda-stages.R:101-115
    set-up: a 30 x 2 layout scored against its own exact KNN, preserve_k = 6), and a five-point
    case worked by hand scores 0.6."""
    from fastembedr_gb300 import synthetic

    layout = np.random.default_rng(13).standard_normal((30, 2)).astype(np.float32)
    idx, _ = synthetic.exact_knn_numpy(layout, 7)
    assert O.knn_preservation(layout, idx, preserve_k=6) == 1.0
    # points on a line at x = 0, 1, 3, 6, 10; layout 2-NN: {1, 2}, {0, 2}, {1, 0}, {2, 4}, {3, 2}
    line = np.array([[0, 0], [1, 0], [3, 0], [6, 0], [10, 0]], np.float32)
    hi = np.array([[1, 3, 2], [2, 0, 3], [4, 3, 0], [2, 4, 1], [3, 0, 1]], np.int32)
    # shared among the first two: 1 of {1, 3}; 2 of {2, 0}; 0 of {4, 3}; 2 of {2, 4}; 1 of {3, 0}
    assert O.knn_preservation(line, hi, preserve_k=2) == pytest.approx((0.5 + 1.0 + 0.0 + 1.0 + 0.5) / 5, abs=1e-15)
    # 1-based labels give the same score
    assert O.knn_preservation(line, hi + 1, preserve_k=2, offset=1) == pytest.approx(0.6, abs=1e-15)


def test_knn_preservation_matches_reference_golden(golden):
    """M1 pinned on the reference's own knn_structure_score_cpp (src/embedding_utils.cpp:1386-1579,
    compiled under the test shim by tests/golden/make_golden.py): preservation of two layouts over
    every row and every 7th row at preserve_k 10 and 15 equals the reference's to the last bits of
    the summation order."""
    g = golden("knn_structure")
    for a, lay in enumerate(g["layouts"]):
        for b, keep in enumerate((g["keep_all"], g["keep_sub"])):
            for c, pk in enumerate(g["preserve_k"]):
                got = O.knn_preservation(lay, g["idx"], keep=keep, preserve_k=int(pk))
                assert got == pytest.approx(g["scores"][a, b, c, 0], abs=1e-15), (a, b, c)


@pytest.mark.parametrize("case", [0, 1, 2])
def test_affine_restatement_matches_reference_golden(golden, case):
    """The FP64 restatement of the landmark affine start that the GPU tests use, against the
    reference's CPU statement of the start (project_embedding_affine_cpp,
    src/embedding_utils.cpp:2120-2335, run under the test shim): equal to 1e-8 of the layout
    scale (about 1e-9 measured: summation order and the float median of the reference)."""
    from affine_restatement import affine_start

    g = golden("landmark_affine")
    m, ridge, ext = g["settings"][case]
    want = g["layouts"][case]
    got = affine_start(g["X"], g["Q"], g["L"], g["idx"] + 1, g["dist"], 1, int(m), float(ridge), float(ext))
    assert not g["fallback"][case].any()
    assert np.abs(got - want).max() <= 1e-8 * np.abs(g["L"]).max()
    np.testing.assert_array_equal(want[5], g["L"][123].astype(np.float64))  # distance 0: the landmark
