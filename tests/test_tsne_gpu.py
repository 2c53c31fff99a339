"""GPU parity of the t-SNE path against the CPU oracle (itself pinned to the reference CPU code).

Checks follow the spec split:
 (a) symmetrised CSR: integer structure bit-exact;
 (b) per-row bisection entropies within 1e-6 relative of the FP64 oracle;
 (c) attractive / repulsive forces on the same Y and P within 1e-4 relative L2 of FP64 oracles,
     with the interpolation error measured separately against exact FP64 repulsion;
 (d) end-to-end KL within 1 % and 15-NN preservation within 0.01 of the reference CPU run.
"""
import numpy as np
import pytest

import oracle as O
from fastembedr_gb300 import _lib, api, synthetic

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(scope="module")
def small():
    x, lab = synthetic.mixture(3000, 20, 6, 31, centre_sd=4.0, within_sd=1.0)
    idx, dist = synthetic.exact_knn_numpy(x, 45)
    return idx, dist, lab


@pytest.fixture(scope="module")
def c1():
    """Plain tsne_knn workload: 10,000 x 50, 10 clusters, exact KNN k = 90, perplexity 30."""
    x, lab = synthetic.plain_tsne_10k()
    idx, dist = synthetic.exact_knn_numpy(x, 90)
    return idx, dist, lab


@pytest.mark.parametrize("case", ["n48", "n300", "duplicated", "coincident", "extreme", "disconnected"])
def test_csr_bit_exact_on_reference_golden(golden, case):
    g = golden("force_" + case)
    a = api.tsne_affinities(g["idx"], g["dist"], float(g["perplexity"]))
    np.testing.assert_array_equal(a["row_ptr"], g["row_ptr"])
    np.testing.assert_array_equal(a["col"], g["col"])
    # values: FP64-sum bisection vs the reference FP32 bisection; the reference's own tolerance
    w = g["weight"]
    assert np.abs(a["val"] - w).sum() / np.abs(w).sum() < 2e-6


def test_csr_bit_exact_and_entropies_plain_10k(c1):
    idx, dist, _ = c1
    a = api.tsne_affinities(idx, dist, 30.0)
    rp, col, val, tot = O.tsne_csr(idx, dist, 30.0)
    np.testing.assert_array_equal(a["row_ptr"], rp)
    np.testing.assert_array_equal(a["col"], col)
    assert np.abs(a["val"] - val).sum() / np.abs(val).sum() < 2e-6
    assert a["total_mass"] == pytest.approx(tot, rel=1e-6)
    # (b) entropies of the GPU rows vs the FP64 oracle rows
    p64, _ = O.row_p_f64(dist, 30.0)
    h64 = -(np.where(p64 > 0, p64 * np.log(np.maximum(p64, 1e-300)), 0.0)).sum(1)
    rel = np.abs(a["entropy"] - h64) / h64
    assert np.median(rel) < 1e-7
    assert np.quantile(rel, 0.999) < 1e-6
    assert np.abs(a["entropy"] - np.log(30.0)).max() < 2e-5
    p = a["p_directed"].astype(np.float64)
    assert np.abs(p - p64).max() < 1e-6


@pytest.mark.parametrize("interp", [0, 1])
@pytest.mark.parametrize("grid", [64, 128, 256])
def test_forces_match_fp64_oracles(small, interp, grid):
    idx, dist, _ = small
    n = idx.shape[0]
    y = (np.random.default_rng(grid + interp).standard_normal((n, 2)) * 6.0).astype(np.float32)
    d = api.tsne_force_diagnostic(idx, dist, y, 15.0, exaggeration=12.0, grid_size=grid, interpolation=interp)
    rp, col, val, _ = O.tsne_csr(idx, dist, 15.0)
    # attractive: FP64 restatement of add_sparse_attractive_gradient_f on the same P
    diff = y[:, None, :].astype(np.float64)
    rows = np.repeat(np.arange(n), np.diff(rp))
    dv = y[rows].astype(np.float64) - y[col].astype(np.float64)
    q = 1.0 / (1.0 + (dv ** 2).sum(1))
    att64 = np.zeros((n, 2))
    np.add.at(att64, rows, 12.0 * val.astype(np.float64)[:, None] * q[:, None] * dv)
    assert rel_l2(d["attractive_force"], att64) < 1e-4
    # repulsion vs the FP64 oracle of the same interpolation scheme
    rep64, z64 = O.interp_rep_f64(y, grid, interp)
    assert rel_l2(d["repulsive_force_fft"], rep64) < 1e-4
    assert d["z_grid"] == pytest.approx(z64, rel=1e-4)
    # exact repulsion and Z vs the FP64 dense oracle
    ex64, zex = O.exact_rep_f64(y)
    assert rel_l2(d["repulsive_force_exact"], ex64) < 1e-5
    assert d["sum_q"] == pytest.approx(zex, rel=1e-7)  # FP32 pair terms, FP64 sums
    # KL vs evaluate_kl_f
    assert d["kl"] == pytest.approx(O.kl(rp, col, val, y), rel=1e-6)
    del diff


def test_interpolation_error_vs_exact_repulsion(small):
    """Approximation error of the grid repulsion against exact FP64 repulsion (N <= 20k),
    reference thresholds of tests/testthat/test-tsne-numerics.R:68-95 for the bilinear stencil."""
    idx, dist, _ = small
    n = idx.shape[0]
    y = (np.random.default_rng(9).standard_normal((n, 2)) * 0.3).astype(np.float32)
    ex64, _ = O.exact_rep_f64(y)
    errs = {}
    for interp in (0, 1):
        for grid, lim in ((32, 1e-2), (64, 3e-3), (128, 1e-3)):
            d = api.tsne_force_diagnostic(idx, dist, y, 15.0, grid_size=grid, interpolation=interp, exact=False,
                                          kl=False)
            errs[(interp, grid)] = rel_l2(d["repulsive_force_fft"], ex64)
            assert errs[(interp, grid)] < lim
            assert np.corrcoef(d["repulsive_force_fft"].ravel(), ex64.ravel())[0, 1] > 0.999
        assert errs[(interp, 32)] > errs[(interp, 64)] > errs[(interp, 128)]
    for grid in (32, 64, 128):
        assert errs[(1, grid)] < errs[(0, grid)]


def test_first_step_matches_reference_cpu(monkeypatch):
    """tests/testthat/test-tsne-numerics.R:239-316: one step from the same Y_init, grid 64."""
    rng = np.random.default_rng(706)
    x = rng.standard_normal((64, 6)).astype(np.float32)
    idx, dist = synthetic.exact_knn_numpy(x, 15)
    init = rng.normal(0, 1e-4, (64, 2)).astype(np.float32)
    monkeypatch.setenv("FASTEMBEDR_TSNE_FFT_GRID", "64")
    monkeypatch.setenv("FASTEMBEDR_TSNE_INTERPOLATION", "bilinear")
    fit = api.tsne_knn(idx, dist, n_neighbors=15, perplexity=5, Y_init=init, early_exaggeration_iter=0, n_iter=1,
                       early_exaggeration=1, exaggeration=1, learning_rate=1, initial_momentum=0, final_momentum=0,
                       max_step_norm=1e6, auto_config=False)
    cpu = O.tsne_run(idx, dist, init, perplexity=5, early_iter=0, n_iter=1, early_exag=1, exag=1, learning_rate=1,
                     m0=0, m1=0, max_step_norm=1e6, grid=64)
    assert rel_l2(fit.layout, cpu.astype(np.float64)) < 2e-3


@pytest.mark.parametrize("case", ["duplicated", "coincident", "extreme", "disconnected"])
def test_pathological_inputs_stay_finite(golden, case):
    g = golden("force_" + case)
    d = api.tsne_force_diagnostic(g["idx"], g["dist"], g["layout"], 2.0, grid_size=64, interpolation=1)
    for key in ("attractive_force", "repulsive_force_fft", "repulsive_force_exact"):
        assert np.all(np.isfinite(d[key])), key
    assert np.isfinite(d["kl"]) and d["sum_q"] > 0
    fit = api.tsne_knn(g["idx"], g["dist"], n_neighbors=g["idx"].shape[1], perplexity=2, Y_init=g["layout"],
                       early_exaggeration_iter=0, n_iter=1, early_exaggeration=1, exaggeration=1, learning_rate=1,
                       initial_momentum=0, final_momentum=0, max_step_norm=1e6, auto_config=False)
    assert np.all(np.isfinite(fit.layout))


def test_invalid_inputs_are_rejected(golden):
    g = golden("force_duplicated")
    bad = g["idx"].copy()
    bad[0, 0] = 10**6
    with pytest.raises(_lib.CudaEmbeddingError, match="out of range"):
        api.tsne_knn(bad, g["dist"], perplexity=2, n_iter=1, early_exaggeration_iter=0)
    dist = g["dist"].copy()
    dist[1, 1] = np.inf
    with pytest.raises(_lib.CudaEmbeddingError, match="finite"):
        api.tsne_knn(g["idx"], dist, perplexity=2, n_iter=1, early_exaggeration_iter=0)
    layout = g["layout"].copy()
    layout[0, 0] = np.inf
    with pytest.raises(ValueError, match="finite"):
        api.tsne_knn(g["idx"], g["dist"], perplexity=2, Y_init=layout, n_iter=1, early_exaggeration_iter=0)
    with pytest.raises(_lib.CudaEmbeddingError, match="finite"):
        api.tsne_force_diagnostic(g["idx"], g["dist"], layout, 2.0)


def test_end_to_end_plain_10k_kl_and_preservation(c1, monkeypatch):
    """(d): full 250 + 750 iteration run vs the reference CPU run (the oracle, bit-identical to it).

    At the reference CPU's own grid (bilinear, 128 nodes for n < 50k) the GPU run must match it
    two-sided: KL within 1 %, 15-NN preservation within 0.01. With the default CUDA grid policy
    (256 nodes, as the reference CUDA backend) the GPU run may only be better: KL at most 1 %
    above, preservation at most 0.01 below."""
    idx, dist, _ = c1
    n = idx.shape[0]
    init = synthetic.tsne_init(n, 7)
    cpu = O.tsne_run(idx, dist, init, perplexity=30, early_iter=250, n_iter=750, learning_rate=n / 12.0)
    rp, col, val, _ = O.tsne_csr(idx, dist, 30.0)
    keep = np.arange(0, n, 5, dtype=np.int32)
    kl_cpu = O.kl(rp, col, val, cpu)
    pc = O.knn_preservation(cpu, idx, keep=keep, preserve_k=15)
    monkeypatch.setenv("FASTEMBEDR_TSNE_FFT_GRID", "128")
    fit = api.tsne_knn(idx, dist, perplexity=30, Y_init=init, early_exaggeration_iter=250, n_iter=750)
    kl_gpu = O.kl(rp, col, val, fit.layout)
    pg = O.knn_preservation(fit.layout, idx, keep=keep, preserve_k=15)
    assert abs(kl_gpu - kl_cpu) / kl_cpu < 0.01, (kl_gpu, kl_cpu)
    assert abs(pg - pc) < 0.01, (pg, pc)
    monkeypatch.delenv("FASTEMBEDR_TSNE_FFT_GRID")
    fit = api.tsne_knn(idx, dist, perplexity=30, Y_init=init, early_exaggeration_iter=250, n_iter=750)
    assert fit.config["fft_grid_size"] == 256
    kl_d = O.kl(rp, col, val, fit.layout)
    pd = O.knn_preservation(fit.layout, idx, keep=keep, preserve_k=15)
    assert kl_d < kl_cpu * 1.01, (kl_d, kl_cpu)
    assert pd > pc - 0.01, (pd, pc)


def test_identical_runs_give_identical_layouts(c1):
    """The whole 250 + 750 iteration job is deterministic: the grid charges are summed as 64-bit
    fixed-point integers (order-independent) and every float reduction has a fixed order, so two
    runs on the same input return the same bits."""
    idx, dist, _ = c1
    n = idx.shape[0]
    init = synthetic.tsne_init(n, 7)
    a = api.tsne_knn(idx, dist, perplexity=30, Y_init=init, early_exaggeration_iter=250, n_iter=750)
    b = api.tsne_knn(idx, dist, perplexity=30, Y_init=init, early_exaggeration_iter=250, n_iter=750)
    assert np.array_equal(a.layout, b.layout)


def test_plan_graph_and_eager_paths_agree(small):
    import torch

    idx, dist, _ = small
    n, k = idx.shape
    d_idx = torch.as_tensor(np.ascontiguousarray(idx.T), device="cuda")
    d_dist = torch.as_tensor(np.ascontiguousarray(dist.T), device="cuda")
    init = synthetic.tsne_init(n, 8)
    outs = []
    for graph in (True, False):
        plan = api.TsnePlan(d_idx, d_dist, n, k, 15.0, init=init)
        plan.run(5, 12.0, n / 12.0, graph=graph)
        outs.append(plan.layout())
        info = plan.info()
        plan.close()
    assert info["launches_per_iteration"] == 6
    # grid charges are fixed-point integer sums and every other reduction has a fixed order, so a
    # graph replay and eager launches give the same bits
    assert np.array_equal(outs[0], outs[1])


def test_spatial_reorder_preserves_results(small, monkeypatch):
    """Periodic spatial reordering permutes storage and relabels P's columns; results, the
    returned order and the KL must not change (up to rounding: the storage order decides which
    points share a warp's float run sums in the scatter)."""
    import torch

    idx, dist, _ = small
    n, k = idx.shape
    d_idx = torch.as_tensor(np.ascontiguousarray(idx.T), device="cuda")
    d_dist = torch.as_tensor(np.ascontiguousarray(dist.T), device="cuda")
    init = (np.random.default_rng(3).standard_normal((n, 2)) * 3).astype(np.float32)
    outs, kls, firsts = [], [], []
    for flag in ("0", "1"):
        monkeypatch.setenv("FASTEMBEDR_TSNE_REORDER", flag)
        plan = api.TsnePlan(d_idx, d_dist, n, k, 15.0, init=init)
        plan.run(1, 1.0, n / 12.0)
        firsts.append(plan.layout())
        plan.run(29, 1.0, n / 12.0)
        outs.append(plan.layout())
        kls.append(plan.kl())
        plan.close()
    # one iteration: rounding only; 30 iterations: that rounding grows chaotically but stays far
    # below what a wrong permutation or relabelling would give (order 1)
    assert rel_l2(firsts[1], firsts[0].astype(np.float64)) < 1e-6
    assert rel_l2(outs[1], outs[0].astype(np.float64)) < 1e-3
    rp, col, val, _ = O.tsne_csr(idx, dist, 15.0)
    for y, kv in zip(outs, kls):
        assert kv == pytest.approx(O.kl(rp, col, val, y), rel=1e-5)


def test_plan_gradient_check_matches_diagnostic_and_oracle(c1):
    """Gradient check of a resident run at a seeded sample: the exact part against the FP64 oracle
    on the plan's layout, the grid part and the attraction against the force diagnostic on the
    same layout and grid, and the size of the grid approximation error."""
    import torch

    idx, dist, _ = c1
    n, k = idx.shape
    d_idx = torch.as_tensor(np.ascontiguousarray(idx.T), device="cuda")
    d_dist = torch.as_tensor(np.ascontiguousarray(dist.T), device="cuda")
    plan = api.TsnePlan(d_idx, d_dist, n, k, 30.0, init=synthetic.tsne_init(n, 5))
    plan.run(250, 12.0, n / 12.0)
    plan.run(100, 1.0, n / 12.0)
    chk = plan.gradient_check(sample=2000, seed=1)
    y = plan.layout()
    grid = plan.info()["grid_size"]
    # the check leaves the optimizer state alone: the next iterations continue as before
    plan.run(5, 1.0, n / 12.0)
    assert np.all(np.isfinite(plan.layout()))
    plan.close()
    rows = chk["rows"]
    assert rows.shape == (2000,) and np.all(np.diff(rows) > 0)
    ex64, z64 = O.exact_rep_f64(y)
    assert chk["z_exact"] == pytest.approx(z64, rel=1e-6)
    assert rel_l2(chk["repulsive_exact"], ex64[rows]) < 1e-5
    d = api.tsne_force_diagnostic(idx, dist, y, 30.0, grid_size=grid, exact=False, kl=False)
    assert rel_l2(chk["attractive"], d["attractive_force"][rows].astype(np.float64)) < 1e-5
    assert rel_l2(chk["repulsive_grid"], d["repulsive_force_fft"][rows].astype(np.float64)) < 1e-3
    assert chk["z_grid"] == pytest.approx(d["z_grid"], rel=1e-4)
    # grid approximation error: the gradient is a small difference of attraction and repulsion
    # once the layout has settled, so its relative error is several times the repulsion's
    assert abs(chk["z_rel_err"]) < 1e-2
    assert chk["repulsion_rel_l2"] < 0.05, chk["repulsion_rel_l2"]
    assert chk["gradient_rel_l2"] < 0.25, chk["gradient_rel_l2"]


def test_device_knn_entry_matches_reference_cpu(c1, monkeypatch):
    """GPU-resident KNN ingestion: the device-pointer entry point on a column-major, 1-based
    device KNN (the layout of the package's GPU KNN object) runs the full 250 + 750 schedule at the
    reference CPU's grid and matches the reference CPU run (oracle): KL within 1 %, 15-NN
    preservation within 0.01. It is also the host entry point's result bit for bit."""
    import torch

    idx, dist, _ = c1
    n, k = idx.shape
    init = synthetic.tsne_init(n, 7)
    monkeypatch.setenv("FASTEMBEDR_TSNE_FFT_GRID", "128")
    lib = _lib.require_gpu()
    d_idx = torch.as_tensor(np.ascontiguousarray((idx + 1).T.astype(np.int32)), device="cuda")
    d_dist = torch.as_tensor(np.ascontiguousarray(dist.T.astype(np.float32)), device="cuda")
    torch.cuda.synchronize()
    out = np.zeros((n, 2), np.float32)
    st = lib.fastembedr_cuda_opentsne_fft_from_device_knn_float(
        d_idx.data_ptr(), d_dist.data_ptr(), init.ctypes.data, 1, n, k, 2, 30.0, 250, 750, 12.0, 1.0, n / 12.0, 0,
        0.8, 0.8, 0.01, 5.0, 4, 1, out.ctypes.data)
    _lib.check(st, "t-SNE from device KNN")
    host = api.tsne_knn(idx, dist, perplexity=30, Y_init=init, early_exaggeration_iter=250, n_iter=750)
    assert np.array_equal(out, host.layout)
    cpu = O.tsne_run(idx, dist, init, perplexity=30, early_iter=250, n_iter=750, learning_rate=n / 12.0)
    rp, col, val, _ = O.tsne_csr(idx, dist, 30.0)
    keep = np.arange(0, n, 5, dtype=np.int32)
    kl_cpu, kl_gpu = O.kl(rp, col, val, cpu), O.kl(rp, col, val, out)
    assert abs(kl_gpu - kl_cpu) / kl_cpu < 0.01, (kl_gpu, kl_cpu)
    pc = O.knn_preservation(cpu, idx, keep=keep, preserve_k=15)
    pg = O.knn_preservation(out, idx, keep=keep, preserve_k=15)
    assert abs(pg - pc) < 0.01, (pg, pc)


def test_attractive_launch_tuning_changes_no_result(small, monkeypatch):
    """The run-time tuner of the attractive pass times (chunk size, resident blocks) candidates on
    the first normal-phase run and keeps the fastest; the pass's result does not depend on the
    launch, so a tuned plan and an untuned one give the same bits."""
    import torch

    idx, dist, _ = small
    n, k = idx.shape
    d_idx = torch.as_tensor(np.ascontiguousarray(idx.T), device="cuda")
    d_dist = torch.as_tensor(np.ascontiguousarray(dist.T), device="cuda")
    init = synthetic.tsne_init(n, 9)
    outs, tunes = [], []
    for flag in ("1", "0"):
        monkeypatch.setenv("FASTEMBEDR_TSNE_AUTOTUNE", flag)
        plan = api.TsnePlan(d_idx, d_dist, n, k, 15.0, init=init)
        plan.run(50, 12.0, n / 12.0)
        plan.run(50, 1.0, n / 12.0)
        outs.append(plan.layout())
        tunes.append(plan.tuning())
        plan.close()
    assert len(tunes[0]["candidates"]) == 6 and all(c["ms"] > 0 for c in tunes[0]["candidates"])
    best = min(tunes[0]["candidates"], key=lambda c: c["ms"])
    assert (tunes[0]["chunk"], tunes[0]["blocks"]) == (best["chunk"], best["blocks"])
    assert tunes[1]["candidates"] == []
    assert np.array_equal(outs[0], outs[1])


def test_double_distance_entry_matches_float_entry(small):
    """The double-distance entry point (R's numeric KNN distances; the reference casts them to
    float, copy_distances_float_sexp in src/tsne_neighbors.cpp:338-363) gives the float entry
    point's layout bit for bit on float-exact distances, with 1-based labels as R passes them."""
    idx, dist, _ = small
    n, k = idx.shape
    lib = _lib.require_gpu()
    init = synthetic.tsne_init(n, 11)
    idx_cm = np.asfortranarray((idx + 1).astype(np.int32))
    outs = []
    for fn, d in ((lib.fastembedr_cuda_opentsne_fft_from_knn_float, np.asfortranarray(dist.astype(np.float32))),
                  (lib.fastembedr_cuda_opentsne_fft_from_knn, np.asfortranarray(dist.astype(np.float32).astype(np.float64)))):
        out = np.zeros((n, 2), np.float32)
        st = fn(idx_cm.ctypes.data, d.ctypes.data, init.ctypes.data, 1, n, k, 2, 15.0, 60, 60, 12.0, 1.0, n / 12.0, 0,
                0.8, 0.8, 0.01, 5.0, 4, 1, out.ctypes.data)
        _lib.check(st, "t-SNE entry")
        outs.append(out)
    assert np.all(np.isfinite(outs[0])) and outs[0].std() > 1e-3
    assert np.array_equal(outs[0], outs[1])
