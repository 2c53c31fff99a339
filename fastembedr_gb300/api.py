"""Python mirror of fastEmbedR's R-facing entry points for the CUDA backend.

R is the reference's host language; this module restates the same signatures, argument
meaning, defaults and recorded configuration (``attr(layout, "fastEmbedR_config")`` /
``fit$parameters``) over the C ABI, so that the tests and the benchmark drive the library the
way ``tsne_knn(..., backend = "cuda")`` drives ``knn_tsne_opentsne_cuda_float_cpp``.

Inputs follow the R conventions: ``indices`` is an (n, k) integer matrix (1- or 0-based, self
excluded or not), ``distances`` the matching (n, k) matrix; layouts are (n, 2) arrays.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np

from . import _lib


def _colmajor(a, dtype):
    return np.asfortranarray(np.asarray(a, dtype=dtype))


def _settle(*tensors):
    """The library reads device inputs on its own streams: finish the producer's stream first
    (torch tensors written on a non-default stream are not covered by the legacy-stream order
    the library applies itself)."""
    for t in tensors:
        if getattr(t, "is_cuda", False):
            import torch

            torch.cuda.current_stream(t.device).synchronize()
            return


def knn_index_offset(indices) -> int:
    """1 when every index lies in [1, n], else 0 (src/embedding_cuda_impl.cpp:933,
    src/tsne_neighbors.cpp:90-101)."""
    idx = np.asarray(indices)
    n = idx.shape[0]
    return 1 if idx.min() >= 1 and idx.max() <= n else 0


@dataclass
class TsneFit:
    layout: np.ndarray
    config: dict = field(default_factory=dict)


def fft_grid_size(n: int) -> int:
    return int(_lib.load().fastembedr_cuda_opentsne_fft_grid_size(int(n)))


def tsne_knn(indices, distances, n_neighbors=None, perplexity=None, n_components=2, Y_init=None, seed=4,
             learning_rate="auto", early_exaggeration_iter=None, early_exaggeration="auto", n_iter=None,
             exaggeration=None, initial_momentum=0.8, final_momentum=0.8, max_step_norm="auto",
             negative_gradient_method="auto", min_gain=0.01, auto_config=True, backend="cuda") -> TsneFit:
    """t-SNE from a supplied KNN graph (R/fast_knn_tsne.R:216-261, policy of R/tsne_control.R:113-231
    and R/tsne_optimizer_helpers.R:151-221), run by the GB300 library."""
    if backend != "cuda":
        raise ValueError("fastembedr_gb300 implements backend = 'cuda' only")
    method = str(negative_gradient_method).lower()
    if method not in ("fft", "fitsne", "fit_sne", "interpolation", "auto"):
        raise ValueError('CUDA openTSNE supports `negative_gradient_method = "fft"` only.')
    if int(n_components) != 2:
        raise ValueError("CUDA openTSNE FFT-grid currently supports exactly two output components.")
    idx = np.asarray(indices)
    dist = np.asarray(distances, np.float32)
    if idx.shape != dist.shape or idx.ndim != 2:
        raise ValueError("KNN `indices` and `distances` must have the same dimensions.")
    k_all = idx.shape[1]
    k = int(n_neighbors) if n_neighbors is not None else k_all
    idx = idx[:, :k]
    dist = dist[:, :k]
    n = idx.shape[0]
    # tsne_auto_parameters_cpp, src/tsne_neighbors.cpp:1820-1868
    max_pn, max_pk = max(1, (n - 1) // 3), max(1, k // 3)
    perp = float(min(30, max_pn, max_pk)) if perplexity is None else float(perplexity)
    if perplexity is None:
        perp = max(1.0, min(perp, float(min(max_pn, max_pk))))
    ee_iter = 250 if early_exaggeration_iter is None else int(early_exaggeration_iter)
    nn_iter = 500 if n_iter is None else int(n_iter)
    ee = 12.0 if (isinstance(early_exaggeration, str) and early_exaggeration == "auto") else float(early_exaggeration)
    ex = 1.0 if exaggeration is None else float(exaggeration)
    opt_sne = bool(auto_config) and isinstance(learning_rate, str) and learning_rate.lower() == "auto"
    if opt_sne:
        lr_auto, lr_value = 0, n / 12.0
    elif isinstance(learning_rate, str):
        lr_auto, lr_value = 1, -1.0
    else:
        lr_auto, lr_value = 0, float(learning_rate)
    if isinstance(max_step_norm, str):
        msn = 5.0
    elif max_step_norm is None or (isinstance(max_step_norm, float) and math.isnan(max_step_norm)):
        msn = float("nan")
    else:
        msn = float(max_step_norm)
    has_init = Y_init is not None
    init = np.ascontiguousarray(Y_init, np.float32) if has_init else np.zeros((n, 2), np.float32)
    if has_init and init.shape != (n, 2):
        raise ValueError("CUDA openTSNE FFT-grid requires a two-dimensional initialization.")
    if has_init and not np.all(np.isfinite(init)):
        raise ValueError("`Y_init` must contain only finite coordinates.")
    out = np.zeros((n, 2), np.float32)
    lib = _lib.require_gpu()
    idx_cm = _colmajor(idx, np.int32)
    dist_cm = _colmajor(dist, np.float32)
    st = lib.fastembedr_cuda_opentsne_fft_from_knn_float(
        idx_cm.ctypes.data, dist_cm.ctypes.data, init.ctypes.data, int(has_init), n, k, 2, perp, ee_iter, nn_iter,
        ee, ex, lr_value, lr_auto, float(initial_momentum), float(final_momentum), float(min_gain), msn,
        int(seed) & 0xFFFFFFFF, knn_index_offset(idx), out.ctypes.data)
    _lib.check(st, "CUDA openTSNE FFT-grid")
    lr_early = n / ee if lr_auto else lr_value
    lr_normal = n / max(ex, 1.0) if lr_auto else lr_value
    config = dict(
        method="tsne", backend="cuda", n=n, n_neighbors=k, perplexity=perp, early_exaggeration_iter=ee_iter,
        n_iter=nn_iter, max_iter=ee_iter + nn_iter, early_exaggeration_iter_actual=ee_iter, n_iter_actual=nn_iter,
        max_iter_actual=ee_iter + nn_iter,
        learning_rate="auto_opt_sne_n_over_early_exaggeration" if opt_sne else ("auto" if lr_auto else lr_value),
        learning_rate_early=lr_early, learning_rate_normal=lr_normal, early_exaggeration=ee, exaggeration=ex,
        initial_momentum=float(initial_momentum), final_momentum=float(final_momentum), min_gain=float(min_gain),
        max_step_norm=msn, optimizer="opentsne_fitsne_fft_grid_native_cuda", repulsion="fft_grid_cuda_gb300",
        fft_grid_size=fft_grid_size(n), probabilities="symmetric_sparse_knn_cuda_float32", precision="float32",
        auto_kld_stop=False, auto_stop_reason="cuda_fft_no_host_kld_monitor", seed=int(seed))
    return TsneFit(out, config)


def tsne_pca_init(data):
    """PCA start of t-SNE computed on the GPU (make_cuda_opentsne_pca_init, R/tsne_pca_init.R:28-50,
    and normalize_opentsne_pca_scores, R/tsne_control.R:515-540): the two leading principal
    components of the centred data, each signed so its largest-magnitude score is positive,
    centred and scaled so the larger standard deviation is 1e-4. (n, 2) float32."""
    x = np.asarray(data)
    is_double = x.dtype != np.float32
    xc = np.asfortranarray(x, np.float64 if is_double else np.float32)
    n, p = xc.shape
    out = np.zeros((n, 2), np.float32)
    st = _lib.require_gpu().fastembedr_cuda_tsne_pca_init(xc.ctypes.data, int(is_double), n, p, out.ctypes.data)
    _lib.check(st, "CUDA PCA initialization")
    return out


def tsne_affinities(indices, distances, perplexity, index_offset=None):
    """Symmetrised CSR P and directed P / entropies from the GPU (diagnostic)."""
    idx = np.asarray(indices)
    n, k = idx.shape
    off = knn_index_offset(idx) if index_offset is None else int(index_offset)
    cap = 2 * n * k
    rp = np.zeros(n + 1, np.int32)
    col = np.zeros(cap, np.int32)
    val = np.zeros(cap, np.float32)
    p = np.zeros((n, k), np.float32)
    h = np.zeros(n, np.float64)
    nnz = C.c_longlong()
    tot = C.c_double()
    lib = _lib.require_gpu()
    idx_cm, dist_cm = _colmajor(idx, np.int32), _colmajor(distances, np.float32)  # kept alive across the call
    st = lib.fastembedr_cuda_tsne_affinities(idx_cm.ctypes.data, dist_cm.ctypes.data, n, k, float(perplexity),
                                             off, rp.ctypes.data, col.ctypes.data, val.ctypes.data, cap,
                                             C.byref(nnz), p.ctypes.data, h.ctypes.data, C.byref(tot))
    _lib.check(st, "CUDA t-SNE affinities")
    m = nnz.value
    return dict(row_ptr=rp, col=col[:m].copy(), val=val[:m].copy(), p_directed=p, entropy=h, total_mass=tot.value)


def tsne_force_diagnostic(indices, distances, layout, perplexity, exaggeration=1.0, grid_size=0, interpolation=0,
                          exact=True, kl=True, index_offset=None):
    """GPU twin of opentsne_force_diagnostic_cpp (src/tsne_neighbors.cpp:1698-1817)."""
    idx = np.asarray(indices)
    n, k = idx.shape
    off = knn_index_offset(idx) if index_offset is None else int(index_offset)
    y = np.ascontiguousarray(layout, np.float32)
    att = np.zeros((n, 2), np.float32)
    rep = np.zeros((n, 2), np.float32)
    rex = np.zeros((n, 2), np.float32) if exact else None
    zg, ze, kv = C.c_double(), C.c_double(), C.c_double()
    lib = _lib.require_gpu()
    idx_cm, dist_cm = _colmajor(idx, np.int32), _colmajor(distances, np.float32)  # kept alive across the call
    st = lib.fastembedr_cuda_tsne_force_diagnostic(
        idx_cm.ctypes.data, dist_cm.ctypes.data, y.ctypes.data, n, k,
        float(perplexity), float(exaggeration), int(grid_size), int(interpolation), off, att.ctypes.data,
        rep.ctypes.data, C.byref(zg), rex.ctypes.data if exact else None, C.byref(ze) if exact else None,
        C.byref(kv) if kl else None)
    _lib.check(st, "CUDA t-SNE force diagnostic")
    out = dict(attractive_force=att, repulsive_force_fft=rep, z_grid=zg.value)
    if exact:
        out.update(repulsive_force_exact=rex, sum_q=ze.value)
    if kl:
        out["kl"] = kv.value
    return out


class TsnePlan:
    """Resident t-SNE instance (P, layout and optimizer state stay in HBM).

    ``indices`` / ``distances`` are device tensors (column-major n x k, i.e. the transpose of a
    row-major (k, n) tensor) or anything exposing ``data_ptr()``.
    """

    def __init__(self, d_indices_cm, d_distances_cm, n, k, perplexity, init=None, index_offset=0, grid_size=0,
                 interpolation=0, seed=4):
        self.lib = _lib.require_gpu()
        self.n = int(n)
        _settle(d_indices_cm, d_distances_cm)
        h = C.c_void_p()
        init_a = None if init is None else np.ascontiguousarray(init, np.float32)
        st = self.lib.fastembedr_tsne_plan_create(_lib.ptr(d_indices_cm), _lib.ptr(d_distances_cm),
                                                  None if init_a is None else init_a.ctypes.data, self.n, int(k),
                                                  float(perplexity), int(index_offset), int(grid_size),
                                                  int(interpolation), int(seed) & 0xFFFFFFFF, C.byref(h))
        _lib.check(st, "t-SNE plan create")
        self.h = h

    def run(self, iters, exaggeration, learning_rate, momentum=0.8, min_gain=0.01, max_step_norm=5.0, graph=True):
        _lib.check(self.lib.fastembedr_tsne_plan_run(self.h, int(iters), float(exaggeration), float(learning_rate),
                                                     float(momentum), float(min_gain), float(max_step_norm),
                                                     int(bool(graph))), "t-SNE plan run")

    def profile(self, iters, exaggeration, learning_rate, momentum=0.8, min_gain=0.01, max_step_norm=5.0):
        tot, stp, grd = C.c_float(), C.c_float(), C.c_float()
        _lib.check(self.lib.fastembedr_tsne_plan_profile(self.h, int(iters), float(exaggeration),
                                                         float(learning_rate), float(momentum), float(min_gain),
                                                         float(max_step_norm), C.byref(tot), C.byref(stp),
                                                         C.byref(grd)), "t-SNE plan profile")
        return dict(total_ms=tot.value, attractive_kernel_ms=stp.value, grid_stage_ms=grd.value)

    def synchronize(self):
        _lib.check(self.lib.fastembedr_tsne_plan_synchronize(self.h), "t-SNE plan synchronize")

    @property
    def stream(self) -> int:
        return int(self.lib.fastembedr_tsne_plan_stream(self.h) or 0)

    def layout(self):
        out = np.zeros((self.n, 2), np.float32)
        _lib.check(self.lib.fastembedr_tsne_plan_layout(self.h, out.ctypes.data), "t-SNE plan layout")
        return out

    def info(self):
        nnz, g, it, la, lr = C.c_longlong(), C.c_int(), C.c_int(), C.c_int(), C.c_int()
        _lib.check(self.lib.fastembedr_tsne_plan_info(self.h, C.byref(nnz), C.byref(g), C.byref(it), C.byref(la),
                                                      C.byref(lr)), "t-SNE plan info")
        return dict(nnz=nnz.value, grid_size=g.value, interpolation=it.value, launches_per_iteration=la.value,
                    launches_per_reorder=lr.value)

    def tuning(self):
        """The attractive pass's run-time launch choice and the candidates it timed."""
        ch, bl, cnt = C.c_int(), C.c_int(), C.c_int()
        cap = 16
        cc, cb, cm = np.zeros(cap, np.int32), np.zeros(cap, np.int32), np.zeros(cap, np.float32)
        _lib.check(self.lib.fastembedr_tsne_plan_tuning(self.h, C.byref(ch), C.byref(bl), cap, C.byref(cnt),
                                                        cc.ctypes.data, cb.ctypes.data, cm.ctypes.data),
                   "t-SNE plan tuning")
        m = min(cnt.value, cap)
        return dict(chunk=ch.value, blocks=bl.value,
                    candidates=[dict(chunk=int(cc[i]), blocks=int(cb[i]), ms=float(cm[i])) for i in range(m)])

    def kl(self):
        v = C.c_double()
        _lib.check(self.lib.fastembedr_tsne_plan_kl(self.h, C.byref(v)), "t-SNE plan KL")
        return v.value

    def gradient_check(self, sample=20000, seed=0, exaggeration=1.0):
        """Grid gradient of the current layout against the exact FP64-summed repulsion at a seeded
        sample of points (``sample`` ids drawn without replacement, or an array of ids)."""
        if np.ndim(sample) == 0:
            rows = np.sort(np.random.default_rng(seed).choice(self.n, min(int(sample), self.n), replace=False))
        else:
            rows = np.asarray(sample)
        rows = np.ascontiguousarray(rows, np.int32)
        m = rows.shape[0]
        attr = np.zeros((m, 2), np.float32)
        rep = np.zeros((m, 2), np.float32)
        rex = np.zeros((m, 2), np.float64)
        zg, ze = C.c_double(), C.c_double()
        _lib.check(self.lib.fastembedr_tsne_plan_gradient_check(self.h, rows.ctypes.data, m, float(exaggeration),
                                                                attr.ctypes.data, rep.ctypes.data, rex.ctypes.data,
                                                                C.byref(zg), C.byref(ze)), "t-SNE gradient check")
        g_grid = attr.astype(np.float64) + rep
        g_exact = attr.astype(np.float64) + rex
        rel = lambda a, b: float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
        return dict(rows=rows, attractive=attr, repulsive_grid=rep, repulsive_exact=rex, z_grid=zg.value,
                    z_exact=ze.value, z_rel_err=(zg.value - ze.value) / ze.value,
                    repulsion_rel_l2=rel(rep, rex), gradient_rel_l2=rel(g_grid, g_exact),
                    repulsion_max_rel=float(np.max(np.linalg.norm(rep - rex, axis=1))
                                            / max(np.max(np.linalg.norm(rex, axis=1)), 1e-300)))

    def close(self):
        if getattr(self, "h", None):
            self.lib.fastembedr_tsne_plan_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------- UMAP
def _concat_knn(knns):
    """Column-major KNN blocks of the instances, one after another (int32 / float32)."""
    idx = np.concatenate([np.asfortranarray(np.asarray(i, np.int32)).ravel(order="F") for i, _ in knns])
    dist = np.concatenate([np.asfortranarray(np.asarray(d, np.float32)).ravel(order="F") for _, d in knns])
    return idx, dist


class TsneBatch:
    """Many independent t-SNE instances optimised together (C ABI fastembedr_tsne_batch_*).

    ``knns`` is a list of ``(indices, distances)`` pairs, one (n_b, k) KNN per instance with its
    own 0- or 1-based row numbers. Every instance follows the single-instance algorithm with its
    own grid, bounding box, Z and learning rate (opt-SNE: n_b / early exaggeration). ``grid_size``:
    "cuda" (the CUDA size policy, 256 / 512 / 1024 nodes by n), "cpu" (the reference CPU policy,
    128 / 256), "adaptive" (per instance and per 25-iteration chunk, the smallest grid of at least
    256 nodes with node spacing <= 0.7 over the current layout) or a power of two for every
    instance."""

    def __init__(self, knns, perplexity=30.0, inits=None, grid_size="cuda", interpolation=0, seed=4):
        grid_size = {"cuda": 0, "cpu": -1, "adaptive": -2}.get(grid_size, grid_size)
        if not knns:
            raise ValueError("at least one instance is required")
        ks = {np.asarray(i).shape[1] for i, _ in knns}
        if len(ks) != 1:
            raise ValueError("every instance needs the same number of neighbours")
        self.k = ks.pop()
        self.sizes = np.array([np.asarray(i).shape[0] for i, _ in knns], np.int32)
        # one row-major array per instance, passed by pointer (no concatenated copy); each
        # instance's 0- or 1-based labels are detected on the device
        idx = [np.ascontiguousarray(i, np.int32) for i, _ in knns]
        dist = [np.ascontiguousarray(d, np.float32) for _, d in knns]
        ys = None if inits is None else [np.ascontiguousarray(y, np.float32) for y in inits]
        ptrs = lambda arrs: (C.c_void_p * len(arrs))(*[a.ctypes.data for a in arrs])
        self.lib = _lib.require_gpu()
        self.h = C.c_void_p()
        st = self.lib.fastembedr_tsne_batch_create_rows(len(knns), self.sizes.ctypes.data, ptrs(idx), ptrs(dist),
                                                        None if ys is None else ptrs(ys), self.k, float(perplexity),
                                                        -1, int(grid_size), int(interpolation),
                                                        int(seed) & 0xFFFFFFFF, C.byref(self.h))
        _lib.check(st, "t-SNE batch create")

    @property
    def stream(self):
        return self.lib.fastembedr_tsne_batch_stream(self.h)

    def run(self, early_exaggeration_iter=250, n_iter=750, early_exaggeration=12.0, exaggeration=1.0,
            learning_rate="auto", initial_momentum=0.8, final_momentum=0.8, min_gain=0.01, max_step_norm=5.0):
        """learning_rate: per-point factor (instance b uses learning_rate x n_b in both phases);
        "auto" is the package's opt-SNE rate n_b / early_exaggeration."""
        lr = -1.0 if learning_rate == "auto" else float(learning_rate)
        _lib.check(self.lib.fastembedr_tsne_batch_run(self.h, int(early_exaggeration_iter), int(n_iter),
                                                      float(early_exaggeration), float(exaggeration), lr,
                                                      float(initial_momentum), float(final_momentum), float(min_gain),
                                                      float(max_step_norm)), "t-SNE batch run")

    def iterate(self, iters, exaggeration, learning_rate_per_point, momentum=0.8, min_gain=0.01, max_step_norm=5.0):
        _lib.check(self.lib.fastembedr_tsne_batch_iterate(self.h, int(iters), float(exaggeration),
                                                          float(learning_rate_per_point), float(momentum),
                                                          float(min_gain), float(max_step_norm)), "t-SNE batch iterate")

    def synchronize(self):
        _lib.check(self.lib.fastembedr_tsne_batch_synchronize(self.h), "t-SNE batch synchronize")

    def layouts(self):
        out = np.zeros((int(self.sizes.sum()), 2), np.float32)
        _lib.check(self.lib.fastembedr_tsne_batch_layout(self.h, out.ctypes.data), "t-SNE batch layout")
        return np.split(out, np.cumsum(self.sizes)[:-1])

    def kl(self, instance):
        v = C.c_double()
        _lib.check(self.lib.fastembedr_tsne_batch_kl(self.h, int(instance), C.byref(v)), "t-SNE batch KL")
        return v.value

    def grids(self):
        g = np.zeros(len(self.sizes), np.int32)
        r = C.c_int()
        _lib.check(self.lib.fastembedr_tsne_batch_grids(self.h, g.ctypes.data, C.byref(r)), "t-SNE batch grids")
        return g, r.value

    def info(self):
        nnz, pts, gc, la, lr = C.c_longlong(), C.c_longlong(), C.c_int(), C.c_int(), C.c_int()
        _lib.check(self.lib.fastembedr_tsne_batch_info(self.h, C.byref(nnz), C.byref(pts), C.byref(gc), C.byref(la),
                                                       C.byref(lr)), "t-SNE batch info")
        return dict(nnz=nnz.value, points=pts.value, grid_classes=gc.value, launches_per_iteration=la.value,
                    launches_per_reorder=lr.value)

    def close(self):
        if getattr(self, "h", None):
            self.lib.fastembedr_tsne_batch_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def tsne_knn_batch(knns, perplexity=30.0, inits=None, seed=4, early_exaggeration_iter=250, n_iter=750,
                   early_exaggeration=12.0, exaggeration=1.0, max_step_norm=5.0, grid_size="cuda"):
    """tsne_knn over many instances at once: the package schedule (opt-SNE learning rate per
    instance) on every instance; returns one (n_b, 2) layout per instance."""
    with TsneBatch(knns, perplexity=perplexity, inits=inits, seed=seed, grid_size=grid_size) as b:
        b.run(early_exaggeration_iter, n_iter, early_exaggeration, exaggeration, max_step_norm=max_step_norm)
        return b.layouts()


@dataclass
class UmapFit:
    layout: np.ndarray
    config: dict = field(default_factory=dict)


def umap_graph(indices, distances, index_offset=None):
    """Default fuzzy graph on the GPU (umap_graph_csr_float_cpp, src/fast_knn_umap.cpp:3996)."""
    idx = np.asarray(indices)
    n, k = idx.shape
    off = knn_index_offset(idx) if index_offset is None else int(index_offset)
    cap = 2 * n * k
    offsets = np.zeros(n + 1, np.int32)
    nb = np.zeros(cap, np.int32)
    w = np.zeros(cap, np.float32)
    e = np.zeros(cap, np.float32)
    nnz, mw = C.c_longlong(), C.c_float()
    lib = _lib.require_gpu()
    idx_cm, dist_cm = _colmajor(idx, np.int32), _colmajor(distances, np.float32)
    st = lib.fastembedr_cuda_umap_graph_from_knn(idx_cm.ctypes.data, dist_cm.ctypes.data, n, k, off,
                                                 offsets.ctypes.data, nb.ctypes.data, w.ctypes.data, e.ctypes.data,
                                                 cap, C.byref(nnz), C.byref(mw))
    _lib.check(st, "CUDA UMAP graph")
    m = nnz.value
    return dict(offsets=offsets, neighbors=nb[:m].copy(), weights=w[:m].copy(), epochs_per_sample=e[:m].copy(),
                max_weight=mw.value)


def umap_optimize_coo(heads, tails, weights, epochs_per_sample, init, n_epochs, a, b, negative_sample_rate=5,
                      learning_rate=1.0, repulsion_strength=1.0, seed=42):
    """The reference C ABI entry fastembedr_cuda_umap_optimize_coo on host arrays."""
    h = np.ascontiguousarray(heads, np.int32)
    t = np.ascontiguousarray(tails, np.int32)
    w = np.ascontiguousarray(weights, np.float32)
    e = np.ascontiguousarray(epochs_per_sample, np.float32)
    y0 = np.ascontiguousarray(init, np.float32)
    out = np.zeros_like(y0)
    lib = _lib.require_gpu()
    st = lib.fastembedr_cuda_umap_optimize_coo(h.ctypes.data, t.ctypes.data, w.ctypes.data, e.ctypes.data,
                                               y0.ctypes.data, y0.shape[0], h.size, int(n_epochs),
                                               int(negative_sample_rate), float(learning_rate), float(a), float(b),
                                               float(repulsion_strength), int(seed) & 0xFFFFFFFF, 0, out.ctypes.data)
    _lib.check(st, "CUDA COO UMAP optimizer")
    return out


def umap_ab_params(min_dist, spread=1.0):
    """Curve parameters a, b (find_ab_params, src/fast_knn_umap.cpp:437-497; host code)."""
    a, b = C.c_double(), C.c_double()
    _lib.load().fastembedr_umap_find_ab_params(float(spread), float(min_dist), C.byref(a), C.byref(b))
    return a.value, b.value


def umap_spectral_n_iter(n, k):
    """Diffusion rounds of the package size policy (umap_size_defaults, R/fast_knn_umap.R:947-965)."""
    if n >= 10000:
        return 30 if k <= 15 else 20
    return 60 if n >= 500 else 50


def umap_spectral_init(indices, distances, spectral_n_iter=50, seed=42, index_offset=None):
    """GPU diffusion start of spectral_knn_init(backend = "cuda") (R/fast_knn_umap.R:1309-1341,
    through fastembedr_cuda_spectral_init_from_knn): row-major (n, 2) float32, whitened."""
    idx = np.asarray(indices)
    n, k = idx.shape
    off = knn_index_offset(idx) if index_offset is None else int(index_offset)
    idx_cm, dist_cm = _colmajor(idx, np.int32), _colmajor(distances, np.float64)
    out = np.zeros((n, 2), np.float32)
    st = _lib.require_gpu().fastembedr_cuda_spectral_init_from_knn(idx_cm.ctypes.data, dist_cm.ctypes.data, n, k,
                                                                   int(spectral_n_iter), int(seed) & 0xFFFFFFFF, off,
                                                                   out.ctypes.data)
    _lib.check(st, "CUDA spectral initialization")
    return out


def umap_spectral_start(indices, distances, spectral_n_iter=50, seed=42, init_scale=float("nan"),
                        index_offset=None):
    """The reference CPU spectral start (spectral_knn_init(backend = "cpu"), R/fast_knn_umap.R:1343-1365)
    computed on the GPU: (n, 2) float64, equal to the CPU start to rounding."""
    idx = np.asarray(indices)
    n, k = idx.shape
    off = knn_index_offset(idx) if index_offset is None else int(index_offset)
    idx_cm, dist_cm = _colmajor(idx, np.int32), _colmajor(distances, np.float32)
    out = np.zeros(2 * n)
    st = _lib.require_gpu().fastembedr_cuda_umap_spectral_init_from_knn(idx_cm.ctypes.data, dist_cm.ctypes.data, n,
                                                                        k, off, int(spectral_n_iter),
                                                                        float(init_scale), int(seed), out.ctypes.data)
    _lib.check(st, "CUDA spectral start")
    return out.reshape(2, n).T.copy()


def umap_spectral_start_csr(offsets, neighbors, weights, spectral_n_iter=50, seed=42, init_scale=float("nan")):
    """The reference CPU spectral start of a symmetric CSR graph (umap_init_from_csr_graph,
    R/fast_knn_umap.R:665-689) computed on the GPU: (n, 2) float64."""
    off = np.ascontiguousarray(offsets, np.int32)
    nb = np.ascontiguousarray(neighbors, np.int32)
    w = np.ascontiguousarray(weights, np.float32)
    n = off.size - 1
    out = np.zeros(2 * n)
    st = _lib.require_gpu().fastembedr_cuda_umap_spectral_init_csr(off.ctypes.data, nb.ctypes.data, w.ctypes.data, n,
                                                                   int(spectral_n_iter), float(init_scale), int(seed),
                                                                   out.ctypes.data)
    _lib.check(st, "CUDA spectral start")
    return out.reshape(2, n).T.copy()


def umap_knn(indices, distances, init="spectral", n_components=2, seed=42, n_epochs=None, min_dist=0.01,
             negative_sample_rate=5, learning_rate=1.0, repulsion_strength=1.0, backend="cuda",
             spectral_n_iter=None, graph_mode="fuzzy", init_scale=float("nan")) -> UmapFit:
    """UMAP from a supplied KNN graph (R/fast_knn_umap.R:1444-1462 with the package policy of
    fast_knn_umap_config, :1008-1032: 200 epochs at n >= 10k else 500, min_dist 0.01, negative
    rate 5, lr 1, repulsion 1). ``init``: "spectral" (default) computes the reference's CPU
    spectral start (what umap_knn feeds every backend, R/umap_core_helpers.R:205-243) on the GPU
    and runs graph -> start -> SGD in one call; "diffusion" is the fused GPU path of
    knn_umap_cuda_fused_impl (src/embedding_cuda_impl.cpp:1716-1770) with its diffusion start and
    the "fuzzy" or "binary" (unit weights) graph; an (n, 2) array is used as given.
    ``spectral_n_iter`` defaults to the package size policy."""
    if backend != "cuda":
        raise ValueError("fastembedr_gb300 implements backend = 'cuda' only")
    if int(n_components) != 2:
        raise ValueError("CUDA UMAP requires a two-dimensional initialization.")
    idx = np.asarray(indices)
    n, k = idx.shape
    epochs = (200 if n >= 10000 else 500) if n_epochs is None else int(n_epochs)
    if isinstance(init, str) and init == "spectral":
        rounds = umap_spectral_n_iter(n, k) if spectral_n_iter is None else int(spectral_n_iter)
        out = np.zeros((n, 2), np.float32)
        idx_cm, dist_cm = _colmajor(idx, np.int32), _colmajor(distances, np.float32)
        st = _lib.require_gpu().fastembedr_cuda_umap_knn_spectral(
            idx_cm.ctypes.data, dist_cm.ctypes.data, n, k, knn_index_offset(idx), epochs, int(negative_sample_rate),
            float(learning_rate), float(min_dist), float(repulsion_strength), rounds, float(init_scale),
            int(seed) & 0xFFFFFFFF, out.ctypes.data)
        _lib.check(st, "CUDA UMAP")
        config = dict(method="umap", backend="cuda", n=n, k=k, n_epochs=epochs, min_dist=float(min_dist),
                      negative_sample_rate=int(negative_sample_rate), learning_rate=float(learning_rate),
                      repulsion_strength=float(repulsion_strength), graph_mode="native_csr_graph",
                      init_backend="cuda_spectral_csr", spectral_n_iter=rounds,
                      graph_prep_backend="cuda_fuzzy_csr", optimizer_math="coo_atomic_edge_sampler_philox",
                      seed=int(seed))
        return UmapFit(out, config)
    if isinstance(init, str):
        if init != "diffusion":
            raise ValueError("init must be an (n, 2) array, 'spectral' or 'diffusion'")
        if graph_mode not in ("fuzzy", "binary"):
            raise ValueError("graph_mode must be 'fuzzy' or 'binary'")
        rounds = umap_spectral_n_iter(n, k) if spectral_n_iter is None else int(spectral_n_iter)
        a, b = umap_ab_params(min_dist)
        import torch

        d_idx = torch.as_tensor(_colmajor(idx, np.int32), device="cuda")
        d_dist = torch.as_tensor(_colmajor(distances, np.float32), device="cuda")
        _settle(d_idx, d_dist)
        out = np.zeros((n, 2), np.float32)
        st = _lib.require_gpu().fastembedr_cuda_umap_from_device_knn_spectral_float(
            d_idx.data_ptr(), d_dist.data_ptr(), n, k, epochs, int(negative_sample_rate), float(learning_rate),
            float(a), float(b), float(repulsion_strength), rounds, int(seed) & 0xFFFFFFFF, knn_index_offset(idx), 0,
            int(graph_mode == "binary"), out.ctypes.data)
        _lib.check(st, "fused CUDA UMAP")
        config = dict(method="umap", backend="cuda", n=n, k=k, n_epochs=epochs, min_dist=float(min_dist),
                      negative_sample_rate=int(negative_sample_rate), learning_rate=float(learning_rate),
                      repulsion_strength=float(repulsion_strength), graph_mode=graph_mode,
                      init_backend="cuda_diffusion", spectral_n_iter=rounds,
                      graph_prep_backend="cuda_fuzzy_csr", optimizer_math="coo_atomic_edge_sampler_philox",
                      seed=int(seed))
        return UmapFit(out, config)
    y0 = np.ascontiguousarray(init, np.float32)
    if y0.shape != (n, 2):
        raise ValueError("init row count must match the KNN graph")
    out = np.zeros((n, 2), np.float32)
    lib = _lib.require_gpu()
    idx_cm, dist_cm = _colmajor(idx, np.int32), _colmajor(distances, np.float32)
    st = lib.fastembedr_cuda_umap_from_knn(idx_cm.ctypes.data, dist_cm.ctypes.data, y0.ctypes.data, n, k,
                                           knn_index_offset(idx), epochs, int(negative_sample_rate),
                                           float(learning_rate), float(min_dist), float(repulsion_strength),
                                           int(seed) & 0xFFFFFFFF, out.ctypes.data)
    _lib.check(st, "CUDA UMAP")
    config = dict(method="umap", backend="cuda", n=n, k=k, n_epochs=epochs, min_dist=float(min_dist),
                  negative_sample_rate=int(negative_sample_rate), learning_rate=float(learning_rate),
                  repulsion_strength=float(repulsion_strength), graph_mode="native_csr_graph",
                  graph_prep_backend="cuda_fuzzy_csr", optimizer_math="coo_atomic_edge_sampler_philox", seed=int(seed))
    return UmapFit(out, config)


def transform_tsne(reference_layout, knn, k=None, perplexity=5.0, initialization="median", Y_init=None,
                   n_iter=250, early_exaggeration_iter=0, learning_rate=0.1, early_exaggeration=4.0,
                   exaggeration=1.5, initial_momentum=0.8, final_momentum=0.8, max_grad_norm=0.25,
                   max_step_norm=math.inf, n_negatives=None, exact_repulsion_threshold=4096, seed=4,
                   backend="cuda"):
    """Place query points into a fixed reference layout (transform_tsne, R/transform_tsne.R:58-104).

    ``knn`` is ``dict(indices=..., distances=...)``: (n_query, k) KNN of each query into the
    reference rows. Policy restated from prepare_tsne_transform_controls (:186-229): n_negatives
    defaults to n_reference when n_reference <= exact_repulsion_threshold, else min(256,
    n_reference). Returns the (n_query, 2) layout and the recorded configuration of
    tsne_transform_config (:323-352)."""
    if backend != "cuda":
        raise ValueError("fastembedr_gb300 implements backend = 'cuda' only")
    ref = np.asarray(reference_layout, np.float64)
    if ref.ndim != 2 or ref.shape[0] < 1:
        raise ValueError("`reference_layout` must be a non-empty matrix.")
    if ref.shape[1] != 2:
        raise ValueError("cuda t-SNE transform currently supports only two-dimensional reference layouts.")
    if not isinstance(knn, dict) or "indices" not in knn or "distances" not in knn:
        raise ValueError("`knn` must contain `indices` and `distances`.")
    idx = np.asarray(knn["indices"])
    dist = np.asarray(knn["distances"], np.float64)
    if idx.shape != dist.shape:
        raise ValueError("KNN `indices` and `distances` must have the same dimensions.")
    if idx.ndim != 2 or idx.shape[0] < 1 or idx.shape[1] < 1:
        raise ValueError("`knn` must have at least one row and one neighbor column.")
    if k is not None:
        k = int(k)
        if k < 1:
            raise ValueError("`k` must be NULL or a positive integer.")
        if k > idx.shape[1]:
            raise ValueError("`k` cannot be larger than the available reference count.")
        idx, dist = idx[:, :k], dist[:, :k]
    nq, kk = idx.shape
    n_ref = ref.shape[0]
    perplexity = float(perplexity)
    if not math.isfinite(perplexity) or perplexity <= 0:
        raise ValueError("`perplexity` must be a positive number.")
    n_iter, early = int(n_iter), int(early_exaggeration_iter)
    if n_iter < 0 or early < 0 or n_iter + early < 1:
        raise ValueError("Transform iteration counts must be non-negative and sum to at least one.")
    threshold = 4096 if exact_repulsion_threshold is None else int(exact_repulsion_threshold)
    if n_negatives is None:
        n_negatives = n_ref if n_ref <= threshold else min(256, n_ref)
    n_negatives = int(n_negatives)
    if n_negatives < 1:
        raise ValueError("`n_negatives` must be NULL or a positive integer.")
    if initialization not in ("median", "weighted", "random"):
        raise ValueError("`initialization` must be 'median', 'weighted', or 'random'.")
    init = 0
    y0 = np.zeros((0, 2))
    if Y_init is not None:
        y0 = np.asarray(Y_init, np.float64)
        if y0.shape != (nq, 2):
            raise ValueError("`Y_init` must have one row per query and the same columns as `reference_layout`.")
        init = 1
    out = np.zeros((2, nq), np.float64)  # column-major n_query x 2
    ref_cm, idx_cm, dist_cm = _colmajor(ref, np.float64), _colmajor(idx, np.int32), _colmajor(dist, np.float64)
    y0_cm = _colmajor(y0, np.float64)
    lib = _lib.require_gpu()
    st = lib.fastembedr_cuda_transform_tsne(ref_cm.ctypes.data, n_ref, idx_cm.ctypes.data, dist_cm.ctypes.data, nq, kk,
                                            y0_cm.ctypes.data if init else None, init, initialization.encode(),
                                            perplexity, n_iter, early, float(learning_rate),
                                            float(early_exaggeration), float(exaggeration), float(initial_momentum),
                                            float(final_momentum), float(max_grad_norm), float(max_step_norm),
                                            n_negatives, threshold, int(seed), out.ctypes.data)
    _lib.check(st, "CUDA t-SNE transform")
    n_neg_eff = min(n_negatives, n_ref)
    exact = n_ref <= max(threshold, 1) or n_neg_eff >= n_ref
    config = dict(method="transform_tsne", backend="cuda", n_reference=n_ref, n_query=nq, k=kk, perplexity=perplexity,
                  n_iter=n_iter, early_exaggeration_iter=early, learning_rate=float(learning_rate),
                  early_exaggeration=float(early_exaggeration), exaggeration=float(exaggeration),
                  initial_momentum=float(initial_momentum), final_momentum=float(final_momentum),
                  max_grad_norm=float(max_grad_norm), max_step_norm=float(max_step_norm), n_negatives=n_neg_eff,
                  exact_repulsion_threshold=threshold, initialization=initialization,
                  optimizer="opentsne_style_fixed_reference_transform_cuda",
                  repulsion="exact_reference_cuda" if exact else "sampled_reference_cuda",
                  affinities="precomputed_query_conditional", affinity_storage="flat_row_major_double",
                  transform_batch_size=nq, transform_batches=1, seed=int(seed),
                  provenance="fixed_reference_tsne_native_cpp")
    return TsneFit(np.ascontiguousarray(out.T), config)


class TransformServer:
    """Resident serving loop for transform_tsne (C ABI fastembedr_transform_server_*).

    The reference layout stays on the device; ``submit`` queues one query batch (its KNN into
    the reference, int32 / float32) and returns a request id at once; ``result`` waits for it.
    Requests are admitted in arrival order against ``memory_budget_bytes`` and run merged with
    whatever else is admitted at the same time; every result equals ``transform_tsne`` on the
    same request. Options follow transform_tsne and are fixed per server."""

    def __init__(self, reference_layout, perplexity=5.0, initialization="median", n_iter=250,
                 early_exaggeration_iter=0, learning_rate=0.1, early_exaggeration=4.0, exaggeration=1.5,
                 initial_momentum=0.8, final_momentum=0.8, max_grad_norm=0.25, max_step_norm=math.inf,
                 n_negatives=None, exact_repulsion_threshold=4096, seed=4, memory_budget_bytes=0, max_inflight=4):
        ref = np.asarray(reference_layout, np.float64)
        if ref.ndim != 2 or ref.shape[0] < 1 or ref.shape[1] != 2:
            raise ValueError("`reference_layout` must be a non-empty two-column matrix.")
        n_ref = ref.shape[0]
        threshold = 4096 if exact_repulsion_threshold is None else int(exact_repulsion_threshold)
        if n_negatives is None:
            n_negatives = n_ref if n_ref <= threshold else min(256, n_ref)
        self.n_reference = n_ref
        self.n_negatives = min(int(n_negatives), n_ref)
        self.exact = n_ref <= max(threshold, 1) or self.n_negatives >= n_ref
        self._lib = _lib.require_gpu()
        self._h = C.c_void_p()
        ref_cm = _colmajor(ref, np.float64)
        st = self._lib.fastembedr_transform_server_create(
            ref_cm.ctypes.data, n_ref, float(perplexity), int(n_iter), int(early_exaggeration_iter),
            float(learning_rate), float(early_exaggeration), float(exaggeration), float(initial_momentum),
            float(final_momentum), float(max_grad_norm), float(max_step_norm), int(n_negatives), threshold, int(seed),
            str(initialization).encode(), int(memory_budget_bytes), int(max_inflight), C.byref(self._h))
        _lib.check(st, "CUDA t-SNE transform server")
        self._shape = {}

    def submit(self, indices, distances) -> int:
        idx = _colmajor(np.asarray(indices), np.int32)
        dist = _colmajor(np.asarray(distances), np.float32)
        if idx.shape != dist.shape or idx.ndim != 2:
            raise ValueError("KNN `indices` and `distances` must have the same dimensions.")
        rid = C.c_ulonglong()
        st = self._lib.fastembedr_transform_server_submit(self._h, idx.ctypes.data, dist.ctypes.data, idx.shape[0],
                                                          idx.shape[1], C.byref(rid))
        _lib.check(st, "CUDA t-SNE transform request")
        self._shape[rid.value] = idx.shape[0]
        return rid.value

    def result(self, request_id, timeout_ms=-1):
        """(layout (n_query, 2), latency_ms) or None when not finished within timeout_ms."""
        nq = self._shape[request_id]
        out = np.zeros((2, nq), np.float64)
        lat = C.c_double()
        st = self._lib.fastembedr_transform_server_wait(self._h, C.c_ulonglong(request_id), int(timeout_ms),
                                                        out.ctypes.data, C.byref(lat))
        if st == 2:
            return None
        del self._shape[request_id]
        _lib.check(st, "CUDA t-SNE transform request")
        return np.ascontiguousarray(out.T), lat.value

    def stats(self) -> dict:
        vals = [C.c_ulonglong() for _ in range(6)] + [C.c_double(), C.c_double(), C.c_longlong(), C.c_double()]
        _lib.check(self._lib.fastembedr_transform_server_stats(self._h, *[C.byref(v) for v in vals]),
                   "CUDA t-SNE transform server stats")
        keys = ("completed", "queries", "groups", "launches", "peak_bytes", "budget_bytes", "device_ms", "iterate_ms",
                "largest_group_queries", "largest_group_iterate_ms")
        return {k: v.value for k, v in zip(keys, vals)}

    def close(self):
        if self._h:
            self._lib.fastembedr_transform_server_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def umap_knn_batch(knns, inits, seed=42, n_epochs=500, min_dist=0.01, negative_sample_rate=5, learning_rate=1.0,
                   repulsion_strength=1.0, return_time=False):
    """umap_knn over many instances at once (C ABI fastembedr_cuda_umap_batch_from_knn_rows): every
    instance gets its own fuzzy graph and the package's SGD; one epoch is one launch over all
    instances' edges. Returns one (n_b, 2) layout per instance (and the SGD device time in ms)."""
    if not knns:
        raise ValueError("at least one instance is required")
    ks = {np.asarray(i).shape[1] for i, _ in knns}
    if len(ks) != 1:
        raise ValueError("every instance needs the same number of neighbours")
    k = ks.pop()
    sizes = np.array([np.asarray(i).shape[0] for i, _ in knns], np.int32)
    offs = {knn_index_offset(i) for i, _ in knns}
    off = 1 if offs == {1} else 0
    # one row-major array per instance, passed by pointer (no concatenated copy)
    idx = [np.ascontiguousarray(i, np.int32) for i, _ in knns]
    dist = [np.ascontiguousarray(d, np.float32) for _, d in knns]
    ys = [np.ascontiguousarray(y, np.float32) for y in inits]
    if len(ys) != len(knns) or any(y.shape != (n, 2) for y, n in zip(ys, sizes)):
        raise ValueError("init row counts must match the KNN graphs")
    lays = [np.zeros((int(n), 2), np.float32) for n in sizes]
    ptrs = lambda arrs: (C.c_void_p * len(arrs))(*[a.ctypes.data for a in arrs])
    ms = C.c_float()
    lib = _lib.require_gpu()
    st = lib.fastembedr_cuda_umap_batch_from_knn_rows(len(knns), sizes.ctypes.data, ptrs(idx), ptrs(dist), ptrs(ys),
                                                      k, off, int(n_epochs), int(negative_sample_rate),
                                                      float(learning_rate), float(min_dist),
                                                      float(repulsion_strength), int(seed) & 0xFFFFFFFF, ptrs(lays),
                                                      C.byref(ms))
    _lib.check(st, "CUDA UMAP batch")
    return (lays, ms.value) if return_time else lays


def landmark_tsne_transform(reference_data, query_data, reference_layout, indices, distances, perplexity=5.0,
                            n_iter=250, early_exaggeration_iter=0, learning_rate=0.1, early_exaggeration=4.0,
                            exaggeration=1.5, initial_momentum=0.8, final_momentum=0.8, max_grad_norm=0.25,
                            max_step_norm=math.inf, n_negatives=256, exact_repulsion_threshold=4096, seed=4,
                            affine_neighbors=8, affine_ridge=1e-3, max_extrapolation=1.5):
    """Landmark t-SNE projection through fastembedr_cuda_landmark_tsne_from_device_knn: the query
    KNN (n_query, k) into the landmarks goes to the device first, as in the reference's
    device-KNN route; the data matrices and the landmark layout are host arrays."""
    import torch

    idx = np.asarray(indices)
    n_query, k = idx.shape
    off = 1 if idx.min() >= 1 and idx.max() <= np.asarray(reference_layout).shape[0] else 0
    d_idx = torch.as_tensor(np.ascontiguousarray(idx.T, np.int32), device="cuda")
    d_dist = torch.as_tensor(np.ascontiguousarray(np.asarray(distances, np.float32).T), device="cuda")
    torch.cuda.current_stream().synchronize()
    X = _colmajor(reference_data, np.float32)
    Q = _colmajor(query_data, np.float32)
    L = _colmajor(reference_layout, np.float32)
    out = np.zeros((n_query, 2), np.float32)
    lib = _lib.require_gpu()
    st = lib.fastembedr_cuda_landmark_tsne_from_device_knn(
        d_idx.data_ptr(), d_dist.data_ptr(), off, X.ctypes.data, Q.ctypes.data, L.ctypes.data, L.shape[0], n_query,
        X.shape[1], k, float(perplexity), int(n_iter), int(early_exaggeration_iter), float(learning_rate),
        float(early_exaggeration), float(exaggeration), float(initial_momentum), float(final_momentum),
        float(max_grad_norm), float(max_step_norm), int(n_negatives), int(exact_repulsion_threshold),
        int(seed) & 0xFFFFFFFF, int(affine_neighbors), float(affine_ridge), float(max_extrapolation), out.ctypes.data)
    _lib.check(st, "CUDA landmark t-SNE")
    return out
