"""CPU oracle for the KNN-input embedding optimizer (TEST INFRASTRUCTURE ONLY).

Two libraries live here:

* ``liborc.so`` -- the plain-C restatement of the reference CPU algorithms
  (``tsne_oracle.c``, ``umap_oracle.c``, ``transform_oracle.c``). It builds anywhere
  with gcc and is the checker used by the GPU parity tests, ``smoke()`` and the
  CPU-baseline leg of ``bench.py``.
* ``_ref/libfastembedr_ref.so`` -- the reference's own CPU cores
  (fastEmbedR ``src/tsne_neighbors.cpp``, ``src/fast_knn_umap.cpp``) compiled where
  they lie against ``rcpp_shim/Rcpp.h``. It only exists where the reference sources
  are present; it pins the restatement and generates ``tests/golden`` fixtures.

Nothing in the product package imports this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_ORC = None
_REF = None

i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")


def reference_sources():
    """Directory of the reference's C++ sources (its src/), from FASTEMBEDR_REFERENCE_SRC; None
    when unset or missing. Only the build of the reference library reads it."""
    path = os.environ.get("FASTEMBEDR_REFERENCE_SRC", "")
    return path if path and os.path.isdir(path) else None


def build(ref: bool = False) -> None:
    """Compile liborc.so (and the reference library when ``ref`` and the reference sources are
    given by FASTEMBEDR_REFERENCE_SRC)."""
    subprocess.run(["make", "-s", "-C", HERE, "liborc.so"], check=True)
    src = reference_sources()
    if ref:
        if src is None:
            raise FileNotFoundError("set FASTEMBEDR_REFERENCE_SRC to the reference's src/ directory")
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF_SRC={src}"], check=True)


def ref_available() -> bool:
    return os.path.exists(os.path.join(HERE, "_ref", "libfastembedr_ref.so"))


def orc() -> C.CDLL:
    global _ORC
    if _ORC is None:
        path = os.path.join(HERE, "liborc.so")
        if not os.path.exists(path):
            build()
        lib = C.CDLL(path)
        I, D, F, V, L = C.c_int, C.c_double, C.c_float, None, C.c_longlong
        sig = {
            "orc_set_threads": (I, [I]),
            "orc_index_offset": (I, [i32p, I, I]),
            "orc_validate_knn": (I, [i32p, f32p, I, I, I]),
            "orc_row_p_f32": (V, [f32p, I, I, D, f32p]),
            "orc_row_p_f64": (V, [f32p, I, I, D, f64p, f64p]),
            "orc_csr_build": (L, [i32p, f32p, I, I, I, i32p, i32p, f32p, L, f64p]),
            "orc_fft_grid_size_cpu": (I, [I]),
            "orc_attractive": (V, [i32p, i32p, f32p, f32p, I, F, f32p]),
            "orc_exact_rep_f32": (V, [f32p, I, f32p, f64p]),
            "orc_exact_rep_f64": (V, [f32p, I, f64p, f64p]),
            "orc_fft_grid_rep_f32": (V, [f32p, I, I, f32p, f64p]),
            "orc_interp_rep_f64": (V, [f32p, I, I, I, f64p, f64p]),
            "orc_update": (V, [f32p, f32p, f32p, f32p, I, F, F, F, F]),
            "orc_zero_mean": (V, [f32p, I]),
            "orc_sum_q": (D, [f32p, I]),
            "orc_kl": (D, [i32p, i32p, f32p, f32p, I]),
            "orc_tsne_run": (I, [i32p, f32p, I, I, f32p, D, I, I, D, D, D, I, D, D, D, D, I, I,
                                 f32p, C.c_void_p, C.c_void_p, I]),
            "orc_tsne_prepare": (C.c_void_p, [i32p, f32p, I, I, f32p, D, I]),
            "orc_tsne_iterate": (V, [C.c_void_p, I, F, F, F, F, F]),
            "orc_tsne_get_y": (V, [C.c_void_p, f32p]),
            "orc_tsne_nnz": (L, [C.c_void_p]),
            "orc_tsne_free": (V, [C.c_void_p]),
            "orc_umap_smooth_knn": (V, [f32p, I, I, f32p, f32p]),
            "orc_umap_graph": (L, [i32p, f32p, I, I, I, i32p, i32p, f32p, f32p, L, f32p]),
            "orc_umap_ab": (V, [D, D, C.POINTER(D), C.POINTER(D)]),
            "orc_umap_ab_cuda_host": (V, [D, D, C.POINTER(D), C.POINTER(D)]),
            "orc_umap_powf_fast": (F, [F, F]),
            "orc_umap_pow": (D, [D, D]),
            "orc_umap_sgd_serial": (V, [I, i32p, i32p, f32p, f64p, I, D, D, I, D, D, I]),
            "orc_umap_sgd_threaded": (V, [I, i32p, i32p, f32p, f64p, I, D, D, I, D, D, I, I]),
            "orc_umap_diffusion_init": (V, [i32p, i32p, f32p, I, I, I, I, f32p]),
            "orc_umap_spectral_init": (V, [i32p, i32p, f32p, I, I, D, I, f64p]),
            "orc_umap_sgd_coo_schedule": (V, [I, I, i32p, i32p, f32p, f32p, I, F, F, I, F, F, C.c_uint]),
            "orc_transform_tsne": (I, [f64p, I, i32p, f64p, I, I, C.c_void_p, I, D, I, I, D, D, D, D, D,
                                       D, D, I, I, I, f64p]),
            "orc_knn_preservation": (D, [f32p, I, i32p, I, I, i32p, I, I]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _ORC = lib
    return _ORC


def ref() -> C.CDLL:
    global _REF
    if _REF is None:
        path = os.path.join(HERE, "_ref", "libfastembedr_ref.so")
        if not os.path.exists(path):
            raise FileNotFoundError("reference CPU library not built (make -C oracle ref)")
        lib = C.CDLL(path)
        I, D, L = C.c_int, C.c_double, C.c_longlong
        lib.ref_last_error.restype = C.c_char_p
        lib.ref_force_diagnostic.restype = I
        lib.ref_force_diagnostic.argtypes = [i32p, f64p, f64p, I, I, D, D, I, I, f64p, f64p, f64p,
                                             i32p, i32p, f64p, L, C.POINTER(L), C.POINTER(D), C.POINTER(D)]
        lib.ref_kl_diagnostic.restype = D
        lib.ref_kl_diagnostic.argtypes = [i32p, f64p, f64p, I, I, D, I]
        lib.ref_tsne_run.restype = I
        lib.ref_tsne_run.argtypes = [i32p, f64p, f64p, I, I, D, I, I, D, D, D, I, D, D, D, D, C.c_char_p,
                                     I, I, I, f64p, f64p, C.POINTER(I), C.POINTER(I)]
        lib.ref_transform.restype = I
        lib.ref_transform.argtypes = [f64p, I, i32p, f64p, I, I, C.c_void_p, I, C.c_char_p, D, I, I, D, D, D,
                                      D, D, D, D, I, I, I, I, f64p]
        lib.ref_umap_graph.restype = I
        lib.ref_umap_graph.argtypes = [i32p, f64p, I, I, I, i32p, i32p, f64p, f64p, L, C.POINTER(L),
                                       C.POINTER(D)]
        lib.ref_umap_sgd.restype = I
        lib.ref_umap_sgd.argtypes = [i32p, i32p, f64p, f64p, I, L, I, D, I, D, D, I, I, f64p]
        lib.ref_umap_diffusion_init.restype = I
        lib.ref_umap_diffusion_init.argtypes = [i32p, i32p, f64p, I, L, I, I, f64p]
        lib.ref_umap_spectral_init.restype = I
        lib.ref_umap_spectral_init.argtypes = [i32p, i32p, f64p, I, L, I, D, I, f64p]
        lib.ref_umap_spectral_knn.restype = I
        lib.ref_umap_spectral_knn.argtypes = [i32p, f64p, I, I, I, I, f64p]
        lib.ref_knn_structure_score.restype = I
        lib.ref_knn_structure_score.argtypes = [f64p, I, i32p, I, i32p, I, I, f64p]
        lib.ref_project_affine.restype = I
        lib.ref_project_affine.argtypes = [f64p, I, f64p, I, I, f64p, i32p, f64p, I, I, D, D, f64p, f64p, i32p]
        _REF = lib
    return _REF


# ---------------------------------------------------------------- numpy helpers (oracle)
def _cm(a, dtype):
    """column-major flat copy of an (n, k) array"""
    return np.ascontiguousarray(np.asarray(a, dtype=dtype).T).ravel()


def index_offset(idx):
    idx = np.asarray(idx, np.int32)
    return orc().orc_index_offset(_cm(idx, np.int32), idx.shape[0], idx.shape[1])


def row_p_f32(dist, perplexity):
    dist = np.asarray(dist, np.float32)
    n, k = dist.shape
    out = np.zeros(n * k, np.float32)
    orc().orc_row_p_f32(_cm(dist, np.float32), n, k, float(perplexity), out)
    return out.reshape(n, k)


def row_p_f64(dist, perplexity):
    dist = np.asarray(dist, np.float32)
    n, k = dist.shape
    out = np.zeros(n * k, np.float64)
    beta = np.zeros(n, np.float64)
    orc().orc_row_p_f64(_cm(dist, np.float32), n, k, float(perplexity), out, beta)
    return out.reshape(n, k), beta


def csr_from_p(idx, p, offset=None):
    idx = np.asarray(idx, np.int32)
    n, k = idx.shape
    if offset is None:
        offset = index_offset(idx)
    cap = 2 * n * k
    rp = np.zeros(n + 1, np.int32)
    col = np.zeros(cap, np.int32)
    val = np.zeros(cap, np.float32)
    tot = np.zeros(1, np.float64)
    nnz = orc().orc_csr_build(_cm(idx, np.int32), np.ascontiguousarray(p, np.float32).ravel(), n, k, offset,
                              rp, col, val, cap, tot)
    return rp, col[:nnz].copy(), val[:nnz].copy(), float(tot[0])


def tsne_csr(idx, dist, perplexity):
    return csr_from_p(idx, row_p_f32(dist, perplexity))


def attractive(rp, col, val, y, exaggeration=1.0):
    y = np.ascontiguousarray(y, np.float32)
    out = np.zeros_like(y)
    orc().orc_attractive(rp, col, val, y.ravel(), y.shape[0], float(exaggeration), out.ravel())
    return out


def exact_rep_f64(y):
    y = np.ascontiguousarray(y, np.float32)
    out = np.zeros(y.shape, np.float64)
    z = np.zeros(1)
    orc().orc_exact_rep_f64(y.ravel(), y.shape[0], out.ravel(), z)
    return out, float(z[0])


def exact_rep_f32(y):
    y = np.ascontiguousarray(y, np.float32)
    out = np.zeros_like(y)
    z = np.zeros(1)
    orc().orc_exact_rep_f32(y.ravel(), y.shape[0], out.ravel(), z)
    return out, float(z[0])


def fft_grid_rep_f32(y, grid):
    y = np.ascontiguousarray(y, np.float32)
    out = np.zeros_like(y)
    z = np.zeros(1)
    orc().orc_fft_grid_rep_f32(y.ravel(), y.shape[0], int(grid), out.ravel(), z)
    return out, float(z[0])


def interp_rep_f64(y, grid, lagrange):
    y = np.ascontiguousarray(y, np.float32)
    out = np.zeros(y.shape, np.float64)
    z = np.zeros(1)
    orc().orc_interp_rep_f64(y.ravel(), y.shape[0], int(grid), int(bool(lagrange)), out.ravel(), z)
    return out, float(z[0])


def kl(rp, col, val, y):
    y = np.ascontiguousarray(y, np.float32)
    return orc().orc_kl(rp, col, val, y.ravel(), y.shape[0])


def tsne_run(idx, dist, init, perplexity=30.0, early_iter=250, n_iter=750, early_exag=12.0, exag=1.0,
             learning_rate=-1.0, m0=0.8, m1=0.8, min_gain=0.01, max_step_norm=5.0, repulsion=0,
             grid=0, kl_every=False):
    idx = np.asarray(idx, np.int32)
    n, k = idx.shape
    y = np.zeros(2 * n, np.float32)
    cap = (early_iter + n_iter) // 50 + 2
    trace = np.zeros(cap, np.float64)
    its = np.zeros(cap, np.int32)
    lr_auto = 1 if learning_rate <= 0 else 0
    st = orc().orc_tsne_run(_cm(idx, np.int32), _cm(dist, np.float32), n, k,
                            np.ascontiguousarray(init, np.float32).ravel(), float(perplexity), int(early_iter),
                            int(n_iter), float(early_exag), float(exag), float(learning_rate), lr_auto, float(m0),
                            float(m1), float(min_gain), float(max_step_norm), int(repulsion), int(grid), y,
                            trace.ctypes.data if kl_every else None, its.ctypes.data if kl_every else None,
                            cap if kl_every else 0)
    if st != 0:
        raise ValueError("oracle rejected the KNN input")
    out = y.reshape(n, 2)
    if kl_every:
        m = int(np.count_nonzero(its))
        return out, trace[:m], its[:m]
    return out


def knn_preservation(y, idx_hi, keep=None, preserve_k=15, offset=0):
    y = np.ascontiguousarray(y, np.float32)
    idx_hi = np.asarray(idx_hi, np.int32)
    n = y.shape[0]
    keep = np.arange(n, dtype=np.int32) if keep is None else np.ascontiguousarray(keep, np.int32)
    return orc().orc_knn_preservation(y.ravel(), n, _cm(idx_hi, np.int32), idx_hi.shape[1], int(offset), keep,
                                      keep.size, int(preserve_k))


def umap_graph(idx, dist, offset=None):
    idx = np.asarray(idx, np.int32)
    n, k = idx.shape
    if offset is None:
        offset = index_offset(idx)
    cap = 2 * n * k
    off = np.zeros(n + 1, np.int32)
    nb = np.zeros(cap, np.int32)
    w = np.zeros(cap, np.float32)
    e = np.zeros(cap, np.float32)
    mw = np.zeros(1, np.float32)
    nnz = orc().orc_umap_graph(_cm(idx, np.int32), _cm(dist, np.float32), n, k, offset, off, nb, w, e, cap, mw)
    return off, nb[:nnz].copy(), w[:nnz].copy(), e[:nnz].copy(), float(mw[0])


def umap_ab(min_dist=0.01, spread=1.0, cuda_host=False):
    a, b = C.c_double(), C.c_double()
    fn = orc().orc_umap_ab_cuda_host if cuda_host else orc().orc_umap_ab
    fn(float(spread), float(min_dist), C.byref(a), C.byref(b))
    return a.value, b.value


def umap_diffusion_init(offsets, neighbors, weights, n_iter, seed, index_offset=0):
    """The reference's diffusion start over a CSR graph (row-major n x 2 float32)."""
    n = len(offsets) - 1
    out = np.zeros((n, 2), np.float32)
    orc().orc_umap_diffusion_init(np.ascontiguousarray(offsets, np.int32), np.ascontiguousarray(neighbors, np.int32),
                                  np.ascontiguousarray(weights, np.float32), n, int(index_offset), int(n_iter),
                                  int(seed), out.ravel())
    return out


def umap_spectral_init(offsets, neighbors, weights, n_iter, seed, init_scale=float("nan")):
    """The reference CPU spectral start over a CSR graph (row-major n x 2 float64)."""
    n = len(offsets) - 1
    out = np.zeros(2 * n)
    orc().orc_umap_spectral_init(np.ascontiguousarray(offsets, np.int32), np.ascontiguousarray(neighbors, np.int32),
                                 np.ascontiguousarray(weights, np.float32), n, int(n_iter), float(init_scale),
                                 int(seed), out)
    return out.reshape(2, n).T.copy()


def umap_sgd_coo(n, heads, tails, eps, init, n_epochs, a, b, nsr=5, lr=1.0, gamma=1.0, seed=42):
    y = np.ascontiguousarray(init, np.float32).copy()
    orc().orc_umap_sgd_coo_schedule(n, heads.size, np.ascontiguousarray(heads, np.int32),
                                    np.ascontiguousarray(tails, np.int32), np.ascontiguousarray(eps, np.float32),
                                    y.ravel(), int(n_epochs), float(a), float(b), int(nsr), float(lr), float(gamma),
                                    int(seed) & 0xFFFFFFFF)
    return y


def transform_tsne(ref_y, idx, dist, y_init=None, init_mode=1, perplexity=5.0, n_iter=250, early_iter=0,
                   learning_rate=0.1, early_exag=4.0, exag=1.5, m0=0.8, m1=0.8, max_grad_norm=0.25,
                   max_step_norm=np.inf, n_negatives=256, exact_threshold=4096, seed=4):
    ref_y = np.ascontiguousarray(ref_y, np.float64)
    idx = np.asarray(idx, np.int32)
    nq, k = idx.shape
    out = np.zeros(2 * nq, np.float64)
    yi = None if y_init is None else np.ascontiguousarray(y_init, np.float64)
    st = orc().orc_transform_tsne(ref_y.ravel(), ref_y.shape[0], _cm(idx, np.int32), _cm(dist, np.float64), nq,
                                  k, yi.ctypes.data if yi is not None else None, 0 if yi is not None else init_mode,
                                  float(perplexity), int(n_iter), int(early_iter), float(learning_rate),
                                  float(early_exag), float(exag), float(m0), float(m1), float(max_grad_norm),
                                  float(max_step_norm), int(n_negatives), int(exact_threshold), int(seed), out)
    if st != 0:
        raise ValueError("oracle rejected the transform input")
    return out.reshape(nq, 2)
