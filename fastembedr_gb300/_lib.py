"""ctypes binding of the native library (C ABI declared in include/fastembedr_cuda.h).

The library is the only compute path: if it is missing or no CUDA device is present, calls
raise instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_LIB = None

i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
vp = C.c_void_p
I, U, F, D, L = C.c_int, C.c_uint, C.c_float, C.c_double, C.c_longlong

# name -> (restype, argtypes); argtypes use void* for arrays so host numpy arrays and raw
# device pointers (ints) are both accepted.
SIGNATURES = {
    "fastembedr_cuda_available": (C.c_bool, []),
    "fastembedr_cuda_embedding_last_error": (C.c_char_p, []),
    "fastembedr_cuda_opentsne_fft_grid_size": (I, [I]),
    "fastembedr_cuda_opentsne_fft_from_knn_float": (I, [vp, vp, vp, I, I, I, I, F, I, I, F, F, F, I, F, F, F, F, U,
                                                        I, vp]),
    "fastembedr_cuda_opentsne_fft_from_knn": (I, [vp, vp, vp, I, I, I, I, F, I, I, F, F, F, I, F, F, F, F, U, I, vp]),
    "fastembedr_cuda_opentsne_fft_from_device_knn_float": (I, [vp, vp, vp, I, I, I, I, F, I, I, F, F, F, I, F, F, F, F,
                                                               U, I, vp]),
    "fastembedr_cuda_tsne_affinities": (I, [vp, vp, I, I, F, I, vp, vp, vp, L, C.POINTER(L), vp, vp, C.POINTER(D)]),
    "fastembedr_cuda_tsne_force_diagnostic": (I, [vp, vp, vp, I, I, F, F, I, I, I, vp, vp, C.POINTER(D), vp,
                                                  C.POINTER(D), C.POINTER(D)]),
    "fastembedr_cuda_umap_optimize_coo": (I, [vp, vp, vp, vp, vp, I, I, I, I, F, F, F, F, U, I, vp]),
    "fastembedr_cuda_umap_graph_from_knn": (I, [vp, vp, I, I, I, vp, vp, vp, vp, L, C.POINTER(L), C.POINTER(F)]),
    "fastembedr_cuda_umap_from_knn": (I, [vp, vp, vp, I, I, I, I, I, F, F, F, U, vp]),
    "fastembedr_cuda_umap_batch_from_knn": (I, [I, vp, vp, vp, vp, I, I, I, I, F, F, F, U, vp, C.POINTER(F)]),
    "fastembedr_cuda_umap_batch_from_knn_rows": (I, [I, vp, vp, vp, vp, I, I, I, I, F, F, F, U, vp, C.POINTER(F)]),
    "fastembedr_cuda_umap_from_knn_profile": (I, [vp, vp, vp, I, I, I, I, I, F, F, F, U, vp, C.POINTER(F),
                                                  C.POINTER(F)]),
    "fastembedr_cuda_tsne_exact_repulsion_noalloc": (I, [vp, I, vp, vp, vp]),
    "fastembedr_cuda_transform_tsne": (I, [vp, I, vp, vp, I, I, vp, I, C.c_char_p, D, I, I, D, D, D, D, D, D, D, I, I,
                                           I, vp]),
    "fastembedr_cuda_landmark_tsne_from_device_knn": (I, [vp, vp, I, vp, vp, vp, I, I, I, I, F, I, I, F, F, F, F, F,
                                                          F, F, I, I, U, I, F, F, vp]),
    "fastembedr_transform_server_create": (I, [vp, I, D, I, I, D, D, D, D, D, D, D, I, I, I, C.c_char_p, C.c_ulonglong,
                                               I, C.POINTER(vp)]),
    "fastembedr_transform_server_submit": (I, [vp, vp, vp, I, I, C.POINTER(C.c_ulonglong)]),
    "fastembedr_transform_server_wait": (I, [vp, C.c_ulonglong, I, vp, C.POINTER(D)]),
    "fastembedr_transform_server_stats": (I, [vp] + [C.POINTER(C.c_ulonglong)] * 6 + [C.POINTER(D)] * 2
                                          + [C.POINTER(L), C.POINTER(D)]),
    "fastembedr_transform_server_destroy": (None, [vp]),
    "fastembedr_tsne_plan_create": (I, [vp, vp, vp, I, I, F, I, I, I, U, C.POINTER(vp)]),
    "fastembedr_tsne_plan_run": (I, [vp, I, F, F, F, F, F, I]),
    "fastembedr_tsne_plan_profile": (I, [vp, I, F, F, F, F, F, C.POINTER(F), C.POINTER(F), C.POINTER(F)]),
    "fastembedr_tsne_plan_synchronize": (I, [vp]),
    "fastembedr_tsne_plan_stream": (vp, [vp]),
    "fastembedr_tsne_plan_layout": (I, [vp, vp]),
    "fastembedr_tsne_plan_info": (I, [vp, C.POINTER(L), C.POINTER(I), C.POINTER(I), C.POINTER(I), C.POINTER(I)]),
    "fastembedr_tsne_plan_tuning": (I, [vp, C.POINTER(I), C.POINTER(I), I, C.POINTER(I), vp, vp, vp]),
    "fastembedr_tsne_plan_kl": (I, [vp, C.POINTER(D)]),
    "fastembedr_cuda_umap_spectral_init_from_knn": (I, [vp, vp, I, I, I, I, D, I, vp]),
    "fastembedr_cuda_umap_spectral_init_csr": (I, [vp, vp, vp, I, I, D, I, vp]),
    "fastembedr_cuda_umap_knn_spectral": (I, [vp, vp, I, I, I, I, I, F, F, F, I, D, U, vp]),
    "fastembedr_umap_find_ab_params": (None, [D, D, C.POINTER(D), C.POINTER(D)]),
    "fastembedr_host_normal_stream_check": (I, []),
    "fastembedr_cuda_opentsne_fft_from_device_knn_float_pca_double": (I, [vp, vp, vp, I, I, I, I, F, I, I, F, F, F, I,
                                                                       F, F, F, F, U, I, vp]),
    "fastembedr_cuda_opentsne_fft_from_device_knn_float_pca_float": (I, [vp, vp, vp, I, I, I, I, F, I, I, F, F, F, I,
                                                                      F, F, F, F, U, I, vp]),
    "fastembedr_cuda_tsne_pca_init": (I, [vp, I, I, I, vp]),
    "fastembedr_cuda_spectral_init_from_knn": (I, [vp, vp, I, I, I, U, I, vp]),
    "fastembedr_cuda_umap_from_knn_spectral": (I, [vp, vp, I, I, I, I, F, F, F, F, I, U, I, I, vp]),
    "fastembedr_cuda_umap_from_knn_spectral_float": (I, [vp, vp, I, I, I, I, F, F, F, F, I, U, I, I, vp]),
    "fastembedr_cuda_umap_from_device_knn_spectral_float": (I, [vp, vp, I, I, I, I, F, F, F, F, I, U, I, I, I, vp]),
    "fastembedr_tsne_plan_gradient_check": (I, [vp, vp, I, F, vp, vp, vp, C.POINTER(D), C.POINTER(D)]),
    "fastembedr_tsne_plan_destroy": (None, [vp]),
    "fastembedr_tsne_batch_create": (I, [I, vp, vp, vp, vp, I, F, I, I, I, U, C.POINTER(vp)]),
    "fastembedr_tsne_batch_create_rows": (I, [I, vp, vp, vp, vp, I, F, I, I, I, U, C.POINTER(vp)]),
    "fastembedr_tsne_batch_run": (I, [vp, I, I, F, F, F, F, F, F, F]),
    "fastembedr_tsne_batch_iterate": (I, [vp, I, F, F, F, F, F]),
    "fastembedr_tsne_batch_synchronize": (I, [vp]),
    "fastembedr_tsne_batch_stream": (vp, [vp]),
    "fastembedr_tsne_batch_layout": (I, [vp, vp]),
    "fastembedr_tsne_batch_kl": (I, [vp, I, C.POINTER(D)]),
    "fastembedr_tsne_batch_info": (I, [vp, C.POINTER(L), C.POINTER(L), C.POINTER(I), C.POINTER(I), C.POINTER(I)]),
    "fastembedr_tsne_batch_grids": (I, [vp, vp, C.POINTER(I)]),
    "fastembedr_tsne_batch_destroy": (None, [vp]),
    "fastembedr_cuda_tsne_batch_from_knn": (I, [I, vp, vp, vp, vp, I, F, I, I, F, F, F, F, F, F, F, U, I, vp]),
}


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True) -> C.CDLL:
    """Load the native library, building it first when it is absent."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(_build.LIB):
            if not build_if_missing:
                raise FileNotFoundError(f"{_build.LIB} is missing; run fastembedr_gb300.build.build()")
            _build.build()
        lib = C.CDLL(_build.LIB)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name, None)
            if fn is None:
                continue
            fn.restype = res
            fn.argtypes = args
        _LIB = lib
    return _LIB


class CudaEmbeddingError(RuntimeError):
    pass


def check(status: int, what: str) -> None:
    if status != 0:
        msg = load().fastembedr_cuda_embedding_last_error()
        raise CudaEmbeddingError(f"{what} failed: {msg.decode() if msg else 'unknown error'}")


def require_gpu() -> C.CDLL:
    lib = load()
    if not lib.fastembedr_cuda_available():
        raise CudaEmbeddingError("No CUDA device is available.")
    return lib


def ptr(a) -> int:
    """Address of a numpy array or a torch tensor (host or device)."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    return a.ctypes.data
