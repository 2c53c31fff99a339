"""CPU-side checks of the boundary: the library loads without a GPU, exports every symbol that
include/fastembedr_cuda.h declares, and reports the absence of a device through the reference's
error convention (no compute is attempted without a GPU)."""
import os
import re

import numpy as np
import pytest

from fastembedr_gb300 import _lib, api

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    syms = set()
    for name in os.listdir(os.path.join(ROOT, "include")):
        if name.endswith(".h"):
            text = open(os.path.join(ROOT, "include", name)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            syms |= set(re.findall(r"\b(fastembedr_\w+)\s*\(", text))
    return syms


def test_header_declares_the_reference_abi():
    syms = declared_symbols()
    for ref in ("fastembedr_cuda_available", "fastembedr_cuda_embedding_last_error",
                "fastembedr_cuda_opentsne_fft_grid_size", "fastembedr_cuda_opentsne_fft_from_knn_float",
                "fastembedr_cuda_opentsne_fft_from_knn", "fastembedr_cuda_opentsne_fft_from_device_knn_float",
                "fastembedr_cuda_spectral_init_from_knn", "fastembedr_cuda_umap_from_knn_spectral",
                "fastembedr_cuda_umap_from_knn_spectral_float", "fastembedr_cuda_umap_from_device_knn_spectral_float"):
        assert ref in syms


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    for s in sorted(declared_symbols()):
        assert hasattr(lib, s), s


def test_grid_policy_matches_reference_cuda(monkeypatch):
    lib = _lib.load()
    monkeypatch.delenv("FASTEMBEDR_TSNE_FFT_GRID", raising=False)
    sizes = (1000, 19999, 20000, 99999, 100000, 10**6)
    monkeypatch.setenv("FASTEMBEDR_TSNE_INTERPOLATION", "bilinear")
    assert [lib.fastembedr_cuda_opentsne_fft_grid_size(n) for n in sizes] == [256, 256, 512, 512, 1024, 1024]
    monkeypatch.setenv("FASTEMBEDR_TSNE_INTERPOLATION", "lagrange")
    assert [lib.fastembedr_cuda_opentsne_fft_grid_size(n) for n in sizes] == [256, 256, 512, 512, 1024, 1024]
    monkeypatch.setenv("FASTEMBEDR_TSNE_FFT_GRID", "64")
    assert lib.fastembedr_cuda_opentsne_fft_grid_size(10**6) == 64


def test_no_device_is_an_error_not_a_fallback():
    lib = _lib.load()
    if lib.fastembedr_cuda_available():
        pytest.skip("a CUDA device is present")
    idx = np.array([[2, 3], [1, 3], [1, 2]], np.int32)
    dist = np.ones((3, 2), np.float32)
    with pytest.raises(_lib.CudaEmbeddingError):
        api.tsne_knn(idx, dist, perplexity=0.5, n_iter=1, early_exaggeration_iter=0)


def test_index_offset_detection():
    assert api.knn_index_offset(np.array([[2, 3], [1, 3], [1, 2]])) == 1
    assert api.knn_index_offset(np.array([[1, 2], [0, 2], [0, 1]])) == 0


@pytest.mark.parametrize("min_dist", [0.01, 0.1, 0.25, 0.5, 0.05])
def test_umap_curve_parameters_match_the_oracle(min_dist):
    """find_ab_params is host code in the library; the oracle restates the reference's."""
    import oracle as O

    a, b = api.umap_ab_params(min_dist)
    ra, rb = O.umap_ab(min_dist)
    assert a == pytest.approx(ra, rel=1e-12) and b == pytest.approx(rb, rel=1e-12)


def test_multithreaded_normal_draws_reproduce_the_standard_library():
    """The spectral start's host draws take the multi-threaded polar path, which checks itself
    bit for bit against std::normal_distribution on std::mt19937 at first use."""
    assert _lib.load().fastembedr_host_normal_stream_check() == 1


def test_spectral_start_csr_checks_its_graph_before_any_device_work():
    """Host-side checks of fastembedr_cuda_umap_spectral_init_csr (validate_csr_inputs plus the
    symmetry the GPU start needs) report errors without a GPU."""
    lib = _lib.load()
    out = np.zeros(6)

    def call(off, nb, w):
        off, nb, w = (np.ascontiguousarray(off, np.int32), np.ascontiguousarray(nb, np.int32),
                      np.ascontiguousarray(w, np.float32))
        st = lib.fastembedr_cuda_umap_spectral_init_csr(off.ctypes.data, nb.ctypes.data, w.ctypes.data, 3, 5, 0.0,
                                                        1, out.ctypes.data)
        return st, lib.fastembedr_cuda_embedding_last_error().decode()

    st, msg = call([0, 1, 2, 3], [1, 2, 0], [1.0, 1.0, 1.0])  # 0->1, 1->2, 2->0: not symmetric
    assert st != 0 and "symmetric" in msg
    st, msg = call([0, 1, 2, 2], [1, 1, 0], [1.0, 1.0, 1.0])  # row 1 holds itself
    assert st != 0 and "self-neighbors" in msg
    st, msg = call([0, 2, 3, 4], [2, 1, 0, 0], [1.0, 1.0, 1.0, 1.0])
    assert st != 0 and "sorted" in msg
    st, msg = call([0, 1, 2, 2], [1, 0, 0], [1.0, -1.0, 1.0])
    assert st != 0 and "positive and finite" in msg
