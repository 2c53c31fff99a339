"""Device PCA start of t-SNE (fastembedr_cuda_opentsne_fft_from_device_knn_float_pca_*,
src/embedding_cuda_kernels.cpp:6265-6321; the reference computes it with RAPIDS RAFT's
covariance-eigen TSVD, src/embedding_cuda_kernels.cpp:3379-3530, and scales it with
finalize_tsne_pca_init_stats_kernel, :1352-1410) against a NumPy FP64 restatement of the same
published algorithm."""
import numpy as np
import pytest

from fastembedr_gb300 import _lib, api, synthetic

pytestmark = pytest.mark.gpu


def pca_start(x):
    """Test-side restatement: float32 centring, FP64 Gram matrix and eigenvectors, scores with
    the largest-magnitude entry positive, then the t-SNE scaling (1e-4 / larger sd)."""
    xf = np.asarray(x, np.float32)
    mean = xf.astype(np.float64).mean(0).astype(np.float32)
    xc = (xf - mean).astype(np.float64)
    w, v = np.linalg.eigh(xc.T @ xc)
    s = xc @ v[:, np.argsort(w)[::-1][:2]]
    for c in range(2):
        if s[np.argmax(np.abs(s[:, c])), c] < 0:
            s[:, c] = -s[:, c]
    s32 = s.astype(np.float32).astype(np.float64)
    n = s32.shape[0]
    m = s32.mean(0)
    ss = np.maximum((s32 ** 2).sum(0) - s32.sum(0) ** 2 / n, 0.0)
    sd = np.sqrt(ss / (n - 1)).max()
    return ((s32 - m) * (1e-4 / sd)).astype(np.float32)


@pytest.mark.parametrize("n,p,dtype", [(20000, 50, np.float32), (3000, 7, np.float64), (500, 2, np.float32),
                                       (4000, 300, np.float32)])
def test_pca_start_matches_restatement(n, p, dtype):
    x, _ = synthetic.mixture(n, p, 6, 50 + p, centre_sd=3.0, anisotropic=True)
    x = x.astype(dtype)
    got = api.tsne_pca_init(x)
    want = pca_start(x)
    assert np.abs(got - want).max() <= 1e-5 * np.abs(want).max(), np.abs(got - want).max()
    assert np.std(got, axis=0, ddof=1).max() == pytest.approx(1e-4, rel=1e-4)


def test_pca_entry_point_runs_tsne_from_the_pca_start():
    """One iteration from the device PCA start equals the plain device-KNN entry point given the
    same start (float atomics: to rounding)."""
    import torch

    x, _ = synthetic.mixture(4000, 20, 5, 60, centre_sd=3.0)
    idx, dist = synthetic.exact_knn_numpy(x, 30)
    n, k = idx.shape
    d_idx = torch.as_tensor(np.ascontiguousarray(idx.T.astype(np.int32)), device="cuda")
    d_dist = torch.as_tensor(np.ascontiguousarray(dist.T.astype(np.float32)), device="cuda")
    torch.cuda.synchronize()
    lib = _lib.require_gpu()
    xf = np.asfortranarray(x.astype(np.float32))
    xd = np.asfortranarray(x.astype(np.float64))
    args = (n, k, 2, 10.0, 0, 1, 12.0, 1.0, 100.0, 0, 0.8, 0.8, 0.01, 5.0, 4, 0)
    outs = {}
    for tag, fn, arr in (("float", lib.fastembedr_cuda_opentsne_fft_from_device_knn_float_pca_float, xf),
                         ("double", lib.fastembedr_cuda_opentsne_fft_from_device_knn_float_pca_double, xd)):
        out = np.zeros((n, 2), np.float32)
        st = fn(d_idx.data_ptr(), d_dist.data_ptr(), arr.ctypes.data, arr.shape[1], *args, out.ctypes.data)
        _lib.check(st, "PCA t-SNE " + tag)
        outs[tag] = out
    init = api.tsne_pca_init(x.astype(np.float32))
    ref = np.zeros((n, 2), np.float32)
    st = lib.fastembedr_cuda_opentsne_fft_from_device_knn_float(d_idx.data_ptr(), d_dist.data_ptr(), init.ctypes.data,
                                                                1, *args, ref.ctypes.data)
    _lib.check(st, "t-SNE from the same start")
    scale = np.abs(ref).max()
    for tag, out in outs.items():
        assert np.abs(out - ref).max() <= 1e-4 * scale, tag


def test_pca_start_rejects_bad_input():
    x = np.random.default_rng(0).normal(size=(100, 5)).astype(np.float32)
    x[3, 2] = np.nan
    with pytest.raises(_lib.CudaEmbeddingError, match="finite"):
        api.tsne_pca_init(x)
    with pytest.raises(_lib.CudaEmbeddingError, match="1024 features"):
        api.tsne_pca_init(np.zeros((10, 1100), np.float32))
