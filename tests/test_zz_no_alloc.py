"""The no-allocation exact repulsion entry point, called through the C ABI.

It serves callers that cannot allocate device memory (the GPU's memory owned by another
framework's pool, or a request path where allocation is not allowed): inputs and outputs are
caller-owned device buffers and the working memory is a fixed array inside the library. The
result must equal the exact repulsion of the allocating diagnostic entry point and the FP64
oracle, on consecutive calls (the shared working array keeps the previous call's contents),
including the largest size the array holds; sizes beyond the array's capacity and misaligned
layouts must be rejected with an error. This file sorts last so a failure here does not stop the
rest of the suite.
"""
import numpy as np
import pytest

import oracle as O
from fastembedr_gb300 import _lib, api, synthetic

pytestmark = pytest.mark.gpu

CAPACITY = 65536


def rel_l2(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-300))


def _call(fn, y, what):
    import torch

    n = y.shape[0]
    d_y = torch.from_numpy(y).cuda()
    d_rep = torch.full((n, 2), float("nan"), dtype=torch.float32, device="cuda")
    d_z = torch.zeros(1, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    _lib.check(fn(d_y.data_ptr(), n, d_rep.data_ptr(), d_z.data_ptr(), None), what)
    return d_rep.cpu().numpy(), float(d_z.item())


def test_noalloc_exact_repulsion_matches_allocating_entry_point_and_oracle():
    lib = _lib.require_gpu()
    fn = lib.fastembedr_cuda_tsne_exact_repulsion_noalloc
    rng = np.random.default_rng(11)
    # two calls in a row at different sizes: the second call's array still holds the first's data
    for call, (n, sd) in enumerate(((3000, 3.0), (1200, 0.5))):
        x = rng.standard_normal((n, 5)).astype(np.float32)
        idx, dist = synthetic.exact_knn_numpy(x, 10)
        y = (rng.standard_normal((n, 2)) * sd).astype(np.float32)
        ref = api.tsne_force_diagnostic(idx, dist, y, 3.0, grid_size=64, exact=True, kl=False)
        rep, z = _call(fn, y, f"no-allocation repulsion (call {call + 1})")
        assert np.all(np.isfinite(rep))
        assert rel_l2(rep, ref["repulsive_force_exact"].astype(np.float64)) < 1e-5
        assert z == pytest.approx(ref["sum_q"], rel=1e-7)
        ex64, z64 = O.exact_rep_f64(y)
        assert rel_l2(rep, ex64) < 1e-5
        assert z == pytest.approx(z64, rel=1e-7)


def test_noalloc_at_full_capacity_matches_oracle():
    lib = _lib.require_gpu()
    fn = lib.fastembedr_cuda_tsne_exact_repulsion_noalloc
    y = (np.random.default_rng(12).standard_normal((CAPACITY, 2)) * 20.0).astype(np.float32)
    ex64, z64 = O.exact_rep_f64(y)
    for call in range(2):
        rep, z = _call(fn, y, f"no-allocation repulsion at capacity (call {call + 1})")
        assert rel_l2(rep, ex64) < 1e-5
        assert z == pytest.approx(z64, rel=1e-7)


def test_noalloc_rejects_sizes_beyond_capacity_and_misaligned_layouts():
    import torch

    lib = _lib.require_gpu()
    fn = lib.fastembedr_cuda_tsne_exact_repulsion_noalloc
    d = torch.zeros((8, 2), dtype=torch.float32, device="cuda")
    st = fn(d.data_ptr(), CAPACITY + 1, d.data_ptr(), None, None)
    assert st == 1
    assert b"capacity" in lib.fastembedr_cuda_embedding_last_error()
    st = fn(d.data_ptr() + 4, 4, d.data_ptr(), None, None)
    assert st == 1
    assert b"aligned" in lib.fastembedr_cuda_embedding_last_error()
