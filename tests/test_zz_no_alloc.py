"""The no-allocation exact repulsion entry point, called through the C ABI.

It serves callers that cannot allocate device memory (the GPU's memory owned by another
framework's pool, or a request path where allocation is not allowed): inputs and outputs are
caller-owned device buffers and the working memory is a fixed array inside the library. The
result must equal the exact repulsion of the allocating diagnostic entry point, on consecutive
calls (the shared working array keeps the previous call's contents), and sizes beyond the
array's capacity must be rejected with an error. This file sorts last so a failure here does not
stop the rest of the suite.
"""
import numpy as np
import pytest

from fastembedr_gb300 import _lib, api, synthetic

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-300))


def test_noalloc_exact_repulsion_matches_allocating_entry_point():
    import torch

    lib = _lib.require_gpu()
    fn = lib.fastembedr_cuda_tsne_exact_repulsion_noalloc
    rng = np.random.default_rng(11)
    for call, (n, sd) in enumerate(((3000, 3.0), (1200, 0.5))):
        x = rng.standard_normal((n, 5)).astype(np.float32)
        idx, dist = synthetic.exact_knn_numpy(x, 10)
        y = (rng.standard_normal((n, 2)) * sd).astype(np.float32)
        ref = api.tsne_force_diagnostic(idx, dist, y, 3.0, grid_size=64, exact=True, kl=False)
        d_y = torch.from_numpy(y).cuda()
        d_rep = torch.full((n, 2), float("nan"), dtype=torch.float32, device="cuda")
        d_z = torch.zeros(1, dtype=torch.float64, device="cuda")
        st = fn(d_y.data_ptr(), n, d_rep.data_ptr(), d_z.data_ptr(), None)
        _lib.check(st, f"no-allocation repulsion (call {call + 1})")
        rep = d_rep.cpu().numpy()
        assert np.all(np.isfinite(rep))
        assert rel_l2(rep, ref["repulsive_force_exact"].astype(np.float64)) < 1e-5
        assert float(d_z.item()) == pytest.approx(ref["sum_q"], rel=1e-7)


def test_noalloc_rejects_sizes_beyond_capacity():
    import torch

    lib = _lib.require_gpu()
    fn = lib.fastembedr_cuda_tsne_exact_repulsion_noalloc
    d = torch.zeros((4, 2), dtype=torch.float32, device="cuda")
    st = fn(d.data_ptr(), 65537, d.data_ptr(), None, None)
    assert st == 1
    assert b"capacity" in lib.fastembedr_cuda_embedding_last_error()
