"""The oracle's restatement of the reference's multi-threaded CPU SGD branch (optimize_layout_csr
with more than one worker at n >= 10000, src/fast_knn_umap.cpp:3224-3350), which the UMAP CPU
baseline times: asynchronous, so it is checked statistically against the serial branch on the
same graph and start, not bit for bit."""
import numpy as np

import oracle as O
from fastembedr_gb300 import synthetic


def test_threaded_sgd_reaches_the_serial_branch():
    O.build()
    x, _ = synthetic.mixture(12000, 20, 8, 77, centre_sd=6.0)
    idx, dist = synthetic.exact_knn_numpy(x, 15)
    n = idx.shape[0]
    off, nb, w, _, _ = O.umap_graph(idx, dist)
    a, b = O.umap_ab(0.01)
    xc = x.astype(np.float64) - x.mean(0)
    _, _, vt = np.linalg.svd(xc[::3], full_matrices=False)
    init = xc @ vt[:2].T
    init *= 10.0 / np.abs(init).max()
    keep = np.arange(0, n, 3, dtype=np.int32)
    pres = []
    for fn, extra in ((O.orc().orc_umap_sgd_serial, ()), (O.orc().orc_umap_sgd_threaded, (4,))):
        emb = np.ascontiguousarray(init.T).ravel().copy()
        fn(n, off, nb, w, emb, 60, a, b, 5, 1.0, 1.0, 42, *extra)
        lay = emb.reshape(2, n).T.astype(np.float32)
        assert np.all(np.isfinite(lay))
        pres.append(O.knn_preservation(lay, idx, keep=keep, preserve_k=15))
    assert abs(pres[0] - pres[1]) < 0.005, pres
