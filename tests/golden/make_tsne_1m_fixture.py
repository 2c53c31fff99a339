"""Generate tests/golden/tsne_1m_cpu_run.json: the reference CPU optimizer's result on the
1M-point t-SNE workload, for the end-to-end parity line of bench.py.

The workload is bench.py's: 1,000,000 x 50 mixture of 30 anisotropic clusters (seed 3), exact
k = 90 KNN (torch brute force on the GPU, as bench.py computes it), perplexity 30, Y_init
N(0, 1e-4^2) (seed 4), 250 iterations at early exaggeration 12 then 750 at 1, opt-SNE learning
rate n / 12, momentum 0.8, the reference CPU grid policy (256 nodes at this size). The CPU run is
the oracle restatement of the reference CPU optimizer (bit-identical to it on every case this
repository pins). Stored: the exact KL of the final layout (all-pairs Z, summed on the GPU by the
library's exact KL, which is pinned to the oracle), its 15-NN preservation over every 500th row,
and SHA-256 digests of the KNN input so bench.py can tell whether it recomputed the same input.

Needs a GPU (KNN and the exact KL) and a few minutes of host CPU. Run:
    python tests/golden/make_tsne_1m_fixture.py OUT.json
then copy OUT.json to tests/golden/tsne_1m_cpu_run.json.
"""
from __future__ import annotations

import hashlib
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402
from fastembedr_gb300 import api  # noqa: E402
from fastembedr_gb300 import synthetic as S  # noqa: E402

N, K, PERP = 1_000_000, 90, 30.0
KEEP_STRIDE = 500


def knn_digest(idx, dist):
    return {"indices_sha256": hashlib.sha256(np.ascontiguousarray(idx, np.int32).tobytes()).hexdigest(),
            "distances_sha256": hashlib.sha256(np.ascontiguousarray(dist, np.float32).tobytes()).hexdigest()}


def layout_quality(idx, dist, y):
    """Exact KL of layout y under the workload's P, and 15-NN preservation over every 500th row."""
    with api.TsneBatch([(idx, dist)], perplexity=PERP, inits=[np.ascontiguousarray(y, np.float32)]) as b:
        kl = b.kl(0)
    keep = np.arange(0, y.shape[0], KEEP_STRIDE, dtype=np.int32)
    return kl, float(O.knn_preservation(y, idx, keep=keep, preserve_k=15))


def main(out):
    x, _ = S.tsne_1m(n=N)
    i_t, d_t = S.exact_knn_torch(x, K, device="cuda")
    idx, dist = i_t.cpu().numpy(), d_t.cpu().numpy()
    init = S.tsne_init(N)
    O.build()
    threads = O.orc().orc_set_threads(0)
    t = time.perf_counter()
    y = O.tsne_run(idx, dist, init, perplexity=PERP, early_iter=250, n_iter=750, learning_rate=N / 12.0)
    cpu_s = time.perf_counter() - t
    kl, pres = layout_quality(idx, dist, y)
    rec = {"workload": "tsne_knn_1M_k90_perp30", "n": N, "k": K, "perplexity": PERP, "iterations": [250, 750],
           "learning_rate": N / 12.0, "grid": "reference CPU policy (256 nodes)", "kl": kl,
           "preservation_15nn": pres, "preservation_rows": f"every {KEEP_STRIDE}th row",
           "cpu_seconds": cpu_s, "cpu_threads": threads, "knn": knn_digest(idx, dist),
           "layout_sd": [float(v) for v in y.std(0)]}
    with open(out, "w") as f:
        json.dump(rec, f, indent=1)
    print(json.dumps(rec))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.join(os.path.dirname(os.path.abspath(__file__)),
                                                              "tsne_1m_cpu_run.json"))
