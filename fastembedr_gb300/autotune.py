"""Calibration of the adaptive box count: KL, final span and time per iteration of one t-SNE
instance per (size, grid) pair, each run as a batch of one with a fixed grid size.

The adaptive policy of the batched form (node spacing <= 0.7 over the current layout, at least
128 nodes) was chosen from this sweep. Run ``python -m fastembedr_gb300.autotune`` on a GPU to
print one JSON line per (n, G).
"""
from __future__ import annotations

import json

import numpy as np

from . import api, synthetic


def calibrate_grid_sizes(sizes=(2000, 10000, 50000, 200000), grids=(64, 128, 256, 512, 1024), k=90,
                         perplexity=30.0, seed=11):
    import torch

    rows = []
    for n in sizes:
        x, _ = synthetic.mixture(n, 50, 10, seed, centre_sd=4.0, lognormal_sizes=True)
        idx, dist = synthetic.exact_knn_torch(x, k)
        knn = (idx.cpu().numpy(), dist.cpu().numpy())
        init = synthetic.tsne_init(n, seed=5)
        for g in grids:
            if n <= 10000 and g > 512:
                continue
            with api.TsneBatch([knn], perplexity=perplexity, inits=[init], grid_size=g) as b:
                stream = torch.cuda.ExternalStream(b.stream)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                b.iterate(250, 12.0, 1.0 / 12.0)
                b.synchronize()
                e0.record(stream)
                b.iterate(750, 1.0, 1.0 / 12.0)
                e1.record(stream)
                b.synchronize()
                lay = b.layouts()[0]
                kl = b.kl(0)
            span = float(np.ptp(lay, 0).max())
            rows.append(dict(n=n, G=g, kl=kl, span=span, h=1.1 * span / (g - 1), ms_iter=e0.elapsed_time(e1) / 750))
    return rows


if __name__ == "__main__":
    for r in calibrate_grid_sizes():
        print(json.dumps(r), flush=True)
